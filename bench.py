#!/usr/bin/env python
"""Benchmark of the GB300 device path for ITensor's two-site DMRG inner loop.

Workload (one "step"): the isolated effective-Hamiltonian apply
H_eff psi = noPrime(((psi L) W1) W2 R) of LocalOp::product
(itensor/mps/localop.h:324-365) on a U(1) block-sparse bond of dimension
m = 1024 split over 31 Sz sectors with Gaussian sizes (sigma = 6 sectors),
local dimension 2, Heisenberg MPO (bond dimension 5); psi, L, R hold N(0,1)
FP64 entries from a fixed seed (synthetic data of the stated shape).

Metric: H_eff TFLOP/s = algorithmic FLOPs (sum over matched block pairs of
2 M N K, FP64-equivalent) per second. The headline form is the split
precision (FP64 operands as exact BF16 integer slices on the tensor pipe),
whose result is checked against the plain FP64 path in the same run; the
plain FP64 path and the DMRG sweep time of the N=20 Heisenberg chain
(5 sweeps, maxdim 10..200, cutoff 1e-10, niter 2) are reported beside it.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

M_BOND, K_SECT, SIGMA, SEED = 1024, 15, 6.0, 20241204
# DRAM traffic of the dominant launches of this workload, from one ncu capture
# (dram__bytes_read.sum + dram__bytes_write.sum; the outputs stay in L2): the
# split form's psi*L prep + GEMM pair, and the plain FP64 psi*L GEMM
PSI_L_SPLIT_DRAM_BYTES = 1671680 + 7174656
PSI_L_F64_DRAM_BYTES = 3777280
METRIC = "H_eff TFLOP/s (isolated apply, m=1024, 31 Sz sectors)"
UNIT = "TFLOP/s"
CONFIG = {"workload": "isolated H_eff apply: U(1) block-sparse L(m x 5 x m) W W R psi, m=1024 over 31 Sz "
                      "sectors (Gaussian sizes, sigma=6), d=2, Heisenberg MPO k=5, FP64 N(0,1) entries",
          "m": M_BOND, "sectors": 2 * K_SECT + 1, "d": 2, "mpo_bond_dim": 5, "seed": SEED,
          "l2": "flushed between timed steps (256 MiB write)"}
HEIS20_SWEEPS = [dict(maxdim=d, mindim=1, cutoff=1e-10, niter=2) for d in (10, 20, 100, 100, 200)]


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


# ---------------------------------------------------------------- CPU oracle (reference arm / baseline)
def _oracle_setup():
    import numpy as np
    from itensor_gb300 import workloads
    from oracle.blocksparse import BSTensor, Index, QN
    wl = workloads.heff_workload(M_BOND, K_SECT, SIGMA, SEED)

    def conv(t):
        inds = [Index([(QN(("Sz", q, 1)), d) for q, d in zip(I["qn"], I["dims"])], dir=I["dir"], id=I["id"],
                      plev=I["plev"]) for I in t["inds"]]
        T = BSTensor(inds)
        off = 0
        for c in t["coords"]:
            c = tuple(int(x) for x in c)
            shp = T.block_shape(c)
            n = int(np.prod(shp))
            T.blocks[c] = np.reshape(t["data"][off:off + n], shp, order="F").copy(order="F")
            off += n
        return T

    return {k: conv(wl[k]) for k in ("psi", "L", "W1", "W2", "R")}


def _oracle_apply_loop(n_applies):
    """Worker: n applies of the oracle's LocalOp::product; returns seconds."""
    from oracle.dmrg import LocalOp
    t = _oracle_setup()
    op = LocalOp(t["W1"], t["W2"], t["L"], t["R"])
    op.product(t["psi"])  # warm
    t0 = time.perf_counter()
    for _ in range(n_applies):
        op.product(t["psi"])
    return time.perf_counter() - t0


_WORKER_OP = None


def _oracle_worker_init():
    """Process-pool initializer: the workload and operator are built once per worker."""
    global _WORKER_OP
    from oracle.dmrg import LocalOp
    t = _oracle_setup()
    _WORKER_OP = (LocalOp(t["W1"], t["W2"], t["L"], t["R"]), t["psi"])
    _WORKER_OP[0].product(_WORKER_OP[1])  # warm


def _oracle_worker_apply(_):
    op, psi = _WORKER_OP
    op.product(psi)
    return 0


def _single_thread_env():
    env = dict(os.environ)
    for k in ("OMP_NUM_THREADS", "OPENBLAS_NUM_THREADS", "MKL_NUM_THREADS"):
        env[k] = "1"
    return env


REF_BENCH = os.path.join(ROOT, "oracle", "_ref", "ref_bench")


def reference_runnable():
    """('', True) when the reference library's timing program (oracle/ref_bench.cc,
    built from the reference's own sources by oracle/Makefile.ref) runs on this
    host, else (why not, False)."""
    if not os.path.exists(REF_BENCH):
        return ("the ITensor C++ reference is built only where its sources lie (the x86 build container); "
                "this host has no build of it (oracle/_ref/ref_bench absent)"), False
    try:
        r = subprocess.run([REF_BENCH], capture_output=True, timeout=60)
    except OSError as e:
        return "oracle/_ref/ref_bench does not run on this host: %s" % e, False
    return ("", True) if r.returncode == 2 else ("oracle/_ref/ref_bench failed: rc %d" % r.returncode, False)


def _reference_heff(threads, budget_s):
    """LocalOp::product of the reference library on the benchmark's bytes
    (written in the reference's ITensor file layout): (applies, seconds)."""
    import tempfile
    from itensor_gb300 import workloads
    from oracle import itensor_file
    wl = workloads.heff_workload(M_BOND, K_SECT, SIGMA, SEED)
    with tempfile.TemporaryDirectory() as d:
        for k in ("psi", "L", "W1", "W2", "R"):
            itensor_file.write(os.path.join(d, k + ".itensor"), wl[k])
        env = dict(os.environ, OMP_NUM_THREADS=str(threads), OPENBLAS_NUM_THREADS="1", MKL_NUM_THREADS="1")
        out = subprocess.run([REF_BENCH, "heff", d, str(budget_s)], capture_output=True, text=True, env=env,
                             timeout=600)
    if out.returncode != 0:
        raise RuntimeError("ref_bench heff: " + out.stderr[-300:])
    r = json.loads(out.stdout.strip().splitlines()[-1])
    return r["n"], r["sec"]


def cpu_baseline(flops_per_apply, budget_s=15.0):
    """The reference's own apply (LocalOp::product of the C++ library) timed on
    one host core where it is built, else the oracle's restatement; a bounded
    sample of the same input."""
    why, ok = reference_runnable()
    if ok:
        try:
            n, sec = _reference_heff(1, budget_s)
            per = sec / n
            return {"value": flops_per_apply / per / 1e12, "unit": UNIT, "cores": 1, "kind": "reference",
                    "sample": "%d applies of the reference library's LocalOp::product (oracle/_ref, LAPACK/BLAS "
                              "build, OMP 1, BLAS 1) on the same input, %.1f ms/apply" % (n, per * 1e3)}
        except (RuntimeError, subprocess.TimeoutExpired, ValueError) as e:
            why = str(e)[:300]
    line = _port_baseline(flops_per_apply, budget_s)
    line["reference_unavailable"] = why
    return line


def _port_baseline(flops_per_apply, budget_s):
    """Oracle apply timed on one host core in a subprocess (bounded sample)."""
    code = ("import sys,json;sys.path.insert(0,%r);import bench;"
            "t1=bench._oracle_apply_loop(1);n=max(1,int(%f/max(t1,1e-3)));"
            "t=bench._oracle_apply_loop(n);print(json.dumps({'n':n,'sec':t}))" % (ROOT, budget_s / 2))
    out = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, env=_single_thread_env(),
                         timeout=600)
    if out.returncode != 0:
        return {"value": None, "unit": UNIT, "cores": 1, "kind": "port", "sample": "failed: " + out.stderr[-300:]}
    r = json.loads(out.stdout.strip().splitlines()[-1])
    per = r["sec"] / r["n"]
    return {"value": flops_per_apply / per / 1e12, "unit": UNIT, "cores": 1, "kind": "port",
            "sample": "%d applies of the numpy oracle (LocalOp::product restatement) on the same input, "
                      "1 thread, %.1f ms/apply" % (r["n"], per * 1e3)}


def run_reference(args):
    rank, world, _ = dist_env()
    if rank != 0:
        return 0
    cores = os.cpu_count() or 1
    flops = _oracle_flops()
    why, ok = reference_runnable()
    if ok:
        # the reference library itself, all host threads (its OpenMP loop over output blocks), BLAS 1
        try:
            _reference_heff(cores, 0.2 * max(1, args.warmup))
            n, sec = _reference_heff(cores, 0.5 * max(1, args.steps))
            value = flops * n / sec / 1e12
            line = {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
                    "steps": args.steps, "warmup": args.warmup, "ms_per_step": sec / n * 1e3,
                    "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
                    "data": "synthetic", "config": CONFIG,
                    "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": "reference",
                                     "sample": "%d applies of the reference library's LocalOp::product "
                                               "(oracle/_ref, OMP_NUM_THREADS=%d, BLAS 1 thread)" % (n, cores)},
                    "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
            print(json.dumps(line))
            return 0
        except (RuntimeError, subprocess.TimeoutExpired, ValueError) as e:
            why = str(e)[:300]
    import multiprocessing as mp
    for k in ("OMP_NUM_THREADS", "OPENBLAS_NUM_THREADS", "MKL_NUM_THREADS"):
        os.environ[k] = "1"
    ctxm = mp.get_context("spawn")
    with ctxm.Pool(cores, initializer=_oracle_worker_init) as pool:
        for _ in range(args.warmup):
            pool.map(_oracle_worker_apply, range(cores), chunksize=1)
        t0 = time.perf_counter()
        for _ in range(args.steps):
            pool.map(_oracle_worker_apply, range(cores), chunksize=1)
        el = time.perf_counter() - t0
    # each step: `cores` independent applies in parallel
    value = flops * cores * args.steps / el / 1e12
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": el / args.steps * 1e3,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": CONFIG,
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": "port",
                             "sample": "each step: %d parallel single-thread applies of the numpy oracle "
                                       "(restatement of LocalOp::product)" % cores,
                             "reference_unavailable": why},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))
    return 0


def _oracle_flops():
    t = _oracle_setup()
    from oracle.blocksparse import contract
    total = 0.0
    # algorithmic flops of the four contractions: sum over matched pairs of 2 M N K
    p = t["psi"]
    for B in (t["L"], t["W1"], t["W2"], t["R"]):
        total += _pair_flops(p, B)
        p = contract(p, B)
    return total


def _pair_flops(A, B):
    import numpy as np
    AtoB = {}
    for i, I in enumerate(A.inds):
        for j, J in enumerate(B.inds):
            if I.same(J):
                AtoB[i] = j
                break
    f = 0.0
    for ca, ba in A.blocks.items():
        for cb, bb in B.blocks.items():
            if all(ca[i] == cb[j] for i, j in AtoB.items()):
                K = int(np.prod([ba.shape[i] for i in AtoB])) if AtoB else 1
                f += 2.0 * (ba.size // K) * (bb.size // K) * K
    return f


# ---------------------------------------------------------------- clocks
class ClockSampler:
    def __init__(self, index=0):
        self.index = index
        self.proc = None
        self.lines = []

    def start(self):
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), "--query-gpu=" + q,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None

    def _read(self):
        for ln in self.proc.stdout:
            self.lines.append(ln.strip())

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx = float(parts[2])
            except ValueError:
                continue
            for n, v in zip(names, parts[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


# ---------------------------------------------------------------- device arm
def measured_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return json.load(f), "measured"
    except OSError:
        return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "bf16_tflops_sustained": 1700.0}, "fallback"


# ---------------------------------------------------------------- many independent solves
BATCH_SEED, SERVE_SEED = 4242, 5151


def ramp_sweeps(maxdim, n=5, cutoff=1e-10):
    """The last n of the sweeps maxdim/8, maxdim/4, maxdim/2, maxdim, maxdim."""
    full = [max(8, maxdim // 8), max(16, maxdim // 4), maxdim // 2, maxdim, maxdim]
    return [dict(maxdim=int(m), mindim=1, cutoff=cutoff, niter=2) for m in full[5 - n:]]


def j1j2_chains(n, seed=BATCH_SEED):
    """Independent J1-J2 Heisenberg chains: J2 ~ U[0, 0.5], N ~ U{16..64},
    maxdim ~ U{64..256}, Sz QN, Neel start, five sweeps ramping to maxdim."""
    import numpy as np
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(n):
        N = int(rng.integers(16, 65))
        J2 = float(rng.uniform(0.0, 0.5))
        md = int(rng.integers(64, 257))
        out.append((dict(type=0, N=N, J=1.0, Jz=1.0, J2=J2), ramp_sweeps(md)))
    return out


def serving_requests(n, seed=SERVE_SEED):
    """Ground-state requests: XXZ chains (Delta ~ U[0, 2], Sz QN) and
    transverse-field Ising chains (h ~ U[0.5, 1.5], parity QN), N ~ U{16..128},
    maxdim ~ U{32..512}, four sweeps ramping to maxdim."""
    import numpy as np
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(n):
        N = int(rng.integers(16, 129))
        md = int(rng.integers(32, 513))
        if rng.uniform() < 0.5:
            m = dict(type=0, N=N, J=1.0, Jz=float(rng.uniform(0.0, 2.0)))
        else:
            m = dict(type=1, N=N, h=float(rng.uniform(0.5, 1.5)))
        out.append((m, ramp_sweeps(md, 4)))
    return out


def pool_shape():
    cores = os.cpu_count() or 1
    return max(1, min(16, cores - 1)), 8


def bench_batched(ctx, n_chains, n_seq, budget_bytes):
    """Batched form: every chain submitted at once to the solver pool in the
    split precision; beside it the plain FP64 path solving chains one after
    the other on one context (a stride sample of the same chains)."""
    import itensor_gb300 as itg
    chains = j1j2_chains(n_chains)
    stride = max(1, n_chains // n_seq)
    sample = list(range(0, n_chains, stride))[:n_seq]
    # plain FP64 path, sequential
    ctx.dmrg(*chains[sample[0]], precision=itg.PREC_F64)  # warm plans and pool
    t0 = time.perf_counter()
    seq = {}
    for i in sample:
        seq[i] = ctx.dmrg(*chains[i], precision=itg.PREC_F64)
    t_seq = time.perf_counter() - t0
    seq_bonds = sum(len(r.bonds) for r in seq.values())
    workers, slots = pool_shape()

    def pool_run(prec):
        pool = itg.Pool(0, workers=workers, slots_per_worker=slots, budget_bytes=budget_bytes)
        try:
            ids = [pool.submit(m, sw, prec) for m, sw in chains]
            t0 = time.perf_counter()
            pool.start()
            pool.drain()
            el = time.perf_counter() - t0
            st = pool.stats()
            res = {i: pool.result(ids[i]) for i in range(n_chains) if pool.record(ids[i]).status == 0}
        finally:
            pool.close()
        return el, st, res

    # the same pool (workers, slots, chains) in plain FP64: separates the
    # precision form's gain from the concurrency's
    t_pool64, st64, res64 = pool_run(itg.PREC_F64)
    t_pool, st, res = pool_run(itg.PREC_OZAKI_BF16)
    pool_bonds = sum(len(r.bonds) for r in res.values())
    # split-precision energies against plain FP64, every chain
    dE = [abs(res[i].energy - res64[i].energy) for i in range(n_chains) if i in res and i in res64]
    dE_seq = [abs(res64[i].energy - seq[i].energy) for i in sample if i in res64]
    seq_rate = len(sample) / t_seq
    pool_rate = len(res) / t_pool
    pool64_rate = len(res64) / t_pool64
    return {"workload": "%d independent J1-J2 chains (J2~U[0,0.5], N~U{16..64}, maxdim~U{64..256}, Sz QN, "
                        "Neel start, 5 sweeps ramping to maxdim, cutoff 1e-10, niter 2; seed %d)" % (n_chains, BATCH_SEED),
            "batched": {"precision": "split (6 BF16 slices, FP32-exact accumulation); FP64 Davidson, eigensolver, SVD",
                        "seconds": t_pool, "solves_per_s": pool_rate, "sweeps_per_s": pool_rate * 5,
                        "bond_steps_per_s": pool_bonds / t_pool, "failed": st["failed"],
                        "workers": workers, "slots_per_worker": slots, "peak_running": st["peak_running"]},
            "pool_f64": {"precision": "plain FP64, the same pool shape and chains", "seconds": t_pool64,
                         "solves_per_s": pool64_rate, "bond_steps_per_s": sum(len(r.bonds) for r in res64.values())
                         / t_pool64, "failed": st64["failed"], "peak_running": st64["peak_running"]},
            "plain_f64_sequential": {"chains": len(sample), "seconds": t_seq, "solves_per_s": seq_rate,
                                     "sweeps_per_s": seq_rate * 5, "bond_steps_per_s": seq_bonds / t_seq,
                                     "sample": "every %dth chain of the same set, one context, one after the other"
                                               % stride},
            "speedup_solves_per_s": pool_rate / seq_rate,
            "speedup_split_over_pool_f64": pool_rate / pool64_rate,
            "speedup_pool_f64_over_sequential_f64": pool64_rate / seq_rate,
            "energy_vs_f64": {"max_abs_dE": max(dE) if dE else None,
                              "within_1e-9": sum(1 for x in dE if x <= 1e-9), "compared": len(dE),
                              "against": "the same chains in the FP64 pool"},
            "pool_f64_vs_sequential_max_abs_dE": max(dE_seq) if dE_seq else None}


def bench_serving(n_req, budget_bytes, load=0.8):
    """Serving: requests arrive as a Poisson stream and are admitted by memory
    while others run. First a saturation pass (every request at t = 0) gives
    the throughput; then a fresh set arrives at rate lambda = load x that
    throughput and the latency distribution is measured."""
    import numpy as np
    import itensor_gb300 as itg
    workers, slots = pool_shape()

    def run(reqs, arrivals):
        pool = itg.Pool(0, workers=workers, slots_per_worker=slots, budget_bytes=budget_bytes)
        try:
            pool.start()
            t0 = time.perf_counter()
            ids = [pool.submit(m, sw, itg.PREC_OZAKI_BF16, arrival=a) for (m, sw), a in zip(reqs, arrivals)]
            pool.drain()
            el = time.perf_counter() - t0
            recs = [pool.record(i) for i in ids]
            st = pool.stats()
        finally:
            pool.close()
        return el, recs, st

    sat_reqs = serving_requests(n_req, SERVE_SEED)
    el, recs, st = run(sat_reqs, [0.0] * n_req)
    ok = [r for r in recs if r.status == 0]
    mu = len(ok) / el
    lam = load * mu
    rng = np.random.default_rng(SERVE_SEED + 1)
    arr = np.cumsum(rng.exponential(1.0 / lam, n_req))
    reqs = serving_requests(n_req, SERVE_SEED + 2)
    el2, recs2, st2 = run(reqs, arr.tolist())
    ok2 = [r for r in recs2 if r.status == 0]
    lat = np.array([r.latency for r in ok2])
    wait = np.array([r.t_admit - r.t_arrive for r in ok2])
    est = np.array([r.est_bytes for r in ok2])
    peak = np.array([r.peak_bytes for r in ok2])
    return {"workload": "%d requests per pass: XXZ (Delta~U[0,2], Sz QN) and transverse-field Ising (h~U[0.5,1.5], "
                        "parity QN) chains, N~U{16..128}, maxdim~U{32..512}, 4 sweeps ramping to maxdim, cutoff "
                        "1e-10, split precision" % n_req,
            "saturation": {"seconds": el, "solves_per_s": mu, "failed": len(recs) - len(ok),
                           "peak_running": st["peak_running"]},
            "poisson": {"lambda_per_s": lam, "load": load, "seconds": el2, "solves_per_s": len(ok2) / el2,
                        "failed": len(recs2) - len(ok2),
                        "latency_s": {"p50": float(np.percentile(lat, 50)), "p90": float(np.percentile(lat, 90)),
                                      "p99": float(np.percentile(lat, 99)), "max": float(lat.max())},
                        "queue_wait_s": {"p50": float(np.percentile(wait, 50)), "p99": float(np.percentile(wait, 99))},
                        "peak_running": st2["peak_running"],
                        "peak_reserved_gb": st2["peak_reserved_bytes"] / 1e9,
                        "hbm_budget_gb": budget_bytes / 1e9,
                        "reserved_occupancy_peak": st2["peak_reserved_bytes"] / budget_bytes,
                        "measured_over_estimate": {"max": float((peak / est).max()),
                                                   "mean": float((peak / est).mean())}},
            "pool": {"workers": workers, "slots_per_worker": slots}}


def run_profile_dmrg(args):
    """One DMRG solve for ncu's launch list: J1-J2 chain N=48, J2=0.3, three
    sweeps with maxdim 64, 128, 256, cutoff 1e-10, niter 2, split precision."""
    import itensor_gb300 as itg
    ctx = itg.Context(0)
    sw = [dict(maxdim=m, mindim=1, cutoff=1e-10, niter=2) for m in (64, 128, 256)]
    t0 = time.perf_counter()
    r = ctx.dmrg(dict(type=0, N=48, J=1.0, Jz=1.0, J2=0.3), sw, precision=itg.PREC_OZAKI_BF16)
    print(json.dumps({"energy": r.energy, "bond_steps": len(r.bonds), "seconds": time.perf_counter() - t0,
                      "phase_seconds": r.phase_seconds, "stats": ctx.stats()}))
    ctx.close()
    return 0


def run_profile_pool(args):
    """A small pool for ncu's launch list: the first `--profile-pool` chains of
    the batched set through the solver pool in plain FP64, one worker with
    eight slots and cross-solve grouping on, so the grouped launches show."""
    import itensor_gb300 as itg
    chains = j1j2_chains(args.profile_pool)
    pool = itg.Pool(0, workers=1, slots_per_worker=8, budget_bytes=8 << 30, grouping=True)
    try:
        ids = [pool.submit(m, sw, itg.PREC_F64) for m, sw in chains]
        t0 = time.perf_counter()
        pool.start()
        pool.drain()
        el = time.perf_counter() - t0
        print(json.dumps({"solves": len(ids), "seconds": el, "grouping": pool.grouping_stats(),
                          "failed": pool.stats()["failed"]}))
    finally:
        pool.close()
    return 0


def cylinder_sweeps(maxdim):
    """The sweep table of the reference's 2D Hubbard sample (sample/hubbard_2d.cc:43-46):
    maxdim 20, 60, 100, 100, 200, 400, 800, 2000, 3000 (capped at `maxdim`), noise
    1e-7, 1e-8, 1e-10, then 0; cutoff 1e-9 and niter 2 as the cylinder workload states."""
    mds = [m for m in (20, 60, 100, 100, 200, 400, 800, 2000, 3000) if m < maxdim] + [maxdim]
    noise = [1e-7, 1e-8, 1e-10]
    return [dict(maxdim=m, mindim=1, cutoff=1e-9, niter=2, noise=noise[i] if i < len(noise) else 0.0)
            for i, m in enumerate(mds)]


def run_cylinder(args):
    """Hubbard model on a 4x16 cylinder (Nx=16, Ny=4 periodic in y, snaked into
    the chain), t=1, U=4, half filling, (Nf, Sz) QN, Neel product start: DMRG in
    the split precision and in plain FP64 on the same sweep table; reports both
    energies, their difference, sweep times and the phase split."""
    import itensor_gb300 as itg
    model = dict(type=2, Lx=16, Ly=4, t=1.0, U=4.0, yperiodic=1)
    sw = cylinder_sweeps(args.cylinder)
    out = {"workload": "hubbard_4x16_cylinder", "t": 1.0, "U": 4.0, "sweeps": sw}
    runs = [(n, {"split": itg.PREC_OZAKI_BF16, "fp64": itg.PREC_F64}[n]) for n in args.cyl_runs.split(",")]
    for name, prec in runs:
        ctx = itg.Context(0)   # a fresh context each: no contraction plans carried over
        clk = ClockSampler(0)
        clk.start()
        t0 = time.perf_counter()
        r = ctx.dmrg(model, sw, precision=prec)
        el = time.perf_counter() - t0
        out[name] = {"energy": r.energy, "seconds": el, "sweep_seconds": r.sweep_seconds,
                     "phase_seconds": r.phase_seconds, "max_link_dim": max(sum(int(x) for x in d) for _, _, d in r.links),
                     "last_sweep_truncerr_max": max(b[4] for b in r.bonds[-(2 * (64 - 1)):]),
                     "clocks": clk.stop()}
        ctx.close()
        print(json.dumps({name: out[name]}), flush=True)
    if "fp64" in out and "split" in out:
        out["energy_diff_split_vs_fp64"] = out["split"]["energy"] - out["fp64"]["energy"]
    print(json.dumps(out))
    return 0


def run_profile_cylinder(args):
    """One cylinder solve for ncu's launch list: the Hubbard 4x16 cylinder on
    the sweep table of run_cylinder up to maxdim `--profile-cylinder`, split
    precision, one context."""
    import itensor_gb300 as itg
    ctx = itg.Context(0)
    t0 = time.perf_counter()
    r = ctx.dmrg(dict(type=2, Lx=16, Ly=4, t=1.0, U=4.0, yperiodic=1), cylinder_sweeps(args.profile_cylinder),
                 precision=itg.PREC_OZAKI_BF16)
    print(json.dumps({"energy": r.energy, "bond_steps": len(r.bonds), "seconds": time.perf_counter() - t0,
                      "phase_seconds": r.phase_seconds, "stats": ctx.stats()}))
    ctx.close()
    return 0


def run_profile(args):
    """Short run of the same workload for ncu: for the split form and plain
    FP64, N prepared applies each (kernels launched one by one)."""
    import torch
    import itensor_gb300 as itg
    from itensor_gb300 import workloads
    ctx = itg.Context(0)
    ctx.set_precision(itg.PREC_OZAKI_BF16, args.slices)
    if args.gemm_variant >= 0:
        ctx.set_gemm_variant(args.gemm_variant)
    wl = workloads.heff_workload(M_BOND, K_SECT, SIGMA, SEED)
    dev = {k: workloads.to_device(ctx, wl[k]) for k in ("psi", "L", "W1", "W2", "R")}
    for prec in (itg.PREC_OZAKI_BF16, itg.PREC_F64):
        h = ctx.heff_prepare(dev["L"], dev["W1"], dev["W2"], dev["R"], dev["psi"], precision=prec, use_graph=False)
        out = torch.empty(h.out_size, dtype=torch.float64, device="cuda")
        for _ in range(args.profile):
            h.run(dev["psi"].device_ptr(), out.data_ptr())
        ctx.sync()
    ctx.close()
    print("profile run done")
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=30)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="gb300")
    ap.add_argument("--slices", type=int, default=6)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-dmrg", action="store_true")
    ap.add_argument("--chains", type=int, default=256, help="independent chains of the batched form (0: skip)")
    ap.add_argument("--seq-chains", type=int, default=16, help="chains solved one by one by the plain FP64 path")
    ap.add_argument("--requests", type=int, default=96, help="requests per serving pass (0: skip)")
    ap.add_argument("--profile-dmrg", action="store_true",
                    help="profiling run for ncu: one J1-J2 chain N=48, J2=0.3, maxdim 64/128/256, split precision")
    ap.add_argument("--profile", type=int, default=0,
                    help="profiling run for ncu: N prepared applies per arithmetic, no graph, no timing")
    ap.add_argument("--gemm-variant", type=int, default=-1,
                    help="with --profile: force the split-precision GEMM variant (0..3 mma.sync, 4 tcgen05)")
    ap.add_argument("--profile-pool", type=int, default=0,
                    help="profiling run for ncu: this many chains through a one-worker pool with grouping on")
    ap.add_argument("--cylinder", type=int, default=0,
                    help="Hubbard 4x16 cylinder DMRG up to this maxdim (3000 in the workload), split and FP64")
    ap.add_argument("--cyl-runs", default="split,fp64", help="with --cylinder: which arithmetics to run")
    ap.add_argument("--profile-cylinder", type=int, default=0,
                    help="profiling run for ncu: one cylinder solve up to this maxdim, split precision")
    args = ap.parse_args()
    if args.impl == "reference":
        return run_reference(args)
    if args.profile:
        return run_profile(args)
    if args.profile_pool:
        return run_profile_pool(args)
    if args.profile_dmrg:
        return run_profile_dmrg(args)
    if args.cylinder:
        return run_cylinder(args)
    if args.profile_cylinder:
        return run_profile_cylinder(args)
    args.warmup = max(args.warmup, 3)
    rank, world, local = dist_env()

    import numpy as np
    import torch
    import itensor_gb300 as itg
    from itensor_gb300 import workloads

    dist = None
    if world > 1:
        import torch.distributed as dist_
        dist_.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
        dist = dist_
    torch.cuda.set_device(local)
    ctx = itg.Context(local)
    ext = torch.cuda.ExternalStream(ctx.stream)
    wl = workloads.heff_workload(M_BOND, K_SECT, SIGMA, SEED)
    dev = {k: workloads.to_device(ctx, wl[k]) for k in ("psi", "L", "W1", "W2", "R")}
    L, W1, W2, R, psi = dev["L"], dev["W1"], dev["W2"], dev["R"], dev["psi"]

    # correctness gate: split form vs plain FP64 on this input
    ref64 = ctx.heff_apply(L, W1, W2, R, psi, precision=itg.PREC_F64).numpy()
    ctx.set_precision(itg.PREC_OZAKI_BF16, args.slices)
    oz = ctx.heff_apply(L, W1, W2, R, psi, precision=itg.PREC_OZAKI_BF16).numpy()
    rel = float(np.max(np.abs(oz - ref64)) / np.max(np.abs(ref64)))

    # algorithmic flops per apply (from the plans) and the dominant kernel
    ctx.profile_begin()
    ctx.heff_apply(L, W1, W2, R, psi, precision=itg.PREC_F64)
    prof = ctx.profile_end()
    flops_apply = sum(f for _, f, _ in prof)
    dom = max(range(len(prof)), key=lambda i: prof[i][1])  # biggest contraction (psi * L step)

    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")
    # prepared applies (plans resolved once); graph replay for the timed value,
    # per-launch events (no graph) for the kernel roofline
    H = {(prec, g): ctx.heff_prepare(L, W1, W2, R, psi, precision=prec, use_graph=g)
         for prec in (itg.PREC_OZAKI_BF16, itg.PREC_F64) for g in (True, False)}
    out_n = H[(itg.PREC_F64, True)].out_size
    outbuf = torch.empty(out_n, dtype=torch.float64, device="cuda")
    psi_ptr, out_ptr = psi.device_ptr(), outbuf.data_ptr()

    def timed(prec, steps, warmup, graph=True, profile=False):
        h = H[(prec, graph)]
        for _ in range(warmup):
            h.run(psi_ptr, out_ptr)
        ctx.sync()
        if dist:
            dist.barrier()
        torch.cuda.synchronize()
        tot = 0.0
        launches0 = ctx.stats()["kernel_launches"]
        if profile:
            ctx.profile_begin()
        for _ in range(steps):
            flush.zero_()
            torch.cuda.synchronize()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(ext)
            h.run(psi_ptr, out_ptr)
            e1.record(ext)
            e1.synchronize()
            tot += e0.elapsed_time(e1)
        pr = ctx.profile_end() if profile else []
        launches = ctx.stats()["kernel_launches"] - launches0
        torch.cuda.synchronize()
        if dist:
            t = torch.tensor([tot], device="cuda")
            dist.all_reduce(t, op=dist.ReduceOp.MAX)
            tot = float(t.item())
        return tot, launches, pr

    clocks = ClockSampler(local)
    clocks.start()
    t_oz, launches, _ = timed(itg.PREC_OZAKI_BF16, args.steps, args.warmup, graph=True)
    clk = clocks.stop()
    n64 = max(3, args.steps // 3)
    t_64, _, _ = timed(itg.PREC_F64, n64, 2, graph=True)
    # kernel-level pass: same steps, launches timed one by one
    t_ozp, _, prof_oz = timed(itg.PREC_OZAKI_BF16, args.steps, 2, graph=False, profile=True)
    t_64p, _, prof_64 = timed(itg.PREC_F64, n64, 2, graph=False, profile=True)

    value = flops_apply * args.steps * world / (t_oz / 1e3) / 1e12
    f64_value = flops_apply * n64 / (t_64 / 1e3) / 1e12

    # roofline of the dominant kernel (the psi*L block GEMM), averaged over the pass
    def dom_stats(pr):
        per = len(prof)
        ms = [pr[i][0] for i in range(dom, len(pr), per)]
        return statistics.mean(ms), pr[dom][1], pr[dom][2]

    peaks, peak_src = measured_peaks()
    dm_ms, dm_flops, dm_kind = dom_stats(prof_oz)
    achieved = dm_flops / (dm_ms / 1e3) / 1e12
    nsl = args.slices * (args.slices + 1) // 2
    roofline = {"bound": "tensor", "achieved": achieved, "peak": peaks["bf16_tflops"], "unit": "TFLOP/s",
                "frac": achieved / peaks["bf16_tflops"], "traffic": PSI_L_SPLIT_DRAM_BYTES,
                "traffic_source": "ncu dram__bytes_read.sum + dram__bytes_write.sum of the psi*L prep + GEMM "
                                  "launches of this workload (profiles/heff_apply_m1024_launch_list.md), bytes "
                                  "per launch pair",
                "kernel": "ozaki_prep<%d> x2 + gemm_ozaki_kernel<%d> (psi*L block GEMM)" % (args.slices, args.slices),
                "note": "achieved = algorithmic FP64-equivalent flops of the psi*L contraction / CUDA-event duration "
                        "of its launches (per-launch events, same steps as the timed region without graph replay); "
                        "peak = dense BF16 burst of %s (of %s); the kernel issues %d BF16 digit products per FP64 "
                        "product" % ("MEASURED_PEAKS.json" if peak_src == "measured" else "the fallback",
                                     peak_src, nsl),
                "digit_product_tflops": achieved * nsl, "digit_product_frac": achieved * nsl / peaks["bf16_tflops"]}
    # the kernel issues mma.sync (not tcgen05): its own pipe's measured rate, from the issue-rate microbenchmark
    try:
        own = ctx.measure_peaks()
        roofline["mma_sync_bf16_tflops_measured"] = own["bf16_mma_sync"]
        roofline["digit_product_frac_of_mma_sync"] = achieved * nsl / own["bf16_mma_sync"]
        roofline["fp64_ffma_tflops_measured"] = own["fp64_ffma"]
    except Exception as e:  # the microbenchmark is context only; the line stands without it
        roofline["mma_sync_bf16_tflops_measured"] = None
        roofline["peaks_error"] = str(e)[:200]
    d64_ms, d64_flops, _ = dom_stats(prof_64)
    # the plain FP64 path's dominant kernel (gemm_f64_kernel, psi*L) against the FP64 FFMA
    # issue rate this library measures (register-only loop; no FP64 figure in MEASURED_PEAKS.json)
    f64_ach = d64_flops / (d64_ms / 1e3) / 1e12
    f64_peak = roofline.get("fp64_ffma_tflops_measured")
    f64_roofline = {"bound": "fp64", "achieved": f64_ach, "peak": f64_peak, "unit": "TFLOP/s",
                    "frac": f64_ach / f64_peak if f64_peak else None, "traffic": PSI_L_F64_DRAM_BYTES,
                    "traffic_source": "ncu DRAM bytes of the psi*L gemm_f64_kernel launch of this workload "
                                      "(profiles/heff_apply_m1024_launch_list.md)",
                    "kernel": "gemm_f64_kernel (psi*L block GEMM)",
                    "note": "peak = FP64 FFMA rate measured by itg_measure_peaks on this GPU (of measured)"}

    # end-to-end through the C-ABI with host buffers: psi host -> device, apply, result -> host
    # (pinned host memory, as a caller that streams states through the apply would hold them)
    psi_pin = torch.from_numpy(np.ascontiguousarray(wl["psi"]["data"])).pin_memory()
    out_pin = torch.empty(out_n, dtype=torch.float64).pin_memory()
    psi_host, out_host = psi_pin.numpy(), out_pin.numpy()
    he = H[(itg.PREC_OZAKI_BF16, True)]
    e2e_t = 0.0
    for i in range(args.warmup + args.steps):
        flush.zero_()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        he.run_host(psi_host, out_host)
        dt = time.perf_counter() - t0
        if i >= args.warmup:
            e2e_t += dt
    # the unprepared public call: tensor from host data + itg_heff_apply + read back
    inds = psi.inds
    coords = wl["psi"]["coords"].reshape(-1)
    e2u_t = 0.0
    for i in range(args.warmup + args.steps):
        t0 = time.perf_counter()
        p = ctx.tensor(inds, coords, psi_host)
        ctx.heff_apply(L, W1, W2, R, p, precision=itg.PREC_OZAKI_BF16).numpy()
        dt = time.perf_counter() - t0
        if i >= args.warmup:
            e2u_t += dt
    e2e = {"value": flops_apply * args.steps / e2e_t / 1e12, "unit": UNIT,
           "h2d_bytes_per_step": int(8 * psi_host.size), "d2h_bytes_per_step": int(8 * out_n),
           "ms_per_step": e2e_t / args.steps * 1e3,
           "api": "itg_heff_run(host=1): pinned host psi -> device, graph-replayed apply, result -> pinned host",
           "unprepared_call": {"value": flops_apply * args.steps / e2u_t / 1e12,
                               "ms_per_step": e2u_t / args.steps * 1e3,
                               "api": "itg_tensor_create(host data) + itg_heff_apply + itg_tensor_read"}}

    # DMRG sweep time: N=20 Heisenberg chain (5 sweeps), plain FP64 and split form
    dmrg = None
    if not args.no_dmrg and rank == 0:
        ref_e = None
        try:
            with open(os.path.join(ROOT, "tests", "golden", "dmrg.json")) as f:
                ref_e = [c for c in json.load(f)["cases"] if c["name"] == "heis20"][0]["energy"]
        except OSError:
            pass
        dmrg = {"model": "S=1/2 Heisenberg N=20, Sz QN, Neel start, 5 sweeps maxdim 10,20,100,100,200, "
                         "cutoff 1e-10, niter 2", "reference_energy": ref_e}
        for name, prec in (("f64", itg.PREC_F64), ("split", itg.PREC_OZAKI_BF16)):
            ctx.dmrg(dict(type=0, N=20), HEIS20_SWEEPS, precision=prec)  # warm (plans, pool)
            runs = []
            for _ in range(3):  # the median of three solves (one solve is ~0.1 s: host hiccups show)
                t0 = time.perf_counter()
                r = ctx.dmrg(dict(type=0, N=20), HEIS20_SWEEPS, precision=prec)
                runs.append(time.perf_counter() - t0)
            dmrg[name] = {"seconds": sorted(runs)[1], "runs_seconds": runs, "sweep_seconds": r.sweep_seconds,
                          "energy": r.energy, "dE": None if ref_e is None else r.energy - ref_e,
                          "heff_applies": r.heff_applies}

    # many independent solves: the batched form and the serving loop (rank 0; replicas elsewhere)
    free_b, total_b = torch.cuda.mem_get_info()
    budget = int(0.8 * total_b)
    batched = serving = None
    if args.chains > 0 and rank == 0:
        batched = bench_batched(ctx, args.chains, args.seq_chains, budget)
    if args.requests > 0 and rank == 0:
        serving = bench_serving(args.requests, budget)

    cpu = None
    if rank == 0 and not args.no_cpu:
        cpu = cpu_baseline(flops_apply)

    if rank == 0:
        line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": t_oz / args.steps, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None,
                "dtype": "f64 (FP64 operands as %d exact BF16 slices, FP32-exact accumulation)" % args.slices,
                "data": "synthetic (seeded N(0,1) blocks of the stated shape)", "config": CONFIG,
                "algorithmic_gflop_per_apply": flops_apply / 1e9,
                "split_vs_f64_max_rel_err": rel,
                "f64_path": {"value": f64_value, "unit": UNIT, "ms_per_step": t_64 / n64,
                             "dominant_kernel_ms": d64_ms,
                             "dominant_kernel_tflops": d64_flops / (d64_ms / 1e3) / 1e12,
                             "roofline": f64_roofline},
                "speedup_split_over_f64": value / f64_value,
                "roofline": roofline, "cpu_baseline": cpu, "e2e": e2e, "gpu_launches": launches,
                "clocks": clk, "dmrg_heis20": dmrg, "batched_chains": batched, "serving": serving}
        print(json.dumps(line))
    ctx.close()
    if dist:
        dist.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
