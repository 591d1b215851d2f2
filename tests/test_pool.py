"""Solver pool (itg_pool_*): many ground-state solves on one GPU with
continuous batching and admission by device-memory estimate.

The central property: a request's result is the same when it runs alone
(itg_dmrg_run on its own context) and when it runs in a mix with others that
overlap it on the device. Kernels are deterministic and solves share nothing
but read-only contraction plans, so the energies and kept dimensions are
compared exactly (the stated tolerance is 0 for dimensions and 1e-12 for
energies, which in practice are bit-identical).

CPU cases (no GPU needed): the memory estimate the pool admits by, and that
creating a pool without a GPU fails with an error code instead of running
anything on the host.
"""
import numpy as np
import pytest

import itensor_gb300 as itg

MIX_ENERGY_TOL = 1e-12

SW_SMALL = [dict(maxdim=m, mindim=1, cutoff=1e-10, niter=2) for m in (8, 16, 32, 32)]

# requests of the serving mix: XXZ chains (Sz QN) and transverse-field Ising chains (parity QN)
MIX = [
    (dict(type=0, N=12, J=1.0, Jz=0.4), SW_SMALL, 0),
    (dict(type=1, N=14, h=0.8), SW_SMALL, 0),
    (dict(type=0, N=16, J=1.0, Jz=1.7), SW_SMALL, 1),
    (dict(type=0, N=10, J=1.0, Jz=1.0, J2=0.3), SW_SMALL, 0),
    (dict(type=1, N=12, h=1.3), SW_SMALL, 1),
    (dict(type=0, N=14, J=1.0, Jz=0.0), SW_SMALL, 0),
]


def test_estimate_grows_with_size():
    sw = [dict(maxdim=64, cutoff=1e-10)]
    e16 = itg.pool_estimate(dict(type=0, N=16), sw)
    e64 = itg.pool_estimate(dict(type=0, N=64), sw)
    e64m = itg.pool_estimate(dict(type=0, N=64), [dict(maxdim=256, cutoff=1e-10)])
    assert 0 < e16 < e64 < e64m
    # the split form adds its digit panels
    assert itg.pool_estimate(dict(type=0, N=64), sw, 1) > e64
    # next-neighbour couplings widen the MPO (bond dimension 8 instead of 5)
    assert itg.pool_estimate(dict(type=0, N=64, J2=0.3), sw) > e64


def test_estimate_bounds_dense_mps():
    # the MPS alone at full bond dimension: N tensors of at most m*d*m FP64 entries
    N, m = 40, 128
    est = itg.pool_estimate(dict(type=1, N=N, h=1.0), [dict(maxdim=m, cutoff=1e-10)])
    assert est >= 8 * (N - 2 * 7) * m * 2 * m


def test_pool_needs_gpu_on_cpu_host():
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    with pytest.raises(itg.ITGError):
        itg.Pool(0, workers=1, slots_per_worker=1)


@pytest.fixture(scope="module")
def ctx():
    import itensor_gb300.build as b
    b.build()
    c = itg.Context(0)
    yield c
    c.close()


@pytest.mark.gpu
def test_split_dmrg_in_fresh_context(golden):
    """Split-precision DMRG from a fresh context, twice (no earlier FP64 run
    warms the plan cache or the memory pool)."""
    c = [x for x in golden("dmrg")["cases"] if x["name"] == "heis20"][0]
    ctx = itg.Context(0)
    try:
        for _ in range(2):
            res = ctx.dmrg(dict(type=0, N=20, J=1.0, Jz=1.0), c["sweeps"], precision=1)
            assert abs(res.energy - c["energy"]) <= 1e-9
    finally:
        ctx.close()


@pytest.mark.gpu
def test_pool_mix_matches_alone(ctx):
    alone = [ctx.dmrg(m, sw, precision=p) for m, sw, p in MIX]
    pool = itg.Pool(0, workers=2, slots_per_worker=3, budget_bytes=8 << 30)
    try:
        ids = [pool.submit(m, sw, p) for m, sw, p in MIX]
        pool.start()
        pool.drain()
        st = pool.stats()
        assert st["done"] == len(MIX) and st["failed"] == 0
        assert st["peak_running"] >= 2          # the solves overlapped
        for i, ref in zip(ids, alone):
            r = pool.result(i)
            assert abs(r.energy - ref.energy) <= MIX_ENERGY_TOL, (i, r.energy, ref.energy)
            assert [b[5] for b in r.bonds] == [b[5] for b in ref.bonds]
            assert [b[4] for b in r.bonds] == pytest.approx([b[4] for b in ref.bonds], abs=1e-14)
            rec = pool.record(i)
            assert rec.status == 0
            assert 0 < rec.peak_bytes <= rec.est_bytes
            assert rec.t_arrive <= rec.t_admit <= rec.t_done
    finally:
        pool.close()


@pytest.mark.gpu
def test_pool_admission_and_arrivals(ctx):
    sw = SW_SMALL
    models = [dict(type=0, N=12 + 2 * (k % 3), Jz=0.5 + 0.25 * k) for k in range(8)]
    est = max(itg.pool_estimate(m, sw) for m in models)
    budget = int(2.5 * est)  # at most two of these fit at once
    pool = itg.Pool(0, workers=2, slots_per_worker=4, budget_bytes=budget)
    try:
        pool.start()
        ids = [pool.submit(m, sw, 0, arrival=0.02 * k) for k, m in enumerate(models)]
        big = pool.submit(dict(type=0, N=64), [dict(maxdim=4096, cutoff=1e-12)], 0)
        pool.drain()
        st = pool.stats()
        assert st["done"] == len(models) and st["failed"] == 1
        assert st["peak_reserved_bytes"] <= budget
        assert st["peak_running"] <= 2
        bad = pool.record(big)
        assert bad.status == 7 and "budget" in bad.error
        for k, i in enumerate(ids):
            rec = pool.record(i)
            assert rec.status == 0
            assert rec.t_arrive >= 0.02 * k - 1e-9
            assert rec.t_admit >= rec.t_arrive
            ref = ctx.dmrg(models[k], sw, precision=0)
            assert abs(rec.energy - ref.energy) <= MIX_ENERGY_TOL
    finally:
        pool.close()


@pytest.mark.gpu
def test_grouped_launches_across_solves_change_nothing():
    """Cross-solve grouping: with several solves on one worker, their
    split-precision contractions run as grouped launches (one prep and one
    GEMM launch covering every solve's blocks). Results are bit-identical to
    the pool without grouping, and the groups do carry several solves each."""
    reqs = [(dict(type=0, N=n, J=1.0, Jz=jz), SW_SMALL) for n, jz in ((14, 0.5), (16, 1.0), (12, 1.5), (18, 0.8),
                                                                     (16, 0.2), (14, 1.2))]
    runs = {}
    for grouping in (False, True):
        pool = itg.Pool(0, workers=1, slots_per_worker=len(reqs), budget_bytes=8 << 30, grouping=grouping)
        try:
            ids = [pool.submit(m, sw, itg.PREC_OZAKI_BF16) for m, sw in reqs]
            pool.start()
            pool.drain()
            runs[grouping] = [pool.result(i) for i in ids]
            launches, contractions = pool.grouping_stats()
        finally:
            pool.close()
        if grouping:
            assert launches > 0 and contractions > launches / 2, (launches, contractions)
        else:
            assert launches == 0
    for a, b in zip(runs[False], runs[True]):
        assert a.energy == b.energy
        assert [x[3:] for x in a.bonds] == [x[3:] for x in b.bonds]


@pytest.mark.gpu
def test_calibrated_admission_packs_more_solves(ctx):
    """Calibrated admission: with a budget that the dense estimate fills with
    one solve, the first two solves of the family run one at a time; after
    them the family is admitted by 2 x its measured peak/estimate ratio and
    several run at once. Results stay identical to lone runs, and no solve
    needs more than it was admitted by."""
    # estimates of ~48 MiB, above the 16 MiB floor of a calibrated admission
    sw = [dict(maxdim=m, mindim=1, cutoff=1e-10, niter=2) for m in (32, 64, 128, 128)]
    models = [dict(type=0, N=32, J=1.0, Jz=0.6 + 0.1 * k) for k in range(10)]
    est = max(itg.pool_estimate(m, sw) for m in models)
    assert est > 32 << 20
    pool = itg.Pool(0, workers=2, slots_per_worker=4, budget_bytes=int(1.5 * est))
    pool.set_calibration(2, 2.0)
    try:
        ids = [pool.submit(m, sw, 0) for m in models]
        pool.start()
        pool.drain()
        st = pool.stats()
        assert st["done"] == len(models) and st["failed"] == 0
        calibrated, retried = pool.calibration_stats()
        assert calibrated >= len(models) - 2 and retried == 0
        assert st["peak_running"] >= 2
        assert st["peak_reserved_bytes"] <= int(1.5 * est)
        for k, i in enumerate(ids):
            rec = pool.record(i)
            adm, reruns = pool.admission(i)
            assert rec.status == 0 and reruns == 0
            assert 0 < rec.peak_bytes <= adm <= rec.est_bytes
            ref = ctx.dmrg(models[k], sw, precision=0)
            assert abs(rec.energy - ref.energy) <= MIX_ENERGY_TOL
    finally:
        pool.close()
