"""dmrg() on a caller's own MPO and initial MPS, and checkpoints, through the
C-ABI on the GPU.

- itg_dmrg_run_mpo with the reference's own MPO tensors (sample/Heisenberg.h
  for the N=20 chain, toMPO for the 4x2 Hubbard ladder) and MPS(InitState)
  tensors, against the run the reference made from them: per-bond energies
  1e-10, truncation errors 1e-12, kept dimensions and link layouts exact. The
  MPS that comes back has the result's energy (oracle contraction, 1e-8: the
  last bond's truncation follows the recorded Davidson energy).
- A DMRG resumed from the reference's binary checkpoint (MPO and MPS written
  by writeToFile) matches the reference's own continued run; the result,
  stored and written in the same layout, reads back unchanged, with the
  reference's link tags carried onto the new links.
- Solver-pool requests on the caller's MPO give the lone run's result exactly.
"""
import os

import numpy as np
import pytest

from helpers import T, check_dmrg_record, device_to_oracle, gpu_tensor, mps_energy, qn_names
import mps_file

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = os.path.join(ROOT, "tests", "golden")


@pytest.fixture(scope="module")
def ctx():
    import itensor_gb300 as itg
    import itensor_gb300.build as b
    b.build()
    c = itg.Context(0)
    yield c
    c.close()


def _mpo_case(golden, name):
    d = golden("mpo_io")
    return [x for x in d["cases"] if x["run"]["name"] == name][0], qn_names(d)


@pytest.mark.parametrize("name", ["heis20", "hubbard4x2"])
def test_dmrg_on_the_reference_mpo_and_mps(ctx, golden, name):
    c, names = _mpo_case(golden, name)
    W = [gpu_tensor(ctx, j, names) for j in c["W"]]
    psi0 = [gpu_tensor(ctx, j, names) for j in c["psi0"]]
    res = ctx.dmrg_mpo(W, psi0, c["run"]["sweeps"], precision=0)
    check_dmrg_record(res, c["run"], names)
    E = mps_energy([device_to_oracle(t, names) for t in res.mps], [T(j) for j in c["W"]])
    assert abs(E - res.energy) < 1e-8


def test_dmrg_on_the_reference_mpo_split_precision(ctx, golden):
    c, names = _mpo_case(golden, "heis20")
    W = [gpu_tensor(ctx, j, names) for j in c["W"]]
    psi0 = [gpu_tensor(ctx, j, names) for j in c["psi0"]]
    res = ctx.dmrg_mpo(W, psi0, c["run"]["sweeps"], precision=1)
    assert abs(res.energy - c["run"]["energy"]) <= 1e-9


def test_dmrg_on_a_sum_of_the_callers_mpos(ctx, golden):
    """nmpo = 2: H + H acts as 2H, so every Davidson energy doubles while the
    states (kept dims, truncation) follow the single-MPO run."""
    c, names = _mpo_case(golden, "heis20")
    W = [gpu_tensor(ctx, j, names) for j in c["W"]]
    psi0 = [gpu_tensor(ctx, j, names) for j in c["psi0"]]
    res = ctx.dmrg_mpo(W, psi0, c["run"]["sweeps"], precision=0, more=[W])
    assert abs(res.energy - 2 * c["run"]["energy"]) < 2e-10
    for a, b in zip(res.bonds, c["run"]["bonds"]):
        assert a[5] == b[5]


@pytest.mark.parametrize("name", ["heis12", "hubbard4x2"])
def test_dmrg_resumes_from_a_reference_checkpoint(ctx, golden, tmp_path, name):
    c = [x for x in golden("checkpoint")["cases"] if x["name"] == name][0]
    W, winfo = ctx.mps_load(os.path.join(GOLDEN, c["mpo"]))
    psi, info = ctx.mps_load(os.path.join(GOLDEN, c["start"]))
    names = info["qn_names"]
    assert [info["leftlim"], info["rightlim"]] == c["start_lims"]
    res = ctx.dmrg_mpo(W, psi, c["sweeps"], precision=0)
    check_dmrg_record(res, c, names)
    # checkpoint the result and read it back: same structure, same numbers
    lims = c["final_lims"]
    out = tmp_path / (name + "_ours.mps")
    ctx.mps_store(res.mps, lims[0], lims[1], names).write(out)
    back, binfo = ctx.mps_load(out)
    assert [binfo["leftlim"], binfo["rightlim"]] == lims and binfo["qn_names"] == names
    for a, b in zip(res.mps, back):
        ca, oa = a.blocks()
        cb, ob = b.blocks()
        assert np.array_equal(ca, cb) and np.array_equal(oa, ob)
        assert [(I.id, I.plev, I.dir) for I in a.inds] == [(I.id, I.plev, I.dir) for I in b.inds]
        assert np.array_equal(a.numpy(), b.numpy())
    # the new links carry the reference's link tags ("Link", "l=<b>")
    sites, _, _ = mps_file.read(str(out))
    for j in range(len(sites) - 1):
        ids = {I["id"] for I in sites[j + 1]["inds"]}
        link = [I for I in sites[j]["inds"] if I["id"] in ids][0]
        assert set(link["tags"].split(",")) == set(c["links"][j]["tags"].split(",")), (j, link["tags"])
    # the written state's energy (independent reader + oracle) is the run's
    Wf, _, _ = mps_file.read(os.path.join(GOLDEN, c["mpo"]))
    assert abs(mps_energy([T(x) for x in sites], [T(x) for x in Wf]) - res.energy) < 1e-8


def test_pool_requests_on_the_callers_mpo_match_the_lone_run(ctx, golden):
    import itensor_gb300 as itg
    c, names = _mpo_case(golden, "hubbard4x2")
    W = [gpu_tensor(ctx, j, names) for j in c["W"]]
    psi0 = [gpu_tensor(ctx, j, names) for j in c["psi0"]]
    sweeps = c["run"]["sweeps"]
    lone = ctx.dmrg_mpo(W, psi0, sweeps, precision=0)
    pool = itg.Pool(0, workers=2, slots_per_worker=2, budget_bytes=8 << 30)
    try:
        ids = [pool.submit_mpo(ctx, W, psi0, sweeps, precision=0, keep_mps=(k == 0)) for k in range(3)]
        other = pool.submit(dict(type=0, N=16, J=1.0, Jz=0.5), [dict(maxdim=32, cutoff=1e-10, niter=2)] * 3)
        pool.start()
        pool.drain()
        assert pool.record(other).status == 0
        for k, i in enumerate(ids):
            rec = pool.record(i)
            assert rec.status == 0, rec.error
            r = pool.result(i, ctx=ctx if k == 0 else None)
            assert r.energy == lone.energy
            assert [b[3:] for b in r.bonds] == [b[3:] for b in lone.bonds]
            if k == 0:
                for a, b in zip(r.mps, lone.mps):
                    assert np.array_equal(a.numpy(), b.numpy())
    finally:
        pool.close()
