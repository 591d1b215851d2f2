"""The benchmark configurations themselves, pinned to the oracle and to the
reference (GPU, through the C-ABI).

- The isolated H_eff apply at the benchmark's size (m = 1024 over 31 Sz
  sectors, Gaussian sizes sigma = 6, N(0,1) blocks, Heisenberg MPO; the same
  bytes the benchmark times) against the oracle's LocalOp::product: exact
  output block list and offsets, values within 1e-12 (FP64) and 1e-11 (split
  precision, 6 BF16 slices) relative to the largest entry.
- The same layout at m = 256 against the reference's own LocalOp::product
  (itensor/mps/localop.h:324-365) on its own inputs (heff_config.json).
- The Hubbard model on the 4 x 16 cylinder (t=1, U=4, half filling, (Nf, Sz)
  QN) against the reference's DMRG on the sample's sweep table up to the
  fixture's maxdim, cutoff 1e-9, no noise (cylinder.json): every bond step's
  energy within 1e-9 relative to |E| (64 sites, energies ~ -54), truncation
  errors 1e-10, kept dimensions and final link layouts exact.
"""
import numpy as np
import pytest

from helpers import (bst_json, check_dmrg_record, gpu_layout_matches, gpu_tensor, qn_names, workload_to_oracle)

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    import itensor_gb300 as itg
    import itensor_gb300.build as b
    b.build()
    c = itg.Context(0)
    yield c
    c.close()


def _relerr(x, ref):
    ref = np.asarray(ref, np.float64)
    return float(np.max(np.abs(np.asarray(x) - ref)) / max(1.0, np.max(np.abs(ref))))


def test_heff_benchmark_size_matches_the_oracle(ctx):
    from itensor_gb300 import workloads
    from oracle.dmrg import LocalOp
    wl = workloads.heff_workload(1024, 15, 6.0, 20241204)   # the benchmark's bytes
    assert wl["nsect"] == 31
    dev = {k: workloads.to_device(ctx, wl[k]) for k in ("psi", "L", "W1", "W2", "R")}
    o = {k: workload_to_oracle(wl[k]) for k in ("psi", "L", "W1", "W2", "R")}
    ref = bst_json(LocalOp(o["W1"], o["W2"], o["L"], o["R"]).product(o["psi"]))
    for prec, tol in ((0, 1e-12), (1, 1e-11)):
        out = ctx.heff_apply(dev["L"], dev["W1"], dev["W2"], dev["R"], dev["psi"], precision=prec)
        same_inds, same_blocks = gpu_layout_matches(out, ref)
        assert same_inds and same_blocks, prec
        assert _relerr(out.numpy(), ref["data"]) <= tol, prec


@pytest.mark.parametrize("prec", [0, 1])
def test_prepared_apply_matches_the_plain_call(ctx, prec):
    """The prepared, graph-replayed apply the benchmark times (itg_heff_create /
    itg_heff_run: the two MPO tensors contracted with each other once, one MPO
    step per apply) against itg_heff_apply (the reference's four-step chain),
    on the benchmark's bytes: same structure, values within the tolerance."""
    import torch
    from itensor_gb300 import workloads
    wl = workloads.heff_workload(1024, 15, 6.0, 20241204)
    dev = {k: workloads.to_device(ctx, wl[k]) for k in ("psi", "L", "W1", "W2", "R")}
    args = (dev["L"], dev["W1"], dev["W2"], dev["R"], dev["psi"])
    ref = ctx.heff_apply(*args, precision=0).numpy()
    for graph in (False, True):
        h = ctx.heff_prepare(*args, precision=prec, use_graph=graph)
        assert h.out_size == ref.size
        out = torch.empty(h.out_size, dtype=torch.float64, device="cuda")
        for _ in range(2):
            h.run(dev["psi"].device_ptr(), out.data_ptr())
        ctx.sync()
        assert _relerr(out.cpu().numpy(), ref) <= (1e-12 if prec == 0 else 1e-11), graph


def test_prepared_apply_host_buffers(ctx):
    """itg_heff_run with host buffers: page-locked ones (read and written by the
    copy kernel through their device addresses) and pageable ones (copy-engine
    transfers) give the device-pointer run's output, bit for bit."""
    import ctypes as C
    import torch
    import itensor_gb300 as itg
    from itensor_gb300 import workloads
    wl = workloads.heff_workload(256, 11, 4.0, 7)
    dev = {k: workloads.to_device(ctx, wl[k]) for k in ("psi", "L", "W1", "W2", "R")}
    h = ctx.heff_prepare(dev["L"], dev["W1"], dev["W2"], dev["R"], dev["psi"], precision=0, use_graph=True)
    out = torch.empty(h.out_size, dtype=torch.float64, device="cuda")
    h.run(dev["psi"].device_ptr(), out.data_ptr())
    ctx.sync()
    want = out.cpu().numpy()
    psi_host = dev["psi"].numpy()
    pin_in = torch.from_numpy(psi_host.copy()).pin_memory()
    pin_out = torch.full((h.out_size,), float("nan"), dtype=torch.float64).pin_memory()
    for _ in range(2):
        ctx._ok(itg.lib().itg_heff_run(ctx.h, h.h, C.c_void_p(pin_in.data_ptr()), C.c_void_p(pin_out.data_ptr()), 1),
                ctx.h)
        assert np.array_equal(pin_out.numpy(), want)
    got = h.run_host(psi_host)
    assert np.array_equal(got, want)


@pytest.mark.parametrize("prec", [0, 1])
def test_heff_benchmark_layout_matches_the_reference(ctx, golden, prec):
    d = golden("heff_config")
    names = qn_names(d)
    c = d["cases"][0]
    L, W1, W2, R, phi = (gpu_tensor(ctx, c[k], names) for k in ("L", "W1", "W2", "R", "phi"))
    out = ctx.heff_apply(L, W1, W2, R, phi, precision=prec)
    same_inds, same_blocks = gpu_layout_matches(out, c["Hphi"])
    assert same_inds and same_blocks
    assert _relerr(out.numpy(), c["Hphi"]["data"]) <= (1e-12 if prec == 0 else 1e-11)


def test_hubbard_cylinder_matches_the_reference(ctx, golden):
    d = golden("cylinder")
    c = d["cases"][0]
    m = c["model"]
    res = ctx.dmrg(dict(type=2, Lx=m["Lx"], Ly=m["Ly"], t=m["t"], U=m["U"], yperiodic=int(m["yperiodic"])),
                   c["sweeps"], precision=0)
    tol = 1e-9 * abs(c["energy"])
    check_dmrg_record(res, c, ["Nf", "Sz"], energy_tol=tol, trunc_tol=1e-10)
