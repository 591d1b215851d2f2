"""The allocation-free contraction exec (itg_contract_exec_noalloc).

It serves callers that cannot let the library allocate device memory during a
call: a host framework whose allocator owns the whole device pool, a
real-time loop that cannot take an allocation's implicit synchronisation, or a
sandbox that forbids cudaMalloc after start-up. It runs a plan built earlier,
with the split-precision digit panels in one fixed device array.

Checked here through the C-ABI: two calls in a row match the pooled entry point
(itg_contract_exec, same arithmetic) within the split-form tolerance, calls
leave the device's free memory unchanged, and a plan too large for the fixed
array is refused with ITG_ERR_RANGE. Kept in its
own file, collected last; it also passes alone in a fresh process.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

SPLIT_RTOL = 1e-11  # split form (6 BF16 slices), as in the other parity tests


@pytest.fixture(scope="module")
def ctx():
    import itensor_gb300 as itg
    import itensor_gb300.build as b
    b.build()
    c = itg.Context(0)
    c.set_precision(itg.PREC_OZAKI_BF16, 6)
    yield c
    c.close()


def _psi_L_plan(ctx, m):
    """psi(l,s1,s2,r) * L(l,w,l'): the first contraction of the H_eff apply."""
    from itensor_gb300 import workloads
    wl = workloads.heff_workload(m=m, K=15, sigma=6.0, seed=11)
    psi = workloads.to_device(ctx, wl["psi"])
    L = workloads.to_device(ctx, wl["L"])
    dims = lambda t: [I["dims"] for I in t["inds"]]
    # labels: contracted l = -1, the rest positive and distinct
    plan = ctx.plan((dims(wl["psi"]), wl["psi"]["coords"]), [-1, 1, 2, 3],
                    (dims(wl["L"]), wl["L"]["coords"]), [-1, 4, 5])
    return plan, psi, L


def test_noalloc_matches_pooled_exec_twice(ctx):
    import torch
    import itensor_gb300 as itg
    plan, psi, L = _psi_L_plan(ctx, 512)
    _, _, size = plan.output()
    assert size > 0
    ref = torch.empty(size, dtype=torch.float64, device="cuda")
    ref64 = torch.empty(size, dtype=torch.float64, device="cuda")
    ctx.contract_exec(plan, psi.device_ptr(), L.device_ptr(), ref.data_ptr(), precision=itg.PREC_OZAKI_BF16)
    ctx.contract_exec(plan, psi.device_ptr(), L.device_ptr(), ref64.data_ptr(), precision=itg.PREC_F64)
    ctx.sync()
    r = ref.cpu().numpy()
    r64 = ref64.cpu().numpy()
    scale = max(1.0, float(np.max(np.abs(r64))))
    assert np.max(np.abs(r - r64)) <= SPLIT_RTOL * scale  # the pooled split path itself is sound
    for call in range(2):
        out = torch.full((size,), float("nan"), dtype=torch.float64, device="cuda")
        ctx.contract_exec_noalloc(plan, psi.device_ptr(), L.device_ptr(), out.data_ptr(), slices=6)
        ctx.sync()
        o = out.cpu().numpy()
        assert np.all(np.isfinite(o)), call
        assert np.max(np.abs(o - r)) <= SPLIT_RTOL * scale, call


def test_noalloc_calls_allocate_no_device_memory(ctx):
    """The defining property: once the plan exists, calls take no device memory.
    The driver's free-memory count stays put across several calls (a call that
    grew any allocator pool, the library's or torch's, would lower it)."""
    import torch
    plan, psi, L = _psi_L_plan(ctx, 512)
    _, _, size = plan.output()
    out = torch.empty(size, dtype=torch.float64, device="cuda")
    ctx.contract_exec_noalloc(plan, psi.device_ptr(), L.device_ptr(), out.data_ptr(), slices=6)  # set-up call
    ctx.sync()
    torch.cuda.synchronize()
    free0 = torch.cuda.mem_get_info()[0]
    for _ in range(3):
        ctx.contract_exec_noalloc(plan, psi.device_ptr(), L.device_ptr(), out.data_ptr(), slices=6)
    ctx.sync()
    assert torch.cuda.mem_get_info()[0] == free0


def test_noalloc_rejects_plans_beyond_the_fixed_array(ctx):
    import torch
    import itensor_gb300 as itg
    plan, psi, L = _psi_L_plan(ctx, 4096)
    _, _, size = plan.output()
    out = torch.zeros(size, dtype=torch.float64, device="cuda")  # full-size, in case the check were missing
    with pytest.raises(itg.ITGError) as e:
        ctx.contract_exec_noalloc(plan, psi.device_ptr(), L.device_ptr(), out.data_ptr(), slices=6)
    assert e.value.code == 7  # ITG_ERR_RANGE
    assert "scratch" in str(e.value)
