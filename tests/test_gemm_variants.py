"""Tile-shape variants of the split-precision block GEMM and the autotuner
that picks among them (itg_set_gemm_variant).

Every variant computes each output element in one thread, pair after pair in
the same order, from the same exact digit products, so the variants must
agree bit for bit; the autotuned run must equal them too. Checked on the
isolated H_eff apply (m = 1024 over 31 Sz sectors), whose two large
contractions are tuned on first use.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_variants_bit_identical():
    import itensor_gb300 as itg
    import itensor_gb300.build as b
    from itensor_gb300 import workloads
    b.build()
    ctx = itg.Context(0)
    try:
        wl = workloads.heff_workload(1024, 15, 6.0, 20241204)
        dev = {k: workloads.to_device(ctx, wl[k]) for k in ("psi", "L", "W1", "W2", "R")}
        args = (dev["L"], dev["W1"], dev["W2"], dev["R"], dev["psi"])
        outs = {}
        for v in (-1, 0, 1, 2, 3, 4):
            ctx.set_gemm_variant(v)
            outs[v] = ctx.heff_apply(*args, precision=itg.PREC_OZAKI_BF16).numpy()
        ctx.set_gemm_variant(-1)
        ref = ctx.heff_apply(*args, precision=itg.PREC_F64).numpy()
        for v in (0, 1, 2, 3, 4):
            assert np.array_equal(outs[v], outs[-1]), v
        rel = np.max(np.abs(outs[-1] - ref)) / np.max(np.abs(ref))
        assert rel < 1e-11
    finally:
        ctx.close()


_STUCK = r"""
import sys
sys.path.insert(0, sys.argv[1])
import numpy as np
import itensor_gb300 as itg
from itensor_gb300 import workloads
ctx = itg.Context(0)
wl = workloads.heff_workload(256, 15, 6.0, 7)
dev = {k: workloads.to_device(ctx, wl[k]) for k in ("psi", "L", "W1", "W2", "R")}
args = (dev["L"], dev["W1"], dev["W2"], dev["R"], dev["psi"])
ctx.set_gemm_variant(4)
try:
    ctx.heff_apply(*args, precision=itg.PREC_OZAKI_BF16).numpy()
    print("NO_ERROR")
except itg.ITGError as e:
    print("CODE", e.code)
# the context stays usable: the FP64 path runs and agrees with itself
a = ctx.heff_apply(*args, precision=itg.PREC_F64).numpy()
b = ctx.heff_apply(*args, precision=itg.PREC_F64).numpy()
print("USABLE", bool(np.array_equal(a, b)))
"""


def test_tensor_core_wait_that_runs_out_reports_timeout(tmp_path):
    """Every wait of the tensor-core kernel is bounded: a wait on a barrier
    that nothing arrives at (ITG_TC_TEST_STUCK_WAIT) gives up after the limit
    (ITG_TC_WAIT_LIMIT clocks, ~5 ms here), the kernel frees its tensor memory
    and returns, and the call reports ITG_ERR_TIMEOUT; the context stays
    usable. Run in a child process (the switches are read once per process)."""
    import os
    import subprocess
    import sys
    import itensor_gb300.build as b
    b.build()
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    env = dict(os.environ, ITG_TC_TEST_STUCK_WAIT="1", ITG_TC_WAIT_LIMIT="10000000")
    r = subprocess.run([sys.executable, "-c", _STUCK, root], capture_output=True, text=True, env=env, timeout=300)
    assert r.returncode == 0, r.stderr[-2000:]
    assert "CODE 5" in r.stdout, r.stdout
    assert "USABLE True" in r.stdout, r.stdout
