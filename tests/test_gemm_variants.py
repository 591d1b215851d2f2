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
        for v in (-1, 0, 1, 2, 3):
            ctx.set_gemm_variant(v)
            outs[v] = ctx.heff_apply(*args, precision=itg.PREC_OZAKI_BF16).numpy()
        ctx.set_gemm_variant(-1)
        ref = ctx.heff_apply(*args, precision=itg.PREC_F64).numpy()
        for v in (0, 1, 2, 3):
            assert np.array_equal(outs[v], outs[-1]), v
        rel = np.max(np.abs(outs[-1] - ref)) / np.max(np.abs(ref))
        assert rel < 1e-11
    finally:
        ctx.close()
