"""CPU-side checks of the C-ABI library: it loads, exports every symbol that
include/itg.h declares, and its host-only entry point (truncate) reproduces
the reference's decisions bit for bit. No compute call needs a GPU here."""
import os
import re
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared():
    names = set()
    for f in os.listdir(os.path.join(ROOT, "include")):
        if f.endswith(".h"):
            src = open(os.path.join(ROOT, "include", f)).read()
            names |= set(re.findall(r"\b(itg_[a-z0-9_]+)\s*\(", src))
    return names


@pytest.fixture(scope="module")
def built():
    import itensor_gb300.build as b
    return b.build()


def test_library_exports_every_declared_symbol(built):
    out = subprocess.run(["nm", "-D", "--defined-only", built], capture_output=True, text=True, check=True).stdout
    exported = set(re.findall(r"\bT (itg_[a-z0-9_]+)$", out, re.M))
    declared = _declared()
    assert declared, "no declarations found"
    missing = declared - exported
    assert not missing, missing


def test_python_mirror_binds_every_declared_symbol(built):
    import itensor_gb300 as itg
    declared = _declared()
    assert declared <= set(itg.SIGNATURES), declared - set(itg.SIGNATURES)
    L = itg.lib()
    for name in declared:
        assert getattr(L, name) is not None


def test_truncate_through_cabi_bit_exact(built, golden):
    import itensor_gb300 as itg
    for c in golden("truncate")["cases"]:
        P, te, lo, up, nd = itg.truncate(c["P"], c["maxdim"], c["mindim"], c["cutoff"], c["absoluteCutoff"],
                                         c["doRelCutoff"], c["respectDegenerate"])
        assert list(P) == c["Pout"]
        assert (te, lo, up, nd) == (c["truncerr"], c["docut_lower"], c["docut_upper"], c["ndegen"])


def test_context_needs_a_gpu_and_fails_loudly(built):
    torch = pytest.importorskip("torch")
    if torch.cuda.is_available():
        pytest.skip("GPU present")
    import itensor_gb300 as itg
    with pytest.raises(itg.ITGError):
        itg.Context(0)
