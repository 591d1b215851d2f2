"""Host-side C++ of the large-block eigensolver (itensor_gb300/csrc/tridiag_ql.cpp),
compiled with the system compiler and run on the CPU: QL eigenpairs, the
lockstep rotation schedules and the kept-vector stage (tests/native)."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_tridiag_ql_and_schedules(tmp_path):
    cxx = shutil.which("g++") or shutil.which("c++")
    if cxx is None:
        pytest.skip("no C++ compiler")
    exe = str(tmp_path / "tridiag_ql_check")
    csrc = os.path.join(ROOT, "itensor_gb300", "csrc")
    subprocess.check_call([cxx, "-O2", "-std=c++17", "-I", csrc, "-o", exe,
                           os.path.join(ROOT, "tests", "native", "tridiag_ql_check.cpp"),
                           os.path.join(csrc, "tridiag_ql.cpp")])
    out = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    assert out.returncode == 0, out.stdout + out.stderr
