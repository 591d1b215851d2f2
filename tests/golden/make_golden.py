"""Regenerates the golden fixtures in this folder from the ITensor C++
reference itself.

Builds the reference library from its own sources (oracle/Makefile.ref, which
reads them in place under REF, default /root/reference) together with the
fixture generator oracle/ref_golden.cc, then runs it with one OpenMP thread:

    python tests/golden/make_golden.py [REF]

cylinder.json (the Hubbard 4 x 16 cylinder up to maxdim 800, about 75 s of
the reference on 8 threads) is made by a separate run of the generator, with
the thread count left to OpenMP.

Needs g++ and the BLAS/LAPACK bundled with scipy. The generator fills every
input from a seeded splitmix64 stream and writes inputs and reference outputs
side by side, so the fixtures are self-contained.
"""
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))


def main():
    ref = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("ITENSOR_REFERENCE", "/root/reference")
    subprocess.check_call(["make", "-f", "oracle/Makefile.ref", "-j8", "REF=" + ref], cwd=ROOT)
    env = dict(os.environ, OMP_NUM_THREADS="1")
    subprocess.check_call([os.path.join(ROOT, "oracle/_ref/ref_golden"), os.path.join(ROOT, "tests/golden"), "all"],
                          cwd=ROOT, env=env)
    subprocess.check_call([os.path.join(ROOT, "oracle/_ref/ref_golden"), os.path.join(ROOT, "tests/golden"),
                           "cylinder", "800"], cwd=ROOT)


if __name__ == "__main__":
    main()
