"""CPU oracle for the two-site DMRG hot path: a numpy restatement of the ITensor
C++ v3 algorithms (block-sparse QN contraction, effective-Hamiltonian apply,
Davidson, density-matrix / SVD bond split, truncation, DMRG sweeps).

TEST INFRASTRUCTURE ONLY. It is imported by ``tests/``, by
``__graft_entry__.smoke()`` and by ``bench.py``'s CPU-baseline / reference arm,
always as the checker. The product path (``itensor_gb300``) never imports it.

Parity pins: every function here is checked against golden fixtures produced by
the reference library itself (``tests/golden/*.json``, generated by
``tests/golden/make_golden.py`` from ``oracle/ref_golden.cc`` linked against the
reference built by ``oracle/Makefile.ref``).
"""
