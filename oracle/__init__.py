"""Test infrastructure only: the CPU oracle for the GKR prove path.

``oracle.gkr_oracle.c`` restates the reference prover/verifier in plain C; the
compiled reference itself (``oracle/_ref``) is available where the reference tree
was present at build time.  Only tests, ``__graft_entry__.smoke`` and bench.py's
CPU-baseline arm import this package.
"""
