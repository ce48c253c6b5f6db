"""CPU oracle for the PSFUN f(A)x path -- TEST INFRASTRUCTURE ONLY.

Only tests/, __graft_entry__.smoke() and the CPU-baseline leg of bench.py may
import this package.  It wraps the C restatement in psfun_oracle.c (built by
oracle/Makefile) and a few dense SciPy oracles.
"""
