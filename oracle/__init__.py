"""CPU oracle for the Wigner-3j mode-coupling / covariance hot path.

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and the
CPU-baseline leg of bench.py, as the checker.  The product library never
imports or links anything here.
"""
