"""CPU oracle for the rans residual path — test infrastructure only.

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg load
this package, and only as the checker.  Parity status: unpinned (the
reference ships no golden vectors and cannot be built without Eigen).
"""
