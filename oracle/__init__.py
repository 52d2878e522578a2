"""TEST INFRASTRUCTURE ONLY: the CPU oracle and the reference-kernel harness.

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg import this package.
The solver library never does.
"""
