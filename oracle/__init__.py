"""CPU oracle for the compressible RHS + SSP-RK path (test infrastructure only).

Only tests/, the smoke check in __graft_entry__.py and bench.py's CPU
baseline / reference arm may import this package.  The GPU product never
imports it.
"""
