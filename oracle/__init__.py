"""CPU oracle of the SimpleFluid SPH step — test infrastructure only.

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg may use
this package, and only as the checker.  The product never imports it.
"""
