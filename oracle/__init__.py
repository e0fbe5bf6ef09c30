"""CPU oracle for the renderer's hot path (test infrastructure only).

Only tests/, __graft_entry__.smoke() and the CPU-baseline leg of bench.py use
this package, as the checker.  The product path never imports it.
"""
