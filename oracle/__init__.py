"""CPU oracle for the FIR / rank-filter path (test infrastructure only).

Nothing in the product imports this package; tests, the smoke check and the
benchmark's CPU-baseline leg use it as the checker.
"""
