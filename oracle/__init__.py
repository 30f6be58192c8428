"""CPU oracle for the ES-PIC hot path: TEST INFRASTRUCTURE ONLY.

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg may
import this package, as the checker.  The product library never calls it.
"""
