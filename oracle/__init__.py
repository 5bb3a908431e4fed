"""CPU oracle for the particle-update path (TEST INFRASTRUCTURE ONLY).

Only tests/, ``__graft_entry__.smoke()`` and bench.py's CPU-baseline leg may
import this package; the product library never does.
"""
