"""CPU oracle of the nsmp3D hot path (test infrastructure only).

Only tests/, __graft_entry__.smoke() (as the checker) and bench.py's CPU
baseline leg import this package.  The product library never does.
"""
