"""TEST INFRASTRUCTURE ONLY: the CPU oracle of the 2DENSE hot path.

``dense_oracle.cpp`` restates the reference Fortran solver line by line; ``oracle.py`` loads it
through ctypes. Only the tests, ``__graft_entry__.smoke()`` and bench.py's CPU-baseline leg may
use this package, and only as the checker or the timed CPU baseline. The product path never
imports it.
"""
