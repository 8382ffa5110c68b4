"""CPU oracle for the BEM hot path (test infrastructure only).

`oracle.ora` wraps `liboracle.so` (built from `wbem_oracle.cpp` by the
Makefile beside it) through ctypes. Only tests, `__graft_entry__.smoke()` and
the CPU-baseline legs of `bench.py` use it; the product library never does.
"""
from .oracle import *  # noqa: F401,F403
