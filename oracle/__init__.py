"""CPU oracle of the hydrodynamic wrench path -- TEST INFRASTRUCTURE ONLY.

Loaded by the tests, by ``__graft_entry__.smoke()`` and by the CPU-baseline
leg of ``bench.py``.  The product library never imports it.
"""
from .oracle import (  # noqa: F401
    REF32, REF64, MIRROR64, MIRROR32, T_N, Oracle, build_oracle, oracle_lib_path,
)
