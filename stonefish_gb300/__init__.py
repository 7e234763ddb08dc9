"""GB300-native geometry-based hydrodynamics for Stonefish bodies.

The package wraps the C ABI of ``include/stonefish_hydro.h`` (library built
from ``stonefish_gb300/csrc``) and provides the mesh builders and seeded
workloads used by the tests and the benchmark.
"""
__version__ = "0.1.0"
