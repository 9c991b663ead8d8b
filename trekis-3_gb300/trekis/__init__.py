"""GB300-native Monte Carlo track loop of TREKIS-3 (host side).

The compute lives in the CUDA library ``_build/libtrekis_gb300.so`` (sources
in ``csrc/``); this package holds the host mirror of the reference's input
objects (``material``), the benchmark workloads (``configs``), the ctypes
binding of the C ABI (``abi``) and the do_Monte_Carlo-style API (``api``).
"""
from . import abi, configs, material  # noqa: F401
