"""GB300-native Newton-load engine for SPICE-class transient simulation.

The compute path is libxg.so (CUDA, sm_103a) behind the C ABI in
include/xg.h; `engine` is the Python host API over it, `abi` the shared
struct definitions, `netlists` seeded workload generators.
"""
from . import abi  # noqa: F401

__all__ = ["abi"]
