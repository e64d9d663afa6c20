"""GB300-native AMOEBA mutual-polarization path (Tinker9 induce/dfield/ufield,
PME, PCG, epolar/empole) behind a C ABI.

Import with ``importlib.import_module("tinker-gpu_gb300")`` (the directory
name carries a dash).  The compute path lives in the CUDA library built from
``csrc/``; ``abi`` loads it and raises if it is missing.
"""
from . import topology, systems, units  # noqa: F401
