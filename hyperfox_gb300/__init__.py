"""GB300-native drop-in for HyperFox's HDG element-local path and trace solve.

The compute path is the CUDA library ``_lib/libhfx_gb300.so`` (C ABI in
``include/hfx_gb300.h``); this package holds its ctypes binding, the build
script and the synthetic mesh generator used by the tests and the bench.
"""
from . import meshgen  # noqa: F401

__all__ = ["meshgen", "capi", "build"]
