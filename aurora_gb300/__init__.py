"""aurora_gb300: a GB300-native (sm_103a) path-tracing backend for Autodesk Aurora.

The compute path is libagb_cuda.so (aurora_gb300/csrc, C ABI in include/agb.h): hand-written CUDA
kernels for BVH traversal, Standard Surface shading, environment importance sampling and
accumulation.  This package is the Python host side: build, the ctypes binding, seeded scene
generators and a thin renderer object.
"""
from . import _abi  # noqa: F401
from ._abi import AgbError, library  # noqa: F401

__all__ = ["AgbError", "library", "api", "scenes", "build"]
