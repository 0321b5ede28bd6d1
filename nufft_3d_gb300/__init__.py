"""GB300-native (sm_103a) implementation of the @nufft_3d hot path.

``nufft_3d`` mirrors the reference MATLAB class; all compute runs in
libnufft3d.so (CUDA, C ABI in include/nufft3d.h).
"""
from ._lib import NufftError, load  # noqa: F401
from .nufft_3d import nufft_3d  # noqa: F401
from .batch import NufftBatch  # noqa: F401

__all__ = ["nufft_3d", "NufftBatch", "NufftError", "load"]
