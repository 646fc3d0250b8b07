"""GB300-native explicit finite-volume time step of libFastMesh.

The device path lives in ``liblfm_gpu.so`` (sm_103a CUDA kernels behind the C
ABI of include/lfm_gpu.h, with the OpenFOAM-free case plugins). This package
holds its ctypes binding (``_native``), the synthetic case generators
(``cases``) and the build recipe (``build``).
"""
from . import cases  # noqa: F401

__all__ = ["cases"]
__version__ = "0.1"
