"""GB300 implementation of the PGURE-SVT denoising path.

The compute runs in libpgsvt.so (hand-written sm_103a CUDA behind the C ABI
of include/pgsvt.h); this package holds its ctypes binding, the ``SVT``
estimator with the reference's Python parameters, and synthetic workloads.
"""
from . import _capi, learned, shard, synth
from ._capi import (COMPAT_ALL, COMPAT_INT_DELTA1, COMPAT_SWAP_MU_SIGMA, COMPAT_ZERO_MOTION,
                    PgsvtError)
from .svt import SVT
from .synth import mixed_noise_model

__all__ = ["SVT", "mixed_noise_model", "PgsvtError", "COMPAT_ALL", "COMPAT_SWAP_MU_SIGMA",
           "COMPAT_ZERO_MOTION", "COMPAT_INT_DELTA1", "_capi", "learned"]
__version__ = "0.1.0"
