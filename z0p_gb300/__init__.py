"""GB300-native (sm_103a) proving backend for z0p's STARK prove path.

Drop-in for ``air::prove`` / ``range::prove`` of FutureProofsTech/z0p: the same
parameters, transcript and VERSION=6 proof bytes, computed by CUDA kernels
behind the C ABI in ``include/z0p_gpu.h`` (``libz0p_gpu.so``). There is no CPU
fallback: without the library or a CUDA device every call raises.
"""
from . import air, fold, fri, range, rng, table, tune  # noqa: A004 - mirrors the reference module names
from ._lib import ERRORS, Z0pError, lib
from .context import Context, default_context
from .transcript import Transcript

__all__ = ["air", "fold", "fri", "range", "rng", "table", "tune", "Transcript", "Context", "default_context", "Z0pError", "ERRORS", "lib"]
