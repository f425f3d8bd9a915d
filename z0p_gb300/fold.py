"""Folded IVC on the GB300 backend — mirrors z0p::fold (src/fold.rs):
hash-chained Fibonacci segments with one batched FRI.

    params = fold.Params.new(seg_steps, blowup, num_queries, final_size, in_a, in_b, out_b)
    acc = fold.Accumulator(params)
    for col_a, col_b in segments:
        acc.add_segment(col_a, col_b, transcript)
    proof = acc.finalize(transcript)     # IvcProof::to_bytes
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from ._lib import FoldParams, check, lib
from .context import default_context
from .transcript import Transcript

P = 2013265921


class Params(FoldParams):
    """fold::Params (src/fold.rs:42-64)."""

    @classmethod
    def new(cls, seg_steps, blowup, num_queries, final_size, in_a, in_b, out_b) -> "Params":
        p = cls()
        check(lib().z0p_fold_params_new(seg_steps, blowup, num_queries, final_size, in_a % P,
                                        in_b % P, out_b % P, C.byref(p)))
        return p

    @classmethod
    def for_security(cls, seg_steps, in_a, in_b, out_b, target_bits) -> "Params":
        p = cls()
        check(lib().z0p_fold_params_for_security(seg_steps, in_a % P, in_b % P, out_b % P,
                                                 target_bits, C.byref(p)))
        return p

    def with_grinding_bits(self, bits: int) -> "Params":
        self.grinding_bits = bits
        return self

    def with_cap_height(self, height: int) -> "Params":
        self.cap_height = height
        return self


_U32P = C.POINTER(C.c_uint32)


_ARRAY_TYPES = {}


def _u32_column(col):
    """A segment column as 32-bit words: a short list of integers becomes a
    ctypes array directly (a few microseconds less per segment than through
    numpy); anything else goes through numpy, which also raises for values
    outside 32 bits (the C boundary then rejects values >= p)."""
    if isinstance(col, (list, tuple)) and len(col) <= 4096:
        try:
            if not col or (min(col) >= 0 and max(col) < 4294967296):
                t = _ARRAY_TYPES.get(len(col))
                if t is None:
                    t = _ARRAY_TYPES[len(col)] = C.c_uint32 * len(col)
                return t(*col)
        except TypeError:
            pass
    return np.ascontiguousarray(np.asarray(col, dtype=np.uint32))


def _u32_ptr(col):
    return col if isinstance(col, C.Array) else col.ctypes.data_as(_U32P)


class Accumulator:
    """fold::Accumulator (src/fold.rs:362-561); segments stay on the context's device."""

    def __init__(self, params: Params, ctx=None):
        self.ctx = ctx or default_context()
        self.params = params
        self.h = C.c_void_p()
        check(lib().z0p_gpu_fold_create(self.ctx.handle, C.byref(params), C.byref(self.h)))

    def close(self):
        if self.h:
            lib().z0p_gpu_fold_destroy(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __len__(self) -> int:
        return lib().z0p_gpu_fold_len(self.h)

    def add_segment(self, col_a, col_b, transcript: Transcript) -> None:
        a, b = _u32_column(col_a), _u32_column(col_b)
        if len(a) != len(b):
            raise ValueError("segment columns must have one length")
        check(lib().z0p_gpu_fold_add_segment(self.h, _u32_ptr(a), _u32_ptr(b), len(a),
                                             C.byref(transcript.state)))

    def finalize(self, transcript: Transcript) -> bytes:
        n = C.c_size_t()
        check(lib().z0p_gpu_fold_proof_size(self.h, C.byref(n)))
        out = (C.c_uint8 * n.value)()
        got = C.c_size_t()
        check(lib().z0p_gpu_fold_finalize(self.h, C.byref(transcript.state), out, n.value,
                                          C.byref(got)))
        return bytes(out)[: got.value]
