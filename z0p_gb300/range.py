"""Range-check AIR on the GB300 backend — mirrors z0p::range (src/range.rs)."""
from __future__ import annotations

import ctypes as C

from ._lib import RangeParams, TranscriptState, check, lib
from .context import default_context
from .transcript import Transcript

P = 2013265921


class Params(RangeParams):
    """range::Params (src/range.rs:30-51)."""

    @classmethod
    def new(cls, n_rows, n_bits, blowup, num_queries, final_size, value) -> "Params":
        p = cls()
        check(lib().z0p_range_params_new(n_rows, n_bits, blowup, num_queries, final_size,
                                         value % P, C.byref(p)))
        return p

    @classmethod
    def for_security(cls, n_rows, n_bits, value, target_bits) -> "Params":
        p = cls()
        check(lib().z0p_range_params_for_security(n_rows, n_bits, value % P, target_bits,
                                                  C.byref(p)))
        return p

    def with_grinding_bits(self, bits: int) -> "Params":
        self.grinding_bits = bits
        return self

    def with_cap_height(self, height: int) -> "Params":
        self.cap_height = height
        return self

    def lde_len(self) -> int:
        return self.n_rows * self.blowup

    def n_columns(self) -> int:
        return self.n_bits + 1

    def proof_size(self) -> int:
        n = C.c_size_t()
        check(lib().z0p_range_proof_size(C.byref(self), C.byref(n)))
        return n.value

    def footprint(self) -> int:
        n = C.c_size_t()
        check(lib().z0p_gpu_range_footprint(C.byref(self), C.byref(n)))
        return n.value


def prove(params: Params, transcript: Transcript, ctx=None) -> bytes:
    """range::prove + Proof::to_bytes (src/range.rs:337-343, 253-269) on the GPU."""
    ctx = ctx or default_context()
    size = params.proof_size()
    buf = (C.c_uint8 * size)()
    n = C.c_size_t()
    check(lib().z0p_gpu_range_prove(ctx.handle, C.byref(params), C.byref(transcript.state), buf,
                                    size, C.byref(n)))
    return bytes(buf)[: n.value]


def prove_zk(params: Params, n_rand: int, rng, transcript: Transcript, ctx=None) -> bytes:
    """range::prove_zk (src/range.rs:393-418): `rng` is a z0p_gb300.rng.ChaCha20."""
    ctx = ctx or default_context()
    n = C.c_size_t()
    check(lib().z0p_range_proof_size_zk(C.byref(params), n_rand, C.byref(n)))
    out = (C.c_uint8 * n.value)()
    check(lib().z0p_gpu_range_prove_zk(ctx.handle, C.byref(params), n_rand, C.byref(rng),
                                       C.byref(transcript.state), out, n.value, C.byref(n)))
    return bytes(out)[: n.value]


def prove_with_columns(params: Params, v_col, bit_cols, transcript: Transcript, ctx=None) -> bytes:
    """range::prove_with_columns (src/range.rs:353-375): the caller's value
    column and n_bits bit columns, proved row by row on the device."""
    import numpy as np

    ctx = ctx or default_context()
    v = np.ascontiguousarray(np.asarray(v_col, dtype=np.uint32))
    bits = [np.ascontiguousarray(np.asarray(b, dtype=np.uint32)) for b in bit_cols]
    ptrs = (C.POINTER(C.c_uint32) * max(1, len(bits)))(
        *[b.ctypes.data_as(C.POINTER(C.c_uint32)) for b in bits])
    lens = (C.c_size_t * max(1, len(bits)))(*[b.size for b in bits])
    n = C.c_size_t()
    rc = lib().z0p_gpu_range_prove_with_columns(ctx.handle, C.byref(params),
                                                v.ctypes.data_as(C.POINTER(C.c_uint32)), v.size, ptrs,
                                                lens, len(bits), C.byref(transcript.state), None, 0,
                                                C.byref(n))
    if rc != 100:  # Z0P_ERR_BUFFER_TOO_SMALL reports the size; anything else is the answer
        check(rc)
    size = n.value
    buf = (C.c_uint8 * size)()
    check(lib().z0p_gpu_range_prove_with_columns(ctx.handle, C.byref(params),
                                                 v.ctypes.data_as(C.POINTER(C.c_uint32)), v.size,
                                                 ptrs, lens, len(bits), C.byref(transcript.state),
                                                 buf, size, C.byref(n)))
    return bytes(buf)[: n.value]


def prove_group(params_list, transcripts, ctx=None):
    """Proves statements of one shape in lockstep (one launch sequence and one
    set of host round trips for the group); proof i equals prove(params_list[i],
    transcripts[i]) alone, and each transcript advances the same way."""
    ctx = ctx or default_context()
    n = len(params_list)
    if n != len(transcripts) or n == 0:
        raise ValueError("one transcript per statement, at least one statement")
    arr = (Params * n)(*params_list)
    size = params_list[0].proof_size()
    bufs = [(C.c_uint8 * size)() for _ in range(n)]
    outs = (C.POINTER(C.c_uint8) * n)(*[C.cast(b, C.POINTER(C.c_uint8)) for b in bufs])
    caps = (C.c_size_t * n)(*([size] * n))
    lens = (C.c_size_t * n)()
    states = (C.POINTER(TranscriptState) * n)(*[C.pointer(t.state) for t in transcripts])
    check(lib().z0p_gpu_range_prove_group(ctx.handle, n, arr, states, outs, caps, lens))
    return [bytes(b)[: lens[i]] for i, b in enumerate(bufs)]
