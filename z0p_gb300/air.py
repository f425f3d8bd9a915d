"""Fibonacci AIR on the GB300 backend — mirrors z0p::air (src/air.rs).

    params = air.Params.for_security(n_steps, a0, b0, b_last, 100)
    proof = air.prove(params, transcript)   # VERSION=6 bytes, air::Proof::to_bytes
"""
from __future__ import annotations

import ctypes as C

from ._lib import AirParams, TranscriptState, check, lib
from .context import default_context
from .transcript import Transcript

P = 2013265921


class Params(AirParams):
    """air::Params (src/air.rs:31-54)."""

    @classmethod
    def new(cls, n_steps, blowup, num_queries, final_size, a0, b0, b_last) -> "Params":
        p = cls()
        check(lib().z0p_air_params_new(n_steps, blowup, num_queries, final_size, a0 % P, b0 % P,
                                       b_last % P, C.byref(p)))
        return p

    @classmethod
    def for_security(cls, n_steps, a0, b0, b_last, target_bits) -> "Params":
        p = cls()
        check(lib().z0p_air_params_for_security(n_steps, a0 % P, b0 % P, b_last % P, target_bits,
                                                C.byref(p)))
        return p

    def with_grinding_bits(self, bits: int) -> "Params":
        self.grinding_bits = bits
        return self

    def with_cap_height(self, height: int) -> "Params":
        self.cap_height = height
        return self

    def lde_len(self) -> int:
        return self.n_steps * self.blowup

    def proof_size(self) -> int:
        n = C.c_size_t()
        check(lib().z0p_air_proof_size(C.byref(self), C.byref(n)))
        return n.value

    def footprint(self) -> int:
        n = C.c_size_t()
        check(lib().z0p_gpu_air_footprint(C.byref(self), C.byref(n)))
        return n.value

    def __repr__(self):
        return (f"air.Params(n_steps={self.n_steps}, blowup={self.blowup}, "
                f"num_queries={self.num_queries}, final_size={self.final_size}, "
                f"grinding_bits={self.grinding_bits}, cap_height={self.cap_height}, "
                f"a0={self.a0}, b0={self.b0}, b_last={self.b_last})")


def trace_last(a0: int, b0: int, n_steps: int):
    """(A[n-1], B[n-1]) of build_trace (src/air.rs:341-354) by 2x2 matrix powers."""
    def mul(x, y):
        return [[(x[0][0] * y[0][0] + x[0][1] * y[1][0]) % P, (x[0][0] * y[0][1] + x[0][1] * y[1][1]) % P],
                [(x[1][0] * y[0][0] + x[1][1] * y[1][0]) % P, (x[1][0] * y[0][1] + x[1][1] * y[1][1]) % P]]

    r, m, e = [[1, 0], [0, 1]], [[0, 1], [1, 1]], n_steps - 1
    while e > 0:
        if e & 1:
            r = mul(r, m)
        m = mul(m, m)
        e >>= 1
    return (r[0][0] * a0 + r[0][1] * b0) % P, (r[1][0] * a0 + r[1][1] * b0) % P


def prove(params: Params, transcript: Transcript, ctx=None) -> bytes:
    """air::prove + Proof::to_bytes (src/air.rs:365-372, 262-281) on the GPU."""
    ctx = ctx or default_context()
    size = params.proof_size()
    buf = (C.c_uint8 * size)()
    n = C.c_size_t()
    check(lib().z0p_gpu_air_prove(ctx.handle, C.byref(params), C.byref(transcript.state), buf,
                                  size, C.byref(n)))
    return bytes(buf)[: n.value]


def prove_into(params: Params, transcript: Transcript, buf, ctx=None) -> int:
    """Proves into a caller-owned ctypes byte buffer; returns the length."""
    ctx = ctx or default_context()
    n = C.c_size_t()
    check(lib().z0p_gpu_air_prove(ctx.handle, C.byref(params), C.byref(transcript.state), buf,
                                  len(buf), C.byref(n)))
    return n.value


def prove_with_trace(params: Params, col_a, col_b, transcript: Transcript, ctx=None) -> bytes:
    """air::prove_with_trace (src/air.rs:381-399): the caller's two columns."""
    import numpy as np

    ctx = ctx or default_context()
    a = np.ascontiguousarray(np.asarray(col_a, dtype=np.uint32))
    b = np.ascontiguousarray(np.asarray(col_b, dtype=np.uint32))
    if len(a) != len(b):
        raise ValueError("trace columns must have one length")
    size = params.proof_size()
    out = (C.c_uint8 * size)()
    n = C.c_size_t()
    u32p = C.POINTER(C.c_uint32)
    check(lib().z0p_gpu_air_prove_with_trace(ctx.handle, C.byref(params), a.ctypes.data_as(u32p),
                                             b.ctypes.data_as(u32p), len(a),
                                             C.byref(transcript.state), out, size, C.byref(n)))
    return bytes(out)[: n.value]


def prove_zk(params: Params, n_rand: int, rng, transcript: Transcript, ctx=None) -> bytes:
    """air::prove_zk (src/air.rs:439-464): `rng` is a z0p_gb300.rng.ChaCha20."""
    ctx = ctx or default_context()
    n = C.c_size_t()
    check(lib().z0p_air_proof_size_zk(C.byref(params), n_rand, C.byref(n)))
    size = n.value
    out = (C.c_uint8 * size)()
    check(lib().z0p_gpu_air_prove_zk(ctx.handle, C.byref(params), n_rand, C.byref(rng),
                                     C.byref(transcript.state), out, size, C.byref(n)))
    return bytes(out)[: n.value]


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
    check(lib().z0p_gpu_air_prove_group(ctx.handle, n, arr, states, outs, caps, lens))
    return [bytes(b)[: lens[i]] for i, b in enumerate(bufs)]
