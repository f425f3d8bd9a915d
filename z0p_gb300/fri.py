"""FRI as a polynomial commitment on the GB300 backend — mirrors z0p::fri's
public commit / open entry points (src/fri.rs:400-666).

    params = fri.Params.new(blowup, num_queries, final_size)
    state = fri.commit(coeffs, params, transcript)       # Commitment on the device
    proof, indices = fri.open(state, transcript)         # Proof::to_bytes, query indices

``state.commitment`` holds Commitment::to_bytes. The layers and trees stay on
the context's device until ``open`` or any other call on that context.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from ._lib import FriParams, check, lib
from .context import default_context
from .transcript import Transcript

COEFFS, COEFFS_EXT, EVALS, EVALS_EXT = 0, 1, 2, 3


class Params(FriParams):
    """fri::Params (src/fri.rs:103-126); fields are public as in the reference,
    and every entry point re-validates them."""

    @classmethod
    def new(cls, blowup, num_queries, final_size) -> "Params":
        p = cls()
        p.blowup, p.num_queries, p.final_size = blowup, num_queries, final_size
        p.grinding_bits, p.cap_height = 0, 0
        return p

    @classmethod
    def for_security(cls, poly_len, target_bits) -> "Params":
        """fri::Params::for_security (src/fri.rs:232-255)."""
        p = cls()
        check(lib().z0p_fri_params_for_security(poly_len, target_bits, C.byref(p)))
        return p

    def with_grinding_bits(self, bits: int) -> "Params":
        self.grinding_bits = bits
        return self

    def with_cap_height(self, height: int) -> "Params":
        self.cap_height = height
        return self


class ProverState:
    """The device-resident commitment (ProverState, src/fri.rs:276-295)."""

    def __init__(self, ctx, params: Params, commitment: bytes, proof_size: int):
        self.ctx = ctx
        self.params = params
        self.commitment = commitment
        self.proof_size = proof_size


def _words(values, ext: bool):
    a = np.ascontiguousarray(np.asarray(values, dtype=np.uint32).reshape(-1))
    n = len(a) // 4 if ext else len(a)
    if ext and len(a) % 4:
        raise ValueError("Ext4 values are 4 words each")
    return a, n


def _commit(form, values, params: Params, transcript: Transcript, degree_bound=0, ctx=None):
    ctx = ctx or default_context()
    a, n = _words(values, form in (COEFFS_EXT, EVALS_EXT))
    clen, plen = C.c_size_t(), C.c_size_t()
    check(lib().z0p_fri_sizes(C.byref(params), form, n, degree_bound, C.byref(clen), C.byref(plen)))
    out = (C.c_uint8 * clen.value)()
    got = C.c_size_t()
    check(lib().z0p_gpu_fri_commit(ctx.handle, C.byref(params), form,
                                   a.ctypes.data_as(C.POINTER(C.c_uint32)), n, degree_bound,
                                   C.byref(transcript.state), out, clen.value, C.byref(got)))
    return ProverState(ctx, params, bytes(out)[: got.value], plen.value)


def commit(poly_coeffs, params: Params, transcript: Transcript, ctx=None) -> ProverState:
    """fri::commit (src/fri.rs:407-433)."""
    return _commit(COEFFS, poly_coeffs, params, transcript, 0, ctx)


def commit_ext(poly_coeffs, params: Params, transcript: Transcript, ctx=None) -> ProverState:
    """fri::commit_ext (src/fri.rs:443-460); 4 words per Ext4 coefficient."""
    return _commit(COEFFS_EXT, poly_coeffs, params, transcript, 0, ctx)


def commit_evals(lde_evals, degree_bound, params: Params, transcript: Transcript,
                 ctx=None) -> ProverState:
    """fri::commit_evals (src/fri.rs:473-499)."""
    return _commit(EVALS, lde_evals, params, transcript, degree_bound, ctx)


def commit_ext_evals(lde_evals, degree_bound, params: Params, transcript: Transcript,
                     ctx=None) -> ProverState:
    """fri::commit_ext_evals (src/fri.rs:508-549); 4 words per Ext4 value."""
    return _commit(EVALS_EXT, lde_evals, params, transcript, degree_bound, ctx)


def open(state: ProverState, transcript: Transcript):  # noqa: A001 - mirrors fri::open
    """fri::open (src/fri.rs:645-666): (Proof::to_bytes, query indices)."""
    out = (C.c_uint8 * state.proof_size)()
    got = C.c_size_t()
    idx = (C.c_uint64 * state.params.num_queries)()
    check(lib().z0p_gpu_fri_open(state.ctx.handle, C.byref(transcript.state), out, state.proof_size,
                                 C.byref(got), idx))
    return bytes(out)[: got.value], list(idx)
