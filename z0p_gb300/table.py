"""Table membership on the GB300 backend — mirrors z0p::table (src/table.rs):
a committed constant column proved to lie in a public table.

    params = table.Params.new(n_rows, blowup, num_queries, final_size, value)
    proof = table.prove(params, entries, transcript)       # table::Proof::to_bytes
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from ._lib import TableParams, check, lib
from .context import default_context
from .transcript import Transcript

P = 2013265921


class Params(TableParams):
    """table::Params (src/table.rs:27-45)."""

    @classmethod
    def new(cls, n_rows, blowup, num_queries, final_size, value) -> "Params":
        p = cls()
        check(lib().z0p_table_params_new(n_rows, blowup, num_queries, final_size, value % P,
                                         C.byref(p)))
        return p

    @classmethod
    def for_security(cls, n_rows, table_len, value, target_bits) -> "Params":
        p = cls()
        check(lib().z0p_table_params_for_security(n_rows, table_len, value % P, target_bits,
                                                  C.byref(p)))
        return p

    def with_grinding_bits(self, bits: int) -> "Params":
        self.grinding_bits = bits
        return self

    def with_cap_height(self, height: int) -> "Params":
        self.cap_height = height
        return self


def _table(entries):
    a = np.ascontiguousarray(np.asarray(entries, dtype=np.uint32))
    return a, a.ctypes.data_as(C.POINTER(C.c_uint32))


def prove(params: Params, table, transcript: Transcript, ctx=None) -> bytes:
    """table::prove (src/table.rs:305-317)."""
    ctx = ctx or default_context()
    a, ap = _table(table)
    n = C.c_size_t()
    check(lib().z0p_table_proof_size(C.byref(params), len(a), 0, C.byref(n)))
    out = (C.c_uint8 * n.value)()
    check(lib().z0p_gpu_table_prove(ctx.handle, C.byref(params), ap, len(a), C.byref(transcript.state),
                                    out, n.value, C.byref(n)))
    return bytes(out)[: n.value]


def prove_zk(params: Params, table, n_rand: int, rng, transcript: Transcript, ctx=None) -> bytes:
    """table::prove_zk (src/table.rs:329-356): `rng` is a z0p_gb300.rng.ChaCha20."""
    ctx = ctx or default_context()
    a, ap = _table(table)
    n = C.c_size_t()
    check(lib().z0p_table_proof_size(C.byref(params), len(a), n_rand, C.byref(n)))
    out = (C.c_uint8 * n.value)()
    check(lib().z0p_gpu_table_prove_zk(ctx.handle, C.byref(params), ap, len(a), n_rand,
                                       C.byref(rng), C.byref(transcript.state), out, n.value,
                                       C.byref(n)))
    return bytes(out)[: n.value]
