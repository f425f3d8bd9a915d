"""CPU oracle for the z0p prove path — TEST INFRASTRUCTURE ONLY.

A plain-C restatement of FutureProofsTech/z0p (src/babybear.rs, ext4.rs,
hash.rs, transcript.rs, merkle.rs, ntt.rs, fri.rs, air.rs, range.rs,
codec.rs) compiled to ``oracle/liboracle.so``. Only the test suite, the
smoke check and the CPU-baseline leg of ``bench.py`` import this module; the
GPU prover never calls it.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "liboracle.so")
SRC = os.path.join(HERE, "z0p_oracle.c")

P = 2013265921

ERRORS = {
    0: "Ok", 1: "EmptyInput", 2: "IndexOutOfBounds", 3: "InvalidDomainSize",
    4: "InvalidBlowup", 5: "NoQueries", 6: "BadMerklePath",
    7: "FriVerificationFailed", 8: "MalformedInput", 9: "RngUnavailable",
}


def build(force: bool = False) -> str:
    """Compile the oracle with gcc (portable C11 + pthreads, no arch flags)."""
    if force or not os.path.exists(LIB_PATH) or os.path.getmtime(LIB_PATH) < max(
        os.path.getmtime(SRC), os.path.getmtime(os.path.join(HERE, "z0p_oracle.h"))
    ):
        tmp = LIB_PATH + f".tmp{os.getpid()}"
        subprocess.check_call(
            ["gcc", "-O3", "-std=c11", "-fPIC", "-shared", "-pthread", "-o", tmp, SRC]
        )
        os.replace(tmp, LIB_PATH)
    return LIB_PATH


class AirParams(C.Structure):
    _fields_ = [
        ("n_steps", C.c_uint64), ("blowup", C.c_uint64), ("num_queries", C.c_uint64),
        ("final_size", C.c_uint64), ("grinding_bits", C.c_uint32), ("cap_height", C.c_uint64),
        ("a0", C.c_uint32), ("b0", C.c_uint32), ("b_last", C.c_uint32),
    ]


class FriParams(C.Structure):
    """fri::Params (src/fri.rs:103-126)."""
    _fields_ = [
        ("blowup", C.c_uint64), ("num_queries", C.c_uint64), ("final_size", C.c_uint64),
        ("grinding_bits", C.c_uint32), ("cap_height", C.c_uint64),
    ]


FRI_COEFFS, FRI_COEFFS_EXT, FRI_EVALS, FRI_EVALS_EXT = 0, 1, 2, 3


class ChaCha20(C.Structure):
    """rng::ChaCha20 (src/rng.rs:81-112): key, nonce, block counter, buffered block."""
    _fields_ = [("key", C.c_uint8 * 32), ("nonce", C.c_uint8 * 12), ("counter", C.c_uint32),
                ("block", C.c_uint8 * 64), ("used", C.c_uint32)]

    @classmethod
    def new(cls, key: bytes, nonce: bytes) -> "ChaCha20":
        s = cls()
        lib().zo_chacha20_init(C.byref(s), key, nonce)
        return s

    def fill_bytes(self, n: int) -> bytes:
        out = (C.c_uint8 * n)()
        lib().zo_chacha20_fill(C.byref(self), out, n)
        return bytes(out)

    def next_field(self) -> int:
        return lib().zo_chacha20_next_field(C.byref(self))


def chacha20_block(key: bytes, counter: int, nonce: bytes) -> bytes:
    out = (C.c_uint8 * 64)()
    lib().zo_chacha20_block(key, counter, nonce, out)
    return bytes(out)


class TableParams(C.Structure):
    """table::Params (src/table.rs:27-45)."""
    _fields_ = [
        ("n_rows", C.c_uint64), ("blowup", C.c_uint64), ("num_queries", C.c_uint64),
        ("final_size", C.c_uint64), ("grinding_bits", C.c_uint32), ("cap_height", C.c_uint64),
        ("value", C.c_uint32),
    ]


class FoldParams(C.Structure):
    """fold::Params (src/fold.rs:42-64)."""
    _fields_ = [
        ("seg_steps", C.c_uint64), ("blowup", C.c_uint64), ("num_queries", C.c_uint64),
        ("final_size", C.c_uint64), ("grinding_bits", C.c_uint32), ("cap_height", C.c_uint64),
        ("in_a", C.c_uint32), ("in_b", C.c_uint32), ("out_b", C.c_uint32),
    ]


def fri_for_security(poly_len: int, target_bits: int) -> FriParams:
    """fri::Params::for_security (src/fri.rs:232-255), from the oracle's tuners."""
    if poly_len == 0:
        raise ValueError("EmptyInput")
    if poly_len & (poly_len - 1) or poly_len * 16 > 1 << 27:
        raise ValueError("InvalidDomainSize")
    q, g = C.c_size_t(), C.c_uint32()
    lib().zo_fri_tune_strength(target_bits, 2000, C.byref(q), C.byref(g))
    fs, ch = C.c_size_t(), C.c_size_t()
    lib().zo_fri_tune_shape(poly_len * 16, q.value, 0, 0, 0, C.byref(fs), C.byref(ch))
    return FriParams(16, q.value, fs.value, g.value, ch.value)


class RangeParams(C.Structure):
    _fields_ = [
        ("n_rows", C.c_uint64), ("n_bits", C.c_uint64), ("blowup", C.c_uint64),
        ("num_queries", C.c_uint64), ("final_size", C.c_uint64),
        ("grinding_bits", C.c_uint32), ("cap_height", C.c_uint64), ("value", C.c_uint32),
    ]


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(LIB_PATH)
        u8p, u32p, u64p, vp = C.POINTER(C.c_uint8), C.POINTER(C.c_uint32), C.POINTER(C.c_uint64), C.c_void_p
        sz = C.c_size_t
        sig = {
            "zo_f_mul": (C.c_uint32, [C.c_uint32, C.c_uint32]),
            "zo_f_pow": (C.c_uint32, [C.c_uint32, C.c_uint64]),
            "zo_f_inv": (C.c_uint32, [C.c_uint32]),
            "zo_f_from_u64": (C.c_uint32, [C.c_uint64]),
            "zo_batch_invert": (None, [u32p, sz]),
            "zo_splitmix64": (C.c_uint64, [u64p]),
            "zo_e_mul": (None, [u32p, u32p, u32p]),
            "zo_e_inv": (None, [u32p, u32p]),
            "zo_blake3": (None, [C.c_char_p, sz, u8p]),
            "zo_leaf64_digest": (None, [C.c_char_p, u8p]),
            "zo_node_digest": (None, [C.c_char_p, C.c_char_p, u8p]),
            "zo_leaf_digest": (None, [C.c_char_p, sz, u8p]),
            "zo_transcript_new": (vp, [C.c_char_p, sz]),
            "zo_transcript_clone": (vp, [vp]),
            "zo_transcript_free": (None, [vp]),
            "zo_transcript_absorb": (None, [vp, C.c_char_p, sz, C.c_char_p, sz]),
            "zo_transcript_challenge_bytes": (None, [vp, C.c_char_p, sz, u8p]),
            "zo_transcript_challenge_ext": (None, [vp, C.c_char_p, sz, u32p]),
            "zo_transcript_challenge_index": (C.c_int, [vp, C.c_char_p, sz, C.c_uint64, u64p]),
            "zo_transcript_grind": (C.c_uint64, [vp, C.c_char_p, sz, C.c_uint32]),
            "zo_transcript_verify_grind": (C.c_int, [vp, C.c_char_p, sz, C.c_uint64, C.c_uint32]),
            "zo_transcript_export": (None, [vp, u8p, u32p, u8p, u32p, u64p, u64p, u64p]),
            "zo_ntt_forward": (C.c_int, [u32p, sz]),
            "zo_ntt_inverse": (C.c_int, [u32p, sz]),
            "zo_evaluate_on_coset": (C.c_int, [u32p, sz, sz, C.c_uint32, u32p]),
            "zo_reed_solomon_extend": (C.c_int, [u32p, sz, sz, u32p]),
            "zo_merkle_flat64_cap": (C.c_int, [C.c_char_p, sz, sz, u8p, C.POINTER(sz)]),
            "zo_merkle_flat_cap": (C.c_int, [C.c_char_p, sz, sz, sz, u8p, C.POINTER(sz)]),
            "zo_fold_values": (None, [u32p, C.c_uint32, u32p, C.c_uint32, u32p]),
            "zo_fold_layer": (None, [u32p, sz, u32p, u32p, u32p, u32p]),
            "zo_fri_tune_shape": (None, [sz, sz, sz, sz, C.c_int, C.POINTER(sz), C.POINTER(sz)]),
            "zo_fri_tune_strength": (None, [C.c_uint32, C.c_uint32, C.POINTER(sz), u32p]),
            "zo_fri_composition_millibits": (C.c_uint32, [sz, sz]),
            "zo_air_params_new": (C.c_int, [C.c_uint64] * 4 + [C.c_uint32] * 3 + [C.POINTER(AirParams)]),
            "zo_air_for_security": (C.c_int, [C.c_uint64, C.c_uint32, C.c_uint32, C.c_uint32, C.c_uint32, C.POINTER(AirParams)]),
            "zo_air_build_trace": (None, [C.c_uint32, C.c_uint32, sz, u32p, u32p]),
            "zo_air_prove": (C.c_int, [C.POINTER(AirParams), vp, C.POINTER(u8p), C.POINTER(sz)]),
            "zo_air_prove_with_trace": (C.c_int, [C.POINTER(AirParams), u32p, u32p, vp, C.POINTER(u8p), C.POINTER(sz)]),
            "zo_air_compose": (C.c_int, [u32p, u32p, u32p, sz, C.c_uint32, C.c_uint32, C.c_uint32,
                                         C.c_uint32, sz, sz, u32p, u32p]),
            "zo_air_composition_at": (None, [C.c_uint32] * 7 + [C.c_uint32, C.c_uint32, sz, u32p, u32p]),
            "zo_air_verify": (C.c_int, [C.POINTER(AirParams), C.c_char_p, sz, vp]),
            "zo_range_params_new": (C.c_int, [C.c_uint64] * 5 + [C.c_uint32, C.POINTER(RangeParams)]),
            "zo_range_for_security": (C.c_int, [C.c_uint64, C.c_uint64, C.c_uint32, C.c_uint32, C.POINTER(RangeParams)]),
            "zo_range_prove": (C.c_int, [C.POINTER(RangeParams), vp, C.POINTER(u8p), C.POINTER(sz)]),
            "zo_range_prove_zk": (C.c_int, [C.POINTER(RangeParams), sz, C.POINTER(ChaCha20), vp,
                                            C.POINTER(u8p), C.POINTER(sz)]),
            "zo_range_prove_with_columns": (C.c_int, [C.POINTER(RangeParams), u32p, vp, C.POINTER(u8p),
                                                      C.POINTER(sz)]),
            "zo_range_verify": (C.c_int, [C.POINTER(RangeParams), C.c_char_p, sz, vp]),
            "zo_fri_commit": (C.c_int, [C.POINTER(FriParams), C.c_int, u32p, sz, C.c_uint64, vp,
                                        C.POINTER(vp), C.POINTER(u8p), C.POINTER(sz)]),
            "zo_fri_open": (C.c_int, [vp, vp, C.POINTER(u8p), C.POINTER(sz), u64p]),
            "zo_fri_state_free": (None, [vp]),
            "zo_fri_verify": (C.c_int, [C.POINTER(FriParams), C.c_char_p, sz, C.c_char_p, sz, vp, u64p]),
            "zo_chacha20_block": (None, [C.c_char_p, C.c_uint32, C.c_char_p, u8p]),
            "zo_chacha20_init": (None, [C.POINTER(ChaCha20), C.c_char_p, C.c_char_p]),
            "zo_chacha20_fill": (None, [C.POINTER(ChaCha20), u8p, sz]),
            "zo_chacha20_next_field": (C.c_uint32, [C.POINTER(ChaCha20)]),
            "zo_air_prove_zk": (C.c_int, [C.POINTER(AirParams), sz, C.POINTER(ChaCha20), vp,
                                          C.POINTER(u8p), C.POINTER(sz)]),
            "zo_table_params_new": (C.c_int, [C.c_uint64] * 4 + [C.c_uint32, C.POINTER(TableParams)]),
            "zo_table_for_security": (C.c_int, [C.c_uint64, C.c_uint64, C.c_uint32, C.c_uint32,
                                                 C.POINTER(TableParams)]),
            "zo_table_prove": (C.c_int, [C.POINTER(TableParams), u32p, sz, vp, C.POINTER(u8p),
                                         C.POINTER(sz)]),
            "zo_table_prove_zk": (C.c_int, [C.POINTER(TableParams), u32p, sz, sz, C.POINTER(ChaCha20),
                                            vp, C.POINTER(u8p), C.POINTER(sz)]),
            "zo_table_verify": (C.c_int, [C.POINTER(TableParams), u32p, sz, C.c_char_p, sz, vp]),
            "zo_fold_params_new": (C.c_int, [C.c_uint64] * 4 + [C.c_uint32] * 3 + [C.POINTER(FoldParams)]),
            "zo_fold_for_security": (C.c_int, [C.c_uint64] + [C.c_uint32] * 4 + [C.POINTER(FoldParams)]),
            "zo_fold_new": (vp, [C.POINTER(FoldParams)]),
            "zo_fold_add_segment": (C.c_int, [vp, u32p, u32p, sz, vp]),
            "zo_fold_finalize": (C.c_int, [vp, vp, C.POINTER(u8p), C.POINTER(sz)]),
            "zo_fold_free": (None, [vp]),
            "zo_fold_verify": (C.c_int, [C.POINTER(FoldParams), C.c_char_p, sz, vp]),
            "zo_free": (None, [vp]),
            "zo_set_max_workers": (None, [sz]),
            "zo_max_workers": (sz, []),
        }
        for name, (res, args) in sig.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def _b(x) -> bytes:
    return x.encode() if isinstance(x, str) else bytes(x)


def u32arr(values):
    import numpy as np

    a = np.ascontiguousarray(np.asarray(values, dtype=np.uint32))
    return a, a.ctypes.data_as(C.POINTER(C.c_uint32))


# ---------------------------------------------------------------- primitives


def blake3(data: bytes) -> bytes:
    out = (C.c_uint8 * 32)()
    lib().zo_blake3(_b(data), len(data), out)
    return bytes(out)


def leaf64_digest(block: bytes) -> bytes:
    assert len(block) == 64
    out = (C.c_uint8 * 32)()
    lib().zo_leaf64_digest(block, out)
    return bytes(out)


def node_digest(left: bytes, right: bytes) -> bytes:
    out = (C.c_uint8 * 32)()
    lib().zo_node_digest(left, right, out)
    return bytes(out)


def leaf_digest(data: bytes) -> bytes:
    out = (C.c_uint8 * 32)()
    lib().zo_leaf_digest(_b(data), len(data), out)
    return bytes(out)


def splitmix64(state: int):
    s = C.c_uint64(state)
    z = lib().zo_splitmix64(C.byref(s))
    return z, s.value


def f_mul(a, b):
    return lib().zo_f_mul(a, b)


def f_inv(a):
    return lib().zo_f_inv(a)


def f_pow(a, e):
    return lib().zo_f_pow(a, e)


def e_mul(x, y):
    """ext4.rs:106-117 product of two Ext4 given as 4 coordinates."""
    a = (C.c_uint32 * 4)(*x)
    b = (C.c_uint32 * 4)(*y)
    out = (C.c_uint32 * 4)()
    lib().zo_e_mul(a, b, out)
    return list(out)


class Transcript:
    """transcript.rs:54-171 restated (handle over the C oracle)."""

    def __init__(self, label=b"", _handle=None):
        self.h = _handle if _handle is not None else lib().zo_transcript_new(_b(label), len(_b(label)))

    def __del__(self):
        if getattr(self, "h", None):
            lib().zo_transcript_free(self.h)
            self.h = None

    def clone(self):
        return Transcript(_handle=lib().zo_transcript_clone(self.h))

    def absorb(self, label, data):
        lib().zo_transcript_absorb(self.h, _b(label), len(_b(label)), _b(data), len(_b(data)))

    def challenge_bytes(self, label) -> bytes:
        out = (C.c_uint8 * 32)()
        lib().zo_transcript_challenge_bytes(self.h, _b(label), len(_b(label)), out)
        return bytes(out)

    def challenge_ext(self, label):
        out = (C.c_uint32 * 4)()
        lib().zo_transcript_challenge_ext(self.h, _b(label), len(_b(label)), out)
        return list(out)

    def challenge_index(self, label, domain):
        out = C.c_uint64()
        rc = lib().zo_transcript_challenge_index(self.h, _b(label), len(_b(label)), domain, C.byref(out))
        return None if rc else out.value

    def grind(self, label, bits):
        return lib().zo_transcript_grind(self.h, _b(label), len(_b(label)), bits)

    def verify_grind(self, label, nonce, bits) -> bool:
        return bool(lib().zo_transcript_verify_grind(self.h, _b(label), len(_b(label)), nonce, bits))

    def export(self):
        tail = (C.c_uint8 * 2048)()
        stack = (C.c_uint8 * (54 * 32))()
        tl, sl = C.c_uint32(), C.c_uint32()
        ni, tot, ctr = C.c_uint64(), C.c_uint64(), C.c_uint64()
        lib().zo_transcript_export(self.h, tail, C.byref(tl), stack, C.byref(sl), C.byref(ni),
                                   C.byref(tot), C.byref(ctr))
        return {
            "tail": bytes(tail)[: tl.value], "stack": bytes(stack)[: 32 * sl.value],
            "stack_len": sl.value, "next_index": ni.value, "total_len": tot.value,
            "counter": ctr.value,
        }


# ------------------------------------------------------------------- params


def air_params_new(n_steps, blowup, num_queries, final_size, a0, b0, b_last,
                   grinding_bits=0, cap_height=0):
    p = AirParams()
    rc = lib().zo_air_params_new(n_steps, blowup, num_queries, final_size, a0, b0, b_last, C.byref(p))
    if rc:
        raise ValueError(ERRORS.get(rc, rc))
    p.grinding_bits = grinding_bits
    p.cap_height = cap_height
    return p


def air_for_security(n_steps, a0, b0, b_last, target_bits=100):
    p = AirParams()
    rc = lib().zo_air_for_security(n_steps, a0, b0, b_last, target_bits, C.byref(p))
    if rc:
        raise ValueError(ERRORS.get(rc, rc))
    return p


def range_params_new(n_rows, n_bits, blowup, num_queries, final_size, value,
                     grinding_bits=0, cap_height=0):
    p = RangeParams()
    rc = lib().zo_range_params_new(n_rows, n_bits, blowup, num_queries, final_size, value, C.byref(p))
    if rc:
        raise ValueError(ERRORS.get(rc, rc))
    p.grinding_bits = grinding_bits
    p.cap_height = cap_height
    return p


def range_for_security(n_rows, n_bits, value, target_bits=100):
    p = RangeParams()
    rc = lib().zo_range_for_security(n_rows, n_bits, value, target_bits, C.byref(p))
    if rc:
        raise ValueError(ERRORS.get(rc, rc))
    return p


def build_trace(a0, b0, n):
    import numpy as np

    a = np.zeros(n, dtype=np.uint32)
    b = np.zeros(n, dtype=np.uint32)
    lib().zo_air_build_trace(a0, b0, n, a.ctypes.data_as(C.POINTER(C.c_uint32)),
                             b.ctypes.data_as(C.POINTER(C.c_uint32)))
    return a, b


# -------------------------------------------------------------- prove/verify


def _take_proof(rc, buf, n):
    if rc:
        raise ValueError(ERRORS.get(rc, rc))
    out = C.string_at(buf, n.value)
    lib().zo_free(buf)
    return out


def air_prove(params: AirParams, t: Transcript) -> bytes:
    buf, n = C.POINTER(C.c_uint8)(), C.c_size_t()
    rc = lib().zo_air_prove(C.byref(params), t.h, C.byref(buf), C.byref(n))
    return _take_proof(rc, buf, n)


def air_prove_with_trace(params: AirParams, col_a, col_b, t: Transcript) -> bytes:
    a, ap = u32arr(col_a)
    b, bp = u32arr(col_b)
    buf, n = C.POINTER(C.c_uint8)(), C.c_size_t()
    rc = lib().zo_air_prove_with_trace(C.byref(params), ap, bp, t.h, C.byref(buf), C.byref(n))
    return _take_proof(rc, buf, n)


def air_prove_zk(params: AirParams, n_rand: int, rng: ChaCha20, t: Transcript) -> bytes:
    """air::prove_zk (src/air.rs:439-464): advances rng and t."""
    buf, n = C.POINTER(C.c_uint8)(), C.c_size_t()
    rc = lib().zo_air_prove_zk(C.byref(params), n_rand, C.byref(rng), t.h, C.byref(buf), C.byref(n))
    return _take_proof(rc, buf, n)


def table_params_new(n_rows, blowup, num_queries, final_size, value) -> TableParams:
    p = TableParams()
    rc = lib().zo_table_params_new(n_rows, blowup, num_queries, final_size, value, C.byref(p))
    if rc:
        raise ValueError(ERRORS[rc])
    return p


def table_for_security(n_rows, table_len, value, target_bits) -> TableParams:
    p = TableParams()
    rc = lib().zo_table_for_security(n_rows, table_len, value, target_bits, C.byref(p))
    if rc:
        raise ValueError(ERRORS[rc])
    return p


def table_prove(params: TableParams, table, t: Transcript) -> bytes:
    """table::prove (src/table.rs:305-317)."""
    a, ap = u32arr(table)
    buf, n = C.POINTER(C.c_uint8)(), C.c_size_t()
    rc = lib().zo_table_prove(C.byref(params), ap, len(a), t.h, C.byref(buf), C.byref(n))
    return _take_proof(rc, buf, n)


def table_prove_zk(params: TableParams, table, n_rand: int, rng: "ChaCha20", t: Transcript) -> bytes:
    """table::prove_zk (src/table.rs:329-356)."""
    a, ap = u32arr(table)
    buf, n = C.POINTER(C.c_uint8)(), C.c_size_t()
    rc = lib().zo_table_prove_zk(C.byref(params), ap, len(a), n_rand, C.byref(rng), t.h,
                                 C.byref(buf), C.byref(n))
    return _take_proof(rc, buf, n)


def table_verify(params: TableParams, table, proof: bytes, t: Transcript) -> int:
    a, ap = u32arr(table)
    return lib().zo_table_verify(C.byref(params), ap, len(a), proof, len(proof), t.h)


def air_verify(params: AirParams, proof: bytes, t: Transcript) -> int:
    return lib().zo_air_verify(C.byref(params), proof, len(proof), t.h)


def range_prove(params: RangeParams, t: Transcript) -> bytes:
    buf, n = C.POINTER(C.c_uint8)(), C.c_size_t()
    rc = lib().zo_range_prove(C.byref(params), t.h, C.byref(buf), C.byref(n))
    return _take_proof(rc, buf, n)


def range_prove_with_columns(params: RangeParams, v_col, bit_cols, t: Transcript) -> bytes:
    """range.rs:353-375: the caller's columns (value column, then n_bits bit columns)."""
    import numpy as np

    cols = np.ascontiguousarray(np.concatenate([np.asarray(v_col, dtype=np.uint32)] +
                                               [np.asarray(b, dtype=np.uint32) for b in bit_cols]))
    if len(bit_cols) != params.n_bits or cols.size != (params.n_bits + 1) * params.n_rows:
        raise ValueError("MalformedInput")
    buf, n = C.POINTER(C.c_uint8)(), C.c_size_t()
    rc = lib().zo_range_prove_with_columns(C.byref(params), cols.ctypes.data_as(C.POINTER(C.c_uint32)),
                                           t.h, C.byref(buf), C.byref(n))
    return _take_proof(rc, buf, n)


def range_prove_zk(params: RangeParams, n_rand: int, rng, t: Transcript) -> bytes:
    """range.rs:393-418: every column masked from the ChaCha20 stream `rng`."""
    buf, n = C.POINTER(C.c_uint8)(), C.c_size_t()
    rc = lib().zo_range_prove_zk(C.byref(params), n_rand, C.byref(rng), t.h, C.byref(buf), C.byref(n))
    return _take_proof(rc, buf, n)


def range_verify(params: RangeParams, proof: bytes, t: Transcript) -> int:
    return lib().zo_range_verify(C.byref(params), proof, len(proof), t.h)


class FriState:
    """fri::ProverState (src/fri.rs:276-295): the committed layers and trees."""

    def __init__(self, handle, commitment: bytes, num_queries: int):
        self.h = handle
        self.commitment = commitment
        self.num_queries = num_queries

    def __del__(self):
        if self.h:
            lib().zo_fri_state_free(self.h)
            self.h = None


def fri_commit(params: FriParams, form: int, values, t: Transcript, degree_bound: int = 0) -> FriState:
    """fri::commit / commit_ext / commit_evals / commit_ext_evals (src/fri.rs:400-549).
    Ext4 values are 4 coordinates each; `values` is the flat coordinate list."""
    a, ap = u32arr(values)
    n = len(a) // 4 if form in (FRI_COEFFS_EXT, FRI_EVALS_EXT) else len(a)
    st, buf, ln = C.c_void_p(), C.POINTER(C.c_uint8)(), C.c_size_t()
    rc = lib().zo_fri_commit(C.byref(params), form, ap, n, degree_bound, t.h, C.byref(st),
                             C.byref(buf), C.byref(ln))
    return FriState(st, _take_proof(rc, buf, ln), params.num_queries)


def fri_open(state: FriState, t: Transcript):
    """fri::open (src/fri.rs:645-666): (proof bytes, query indices)."""
    idx = (C.c_uint64 * state.num_queries)()
    buf, ln = C.POINTER(C.c_uint8)(), C.c_size_t()
    rc = lib().zo_fri_open(state.h, t.h, C.byref(buf), C.byref(ln), idx)
    return _take_proof(rc, buf, ln), list(idx)


def fri_verify(params: FriParams, commitment: bytes, proof: bytes, t: Transcript):
    """fri::verify (src/fri.rs:694-858): (status, query indices)."""
    idx = (C.c_uint64 * max(1, params.num_queries))()
    rc = lib().zo_fri_verify(C.byref(params), commitment, len(commitment), proof, len(proof), t.h, idx)
    return rc, list(idx)[: params.num_queries]


def fold_params_new(seg_steps, blowup, num_queries, final_size, in_a, in_b, out_b) -> FoldParams:
    p = FoldParams()
    rc = lib().zo_fold_params_new(seg_steps, blowup, num_queries, final_size, in_a, in_b, out_b,
                                  C.byref(p))
    if rc:
        raise ValueError(ERRORS[rc])
    return p


def fold_for_security(seg_steps, in_a, in_b, out_b, target_bits) -> FoldParams:
    p = FoldParams()
    rc = lib().zo_fold_for_security(seg_steps, in_a, in_b, out_b, target_bits, C.byref(p))
    if rc:
        raise ValueError(ERRORS[rc])
    return p


class Accumulator:
    """fold::Accumulator (src/fold.rs:362-561)."""

    def __init__(self, params: FoldParams):
        self.params = params
        self.h = lib().zo_fold_new(C.byref(params))
        self.n = 0

    def __del__(self):
        if self.h:
            lib().zo_fold_free(self.h)
            self.h = None

    def add_segment(self, col_a, col_b, t: Transcript) -> None:
        a, ap = u32arr(col_a)
        b, bp = u32arr(col_b)
        if len(a) != len(b):
            raise ValueError("MalformedInput")
        rc = lib().zo_fold_add_segment(self.h, ap, bp, len(a), t.h)
        if rc:
            raise ValueError(ERRORS[rc])
        self.n += 1

    def finalize(self, t: Transcript) -> bytes:
        buf, n = C.POINTER(C.c_uint8)(), C.c_size_t()
        rc = lib().zo_fold_finalize(self.h, t.h, C.byref(buf), C.byref(n))
        return _take_proof(rc, buf, n)


def fold_verify(params: FoldParams, proof: bytes, t: Transcript) -> int:
    return lib().zo_fold_verify(C.byref(params), proof, len(proof), t.h)


# ------------------------------------------------------------ kernel pieces


def ntt_inverse(values):
    a, ap = u32arr(values)
    a = a.copy()
    rc = lib().zo_ntt_inverse(a.ctypes.data_as(C.POINTER(C.c_uint32)), len(a))
    if rc:
        raise ValueError(ERRORS[rc])
    return a


def ntt_forward(values):
    a, _ = u32arr(values)
    a = a.copy()
    rc = lib().zo_ntt_forward(a.ctypes.data_as(C.POINTER(C.c_uint32)), len(a))
    if rc:
        raise ValueError(ERRORS[rc])
    return a


def evaluate_on_coset(coeffs, blowup, shift=31):
    import numpy as np

    a, ap = u32arr(coeffs)
    out = np.zeros(len(a) * blowup, dtype=np.uint32)
    rc = lib().zo_evaluate_on_coset(ap, len(a), blowup, shift, out.ctypes.data_as(C.POINTER(C.c_uint32)))
    if rc:
        raise ValueError(ERRORS[rc])
    return out


def reed_solomon_extend(values, blowup):
    import numpy as np

    a, ap = u32arr(values)
    out = np.zeros(len(a) * blowup, dtype=np.uint32)
    rc = lib().zo_reed_solomon_extend(ap, len(a), blowup, out.ctypes.data_as(C.POINTER(C.c_uint32)))
    if rc:
        raise ValueError(ERRORS[rc])
    return out


def merkle_flat64_cap(flat: bytes, cap_height: int):
    out = (C.c_uint8 * (32 * 256))()
    n = C.c_size_t()
    rc = lib().zo_merkle_flat64_cap(flat, len(flat), cap_height, out, C.byref(n))
    if rc:
        raise ValueError(ERRORS[rc])
    return bytes(out)[: 32 * n.value]


def merkle_flat_cap(flat: bytes, leaf_len: int, cap_height: int):
    out = (C.c_uint8 * (32 * 256))()
    n = C.c_size_t()
    rc = lib().zo_merkle_flat_cap(flat, len(flat), leaf_len, cap_height, out, C.byref(n))
    if rc:
        raise ValueError(ERRORS[rc])
    return bytes(out)[: 32 * n.value]


def fold_layer(values, first_points, challenges):
    """values: uint32 array of 4*n (Ext4 coords), bit-reversed; returns (next, next_points)."""
    import numpy as np

    v, vp = u32arr(values)
    fp, fpp = u32arr(first_points)
    ch, chp = u32arr(challenges)
    n = len(v) // 4
    out = np.zeros(4 * (n // 4), dtype=np.uint32)
    outp = np.zeros(max(n // 16, 1), dtype=np.uint32)
    lib().zo_fold_layer(vp, n, fpp, chp, out.ctypes.data_as(C.POINTER(C.c_uint32)),
                        outp.ctypes.data_as(C.POINTER(C.c_uint32)))
    return out, outp[: n // 16]


def air_compose(col_a, col_b, points, w_last, a0, b0, b_last, n, offset, alphas):
    """air::compose over caller points; alphas (5, 4); returns (m, 4) uint32."""
    import numpy as np

    a, ap = u32arr(col_a)
    b, bp = u32arr(col_b)
    pt, ptp = u32arr(points)
    al, alp = u32arr(np.asarray(alphas).reshape(-1))
    out = np.zeros((len(a), 4), dtype=np.uint32)
    rc = lib().zo_air_compose(ap, bp, ptp, len(a), w_last, a0, b0, b_last, n, offset, alp,
                              out.ctypes.data_as(C.POINTER(C.c_uint32)))
    if rc:
        raise ValueError(ERRORS[rc])
    return out


def air_composition_at(a, b, an, bn, x, w_last, a0, b0, b_last, n, alphas):
    import numpy as np

    al, alp = u32arr(np.asarray(alphas).reshape(-1))
    out = np.zeros(4, dtype=np.uint32)
    lib().zo_air_composition_at(a, b, an, bn, x, w_last, a0, b0, b_last, n, alp,
                                out.ctypes.data_as(C.POINTER(C.c_uint32)))
    return out


def set_max_workers(n: int):
    lib().zo_set_max_workers(n)


def max_workers() -> int:
    return lib().zo_max_workers()
