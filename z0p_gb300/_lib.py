"""ctypes binding of libz0p_gpu.so (include/z0p_gpu.h).

Loading fails loudly: there is no CPU fallback anywhere in this package.
"""
from __future__ import annotations

import ctypes as C
import os

from . import build as _build

ERRORS = {
    0: "Ok", 1: "EmptyInput", 2: "IndexOutOfBounds", 3: "InvalidDomainSize",
    4: "InvalidBlowup", 5: "NoQueries", 6: "BadMerklePath", 7: "FriVerificationFailed",
    8: "MalformedInput", 9: "RngUnavailable", 100: "BufferTooSmall", 101: "Cuda",
    102: "OutOfMemory", 103: "Unsupported", 104: "DeviceTimeout", 105: "Admission",
    106: "InvalidArgument", 107: "Cancelled",
}


class Z0pError(Exception):
    """A non-zero status from the C ABI (code mirrors z0p::Error for 1..9)."""

    def __init__(self, code: int, reason: str = ""):
        self.code = code
        self.name = ERRORS.get(code, f"Status{code}")
        super().__init__(f"{self.name} ({code})" + (f": {reason}" if reason else ""))


class AirParams(C.Structure):
    _fields_ = [
        ("n_steps", C.c_uint64), ("blowup", C.c_uint64), ("num_queries", C.c_uint64),
        ("final_size", C.c_uint64), ("grinding_bits", C.c_uint32), ("cap_height", C.c_uint64),
        ("a0", C.c_uint32), ("b0", C.c_uint32), ("b_last", C.c_uint32),
    ]


class Schedule(C.Structure):
    _fields_ = [("ntt_log_n1", C.c_uint8 * 32), ("ntt_radix32", C.c_uint8 * 32), ("merkle_top_log", C.c_uint32),
                ("grind_ctas_per_sm", C.c_uint32)]


class TuneReport(C.Structure):
    _fields_ = [("ntt_default_us", C.c_float * 32), ("ntt_best_us", C.c_float * 32),
                ("merkle_default_us", C.c_float), ("merkle_best_us", C.c_float),
                ("grind_default_us", C.c_float), ("grind_best_us", C.c_float),
                ("wall_ms", C.c_float)]


class ChaChaState(C.Structure):
    _fields_ = [("key", C.c_uint8 * 32), ("nonce", C.c_uint8 * 12), ("counter", C.c_uint32),
                ("block", C.c_uint8 * 64), ("used", C.c_uint32)]


class FriParams(C.Structure):
    _fields_ = [
        ("blowup", C.c_uint64), ("num_queries", C.c_uint64), ("final_size", C.c_uint64),
        ("grinding_bits", C.c_uint32), ("cap_height", C.c_uint64),
    ]


class TableParams(C.Structure):
    _fields_ = [
        ("n_rows", C.c_uint64), ("blowup", C.c_uint64), ("num_queries", C.c_uint64),
        ("final_size", C.c_uint64), ("grinding_bits", C.c_uint32), ("cap_height", C.c_uint64),
        ("value", C.c_uint32),
    ]


class FoldParams(C.Structure):
    _fields_ = [
        ("seg_steps", C.c_uint64), ("blowup", C.c_uint64), ("num_queries", C.c_uint64),
        ("final_size", C.c_uint64), ("grinding_bits", C.c_uint32), ("cap_height", C.c_uint64),
        ("in_a", C.c_uint32), ("in_b", C.c_uint32), ("out_b", C.c_uint32),
    ]


class RangeParams(C.Structure):
    _fields_ = [
        ("n_rows", C.c_uint64), ("n_bits", C.c_uint64), ("blowup", C.c_uint64),
        ("num_queries", C.c_uint64), ("final_size", C.c_uint64),
        ("grinding_bits", C.c_uint32), ("cap_height", C.c_uint64), ("value", C.c_uint32),
    ]


class Stats(C.Structure):
    _fields_ = [("launches", C.c_uint64), ("h2d_bytes", C.c_uint64), ("d2h_bytes", C.c_uint64),
                ("syncs", C.c_uint64), ("proofs", C.c_uint64), ("sync_wait_ns", C.c_uint64),
                ("prove_ns", C.c_uint64)]


class TranscriptState(C.Structure):
    _fields_ = [
        ("tail", C.c_uint8 * 2048), ("tail_len", C.c_uint32),
        ("stack", (C.c_uint8 * 32) * 54), ("stack_len", C.c_uint32),
        ("next_index", C.c_uint64), ("total_len", C.c_uint64), ("counter", C.c_uint64),
    ]


class Job(C.Structure):
    _fields_ = [
        ("kind", C.c_int), ("air", AirParams), ("range", RangeParams),
        ("transcript", C.POINTER(TranscriptState)), ("out", C.POINTER(C.c_uint8)),
        ("cap", C.c_size_t), ("len", C.c_size_t), ("status", C.c_int),
        ("submit_s", C.c_double), ("start_s", C.c_double), ("end_s", C.c_double),
    ]


_lib = None


def lib():
    global _lib
    if _lib is None:
        path = _build.LIB_PATH
        if not os.path.exists(path):
            path = _build.build()
        L = C.CDLL(path)
        P = C.POINTER
        u8p, u32p, u64p, sz = P(C.c_uint8), P(C.c_uint32), P(C.c_uint64), C.c_size_t
        vp = C.c_void_p
        sig = {
            "z0p_gpu_abi_version": (C.c_int, []),
            "z0p_gpu_last_reason": (C.c_char_p, []),
            "z0p_transcript_init": (C.c_int, [P(TranscriptState), C.c_char_p, sz]),
            "z0p_transcript_absorb": (C.c_int, [P(TranscriptState), C.c_char_p, sz, C.c_char_p, sz]),
            "z0p_transcript_challenge_bytes": (C.c_int, [P(TranscriptState), C.c_char_p, sz, u8p]),
            "z0p_transcript_challenge_ext": (C.c_int, [P(TranscriptState), C.c_char_p, sz, u32p]),
            "z0p_transcript_challenge_index": (C.c_int, [P(TranscriptState), C.c_char_p, sz, C.c_uint64, u64p]),
            "z0p_air_params_new": (C.c_int, [C.c_uint64] * 4 + [C.c_uint32] * 3 + [P(AirParams)]),
            "z0p_air_params_for_security": (C.c_int, [C.c_uint64] + [C.c_uint32] * 4 + [P(AirParams)]),
            "z0p_range_params_new": (C.c_int, [C.c_uint64] * 5 + [C.c_uint32, P(RangeParams)]),
            "z0p_range_params_for_security": (C.c_int, [C.c_uint64, C.c_uint64, C.c_uint32, C.c_uint32, P(RangeParams)]),
            "z0p_air_proof_size": (C.c_int, [P(AirParams), P(sz)]),
            "z0p_range_proof_size": (C.c_int, [P(RangeParams), P(sz)]),
            "z0p_gpu_air_footprint": (C.c_int, [P(AirParams), P(sz)]),
            "z0p_gpu_range_footprint": (C.c_int, [P(RangeParams), P(sz)]),
            "z0p_gpu_ctx_create": (C.c_int, [C.c_int, P(vp)]),
            "z0p_gpu_ctx_destroy": (None, [vp]),
            "z0p_gpu_ctx_stream": (vp, [vp]),
            "z0p_gpu_ctx_device_bytes": (sz, [vp]),
            "z0p_gpu_ctx_trim": (C.c_int, [vp]),
            "z0p_gpu_ctx_set_gates": (C.c_int, [vp, C.c_int]),
            "z0p_gpu_ctx_reserve_group": (C.c_int, [vp, C.c_uint32]),
            "z0p_gpu_blake3_ceiling": (C.c_int, [vp, P(C.c_double)]),
            "z0p_range_proof_size_zk": (C.c_int, [P(RangeParams), sz, P(sz)]),
            "z0p_gpu_range_prove_zk": (C.c_int, [vp, P(RangeParams), sz, P(ChaChaState),
                                                 P(TranscriptState), P(C.c_uint8), sz, P(sz)]),
            "z0p_gpu_range_prove_with_columns": (C.c_int, [vp, P(RangeParams), P(C.c_uint32), sz,
                                                           P(P(C.c_uint32)), P(sz), sz,
                                                           P(TranscriptState), P(C.c_uint8), sz, P(sz)]),
            "z0p_schedule_default": (C.c_int, [P(Schedule)]),
            "z0p_gpu_schedule_get": (C.c_int, [C.c_int, P(Schedule)]),
            "z0p_gpu_schedule_set": (C.c_int, [C.c_int, P(Schedule)]),
            "z0p_gpu_autotune": (C.c_int, [vp, C.c_uint32, P(Schedule), P(TuneReport)]),
            "z0p_gpu_ctx_stats": (C.c_int, [vp, P(Stats)]),
            "z0p_gpu_ctx_set_profiling": (C.c_int, [vp, C.c_int]),
            "z0p_gpu_ctx_profile": (C.c_int, [vp, C.c_char_p, sz, P(sz)]),
            "z0p_gpu_air_prove": (C.c_int, [vp, P(AirParams), P(TranscriptState), u8p, sz, P(sz)]),
            "z0p_gpu_range_prove": (C.c_int, [vp, P(RangeParams), P(TranscriptState), u8p, sz, P(sz)]),
            "z0p_gpu_air_prove_with_trace": (C.c_int, [vp, P(AirParams), P(C.c_uint32), P(C.c_uint32),
                                                       sz, P(TranscriptState), P(C.c_uint8), sz,
                                                       P(sz)]),
            "z0p_air_proof_size_zk": (C.c_int, [P(AirParams), sz, P(sz)]),
            "z0p_gpu_air_prove_zk": (C.c_int, [vp, P(AirParams), sz, P(ChaChaState),
                                               P(TranscriptState), P(C.c_uint8), sz, P(sz)]),
            "z0p_table_params_new": (C.c_int, [C.c_uint64] * 4 + [C.c_uint32, P(TableParams)]),
            "z0p_table_params_for_security": (C.c_int, [C.c_uint64, C.c_uint64, C.c_uint32, C.c_uint32,
                                                        P(TableParams)]),
            "z0p_table_proof_size": (C.c_int, [P(TableParams), sz, sz, P(sz)]),
            "z0p_gpu_table_prove": (C.c_int, [vp, P(TableParams), P(C.c_uint32), sz, P(TranscriptState),
                                              P(C.c_uint8), sz, P(sz)]),
            "z0p_gpu_table_prove_zk": (C.c_int, [vp, P(TableParams), P(C.c_uint32), sz, sz,
                                                 P(ChaChaState), P(TranscriptState), P(C.c_uint8), sz,
                                                 P(sz)]),
            "z0p_fold_params_new": (C.c_int, [C.c_uint64] * 4 + [C.c_uint32] * 3 + [P(FoldParams)]),
            "z0p_fold_params_for_security": (C.c_int, [C.c_uint64] + [C.c_uint32] * 4 + [P(FoldParams)]),
            "z0p_gpu_fold_create": (C.c_int, [vp, P(FoldParams), P(vp)]),
            "z0p_gpu_fold_destroy": (None, [vp]),
            "z0p_gpu_fold_len": (sz, [vp]),
            "z0p_gpu_fold_add_segment": (C.c_int, [vp, P(C.c_uint32), P(C.c_uint32), sz,
                                                   P(TranscriptState)]),
            "z0p_gpu_fold_proof_size": (C.c_int, [vp, P(sz)]),
            "z0p_gpu_fold_finalize": (C.c_int, [vp, P(TranscriptState), P(C.c_uint8), sz, P(sz)]),
            "z0p_fri_params_for_security": (C.c_int, [C.c_uint64, C.c_uint32, P(FriParams)]),
            "z0p_fri_sizes": (C.c_int, [P(FriParams), C.c_int, sz, C.c_uint64, P(sz), P(sz)]),
            "z0p_gpu_fri_commit": (C.c_int, [vp, P(FriParams), C.c_int, P(C.c_uint32), sz, C.c_uint64,
                                             P(TranscriptState), P(C.c_uint8), sz, P(sz)]),
            "z0p_gpu_fri_open": (C.c_int, [vp, P(TranscriptState), P(C.c_uint8), sz, P(sz),
                                           P(C.c_uint64)]),
            "z0p_gpu_air_prove_group": (C.c_int, [vp, sz, P(AirParams), P(P(TranscriptState)),
                                                  P(u8p), P(sz), P(sz)]),
            "z0p_gpu_range_prove_group": (C.c_int, [vp, sz, P(RangeParams), P(P(TranscriptState)),
                                                    P(u8p), P(sz), P(sz)]),
            "z0p_gpu_rs_extend": (C.c_int, [vp, vp, C.c_uint64, C.c_uint64, C.c_uint64, vp]),
            "z0p_gpu_air_compose": (C.c_int, [vp, P(AirParams), u32p, vp]),
            "z0p_gpu_rs_extend_noalloc": (C.c_int, [vp, C.c_uint64, C.c_uint64, C.c_uint64, vp, vp]),
            "z0p_gpu_pool_create": (C.c_int, [C.c_int, C.c_int, sz, P(vp)]),
            "z0p_gpu_pool_destroy": (None, [vp]),
            "z0p_gpu_pool_submit": (C.c_int, [vp, P(Job), u64p]),
            "z0p_gpu_pool_wait": (C.c_int, [vp, C.c_uint64, C.c_int]),
            "z0p_gpu_pool_prove_all": (C.c_int, [vp, P(Job), sz]),
            "z0p_gpu_pool_clock": (C.c_double, [vp]),
            "z0p_gpu_merkle_flat64_cap": (C.c_int, [vp, vp, C.c_uint64, C.c_uint64, u8p, u64p]),
            "z0p_gpu_fri_fold": (C.c_int, [vp, vp, C.c_uint64, C.c_uint64, C.c_uint64, u32p, vp]),
            "z0p_gpu_grind": (C.c_int, [vp, C.c_char_p, sz, C.c_uint32, u64p]),
        }
        for name, (res, args) in sig.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def check(rc: int):
    if rc != 0:
        reason = lib().z0p_gpu_last_reason()
        raise Z0pError(rc, reason.decode(errors="replace") if reason else "")
