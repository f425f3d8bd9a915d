"""Batched and served proving over a pool of prover contexts.

Mirrors include/z0p_gpu.h ("batching / serving"): a native worker pool where
each worker owns a CUDA stream and workspace, a FIFO queue, and admission by
device footprint (HBM budget). Proof bytes and transcript post-states are the
same as proving each statement alone.
"""
from __future__ import annotations

import ctypes as C

from . import air as _air
from . import range as _range
from ._lib import Job, check, lib
from .transcript import Transcript

AIR, RANGE = 0, 1


class Pool:
    def __init__(self, device: int = 0, workers: int = 8, hbm_budget: int = 0):
        self.handle = C.c_void_p()
        check(lib().z0p_gpu_pool_create(device, workers, hbm_budget, C.byref(self.handle)))
        self._live = {}

    def close(self):
        if self.handle:
            lib().z0p_gpu_pool_destroy(self.handle)
            self.handle = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def clock(self) -> float:
        return lib().z0p_gpu_pool_clock(self.handle)

    @staticmethod
    def make_job(params, transcript: Transcript):
        """A Job for air.Params or range.Params; the transcript is advanced in place."""
        j = Job()
        if isinstance(params, _air.Params):
            j.kind = AIR
            C.memmove(C.byref(j.air), C.byref(params), C.sizeof(params))
        elif isinstance(params, _range.Params):
            j.kind = RANGE
            C.memmove(C.byref(j.range), C.byref(params), C.sizeof(params))
        else:
            raise TypeError("params must be air.Params or range.Params")
        size = params.proof_size()
        buf = (C.c_uint8 * size)()
        j.transcript = C.pointer(transcript.state)
        j.out = C.cast(buf, C.POINTER(C.c_uint8))
        j.cap = size
        j._buf, j._t = buf, transcript  # keep alive
        return j

    def submit(self, job: Job) -> int:
        t = C.c_uint64()
        check(lib().z0p_gpu_pool_submit(self.handle, C.byref(job), C.byref(t)))
        self._live[t.value] = job
        return t.value

    def wait(self, ticket: int, timeout_ms: int = -1) -> bytes:
        rc = lib().z0p_gpu_pool_wait(self.handle, ticket, timeout_ms)
        job = self._live.pop(ticket)
        check(rc)
        return bytes(job._buf)[: job.len]

    def prove_all(self, jobs):
        """Proves a list of Jobs; returns their proof bytes in order."""
        arr = (Job * len(jobs))()
        for i, j in enumerate(jobs):
            arr[i] = j
        rc = lib().z0p_gpu_pool_prove_all(self.handle, arr, len(jobs))
        for i, j in enumerate(jobs):
            j.status, j.len = arr[i].status, arr[i].len
            j.submit_s, j.start_s, j.end_s = arr[i].submit_s, arr[i].start_s, arr[i].end_s
        check(rc)
        return [bytes(j._buf)[: j.len] for j in jobs]
