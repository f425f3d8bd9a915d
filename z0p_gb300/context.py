"""Prover contexts: one CUDA stream plus a grow-only device workspace."""
from __future__ import annotations

import ctypes as C
import json
import threading

from ._lib import Stats, check, lib


class Context:
    """z0p_gpu_ctx_create(device) — raises Z0pError when no CUDA device exists."""

    def __init__(self, device: int = 0):
        self.device = device
        self.handle = C.c_void_p()
        check(lib().z0p_gpu_ctx_create(device, C.byref(self.handle)))

    def close(self):
        if self.handle:
            lib().z0p_gpu_ctx_destroy(self.handle)
            self.handle = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def stream(self) -> int:
        """The context's cudaStream_t as an integer handle."""
        return lib().z0p_gpu_ctx_stream(self.handle) or 0

    @property
    def device_bytes(self) -> int:
        return lib().z0p_gpu_ctx_device_bytes(self.handle)

    def blake3_ceiling(self) -> float:
        """Measured BLAKE3 throughput ceiling of the device, G compressions/s."""
        g = C.c_double()
        check(lib().z0p_gpu_blake3_ceiling(self.handle, C.byref(g)))
        return g.value

    def trim(self) -> None:
        """Hand the proof workspace back to the library's device memory pool."""
        check(lib().z0p_gpu_ctx_trim(self.handle))

    def set_gates(self, on: bool) -> None:
        """Gated launches on (the default: lower single-proof latency) or off
        (contexts proving side by side); the proof bytes do not change."""
        check(lib().z0p_gpu_ctx_set_gates(self.handle, 1 if on else 0))

    def reserve_group(self, max_group: int) -> None:
        """Reserve constant slots for proof groups of up to max_group statements."""
        check(lib().z0p_gpu_ctx_reserve_group(self.handle, max_group))

    def stats(self) -> dict:
        s = Stats()
        check(lib().z0p_gpu_ctx_stats(self.handle, C.byref(s)))
        return {k: getattr(s, k) for k, _ in Stats._fields_}

    def set_profiling(self, on: bool) -> None:
        check(lib().z0p_gpu_ctx_set_profiling(self.handle, 1 if on else 0))

    def profile(self) -> dict:
        """Per-stage {name: {"ms", "calls", "kernels"}} since the last call (profiling mode)."""
        n = C.c_size_t()
        lib().z0p_gpu_ctx_profile(self.handle, None, 0, C.byref(n))
        buf = C.create_string_buffer(n.value + 64)
        check(lib().z0p_gpu_ctx_profile(self.handle, buf, len(buf), C.byref(n)))
        return json.loads(buf.value.decode())


_default = {}
_lock = threading.Lock()


def default_context(device: int = 0) -> Context:
    with _lock:
        ctx = _default.get(device)
        if ctx is None:
            ctx = _default[device] = Context(device)
        return ctx
