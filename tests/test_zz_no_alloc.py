"""The allocation-free LDE entry point against the allocating one (GPU).

z0p_gpu_rs_extend_noalloc serves callers that may not allocate device memory:
a process whose device heap belongs to another allocator, a loop in which
cudaMalloc/cudaFree would synchronise the device, or a deployment whose
memory budget is fixed when the library loads. It works in static device
arrays of this library, so it must return the same words as
z0p_gpu_rs_extend. This file checks that on two calls in a row (the second
reuses the scratch the first left behind) and checks that sizes above the
static limit are refused. The comparison is bit-exact, because the
arithmetic is exact mod p.
"""
import ctypes as C

import pytest

pytestmark = pytest.mark.gpu

LIMIT = 1 << 20  # n * batch * blowup accepted by the allocation-free entry


def _bind(z0p):
    L = z0p.lib()
    fn = L.z0p_gpu_rs_extend_noalloc
    fn.restype = C.c_int
    fn.argtypes = [C.c_void_p, C.c_uint64, C.c_uint64, C.c_uint64, C.c_void_p, C.c_void_p]
    return L, fn


def test_noalloc_matches_allocating_entry_two_calls(z0p, gpu_ctx):
    torch = pytest.importorskip("torch")
    import numpy as np

    L, noalloc = _bind(z0p)
    P = 2013265921
    rng = np.random.default_rng(20261203)
    stream = torch.cuda.current_stream()
    # Two calls in a row: a four-step size, then a single-CTA size whose
    # smaller footprint leaves the first call's words in the scratch.
    for logn, batch, blowup in [(15, 2, 16), (9, 3, 8)]:
        n = 1 << logn
        vals = rng.integers(0, P, size=batch * n, dtype=np.uint64).astype(np.int64)
        d_in = torch.from_numpy(vals).to(torch.int32).cuda()
        ref = torch.zeros(batch * n * blowup, dtype=torch.int32, device="cuda")
        out = torch.full((batch * n * blowup,), -1, dtype=torch.int32, device="cuda")
        torch.cuda.synchronize()
        rc = L.z0p_gpu_rs_extend(gpu_ctx.handle, C.c_void_p(d_in.data_ptr()), n, batch, blowup,
                                 C.c_void_p(ref.data_ptr()))
        assert rc == 0, L.z0p_gpu_last_reason()
        rc = noalloc(C.c_void_p(d_in.data_ptr()), n, batch, blowup, C.c_void_p(out.data_ptr()),
                     C.c_void_p(stream.cuda_stream))
        assert rc == 0, L.z0p_gpu_last_reason()
        torch.cuda.synchronize()
        assert torch.equal(out, ref), (logn, batch, blowup)


def test_noalloc_rejects_sizes_above_limit(z0p):
    torch = pytest.importorskip("torch")
    L, noalloc = _bind(z0p)
    d = torch.zeros(1 << 16, dtype=torch.int32, device="cuda")
    o = torch.zeros(1 << 16, dtype=torch.int32, device="cuda")
    # 2^16 * 4 * 8 = 2^21 > 2^20 output elements: refused before any launch.
    rc = noalloc(C.c_void_p(d.data_ptr()), 1 << 16, 4, 8, C.c_void_p(o.data_ptr()), None)
    assert rc == 103
    assert b"static scratch limit" in L.z0p_gpu_last_reason()
