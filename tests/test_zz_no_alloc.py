"""The allocation-free LDE entry point against the allocating one and the
oracle (GPU).

z0p_gpu_rs_extend_noalloc serves callers that may not allocate device memory:
a process whose device heap belongs to another allocator, a loop in which
cudaMalloc/cudaFree would synchronise the device, or a deployment whose
memory budget is fixed when the library loads. It works in static device
arrays of this library, so it must return the same words as
z0p_gpu_rs_extend and as the oracle's reed_solomon_extend
(src/ntt.rs:436-439). The comparison is bit-exact, because the arithmetic is
exact mod p.

Every call runs on a stream created non-blocking, so when this file runs
alone in a fresh process the very first call (the one that uploads the
static tables) is not ordered after the legacy stream by anything but the
set-up's own wait. Three calls in a row reuse the scratch: a four-step size,
a smaller four-step size under a different split (the intermediate regions
still hold the first call's words), and a one-CTA size. Sizes above the
static limit are refused.
"""
import ctypes as C

import pytest

pytestmark = pytest.mark.gpu

LIMIT = 1 << 20  # n * batch * blowup accepted by the allocation-free entry
P = 2013265921


def _bind(z0p):
    L = z0p.lib()
    fn = L.z0p_gpu_rs_extend_noalloc
    fn.restype = C.c_int
    fn.argtypes = [C.c_void_p, C.c_uint64, C.c_uint64, C.c_uint64, C.c_void_p, C.c_void_p]
    return L, fn


def test_noalloc_matches_allocating_entry_and_oracle(z0p, gpu_ctx, oracle):
    torch = pytest.importorskip("torch")
    import numpy as np

    L, noalloc = _bind(z0p)
    rng = np.random.default_rng(20261203)
    stream = torch.cuda.Stream()  # created with cudaStreamNonBlocking
    for logn, batch, blowup in [(15, 2, 16), (13, 3, 2), (9, 3, 8)]:
        n = 1 << logn
        vals = rng.integers(0, P, size=batch * n, dtype=np.uint64).astype(np.uint32)
        d_in = torch.from_numpy(vals.view(np.int32)).cuda()
        ref = torch.zeros(batch * n * blowup, dtype=torch.int32, device="cuda")
        out = torch.full((batch * n * blowup,), -1, dtype=torch.int32, device="cuda")
        torch.cuda.synchronize()
        rc = L.z0p_gpu_rs_extend(gpu_ctx.handle, C.c_void_p(d_in.data_ptr()), n, batch, blowup,
                                 C.c_void_p(ref.data_ptr()))
        assert rc == 0, L.z0p_gpu_last_reason()
        rc = noalloc(C.c_void_p(d_in.data_ptr()), n, batch, blowup, C.c_void_p(out.data_ptr()),
                     C.c_void_p(stream.cuda_stream))
        assert rc == 0, L.z0p_gpu_last_reason()
        stream.synchronize()
        assert torch.equal(out, ref), (logn, batch, blowup)
        got = out.cpu().numpy().view(np.uint32).reshape(batch, n * blowup)
        for b in range(batch):
            want = oracle.reed_solomon_extend(vals[b * n:(b + 1) * n], blowup)
            assert np.array_equal(got[b], want), (logn, batch, blowup, b)


def test_noalloc_rejects_sizes_above_limit(z0p):
    torch = pytest.importorskip("torch")
    L, noalloc = _bind(z0p)
    d = torch.zeros(1 << 16, dtype=torch.int32, device="cuda")
    o = torch.zeros(1 << 16, dtype=torch.int32, device="cuda")
    # 2^16 * 4 * 8 = 2^21 > 2^20 output elements: refused before any launch.
    rc = noalloc(C.c_void_p(d.data_ptr()), 1 << 16, 4, 8, C.c_void_p(o.data_ptr()), None)
    assert rc == 103
    assert b"static scratch limit" in L.z0p_gpu_last_reason()
    # batch * blowup above one launch's 65535 transforms: z0p_gpu_rs_extend's code.
    rc = noalloc(C.c_void_p(d.data_ptr()), 2, 1 << 14, 4, C.c_void_p(o.data_ptr()), None)
    assert rc == 3
