"""The kernel-sweep configuration at its full column sizes: one column of
2^20 and one of 2^22 from the sweep's splitmix64 stream, extended at blowup
16 (2^24 and 2^26 points); the LDE, the Merkle cap of the column's flat
buffer and the first fold layer equal the oracle's."""
import ctypes as C
import os
import sys

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)


def _brev(logm):
    import torch

    i = torch.arange(1 << logm, device="cuda", dtype=torch.int64)
    r = torch.zeros_like(i)
    for b in range(logm):
        r |= ((i >> b) & 1) << (logm - 1 - b)
    return r


def _points(oracle, logm):
    # quad-leader points 31 * omega^brev(4 i) for i < m / 4 (fri.rs:1086-1094), vectorised
    P = np.uint64(oracle.P)
    m = 1 << logm
    idx = np.arange(m // 4, dtype=np.uint64) * np.uint64(4)
    rev = np.zeros_like(idx)
    for b in range(logm):
        rev |= ((idx >> np.uint64(b)) & np.uint64(1)) << np.uint64(logm - 1 - b)
    w = oracle.f_pow(31, (oracle.P - 1) >> logm)
    acc = np.ones(m // 4, dtype=np.uint64)
    sq = np.uint64(w)
    for b in range(logm):
        bit = ((rev >> np.uint64(b)) & np.uint64(1)).astype(bool)
        acc[bit] = acc[bit] * sq % P
        sq = sq * sq % P
    return (acc * np.uint64(31) % P).astype(np.uint32)


@pytest.mark.parametrize("logn", [20, 22])
def test_full_size_column_matches_oracle(z0p, oracle, gpu_ctx, logn):
    torch = pytest.importorskip("torch")
    import bench

    n, B = 1 << logn, 16
    m, logm = n * B, logn + 4
    vals = bench.sweep_values(12345, n)
    d_in = torch.from_numpy(vals.view(np.int32)).cuda()
    d_lde = torch.empty(m, dtype=torch.int32, device="cuda")
    torch.cuda.synchronize()
    L = z0p.lib()
    assert L.z0p_gpu_rs_extend(gpu_ctx.handle, C.c_void_p(d_in.data_ptr()), n, 1, B,
                               C.c_void_p(d_lde.data_ptr())) == 0
    lde = d_lde.cpu().numpy().view(np.uint32)
    assert np.array_equal(lde, oracle.reed_solomon_extend(vals, B))
    out = (C.c_uint8 * (32 * 16))()
    cnt = C.c_uint64()
    assert L.z0p_gpu_merkle_flat64_cap(gpu_ctx.handle, C.c_void_p(d_lde.data_ptr()), 4 * m, 4, out,
                                       C.byref(cnt)) == 0
    assert bytes(out)[:32 * cnt.value] == oracle.merkle_flat64_cap(lde.tobytes(), 4)
    lifted = torch.zeros(4 * m, dtype=torch.int32, device="cuda")
    lifted[0::4] = d_lde[_brev(logm)]
    nxt = torch.empty(m, dtype=torch.int32, device="cuda")
    ch = [(7 * i + 3) % oracle.P for i in range(12)]
    torch.cuda.synchronize()
    assert L.z0p_gpu_fri_fold(gpu_ctx.handle, C.c_void_p(lifted.data_ptr()), m, m, 0,
                              (C.c_uint32 * 12)(*ch), C.c_void_p(nxt.data_ptr())) == 0
    ref, _ = oracle.fold_layer(lifted.cpu().numpy().view(np.uint32), _points(oracle, logm),
                               np.array(ch, dtype=np.uint32))
    assert np.array_equal(nxt.cpu().numpy().view(np.uint32), ref)
