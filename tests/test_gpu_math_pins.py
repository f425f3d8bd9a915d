"""The device path against direct mathematics (GPU), independently of the
oracle.

The byte-identity tests compare the device with the oracle, a restatement
of the reference. These compare the device with the definitions the
reference's own tests check its algorithms against, written in numpy
(tests/fieldmath.py):
  * the coset LDE against Horner / Lagrange evaluation of the interpolant
    at 31 * omega_m^k (src/ntt.rs:477-507, 548-575): every point for
    n <= 2^12, and at 2^20 4096 sampled points of a sparse polynomial plus
    eight points of a dense one;
  * the composition layer against composition_at written from its
    definition (src/air.rs:938-962; the reference's batched-vs-scalar test
    is src/air.rs:1155-1242). The device evaluates only on the 31-coset,
    where x - 1, x - w_last and x^n - 1 never vanish (31^n has odd order
    15 * 2^(27 - log n) > 1 in the multiplicative group, so x^n = 31^n *
    omega^(jn) is not 1), so the singular rows of the reference's unit-
    domain case cannot arise on the device; that case is pinned on the
    oracle in tests/test_math_pins.py;
  * the fold against the fold of a polynomial on the materialized point
    layers (src/fri.rs:1481-1505): the device's fold of P's evaluations
    on layer d must be Q = A + r0 B + r1 C + r2 D on layer d + 1.
"""
import ctypes as C

import numpy as np
import pytest

import fieldmath as F

pytestmark = pytest.mark.gpu


def _dev(a):
    import torch

    return torch.from_numpy(np.ascontiguousarray(np.asarray(a, dtype=np.uint32)).view(np.int32)).cuda()


def _host(t):
    return t.cpu().numpy().view(np.uint32).astype(np.uint64)


def _rs_extend(z0p, ctx, values, blowup):
    import torch

    n = len(values)
    d_in = _dev(values)
    d_out = torch.empty(n * blowup, dtype=torch.int32, device="cuda")
    torch.cuda.synchronize()
    rc = z0p.lib().z0p_gpu_rs_extend(ctx.handle, C.c_void_p(d_in.data_ptr()), n, 1, blowup,
                                     C.c_void_p(d_out.data_ptr()))
    assert rc == 0, z0p.lib().z0p_gpu_last_reason()
    return _host(d_out)


@pytest.mark.parametrize("logn,blowup", [(0, 2), (3, 4), (7, 16), (10, 8), (12, 16), (13, 4)])
def test_lde_matches_horner_every_point(z0p, gpu_ctx, logn, blowup):
    pytest.importorskip("torch")
    n = 1 << logn
    rng = np.random.default_rng(1000 + logn)
    v = rng.integers(0, F.P, size=n, dtype=np.uint64)
    got = _rs_extend(z0p, gpu_ctx, v, blowup)
    logm = logn + blowup.bit_length() - 1
    pts = F.powers(F.root(logm), n * blowup, F.GEN)
    assert np.array_equal(got, F.horner(F.dft_inverse(v), pts))


def test_lde_2p20_sparse_polynomial_at_4096_points(z0p, gpu_ctx):
    pytest.importorskip("torch")
    logn, blowup = 20, 16
    n, logm = 1 << logn, logn + 4
    rng = np.random.default_rng(20)
    exps = np.unique(np.concatenate([[0, 1, n - 1, n // 2],
                                     rng.integers(0, n, size=60, dtype=np.int64)]))
    coef = rng.integers(1, F.P, size=len(exps), dtype=np.uint64)
    w = F.root(logn)
    values = np.zeros(n, dtype=np.uint64)
    for e, c in zip(exps, coef):  # values on <omega_n>: sum_t c_t omega^(k e_t)
        values = (values + F.powers(F.pow_scalar(w, int(e)), n) * c) % F._P
    got = _rs_extend(z0p, gpu_ctx, values, blowup)
    k = np.unique(np.concatenate([[0, 1, 15, 16, (n << 4) - 1],
                                  rng.integers(0, n << 4, size=4091, dtype=np.int64)]))
    x = F.mul(F.pow_vec(np.full(len(k), F.root(logm), dtype=np.uint64), k.astype(np.uint64)), F.GEN)
    want = np.zeros(len(k), dtype=np.uint64)
    for e, c in zip(exps, coef):
        want = (want + F.pow_vec(x, int(e)) * c) % F._P
    assert np.array_equal(got[k], want)


def test_lde_2p20_dense_values_barycentric(z0p, gpu_ctx):
    pytest.importorskip("torch")
    logn, blowup = 20, 16
    n, logm = 1 << logn, logn + 4
    rng = np.random.default_rng(21)
    v = rng.integers(0, F.P, size=n, dtype=np.uint64)
    got = _rs_extend(z0p, gpu_ctx, v, blowup)
    k = np.array([0, 1, 17, (n << 4) - 1, 123456, 7 << 20, 9999999, (n << 4) // 3], dtype=np.int64)
    x = F.mul(F.pow_vec(np.full(len(k), F.root(logm), dtype=np.uint64), k.astype(np.uint64)), F.GEN)
    assert np.array_equal(got[k], F.barycentric(v, x))


def _compose(z0p, ctx, params, alphas):
    import torch

    m = params.n_steps * params.blowup
    out = torch.empty(4 * m, dtype=torch.int32, device="cuda")
    al = (C.c_uint32 * 20)(*[int(a) for a in np.asarray(alphas).reshape(-1)])
    torch.cuda.synchronize()
    rc = z0p.lib().z0p_gpu_air_compose(ctx.handle, C.byref(params), al, C.c_void_p(out.data_ptr()))
    assert rc == 0, z0p.lib().z0p_gpu_last_reason()
    return _host(out).reshape(m, 4)


# (n, blowup, queries, final): valid air::Params shapes
COMPOSE_SHAPES = [(4, 4, 4, 4), (16, 8, 8, 8), (64, 8, 12, 8), (256, 16, 8, 16), (1024, 16, 40, 16),
                  (1 << 12, 4, 8, 16)]


@pytest.mark.parametrize("shape", COMPOSE_SHAPES, ids=[f"n{s[0]}_B{s[1]}" for s in COMPOSE_SHAPES])
@pytest.mark.parametrize("honest", [True, False])
def test_compose_matches_composition_at_every_row(z0p, gpu_ctx, shape, honest):
    pytest.importorskip("torch")
    n, B, q, fin = shape
    rng = np.random.default_rng(n * 7 + B + honest)
    a0, b0 = (int(x) for x in rng.integers(0, F.P, size=2))
    ta, tb = F.fib_trace(a0, b0, n)
    b_last = int(tb[-1]) if honest else (int(tb[-1]) + 3) % F.P
    params = z0p.air.Params.new(n, B, q, fin, a0, b0, b_last)
    alphas = rng.integers(0, F.P, size=(5, 4), dtype=np.uint64)
    layer0 = _compose(z0p, gpu_ctx, params, alphas)
    m, logn = n * B, n.bit_length() - 1
    logm = (m).bit_length() - 1
    x = F.powers(F.root(logm), m, F.GEN)          # row k at 31 * omega_m^k
    xn = F.mul(x, F.root(logn))                   # next trace row: omega_n x
    ca, cb = F.dft_inverse(ta), F.dft_inverse(tb)
    want = F.composition_at(F.horner(ca, x), F.horner(cb, x), F.horner(ca, xn), F.horner(cb, xn),
                            x, n, a0, b0, b_last, alphas)
    rows = F.brev(np.arange(m), logm)             # layer-0 position P holds row brev(P)
    assert np.array_equal(layer0, want[rows])


def test_compose_2p14_sampled_rows(z0p, gpu_ctx):
    pytest.importorskip("torch")
    n, B = 1 << 14, 16
    rng = np.random.default_rng(14)
    a0, b0 = (int(x) for x in rng.integers(0, F.P, size=2))
    ta, tb = F.fib_trace(a0, b0, n)
    params = z0p.air.Params.for_security(n, a0, b0, int(tb[-1]), 100)
    alphas = rng.integers(0, F.P, size=(5, 4), dtype=np.uint64)
    layer0 = _compose(z0p, gpu_ctx, params, alphas)
    m, logm = n * B, 18
    pos = np.unique(np.concatenate([[0, 1, m - 1], rng.integers(0, m, size=61)])).astype(np.uint64)
    rows = F.brev(pos, logm)
    x = F.mul(F.pow_vec(np.full(len(rows), F.root(logm), dtype=np.uint64), rows), F.GEN)
    xn = F.mul(x, F.root(14))
    want = F.composition_at(F.barycentric(ta, x), F.barycentric(tb, x), F.barycentric(ta, xn),
                            F.barycentric(tb, xn), x, n, a0, b0, int(tb[-1]), alphas)
    assert np.array_equal(layer0[pos.astype(np.int64)], want)


def _fold(z0p, ctx, vals, lde_len, depth, ch):
    import torch

    n = len(vals)
    d_in = _dev(vals.reshape(-1))
    d_out = torch.empty(n, dtype=torch.int32, device="cuda")  # n/4 Ext4 values
    cha = (C.c_uint32 * 12)(*[int(c) for c in ch.reshape(-1)])
    torch.cuda.synchronize()
    rc = z0p.lib().z0p_gpu_fri_fold(ctx.handle, C.c_void_p(d_in.data_ptr()), n, lde_len, depth, cha,
                                    C.c_void_p(d_out.data_ptr()))
    assert rc == 0, z0p.lib().z0p_gpu_last_reason()
    return _host(d_out).reshape(-1, 4)


@pytest.mark.parametrize("logm,depth", [(4, 0), (8, 1), (10, 0), (12, 2), (14, 1), (16, 2), (18, 3)])
def test_fold_of_polynomial_on_materialized_layers(z0p, gpu_ctx, logm, depth):
    pytest.importorskip("torch")
    layers = F.layer_points(logm, depth + 1)
    pts, nxt = layers[depth], layers[depth + 1]
    n = len(pts)
    rng = np.random.default_rng(logm * 10 + depth)
    coeffs = rng.integers(0, F.P, size=(n, 4), dtype=np.uint64)  # full degree < n
    ch = rng.integers(0, F.P, size=(3, 4), dtype=np.uint64)
    got = _fold(z0p, gpu_ctx, F.e_horner(coeffs, pts), 1 << logm, depth, ch)
    assert np.array_equal(got, F.e_horner(F.fold_poly(coeffs, ch), nxt))


def test_fold_2p22_layer_low_degree_polynomial(z0p, gpu_ctx):
    # A layer of 2^22 values at depth 1 of an LDE of 2^24 (the x^-1 of every
    # quad comes from the device's twiddle tables at full size).
    pytest.importorskip("torch")
    logm, depth = 24, 1
    layers = F.layer_points(logm, depth + 1)
    pts, nxt = layers[depth], layers[depth + 1]
    rng = np.random.default_rng(2224)
    coeffs = rng.integers(0, F.P, size=(64, 4), dtype=np.uint64)
    ch = rng.integers(0, F.P, size=(3, 4), dtype=np.uint64)
    got = _fold(z0p, gpu_ctx, F.e_horner(coeffs, pts), 1 << logm, depth, ch)
    assert np.array_equal(got, F.e_horner(F.fold_poly(coeffs, ch), nxt))
