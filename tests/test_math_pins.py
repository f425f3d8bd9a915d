"""The oracle against direct mathematics (CPU).

These restate the reference's own checks of its algorithms against the
definitions they compute, with the definitions written independently in
numpy (tests/fieldmath.py), so that a convention error the oracle's prover
and its restated verifier shared (coset shift, root of unity, bit reversal,
quad order, fold formula, composition terms) would show here:
  * ntt_matches_horner, coset_matches_horner and the large spot check
    (src/ntt.rs:477-507, 548-575);
  * batched_compose_matches_scalar (src/air.rs:1155-1242), with the
    composition also written from its definition (src/air.rs:938-962);
  * on_demand_point_at_matches_materialized_layers (src/fri.rs:1481-1505),
    here as the fold of a polynomial's evaluations on the materialized
    layers, which must be the folded polynomial's evaluations on the next
    layer (the closed form of src/fri.rs:1304-1331).
The same pins run against the device in tests/test_gpu_math_pins.py.
"""
import numpy as np
import pytest

import fieldmath as F


def _seeded(oracle, seed, n):
    out = np.empty(n, dtype=np.uint64)
    s = seed
    for i in range(n):
        z, s = oracle.splitmix64(s)
        out[i] = z % F.P
    return out


def test_ntt_forward_matches_horner(oracle):
    # src/ntt.rs:477-490
    for logn in (0, 1, 5, 9):
        n = 1 << logn
        c = _seeded(oracle, 0x1111222233334444 + logn, n)
        got = oracle.ntt_forward(c).astype(np.uint64)
        pts = F.powers(F.root(logn), n)
        assert np.array_equal(got, F.horner(c, pts)), logn


def test_coset_matches_horner(oracle):
    # src/ntt.rs:492-507: n = 8, blowup 4, shift GENERATOR; and larger shapes
    for logn, blowup in [(3, 4), (6, 2), (8, 16), (10, 8)]:
        n = 1 << logn
        c = _seeded(oracle, 0x5555666677778888 + logn, n)
        got = oracle.evaluate_on_coset(c, blowup).astype(np.uint64)
        logm = logn + blowup.bit_length() - 1
        pts = F.powers(F.root(logm), n * blowup, F.GEN)
        assert np.array_equal(got, F.horner(c, pts)), (logn, blowup)


def test_reed_solomon_extend_matches_interpolant(oracle):
    # reed_solomon_extend = interpolate then the 31-coset (src/ntt.rs:436-439):
    # every output is the values' interpolant at 31 * omega_m^k.
    for logn, blowup in [(0, 4), (2, 2), (7, 16), (10, 4)]:
        n = 1 << logn
        v = _seeded(oracle, 0x9999AAAABBBBCCCC + logn, n)
        got = oracle.reed_solomon_extend(v, blowup).astype(np.uint64)
        coeffs = F.dft_inverse(v)
        logm = logn + blowup.bit_length() - 1
        pts = F.powers(F.root(logm), n * blowup, F.GEN)
        assert np.array_equal(got, F.horner(coeffs, pts)), (logn, blowup)
        # the barycentric form agrees at a few points (it is used at 2^20 on the GPU)
        k = np.array([0, 1, n * blowup - 1, (n * blowup) // 3], dtype=np.int64)
        assert np.array_equal(got[k], F.barycentric(v, pts[k])), (logn, blowup)


def _compose_case(oracle):
    # src/air.rs:1158-1180: n = 16, m = 8n, splitmix64 columns, cols[0][0] = 0
    n, m = 16, 128
    draws = _seeded(oracle, 0x123456789ABCDEF1, 2 * m)
    a = draws[0::2].copy()
    b = draws[1::2].copy()
    a[0] = 0
    alphas = np.array([[1, 0, 0, 0], [2, 0, 0, 0], [3, 0, 0, 0], [4, 0, 0, 0], [5, 0, 0, 0]],
                      dtype=np.uint64)
    return n, m, a, b, alphas


@pytest.mark.parametrize("domain", ["lde", "unit"])
def test_batched_compose_matches_scalar_and_definition(oracle, domain):
    n, m, a, b, alphas = _compose_case(oracle)
    offset = 5  # not a divisor of m: the wrap-around is exercised
    logm = m.bit_length() - 1
    if domain == "lde":
        pts = F.powers(F.root(logm), m, F.GEN)
    else:  # rows at 1 and w_last hit zero denominators; every n-th root zeroes x^n - 1
        pts = F.powers(F.root(logm), m)
    w_last = F.pow_scalar(F.root(n.bit_length() - 1), n - 1)
    a0, b0, b_last = 1, 1, 2
    batched = oracle.air_compose(a, b, pts, w_last, a0, b0, b_last, n, offset, alphas)
    nx = (np.arange(m) + offset) % m
    for i in range(m):
        scalar = oracle.air_composition_at(int(a[i]), int(b[i]), int(a[nx[i]]), int(b[nx[i]]),
                                           int(pts[i]), w_last, a0, b0, b_last, n, alphas)
        assert np.array_equal(batched[i], scalar), i
    direct = F.composition_at(a, b, a[nx], b[nx], pts, n, a0, b0, b_last, alphas)
    assert np.array_equal(batched.astype(np.uint64), direct)
    if domain == "unit":
        assert (pts == 1).any() and (pts == w_last).any()


def test_fold_layer_folds_the_polynomial(oracle):
    # Layer d of an LDE of length 2^logm holds the evaluations of P on the
    # materialized point layer d; the oracle's fold with the point_at leaders
    # must give Q = A + r0 B + r1 C + r2 D on layer d + 1.
    rng = np.random.default_rng(7)
    for logm, depth in [(4, 0), (6, 1), (8, 0), (8, 2), (10, 1), (12, 3)]:
        layers = F.layer_points(logm, depth + 1)
        pts, nxt = layers[depth], layers[depth + 1]
        n = len(pts)
        coeffs = rng.integers(0, F.P, size=(n, 4), dtype=np.uint64)
        vals = F.e_horner(coeffs, pts)
        ch = rng.integers(0, F.P, size=(3, 4), dtype=np.uint64)
        got, _ = oracle.fold_layer(vals.reshape(-1), pts[0::4], ch.reshape(-1))
        want = F.e_horner(F.fold_poly(coeffs, ch), nxt)
        assert np.array_equal(got.reshape(-1, 4).astype(np.uint64), want), (logm, depth)
        # the quad of leader x is (x, -x, j0 x, -j0 x), j0 = omega_4 (src/fri.rs:1266-1272)
        j0 = F.root(2)
        x = pts[0::4]
        assert np.array_equal(pts[1::4], F.sub(0, x))
        assert np.array_equal(pts[2::4], F.mul(x, j0))
        assert np.array_equal(pts[3::4], F.sub(0, F.mul(x, j0)))


def test_fieldmath_against_reference_identities(oracle):
    # The numpy field itself: 2 * 1006632961 = 1 (src/babybear.rs:379),
    # root orders (src/babybear.rs:402-412), Fp4 against the oracle's product.
    assert F.mul(2, 1006632961) == 1
    for k in (1, 2, 10, 27):
        w = F.root(k)
        assert F.pow_scalar(w, 1 << k) == 1 and F.pow_scalar(w, 1 << (k - 1)) == F.P - 1
    rng = np.random.default_rng(3)
    x = rng.integers(0, F.P, size=(64, 4), dtype=np.uint64)
    y = rng.integers(0, F.P, size=(64, 4), dtype=np.uint64)
    prod = F.e_mul(x, y)
    for i in range(64):
        assert list(prod[i]) == list(oracle.e_mul(list(map(int, x[i])), list(map(int, y[i]))))
