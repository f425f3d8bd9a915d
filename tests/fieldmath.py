"""Direct BabyBear / Fp4 mathematics in numpy, for parity pins that do not go
through the oracle's restatement.

Everything here follows the field definitions, not the reference's
algorithms:
  * p = 2^31 - 2^27 + 1 (src/babybear.rs:26), generator 31 (:36), and the
    root of unity of order 2^k is 31^((p - 1) / 2^k) (:183-208);
  * Fp4 = Fp2[v] / (v^2 - u), Fp2 = Fp[u] / (u^2 - 11), an element
    a + b u + c v + d uv stored as [a, b, c, d] (src/ext4.rs:1-30),
    multiplied here schoolbook-style in that basis;
  * inverses by Fermat's little theorem (x^(p-2), 0 -> 0);
  * polynomial evaluation by Horner's rule or, where the coefficients are
    not at hand, by the barycentric Lagrange formula on the subgroup
    <omega_n>: P(x) = (x^n - 1) / n * sum_i v_i omega^i / (x - omega^i).
Arrays are numpy uint64 holding canonical values (< p); every product of
two canonical values fits in 62 bits.
"""
import numpy as np

P = 2013265921
GEN = 31
_P = np.uint64(P)


def mul(a, b):
    return (np.asarray(a, dtype=np.uint64) * np.asarray(b, dtype=np.uint64)) % _P


def add(a, b):
    return (np.asarray(a, dtype=np.uint64) + np.asarray(b, dtype=np.uint64)) % _P


def sub(a, b):
    return (np.asarray(a, dtype=np.uint64) + _P - np.asarray(b, dtype=np.uint64)) % _P


def pow_scalar(x: int, e: int) -> int:
    return pow(int(x) % P, int(e), P)


def pow_vec(x, e):
    """x^e elementwise; e a non-negative int or an array of them."""
    x = np.asarray(x, dtype=np.uint64) % _P
    e = np.broadcast_to(np.asarray(e, dtype=np.uint64), x.shape).copy()
    acc = np.ones_like(x)
    base = x.copy()
    while np.any(e):
        bit = (e & np.uint64(1)).astype(bool)
        acc[bit] = acc[bit] * base[bit] % _P
        base = base * base % _P
        e >>= np.uint64(1)
    return acc


def inv_vec(x):
    """Fermat inverse, with 0 -> 0 (src/babybear.rs:167-169)."""
    return pow_vec(x, P - 2)


def root(logn: int) -> int:
    """Generator of the subgroup of order 2^logn."""
    return pow_scalar(GEN, (P - 1) >> logn)


def powers(w: int, n: int, start: int = 1):
    """[start * w^i for i < n] by repeated doubling of a vector (no chain)."""
    out = np.empty(n, dtype=np.uint64)
    out[0] = start % P
    k = 1
    while k < n:
        step = pow_scalar(w, k)
        t = min(k, n - k)
        out[k:k + t] = out[:t] * np.uint64(step) % _P
        k += t
    return out


def brev(i, bits: int):
    i = np.asarray(i, dtype=np.uint64)
    r = np.zeros_like(i)
    for b in range(bits):
        r |= ((i >> np.uint64(b)) & np.uint64(1)) << np.uint64(bits - 1 - b)
    return r


def horner(coeffs, x):
    """sum_i c_i x^i at every point of x (coefficients ascending)."""
    x = np.asarray(x, dtype=np.uint64)
    acc = np.zeros_like(x)
    for c in np.asarray(coeffs, dtype=np.uint64)[::-1]:
        acc = (acc * x + c) % _P
    return acc


def dft_inverse(values):
    """Coefficients of the interpolant of values on <omega_n>, by the direct
    O(n^2) sum c_i = n^-1 sum_k v_k omega^(-ik)."""
    v = np.asarray(values, dtype=np.uint64)
    n = len(v)
    logn = n.bit_length() - 1
    winv = pow_scalar(root(logn), P - 2)
    tab = powers(winv, n)
    k = np.arange(n, dtype=np.uint64)
    ninv = pow_scalar(n, P - 2)
    out = np.empty(n, dtype=np.uint64)
    for i in range(n):
        row = tab[(k * np.uint64(i)) % np.uint64(n)]
        out[i] = int(np.sum(v * row % _P) % _P) * ninv % P
    return out


def barycentric(values, x, chunk: int = 1 << 22):
    """The interpolant of values on <omega_n> evaluated at points x, none of
    which lies in <omega_n>."""
    v = np.asarray(values, dtype=np.uint64)
    n = len(v)
    logn = n.bit_length() - 1
    w = powers(root(logn), n)
    vw = v * w % _P
    ninv = pow_scalar(n, P - 2)
    out = np.empty(len(x), dtype=np.uint64)
    per = max(1, chunk // n)
    for s in range(0, len(x), per):
        xs = np.asarray(x[s:s + per], dtype=np.uint64)
        den = (xs[:, None] + _P - w[None, :]) % _P
        inv = inv_vec(den)
        acc = np.sum(vw[None, :] * inv % _P, axis=1) % _P
        van = sub(pow_vec(xs, n), 1)
        out[s:s + per] = acc * van % _P * np.uint64(ninv) % _P
    return out


# ------------------------------------------------------------------ Fp4 ----
def e_mul(x, y):
    """Fp4 product of arrays of shape (..., 4), schoolbook in the basis
    {1, u, v, uv} with u^2 = 11 and v^2 = u."""
    x = np.asarray(x, dtype=np.uint64)
    y = np.asarray(y, dtype=np.uint64)
    a, b, c, d = (x[..., i] for i in range(4))
    e, f, g, h = (y[..., i] for i in range(4))
    m = lambda s, t: s * t % _P  # noqa: E731
    eleven = np.uint64(11)
    # (X0 + X1 v)(Y0 + Y1 v) = X0 Y0 + u X1 Y1 + (X0 Y1 + X1 Y0) v, X0 = a + b u, ...
    # Fp2: (s0 + s1 u)(t0 + t1 u) = s0 t0 + 11 s1 t1 + (s0 t1 + s1 t0) u
    x0y0_0 = (m(a, e) + eleven * m(b, f)) % _P
    x0y0_1 = (m(a, f) + m(b, e)) % _P
    x1y1_0 = (m(c, g) + eleven * m(d, h)) % _P
    x1y1_1 = (m(c, h) + m(d, g)) % _P
    # u * (s0 + s1 u) = 11 s1 + s0 u
    r0 = (x0y0_0 + eleven * x1y1_1) % _P
    r1 = (x0y0_1 + x1y1_0) % _P
    r2 = (m(a, g) + eleven * m(b, h) + m(c, e) + eleven * m(d, f)) % _P
    r3 = (m(a, h) + m(b, g) + m(c, f) + m(d, e)) % _P
    return np.stack([r0, r1, r2, r3], axis=-1)


def e_mul_base(x, s):
    x = np.asarray(x, dtype=np.uint64)
    return x * np.asarray(s, dtype=np.uint64)[..., None] % _P


def e_horner(coeffs, x):
    """sum_i c_i x^i for Fp4 coefficients (n, 4) at base-field points x."""
    x = np.asarray(x, dtype=np.uint64)
    acc = np.zeros(x.shape + (4,), dtype=np.uint64)
    for c in np.asarray(coeffs, dtype=np.uint64)[::-1]:
        acc = (acc * x[..., None] + c) % _P
    return acc


# -------------------------------------------------------- AIR definition ----
def fib_trace(a0: int, b0: int, n: int):
    """A[i+1] = B[i], B[i+1] = A[i] + B[i] (src/air.rs:341-354)."""
    a = np.empty(n, dtype=np.uint64)
    b = np.empty(n, dtype=np.uint64)
    x, y = a0 % P, b0 % P
    for i in range(n):
        a[i], b[i] = x, y
        x, y = y, (x + y) % P
    return a, b


def composition_at(a, b, an, bn, x, n, a0, b0, b_last, alphas):
    """The AIR composition at points x (src/air.rs:938-962), written from its
    definition: the transition constraints divided by the transition
    vanishing polynomial (x^n - 1) / (x - w_last), the boundary constraints
    by x - 1 and x - w_last, combined with the Fp4 alphas (5, 4)."""
    logn = n.bit_length() - 1
    w_last = pow_scalar(root(logn), n - 1)
    x = np.asarray(x, dtype=np.uint64)
    z_trans = mul(sub(pow_vec(x, n), 1), inv_vec(sub(x, w_last)))
    iz = inv_vec(z_trans)
    terms = [
        mul(sub(an, b), iz),
        mul(sub(bn, add(a, b)), iz),
        mul(sub(a, a0), inv_vec(sub(x, 1))),
        mul(sub(b, b0), inv_vec(sub(x, 1))),
        mul(sub(b, b_last), inv_vec(sub(x, w_last))),
    ]
    out = np.zeros(x.shape + (4,), dtype=np.uint64)
    for t, al in zip(terms, np.asarray(alphas, dtype=np.uint64)):
        out = (out + t[..., None] * al[None, :]) % _P
    return out


def fold_poly(coeffs, ch):
    """The arity-4 fold of a polynomial (src/fri.rs:1304-1331 in closed form):
    P(X) = A(X^4) + X B(X^4) + X^2 C(X^4) + X^3 D(X^4) folds to
    A + r0 B + r1 C + r2 D. coeffs (n, 4) Fp4, ch (3, 4)."""
    c = np.asarray(coeffs, dtype=np.uint64)
    parts = [c[k::4] for k in range(4)]
    out = parts[0].copy()
    for k in range(3):
        out = (out + e_mul(parts[k + 1], np.broadcast_to(ch[k], parts[k + 1].shape))) % _P
    return out


def layer_points(logm: int, depths: int):
    """The materialized FRI point layers: layer 0 is the bit-reversed coset
    31 * <omega_m>, and layer d+1 holds the fourth powers of layer d's every
    fourth point (src/fri.rs:1481-1505)."""
    m = 1 << logm
    coset = powers(root(logm), m, GEN)
    layers = [coset[brev(np.arange(m), logm)]]
    for _ in range(depths):
        q = layers[-1][0::4]
        layers.append(pow_vec(q, 4))
    return layers
