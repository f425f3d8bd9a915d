"""range::prove on its constant trace (compact trees and per-coset FRI
layers) and range::prove_with_columns (row by row) on the GPU: both equal
the oracle, which transforms and hashes every row; constant columns proved
through either path give the same bytes."""
import random

import pytest

pytestmark = pytest.mark.gpu

P = 2**31 - 2**27 + 1

CASES = [
    # n_rows, n_bits, blowup, queries, final, grinding, cap, value
    (8, 16, 8, 8, 4, 0, 0, 12345),          # published `range 16-bit` shape; F < B, honest
    (2, 4, 8, 4, 4, 0, 0, 9),               # two rows, honest
    (1 << 10, 16, 16, 20, 16, 4, 3, 40000),
    (1 << 12, 8, 8, 12, 8, 0, 8, 255),      # cap above the uniform levels
    (64, 4, 8, 8, 8, 0, 0, 300),            # out of range, F = B
    (1 << 10, 8, 16, 12, 16, 2, 2, 70000),  # out of range, F = B = 16
    (256, 6, 32, 10, 128, 0, 5, 1 << 20),   # out of range, F = 4B
    (256, 6, 32, 10, 512, 0, 1, 33),        # honest, F = 16B
    (64, 4, 16, 8, 4, 0, 0, 300),           # out of range, F < B: row-by-row path
    (16, 3, 8, 6, 2, 0, 0, 5),              # F = 2: row-by-row path
    (1 << 14, 24, 16, 40, 16, 8, 4, P - 1),  # 24 bits, out of range
]


def _pair(z0p, oracle, case):
    n, bits, blowup, q, final, grind, cap, value = case
    pz = z0p.range.Params.new(n, bits, blowup, q, final, value).with_grinding_bits(grind) \
        .with_cap_height(cap)
    po = oracle.range_params_new(n, bits, blowup, q, final, value, grind, cap)
    return pz, po


def _columns(n, bits, value):
    return [value] * n, [[(value >> c) & 1] * n for c in range(bits)]


@pytest.mark.parametrize("case", CASES, ids=[f"n{c[0]}-b{c[1]}-B{c[2]}-F{c[4]}-v{c[7]}" for c in CASES])
def test_range_prove_matches_oracle(z0p, oracle, gpu_ctx, case):
    pz, po = _pair(z0p, oracle, case)
    tg, to = z0p.Transcript(b"rc"), oracle.Transcript(b"rc")
    proof = z0p.range.prove(pz, tg, gpu_ctx)
    assert proof == oracle.range_prove(po, to)
    assert tg.export() == to.export()
    honest = case[7] < (1 << case[1])
    assert (oracle.range_verify(po, proof, oracle.Transcript(b"rc")) == 0) == honest


@pytest.mark.parametrize("case", CASES[:8], ids=[f"n{c[0]}-v{c[7]}" for c in CASES[:8]])
def test_constant_columns_prove_the_same_through_both_paths(z0p, oracle, gpu_ctx, case):
    pz, _ = _pair(z0p, oracle, case)
    v, bits = _columns(case[0], case[1], case[7])
    a = z0p.range.prove(pz, z0p.Transcript(b"both"), gpu_ctx)
    b = z0p.range.prove_with_columns(pz, v, bits, z0p.Transcript(b"both"), gpu_ctx)
    assert a == b


@pytest.mark.parametrize("n,bits,blowup,final", [(64, 4, 8, 8), (1 << 10, 8, 16, 16), (256, 15, 4, 4)])
def test_prove_with_columns_matches_oracle(z0p, oracle, gpu_ctx, n, bits, blowup, final):
    rng = random.Random(n * 7 + bits)
    v = [rng.randrange(P) for _ in range(n)]
    cols = [[rng.randrange(2) if rng.random() < 0.9 else rng.randrange(P) for _ in range(n)]
            for _ in range(bits)]
    pz = z0p.range.Params.new(n, bits, blowup, 8, final, 77).with_cap_height(2)
    po = oracle.range_params_new(n, bits, blowup, 8, final, 77, 0, 2)
    tg, to = z0p.Transcript(b"cols"), oracle.Transcript(b"cols")
    proof = z0p.range.prove_with_columns(pz, v, cols, tg, gpu_ctx)
    assert proof == oracle.range_prove_with_columns(po, v, cols, to)
    assert tg.export() == to.export()
    assert oracle.range_verify(po, proof, oracle.Transcript(b"cols")) != 0


def test_prove_with_columns_errors(z0p, gpu_ctx):
    pz = z0p.range.Params.new(16, 3, 4, 6, 4, 5)
    v, bits = _columns(16, 3, 5)
    t = z0p.Transcript(b"cols-err")
    before = t.export()
    for vv, bb in [(v[:8], bits), (v, bits[:2]), (v, bits[:2] + [bits[2][:15]]),
                   (v[:15] + [P], bits), (v, bits[:2] + [[1] * 15 + [P + 3]])]:
        with pytest.raises(z0p.Z0pError) as e:
            z0p.range.prove_with_columns(pz, vv, bb, t, gpu_ctx)
        assert e.value.code == 8
        assert t.export() == before


def test_groups_mix_in_and_out_of_range_values(z0p, oracle, gpu_ctx):
    n = 1 << 10
    values = [5, 1 << 20, 65535, 70000, 0, P - 1]
    params = [z0p.range.Params.for_security(n, 16, v, 100) for v in values]
    ts = [z0p.Transcript(b"grp%d" % i) for i in range(len(values))]
    group = z0p.range.prove_group(params, ts, gpu_ctx)
    for i, v in enumerate(values):
        po = oracle.range_for_security(n, 16, v, 100)
        assert group[i] == oracle.range_prove(po, oracle.Transcript(b"grp%d" % i)), v
        assert group[i] == z0p.range.prove(params[i], z0p.Transcript(b"grp%d" % i), gpu_ctx)


@pytest.mark.parametrize("n,bits,blowup,final,n_rand,value", [
    (8, 4, 8, 8, 8, 5), (64, 8, 16, 32, 40, 200), (256, 16, 8, 16, 100, 300), (1 << 12, 16, 16, 32, 1 << 12, 1234)])
def test_range_prove_zk_matches_oracle(z0p, oracle, gpu_ctx, n, bits, blowup, final, n_rand, value):
    pz = z0p.range.Params.new(n, bits, blowup, 8, final, value).with_cap_height(2)
    po = oracle.range_params_new(n, bits, blowup, 8, final, value, 0, 2)
    key, nonce = bytes([n % 251]) * 32, bytes([3]) * 12
    rz, ro = z0p.rng.ChaCha20.new(key, nonce), oracle.ChaCha20.new(key, nonce)
    tg, to = z0p.Transcript(b"rzk"), oracle.Transcript(b"rzk")
    proof = z0p.range.prove_zk(pz, n_rand, rz, tg, gpu_ctx)
    assert proof == oracle.range_prove_zk(po, n_rand, ro, to)
    assert tg.export() == to.export()
    assert (bytes(rz.block), rz.counter, rz.used) == (bytes(ro.block), ro.counter, ro.used)
    assert (oracle.range_verify(po, proof, oracle.Transcript(b"rzk")) == 0) == (value < (1 << bits))


def test_range_prove_zk_errors_leave_state(z0p, gpu_ctx):
    pz = z0p.range.Params.new(64, 8, 16, 8, 32, 5)
    rz = z0p.rng.ChaCha20.new(bytes(32), bytes(12))
    t = z0p.Transcript(b"rzk-err")
    before_t, before_r = t.export(), rz.export()
    with pytest.raises(z0p.Z0pError) as e:
        z0p.range.prove_zk(pz, 7, rz, t, gpu_ctx)
    assert e.value.code == 8
    assert t.export() == before_t and rz.export() == before_r
