"""The general two-column AIR prover on the GPU: air::prove_with_trace and
air::prove_zk (src/air.rs:381-464). Proof bytes, transcript post-states and
the ChaCha20 stream state equal the oracle's; the oracle's verifier accepts
honest and masked proofs; an honest trace proves to the same bytes as the
linked path (the reference's own linked_lde cross-check, src/air.rs:1013-1022)."""
import random

import pytest

pytestmark = pytest.mark.gpu

P = 2**31 - 2**27 + 1


def _params(z0p, oracle, n, blowup, q, final, grind=0, cap=0, a0=1, b0=1):
    _, b = oracle.build_trace(a0, b0, n)
    b_last = int(b[-1])
    pz = z0p.air.Params.new(n, blowup, q, final, a0, b0, b_last).with_grinding_bits(grind) \
        .with_cap_height(cap)
    po = oracle.air_params_new(n, blowup, q, final, a0, b0, b_last)
    po.grinding_bits, po.cap_height = grind, cap
    return pz, po


SHAPES = [(64, 8, 8, 8, 0, 0), (1 << 10, 16, 20, 16, 8, 3), (1 << 12, 4, 12, 4, 0, 2)]


@pytest.mark.parametrize("shape", SHAPES, ids=[f"n{s[0]}-B{s[1]}" for s in SHAPES])
def test_prove_with_trace_honest_equals_linked_and_oracle(z0p, oracle, gpu_ctx, shape):
    n, blowup, q, final, grind, cap = shape
    pz, po = _params(z0p, oracle, n, blowup, q, final, grind, cap, 5, 7)
    a, b = oracle.build_trace(5, 7, n)
    tg = z0p.Transcript(b"pwt")
    proof = z0p.air.prove_with_trace(pz, a, b, tg, gpu_ctx)
    to = oracle.Transcript(b"pwt")
    assert proof == oracle.air_prove_with_trace(po, a, b, to)
    assert tg.export() == to.export()
    assert proof == z0p.air.prove(pz, z0p.Transcript(b"pwt"), gpu_ctx)


def test_prove_with_trace_forged_columns(z0p, oracle, gpu_ctx):
    n = 256
    pz, po = _params(z0p, oracle, n, 16, 10, 16)
    rng = random.Random(11)
    a = [rng.randrange(P) for _ in range(n)]
    b = [rng.randrange(P) for _ in range(n)]
    tg, to = z0p.Transcript(b"forged"), oracle.Transcript(b"forged")
    proof = z0p.air.prove_with_trace(pz, a, b, tg, gpu_ctx)
    assert proof == oracle.air_prove_with_trace(po, a, b, to)
    assert tg.export() == to.export()
    assert oracle.air_verify(po, proof, oracle.Transcript(b"forged")) != 0


ZK = [
    # n, blowup, queries, final, grinding, cap, n_rand, key byte
    (32, 8, 4, 4, 0, 0, 64, 1),
    (64, 8, 8, 8, 4, 2, 128, 2),
    (1 << 10, 16, 12, 8, 6, 3, 192, 3),
    (1 << 12, 16, 40, 8, 0, 4, 640, 4),
]


@pytest.mark.parametrize("case", ZK, ids=[f"n{c[0]}-r{c[6]}" for c in ZK])
def test_prove_zk_matches_oracle(z0p, oracle, gpu_ctx, case):
    n, blowup, q, final, grind, cap, n_rand, kb = case
    pz, po = _params(z0p, oracle, n, blowup, q, final, grind, cap)
    key, nonce = bytes([kb]) * 32, bytes([kb + 1]) * 12
    rz, ro = z0p.rng.ChaCha20.new(key, nonce), oracle.ChaCha20.new(key, nonce)
    tg, to = z0p.Transcript(b"zk"), oracle.Transcript(b"zk")
    proof = z0p.air.prove_zk(pz, n_rand, rz, tg, gpu_ctx)
    assert proof == oracle.air_prove_zk(po, n_rand, ro, to)
    assert tg.export() == to.export()
    assert (bytes(rz.block), rz.counter, rz.used) == (bytes(ro.block), ro.counter, ro.used)
    assert oracle.air_verify(po, proof, oracle.Transcript(b"zk")) == 0


def test_zk_errors_leave_transcript_and_stream(z0p, oracle, gpu_ctx):
    pz, _ = _params(z0p, oracle, 32, 8, 4, 4)
    rz = z0p.rng.ChaCha20.new(bytes(32), bytes(12))
    t = z0p.Transcript(b"zk-err")
    before_t, before_r = t.export(), rz.export()
    with pytest.raises(z0p.Z0pError) as e:
        z0p.air.prove_zk(pz, 63, rz, t, gpu_ctx)  # 16 * num_queries = 64
    assert e.value.code == 8
    assert t.export() == before_t and rz.export() == before_r
    a, b = oracle.build_trace(1, 1, 32)
    for cols, code in [((list(a)[:16], list(b)[:16]), 8), ((list(a)[:31] + [P], list(b)), 8)]:
        with pytest.raises(z0p.Z0pError) as e:
            z0p.air.prove_with_trace(pz, cols[0], cols[1], t, gpu_ctx)
        assert e.value.code == code
        assert t.export() == before_t
