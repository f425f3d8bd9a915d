"""Proof groups (GPU): statements of one shape proved in lockstep.

Covers z0p_gpu_air_prove_group / z0p_gpu_range_prove_group of
include/z0p_gpu.h. Each proof of a group must equal the oracle's proof of
that statement alone (and the single-proof path's), and each transcript must
end in the oracle's post-state. Groups above the library's group limit are
split; a group of mixed shapes is refused before any device work and leaves
every transcript untouched.
"""
import pytest

pytestmark = pytest.mark.gpu


def _air_statements(z0p, oracle, n, count, seed, target=100, lie_at=None):
    P = oracle.P
    state = seed
    out = []
    for i in range(count):
        z1, state = oracle.splitmix64(state)
        z2, state = oracle.splitmix64(state)
        a0, b0 = z1 % P, z2 % P
        _, b_last = z0p.air.trace_last(a0, b0, n)
        if i == lie_at:
            b_last = (b_last + 1) % P  # a false claim still proves (src/air.rs:356-364)
        out.append((z0p.air.Params.for_security(n, a0, b0, b_last, target),
                    oracle.air_for_security(n, a0, b0, b_last, target)))
    return out


def test_air_group_matches_oracle_and_alone(z0p, oracle, gpu_ctx):
    for n, count in [(64, 3), (1 << 10, 5), (1 << 13, 4)]:
        stmts = _air_statements(z0p, oracle, n, count, 0x5EED000000000010 + n, lie_at=1)
        labels = [b"group/air-%d-%d" % (n, i) for i in range(count)]
        ts = [z0p.Transcript(l) for l in labels]
        ts[2 % count].absorb(b"prefix", b"p" * 1500)  # transcripts need not start alike
        proofs = z0p.air.prove_group([pz for pz, _ in stmts], ts, gpu_ctx)
        for i, ((pz, po), proof, t) in enumerate(zip(stmts, proofs, ts)):
            to = oracle.Transcript(labels[i])
            if i == 2 % count:
                to.absorb(b"prefix", b"p" * 1500)
            assert proof == oracle.air_prove(po, to), (n, i)
            assert t.export() == to.export(), (n, i)
            alone = z0p.Transcript(labels[i])
            if i == 2 % count:
                alone.absorb(b"prefix", b"p" * 1500)
            assert z0p.air.prove(pz, alone, gpu_ctx) == proof


def test_range_group_matches_oracle(z0p, oracle, gpu_ctx):
    values = [0, 1, 40000, 65535, 12345]
    pz = [z0p.range.Params.for_security(1 << 12, 16, v, 100) for v in values]
    po = [oracle.range_for_security(1 << 12, 16, v, 100) for v in values]
    ts = [z0p.Transcript(b"group/range-%d" % i) for i in range(len(values))]
    proofs = z0p.range.prove_group(pz, ts, gpu_ctx)
    for i, proof in enumerate(proofs):
        to = oracle.Transcript(b"group/range-%d" % i)
        assert proof == oracle.range_prove(po[i], to), i
        assert ts[i].export() == to.export()


def test_group_larger_than_the_limit_is_split(z0p, oracle, gpu_ctx):
    stmts = _air_statements(z0p, oracle, 16, 70, 0x5EED000000000020, target=32)
    ts = [z0p.Transcript(b"big-%d" % i) for i in range(len(stmts))]
    proofs = z0p.air.prove_group([pz for pz, _ in stmts], ts, gpu_ctx)
    for i in (0, 1, 63, 64, 69):
        assert proofs[i] == oracle.air_prove(stmts[i][1], oracle.Transcript(b"big-%d" % i)), i


def test_mixed_shapes_are_refused_untouched(z0p, oracle, gpu_ctx):
    a = z0p.air.Params.for_security(64, 1, 1, z0p.air.trace_last(1, 1, 64)[1], 100)
    b = z0p.air.Params.for_security(128, 1, 1, z0p.air.trace_last(1, 1, 128)[1], 100)
    ts = [z0p.Transcript(b"m0"), z0p.Transcript(b"m1")]
    before = [t.export() for t in ts]
    with pytest.raises(z0p.Z0pError) as e:
        z0p.air.prove_group([a, b], ts, gpu_ctx)
    assert e.value.code == 106
    assert [t.export() for t in ts] == before


def test_group_on_a_context_short_of_constant_slots(z0p, oracle):
    """When the process's constant slots run short, reserve_group reports
    OutOfMemory and keeps the old reservation, and a group call on that
    context is proved as smaller consecutive groups, byte for byte."""
    held = []
    short = None
    try:
        for _ in range(4):  # 168 slots: at most two ranges of 64 fit
            c = z0p.Context(0)
            held.append(c)
            try:
                c.reserve_group(64)
            except z0p.Z0pError as e:
                assert e.code == 102
                short = c
                break
        assert short is not None
        stmts = _air_statements(z0p, oracle, 64, 9, 0x5EED000000000030)
        ts = [z0p.Transcript(b"short-%d" % i) for i in range(len(stmts))]
        proofs = z0p.air.prove_group([pz for pz, _ in stmts], ts, short)
        for i, ((_, po), proof) in enumerate(zip(stmts, proofs)):
            assert proof == oracle.air_prove(po, oracle.Transcript(b"short-%d" % i)), i
    finally:
        for c in held:
            c.close()
