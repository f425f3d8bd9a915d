"""Folded IVC on the GPU (z0p_gpu_fold_*): proof bytes and transcript
post-states equal the oracle's restatement of src/fold.rs, the oracle's
verifier accepts them, the published `fold 4x8 fib` size reproduces, and the
accumulator fails the reference's way on bad input."""
import pytest

pytestmark = pytest.mark.gpu

P = 2**31 - 2**27 + 1


def chained(oracle, seg, count, a=1, b=1):
    out = []
    for _ in range(count):
        ca, cb = oracle.build_trace(a, b, seg)
        a, b = int(ca[-1]), int(cb[-1])
        out.append(([int(v) for v in ca], [int(v) for v in cb]))
    return out


def both(z0p, oracle, traces, pz, po, label, ctx):
    tg, to = z0p.Transcript(label), oracle.Transcript(label)
    acc = z0p.fold.Accumulator(pz, ctx)
    oacc = oracle.Accumulator(po)
    for ca, cb in traces:
        acc.add_segment(ca, cb, tg)
        oacc.add_segment(ca, cb, to)
        assert tg.export() == to.export()
    assert len(acc) == len(traces)
    proof = acc.finalize(tg)
    oproof = oacc.finalize(to)
    acc.close()
    return proof, oproof, tg, to


CASES = [
    # seg, blowup, queries, final, grinding, cap, segments
    (8, 8, 8, 4, 0, 0, 3),
    (8, 4, 6, 2, 4, 1, 2),
    (64, 16, 20, 16, 8, 2, 5),
    (1 << 10, 8, 12, 8, 0, 3, 2),
    (1 << 12, 16, 30, 16, 6, 4, 3),
    # one-launch segment commits (fold_segment: S B <= 256) at their edges:
    # two-row segments, a cap at the leaves, 256 rows at two splits
    (2, 16, 4, 8, 0, 0, 3),
    (4, 8, 6, 8, 2, 5, 2),
    (16, 16, 10, 4, 0, 2, 2),
    (32, 8, 8, 4, 3, 1, 3),
]


@pytest.mark.parametrize("case", CASES, ids=[f"s{c[0]}-B{c[1]}-k{c[6]}" for c in CASES])
def test_ivc_matches_oracle(z0p, oracle, gpu_ctx, case):
    seg, blowup, q, final, grind, cap, count = case
    traces = chained(oracle, seg, count)
    out_b = traces[-1][1][-1]
    pz = z0p.fold.Params.new(seg, blowup, q, final, 1, 1, out_b).with_grinding_bits(grind) \
        .with_cap_height(cap)
    po = oracle.fold_params_new(seg, blowup, q, final, 1, 1, out_b)
    po.grinding_bits, po.cap_height = grind, cap
    proof, oproof, tg, to = both(z0p, oracle, traces, pz, po, b"ivc/%d" % seg, gpu_ctx)
    assert proof == oproof
    assert tg.export() == to.export()
    assert oracle.fold_verify(po, proof, oracle.Transcript(b"ivc/%d" % seg)) == 0


def test_published_fold_row(z0p, oracle, gpu_ctx):
    # docs/benchmarks.md:127, tools/baseline.json:50-54; benches/speed_size.rs:432-449.
    traces = chained(oracle, 8, 4)
    out_b = traces[-1][1][-1]
    pz = z0p.fold.Params.new(8, 8, 8, 4, 1, 1, out_b)
    po = oracle.fold_params_new(8, 8, 8, 4, 1, 1, out_b)
    proof, oproof, _, _ = both(z0p, oracle, traces, pz, po, b"bench/fold", gpu_ctx)
    assert proof == oproof
    assert len(proof) == 16845


def test_for_security_production_shape(z0p, oracle, gpu_ctx):
    traces = chained(oracle, 1 << 12, 3)
    out_b = traces[-1][1][-1]
    pz = z0p.fold.Params.for_security(1 << 12, 1, 1, out_b, 100)
    po = oracle.fold_for_security(1 << 12, 1, 1, out_b, 100)
    assert (pz.num_queries, pz.grinding_bits, pz.final_size, pz.cap_height) == \
        (po.num_queries, po.grinding_bits, po.final_size, po.cap_height)
    proof, oproof, _, _ = both(z0p, oracle, traces, pz, po, b"ivc/prod", gpu_ctx)
    assert proof == oproof
    assert oracle.fold_verify(po, proof, oracle.Transcript(b"ivc/prod")) == 0


def test_bad_segment_folds_the_same_and_fails_verify(z0p, oracle, gpu_ctx):
    traces = chained(oracle, 16, 2)
    traces[1][1][5] = (traces[1][1][5] + 1) % P
    out_b = traces[-1][1][-1]
    pz = z0p.fold.Params.new(16, 4, 8, 4, 1, 1, out_b)
    po = oracle.fold_params_new(16, 4, 8, 4, 1, 1, out_b)
    proof, oproof, _, _ = both(z0p, oracle, traces, pz, po, b"ivc/bad", gpu_ctx)
    assert proof == oproof
    assert oracle.fold_verify(po, proof, oracle.Transcript(b"ivc/bad")) != 0


def test_accumulator_errors(z0p, oracle, gpu_ctx):
    f = z0p.fold
    pz = f.Params.new(8, 8, 8, 4, 1, 1, 1)
    t = z0p.Transcript(b"ivc/err")
    before = t.export()
    acc = f.Accumulator(pz, gpu_ctx)
    with pytest.raises(z0p.Z0pError) as e:
        acc.finalize(t)
    assert e.value.code == 1  # EmptyInput
    with pytest.raises(z0p.Z0pError) as e:
        acc.add_segment([1] * 4, [1] * 4, t)
    assert e.value.code == 8  # columns must match seg_steps
    with pytest.raises(z0p.Z0pError) as e:
        acc.add_segment([1] * 7 + [P], [1] * 8, t)
    assert e.value.code == 8  # not a canonical element
    assert t.export() == before and len(acc) == 0
    ca, cb = chained(oracle, 8, 1)[0]
    acc.add_segment(ca, cb, t)
    acc.finalize(t)
    for call in (lambda: acc.finalize(t), lambda: acc.add_segment(ca, cb, t)):
        with pytest.raises(z0p.Z0pError) as e:
            call()
        assert e.value.code == 106
    acc.close()
