"""Folded IVC in the oracle (CPU): hash-chained Fibonacci segments plus one
batched FRI (src/fold.rs). Restates the reference's fold tests
(src/fold.rs:918-1235): honest chains verify, broken chains, forged segments,
tampered openings and wrong transcripts are rejected, the parameter rules and
for_security pins hold, and the wire format fails closed."""
import pytest

P = 2**31 - 2**27 + 1


def chained_traces(oracle, seg, count, a=1, b=1):
    """src/fold.rs:896-906: count Fibonacci segments of seg rows from (a, b)."""
    out = []
    for _ in range(count):
        ca, cb = oracle.build_trace(a, b, seg)
        a, b = int(ca[-1]), int(cb[-1])
        out.append((ca, cb))
    return out


def prove(oracle, params, traces, label):
    t = oracle.Transcript(label)
    acc = oracle.Accumulator(params)
    for ca, cb in traces:
        acc.add_segment(ca, cb, t)
    return acc.finalize(t)


def test_honest_ivc_verifies(oracle):
    traces = chained_traces(oracle, 8, 3)
    params = oracle.fold_params_new(8, 8, 8, 4, 1, 1, int(traces[-1][1][-1]))
    proof = prove(oracle, params, traces, b"fold-e2e")
    assert int.from_bytes(proof[1:5], "little") == 3  # three steps
    assert oracle.fold_verify(params, proof, oracle.Transcript(b"fold-e2e")) == 0


def test_rejects_bad_params(oracle):
    for args in [(3, 8, 8, 4), (8, 2, 8, 4), (8, 8, 0, 4), (1 << 63, 4, 8, 4)]:
        with pytest.raises(ValueError):
            oracle.fold_params_new(*args, 1, 1, 1)


def test_for_security_roundtrip(oracle):
    traces = chained_traces(oracle, 8, 2)
    params = oracle.fold_for_security(8, 1, 1, int(traces[-1][1][-1]), 12)
    assert params.blowup == 16
    assert (params.num_queries, params.grinding_bits) == (3, 6)
    assert params.cap_height <= 4
    proof = prove(oracle, params, traces, b"fold-forsec")
    assert oracle.fold_verify(params, proof, oracle.Transcript(b"fold-forsec")) == 0
    with pytest.raises(ValueError):
        oracle.fold_for_security(3, 1, 1, 1, 12)


def test_empty_accumulator_cannot_finalize(oracle):
    acc = oracle.Accumulator(oracle.fold_params_new(8, 8, 8, 4, 1, 1, 1))
    with pytest.raises(ValueError) as e:
        acc.finalize(oracle.Transcript(b"fold-empty"))
    assert str(e.value) == "EmptyInput"


def test_broken_chain_and_false_claim_fail(oracle):
    good = chained_traces(oracle, 8, 2)
    out_b = int(good[-1][1][-1])
    # second segment restarted from (1, 1): the link does not hold
    bad = [good[0], chained_traces(oracle, 8, 1)[0]]
    params = oracle.fold_params_new(8, 8, 8, 4, 1, 1, int(bad[-1][1][-1]))
    proof = prove(oracle, params, bad, b"fold-chain")
    assert oracle.fold_verify(params, proof, oracle.Transcript(b"fold-chain")) != 0
    wrong = oracle.fold_params_new(8, 8, 8, 4, 1, 1, (out_b + 1) % P)
    proof = prove(oracle, wrong, good, b"fold-claim")
    assert oracle.fold_verify(wrong, proof, oracle.Transcript(b"fold-claim")) != 0


def test_bad_segment_rejected(oracle):
    # A segment that is not a Fibonacci run folds honestly and fails FRI.
    traces = chained_traces(oracle, 8, 2)
    ca, cb = traces[1]
    cb = list(cb)
    cb[3] = (int(cb[3]) + 1) % P
    traces[1] = (ca, cb)
    params = oracle.fold_params_new(8, 8, 8, 4, 1, 1, int(cb[-1]))
    proof = prove(oracle, params, traces, b"fold-bad")
    assert oracle.fold_verify(params, proof, oracle.Transcript(b"fold-bad")) != 0


def test_tampered_opening_and_wrong_transcript_fail(oracle):
    traces = chained_traces(oracle, 8, 2)
    params = oracle.fold_params_new(8, 8, 8, 4, 1, 1, int(traces[-1][1][-1]))
    proof = prove(oracle, params, traces, b"fold-tamper")
    # step 0: claims (16) + cap (4 + 32) + count (4) + index (8): first column value
    at = 1 + 4 + 16 + 36 + 4 + 8
    bad = bytearray(proof)
    bad[at] ^= 1
    assert oracle.fold_verify(params, bytes(bad), oracle.Transcript(b"fold-tamper")) != 0
    assert oracle.fold_verify(params, proof, oracle.Transcript(b"fold-other")) != 0


def test_encoding_fails_closed(oracle):
    traces = chained_traces(oracle, 8, 2)
    params = oracle.fold_params_new(8, 8, 8, 4, 1, 1, int(traces[-1][1][-1]))
    proof = prove(oracle, params, traces, b"fold-codec")
    for bad in (proof[:-1], proof + b"\0", bytes([proof[0] ^ 1]) + proof[1:], b""):
        assert oracle.fold_verify(params, bad, oracle.Transcript(b"fold-codec")) == 8


def test_capped_roundtrip(oracle):
    traces = chained_traces(oracle, 8, 2)
    params = oracle.fold_params_new(8, 8, 8, 4, 1, 1, int(traces[-1][1][-1]))
    params.cap_height = 2
    proof = prove(oracle, params, traces, b"fold-cap")
    assert int.from_bytes(proof[21:25], "little") == 4  # 2^2 cap digests
    assert oracle.fold_verify(params, proof, oracle.Transcript(b"fold-cap")) == 0
    plain = oracle.fold_params_new(8, 8, 8, 4, 1, 1, int(traces[-1][1][-1]))
    assert oracle.fold_verify(plain, proof, oracle.Transcript(b"fold-cap")) != 0


def test_published_fold_row_size(oracle):
    # docs/benchmarks.md:127 and tools/baseline.json:50-54 (`fold 4x8 fib`),
    # workload of benches/speed_size.rs:432-449: 4 segments of 8 rows from
    # (1, 1), Params::new(8, 8, 8, 4, 1, 1, out_b), label "bench/fold".
    traces = chained_traces(oracle, 8, 4)
    params = oracle.fold_params_new(8, 8, 8, 4, 1, 1, int(traces[-1][1][-1]))
    proof = prove(oracle, params, traces, b"bench/fold")
    assert len(proof) == 16845
    assert oracle.fold_verify(params, proof, oracle.Transcript(b"bench/fold")) == 0
