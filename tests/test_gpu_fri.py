"""FRI as a polynomial commitment on the GPU (z0p_gpu_fri_commit / _open):
commitment bytes, proof bytes, query indices and transcript post-states equal
the oracle's (src/fri.rs:400-666) in every input form, the oracle's verifier
accepts them, and the entry checks fail the same way with the transcript
untouched."""
import random

import pytest

pytestmark = pytest.mark.gpu

P = 2**31 - 2**27 + 1


def _values(n, seed):
    rng = random.Random(seed)
    return [rng.randrange(P) for _ in range(n)]


def _low_degree_evals(oracle, n, bound, ext, seed):
    """n evaluations on the 31-coset of a random polynomial of degree <= bound
    (bound + 1 a power of two), coordinate by coordinate for Ext4."""
    k = bound + 1
    coords = [oracle.evaluate_on_coset(_values(k, seed + c), n // k) for c in range(4 if ext else 1)]
    if not ext:
        return [int(v) for v in coords[0]]
    return [int(coords[c][i]) for i in range(n) for c in range(4)]


def _pair(z0p, oracle, blowup, q, final, grind=0, cap=0):
    return (z0p.fri.Params.new(blowup, q, final).with_grinding_bits(grind).with_cap_height(cap),
            oracle.FriParams(blowup, q, final, grind, cap))


def _gpu_commit(z0p, form, values, pz, t, bound, ctx):
    f = z0p.fri
    if form == f.COEFFS:
        return f.commit(values, pz, t, ctx)
    if form == f.COEFFS_EXT:
        return f.commit_ext(values, pz, t, ctx)
    if form == f.EVALS:
        return f.commit_evals(values, bound, pz, t, ctx)
    return f.commit_ext_evals(values, bound, pz, t, ctx)


CASES = [
    # form, n, blowup, queries, final, grinding, cap, degree bound (evals forms)
    (0, 1, 16, 8, 4, 0, 0, 0),
    (0, 2, 8, 8, 4, 0, 1, 0),
    (0, 16, 4, 8, 4, 0, 0, 0),
    (0, 64, 8, 12, 8, 6, 2, 0),
    (0, 1 << 10, 16, 20, 16, 8, 4, 0),
    (0, 1 << 13, 2, 30, 4, 0, 3, 0),
    (1, 16, 4, 8, 4, 0, 2, 0),
    (1, 1 << 11, 8, 16, 16, 4, 4, 0),
    (2, 64, 4, 8, 16, 0, 0, 7),
    (2, 1 << 12, 16, 10, 16, 5, 3, 255),
    (3, 256, 4, 8, 4, 0, 1, 63),
    (3, 1 << 14, 4, 24, 16, 0, 4, 1023),
    # 256-digest caps and a 1024-value final layer: the device transcript
    # absorbs about 16 KB per layer, crossing chunks and merging its stack.
    (0, 1 << 12, 4, 8, 1024, 3, 8, 0),
]


@pytest.mark.parametrize("case", CASES, ids=[f"form{c[0]}-n{c[1]}-B{c[2]}" for c in CASES])
def test_commit_open_matches_oracle(z0p, oracle, gpu_ctx, case):
    form, n, blowup, q, final, grind, cap, bound = case
    ext = form in (1, 3)
    if form >= 2:
        values = _low_degree_evals(oracle, n, bound, ext, hash(case) & 0xFFFF)
    else:
        values = _values(n * (4 if ext else 1), hash(case) & 0xFFFF)
    pz, po = _pair(z0p, oracle, blowup, q, final, grind, cap)
    label = b"pcs/%d" % n
    tg, to = z0p.Transcript(label), oracle.Transcript(label)
    tg.absorb(b"prefix", b"p" * 100)
    to.absorb(b"prefix", b"p" * 100)
    st = _gpu_commit(z0p, form, values, pz, tg, bound, gpu_ctx)
    so = oracle.fri_commit(po, form, values, to, bound)
    assert st.commitment == so.commitment
    assert tg.export() == to.export()
    proof, idx = z0p.fri.open(st, tg)
    oproof, oidx = oracle.fri_open(so, to)
    assert proof == oproof
    assert idx == oidx
    assert tg.export() == to.export()
    tv = oracle.Transcript(label)
    tv.absorb(b"prefix", b"p" * 100)
    rc, vidx = oracle.fri_verify(po, st.commitment, proof, tv)
    assert rc == 0 and vidx == idx


def test_production_size_commitment(z0p, oracle, gpu_ctx):
    # 2^16 coefficients at blowup 16 (LDE 2^20), the for_security(100) shape.
    values = _values(1 << 16, 0xF00D)
    pz, po = _pair(z0p, oracle, 16, 40, 16, 20, 4)
    tg, to = z0p.Transcript(b"pcs/big"), oracle.Transcript(b"pcs/big")
    st = z0p.fri.commit(values, pz, tg, gpu_ctx)
    so = oracle.fri_commit(po, 0, values, to)
    assert st.commitment == so.commitment
    proof, idx = z0p.fri.open(st, tg)
    assert (proof, idx) == oracle.fri_open(so, to)
    assert tg.export() == to.export()


def test_long_history_transcript(z0p, oracle, gpu_ctx):
    """The commitment's transcript steps run on the device from a state with
    chunks already pushed (stack, counters and block cache handed over)."""
    values = _values(1 << 10, 5)
    pz, po = _pair(z0p, oracle, 8, 12, 8, 4, 2)
    tg, to = z0p.Transcript(b"pcs/long"), oracle.Transcript(b"pcs/long")
    pad = bytes((7 * i + 3) % 251 for i in range(5000))
    for t in (tg, to):
        t.absorb(b"pad", pad)
        t.absorb(b"pad2", pad[:77])
    st = z0p.fri.commit(values, pz, tg, gpu_ctx)
    so = oracle.fri_commit(po, 0, values, to)
    assert tg.export() == to.export()
    assert z0p.fri.open(st, tg) == oracle.fri_open(so, to)
    assert tg.export() == to.export()


def test_something_between_commit_and_open(z0p, oracle, gpu_ctx):
    values = _values(64, 3)
    pz, po = _pair(z0p, oracle, 4, 8, 4)
    tg, to = z0p.Transcript(b"pcs/mid"), oracle.Transcript(b"pcs/mid")
    st = z0p.fri.commit(values, pz, tg, gpu_ctx)
    so = oracle.fri_commit(po, 0, values, to)
    tg.absorb(b"other", b"commitment")
    to.absorb(b"other", b"commitment")
    assert z0p.fri.open(st, tg) == oracle.fri_open(so, to)


def test_entry_errors_leave_the_transcript(z0p, gpu_ctx):
    f = z0p.fri
    pz = f.Params.new(4, 8, 4)
    t = z0p.Transcript(b"pcs/err")
    before = t.export()
    cases = [
        (lambda: f.commit([], pz, t, gpu_ctx), 1),                      # EmptyInput
        (lambda: f.commit([1, 2, 3], pz, t, gpu_ctx), 3),               # InvalidDomainSize
        (lambda: f.commit_evals([1] * 64, 64, pz, t, gpu_ctx), 8),      # bound >= LDE size
        (lambda: f.commit_evals([1] * 64, 32, pz, t, gpu_ctx), 8),      # rate >= 1/2
        (lambda: f.commit([1] * 1, f.Params.new(4, 8, 4), t, gpu_ctx), 3),  # no fold
        (lambda: f.commit([1] * 16, f.Params.new(3, 8, 4), t, gpu_ctx), 4),  # InvalidBlowup
        (lambda: f.commit([1] * 16, f.Params.new(4, 0, 4), t, gpu_ctx), 5),  # NoQueries
        (lambda: f.commit([1] * 15 + [P], pz, t, gpu_ctx), 8),          # non-canonical
        (lambda: f.commit_ext_evals([1] * 255 + [P + 5], 15, pz, t, gpu_ctx), 8),
    ]
    for call, code in cases:
        with pytest.raises(z0p.Z0pError) as e:
            call()
        assert e.value.code == code
        assert t.export() == before


def test_open_needs_a_fresh_commitment(z0p, oracle, gpu_ctx):
    f = z0p.fri
    pz = f.Params.new(4, 8, 4)
    t = z0p.Transcript(b"pcs/stale")
    st = f.commit(_values(16, 9), pz, t, gpu_ctx)
    f.open(st, t)
    with pytest.raises(z0p.Z0pError) as e:  # already opened
        f.open(st, t)
    assert e.value.code == 106
    st = f.commit(_values(16, 9), pz, t, gpu_ctx)
    a = z0p.air.Params.for_security(64, 1, 1, z0p.air.trace_last(1, 1, 64)[1], 32)
    z0p.air.prove(a, z0p.Transcript(b"other"), gpu_ctx)  # reuses the workspace
    before = t.export()
    with pytest.raises(z0p.Z0pError) as e:
        f.open(st, t)
    assert e.value.code == 106
    assert t.export() == before


@pytest.mark.parametrize("n,label,size", [(256, b"bench/fri-prod", 29378),
                                          (1024, b"bench/fri-prod-big", 43174)])
def test_published_production_rows(z0p, oracle, gpu_ctx, n, label, size):
    # docs/benchmarks.md:24,26 with benches/speed_size.rs:607-647, 756-795.
    coeffs = [(((i * 0x9E3779B9) + 17) % 2**32) % P for i in range(n)]
    pz = z0p.fri.Params.for_security(n, 100)
    po = oracle.fri_for_security(n, 100)
    assert (pz.num_queries, pz.final_size, pz.grinding_bits, pz.cap_height) == \
        (po.num_queries, po.final_size, po.grinding_bits, po.cap_height)
    tg, to = z0p.Transcript(label), oracle.Transcript(label)
    st = z0p.fri.commit(coeffs, pz, tg, gpu_ctx)
    proof, idx = z0p.fri.open(st, tg)
    so = oracle.fri_commit(po, 0, coeffs, to)
    assert st.commitment == so.commitment
    assert (proof, idx) == oracle.fri_open(so, to)
    assert len(st.commitment) + len(proof) == size
