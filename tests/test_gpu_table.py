"""Table membership on the GPU (z0p_gpu_table_prove / _zk): proof bytes,
transcript post-states and the stream state equal the oracle's restatement
of src/table.rs; the published `table 4-entry` size reproduces; members
verify and non-members fail in the oracle's verifier."""
import random

import pytest

pytestmark = pytest.mark.gpu

P = 2**31 - 2**27 + 1
TABLE = [10, 20, 30, 40]

CASES = [
    # n_rows, blowup, queries, final, grinding, cap, value, table size
    (8, 8, 8, 4, 0, 0, 30, 4),
    (8, 8, 8, 4, 0, 2, 99, 4),
    (64, 32, 12, 8, 4, 3, None, 7),
    (1 << 10, 16, 20, 16, 6, 4, None, 3),
    (1 << 12, 8, 16, 8, 0, 4, None, 2),
]


def _case(case):
    n, blowup, q, final, grind, cap, value, tlen = case
    rng = random.Random(n * 31 + tlen)
    table = TABLE if tlen == 4 else [rng.randrange(P) for _ in range(tlen)]
    if value is None:
        value = table[rng.randrange(tlen)]
    return n, blowup, q, final, grind, cap, value, table


@pytest.mark.parametrize("case", CASES, ids=[f"n{c[0]}-B{c[1]}-T{c[7]}" for c in CASES])
def test_table_matches_oracle(z0p, oracle, gpu_ctx, case):
    n, blowup, q, final, grind, cap, value, table = _case(case)
    pz = z0p.table.Params.new(n, blowup, q, final, value).with_grinding_bits(grind) \
        .with_cap_height(cap)
    po = oracle.table_params_new(n, blowup, q, final, value)
    po.grinding_bits, po.cap_height = grind, cap
    tg, to = z0p.Transcript(b"tab"), oracle.Transcript(b"tab")
    proof = z0p.table.prove(pz, table, tg, gpu_ctx)
    assert proof == oracle.table_prove(po, table, to)
    assert tg.export() == to.export()
    rc = oracle.table_verify(po, table, proof, oracle.Transcript(b"tab"))
    assert (rc == 0) == (value in table)


def test_published_table_row(z0p, oracle, gpu_ctx):
    # benches/speed_size.rs:301-305, docs/benchmarks.md:125.
    pz = z0p.table.Params.new(8, 8, 8, 4, 30)
    proof = z0p.table.prove(pz, TABLE, z0p.Transcript(b"bench/table"), gpu_ctx)
    po = oracle.table_params_new(8, 8, 8, 4, 30)
    assert proof == oracle.table_prove(po, TABLE, oracle.Transcript(b"bench/table"))
    assert len(proof) == 4673


@pytest.mark.parametrize("n,n_rand", [(8, 24), (256, 200), (1 << 10, 1000)])
def test_table_zk_matches_oracle(z0p, oracle, gpu_ctx, n, n_rand):
    pz = z0p.table.Params.new(n, 8, 8, 4, 20)
    po = oracle.table_params_new(n, 8, 8, 4, 20)
    key, nonce = bytes([n % 251]) * 32, bytes([7]) * 12
    rz, ro = z0p.rng.ChaCha20.new(key, nonce), oracle.ChaCha20.new(key, nonce)
    tg, to = z0p.Transcript(b"tab-zk"), oracle.Transcript(b"tab-zk")
    proof = z0p.table.prove_zk(pz, TABLE, n_rand, rz, tg, gpu_ctx)
    assert proof == oracle.table_prove_zk(po, TABLE, n_rand, ro, to)
    assert tg.export() == to.export()
    assert (bytes(rz.block), rz.counter, rz.used) == (bytes(ro.block), ro.counter, ro.used)
    assert oracle.table_verify(po, TABLE, proof, oracle.Transcript(b"tab-zk")) == 0


def test_table_errors(z0p, gpu_ctx):
    pz = z0p.table.Params.new(8, 8, 8, 4, 30)
    t = z0p.Transcript(b"tab-err")
    before = t.export()
    for table, code in [([1], 8), ([], 8), ([1, P], 8)]:
        with pytest.raises(z0p.Z0pError) as e:
            z0p.table.prove(pz, table, t, gpu_ctx)
        assert e.value.code == code
    with pytest.raises(z0p.Z0pError) as e:
        z0p.table.prove_zk(pz, TABLE, 7, z0p.rng.ChaCha20.new(bytes(32), bytes(12)), t, gpu_ctx)
    assert e.value.code == 8
    assert t.export() == before


@pytest.mark.parametrize("n,blowup,final,tlen,member", [
    (8, 8, 4, 4, True), (16, 8, 8, 4, False), (1 << 10, 16, 16, 5, False), (1 << 10, 16, 4, 5, False),
    (2, 8, 4, 3, True), (1 << 12, 8, 32, 2, False)])
def test_constant_column_paths_match_oracle(z0p, oracle, gpu_ctx, n, blowup, final, tlen, member):
    # Members and non-members on the compact path (final >= blowup or a
    # member), and a non-member with final < blowup on the row-by-row path.
    rng = random.Random(n + tlen)
    table = [rng.randrange(P) for _ in range(tlen)]
    value = table[1] if member else rng.randrange(P)
    pz = z0p.table.Params.new(n, blowup, 8, final, value).with_cap_height(3)
    po = oracle.table_params_new(n, blowup, 8, final, value)
    po.cap_height = 3
    tg, to = z0p.Transcript(b"tab-c"), oracle.Transcript(b"tab-c")
    proof = z0p.table.prove(pz, table, tg, gpu_ctx)
    assert proof == oracle.table_prove(po, table, to)
    assert tg.export() == to.export()
    assert (oracle.table_verify(po, table, proof, oracle.Transcript(b"tab-c")) == 0) == member
