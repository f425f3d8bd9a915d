"""Table membership in the oracle (CPU): src/table.rs restated and checked
against the reference's own table tests (src/table.rs:678-830) and the
published `table 4-entry` proof size (docs/benchmarks.md:125)."""
import pytest

P = 2**31 - 2**27 + 1
TABLE = [10, 20, 30, 40]


def prove(oracle, params, label, table=TABLE):
    return oracle.table_prove(params, table, oracle.Transcript(label))


def test_honest_member_verifies(oracle):
    p = oracle.table_params_new(8, 8, 8, 4, 30)
    proof = prove(oracle, p, b"table-e2e")
    assert oracle.table_verify(p, TABLE, proof, oracle.Transcript(b"table-e2e")) == 0


def test_published_table_row_size(oracle):
    # benches/speed_size.rs:301-305: Params::new(8, 8, 8, 4, 30), label "bench/table".
    p = oracle.table_params_new(8, 8, 8, 4, 30)
    proof = prove(oracle, p, b"bench/table")
    assert len(proof) == 4673
    assert oracle.table_verify(p, TABLE, proof, oracle.Transcript(b"bench/table")) == 0


def test_rejects_bad_params_and_tables(oracle):
    for args in [(3, 8, 8, 4), (8, 1, 8, 4), (8, 8, 0, 4), (1 << 63, 4, 8, 4)]:
        with pytest.raises(ValueError):
            oracle.table_params_new(*args, 1)
    p = oracle.table_params_new(8, 8, 8, 4, 30)
    for bad in ([1], []):
        with pytest.raises(ValueError) as e:
            oracle.table_prove(p, bad, oracle.Transcript(b"t"))
        assert str(e.value) == "MalformedInput"


def test_for_security_roundtrip(oracle):
    p = oracle.table_for_security(8, 4, 30, 12)
    assert p.blowup == 16
    assert (p.num_queries, p.grinding_bits) == (6, 6)
    assert p.cap_height <= 4
    proof = prove(oracle, p, b"table-forsec")
    assert oracle.table_verify(p, TABLE, proof, oracle.Transcript(b"table-forsec")) == 0
    for args in [(3, 4), (8, 1)]:
        with pytest.raises(ValueError):
            oracle.table_for_security(*args, 1, 12)


def test_capped_roundtrip_and_forged_cap(oracle):
    p = oracle.table_params_new(8, 8, 8, 4, 30)
    p.cap_height = 2
    proof = prove(oracle, p, b"table-cap")
    assert int.from_bytes(proof[1:5], "little") == 4
    assert oracle.table_verify(p, TABLE, proof, oracle.Transcript(b"table-cap")) == 0
    bad = bytearray(proof)
    bad[5] ^= 1
    assert oracle.table_verify(p, TABLE, bytes(bad), oracle.Transcript(b"table-cap")) != 0
    plain = oracle.table_params_new(8, 8, 8, 4, 30)
    assert oracle.table_verify(plain, TABLE, proof, oracle.Transcript(b"table-cap")) != 0


def test_non_member_and_tamper_fail(oracle):
    p = oracle.table_params_new(8, 8, 8, 4, 99)
    proof = prove(oracle, p, b"table-nonmember")
    assert oracle.table_verify(p, TABLE, proof, oracle.Transcript(b"table-nonmember")) != 0
    p = oracle.table_params_new(8, 8, 8, 4, 30)
    proof = prove(oracle, p, b"table-tamper")
    bad = bytearray(proof)
    bad[-(4 + 33 * 6) - 4] ^= 1  # the last opening's value
    assert oracle.table_verify(p, TABLE, bytes(bad), oracle.Transcript(b"table-tamper")) != 0


def test_zk_member_verifies_and_budget(oracle):
    p = oracle.table_params_new(8, 8, 8, 4, 30)
    rng = oracle.ChaCha20.new(bytes([5]) * 32, bytes(12))
    proof = oracle.table_prove_zk(p, TABLE, 24, rng, oracle.Transcript(b"table-zk"))
    assert oracle.table_verify(p, TABLE, proof, oracle.Transcript(b"table-zk")) == 0
    with pytest.raises(ValueError) as e:
        oracle.table_prove_zk(p, TABLE, 7, oracle.ChaCha20.new(bytes(32), bytes(12)),
                              oracle.Transcript(b"t"))
    assert str(e.value) == "MalformedInput"
