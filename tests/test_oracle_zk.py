"""Zero-knowledge AIR proofs in the oracle (CPU): the ChaCha20 stream
(src/rng.rs) against its RFC 8439 vectors and the reference's stream tests,
and air::prove_zk (src/air.rs:439-464, src/blind.rs:40-78): masked proofs
verify with the plain verifier, differ with the masking stream, and the
hiding budget is enforced."""
import pytest

# RFC 8439 section 2.3.2, as pinned by src/rng.rs:230-247.
RFC_KEY = bytes(range(32))
RFC_NONCE = bytes([0, 0, 0, 9, 0, 0, 0, 0x4A, 0, 0, 0, 0])
RFC_BLOCK = bytes.fromhex(
    "10f1e7e4d13b5915500fdd1fa32071c4c7d1f4c733c068030422aa9ac3d46c4e"
    "d2826446079faa0914c2d705d98b02a2b5129cd1de164eb9cbd083e8a2503c4e")


def test_chacha20_block_matches_rfc_8439(oracle):
    assert oracle.chacha20_block(RFC_KEY, 1, RFC_NONCE) == RFC_BLOCK


def test_stream_matches_blocks_and_is_unaligned(oracle):
    # src/rng.rs:250-285
    key, nonce = bytes([7]) * 32, bytes([9]) * 12
    s = oracle.ChaCha20.new(key, nonce)
    assert s.fill_bytes(64) == oracle.chacha20_block(key, 0, nonce)
    assert s.fill_bytes(64) == oracle.chacha20_block(key, 1, nonce)
    a = oracle.ChaCha20.new(bytes([3]) * 32, bytes([5]) * 12)
    b = oracle.ChaCha20.new(bytes([3]) * 32, bytes([5]) * 12)
    x = a.fill_bytes(5) + a.fill_bytes(95)
    assert x == b.fill_bytes(100)


def test_next_field_is_rejection_sampled(oracle):
    # src/rng.rs:157-167: words at or above 2p are skipped.
    P = 2**31 - 2**27 + 1
    s = oracle.ChaCha20.new(bytes([1]) * 32, bytes(12))
    w = oracle.ChaCha20.new(bytes([1]) * 32, bytes(12))
    for _ in range(200):
        v = s.next_field()
        while True:
            word = int.from_bytes(w.fill_bytes(4), "little")
            if word < 2 * P:
                break
        assert v == word % P


def _zk(oracle, n, n_rand, key, label=b"zk"):
    a, b = oracle.build_trace(1, 1, n)
    params = oracle.air_params_new(n, 8, 4, 4, 1, 1, int(b[-1]))
    rng = oracle.ChaCha20.new(key, bytes(12))
    return params, oracle.air_prove_zk(params, n_rand, rng, oracle.Transcript(label))


def test_masked_proofs_verify_and_depend_on_the_stream(oracle):
    params, p1 = _zk(oracle, 32, 64, bytes([1]) * 32)
    _, p2 = _zk(oracle, 32, 64, bytes([2]) * 32)
    assert p1 != p2
    assert oracle.air_verify(params, p1, oracle.Transcript(b"zk")) == 0
    assert oracle.air_verify(params, p2, oracle.Transcript(b"zk")) == 0
    plain = oracle.air_prove(params, oracle.Transcript(b"zk"))
    assert len(plain) < len(p1)  # the masked LDE is longer


def test_hiding_budget_is_enforced(oracle):
    with pytest.raises(ValueError) as e:
        _zk(oracle, 16, 63, bytes(32))  # 16 * num_queries = 64
    assert str(e.value) == "MalformedInput"


def test_tampered_masked_proof_fails(oracle):
    params, p = _zk(oracle, 32, 64, bytes([4]) * 32)
    bad = bytearray(p)
    bad[-70] ^= 1
    assert oracle.air_verify(params, bytes(bad), oracle.Transcript(b"zk")) != 0


def test_range_prove_zk_verifies_and_depends_on_the_stream(oracle):
    # range.rs:393-418: masked columns verify with the plain verifier; the
    # hiding budget n_rand >= num_queries is enforced.
    p = oracle.range_params_new(64, 8, 16, 8, 32, 200)
    a = oracle.range_prove_zk(p, 40, oracle.ChaCha20.new(bytes(32), bytes(12)), oracle.Transcript(b"rz"))
    b = oracle.range_prove_zk(p, 40, oracle.ChaCha20.new(bytes([1]) * 32, bytes(12)),
                              oracle.Transcript(b"rz"))
    assert a != b
    assert oracle.range_verify(p, a, oracle.Transcript(b"rz")) == 0
    assert oracle.range_verify(p, b, oracle.Transcript(b"rz")) == 0
    bad = oracle.range_params_new(64, 8, 16, 8, 32, 300)  # 300 needs 9 bits
    c = oracle.range_prove_zk(bad, 40, oracle.ChaCha20.new(bytes(32), bytes(12)), oracle.Transcript(b"rz"))
    assert oracle.range_verify(bad, c, oracle.Transcript(b"rz")) != 0
    with pytest.raises(ValueError) as e:
        oracle.range_prove_zk(p, 7, oracle.ChaCha20.new(bytes(32), bytes(12)), oracle.Transcript(b"rz"))
    assert str(e.value) == "MalformedInput"
