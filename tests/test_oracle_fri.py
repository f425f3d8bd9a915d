"""FRI as a polynomial commitment in the oracle (CPU): commit / commit_ext /
commit_evals / commit_ext_evals, open and verify (src/fri.rs:400-858).

Restates the reference's own FRI tests (src/fri.rs:1458-1911) on the oracle:
honest proofs verify, tampered values, transcripts, nonces and caps are
rejected, the cap height shortens the paths as the reference pins, and the
entry checks return the reference's errors in its order.
"""
import pytest

P = 2**31 - 2**27 + 1


def random_poly(oracle, n, seed):
    """src/fri.rs:1463-1465: Field::from_u64(splitmix64(seed)) per coefficient."""
    out = []
    for _ in range(n):
        z, seed = oracle.splitmix64(seed)
        out.append(z % P)
    return out, seed


def fri_params(oracle, blowup, q, final, grind=0, cap=0):
    return oracle.FriParams(blowup, q, final, grind, cap)


def commit_open(oracle, params, form, values, label, degree_bound=0):
    t = oracle.Transcript(label)
    st = oracle.fri_commit(params, form, values, t, degree_bound)
    proof, idx = oracle.fri_open(st, t)
    return st.commitment, proof, idx, t


def test_honest_proofs_verify_in_every_form(oracle):
    seed = 0x1234ABCD5678EF00
    poly, seed = random_poly(oracle, 16, seed)
    ext, seed = random_poly(oracle, 64, seed)
    params = fri_params(oracle, 4, 8, 4)
    lde = oracle.evaluate_on_coset(poly, 4)
    cases = [(oracle.FRI_COEFFS, poly, 0), (oracle.FRI_COEFFS_EXT, ext, 0),
             (oracle.FRI_EVALS, lde, 15)]
    ext_lde = []
    coords = [oracle.evaluate_on_coset(ext[c::4], 4) for c in range(4)]
    for k in range(64):
        ext_lde += [int(coords[c][k]) for c in range(4)]
    cases.append((oracle.FRI_EVALS_EXT, ext_lde, 15))
    for form, values, bound in cases:
        c, p, idx, _ = commit_open(oracle, params, form, values, b"fri-e2e", bound)
        rc, vidx = oracle.fri_verify(params, c, p, oracle.Transcript(b"fri-e2e"))
        assert rc == 0, form
        assert vidx == idx


def test_ext_coefficients_match_the_evals_form_on_layer_zero(oracle):
    # commit_ext(coeffs) and commit_ext_evals(LDE, n - 1) commit the same
    # layer 0: the first cap agrees (the dims differ, so later caps do not).
    ext, _ = random_poly(oracle, 4 * 256, 0x77)
    params = fri_params(oracle, 4, 8, 16, cap=2)
    coords = [oracle.evaluate_on_coset(ext[c::4], 4) for c in range(4)]
    lde = [int(coords[c][k]) for k in range(1024) for c in range(4)]
    a, *_ = commit_open(oracle, params, oracle.FRI_COEFFS_EXT, ext, b"x")
    b, *_ = commit_open(oracle, params, oracle.FRI_EVALS_EXT, lde, b"x", 255)
    # version (1) + lde, poly, deg (24) + count (4) + cap count (4): cap 0 follows.
    assert a[33:33 + 4 * 32] == b[33:33 + 4 * 32]
    assert a[9:17] != b[9:17]  # poly_len: 256 vs 1024


def test_tampered_value_and_wrong_transcript_fail(oracle):
    params = fri_params(oracle, 4, 8, 4)
    poly, _ = random_poly(oracle, 16, 0x9999000011112222)
    c, p, _, _ = commit_open(oracle, params, oracle.FRI_COEFFS, poly, b"fri-tamper")
    # first opened value: version 1 + final count 4 + 4 x 16 + nonce 8 + query
    # count 4 + fold count 4 bytes in.
    at = 1 + 4 + 16 * 4 + 8 + 4 + 4
    bad = bytearray(p)
    bad[at] ^= 1
    assert oracle.fri_verify(params, c, bytes(bad), oracle.Transcript(b"fri-tamper"))[0] != 0
    assert oracle.fri_verify(params, c, p, oracle.Transcript(b"fri-B"))[0] != 0


def test_larger_domain_has_four_layers(oracle):
    params = fri_params(oracle, 8, 12, 8)
    poly, _ = random_poly(oracle, 64, 0x0BADF00DDEADBEEF)
    c, p, _, _ = commit_open(oracle, params, oracle.FRI_COEFFS, poly, b"fri-big")
    assert int.from_bytes(c[25:29], "little") == 4  # 512 -> 128 -> 32 -> 8
    assert oracle.fri_verify(params, c, p, oracle.Transcript(b"fri-big"))[0] == 0


def test_grinding_roundtrip_and_forged_nonce(oracle):
    params = fri_params(oracle, 4, 8, 4, grind=16)
    poly, _ = random_poly(oracle, 16, 0x600D600D600D600D)
    c, p, _, _ = commit_open(oracle, params, oracle.FRI_COEFFS, poly, b"fri-grind")
    assert oracle.fri_verify(params, c, p, oracle.Transcript(b"fri-grind"))[0] == 0
    at = 1 + 4 + 16 * 4  # the nonce
    nonce = int.from_bytes(p[at:at + 8], "little")
    bad = p[:at] + ((nonce + 1) % 2**64).to_bytes(8, "little") + p[at + 8:]
    assert oracle.fri_verify(params, c, bad, oracle.Transcript(b"fri-grind"))[0] != 0
    plain = fri_params(oracle, 4, 8, 4)
    assert oracle.fri_verify(plain, c, p, oracle.Transcript(b"fri-grind"))[0] != 0


def test_cap_height_shortens_paths(oracle):
    # src/fri.rs:1781-1811: LDE 64, layers 64 (depth 4 quads) and 16 (depth 2).
    poly, _ = random_poly(oracle, 16, 0xC4C4C4C4C4C4C4C4)
    for h in (1, 2, 3):
        params = fri_params(oracle, 4, 8, 4, cap=h)
        c, p, _, _ = commit_open(oracle, params, oracle.FRI_COEFFS, poly, b"fri-cap")
        caps = []
        at = 29
        for _ in range(3):
            n = int.from_bytes(c[at:at + 4], "little")
            caps.append(n)
            at += 4 + 32 * n
        assert caps == [1 << min(h, 4), 1 << min(h, 2), 1]
        per_query = 4 + sum(64 + 4 + 33 * (d - 2 - min(h, d - 2)) for d in (6, 4))
        assert len(p) == 1 + 4 + 16 * 4 + 8 + 4 + 8 * per_query
        assert oracle.fri_verify(params, c, p, oracle.Transcript(b"fri-cap"))[0] == 0
        bad = bytearray(c)
        bad[33] ^= 1  # first cap digest
        assert oracle.fri_verify(params, bytes(bad), p, oracle.Transcript(b"fri-cap"))[0] != 0


def test_lowered_bound_fails_final_check(oracle):
    params = fri_params(oracle, 4, 8, 16)
    evals, _ = random_poly(oracle, 64, 0x2B2B2B2B2B2B2B2B)
    c, p, _, _ = commit_open(oracle, params, oracle.FRI_EVALS, evals, b"fri-lowbound", 7)
    assert oracle.fri_verify(params, c, p, oracle.Transcript(b"fri-lowbound"))[0] != 0


def test_entry_checks_in_reference_order(oracle):
    params = fri_params(oracle, 4, 8, 4)
    t = oracle.Transcript(b"fri-test")
    errs = {}
    for name, (form, values, bound) in {
        "empty": (oracle.FRI_COEFFS, [], 0),
        "not_pow2": (oracle.FRI_COEFFS, [1, 1, 1], 0),
        "ext_empty": (oracle.FRI_COEFFS_EXT, [], 0),
        "evals_bound": (oracle.FRI_EVALS, [1] * 64, 64),
        "evals_rate": (oracle.FRI_EVALS, [1] * 64, 32),
        "no_fold": (oracle.FRI_COEFFS, [1] * 1, 0),
        "too_big": (oracle.FRI_COEFFS, [0] * (1 << 20), 0),
    }.items():
        p = fri_params(oracle, 256, 8, 4) if name == "too_big" else params
        with pytest.raises(ValueError) as e:
            oracle.fri_commit(p, form, values, t, bound)
        errs[name] = str(e.value)
    assert errs == {"empty": "EmptyInput", "not_pow2": "InvalidDomainSize",
                    "ext_empty": "EmptyInput", "evals_bound": "MalformedInput",
                    "evals_rate": "MalformedInput", "no_fold": "InvalidDomainSize",
                    "too_big": "InvalidDomainSize"}
    with pytest.raises(ValueError) as e:
        oracle.fri_commit(fri_params(oracle, 3, 8, 4), oracle.FRI_COEFFS, [1] * 16, t)
    assert str(e.value) == "InvalidBlowup"


def bench_coeffs(n):
    """benches/speed_size.rs:609-611: Field::new(i.wrapping_mul(0x9e37_79b9) + 17)."""
    return [(((i * 0x9E3779B9) + 17) % 2**32) % P for i in range(n)]


def test_for_security_matches_the_reference_pins(oracle):
    # src/fri.rs:1814-1836
    p = oracle.fri_for_security(16, 40)
    assert (p.num_queries, p.grinding_bits) == (10, 20) and p.cap_height <= 4
    p = oracle.fri_for_security(16, 10)
    assert (p.num_queries, p.grinding_bits) == (3, 5)
    for bad in (0, 3, 1 << 24):
        with pytest.raises(ValueError):
            oracle.fri_for_security(bad, 40)


@pytest.mark.parametrize("n,label,size", [(256, b"bench/fri-prod", 29378),
                                          (1024, b"bench/fri-prod-big", 43174)])
def test_published_production_sizes(oracle, n, label, size):
    # docs/benchmarks.md:24,26 (`fri prod` rows): commitment + proof bytes.
    p = oracle.fri_for_security(n, 100)
    assert (p.blowup, p.num_queries, p.grinding_bits, p.cap_height, p.final_size) == (16, 40, 20, 4, 16)
    c, proof, _, _ = commit_open(oracle, p, oracle.FRI_COEFFS, bench_coeffs(n), label)
    assert len(c) + len(proof) == size
    assert oracle.fri_verify(p, c, proof, oracle.Transcript(label))[0] == 0
