"""Regenerates tests/golden/proofs.json from the C oracle.

The reference (pure Rust) cannot be built in this environment, so the golden
proofs are the oracle's, and the oracle is pinned to the reference's own
known answers by tests/test_oracle.py (BLAKE3 KATs, size pins, tuner pins,
verifier acceptance). Each case records the parameters, transcript label,
proof length and SHA-256 of the proof bytes; the GPU tests compare the device
prover against these digests as well as against a live oracle run.

    python tests/golden/make_golden.py
"""
import hashlib
import json
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

import oracle as O  # noqa: E402

P = O.P


def seeded_pair(seed):
    z1, s = O.splitmix64(seed)
    z2, _ = O.splitmix64(s)
    return z1 % P, z2 % P


def air_case(name, n, blowup, q, final, a0, b0, label, grinding=0, cap=0, prod=False):
    _, b = O.build_trace(a0, b0, n)
    b_last = int(b[-1])
    if prod:
        p = O.air_for_security(n, a0, b0, b_last, 100)
    else:
        p = O.air_params_new(n, blowup, q, final, a0, b0, b_last, grinding, cap)
    proof = O.air_prove(p, O.Transcript(label.encode()))
    assert O.air_verify(p, proof, O.Transcript(label.encode())) == 0, name
    return {
        "name": name, "kind": "air", "n": p.n_steps, "blowup": p.blowup, "queries": p.num_queries,
        "final": p.final_size, "grinding": p.grinding_bits, "cap": p.cap_height, "a0": p.a0,
        "b0": p.b0, "b_last": p.b_last, "label": label, "len": len(proof),
        "sha256": hashlib.sha256(proof).hexdigest(),
    }


def range_case(name, n, bits, blowup, q, final, value, label, grinding=0, cap=0, prod=False):
    if prod:
        p = O.range_for_security(n, bits, value, 100)
    else:
        p = O.range_params_new(n, bits, blowup, q, final, value, grinding, cap)
    proof = O.range_prove(p, O.Transcript(label.encode()))
    ok = O.range_verify(p, proof, O.Transcript(label.encode())) == 0
    return {
        "name": name, "kind": "range", "n": p.n_rows, "n_bits": p.n_bits, "blowup": p.blowup,
        "queries": p.num_queries, "final": p.final_size, "grinding": p.grinding_bits,
        "cap": p.cap_height, "value": p.value, "label": label, "len": len(proof),
        "sha256": hashlib.sha256(proof).hexdigest(), "verifies": ok,
    }


def main():
    cases = [
        air_case("air n2 b4", 2, 4, 3, 2, 1, 1, "edge/n2"),
        air_case("air n4 b8 f2", 4, 8, 5, 2, 3, 5, "edge/n4", cap=1),
        air_case("air fib16", 16, 8, 8, 8, 1, 1, "fib-e2e"),
        air_case("air fib64 bench", 64, 8, 12, 8, 1, 1, "bench/air"),
        air_case("air fib1024 bench", 1024, 8, 12, 8, 1, 1, "bench/air1024"),
        air_case("air n256 b4 grind8 cap3", 256, 4, 7, 4, 2, 9, "edge/b4", grinding=8, cap=3),
        air_case("air n128 b32 f32 cap8", 128, 32, 9, 16, 5, 6, "edge/b32", grinding=4, cap=8),
        air_case("air prod 64", 64, 0, 0, 0, 1, 1, "bench/air-prod", prod=True),
        air_case("air prod 1024", 1024, 0, 0, 0, 1, 1, "bench/air-scale", prod=True),
        air_case("air prod 8192", 8192, 0, 0, 0, 1, 1, "bench/air-scale", prod=True),
        air_case("air prod 65536 seeded", 65536, 0, 0, 0, *seeded_pair(0x5EED000000000002),
                 "bench/air-scale", prod=True),
        range_case("range 16-bit bench", 8, 16, 8, 8, 4, 12345, "bench/range"),
        range_case("range 1-bit", 16, 1, 4, 5, 4, 1, "edge/range1"),
        range_case("range 24-bit", 32, 24, 8, 6, 4, 9999999, "edge/range24", grinding=3, cap=2),
        range_case("range 15-bit b2", 64, 15, 2, 4, 2, 30000, "edge/range15"),
        range_case("range dishonest", 16, 4, 8, 8, 8, 17, "edge/range-bad"),
        range_case("range prod 4096", 4096, 16, 0, 0, 0, 54321, "bench/range", prod=True),
    ]
    out = {"generator": "tests/golden/make_golden.py (C oracle)", "cases": cases}
    with open(os.path.join(HERE, "proofs.json"), "w") as f:
        json.dump(out, f, indent=1)
    print(f"wrote {len(cases)} cases")


if __name__ == "__main__":
    main()
