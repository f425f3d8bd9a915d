"""GPU parity: the device prover against the oracle, byte for byte.

Every case proves on the GB300 through the C ABI and compares the proof with
(a) a live oracle proof on the same parameters, seed and transcript label and
(b) the committed golden digest; the oracle verifier must accept the GPU
proof, and the transcript must be left in the oracle's post-state.
"""
import hashlib
import json
import os

import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLD = json.load(open(os.path.join(ROOT, "tests", "golden", "proofs.json")))["cases"]


def _air_pair(z0p, oracle, case):
    po = oracle.air_params_new(case["n"], case["blowup"], case["queries"], case["final"], case["a0"],
                               case["b0"], case["b_last"], case["grinding"], case["cap"])
    pz = z0p.air.Params.new(case["n"], case["blowup"], case["queries"], case["final"], case["a0"],
                            case["b0"], case["b_last"])
    pz.grinding_bits = case["grinding"]
    pz.cap_height = case["cap"]
    return po, pz


def _range_pair(z0p, oracle, case):
    po = oracle.range_params_new(case["n"], case["n_bits"], case["blowup"], case["queries"], case["final"],
                                 case["value"], case["grinding"], case["cap"])
    pz = z0p.range.Params.new(case["n"], case["n_bits"], case["blowup"], case["queries"], case["final"],
                              case["value"])
    pz.grinding_bits = case["grinding"]
    pz.cap_height = case["cap"]
    return po, pz


@pytest.mark.parametrize("case", GOLD, ids=[c["name"] for c in GOLD])
def test_golden_case_byte_identical(z0p, oracle, gpu_ctx, case):
    label = case["label"].encode()
    if case["kind"] == "air":
        po, pz = _air_pair(z0p, oracle, case)
        tz = z0p.Transcript(label)
        proof = z0p.air.prove(pz, tz, gpu_ctx)
        to = oracle.Transcript(label)
        ref = oracle.air_prove(po, to)
        assert oracle.air_verify(po, proof, oracle.Transcript(label)) == 0
    else:
        po, pz = _range_pair(z0p, oracle, case)
        tz = z0p.Transcript(label)
        proof = z0p.range.prove(pz, tz, gpu_ctx)
        to = oracle.Transcript(label)
        ref = oracle.range_prove(po, to)
        ok = oracle.range_verify(po, proof, oracle.Transcript(label)) == 0
        assert ok == case["verifies"]
    assert len(proof) == case["len"]
    assert proof == ref
    assert hashlib.sha256(proof).hexdigest() == case["sha256"]
    assert tz.export() == to.export()


def test_air_prod_1m_byte_identical(z0p, oracle, gpu_ctx):
    """Fibonacci 2^20 steps, production schedule, seeded initial pair."""
    n = 1 << 20
    P = oracle.P
    z1, s = oracle.splitmix64(0x5EED000000000001)
    z2, _ = oracle.splitmix64(s)
    a0, b0 = z1 % P, z2 % P
    _, b = oracle.build_trace(a0, b0, n)
    po = oracle.air_for_security(n, a0, b0, int(b[-1]), 100)
    pz = z0p.air.Params.for_security(n, a0, b0, int(b[-1]), 100)
    proof = z0p.air.prove(pz, z0p.Transcript(b"bench/air-scale"), gpu_ctx)
    assert len(proof) == 203553
    ref = oracle.air_prove(po, oracle.Transcript(b"bench/air-scale"))
    assert proof == ref
    assert oracle.air_verify(po, proof, oracle.Transcript(b"bench/air-scale")) == 0


def test_chained_proofs_on_one_transcript(z0p, oracle, gpu_ctx):
    """Proofs chained on one transcript (src/transcript.rs:37-40)."""
    _, b = oracle.build_trace(1, 1, 64)
    po = oracle.air_params_new(64, 8, 12, 8, 1, 1, int(b[-1]), 6, 2)
    pz = z0p.air.Params.new(64, 8, 12, 8, 1, 1, int(b[-1])).with_grinding_bits(6).with_cap_height(2)
    ro = oracle.range_params_new(16, 8, 8, 6, 8, 200, 4, 1)
    rz = z0p.range.Params.new(16, 8, 8, 6, 8, 200).with_grinding_bits(4).with_cap_height(1)
    to, tz = oracle.Transcript(b"chain"), z0p.Transcript(b"chain")
    to.absorb(b"prefix", b"x" * 3000)
    tz.absorb(b"prefix", b"x" * 3000)
    for _ in range(2):
        assert z0p.air.prove(pz, tz, gpu_ctx) == oracle.air_prove(po, to)
        assert z0p.range.prove(rz, tz, gpu_ctx) == oracle.range_prove(ro, to)
        assert tz.export() == to.export()


def test_trim_and_regrow_workspace(z0p, oracle):
    """Proofs after the workspace went back to the pool (and grew again) are unchanged."""
    from z0p_gb300.context import Context

    ctx = Context(0)
    shapes = [(256, 1, 2), (1 << 12, 3, 4), (64, 5, 6)]
    for n, a0, b0 in shapes:
        _, b = oracle.build_trace(a0, b0, n)
        pz = z0p.air.Params.for_security(n, a0, b0, int(b[-1]), 100)
        po = oracle.air_for_security(n, a0, b0, int(b[-1]), 100)
        ref = oracle.air_prove(po, oracle.Transcript(b"trim"))
        assert z0p.air.prove(pz, z0p.Transcript(b"trim"), ctx) == ref
        held = ctx.device_bytes
        ctx.trim()
        assert ctx.device_bytes < min(held, 1 << 20)  # twiddle tables and counters stay
        assert z0p.air.prove(pz, z0p.Transcript(b"trim"), ctx) == ref
    ctx.close()


def test_forged_and_dishonest_statements_prove_structurally(z0p, oracle, gpu_ctx):
    """False claims still prove (src/air.rs:356-364) and fail verification."""
    _, b = oracle.build_trace(1, 1, 32)
    lie = (int(b[-1]) + 5) % oracle.P
    po = oracle.air_params_new(32, 8, 8, 16, 1, 1, lie)
    pz = z0p.air.Params.new(32, 8, 8, 16, 1, 1, lie)
    proof = z0p.air.prove(pz, z0p.Transcript(b"lie"), gpu_ctx)
    assert proof == oracle.air_prove(po, oracle.Transcript(b"lie"))
    assert oracle.air_verify(po, proof, oracle.Transcript(b"lie")) != 0


def test_buffer_too_small_and_errors(z0p, gpu_ctx):
    import ctypes as C

    p = z0p.air.Params.for_security(1024, 1, 1, 1, 100)
    buf = (C.c_uint8 * 100)()
    n = C.c_size_t()
    t = z0p.Transcript(b"x")
    before = t.export()
    rc = z0p.lib().z0p_gpu_air_prove(gpu_ctx.handle, C.byref(p), C.byref(t.state), buf, 100, C.byref(n))
    assert rc == 100 and n.value == 68573
    assert t.export() == before  # no transcript mutation on failure
    bad = z0p.air.Params.for_security(1024, 1, 1, 1, 100)
    bad.num_queries = 0
    with pytest.raises(z0p.Z0pError) as e:
        z0p.air.prove(bad, z0p.Transcript(b"x"), gpu_ctx)
    assert e.value.code == 5


# ------------------------------------------------------- per-stage kernels --


def _torch():
    return pytest.importorskip("torch")


def test_rs_extend_matches_oracle(z0p, oracle, gpu_ctx):
    torch = _torch()
    import ctypes as C
    import numpy as np

    rng = np.random.default_rng(7)
    for logn, batch, blowup in [(4, 3, 16), (10, 2, 16), (13, 4, 16), (16, 2, 8), (17, 1, 4), (10, 2, 64),
                                (3, 1, 128)]:
        n = 1 << logn
        vals = rng.integers(0, oracle.P, size=(batch, n), dtype=np.uint64).astype(np.uint32)
        d_in = torch.from_numpy(vals.astype(np.int64)).to(torch.int32).cuda()
        d_out = torch.empty(batch * n * blowup, dtype=torch.int32, device="cuda")
        torch.cuda.synchronize()
        rc = z0p.lib().z0p_gpu_rs_extend(gpu_ctx.handle, C.c_void_p(d_in.data_ptr()), n, batch, blowup,
                                         C.c_void_p(d_out.data_ptr()))
        assert rc == 0, z0p.lib().z0p_gpu_last_reason()
        got = d_out.cpu().numpy().view(np.uint32).reshape(batch, n * blowup)
        for c in range(batch):
            assert np.array_equal(got[c], oracle.reed_solomon_extend(vals[c], blowup)), (logn, c)


def test_merkle_cap_matches_oracle(z0p, oracle, gpu_ctx):
    torch = _torch()
    import ctypes as C
    import numpy as np

    rng = np.random.default_rng(11)
    # power-of-two and padded (duplicate-last, src/merkle.rs:350-360) leaf counts
    for leaves, cap_h in [(1, 0), (2, 1), (64, 4), (1 << 12, 4), (1 << 15, 8), (1 << 18, 2),
                          (3, 1), (5, 4), (1000, 3), (4097, 8), (3 * (1 << 14), 4)]:
        flat = rng.integers(0, 256, size=leaves * 64, dtype=np.uint8)
        d = torch.from_numpy(flat).cuda()
        out = (C.c_uint8 * (32 * 256))()
        cnt = C.c_uint64()
        torch.cuda.synchronize()
        rc = z0p.lib().z0p_gpu_merkle_flat64_cap(gpu_ctx.handle, C.c_void_p(d.data_ptr()), leaves * 64,
                                                 cap_h, out, C.byref(cnt))
        assert rc == 0
        assert bytes(out)[: 32 * cnt.value] == oracle.merkle_flat64_cap(flat.tobytes(), cap_h), leaves


def test_kernel_sweep_shape_matches_oracle(z0p, oracle, gpu_ctx):
    """The kernel-sweep configuration at reduced n: 64 seeded columns with
    log2 n uniform in {8..12}; each column's LDE at blowup 16
    (reed_solomon_extend, src/ntt.rs:436-439); a Merkle cap over each
    equal-n group's row-major flat buffer (leaf = 16 consecutive limbs,
    src/merkle.rs:93-110); then the FRI fold chain on each LDE lifted to Fp4
    and bit-reversed, with seeded challenges, while the degree bound
    (n - 1) >> 2f is at least 8 (src/fri.rs:1273-1331)."""
    torch = _torch()
    import ctypes as C
    import numpy as np

    P, B = oracle.P, 16
    state = 0x5EED000000000003
    groups = {}
    for _ in range(64):
        z, state = oracle.splitmix64(state)
        logn = 8 + z % 5
        col = np.empty(1 << logn, dtype=np.uint32)
        for i in range(col.size):
            z, state = oracle.splitmix64(state)
            col[i] = z % P
        groups.setdefault(logn, []).append(col)
    for logn, cols in sorted(groups.items()):
        n, k = 1 << logn, len(cols)
        m = n * B
        d_in = torch.from_numpy(np.stack(cols).astype(np.int64)).to(torch.int32).cuda()
        d_lde = torch.empty(k * m, dtype=torch.int32, device="cuda")
        torch.cuda.synchronize()
        assert z0p.lib().z0p_gpu_rs_extend(gpu_ctx.handle, C.c_void_p(d_in.data_ptr()), n, k, B,
                                           C.c_void_p(d_lde.data_ptr())) == 0
        lde = d_lde.cpu().numpy().view(np.uint32).reshape(k, m)
        for c in range(k):
            assert np.array_equal(lde[c], oracle.reed_solomon_extend(cols[c], B)), (logn, c)
        # Merkle over the row-major flat buffer of the group (k may not be a power of two).
        flat = np.ascontiguousarray(lde.T).reshape(-1)
        d_flat = torch.from_numpy(flat.view(np.int32).copy()).cuda()
        out = (C.c_uint8 * (32 * 256))()
        cnt = C.c_uint64()
        torch.cuda.synchronize()
        assert z0p.lib().z0p_gpu_merkle_flat64_cap(gpu_ctx.handle, C.c_void_p(d_flat.data_ptr()),
                                                   flat.size * 4, 4, out, C.byref(cnt)) == 0
        assert bytes(out)[: 32 * cnt.value] == oracle.merkle_flat64_cap(flat.tobytes(), 4), logn
        # FRI fold chain on the first column of the group.
        logm = logn + 4
        omega = oracle.f_pow(31, (P - 1) >> logm)
        lifted = np.zeros(4 * m, dtype=np.uint32)
        br = [int(format(i, f"0{logm}b")[::-1], 2) for i in range(m)]
        lifted[0::4] = lde[0][br]
        pts = [oracle.f_mul(31, oracle.f_pow(omega, int(format(4 * i, f"0{logm}b")[::-1], 2)))
               for i in range(m // 4)]
        cur = lifted
        d_cur = torch.from_numpy(cur.astype(np.int64)).to(torch.int32).cuda()
        depth = 0
        while ((n - 1) >> (2 * depth)) >= 8:
            ch = []
            for _ in range(12):
                z, state = oracle.splitmix64(state)
                ch.append(z % P)
            ref, pts = oracle.fold_layer(cur, pts, np.array(ch, dtype=np.uint32))
            nl = cur.size // 4
            d_next = torch.empty(nl // 4 * 4, dtype=torch.int32, device="cuda")
            torch.cuda.synchronize()
            rc = z0p.lib().z0p_gpu_fri_fold(gpu_ctx.handle, C.c_void_p(d_cur.data_ptr()), nl, m, depth,
                                            (C.c_uint32 * 12)(*ch), C.c_void_p(d_next.data_ptr()))
            assert rc == 0
            got = d_next.cpu().numpy().view(np.uint32)
            assert np.array_equal(got, ref), (logn, depth)
            cur, d_cur = ref, d_next
            depth += 1


def test_fri_fold_matches_oracle(z0p, oracle, gpu_ctx):
    torch = _torch()
    import ctypes as C
    import numpy as np

    P = oracle.P
    rng = np.random.default_rng(3)
    for logm, depth in [(6, 0), (10, 0), (12, 1), (16, 0), (18, 2), (20, 1)]:
        m = 1 << logm
        n = m >> (2 * depth)
        vals = rng.integers(0, P, size=4 * n, dtype=np.uint64).astype(np.uint32)
        ch = rng.integers(0, P, size=12, dtype=np.uint64).astype(np.uint32)
        # quad leaders of layer `depth` (fri::point_at, src/fri.rs:1108-1115)
        omega = oracle.f_pow(31, (P - 1) >> logm)
        bits = logm - 2 * depth
        pts = []
        for i in range(n // 4):
            e = int(format(4 * i, f"0{bits}b")[::-1], 2)
            pts.append(oracle.f_pow(oracle.f_mul(31, oracle.f_pow(omega, e)), 4 ** depth))
        ref, _ = oracle.fold_layer(vals, pts, ch)
        d_in = torch.from_numpy(vals.astype(np.int64)).to(torch.int32).cuda()
        d_out = torch.empty(n, dtype=torch.int32, device="cuda")
        torch.cuda.synchronize()
        rc = z0p.lib().z0p_gpu_fri_fold(gpu_ctx.handle, C.c_void_p(d_in.data_ptr()), n, m, depth,
                                        (C.c_uint32 * 12)(*ch.tolist()), C.c_void_p(d_out.data_ptr()))
        assert rc == 0
        assert np.array_equal(d_out.cpu().numpy().view(np.uint32), ref), (logm, depth)


def test_grind_matches_oracle(z0p, oracle, gpu_ctx):
    """Minimum nonce equals the reference's sequential scan (src/transcript.rs:263-281)."""
    import ctypes as C

    for bits, label in [(1, b"a"), (8, b"b"), (13, b"c"), (18, b"d"), (20, b"fri-pow")]:
        t = oracle.Transcript(b"grind-" + label)
        t.absorb(b"stmt", b"hello")
        # head = H(history) || LE64(|"fri-pow"|) || "fri-pow" (src/transcript.rs:182-189)
        head = _history_digest(oracle, b"grind-" + label) + (7).to_bytes(8, "little") + b"fri-pow"
        nonce = C.c_uint64()
        rc = z0p.lib().z0p_gpu_grind(gpu_ctx.handle, head, len(head), bits, C.byref(nonce))
        assert rc == 0
        assert nonce.value == t.grind(b"fri-pow", bits), bits


def _history_digest(oracle, label):
    # BLAKE3 of the framed history Transcript::new(label); absorb("stmt","hello")
    def frame(l, d):
        return len(l).to_bytes(8, "little") + l + len(d).to_bytes(8, "little") + d

    return oracle.blake3(frame(b"domain", label) + frame(b"stmt", b"hello"))


_UNGATED = r"""
import sys
sys.path.insert(0, sys.argv[1])
import z0p_gb300 as Z
ctx = Z.default_context(0)
out = []
for n, (b, q, f, g, c) in [(64, (8, 12, 8, 0, 0)), (1024, (16, 40, 16, 20, 4)), (256, (4, 12, 4, 2, 1))]:
    p = Z.air.Params.new(n, b, q, f, 1, 1, 0)
    p.grinding_bits = g
    p.cap_height = c
    out.append(Z.air.prove(p, Z.Transcript(b"ungated/%d" % n), ctx).hex())
fp = Z.fri.Params.new(4, 12, 4)
vals = [(7 * i + 3) % 2013265921 for i in range(256)]
st = Z.fri.commit(vals, fp, Z.Transcript(b"ungated/fri"), ctx)
out.append(st.commitment.hex())
print(" ".join(out))
"""


def test_ungated_folds_prove_the_same_bytes(z0p, oracle, gpu_ctx):
    """Where launches are serialised (an injected tool, CUDA_LAUNCH_BLOCKING),
    the small folds are launched after their tables instead of behind gates
    (Z0P_GATES=0 forces the same): the proof bytes do not change."""
    import subprocess
    import sys
    env = dict(os.environ, Z0P_GATES="0")
    r = subprocess.run([sys.executable, "-c", _UNGATED, ROOT], capture_output=True, text=True,
                       env=env, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    ungated = r.stdout.split()
    gated = []
    for n, (b, q, f, g, c) in [(64, (8, 12, 8, 0, 0)), (1024, (16, 40, 16, 20, 4)),
                               (256, (4, 12, 4, 2, 1))]:
        pz = z0p.air.Params.new(n, b, q, f, 1, 1, 0)
        pz.grinding_bits = g
        pz.cap_height = c
        proof = z0p.air.prove(pz, z0p.Transcript(b"ungated/%d" % n), gpu_ctx)
        po = oracle.air_params_new(n, b, q, f, 1, 1, 0, g, c)
        assert proof == oracle.air_prove(po, oracle.Transcript(b"ungated/%d" % n))
        gated.append(proof.hex())
    fp = z0p.fri.Params.new(4, 12, 4)
    vals = [(7 * i + 3) % 2013265921 for i in range(256)]
    gated.append(z0p.fri.commit(vals, fp, z0p.Transcript(b"ungated/fri"), gpu_ctx).commitment.hex())
    assert ungated == gated


_FRESH_SEQUENCE = r"""
import json, sys
sys.path.insert(0, sys.argv[1])
import z0p_gb300 as Z
cases = json.loads(sys.argv[2])
ctx = Z.Context(0)
out = []
for c in cases:
    p = Z.air.Params.new(c["n"], c["blowup"], c["queries"], c["final"], c["a0"], c["b0"], c["b_last"])
    p.grinding_bits = c["grinding"]
    p.cap_height = c["cap"]
    out.append(Z.air.prove(p, Z.Transcript(c["label"].encode()), ctx).hex())
print(" ".join(out))
"""


def test_fresh_context_sequence(z0p, oracle):
    """A fresh context proves a proof without gated launches and then one
    with them (its first gated tail uses the first epoch); the mapped buffer
    still holds the first proof's values where the second's gate words go,
    and the bytes must not depend on them."""
    import subprocess
    import sys
    names = ["air n2 b4", "air fib16", "air n4 b8 f2", "air fib64 bench"]
    cases = [next(c for c in GOLD if c["name"] == n) for n in names]
    r = subprocess.run([sys.executable, "-c", _FRESH_SEQUENCE, ROOT, json.dumps(cases)],
                       capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    got = [bytes.fromhex(x) for x in r.stdout.split()]
    for c, proof in zip(cases, got):
        po, _ = _air_pair(z0p, oracle, c)
        assert proof == oracle.air_prove(po, oracle.Transcript(c["label"].encode())), c["name"]


def test_context_without_gates_proves_the_same_bytes(z0p, oracle):
    """z0p_gpu_ctx_set_gates(ctx, 0), as a pool of several workers sets on its
    contexts: the small folds, the PoW search and the gather wait for their
    inputs on the host; the bytes equal the gated context's and the oracle's."""
    gated, ungated = z0p.Context(0), z0p.Context(0)
    ungated.set_gates(False)
    for name in ["air fib64 bench", "air n256 b4 grind8 cap3", "air prod 1024"]:
        c = next(x for x in GOLD if x["name"] == name)
        po, pz = _air_pair(z0p, oracle, c)
        a = z0p.air.prove(pz, z0p.Transcript(c["label"].encode()), gated)
        b = z0p.air.prove(pz, z0p.Transcript(c["label"].encode()), ungated)
        assert a == b == oracle.air_prove(po, oracle.Transcript(c["label"].encode())), name
