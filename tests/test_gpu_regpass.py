"""The register-pass NTT variants (launch schedule variant 2: two register
passes per half with one shared-memory transpose, pass-1 tiles by TMA tensor
copies and pass-2 rows by bulk copies; variant 3: the same tiles streamed
through a resident grid) against the oracle on every path that
reaches it: the interpolation (inverse, 31^k / n scaling) and the coset LDE
of z0p_gpu_rs_extend for every half size 2^6..2^12 and batched inputs, the
FRI commitment of base coefficients (31^i applied on load), the caller
columns of prove_with_trace (checked on load), and whole proofs."""
import ctypes as C
import random

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

P = 2**31 - 2**27 + 1


@pytest.fixture(params=["ntt_regpass", "ntt_regstream"])
def regpass(z0p, request):
    # Variant 2 (one tile per CTA) and variant 3 (streamed: a resident grid,
    # two tile buffers per CTA; 2^12 halves take variant 2's kernel).
    before = z0p.tune.to_dict(z0p.tune.get(0))

    def use(splits):
        z0p.tune.set(z0p.tune.from_dict({"ntt_log_n1": {str(l): s for l, s in splits.items()},
                                         request.param: sorted(splits)}), 0)
    yield use
    z0p.tune.set(z0p.tune.from_dict(before), 0)


def _rs_extend(z0p, ctx, vals, batch, blowup):
    torch = pytest.importorskip("torch")
    n = vals.size // batch
    d_in = torch.from_numpy(vals.view(np.int32)).cuda()
    d_out = torch.empty(vals.size * blowup, dtype=torch.int32, device="cuda")
    torch.cuda.synchronize()
    rc = z0p.lib().z0p_gpu_rs_extend(ctx.handle, C.c_void_p(d_in.data_ptr()), n, batch, blowup,
                                     C.c_void_p(d_out.data_ptr()))
    assert rc == 0, z0p.lib().z0p_gpu_last_reason()
    return d_out.cpu().numpy().view(np.uint32)


# (log n, pass-1 log length, batch, blowup): halves 8/6, 8/8, 8/10, 10/10,
# 10/12, 12/10, 12/12 (a pass 1 of 2^6 points is outside every split range)
CASES = [(14, 8, 3, 4), (16, 8, 1, 16), (18, 8, 1, 8), (20, 10, 1, 16), (20, 10, 2, 4),
         (22, 10, 1, 4), (22, 12, 1, 2), (24, 12, 1, 2)]


@pytest.mark.parametrize("case", CASES, ids=[f"n{c[0]}-s{c[1]}-b{c[2]}-B{c[3]}" for c in CASES])
def test_regpass_lde_matches_oracle(z0p, oracle, gpu_ctx, regpass, case):
    logn, split, batch, blowup = case
    assert max(7, logn - 13) <= split <= min(13, logn - 6)
    regpass({logn: split})
    n = 1 << logn
    vals = np.random.default_rng(logn * 100 + split).integers(0, P, size=batch * n,
                                                              dtype=np.uint64).astype(np.uint32)
    got = _rs_extend(z0p, gpu_ctx, vals, batch, blowup).reshape(batch, n * blowup)
    for b in range(batch):
        assert np.array_equal(got[b], oracle.reed_solomon_extend(vals[b * n:(b + 1) * n], blowup)), b


def test_regpass_fri_commit_base_coefficients(z0p, oracle, gpu_ctx, regpass):
    # 2^14 base coefficients at blowup 16: the LDE transform scales them by
    # 31^i as it loads them.
    regpass({14: 8})
    rng = random.Random(14)
    values = [rng.randrange(P) for _ in range(1 << 14)]
    pz = z0p.fri.Params.new(16, 20, 16).with_grinding_bits(4).with_cap_height(3)
    po = oracle.FriParams(16, 20, 16, 4, 3)
    tg, to = z0p.Transcript(b"reg/pcs"), oracle.Transcript(b"reg/pcs")
    st = z0p.fri.commit(values, pz, tg, gpu_ctx)
    so = oracle.fri_commit(po, 0, values, to)
    assert st.commitment == so.commitment
    assert z0p.fri.open(st, tg) == oracle.fri_open(so, to)


def test_regpass_prove_with_trace_and_bad_columns(z0p, oracle, gpu_ctx, regpass):
    # The caller's columns are interpolated by the register passes, which
    # check every word on load.
    regpass({14: 8})
    n = 1 << 14
    a, b = oracle.build_trace(5, 7, n)
    pz = z0p.air.Params.new(n, 4, 12, 4, 5, 7, int(b[-1])).with_grinding_bits(4).with_cap_height(2)
    po = oracle.air_params_new(n, 4, 12, 4, 5, 7, int(b[-1]))
    po.grinding_bits, po.cap_height = 4, 2
    tg, to = z0p.Transcript(b"reg/pwt"), oracle.Transcript(b"reg/pwt")
    assert z0p.air.prove_with_trace(pz, a, b, tg, gpu_ctx) == oracle.air_prove_with_trace(po, a, b, to)
    assert tg.export() == to.export()
    bad = [int(v) for v in a]
    bad[n // 3] = P + 5
    t = z0p.Transcript(b"reg/bad")
    before = t.export()
    with pytest.raises(z0p.Z0pError) as e:
        z0p.air.prove_with_trace(pz, bad, b, t, gpu_ctx)
    assert e.value.code == 8
    assert t.export() == before


@pytest.mark.parametrize("logn", [16, 20])
def test_regpass_proofs_match_oracle(z0p, oracle, gpu_ctx, regpass, logn):
    regpass({logn: logn // 2})
    n = 1 << logn
    _, b = oracle.build_trace(3, 9, n)
    pz = z0p.air.Params.for_security(n, 3, 9, int(b[-1]), 100)
    po = oracle.air_for_security(n, 3, 9, int(b[-1]), 100)
    assert z0p.air.prove(pz, z0p.Transcript(b"reg/air"), gpu_ctx) == \
        oracle.air_prove(po, oracle.Transcript(b"reg/air"))
