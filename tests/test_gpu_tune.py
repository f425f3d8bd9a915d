"""Launch schedules and the autotuner on the GPU: every NTT split the
schedule can name gives the oracle's LDE bit for bit, proofs are
byte-identical under non-default schedules, and autotuning installs a valid
schedule without changing a proof."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _torch():
    return pytest.importorskip("torch")


@pytest.fixture
def restore_schedule(z0p):
    before = z0p.tune.to_dict(z0p.tune.get(0))
    yield
    z0p.tune.set(z0p.tune.from_dict(before), 0)


def _lde(z0p, ctx, vals, blowup):
    torch = _torch()
    n = vals.size
    d_in = torch.from_numpy(vals.astype(np.int64)).to(torch.int32).cuda()
    d_out = torch.empty(n * blowup, dtype=torch.int32, device="cuda")
    torch.cuda.synchronize()
    rc = z0p.lib().z0p_gpu_rs_extend(ctx.handle, C.c_void_p(d_in.data_ptr()), n, 1, blowup,
                                     C.c_void_p(d_out.data_ptr()))
    assert rc == 0, z0p.lib().z0p_gpu_last_reason()
    return d_out.cpu().numpy().view(np.uint32)


@pytest.mark.parametrize("logn", [13, 14, 16, 17, 20])
def test_every_ntt_split_matches_oracle(z0p, oracle, gpu_ctx, restore_schedule, logn):
    # Every split in [max(7, l - 13), min(13, l - 6)]: all pass-1 and pass-2
    # instantiations at l = 20.
    vals = np.random.default_rng(logn).integers(0, oracle.P, size=1 << logn,
                                                dtype=np.uint64).astype(np.uint32)
    ref = oracle.reed_solomon_extend(vals, 16)
    lo, hi = max(7, logn - 13), min(13, logn - 6)
    for split in range(lo, hi + 1):
        variants = [{}, {"ntt_radix32": [logn]}]  # register groups of 16 and of 32
        if split % 2 == 0 and (logn - split) % 2 == 0 and 6 <= logn - split <= 12 and split <= 12:
            variants.append({"ntt_regpass": [logn]})  # register passes
            variants.append({"ntt_regstream": [logn]})  # streamed through a resident grid
        for v in variants:
            z0p.tune.set(z0p.tune.from_dict({"ntt_log_n1": {str(logn): split}, **v}), 0)
            assert np.array_equal(_lde(z0p, gpu_ctx, vals, 16), ref), (logn, split, v)


SCHEDULES = [
    {"ntt_log_n1": {"16": 7, "14": 8, "13": 7}, "merkle_top_log": 10, "grind_ctas_per_sm": 1},
    {"ntt_log_n1": {"16": 10, "14": 7}, "ntt_radix32": [14, 16, 20], "merkle_top_log": 18,
     "grind_ctas_per_sm": 8},
    {"ntt_log_n1": {"16": 8, "14": 8}, "ntt_regpass": [14, 16], "merkle_top_log": 14},
    {"ntt_log_n1": {"16": 8, "14": 8}, "ntt_regstream": [14, 16], "merkle_top_log": 14},
    {"merkle_top_log": 12, "grind_ctas_per_sm": 16},
]


def test_proofs_identical_under_every_schedule(z0p, oracle, gpu_ctx, restore_schedule):
    # A 2^16-step AIR proof (LDE 16 x 2^16, trees of 2^17 and 2^18 leaves,
    # 20-bit PoW) and a 2^14-row range proof, proved under the default and
    # three other schedules.
    n = 1 << 16
    _, b = oracle.build_trace(3, 5, n)
    air = z0p.air.Params.for_security(n, 3, 5, int(b[-1]), 100)
    rng_p = z0p.range.Params.for_security(1 << 14, 16, 4242, 100)

    def both():
        return (z0p.air.prove(air, z0p.Transcript(b"tune"), gpu_ctx),
                z0p.range.prove(rng_p, z0p.Transcript(b"tune-r"), gpu_ctx))

    z0p.tune.set(z0p.tune.default(), 0)
    base = both()
    po = oracle.air_params_new(n, air.blowup, air.num_queries, air.final_size, 3, 5, int(b[-1]),
                               air.grinding_bits, air.cap_height)
    assert base[0] == oracle.air_prove(po, oracle.Transcript(b"tune"))
    for d in SCHEDULES:
        z0p.tune.set(z0p.tune.from_dict(d), 0)
        assert both() == base, d


def test_autotune_installs_schedule_and_keeps_bytes(z0p, gpu_ctx, restore_schedule):
    n = 1 << 14
    _, b_last = z0p.air.trace_last(1, 1, n)
    air = z0p.air.Params.for_security(n, 1, 1, b_last, 100)
    z0p.tune.set(z0p.tune.default(), 0)
    before = z0p.air.prove(air, z0p.Transcript(b"autotune"), gpu_ctx)
    sched, report = z0p.tune.autotune(gpu_ctx, max_log_n=16)
    assert z0p.tune.to_dict(z0p.tune.get(0)) == z0p.tune.to_dict(sched)
    assert set(report["ntt_us"]) == {"13", "14", "15", "16"}
    for v in report["ntt_us"].values():
        assert 0 < v["chosen"] <= v["default"]
    assert 0 < report["merkle_2p21_us"]["chosen"] <= report["merkle_2p21_us"]["default"]
    assert 0 < report["grind_8x20bit_us"]["chosen"] <= report["grind_8x20bit_us"]["default"]
    assert z0p.air.prove(air, z0p.Transcript(b"autotune"), gpu_ctx) == before
