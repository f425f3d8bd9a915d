"""Batched and served proving (GPU): every result equals the proof made alone.

Covers the pool of include/z0p_gpu.h. A mixed batch of Fibonacci and
range-check jobs of uneven sizes must give, for every job:
- the single-proof path's bytes and the oracle's bytes;
- the oracle's transcript post-state.
Served submissions that arrive while other jobs run must give the same
results. Admission rejects a job larger than the HBM budget before any work.
"""
import threading
import time

import pytest

pytestmark = pytest.mark.gpu


def _jobs(z0p, oracle, seed, n_air, n_range, log_lo=6, log_hi=13):
    P = oracle.P
    state = seed
    out = []
    for i in range(n_air + n_range):
        z, state = oracle.splitmix64(state)
        if i < n_air:
            logn = log_lo + z % (log_hi - log_lo + 1)
            z1, state = oracle.splitmix64(state)
            z2, state = oracle.splitmix64(state)
            a0, b0 = z1 % P, z2 % P
            _, b_last = z0p.air.trace_last(a0, b0, 1 << logn)
            pz = z0p.air.Params.for_security(1 << logn, a0, b0, b_last, 100)
            po = oracle.air_for_security(1 << logn, a0, b0, b_last, 100)
            out.append(("air", pz, po, b"batch/air-%d" % i))
        else:
            logn = 6 + z % 5
            z1, state = oracle.splitmix64(state)
            value = z1 % (1 << 16)
            pz = z0p.range.Params.for_security(1 << logn, 16, value, 100)
            po = oracle.range_for_security(1 << logn, 16, value, 100)
            out.append(("range", pz, po, b"batch/range-%d" % i))
    return out


def _oracle_proof(oracle, kind, po, label):
    t = oracle.Transcript(label)
    proof = (oracle.air_prove if kind == "air" else oracle.range_prove)(po, t)
    return proof, t.export()


def test_batch_matches_alone_and_oracle(z0p, oracle, gpu_ctx):
    from z0p_gb300.pool import Pool

    specs = _jobs(z0p, oracle, 0x5EED000000000003, 10, 6)
    pool = Pool(0, workers=6)
    transcripts = [z0p.Transcript(label) for _, _, _, label in specs]
    jobs = [pool.make_job(pz, t) for (_, pz, _, _), t in zip(specs, transcripts)]
    proofs = pool.prove_all(jobs)
    for (kind, pz, po, label), proof, t in zip(specs, proofs, transcripts):
        ref, ref_state = _oracle_proof(oracle, kind, po, label)
        assert proof == ref, label
        assert t.export() == ref_state, label
        alone = (z0p.air if kind == "air" else z0p.range).prove(pz, z0p.Transcript(label), gpu_ctx)
        assert alone == proof, label
    pool.close()


def test_served_arrivals_overlap(z0p, oracle):
    from z0p_gb300.pool import Pool

    specs = _jobs(z0p, oracle, 0x5EED000000000004, 8, 4, log_lo=8, log_hi=14)
    pool = Pool(0, workers=4)
    tickets = {}
    transcripts = {}

    def arrive():
        for i, (kind, pz, po, label) in enumerate(specs):
            transcripts[i] = z0p.Transcript(label)
            tickets[i] = pool.submit(pool.make_job(pz, transcripts[i]))
            time.sleep(0.002)

    th = threading.Thread(target=arrive)
    th.start()
    th.join()
    for i, (kind, pz, po, label) in enumerate(specs):
        proof = pool.wait(tickets[i], 60000)
        ref, ref_state = _oracle_proof(oracle, kind, po, label)
        assert proof == ref, label
        assert transcripts[i].export() == ref_state
    pool.close()


def test_admission_rejects_oversized_job(z0p):
    from z0p_gb300.pool import Pool

    pool = Pool(0, workers=1, hbm_budget=64 << 20)
    big = z0p.air.Params.for_security(1 << 20, 1, 1, 1, 100)
    with pytest.raises(z0p.Z0pError) as e:
        pool.submit(pool.make_job(big, z0p.Transcript(b"big")))
    assert e.value.code == 105
    # a job that fits still runs on the same pool
    small = z0p.air.Params.for_security(1 << 8, 1, 1, z0p.air.trace_last(1, 1, 1 << 8)[1], 100)
    t = pool.submit(pool.make_job(small, z0p.Transcript(b"small")))
    assert len(pool.wait(t, 60000)) == small.proof_size()
    pool.close()
