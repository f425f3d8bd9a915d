"""Benchmark: proved Fibonacci-AIR steps/s on the GB300 prove path.

Workload (one step = one proof): Fibonacci AIR with 2^20 steps, production
schedule air::Params::for_security(N, a0, b0, b_last, 100) — blowup 16
(LDE 2^24), 40 queries, 20-bit PoW, cap height 4, final layer 16 — with the
initial pair drawn from splitmix64 seeded 0x5EED000000000001 (per rank: the
rank is added to the seed). Every proof is byte-exact with the reference's
format (checked against the CPU oracle once per run, outside the timed
region).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]

Prints one JSON line (rank 0). `--impl reference` times the CPU prover
(the C restatement in oracle/, all host threads) on the same workload.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

P = 2013265921
LOG_N = 20
N_STEPS = 1 << LOG_N
SEED = 0x5EED000000000001
# The reference's published 2^20-step Fibonacci prove on its 16-core machine:
# 1,733.55 ms, i.e. 604,872 steps/s (docs/benchmarks.md:30-36).
PUBLISHED_STEPS_PER_S = 604872.0
LABEL = b"bench/air-scale"
METRIC = "proved AIR steps/s (batched vs plain, byte-exact proofs); p50/p99 prove latency"


def bench_config():
    """The workload's config, identical in the GB300 and reference lines."""
    return {"workload": "fibonacci-air prove, 2^20 steps, for_security(100): B16 Q40 G20 C4 F16",
            "n_steps": N_STEPS, "lde_len": N_STEPS * 16, "proof_bytes": 203553,
            "l2": "inputs larger than L2: per-proof working set ~0.9 GB > 129 MB L2"}


def splitmix64(state):
    state = (state + 0x9E3779B97F4A7C15) & (2**64 - 1)
    z = state
    z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & (2**64 - 1)
    z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & (2**64 - 1)
    return z ^ (z >> 31), state


def workload(rank=0):
    z1, s = splitmix64(SEED + rank)
    z2, _ = splitmix64(s)
    return z1 % P, z2 % P


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def aggregate_replicas(dist, dev_ms, wall_s, device):
    """Replicas: every rank proves its own proofs; the job's time is the
    slowest rank's (device-event and wall clock), so value = all ranks'
    steps / that time. No data crosses ranks but these two numbers."""
    if dist is None:
        return dev_ms, wall_s
    import torch

    t = torch.tensor([dev_ms, wall_s], device=device, dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t[0]), float(t[1])


# ------------------------------------------------------------------ clocks --
REASONS = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]


class ClockSampler:
    """nvidia-smi sampling during the timed region (read-only queries)."""

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.lines = []

    def start(self):
        q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
             "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
             "clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.index}", f"--query-gpu={q}", "--format=csv,noheader,nounits",
                 "-lms", "100"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except (OSError, FileNotFoundError):
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, mx, reasons, power = [], [], set(), []
        for line in self.lines:
            parts = [x.strip() for x in line.split(",")]
            if len(parts) < 7:
                continue
            try:
                sm.append(float(parts[0]))
                mx.append(float(parts[1]))
                power.append(float(parts[2]))
            except ValueError:
                continue
            for name, v in zip(REASONS, parts[3:7]):
                if v.lower().startswith("active"):
                    reasons.add(name)
        return {
            "sm_mhz": statistics.median(sm) if sm else None,
            "sm_max_mhz": max(mx) if mx else None,
            "power_w_max": max(power) if power else None,
            "samples": len(sm),
            "reasons": sorted(reasons),
        }


# ---------------------------------------------------------------- roofline --
def measured_peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(path) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback"


def measured_traffic():
    """Per stage, one captured launch of its main kernel in this workload
    (profiles/traffic_air_prove_2p20.json, ncu with -k <kernel> -c 1): its
    DRAM bytes, its algorithmic bytes and its ALU-pipe %, or {}."""
    try:
        with open(os.path.join(ROOT, "profiles", "traffic_air_prove_2p20.json")) as f:
            return json.load(f)["stages"]
    except (OSError, KeyError, ValueError):
        return {}


def measured_alu():
    """Per-stage ALU-pipe % of the dominant kernel from the same committed
    ncu captures, or {}."""
    return {k: v["alu_pipe_pct"] for k, v in measured_traffic().items() if "alu_pipe_pct" in v}


def stage_work(n, params):
    """Algorithmic bytes / BLAKE3 compressions per stage of one proof."""
    m = n * params.blowup
    F = params.final_size
    layers = []
    L = m
    while True:
        layers.append(L)
        if L <= F:
            break
        L //= 4
    # Column B is derived from A (linked column), so one column is
    # interpolated and extended; the trace-leaf pass stores 1/(x - w_last)
    # per row for the composition.
    work = {
        "trace": {"bytes": 8 * n},                       # both columns written
        "intt": {"bytes": 8 * n},                        # column A: read + write
        "ntt": {"bytes": 4 * n + 4 * m},                 # coefficients in, coset LDE out
        "trace_leaves": {"bytes": 4 * m + 4 * m + 32 * (m // 8), "compressions": m // 8},
        "air_compose_leaves": {"bytes": 4 * m + 4 * m + 16 * m + 32 * (m // 4), "compressions": m // 4},
        "fri_fold_leaves": {"bytes": sum(16 * l + 4 * l + 32 * (l // 16) for l in layers[:-1] if l >= 16),
                            "compressions": sum(l // 16 for l in layers[:-1] if l >= 16)},
        "grind": {"compressions": 1 << params.grinding_bits},  # expected nonces
    }
    nodes = (m // 8 - 1) + sum((l // 4 if l % 4 == 0 else l) - 1 for l in layers)
    work["merkle_levels"] = {"bytes": 96 * nodes, "compressions": 2 * nodes}
    return work


class UtilSampler:
    """nvidia-smi utilization.gpu every 20 ms (the percent of the driver's
    sample window in which a kernel was running; read-only query)."""

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.index}", "--query-gpu=utilization.gpu",
                 "--format=csv,noheader,nounits", "-lms", "20"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=lambda: [self.lines.append(x.strip()) for x in self.proc.stdout],
                                      daemon=True)
            self.t.start()
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def stop(self):
        if not self.proc:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        v = []
        for x in self.lines:
            try:
                v.append(float(x))
            except ValueError:
                pass
        if not v:
            return None
        return {"samples": len(v), "mean_pct": round(statistics.mean(v), 1),
                "median_pct": statistics.median(v), "p10_pct": _pct(v, 0.1)}


def _device_work_ms(Z, ctx, specs):
    """Device time of each proof of specs proved alone: the sum of its kernel
    stages, timed by the library's CUDA events (profiling mode)."""
    out = []
    ctx.set_profiling(True)
    try:
        for params, _, label in specs:
            mod = Z.air if isinstance(params, Z.air.Params) else Z.range
            mod.prove(params, Z.Transcript(label), ctx)
            prof = ctx.profile()
            prof.pop("host", None)
            out.append(sum(v["ms"] for v in prof.values()))
    finally:
        ctx.set_profiling(False)
    return out


# ------------------------------------------------- batched / served configs --
def _mix_params(Z, seed, n_air, n_range, air_logs, range_logs):
    """Seeded job mix: Fibonacci AIRs (log2 steps uniform in air_logs) and
    16-bit range checks (log2 rows uniform in range_logs), for_security(100)."""
    state = seed
    specs = []
    for i in range(n_air + n_range):
        z, state = splitmix64(state)
        if i < n_air:
            logn = air_logs[z % len(air_logs)]
            z1, state = splitmix64(state)
            z2, state = splitmix64(state)
            a0, b0 = z1 % P, z2 % P
            _, b_last = Z.air.trace_last(a0, b0, 1 << logn)
            specs.append((Z.air.Params.for_security(1 << logn, a0, b0, b_last, 100), 1 << logn,
                          b"bench/air-scale"))
        else:
            logn = range_logs[z % len(range_logs)]
            z1, state = splitmix64(state)
            specs.append((Z.range.Params.for_security(1 << logn, 16, z1 % (1 << 16), 100),
                          1 << logn, b"bench/range"))
    return specs


def _prove_plain(Z, ctx, specs):
    out, lat = [], []
    for params, _, label in specs:
        t0 = time.perf_counter()
        mod = Z.air if isinstance(params, Z.air.Params) else Z.range
        out.append(mod.prove(params, Z.Transcript(label), ctx))
        lat.append(time.perf_counter() - t0)
    return out, lat


def _pct(xs, q):
    xs = sorted(xs)
    return xs[min(len(xs) - 1, int(q * len(xs)))]


def run_batched(Z, ctx, workers=16):
    """256 proofs: 192 Fibonacci (2^10..2^18 steps) + 64 range (2^12..2^16 rows)."""
    from z0p_gb300.pool import Pool

    specs = _mix_params(Z, 0x5EED000000000003, 192, 64, list(range(10, 19)), list(range(12, 17)))
    steps = sum(n for _, n, _ in specs)
    _prove_plain(Z, ctx, specs[:8])  # warm the plain context
    t0 = time.perf_counter()
    plain, plain_lat = _prove_plain(Z, ctx, specs)
    t_plain = time.perf_counter() - t0
    pool = Pool(ctx.device, workers=workers)
    warm = [pool.make_job(p, Z.Transcript(l)) for p, _, l in specs[:2 * workers]]
    pool.prove_all(warm)
    jobs = [pool.make_job(p, Z.Transcript(l)) for p, _, l in specs]
    t0 = time.perf_counter()
    batched = pool.prove_all(jobs)
    t_batch = time.perf_counter() - t0
    lat = [j.end_s - j.submit_s for j in jobs]
    pool.close()
    return {
        "workload": "192 fibonacci (2^10..2^18 steps) + 64 range-16 (2^12..2^16 rows), for_security(100)",
        "proofs": len(specs), "steps": steps, "workers": workers,
        "plain_serial_s": t_plain, "batched_s": t_batch,
        "plain_steps_per_s": steps / t_plain, "batched_steps_per_s": steps / t_batch,
        "speedup_vs_plain": t_plain / t_batch,
        "byte_identical_to_plain": all(a == b for a, b in zip(plain, batched)),
        "plain_latency_ms": {"p50": 1e3 * _pct(plain_lat, 0.5), "p99": 1e3 * _pct(plain_lat, 0.99)},
        "batched_latency_ms": {"p50": 1e3 * _pct(lat, 0.5), "p99": 1e3 * _pct(lat, 0.99)},
    }


def run_fri_pcs(Z, ctx, reps=5):
    """FRI as a polynomial commitment (fri::commit + fri::open): the reference's
    `fri prod` rows (docs/benchmarks.md:24,26; coefficients and labels of
    benches/speed_size.rs:607-647, 756-795) and a 2^20-coefficient commitment.
    Host coefficients in, commitment and proof bytes out, per call."""
    rows = []
    for n, label, ref_ms, ref_bytes in [(256, b"bench/fri-prod", 10.59, 29378),
                                        (1024, b"bench/fri-prod-big", 21.50, 43174),
                                        (1 << 20, b"bench/fri-pcs-2p20", None, None)]:
        coeffs = bench_coeffs(n)
        params = Z.fri.Params.for_security(n, 100)
        times, size = [], 0
        for _ in range(reps + 1):
            t = Z.Transcript(label)
            t0 = time.perf_counter()
            st = Z.fri.commit(coeffs, params, t, ctx)
            proof, _ = Z.fri.open(st, t)
            times.append(time.perf_counter() - t0)
            size = len(st.commitment) + len(proof)
        ms = 1e3 * sorted(times[1:])[len(times[1:]) // 2]
        rows.append({"poly_len": n, "lde_len": 16 * n, "ms": round(ms, 4), "bytes": size,
                     "reference_ms_16_cores": ref_ms, "reference_bytes": ref_bytes,
                     "bytes_match_reference": None if ref_bytes is None else size == ref_bytes})
    return {"workload": "fri::Params::for_security(n, 100): B16 Q40 G20 C4 F16; commit + open",
            "rows": rows}


def bench_coeffs(n):
    """benches/speed_size.rs:203-205, 609-611: Field::new(i.wrapping_mul(0x9e37_79b9) + 17)."""
    import numpy as np

    i = np.arange(n, dtype=np.uint64)
    return (((i * 0x9E3779B9) + 17) % 2**32 % P).astype(np.uint32)


def run_published(Z, ctx):
    """Every published prove row of the reference that this backend covers
    (docs/benchmarks.md:21-27, 119-127), on the reference's own workloads,
    parameters and labels (benches/speed_size.rs:201-483, 607-795): the
    median wall-clock of the public call (host inputs in, proof bytes in host
    memory out) beside the reference's published 16-core time, and the proof
    size beside its published size."""
    def fib_params(n, new_args=None):
        _, b_last = Z.air.trace_last(1, 1, n)
        if new_args:
            return Z.air.Params.new(n, *new_args, 1, 1, b_last)
        return Z.air.Params.for_security(n, 1, 1, b_last, 100)

    def fri_row(params, n, label):
        coeffs = bench_coeffs(n)

        def run():
            t = Z.Transcript(label)
            st = Z.fri.commit(coeffs, params, t, ctx)
            proof, _ = Z.fri.open(st, t)
            return len(st.commitment) + len(proof)
        return run

    def air_row(params, label):
        return lambda: len(Z.air.prove(params, Z.Transcript(label), ctx))

    def range_row():
        params = Z.range.Params.new(8, 16, 8, 8, 4, 12345)
        return lambda: len(Z.range.prove(params, Z.Transcript(b"bench/range"), ctx))

    def table_row():
        params = Z.table.Params.new(8, 8, 8, 4, 30)
        return lambda: len(Z.table.prove(params, [10, 20, 30, 40], Z.Transcript(b"bench/table"), ctx))

    def fold_row():
        segs, a, b = [], 1, 1
        for _ in range(4):
            ca, cb = [], []
            for _ in range(8):
                ca.append(a)
                cb.append(b)
                a, b = b, (a + b) % P
            a, b = ca[-1], cb[-1]
            segs.append((ca, cb))
        params = Z.fold.Params.new(8, 8, 8, 4, 1, 1, segs[-1][1][-1])

        def run():
            t = Z.Transcript(b"bench/fold")
            acc = Z.fold.Accumulator(params, ctx)
            for ca, cb in segs:
                acc.add_segment(ca, cb, t)
            n = len(acc.finalize(t))
            acc.close()
            return n
        return run

    rows = [
        ("fri poly256 B4 Q12", fri_row(Z.fri.Params.new(4, 12, 4), 256, b"bench/fri"), 0.15, 11522),
        ("air fib64", air_row(fib_params(64, (8, 12, 8)), b"bench/air"), 0.17, 15465),
        ("range 16-bit", range_row(), 0.10, 5217),
        ("table 4-entry", table_row(), 0.04, 4673),
        ("fold 4x8 fib", fold_row(), 0.19, 16845),
        ("air fib1024", air_row(fib_params(1024, (8, 12, 8)), b"bench/air1024"), 2.01, 28257),
        ("fri prod B16Q40G20C4F16 (poly-256)",
         fri_row(Z.fri.Params.for_security(256, 100), 256, b"bench/fri-prod"), 10.59, 29378),
        ("air prod B16Q40G20C4F16 (fib-64)", air_row(fib_params(64), b"bench/air-prod"), 11.99, 33061),
        ("fri prod P1024 B16Q40G20C4F16",
         fri_row(Z.fri.Params.for_security(1024, 100), 1024, b"bench/fri-prod-big"), 21.50, 43174),
        ("air prod N1024", air_row(fib_params(1024), b"bench/air-scale"), 37.05, 68573),
        ("air prod N8192", air_row(fib_params(8192), b"bench/air-scale"), 49.81, 101233),
        ("air prod N65536", air_row(fib_params(65536), b"bench/air-scale"), 115.49, 141641),
        ("air prod N1048576", air_row(fib_params(1 << 20), b"bench/air-scale"), 1733.55, 203553),
    ]
    out = []
    for name, run, ref_ms, ref_bytes in rows:
        size = run()  # warm-up (first use of a shape allocates its workspace)
        times = []
        for _ in range(21):
            t0 = time.perf_counter()
            run()
            times.append(time.perf_counter() - t0)
        ms = 1e3 * statistics.median(times)
        out.append({"row": name, "ms": round(ms, 4), "reference_ms_16_cores": ref_ms,
                    "speedup": round(ref_ms / ms, 2), "bytes": size, "reference_bytes": ref_bytes,
                    "bytes_match_reference": size == ref_bytes})
    return {"timing": "median of 21 calls after one warm-up; host inputs in, proof bytes in host memory",
            "rows": out}


def run_scale(Z, ctx, reps=5):
    """The other prove entry points at 2^20 rows, production schedule
    (for_security(100)): range::prove (16-bit, value 12,345; the batched and
    served mixes use the same shape at smaller n) and the same columns
    through range::prove_with_columns (row by row), range::prove_zk
    (n_rand = num_queries), table::prove_zk and air::prove_zk with
    n_rand = 16 * num_queries (src/air.rs:445-458; padded
    trace 2^21, LDE 2^25, final layer 32), and air::prove_with_trace on host
    columns."""
    import numpy as np

    n = 1 << 20
    a0, b0 = workload(0)
    _, b_last = Z.air.trace_last(a0, b0, n)
    air_p = Z.air.Params.for_security(n, a0, b0, b_last, 100)
    range_p = Z.range.Params.for_security(n, 16, 12345, 100)
    n_rand = 16 * air_p.num_queries
    # The masked LDE is 2^25 rows; its FRI ends in a 32-value layer (the
    # fold chain divides m / final_size by 4).
    zk_p = Z.air.Params.new(n, 16, air_p.num_queries, 32, a0, b0, b_last) \
        .with_grinding_bits(air_p.grinding_bits).with_cap_height(air_p.cap_height)
    ca = np.empty(n, np.uint32)
    cb = np.empty(n, np.uint32)
    a, b = a0, b0
    for i in range(n):  # the Fibonacci trace, built once on the host
        ca[i], cb[i] = a, b
        a, b = b, (a + b) % P
    rv = np.full(n, 12345, np.uint32)
    rbits = [np.full(n, (12345 >> c) & 1, np.uint32) for c in range(16)]
    table = [10, 20, 30, 12345]
    range_zk_p = Z.range.Params.new(n, 16, 16, air_p.num_queries, 32, 12345) \
        .with_grinding_bits(air_p.grinding_bits).with_cap_height(air_p.cap_height)
    table_p = Z.table.Params.new(n, 16, air_p.num_queries, 32, 12345) \
        .with_grinding_bits(air_p.grinding_bits).with_cap_height(air_p.cap_height)
    cases = [
        ("range::prove 16-bit, 2^20 rows", n, lambda: Z.range.prove(range_p, Z.Transcript(b"bench/range"), ctx)),
        ("range::prove_with_columns, the same columns row by row", n,
         lambda: Z.range.prove_with_columns(range_p, rv, rbits, Z.Transcript(b"bench/range"), ctx)),
        ("table::prove_zk, 2^20 rows, 4 entries, n_rand %d" % n_rand, n,
         lambda: Z.table.prove_zk(table_p, table, n_rand, Z.rng.ChaCha20.new(bytes(32), bytes(12)),
                                  Z.Transcript(b"bench/table-zk"), ctx)),
        ("air::prove_zk, 2^20 steps, n_rand %d" % n_rand, n,
         lambda: Z.air.prove_zk(zk_p, n_rand, Z.rng.ChaCha20.new(bytes(32), bytes(12)),
                                Z.Transcript(b"bench/air-zk"), ctx)),
        ("range::prove_zk 16-bit, 2^20 rows, n_rand %d (LDE 2^25, final 32)" % air_p.num_queries, n,
         lambda: Z.range.prove_zk(range_zk_p, air_p.num_queries, Z.rng.ChaCha20.new(bytes(32), bytes(12)),
                                  Z.Transcript(b"bench/range-zk"), ctx)),
        ("air::prove_with_trace, 2^20 steps (host columns)", n,
         lambda: Z.air.prove_with_trace(air_p, ca, cb, Z.Transcript(b"bench/air-scale"), ctx)),
    ]
    rows = []
    for name, steps, run in cases:
        size = len(run())
        times = []
        for _ in range(reps):
            t0 = time.perf_counter()
            run()
            times.append(time.perf_counter() - t0)
        ms = 1e3 * statistics.median(times)
        rows.append({"row": name, "ms": round(ms, 4), "rows_per_s": round(steps / (ms / 1e3)),
                     "bytes": size})
    return {"workload": "for_security(100): B16 Q40 G20 C4 F16", "rows": rows}


def sweep_values(start, count):
    """Elements start..start+count of the kernel-sweep stream:
    Field::from_u64(splitmix64) with the state advanced once per element
    (gf2.rs:425-431, babybear.rs:66-69), vectorised."""
    import numpy as np

    s = (np.uint64(SWEEP_SEED) + (np.arange(start + 1, start + count + 1, dtype=np.uint64)
                                  * np.uint64(0x9E3779B97F4A7C15)))
    z = (s ^ (s >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
    z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
    z = z ^ (z >> np.uint64(31))
    return (z % np.uint64(P)).astype(np.uint32)


SWEEP_SEED = 0x5EED000000000003


def sweep_columns():
    """The kernel-sweep configuration: 64 columns, log2 n uniform in {16..22}
    (one splitmix64 draw each), grouped by n; column values follow in one
    stream, column after column."""
    state = SWEEP_SEED ^ 0xC0FFEE
    logs = []
    for _ in range(64):
        z, state = splitmix64(state)
        logs.append(16 + z % 7)
    cols, at = [], 0
    for logn in logs:
        cols.append((logn, at))
        at += 1 << logn
    return cols


def device_seconds(ctx, fn):
    """Device time of the kernel stages fn runs on ctx's stream: the
    library's CUDA events around every stage (profiling mode), summed."""
    ctx.set_profiling(True)
    try:
        fn()
        prof = ctx.profile()
    finally:
        ctx.set_profiling(False)
    prof.pop("host", None)
    return sum(v["ms"] for v in prof.values()) / 1e3


def run_sweep(Z, ctx):
    """The kernel-sweep configuration at full size: per equal-n group, the
    coset LDE at blowup 16 (reed_solomon_extend, ntt.rs:436-439), a Merkle
    cap over the group's row-major flat buffer (from_flat64, merkle.rs:93-110)
    and, per column, the arity-4 fold chain (fri.rs:1273-1331) on the LDE
    lifted to Fp4 and bit-reversed, with seeded challenges, while the degree
    bound (n - 1) >> 2f is at least 8. Device inputs. Each stage is timed
    on the device: the library's CUDA events on the context stream around
    every kernel stage of the call (profiling mode), summed, after an
    untimed call of the same size (which sizes the workspace); host launch
    and synchronisation gaps are excluded, and layouts between stages
    (transpose, lift, bit reversal) are untimed."""
    import ctypes as C

    import numpy as np
    import torch

    from z0p_gb300._lib import check

    peak, peak_kind = measured_peaks()
    L = Z.lib()
    groups = {}
    for logn, at in sweep_columns():
        groups.setdefault(logn, []).append(at)
    B = 16
    t_lde = t_merkle = t_fold = 0.0
    by_lde = by_merkle = by_fold = 0
    compressions = 0
    rows = []
    state = SWEEP_SEED ^ 0xF01D
    for logn in sorted(groups):
        n, k = 1 << logn, len(groups[logn])
        m = n * B
        vals = np.concatenate([sweep_values(at, n) for at in groups[logn]])
        d_in = torch.from_numpy(vals.view(np.int32)).cuda()
        d_lde = torch.empty(k * m, dtype=torch.int32, device="cuda")
        torch.cuda.synchronize()
        def lde():
            check(L.z0p_gpu_rs_extend(ctx.handle, C.c_void_p(d_in.data_ptr()), n, k, B,
                                      C.c_void_p(d_lde.data_ptr())))
        lde()  # sizes the workspace for this n
        dt_lde = device_seconds(ctx, lde)
        flat = d_lde.view(k, m).t().contiguous()  # row-major: leaf = 16 consecutive limbs
        torch.cuda.synchronize()
        out = (C.c_uint8 * (32 * 16))()
        cnt = C.c_uint64()
        def merkle():
            check(L.z0p_gpu_merkle_flat64_cap(ctx.handle, C.c_void_p(flat.data_ptr()), 4 * k * m, 4, out,
                                              C.byref(cnt)))
        merkle()
        dt_merkle = device_seconds(ctx, merkle)
        del flat
        leaves = k * m // 16
        npad = 1 << (leaves - 1).bit_length()
        dt_fold, fold_bytes = 0.0, 0
        logm = logn + 4
        br = torch.arange(m, device="cuda", dtype=torch.int64)
        rev = torch.zeros_like(br)
        for b in range(logm):
            rev |= ((br >> b) & 1) << (logm - 1 - b)
        for c in range(-1, k):  # column -1: an untimed pass over column 0 sizes the workspace
            lifted = torch.zeros(4 * m, dtype=torch.int32, device="cuda")
            lifted[0::4] = d_lde[max(c, 0) * m:(max(c, 0) + 1) * m][rev]
            cur, depth = lifted, 0
            while ((n - 1) >> (2 * depth)) >= 8:
                ch = []
                for _ in range(12):
                    z, state = splitmix64(state)
                    ch.append(z % P)
                nl = cur.numel() // 16
                nxt = torch.empty(4 * nl, dtype=torch.int32, device="cuda")
                torch.cuda.synchronize()
                dt = device_seconds(ctx, lambda: check(L.z0p_gpu_fri_fold(
                    ctx.handle, C.c_void_p(cur.data_ptr()), cur.numel() // 4, m, depth,
                    (C.c_uint32 * 12)(*ch), C.c_void_p(nxt.data_ptr()))))
                if c >= 0:
                    dt_fold += dt
                    fold_bytes += 16 * (cur.numel() // 4) + 4 * (cur.numel() // 4) + 32 * (nl // 4)
                    compressions += nl // 4
                cur, depth = nxt, depth + 1
            del lifted, cur
        del d_lde, d_in, br, rev
        torch.cuda.empty_cache()
        b_lde = k * (4 * n + 4 * m)
        b_merkle = 4 * k * m + 32 * (2 * npad - 1)
        compressions += npad + 2 * (npad - 1)
        t_lde += dt_lde
        t_merkle += dt_merkle
        t_fold += dt_fold
        by_lde += b_lde
        by_merkle += b_merkle
        by_fold += fold_bytes
        rows.append({"log2_n": logn, "columns": k, "lde_ms": round(1e3 * dt_lde, 3),
                     "lde_gbs": round(b_lde / dt_lde / 1e9, 1), "merkle_ms": round(1e3 * dt_merkle, 3),
                     "fold_ms": round(1e3 * dt_fold, 3), "cap": bytes(out)[:32 * cnt.value].hex()[:16]})

    def stage(t, by):
        return {"ms": round(1e3 * t, 3), "alg_bytes": by, "gbs": round(by / t / 1e9, 1),
                "frac_hbm": round(by / t / 1e9 / peak, 4)}
    return {"workload": "64 columns, log2 n uniform in {16..22}, blowup 16; splitmix64 values",
            "timing": "device time: CUDA events on the context stream around each kernel stage, after a warm call",
            "peak_gbs": peak, "peak_source": peak_kind,
            "lde": stage(t_lde, by_lde), "merkle": dict(stage(t_merkle, by_merkle)),
            "fold": stage(t_fold, by_fold), "blake3_compressions": compressions, "groups": rows}


def run_rare(Z, ctx, reps=5):
    """The shapes that reach the kernels no production shape reaches: a FRI
    commitment whose final layer has fewer than four values (its last fold is
    fri_fold_plain, and the final layer's one-value leaves are leaf16,
    fri::commit_layer_values, src/fri.rs:1422-1428), and a range proof of an
    out-of-range value whose final layer is below the blowup (the row-by-row
    path, whose constant columns fill_columns writes). Median wall time of
    the public call and the proof size (bytes against the oracle: the GPU
    tests)."""
    vals = [(7 * i + 3) % P for i in range(1 << 10)]
    fz = Z.fri.Params.new(8, 8, 2).with_grinding_bits(0).with_cap_height(0)
    rz = Z.range.Params.new(1 << 10, 4, 16, 8, 4, 300)

    def fri():
        t = Z.Transcript(b"bench/rare-fri")
        st = Z.fri.commit(vals, fz, t, ctx)
        return st.commitment + Z.fri.open(st, t)[0]

    def rng():
        return Z.range.prove(rz, Z.Transcript(b"bench/rare-range"), ctx)
    rows = []
    for name, fn in [("fri 2^10 coefficients B8 Q8 final 2 (fri_fold_plain, leaf16)", fri),
                     ("range 2^10 rows 4 bits B16 final 4, value 300 (fill_columns)", rng)]:
        out = fn()
        times = []
        for _ in range(reps):
            t0 = time.perf_counter()
            fn()
            times.append(time.perf_counter() - t0)
        rows.append({"row": name, "ms": round(1e3 * statistics.median(times), 4), "bytes": len(out)})
    return {"rows": rows}


def run_table(Z, ctx, reps=5):
    """Table membership (table::prove): the reference's `table 4-entry` row
    (docs/benchmarks.md:125; workload of benches/speed_size.rs:301-305) and a
    2^20-row column against a 4-entry table at for_security(100). Host table in,
    proof bytes out, per call."""
    rows = []
    table = [10, 20, 30, 40]
    for n, label, ref_ms, ref_bytes in [(8, b"bench/table", 0.04, 4673),
                                        (1 << 20, b"bench/table-2p20", None, None)]:
        if n == 8:
            params = Z.table.Params.new(8, 8, 8, 4, 30)
        else:
            params = Z.table.Params.for_security(n, len(table), 30, 100)
        times, size = [], 0
        for _ in range(reps + 1):
            t = Z.Transcript(label)
            t0 = time.perf_counter()
            proof = Z.table.prove(params, table, t, ctx)
            times.append(time.perf_counter() - t0)
            size = len(proof)
        ms = 1e3 * sorted(times[1:])[len(times[1:]) // 2]
        rows.append({"n_rows": n, "lde_len": n * params.blowup, "ms": round(ms, 4), "bytes": size,
                     "reference_ms_16_cores": ref_ms, "reference_bytes": ref_bytes,
                     "bytes_match_reference": None if ref_bytes is None else size == ref_bytes})
    return {"workload": "constant column in a 4-entry table [10, 20, 30, 40], value 30", "rows": rows}


def run_fold_ivc(Z, ctx, reps=3):
    """Folded IVC (fold::Accumulator): the reference's `fold 4x8 fib` row
    (docs/benchmarks.md:127; workload of benches/speed_size.rs:432-449) and
    16 segments of 2^16 rows at for_security(100). Host columns in, proof
    bytes out; a step is add_segment for every segment plus finalize."""
    import numpy as np

    P = 2013265921

    def chain(seg, count):
        out, a, b = [], 1, 1
        for _ in range(count):
            ca, cb = np.empty(seg, np.uint32), np.empty(seg, np.uint32)
            for i in range(seg):
                ca[i], cb[i] = a, b
                a, b = b, (a + b) % P
            a, b = int(ca[-1]), int(cb[-1])  # the next segment restarts at the last row
            out.append((ca, cb))
        return out

    rows = []
    for seg, count, label, ref_ms, ref_bytes in [(8, 4, b"bench/fold", 0.19, 16845),
                                                 (1 << 16, 16, b"bench/fold-2p16x16", None, None)]:
        traces = chain(seg, count)
        out_b = int(traces[-1][1][-1])
        if seg == 8:
            params = Z.fold.Params.new(8, 8, 8, 4, 1, 1, out_b)
        else:
            params = Z.fold.Params.for_security(seg, 1, 1, out_b, 100)
        times, size = [], 0
        for _ in range(reps + 1):
            t = Z.Transcript(label)
            t0 = time.perf_counter()
            acc = Z.fold.Accumulator(params, ctx)
            for ca, cb in traces:
                acc.add_segment(ca, cb, t)
            proof = acc.finalize(t)
            times.append(time.perf_counter() - t0)
            acc.close()
            size = len(proof)
        ms = 1e3 * sorted(times[1:])[len(times[1:]) // 2]
        rows.append({"segments": count, "seg_steps": seg, "steps": count * seg, "ms": round(ms, 4),
                     "steps_per_s": round(count * seg / (ms / 1e3)), "bytes": size,
                     "reference_ms_16_cores": ref_ms, "reference_bytes": ref_bytes,
                     "bytes_match_reference": None if ref_bytes is None else size == ref_bytes})
    return {"workload": "Fibonacci segments chained from (1, 1), one batched FRI", "rows": rows}


def run_served(Z, ctx, rates=(100, 200, 400, None), requests=120, workers=16, budget=180 << 30):
    """Poisson arrivals of mixed Fibonacci (2^10..2^22) / range (2^12..2^18) requests.
    A rate of None submits the whole set at once (saturation)."""
    import random
    import threading

    from z0p_gb300.pool import Pool

    free, _ = __import__("torch").cuda.mem_get_info(ctx.device)
    budget = min(budget, int(free * 0.9))
    pool = Pool(ctx.device, workers=workers, hbm_budget=budget)
    out = []
    for ri, rate in enumerate(rates):
        seed = 0x5EED000000000004 + (977 * ri if rate else 0)  # saturation: the plain run's set
        specs = _mix_params(Z, seed, (3 * requests) // 4,
                            requests - (3 * requests) // 4, list(range(10, 23)), list(range(12, 19)))
        rng = random.Random(0x5EED0005 + ri)
        steps = sum(n for _, n, _ in specs)
        jobs = [pool.make_job(p, Z.Transcript(l)) for p, _, l in specs]
        tickets = [None] * len(jobs)

        def arrive():
            for i, j in enumerate(jobs):
                tickets[i] = pool.submit(j)
                if rate:
                    time.sleep(rng.expovariate(rate))

        util = UtilSampler(ctx.device).start() if rate is None else None
        t0 = pool.clock()
        th = threading.Thread(target=arrive)
        th.start()
        th.join()
        for t in tickets:
            pool.wait(t)
        t1 = max(j.end_s for j in jobs)
        if util:
            sat_util, sat_wall = util.stop(), t1 - t0
        lat = [j.end_s - j.submit_s for j in jobs]
        out.append({"rate_per_s": rate if rate else "saturate", "requests": len(jobs), "steps": steps,
                    "steps_per_s": steps / (t1 - t0),
                    "latency_ms": {"p50": 1e3 * _pct(lat, 0.5), "p99": 1e3 * _pct(lat, 0.99)}})
    pool.close()
    # the same request set proved one at a time on the plain path
    specs = _mix_params(Z, 0x5EED000000000004, (3 * requests) // 4, requests - (3 * requests) // 4,
                        list(range(10, 23)), list(range(12, 19)))
    util = UtilSampler(ctx.device).start()
    t0 = time.perf_counter()
    _, lat = _prove_plain(Z, ctx, specs)
    t_plain = time.perf_counter() - t0
    plain_util = util.stop()
    # Device work of the same set: each proof alone, its kernel stages summed.
    work = _device_work_ms(Z, ctx, specs)
    work_ms = sum(work)
    big = sorted(work, reverse=True)[:len(work) // 10]
    steps = sum(n for _, n, _ in specs)
    sat = [r for r in out if r["rate_per_s"] == "saturate"]
    return {"workload": "poisson arrivals; 75% fibonacci 2^10..2^22, 25% range-16 2^12..2^18",
            "workers": workers, "hbm_budget_gb": budget / 2**30, "by_rate": out,
            "plain_one_at_a_time": {"steps_per_s": steps / t_plain,
                                    "latency_ms": {"p50": 1e3 * _pct(lat, 0.5), "p99": 1e3 * _pct(lat, 0.99)}},
            "saturated_vs_plain": (sat[0]["steps_per_s"] / (steps / t_plain)) if sat else None,
            "device_busy": {
                "how": "work = sum over the request set of each proof's kernel-stage time alone (CUDA events); "
                       "busy = work / wall; util = nvidia-smi utilization.gpu every 20 ms",
                "work_ms": round(work_ms, 2),
                "work_ms_largest_tenth_of_requests": round(sum(big), 2),
                "plain": {"wall_ms": round(1e3 * t_plain, 2), "busy_pct": round(100 * work_ms / (1e3 * t_plain), 1),
                          "util": plain_util},
                "saturated": ({"wall_ms": round(1e3 * sat_wall, 2),
                               "busy_pct": round(100 * work_ms / (1e3 * sat_wall), 1), "util": sat_util}
                              if sat else None),
                "plain_wall_over_work": round(t_plain * 1e3 / work_ms, 2),
            }}


# -------------------------------------------------------------------- arms --
def run_reference(args):
    ws, rank, _ = dist_env()
    if rank != 0:
        return 0
    import oracle as O

    O.build()
    O.set_max_workers(0)
    cores = O.max_workers()
    a0, b0 = workload(0)
    _, b = O.build_trace(a0, b0, N_STEPS)
    params = O.air_for_security(N_STEPS, a0, b0, int(b[-1]), 100)
    for _ in range(args.warmup):
        O.air_prove(params, O.Transcript(LABEL))
    times = []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        proof = O.air_prove(params, O.Transcript(LABEL))
        times.append(time.perf_counter() - t0)
    assert len(proof) == 203553
    total = sum(times)
    value = args.steps * N_STEPS / total
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": "steps/s",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1000 * total / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": value / PUBLISHED_STEPS_PER_S, "dtype": "u32 (BabyBear mod p, BLAKE3 ARX)",
        "data": "synthetic (seeded)",
        "config": bench_config(),
        "cpu_baseline": {"value": value, "unit": "steps/s", "cores": cores, "kind": "port",
                         "sample": f"{args.steps} full 2^20-step proofs after {args.warmup} warm-up"},
        "e2e": {"value": value, "unit": "steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "latency_ms": {"p50": 1000 * statistics.median(times), "max": 1000 * max(times)},
    }
    print(json.dumps(line), flush=True)
    return 0


def cpu_baseline_sample():
    import oracle as O

    O.build()
    O.set_max_workers(0)
    a0, b0 = workload(0)
    _, b = O.build_trace(a0, b0, N_STEPS)
    params = O.air_for_security(N_STEPS, a0, b0, int(b[-1]), 100)
    t0 = time.perf_counter()
    proof = O.air_prove(params, O.Transcript(LABEL))
    dt = time.perf_counter() - t0
    return proof, {"value": N_STEPS / dt, "unit": "steps/s", "cores": O.max_workers(), "kind": "port",
                   "sample": "one full 2^20-step proof (same workload) on all host threads"}


def run_gpu(args):
    ws, rank, local = dist_env()
    import torch

    import z0p_gb300 as Z

    Z.build.build()
    torch.cuda.set_device(local)
    dist = None
    if ws > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    ctx = Z.Context(local)
    # Launch schedule: read from a file the autotuner wrote (--schedule), or
    # measured here by the autotuner, outside every timed region (sections
    # run alone keep the default unless given a file).
    if args.schedule:
        sched = Z.tune.load(args.schedule)
        Z.tune.set(sched, local)
        tune_info = {"source": args.schedule, "schedule": Z.tune.to_dict(sched)}
    elif not args.only:
        sched, report = Z.tune.autotune(ctx, max_log_n=22)
        tune_info = {"source": "autotune (live)", "schedule": Z.tune.to_dict(sched), "report": report}
    if args.only:
        # One section alone (for profilers and quick checks): no headline line.
        fn = {"published": run_published, "scale": run_scale, "sweep": run_sweep, "fri_pcs": run_fri_pcs,
              "fold_ivc": run_fold_ivc, "rare": run_rare,
              "table": run_table, "batched": run_batched, "served": run_served}[args.only]
        print(json.dumps({"section": args.only, "result": fn(Z, ctx)}), flush=True)
        return 0
    stream = torch.cuda.ExternalStream(ctx.stream, device=torch.device("cuda", local))
    a0, b0 = workload(rank)
    _, b_last = Z.air.trace_last(a0, b0, N_STEPS)
    params = Z.air.Params.for_security(N_STEPS, a0, b0, b_last, 100)
    size = params.proof_size()
    import ctypes as C

    out = (C.c_uint8 * size)()

    def prove_once():
        t = Z.Transcript(LABEL)
        return Z.air.prove_into(params, t, out, ctx)

    for _ in range(args.warmup):
        prove_once()
    proof0 = bytes(out)

    # --- timed region: device events on the context stream + host wall clock
    def barrier():
        if dist is not None:
            dist.barrier()
        torch.cuda.synchronize()

    sampler = ClockSampler(local)
    sampler.start()
    time.sleep(0.3)
    barrier()
    st0 = ctx.stats()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    lat = []
    ev0.record(stream)
    w0 = time.perf_counter()
    for _ in range(args.steps):
        t1 = time.perf_counter()
        prove_once()
        lat.append(time.perf_counter() - t1)
    ev1.record(stream)
    w1 = time.perf_counter()
    barrier()
    st1 = ctx.stats()
    clocks = sampler.stop()
    dev_ms = ev0.elapsed_time(ev1)
    wall_s = w1 - w0
    dev_ms, wall_s = aggregate_replicas(dist, dev_ms, wall_s, "cuda")

    # --- per-stage timing (CUDA events on the context stream) ---------------
    prof_steps = 0 if args.quick else 2
    prof = {}
    if prof_steps:
        ctx.set_profiling(True)
        for _ in range(prof_steps):
            prove_once()
        prof = ctx.profile()
        ctx.set_profiling(False)

    batched = served = fri_pcs = fold_ivc = table_row = published = scale = sweep = None
    if not args.quick and ws == 1:
        batched = run_batched(Z, ctx)
        served = run_served(Z, ctx)
        fri_pcs = run_fri_pcs(Z, ctx)
        fold_ivc = run_fold_ivc(Z, ctx)
        table_row = run_table(Z, ctx)
        published = run_published(Z, ctx)
        scale = run_scale(Z, ctx)
        sweep = run_sweep(Z, ctx)

    if rank != 0:
        if dist is not None:
            dist.destroy_process_group()
        return 0

    # --- parity of the measured proof (outside every timed region) ----------
    if args.quick:
        cpu_proof, cpu = None, None
        parity = None
    else:
        cpu_proof, cpu = cpu_baseline_sample()
        parity = proof0 == cpu_proof

    peak, peak_kind = measured_peaks()
    hash_ceiling = None if args.quick else ctx.blake3_ceiling()  # G compressions/s, live
    work = stage_work(N_STEPS, params)
    host = prof.pop("host", {})
    host_sites = {}
    for name, v in host.items():
        if "calls" in v:
            host_sites[name] = {"calls_per_proof": v["calls"] / prof_steps,
                                "blocked_ms": round(v["wait_ms"] / prof_steps, 4),
                                "host_before_ms": round(v["before_ms"] / prof_steps, 4)}
        else:
            host_sites[name] = {"host_ms": round(v["ms"] / prof_steps, 4)}
    stages = {}
    for name, v in prof.items():
        per = v["ms"] / prof_steps
        w = work.get(name, {})
        ent = {"ms_per_proof": round(per, 4),
               "launches_per_proof": v.get("kernels", v["calls"]) / prof_steps,
               "stage_calls_per_proof": v["calls"] / prof_steps}
        if "bytes" in w:
            ent["alg_bytes"] = w["bytes"]
            ent["gbs"] = round(w["bytes"] / (per / 1e3) / 1e9, 1) if per > 0 else None
            ent["frac_hbm"] = round(ent["gbs"] / peak, 4) if ent["gbs"] else None
        if "compressions" in w:
            ent["blake3_compressions"] = w["compressions"]
            ent["gcompress_per_s"] = round(w["compressions"] / (per / 1e3) / 1e9, 3) if per > 0 else None
            ent["frac_hash_ceiling"] = (round(ent["gcompress_per_s"] / hash_ceiling, 4)
                                        if ent["gcompress_per_s"] and hash_ceiling else None)
        stages[name] = ent
    dominant = max(stages, key=lambda k: stages[k]["ms_per_proof"]) if stages else None
    roof = None
    if dominant:
        d = stages[dominant]
        per_launch_ms = d["ms_per_proof"] / max(d["launches_per_proof"], 1)
        alg = d.get("alg_bytes", 0) / max(d["launches_per_proof"], 1)
        achieved = alg / (per_launch_ms / 1e3) / 1e9 if per_launch_ms > 0 else 0.0
        # DRAM bytes per launch: the captured launch's ratio of DRAM to
        # algorithmic bytes, applied to this stage's average launch.
        cap = measured_traffic().get(dominant, {})
        traffic = (cap["dram_bytes"] / cap["alg_bytes"] * alg) if cap.get("alg_bytes") else None
        # BLAKE3 stages are bound by integer issue (ALU pipe), not by HBM.
        bound = "int32" if "blake3_compressions" in d else "hbm"
        roof = {"kernel": dominant, "bound": bound, "achieved": round(achieved, 1), "peak": peak,
                "unit": "GB/s", "frac": round(achieved / peak, 4),
                # ncu dram__bytes_read.sum + dram__bytes_write.sum, per launch like achieved
                "traffic": round(traffic) if traffic else None,
                "traffic_source": cap.get("launch"),
                "alg_bytes_per_launch": round(alg),
                "peak_source": peak_kind}
        if "blake3_compressions" in d:
            # BLAKE3 stages are bound by integer issue, not HBM: their fraction
            # of the device's measured hash ceiling is the meaningful one.
            roof["int32"] = {"achieved_gcompress_per_s": d["gcompress_per_s"],
                             "ceiling_gcompress_per_s": round(hash_ceiling, 2),
                             "frac": d["frac_hash_ceiling"],
                             "ceiling_source": "z0p_gpu_blake3_ceiling (register-resident node hashes)",
                             "alu_pipe_pct": measured_alu().get(dominant)}
    steps_total = args.steps * ws * N_STEPS
    value = steps_total / (dev_ms / 1e3)
    e2e = steps_total / wall_s
    line = {
        "metric": METRIC, "value": value, "unit": "steps/s", "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": dev_ms / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": value / PUBLISHED_STEPS_PER_S,
        "dtype": "u32 (BabyBear mod p, BLAKE3 ARX)",
        "data": "synthetic (seeded splitmix64 initial pair)",
        "config": bench_config(),
        "parallelism": f"replicas x{ws}",
        "byte_identical_to_oracle": parity,
        "e2e": {"value": e2e, "unit": "steps/s",
                "h2d_bytes_per_step": (st1["h2d_bytes"] - st0["h2d_bytes"]) // args.steps,
                "d2h_bytes_per_step": (st1["d2h_bytes"] - st0["d2h_bytes"]) // args.steps},
        "gpu_launches": st1["launches"] - st0["launches"],
        "latency_ms": {"p50": 1000 * statistics.median(lat),
                       "p99": 1000 * sorted(lat)[min(len(lat) - 1, int(0.99 * len(lat)))]},
        "host_syncs_per_step": (st1["syncs"] - st0["syncs"]) / args.steps,
        "host_ms_per_step": {
            "prove_wall": (st1["prove_ns"] - st0["prove_ns"]) / 1e6 / args.steps,
            "blocked_in_sync": (st1["sync_wait_ns"] - st0["sync_wait_ns"]) / 1e6 / args.steps,
            "by_sync_site": host_sites},
        "clocks": clocks,
        "roofline": roof,
        "cpu_baseline": cpu,
        # secondary sections, the bulky ones first ...
        "kernel_sweep": sweep,
        "published_rows": published,
        "scale_rows": scale,
        "fold_ivc": fold_ivc,
        "table": table_row,
        "fri_pcs": fri_pcs,
        "launch_schedule": tune_info,
        "served": served,
        "batched": batched,
        "stages": stages,
    }
    # ... and a compact summary last, so that a reader keeping only the end
    # of the line still sees the batched / served ratios and the stage times.
    line["summary"] = summary(line)
    print(json.dumps(line), flush=True)
    if dist is not None:
        dist.destroy_process_group()
    return 0


def summary(line):
    """The evidence a short tail of the JSON line must carry."""
    r2 = lambda x: None if x is None else round(x, 2)  # noqa: E731
    out = {"value_msteps_per_s": r2(line["value"] / 1e6), "e2e_msteps_per_s": r2(line["e2e"]["value"] / 1e6),
           "ms_per_step": round(line["ms_per_step"], 4)}
    b = line.get("batched")
    if b:
        out["batched"] = {"speedup_vs_plain": r2(b["speedup_vs_plain"]),
                          "msteps_per_s": r2(b["batched_steps_per_s"] / 1e6),
                          "plain_msteps_per_s": r2(b["plain_steps_per_s"] / 1e6),
                          "byte_identical": b["byte_identical_to_plain"],
                          "p50_p99_ms": [r2(b["batched_latency_ms"]["p50"]), r2(b["batched_latency_ms"]["p99"])]}
    sv = line.get("served")
    if sv:
        out["served"] = {"saturated_vs_plain": r2(sv["saturated_vs_plain"]),
                         "by_rate": {str(r["rate_per_s"]): [r2(r["steps_per_s"] / 1e6), r2(r["latency_ms"]["p50"]),
                                                            r2(r["latency_ms"]["p99"])] for r in sv["by_rate"]},
                         "by_rate_fields": "M steps/s, p50 ms, p99 ms"}
        if sv.get("device_busy"):
            d = sv["device_busy"]
            out["served"]["busy_pct_plain_sat"] = [d["plain"]["busy_pct"],
                                                   d["saturated"]["busy_pct"] if d["saturated"] else None]
            out["served"]["plain_wall_over_work"] = d["plain_wall_over_work"]
    st = line.get("stages")
    if st:
        out["stages_ms_frac"] = {k: [v["ms_per_proof"], v.get("frac_hbm"), v.get("frac_hash_ceiling")]
                                 for k, v in st.items() if v["ms_per_proof"] >= 0.005}
    ks = line.get("kernel_sweep")
    if ks:
        out["kernel_sweep_frac_hbm"] = {k: ks[k]["frac_hbm"] for k in ("lde", "merkle", "fold")}
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--quick", action="store_true",
                    help="skip the CPU baseline, parity check and per-stage pass (for profilers)")
    ap.add_argument("--schedule", default=None,
                    help="launch schedule file written by z0p_gb300.tune.save (default: autotune live)")
    ap.add_argument("--only", default=None,
                    choices=["published", "scale", "sweep", "fri_pcs", "fold_ivc", "table", "batched",
                             "served", "rare"],
                    help="run one secondary section alone and print its JSON (no headline line)")
    args = ap.parse_args()
    if args.impl == "reference":
        return run_reference(args)
    return run_gpu(args)


if __name__ == "__main__":
    sys.exit(main())
