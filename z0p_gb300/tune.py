"""Launch schedules and their autotuner (no counterpart in the reference).

A schedule picks, per device, the four-step NTT split and pass variant
(shared-memory passes in register groups of 16 or 32, or register passes
with TMA-loaded tiles, one tile per CTA or streamed through a resident
grid) for each transform size, the Merkle level where one
top kernel takes over, and the proof-of-work grid. Every schedule gives byte-identical proofs.

    sched, report = tune.autotune(ctx)        # measure and install
    tune.save("gb300.schedule.json", sched)   # later: tune.set(tune.load(...))
"""
from __future__ import annotations

import ctypes as C
import json

from ._lib import Schedule, TuneReport, check, lib


def default() -> Schedule:
    s = Schedule()
    check(lib().z0p_schedule_default(C.byref(s)))
    return s


def get(device: int = 0) -> Schedule:
    s = Schedule()
    check(lib().z0p_gpu_schedule_get(device, C.byref(s)))
    return s


def set(schedule: Schedule, device: int = 0) -> None:  # noqa: A001 - module-level verb
    check(lib().z0p_gpu_schedule_set(device, C.byref(schedule)))


def to_dict(s: Schedule) -> dict:
    return {"ntt_log_n1": {str(l): int(s.ntt_log_n1[l]) for l in range(32) if s.ntt_log_n1[l]},
            "ntt_radix32": sorted(l for l in range(32) if s.ntt_radix32[l] == 1),
            "ntt_regpass": sorted(l for l in range(32) if s.ntt_radix32[l] == 2),
            "ntt_regstream": sorted(l for l in range(32) if s.ntt_radix32[l] == 3),
            "merkle_top_log": int(s.merkle_top_log), "grind_ctas_per_sm": int(s.grind_ctas_per_sm)}


def from_dict(d: dict) -> Schedule:
    s = default()
    for l, v in d.get("ntt_log_n1", {}).items():
        s.ntt_log_n1[int(l)] = int(v)
    for l in d.get("ntt_radix32", []):
        s.ntt_radix32[int(l)] = 1
    for l in d.get("ntt_regpass", []):  # register passes (pass variant 2)
        s.ntt_radix32[int(l)] = 2
    for l in d.get("ntt_regstream", []):  # streamed register passes (variant 3)
        s.ntt_radix32[int(l)] = 3
    s.merkle_top_log = int(d.get("merkle_top_log", s.merkle_top_log))
    s.grind_ctas_per_sm = int(d.get("grind_ctas_per_sm", s.grind_ctas_per_sm))
    return s


def save(path: str, s: Schedule) -> None:
    with open(path, "w") as f:
        json.dump(to_dict(s), f, indent=1, sort_keys=True)


def load(path: str) -> Schedule:
    with open(path) as f:
        return from_dict(json.load(f))


def shipped(name: str = "gb300") -> Schedule:
    """A schedule the autotuner wrote on that hardware, shipped with the
    package (schedules/<name>.json)."""
    import os

    return load(os.path.join(os.path.dirname(os.path.abspath(__file__)), "schedules", name + ".json"))


def autotune(ctx, max_log_n: int = 22):
    """Times every field's candidates on ctx's device, installs the winners
    (a candidate must beat the default by 3%) and returns (schedule, report)
    with the measured device times in µs."""
    s, r = Schedule(), TuneReport()
    check(lib().z0p_gpu_autotune(ctx.handle, max_log_n, C.byref(s), C.byref(r)))
    report = {
        "ntt_us": {str(l): {"default": round(r.ntt_default_us[l], 2), "chosen": round(r.ntt_best_us[l], 2)}
                   for l in range(32) if r.ntt_default_us[l] > 0},
        "merkle_2p21_us": {"default": round(r.merkle_default_us, 2), "chosen": round(r.merkle_best_us, 2)},
        "grind_8x20bit_us": {"default": round(r.grind_default_us, 2), "chosen": round(r.grind_best_us, 2)},
        "wall_ms": round(r.wall_ms, 1),
    }
    return s, report
