"""The host transcript used inside a prove call, as one long-lived object.

Covers host.cpp's Transcript/Hasher with their cached chunk chaining values
(the C-ABI transcript functions rebuild the cache on every call, so they do
not exercise a cache carried across many operations). A small C++ driver is
compiled against host.cpp and the oracle and compares outputs and the full
streaming state after every operation.
"""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.mark.skipif(shutil.which("g++") is None or shutil.which("gcc") is None,
                    reason="needs gcc/g++")
def test_long_lived_transcript_matches_oracle(tmp_path):
    csrc = os.path.join(ROOT, "z0p_gb300", "csrc")
    orc = os.path.join(ROOT, "oracle")
    obj = str(tmp_path / "oracle.o")
    exe = str(tmp_path / "transcript_check")
    subprocess.run(["gcc", "-O2", "-std=c11", "-pthread", "-c", os.path.join(orc, "z0p_oracle.c"),
                    "-o", obj], check=True)
    subprocess.run(["g++", "-O2", "-std=c++17", "-pthread", "-I" + csrc, "-I" + orc,
                    "-I" + os.path.join(ROOT, "include"),
                    os.path.join(ROOT, "tests", "transcript_check.cpp"),
                    os.path.join(csrc, "host.cpp"), obj, "-o", exe], check=True)
    r = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    assert r.stdout.startswith("ok "), r.stdout


def _fresh_thread(fn):
    """fn() on a new thread, whose per-thread hasher memo is empty."""
    import threading
    out = {}
    th = threading.Thread(target=lambda: out.setdefault("v", fn()))
    th.start()
    th.join()
    return out["v"]


def test_cache_memo_is_keyed_by_content(z0p):
    """The C-ABI calls rebuild the hasher from the caller's state; the per-
    thread memo of the last cache may only be reused where the tail repeats
    the cached blocks. A state with the same chunk count and tail length but
    a different byte inside a cached block squeezes as from scratch."""
    T = z0p.Transcript
    base = T(b"memo")
    base.absorb(b"x", bytes(range(256)) * 6)  # chunk 1 open, chunk 0 pushed
    for pos in (3, 700, 1100):  # inside the first chunk's and the tail's blocks
        warm = base.clone()
        warm.challenge_bytes(b"warm")  # leaves this thread's memo on base's tail
        changed = base.clone()
        tl = changed.state.tail_len
        at = pos % tl
        changed.state.tail[at] ^= 0x5A
        got = changed.clone().challenge_bytes(b"q")
        assert got == _fresh_thread(lambda: changed.clone().challenge_bytes(b"q"))
        assert got != base.clone().challenge_bytes(b"q")
        # and the unchanged state reuses the memo to the same result
        again = base.clone().challenge_bytes(b"q")
        assert again == _fresh_thread(lambda: base.clone().challenge_bytes(b"q"))


def test_interleaved_transcripts_match_oracle(z0p, oracle):
    """Several transcripts advanced in turn on one thread (each call meets the
    memo of another transcript) agree with the oracle after every step."""
    import random
    rng = random.Random(11)
    pairs = [(z0p.Transcript(b"il%d" % i), oracle.Transcript(b"il%d" % i)) for i in range(3)]
    for step in range(600):
        g, o = pairs[rng.randrange(3)]
        op = rng.randrange(3)
        if op == 0:
            data = bytes(rng.randrange(256) for _ in range(rng.randrange(0, 900)))
            g.absorb(b"d", data)
            o.absorb(b"d", data)
        elif op == 1:
            assert g.challenge_bytes(b"c") == o.challenge_bytes(b"c"), step
        else:
            assert g.challenge_index(b"i", 1 << 20) == o.challenge_index(b"i", 1 << 20), step
        assert g.export() == o.export(), step
