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
