"""In-tree build of libz0p_gpu.so for sm_103a (GB300).

Three translation units compiled in parallel — the CUDA kernels with nvcc,
the host driver and C ABI with g++ — and linked by nvcc into
``z0p_gb300/libz0p_gpu.so`` with the CUDA runtime linked statically.
"""
from __future__ import annotations

import os
import shutil
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
INCLUDE = os.path.join(os.path.dirname(HERE), "include")
BUILD_DIR = os.path.join(HERE, "_build")
LIB_PATH = os.path.join(HERE, "libz0p_gpu.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def _cuda_home() -> str:
    home = os.environ.get("CUDA_HOME") or os.environ.get("CUDA_PATH")
    if home and os.path.isdir(home):
        return home
    nvcc = shutil.which("nvcc")
    if nvcc:
        return os.path.dirname(os.path.dirname(os.path.realpath(nvcc)))
    return "/usr/local/cuda"


def sources():
    return sorted(
        os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cu", ".cpp", ".h", ".cuh"))
    ) + [os.path.join(INCLUDE, "z0p_gpu.h")]


def _stale() -> bool:
    if not os.path.exists(LIB_PATH):
        return True
    t = os.path.getmtime(LIB_PATH)
    return any(os.path.getmtime(s) > t for s in sources())


def build(force: bool = False, verbose: bool = False) -> str:
    if not force and not _stale():
        return LIB_PATH
    cuda = _cuda_home()
    nvcc = os.path.join(cuda, "bin", "nvcc")
    os.makedirs(BUILD_DIR, exist_ok=True)
    common = ["-O3", "-std=c++17", "-I" + INCLUDE, "-I" + CSRC]
    jobs = []
    obj_k = os.path.join(BUILD_DIR, "kernels.o")
    jobs.append([nvcc, *ARCH, "-lineinfo", *common, "-Xcompiler", "-fPIC", "-c",
                 os.path.join(CSRC, "kernels.cu"), "-o", obj_k])
    objs = [obj_k]
    for name in ("host.cpp", "prover.cpp", "pool.cpp"):
        obj = os.path.join(BUILD_DIR, name.replace(".cpp", ".o"))
        jobs.append(["g++", *common, "-fPIC", "-Wall", "-Wextra", "-Wno-unused-parameter",
                     "-I" + os.path.join(cuda, "include"), "-c", os.path.join(CSRC, name), "-o", obj])
        objs.append(obj)
    procs = [subprocess.Popen(j, stdout=subprocess.PIPE, stderr=subprocess.STDOUT) for j in jobs]
    errors = []
    for j, p in zip(jobs, procs):
        out, _ = p.communicate()
        if p.returncode != 0:
            errors.append(" ".join(j) + "\n" + out.decode(errors="replace"))
        elif verbose and out:
            print(out.decode(errors="replace"))
    if errors:
        raise RuntimeError("libz0p_gpu build failed:\n" + "\n".join(errors))
    tmp = LIB_PATH + f".tmp{os.getpid()}"
    link = [nvcc, *ARCH, "-shared", "-o", tmp, *objs, "-cudart", "static", "-lpthread"]
    r = subprocess.run(link, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)
    if r.returncode != 0:
        raise RuntimeError("libz0p_gpu link failed:\n" + r.stdout.decode(errors="replace"))
    os.replace(tmp, LIB_PATH)
    return LIB_PATH


if __name__ == "__main__":
    print(build(force=True, verbose=True))
