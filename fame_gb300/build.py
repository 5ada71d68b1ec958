"""Build of the native library (CUDA kernels for sm_103a + host C++), in tree.

``python -m fame_gb300.build`` or ``fame_gb300.build.build()`` compiles
``fame_gb300/csrc`` into ``fame_gb300/libfame_gpu.so`` with nvcc, one
translation unit per process, and skips the work when the library is newer
than every source file.
"""
from __future__ import annotations

import concurrent.futures as cf
import glob
import os
import shutil
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
INCLUDE = os.path.join(os.path.dirname(HERE), "include")
LIB = os.path.join(HERE, "libfame_gpu.so")
OBJDIR = os.path.join(HERE, "_build")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-O3", "-I", INCLUDE]
CXX_FLAGS = ["-O3", "-std=c++17", "-fPIC", "-pthread", "-I", INCLUDE]


def _nvcc() -> str:
    for c in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build fame_gb300")


def _sources():
    return sorted(glob.glob(os.path.join(CSRC, "*.cu")) + glob.glob(os.path.join(CSRC, "*.cpp")))


def _deps():
    return _sources() + sorted(glob.glob(os.path.join(CSRC, "*.h")) + glob.glob(os.path.join(CSRC, "*.cuh"))) + \
        [os.path.join(INCLUDE, "fame_gpu.h")]


def up_to_date() -> bool:
    if not os.path.exists(LIB):
        return False
    t = os.path.getmtime(LIB)
    return all(os.path.getmtime(p) <= t for p in _deps())


def build(force: bool = False, verbose: bool = False) -> str:
    if not force and up_to_date():
        return LIB
    nvcc = _nvcc()
    os.makedirs(OBJDIR, exist_ok=True)
    jobs = []
    for src in _sources():
        obj = os.path.join(OBJDIR, os.path.basename(src) + ".o")
        if src.endswith(".cu"):
            cmd = [nvcc] + NVCC_FLAGS + ["-c", src, "-o", obj]
        else:
            cmd = [os.environ.get("CXX", "g++")] + CXX_FLAGS + ["-c", src, "-o", obj]
        jobs.append((cmd, obj))

    def run(cmd):
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("compile failed: %s\n%s%s" % (" ".join(cmd), r.stdout, r.stderr))
        if verbose:
            print(r.stdout + r.stderr)

    with cf.ThreadPoolExecutor(max_workers=len(jobs)) as ex:
        list(ex.map(run, [c for c, _ in jobs]))
    tmp = LIB + ".tmp"
    run([nvcc] + ARCH + ["-shared", "-o", tmp] + [o for _, o in jobs] + ["-lpthread", "-lz"])
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force=True, verbose=True))
