"""Builds FAME's own command-line program twice from the reference sources
staged by oracle/build_ref.sh (oracle/_ref/src_100_550: READLEN 100, MAXPDIST
550, CORENUM of this machine):

* oracle/_ref/gpu_host/FAME_stock: the sources as they are;
* oracle/_ref/gpu_host/FAME_gpu: the same sources with the bodies of
  ReadQueue::matchReads and ReadQueue::matchPairedReads replaced by calls
  into libfame_gpu.so, and the tally copy added at the start of
  printMethylationLevels and printSCMethylationLevels
  (tests/reference_host/gpu_bodies.inc, the code INTEGRATION.md shows),
  linked against fame_gb300/libfame_gpu.so.

Test infrastructure (tests/test_gpu_reference_host.py): nothing here is part
of the library.  Only files under oracle/_ref/gpu_host are written.
"""
from __future__ import annotations

import os
import re
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
SRC = os.path.join(ROOT, "oracle", "_ref", "src_100_550")
OUT = os.path.join(ROOT, "oracle", "_ref", "gpu_host")
SOURCES = ["main.cpp", "ReadQueue.cpp", "RefGenome.cpp", "RefReader_istr.cpp", "Read.cpp", "CONST.cpp",
           "DnaBitStr.cpp", "gzstream/gzstream.C"]


def sections():
    """The named parts of gpu_bodies.inc (split at lines '//@@ NAME')."""
    out, name = {}, None
    for line in open(os.path.join(HERE, "gpu_bodies.inc")):
        m = re.match(r"//@@ (\w+)", line)
        if m:
            name = m.group(1)
            out[name] = []
        elif name:
            out[name].append(line)
    return {k: "".join(v) for k, v in out.items()}


def body_span(src: str, signature: str):
    """(start, end) of the brace-enclosed body of the function whose definition
    starts with `signature`, skipping comments, strings and character literals."""
    at = src.index(signature)
    i = src.index("{", at)
    depth, j, n = 0, i, len(src)
    while j < n:
        c = src[j]
        if src.startswith("//", j):
            j = src.index("\n", j)
            continue
        if src.startswith("/*", j):
            j = src.index("*/", j) + 2
            continue
        if c in "\"'":
            k = j + 1
            while src[k] != c:
                k += 2 if src[k] == "\\" else 1
            j = k + 1
            continue
        if c == "{":
            depth += 1
        elif c == "}":
            depth -= 1
            if depth == 0:
                return i, j + 1
        j += 1
    raise ValueError("unbalanced body: " + signature)


def patch_readqueue(text: str, parts: dict) -> str:
    for sig, name in (("bool ReadQueue::matchPairedReads(", "MATCH_PAIRED_READS"),
                      ("bool ReadQueue::matchReads(", "MATCH_READS")):
        a, b = body_span(text, sig)
        text = text[:a] + parts[name] + text[b:]
    for sig, name in (("void ReadQueue::printMethylationLevels(", "BEFORE_REPORT"),
                      ("void ReadQueue::printSCMethylationLevels(", "BEFORE_SC_REPORT")):
        a, b = body_span(text, sig)
        text = text[:a + 1] + "\n" + parts[name] + text[a + 1:]
    # the helper after the file's includes
    inc = [m.end() for m in re.finditer(r"^#include[^\n]*\n", text, flags=re.M)]
    at = inc[-1] if inc else 0
    return text[:at] + parts["HELPER"] + text[at:]


def compile_fame(src_dir: str, exe: str, gpu: bool):
    cmd = ["g++", "-std=c++14", "-O2", "-fopenmp", "-w", "-I", src_dir,
           "-I", os.path.join(src_dir, "hopscotch-map", "include", "tsl")]
    if gpu:
        cmd += ["-I", os.path.join(ROOT, "include")]
    cmd += [os.path.join(src_dir, s) for s in SOURCES] + ["-o", exe, "-lz"]
    if gpu:
        lib = os.path.join(ROOT, "fame_gb300")
        cmd += ["-L", lib, "-lfame_gpu", "-Wl,-rpath," + lib]
    subprocess.run(cmd, check=True)


def build() -> dict:
    if not os.path.exists(os.path.join(SRC, "main.cpp")):
        raise FileNotFoundError("staged reference sources with main.cpp not found (oracle/build_ref.sh)")
    os.makedirs(OUT, exist_ok=True)
    exes = {}
    for kind in ("stock", "gpu"):
        d = os.path.join(OUT, "src_" + kind)
        shutil.rmtree(d, ignore_errors=True)
        shutil.copytree(SRC, d)
        if kind == "gpu":
            p = os.path.join(d, "ReadQueue.cpp")
            with open(p) as f:
                t = f.read()
            with open(p, "w") as f:
                f.write(patch_readqueue(t, sections()))
        exes[kind] = os.path.join(OUT, "FAME_" + kind)
    import concurrent.futures as cf
    with cf.ThreadPoolExecutor(2) as ex:
        list(ex.map(lambda k: compile_fame(os.path.join(OUT, "src_" + k), exes[k], k == "gpu"), exes))
    return exes


if __name__ == "__main__":
    print(build(), file=sys.stderr)
