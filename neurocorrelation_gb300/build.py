"""Builds libneucor_gb300.so in-tree for sm_103a (nvcc, no CMake).

Each translation unit compiles in parallel, then nvcc links the shared library into
neurocorrelation_gb300/_lib/.  Device code is built with --fmad=false and host code
with -ffp-contract=off: every multiply and add rounds on its own, as the reference's
arithmetic does.
"""
from __future__ import annotations

import concurrent.futures as cf
import hashlib
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT_DIR = os.path.join(HERE, "_lib")
LIB = os.path.join(OUT_DIR, "libneucor_gb300.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def _nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the GB300 library cannot be built")


def _sources():
    srcs = sorted(f for f in os.listdir(CSRC) if f.endswith((".cu", ".cpp")))
    headers = sorted(f for f in os.listdir(CSRC) if f.endswith((".h", ".cuh")))
    return srcs, headers


def _fingerprint(srcs, headers) -> str:
    h = hashlib.sha256()
    for f in srcs + headers:
        with open(os.path.join(CSRC, f), "rb") as fh:
            h.update(f.encode() + b"\0" + fh.read())
    inc = os.path.join(os.path.dirname(HERE), "include", "neucor_gb300.h")
    with open(inc, "rb") as fh:
        h.update(fh.read())
    h.update(" ".join(ARCH).encode())
    return h.hexdigest()


def build(force: bool = False, verbose: bool = False) -> str:
    srcs, headers = _sources()
    os.makedirs(OUT_DIR, exist_ok=True)
    stamp = os.path.join(OUT_DIR, "build.stamp")
    fp = _fingerprint(srcs, headers)
    if not force and os.path.exists(LIB) and os.path.exists(stamp) and open(stamp).read() == fp:
        return LIB
    nvcc = _nvcc()
    cuda_inc = os.path.join(os.path.dirname(os.path.dirname(nvcc)), "include")
    objs = []
    cmds = []
    for f in srcs:
        src = os.path.join(CSRC, f)
        obj = os.path.join(OUT_DIR, f + ".o")
        objs.append(obj)
        if f.endswith(".cu"):
            cmd = [nvcc, *ARCH, "-O3", "-lineinfo", "--fmad=false", "-std=c++17", "-Xcompiler",
                   "-fPIC,-ffp-contract=off", "-c", src, "-o", obj]
        else:
            cmd = ["g++", "-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-I" + cuda_inc, "-c", src, "-o", obj]
        cmds.append(cmd)

    def run(cmd):
        r = subprocess.run(cmd, capture_output=True, text=True)
        return cmd, r

    with cf.ThreadPoolExecutor(max_workers=min(8, len(cmds))) as ex:
        for cmd, r in ex.map(run, cmds):
            if verbose or r.returncode != 0:
                sys.stderr.write(" ".join(cmd) + "\n" + r.stdout + r.stderr)
            if r.returncode != 0:
                raise RuntimeError(f"compile failed: {cmd[-3]}")
    tmp = LIB + ".tmp"
    link = [nvcc, *ARCH, "-shared", "-o", tmp, *objs, "-lpthread"]
    r = subprocess.run(link, capture_output=True, text=True)
    if r.returncode != 0:
        sys.stderr.write(r.stdout + r.stderr)
        raise RuntimeError("link failed")
    os.replace(tmp, LIB)
    with open(stamp, "w") as fh:
        fh.write(fp)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
