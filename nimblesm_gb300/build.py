"""Builds the engine's shared library for sm_103a with nvcc, in the source tree.

nimblesm_gb300/csrc/*.cu -> nimblesm_gb300/_lib/libnimble_gb300.so.  The node,
setup and no-allocation time-step kernels are compiled with --fmad=false (their sums and products
round as the reference's host code does); the element kernels keep FMA
contraction.  Translation units compile in parallel; only changed ones are
rebuilt.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT_DIR = os.path.join(HERE, "_lib")
LIB = os.path.join(OUT_DIR, "libnimble_gb300.so")
INCLUDE = os.path.join(os.path.dirname(HERE), "include")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-ffp-contract=off", "-I" + INCLUDE]
NO_FMAD = {"node_kernels.cu", "setup_kernels.cu", "noalloc_dt.cu", "host_loop.cu"}


def _sources():
    return sorted(f for f in os.listdir(CSRC) if f.endswith(".cu"))


def _headers_mtime():
    hs = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    hs += [os.path.join(INCLUDE, f) for f in os.listdir(INCLUDE) if f.endswith(".h")]
    return max((os.path.getmtime(h) for h in hs), default=0.0)


def _compile(src, nvcc, verbose):
    obj = os.path.join(OUT_DIR, "obj", src.replace(".cu", ".o"))
    srcp = os.path.join(CSRC, src)
    if os.path.exists(obj) and os.path.getmtime(obj) >= max(os.path.getmtime(srcp), _headers_mtime()):
        return obj, ""
    flags = ARCH + COMMON + (["--fmad=false"] if src in NO_FMAD else [])
    if verbose:
        flags = flags + ["-Xptxas", "-v"]
    cmd = [nvcc] + flags + ["-c", srcp, "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src}:\n{r.stderr}")
    return obj, r.stderr


def build(verbose: bool = False, nvcc: str | None = None) -> str:
    nvcc = nvcc or os.environ.get("NVCC", "nvcc")
    os.makedirs(os.path.join(OUT_DIR, "obj"), exist_ok=True)
    with cf.ThreadPoolExecutor(max_workers=8) as ex:
        results = list(ex.map(lambda s: _compile(s, nvcc, verbose), _sources()))
    objs = [o for o, _ in results]
    if verbose:
        for _, log in results:
            if log:
                print(log)
    if not os.path.exists(LIB) or os.path.getmtime(LIB) < max(os.path.getmtime(o) for o in objs):
        tmp = LIB + ".tmp"
        cmd = [nvcc] + ARCH + ["-shared", "-o", tmp] + objs
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stderr}")
        os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    import sys
    print(build(verbose="-v" in sys.argv))
