"""Builds libcrt.so in-tree with nvcc for sm_103a.

Each CUDA translation unit compiles in parallel to an object under
realtimeraytracing_gb300/_build/, then links into
realtimeraytracing_gb300/libcrt.so.  The build and trace units use
-fmad=false so every float operation rounds once, as the reference's CPU code
does; the learned-predictor unit keeps fused multiply-add.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
OBJ = os.path.join(PKG, "_build")
LIB = os.path.join(PKG, "libcrt.so")
INCLUDE = os.path.join(ROOT, "include")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-I", INCLUDE, "-I", CSRC]
# (source, extra flags)
UNITS = [
    ("crt_build.cu", ["-fmad=false"]),
    ("crt_trace.cu", ["-fmad=false"]),
    ("crt_frame.cu", ["-fmad=false"]),
    ("crt_refit.cu", ["-fmad=false"]),
    ("crt_optimize.cu", ["-fmad=false"]),
    ("crt_import.cu", ["-fmad=false"]),
    ("crt_mesh.cu", []),
    ("crt_api.cu", ["-fmad=false"]),
    ("crt_noalloc.cu", ["-fmad=false"]),
    ("crt_predictor.cu", []),
]


def nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _stale(target: str, deps: list[str]) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build(force: bool = False, verbose: bool = False) -> str:
    os.makedirs(OBJ, exist_ok=True)
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    headers.append(os.path.join(INCLUDE, "crt.h"))
    procs, objs = [], []
    for src, extra in UNITS:
        s = os.path.join(CSRC, src)
        o = os.path.join(OBJ, src.replace(".cu", ".o"))
        objs.append(o)
        if force or _stale(o, [s, __file__] + headers):
            cmd = [nvcc(), *ARCH, *COMMON, *extra, "-c", s, "-o", o]
            if verbose:
                print(" ".join(cmd), file=sys.stderr)
            procs.append((cmd, subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)))
    failed = []
    for cmd, p in procs:
        out, _ = p.communicate()
        if p.returncode != 0:
            failed.append((cmd, out.decode(errors="replace")))
    if failed:
        msg = "\n\n".join(" ".join(c) + "\n" + o for c, o in failed)
        raise RuntimeError("nvcc failed:\n" + msg)
    if force or procs or _stale(LIB, objs):
        cmd = [nvcc(), *ARCH, "-shared", "-cudart", "static", "-o", LIB, *objs]
        subprocess.run(cmd, check=True)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
