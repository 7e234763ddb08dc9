"""Builds the CUDA library in-tree: stonefish_gb300/lib/libstonefish_hydro.so.

Device code is compiled for sm_103a only, with ``-fmad=false`` (no FMA
contraction: each face's FP32 arithmetic stays in the reference's operation
order) and IEEE division and square root.  Translation units compile in
parallel and link into one shared library with the CUDA runtime linked
statically.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
LIB_DIR = os.path.join(HERE, "lib")
OBJ_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(LIB_DIR, "libstonefish_hydro.so")

SOURCES = ["hydro_kernels.cu", "hydro_api.cu", "hydro_nn.cu", "hydro_rollout.cu", "hydro_mlp_tc.cu", "hydro_cable.cu", "hydro_fft_ocean.cu",
           "hydro_ingest.cu", "hydro_approx.cu"]
HEADERS = ["hydro_device.cuh", "hydro_internal.h", "hydro_pair.cuh"]

NVCC_FLAGS = [
    "-O3", "-std=c++17", "-lineinfo",
    "-gencode", "arch=compute_103a,code=sm_103a",
    "-fmad=false", "-prec-div=true", "-prec-sqrt=true", "-ftz=false",
    "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off",
    "-Xptxas", "-warn-spills",
]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _stale(target: str, deps: list[str]) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build(force: bool = False, verbose: bool = False, extra_flags: list[str] | None = None) -> str:
    os.makedirs(LIB_DIR, exist_ok=True)
    os.makedirs(OBJ_DIR, exist_ok=True)
    include = os.path.join(os.path.dirname(HERE), "include", "stonefish_hydro.h")
    headers = [os.path.join(CSRC, h) for h in HEADERS] + [include]
    flags = NVCC_FLAGS + (extra_flags or [])
    procs, objs = [], []
    for src in SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(OBJ_DIR, src.replace(".cu", ".o"))
        objs.append(o)
        if force or _stale(o, [s] + headers + [__file__]):
            cmd = [nvcc(), *flags, "-c", s, "-o", o]
            if verbose:
                print(" ".join(cmd), file=sys.stderr)
            procs.append((cmd, subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)))
    for cmd, p in procs:
        out, _ = p.communicate()
        if p.returncode != 0:
            raise RuntimeError("nvcc failed:\n" + " ".join(cmd) + "\n" + out.decode(errors="replace"))
        if verbose and out:
            print(out.decode(errors="replace"), file=sys.stderr)
    if force or procs or _stale(LIB, objs):
        cmd = [nvcc(), "-shared", "-gencode", "arch=compute_103a,code=sm_103a", "-o", LIB, *objs]
        r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)
        if r.returncode != 0:
            raise RuntimeError("link failed:\n" + r.stdout.decode(errors="replace"))
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
