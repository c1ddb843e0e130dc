"""Build recipe of the in-tree CUDA library ``_build/libwg_gpu.so`` (sm_103a only).

Compiled with nvcc directly (no cmake): every translation unit in parallel,
then one shared library.  Device code lets the compiler contract a multiply
and a dependent add into one FMA (nvcc's default): the FP64 day step is bound by
the FP64 pipe, and an FMA is one instruction where the pair is two; the results
stay within the FP64 path's parity bound of the reference's separately rounded
arithmetic.  Host code is compiled with ``-ffp-contract=off`` so that x86 and
Arm hosts produce the same constants.
"""
from __future__ import annotations

import os
import shutil
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_build")
LIB = os.path.join(OUT, "libwg_gpu.so")
SOURCES = ["wg_kernels.cu", "wg_capi.cpp", "wg_peak.cu", "wg_noalloc.cu", "wg_tune.cpp", "wg_mlp.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def flags(extra=()):
    return [*ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-ffp-contract=off,-O2",
            "-I", os.path.join(HERE, "..", "include"), *extra]


def build(verbose: bool = False, ptxas_info: bool = False) -> str:
    os.makedirs(OUT, exist_ok=True)
    cc = nvcc()
    procs = []
    objs = []
    for src in SOURCES:
        obj = os.path.join(OUT, os.path.splitext(src)[0] + ".o")
        objs.append(obj)
        extra = ["-Xptxas", "-v"] if ptxas_info and src.endswith(".cu") else []
        x = ["-x", "cu"] if src.endswith(".cpp") else []
        cmd = [cc, *flags(extra), *x, "-c", os.path.join(CSRC, src), "-o", obj]
        procs.append((cmd, subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)))
    for cmd, p in procs:
        out, _ = p.communicate()
        if verbose or ptxas_info:
            print(out)
        if p.returncode:
            raise RuntimeError(f"nvcc failed ({' '.join(cmd)}):\n{out}")
    link = [cc, *ARCH, "-shared", "-o", LIB, *objs, "-lcudart"]
    r = subprocess.run(link, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode:
        raise RuntimeError(f"link failed:\n{r.stdout}")
    build_synth()
    return LIB


SYNTH_LIB = os.path.join(OUT, "libwg_synth.so")


def build_synth() -> str:
    """Host-only generator helpers (no CUDA): priority-flood + D8 for large grids."""
    os.makedirs(OUT, exist_ok=True)
    cmd = [shutil.which("g++") or "g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-ffp-contract=off",
           os.path.join(CSRC, "wg_synth.cpp"), "-o", SYNTH_LIB]
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode:
        raise RuntimeError(f"g++ failed:\n{r.stdout}")
    return SYNTH_LIB


if __name__ == "__main__":
    import sys
    print(build(verbose=True, ptxas_info="-v" in sys.argv))
