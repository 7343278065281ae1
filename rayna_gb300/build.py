"""Build recipe of the native library ``rayna_gb300/_lib/librayna_gpu.so``.

Every translation unit is compiled by nvcc for sm_103a in parallel, then
linked into one shared library against the shared CUDA runtime. Device code is
compiled with ``-fmad=false`` and host code with ``-ffp-contract=off``: fused
multiply-adds appear only where the source writes them, which keeps the
closed-form intersection arithmetic reproducible on the CPU.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
OUT_DIR = os.path.join(HERE, "_lib")
BUILD_DIR = os.path.join(ROOT, "_build", "rayna_gpu")
LIB = os.path.join(OUT_DIR, "librayna_gpu.so")

SOURCES = ["renderer.cpp", "bvh_build.cpp", "megakernel.cu", "wavefront.cu", "adjoint.cu", "batch.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc_path() -> str:
    p = shutil.which("nvcc")
    if p:
        return p
    cand = "/usr/local/cuda/bin/nvcc"
    if os.path.exists(cand):
        return cand
    raise RuntimeError("nvcc not found")


def cuda_lib_dir(nvcc: str) -> str:
    return os.path.join(os.path.dirname(os.path.dirname(os.path.realpath(nvcc))), "lib64")


def common_flags(extra: list | None = None) -> list:
    return ARCH + ["-O3", "-lineinfo", "-std=c++17", "-fmad=false", "-I", os.path.join(ROOT, "include"),
                   "-Xcompiler", "-fPIC,-ffp-contract=off,-O2", "--expt-relaxed-constexpr"] + (extra or [])


def build(verbose: bool = False, ptxas_info: bool = False) -> str:
    """Compiles and links the library; returns its path."""
    nvcc = nvcc_path()
    os.makedirs(BUILD_DIR, exist_ok=True)
    os.makedirs(OUT_DIR, exist_ok=True)
    extra = ["-Xptxas", "-v"] if ptxas_info else []
    procs = []
    objs = []
    for src in SOURCES:
        obj = os.path.join(BUILD_DIR, os.path.splitext(src)[0] + ".o")
        objs.append(obj)
        cmd = [nvcc] + common_flags(extra) + ["-c", os.path.join(CSRC, src), "-o", obj]
        if verbose:
            print(" ".join(cmd), file=sys.stderr)
        procs.append((src, subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)))
    failed = []
    logs = {}
    for src, p in procs:
        out, _ = p.communicate()
        logs[src] = out
        if p.returncode != 0:
            failed.append(src)
    if verbose or ptxas_info:
        for src, out in logs.items():
            if out.strip():
                print(f"--- {src}\n{out}", file=sys.stderr)
    if failed:
        msg = "\n".join(f"--- {s}\n{logs[s]}" for s in failed)
        raise RuntimeError(f"nvcc failed for {failed}:\n{msg}")
    tmp = LIB + ".tmp"
    libdir = cuda_lib_dir(nvcc)
    cmd = [nvcc] + ARCH + ["-shared", "-cudart", "shared", "-o", tmp] + objs + [
        "-Xlinker", f"-rpath,{libdir}", "-L", libdir]
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}")
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv, ptxas_info="--ptxas" in sys.argv))
