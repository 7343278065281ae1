"""Build recipe of the native library, in two arithmetic builds of one source.

``rayna_gb300/_lib/librayna_gpu.so`` is the performance build: device code
compiled with ``-fmad=true``, so the compiler may fuse a multiply and an add
into one FMA wherever it finds them (measured 1.07x on the SDF workload and
1.23x on the sphere workload's megakernel, where CUDA's math functions carry
most of the fusable arithmetic). It is what renders by default and what the
benchmark times; it is held to statistical parity with the faithful f64
oracle.

``rayna_gb300/_lib/librayna_gpu_exact.so`` is the arithmetic-contract build:
device code with ``-fmad=false`` and host code with ``-ffp-contract=off``, so
fused multiply-adds appear only where the source writes them. The CPU oracle's
f32 policy follows the same contract, which makes the closed-form
intersections bit-exact between the two; the bit-exact parity tests load it.

Every translation unit of both builds is compiled by nvcc for sm_103a in
parallel, then each build is linked into one shared library against the
shared CUDA runtime.
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
LIB_EXACT = os.path.join(OUT_DIR, "librayna_gpu_exact.so")

SOURCES = ["renderer.cpp", "bvh_build.cpp", "megakernel.cu", "wavefront.cu", "adjoint.cu", "batch.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# build name -> (library, device -fmad flag)
VARIANTS = {"fast": (LIB, "-fmad=true"), "exact": (LIB_EXACT, "-fmad=false")}


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


def common_flags(extra: list | None = None, fmad: str = "-fmad=false") -> list:
    return ARCH + ["-O3", "-lineinfo", "-std=c++17", fmad, "-I", os.path.join(ROOT, "include"),
                   "-Xcompiler", "-fPIC,-ffp-contract=off,-O2", "--expt-relaxed-constexpr"] + (extra or [])


def build(verbose: bool = False, ptxas_info: bool = False, variants=("fast", "exact")) -> str:
    """Compiles and links the libraries of `variants`, every translation unit
    in parallel; returns the path of the first."""
    nvcc = nvcc_path()
    os.makedirs(OUT_DIR, exist_ok=True)
    extra = ["-Xptxas", "-v"] if ptxas_info else []
    procs = []
    objs = {v: [] for v in variants}
    for v in variants:
        bdir = os.path.join(BUILD_DIR, v)
        os.makedirs(bdir, exist_ok=True)
        for src in SOURCES:
            obj = os.path.join(bdir, os.path.splitext(src)[0] + ".o")
            objs[v].append(obj)
            cmd = [nvcc] + common_flags(extra, VARIANTS[v][1]) + ["-c", os.path.join(CSRC, src), "-o", obj]
            if verbose:
                print(" ".join(cmd), file=sys.stderr)
            procs.append((f"{v}/{src}", subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT,
                                                         text=True)))
    failed = []
    logs = {}
    for name, p in procs:
        out, _ = p.communicate()
        logs[name] = out
        if p.returncode != 0:
            failed.append(name)
    if verbose or ptxas_info:
        for name, out in logs.items():
            if out.strip():
                print(f"--- {name}\n{out}", file=sys.stderr)
    if failed:
        msg = "\n".join(f"--- {s}\n{logs[s]}" for s in failed)
        raise RuntimeError(f"nvcc failed for {failed}:\n{msg}")
    libdir = cuda_lib_dir(nvcc)
    for v in variants:
        lib = VARIANTS[v][0]
        tmp = lib + ".tmp"
        cmd = [nvcc] + ARCH + ["-shared", "-cudart", "shared", "-o", tmp] + objs[v] + [
            "-Xlinker", f"-rpath,{libdir}", "-L", libdir]
        r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link of {v} failed:\n{r.stdout}")
        os.replace(tmp, lib)
    return VARIANTS[variants[0]][0]


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv, ptxas_info="--ptxas" in sys.argv))
