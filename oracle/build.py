"""Build recipe of the CPU oracle (test infrastructure only).

Compiles oracle/oracle_capi.cpp into oracle/_build/liborc.so with
``-ffp-contract=off`` so that only the fused multiply-adds written in the
source are fused (the GpuF32 policy relies on it).
"""
from __future__ import annotations

import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "_build", "liborc.so")


def build() -> str:
    os.makedirs(os.path.dirname(OUT), exist_ok=True)
    src = os.path.join(HERE, "oracle_capi.cpp")
    hdr = os.path.join(HERE, "rayna_oracle.hpp")
    if os.path.exists(OUT) and os.path.getmtime(OUT) > max(os.path.getmtime(src), os.path.getmtime(hdr)):
        return OUT
    tmp = OUT + ".tmp"
    cmd = ["g++", "-std=c++17", "-O2", "-ffp-contract=off", "-fPIC", "-shared", "-pthread", "-o", tmp, src]
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"oracle build failed:\n{r.stdout}")
    os.replace(tmp, OUT)
    return OUT


if __name__ == "__main__":
    print(build())
