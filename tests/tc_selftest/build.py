"""Build recipe of the test-only tcgen05 self-test library (libtcselftest.so, sm_103a).

Compiles tc_gemm_selftest.cu against the product's tcgen05 helpers (matx_gb300/csrc/tc.cuh)
into tests/tc_selftest/libtcselftest.so (git-ignored).  Test infrastructure only.
"""
from __future__ import annotations

import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
SRC = os.path.join(HERE, "tc_gemm_selftest.cu")
LIB = os.path.join(HERE, "libtcselftest.so")


def build() -> str:
    sys.path.insert(0, ROOT)
    from matx_gb300.build import nvcc, ARCH
    deps = [SRC, os.path.join(ROOT, "matx_gb300", "csrc", "tc.cuh")]
    if os.path.exists(LIB) and os.path.getmtime(LIB) >= max(os.path.getmtime(d) for d in deps):
        return LIB
    cmd = [nvcc(), *ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler",
           "-fvisibility=hidden", "-I", os.path.join(ROOT, "matx_gb300", "csrc"), "-shared", SRC, "-o",
           LIB + ".tmp", "-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {SRC}:\n{r.stdout}\n{r.stderr}")
    os.replace(LIB + ".tmp", LIB)
    return LIB


if __name__ == "__main__":
    print(build())
