"""Build recipe for the CPU oracle (test infrastructure): g++ on
oracle/pm_oracle.cpp -> oracle/liboracle.so.  Strict IEEE FP32: no FMA
contraction, no fast-math, so its results match the CUDA kernels bit for bit
where they are meant to."""
from __future__ import annotations

import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
LIB = os.path.join(HERE, "liboracle.so")


def _arch_flags():
    """fmaf() is exact everywhere; on x86-64 hosts with FMA, -mfma makes it an
    instruction instead of a libm call (results are identical)."""
    import platform
    if platform.machine() in ("x86_64", "AMD64"):
        try:
            if " fma " in open("/proc/cpuinfo").read():
                return ["-mfma"]
        except OSError:
            pass
    return []


def build(force: bool = False, verbose: bool = False) -> str:
    src = os.path.join(HERE, "pm_oracle.cpp")
    deps = [src, os.path.join(ROOT, "include", "cvtpm.h"),
            os.path.join(ROOT, "cvt_gb300", "csrc", "pm_math.h")]
    if not force and os.path.exists(LIB) and all(os.path.getmtime(LIB) >= os.path.getmtime(d) for d in deps):
        return LIB
    cmd = ["g++", "-std=c++17", "-O2", "-fPIC", "-shared", "-fopenmp",
           "-ffp-contract=off", "-fno-fast-math", "-fno-finite-math-only", *_arch_flags(),
           "-I", os.path.join(ROOT, "include"), "-I", os.path.join(ROOT, "cvt_gb300", "csrc"),
           src, "-o", LIB + ".tmp"]
    if verbose:
        print(" ".join(cmd), file=sys.stderr)
    subprocess.run(cmd, check=True)
    os.replace(LIB + ".tmp", LIB)
    return LIB


if __name__ == "__main__":
    print(build(force=True, verbose=True))
