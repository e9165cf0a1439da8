"""Build recipe for the oracle (test infrastructure only).

Compiles gbde_oracle.cpp with g++ into oracle/liboracle_gbde.so.  Only the
tests, the smoke check and the benchmark's CPU-baseline leg load it.
-ffp-contract=off keeps the normal transform's rounding identical to the
device stream (only explicit fma()).  No -march flags: the same source
builds on x86-64 and aarch64.
"""
import os
import shutil
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "gbde_oracle.cpp")
LIB = os.path.join(HERE, "liboracle_gbde.so")
DEPS = [SRC, os.path.join(HERE, "..", "include", "gbde.h"),
        os.path.join(HERE, "..", "differentialequations.jl_gb300", "csrc", "tableaus.h"),
        os.path.join(HERE, "..", "differentialequations.jl_gb300", "csrc", "dense_coeffs.h"),
        os.path.join(HERE, "..", "differentialequations.jl_gb300", "csrc", "controller.h"),
        os.path.join(HERE, "..", "differentialequations.jl_gb300", "csrc", "philox.h"),
        os.path.join(HERE, "..", "differentialequations.jl_gb300", "csrc", "common.cuh"),
        __file__]


def build(force=False):
    if not force and os.path.exists(LIB) and all(
            os.path.getmtime(d) <= os.path.getmtime(LIB) for d in DEPS):
        return LIB
    cxx = shutil.which("g++") or "g++"
    tmp = LIB + ".tmp"
    cmd = [cxx, "-std=c++17", "-O2", "-ffp-contract=off", "-fPIC", "-shared", "-pthread",
           SRC, "-o", tmp]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + r.stdout + r.stderr)
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force=True))
