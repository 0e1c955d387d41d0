"""Build recipe for the oracle's C++ restatement (test infrastructure only).

Compiles oracle/oracle.cpp into oracle/_build/liboracle.so with g++ and
OpenMP.  The reference's own SL-path code is built separately into
oracle/_ref by oracle/build_ref.py (its drivers need PVFMM, MPI, BLAS/LAPACK
and FFTW, which are absent; the SL-path headers compile against the
stand-ins of oracle/ref_stubs/).
"""
import os
import platform
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "liboracle.so")
SRC = os.path.join(HERE, "oracle.cpp")


def build(force=False, verbose=False):
    os.makedirs(BUILD, exist_ok=True)
    if (not force and os.path.exists(LIB)
            and os.path.getmtime(LIB) >= os.path.getmtime(SRC)):
        return LIB
    cmd = ["g++", "-O3", "-std=c++17", "-fopenmp", "-ffp-contract=off", "-fPIC",
           "-shared", SRC, "-o", LIB + ".tmp"]
    if platform.machine() in ("x86_64", "AMD64"):
        cmd.insert(1, "-mfma")  # hardware FMA for std::fma (results are identical without)
    if verbose:
        print(" ".join(cmd), file=sys.stderr)
    subprocess.check_call(cmd)
    os.replace(LIB + ".tmp", LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
