"""Build recipe for oracle/_ref/libref.so (test infrastructure only).

Compiles the reference's own SL-path sources where they lie (the tbslas
source tree: src/semilag/traj.inc, src/semilag/semilag.inc,
src/tree/tree_functor.h, src/tree/tree_utils.h, src/tree/tree_semilag.h,
src/utils/cheb.h, src/utils/common.h) through oracle/ref_pin.cpp, with
oracle/ref_stubs/ standing in for the dependencies the reference does not
vendor (PVFMM and MPI; both restated there for one process).  The reference's
own build system is not used.

Flags: g++ -O3 -fopenmp with multiply-add contraction on an FMA target
(-ffp-contract=fast; on x86-64 -mfma with -mtune=skylake, a tuning that
contracts accumulation chains -- g++'s generic x86 tuning leaves chains such
as vec_eval's w += px * c unfused), the rounding an optimising build of the
reference gets on a current CPU.  The reference's sources exist only
on the development machine: build() returns None when they are absent, and
tests that need the library skip; the committed fixtures
(tests/golden/ref_*.npz, written by tests/golden/make_ref_golden.py from this
library) pin the oracle everywhere else.
"""
import os
import platform
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "_ref")
LIB = os.path.join(OUT, "libref.so")
SRC = os.path.join(HERE, "ref_pin.cpp")
STUBS = os.path.join(HERE, "ref_stubs")
REFERENCE_SRC = os.environ.get("TBSLAS_REFERENCE_SRC", "/root/reference/src")


def available():
    return os.path.isfile(os.path.join(REFERENCE_SRC, "tree", "tree_semilag.h"))


def build(force=False, verbose=False):
    if not available():
        return None
    os.makedirs(OUT, exist_ok=True)
    deps = [SRC] + [os.path.join(STUBS, f) for f in os.listdir(STUBS)]
    if (not force and os.path.exists(LIB)
            and all(os.path.getmtime(LIB) >= os.path.getmtime(d) for d in deps)):
        return LIB
    cmd = ["g++", "-O3", "-std=c++14", "-fopenmp", "-ffp-contract=fast", "-fpermissive",
           "-fPIC", "-shared", "-I", STUBS, "-I", REFERENCE_SRC, SRC, "-o", LIB + ".tmp"]
    if platform.machine() in ("x86_64", "AMD64"):
        cmd[1:1] = ["-mfma", "-mtune=skylake"]
    if verbose:
        print(" ".join(cmd), file=sys.stderr)
    subprocess.check_call(cmd)
    os.replace(LIB + ".tmp", LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
