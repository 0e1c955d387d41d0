"""Builds libtbslas_gb300.so in-tree (sm_103a only).

Every translation unit under csrc/ is compiled in parallel with nvcc
(-gencode arch=compute_103a,code=sm_103a), then linked into
tbslas_gb300/libtbslas_gb300.so.  Objects live in tbslas_gb300/_build/.
"""
import concurrent.futures as cf
import glob
import os
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
INCLUDE = os.path.join(ROOT, "include")
BUILD = os.path.join(PKG, "_build")
LIB = os.path.join(PKG, "libtbslas_gb300.so")

NVCC = os.environ.get("NVCC", "/usr/local/cuda/bin/nvcc"
                      if os.path.exists("/usr/local/cuda/bin/nvcc") else "nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-std=c++17", "-lineinfo", "-I" + INCLUDE, "-I" + CSRC,
          "-Xcompiler", "-fPIC,-fopenmp,-ffp-contract=off", "-diag-suppress", "550"]


def _sources():
    return sorted(glob.glob(os.path.join(CSRC, "*.cu")) + glob.glob(os.path.join(CSRC, "*.cpp")))


def _headers():
    return (glob.glob(os.path.join(CSRC, "*.h")) + glob.glob(os.path.join(CSRC, "*.cuh"))
            + glob.glob(os.path.join(INCLUDE, "*.h")))


def _obj(src):
    return os.path.join(BUILD, os.path.basename(src) + ".o")


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def _compile(src, verbose):
    cmd = [NVCC] + ARCH + COMMON + ["-c", src, "-o", _obj(src)]
    if verbose:
        print(" ".join(cmd), file=sys.stderr)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("nvcc failed for %s:\n%s%s" % (src, r.stdout, r.stderr))
    return src


def build(force=False, verbose=False, jobs=None):
    os.makedirs(BUILD, exist_ok=True)
    srcs = _sources()
    hdrs = _headers()
    todo = [s for s in srcs if force or _stale(_obj(s), [s] + hdrs)]
    if todo:
        jobs = jobs or max(1, min(len(todo), os.cpu_count() or 4))
        with cf.ThreadPoolExecutor(jobs) as ex:
            for f in [ex.submit(_compile, s, verbose) for s in todo]:
                f.result()
    objs = [_obj(s) for s in srcs]
    if force or todo or _stale(LIB, objs):
        cmd = [NVCC] + ARCH + ["-shared", "-o", LIB + ".tmp"] + objs + ["-lgomp"]
        if verbose:
            print(" ".join(cmd), file=sys.stderr)
        subprocess.check_call(cmd)
        os.replace(LIB + ".tmp", LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
