"""The exact integer-pipe forms of FP64 operations the kernels use
(tbslas_gb300/csrc/fp64_bits.cuh: coordinate tests, Morton quantisation,
power-of-two scalings, products by T_0, the tricubic stencil's split and
Lagrange offsets) give the FP64 operation's bits for special values and
seeded random inputs.  Compiled and run on the host; no GPU needed."""
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)


def test_fp64_bits_match_fp64_operations(tmp_path):
    exe = str(tmp_path / "fp64_bits_check")
    subprocess.check_call(["g++", "-O2", "-std=c++17", "-ffp-contract=off",
                           "-Wno-unknown-pragmas",
                           "-I" + os.path.join(ROOT, "tbslas_gb300", "csrc"),
                           os.path.join(HERE, "cpp", "fp64_bits_check.cpp"), "-o", exe])
    r = subprocess.run([exe], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    assert " mismatches 0" in r.stdout, r.stdout
