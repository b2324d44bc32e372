"""CPU check of the integer halving the FP64 kernels use in place of a
multiply by 0.5 (csrc/halve.cuh): equal to IEEE x * 0.5 bit for bit on
seeded bit patterns, subnormal results and ties included."""
import ctypes
import os
import subprocess

from conftest import PKG_DIR, ROOT


def test_halve_bits_matches_ieee(tmp_path):
    out = tmp_path / "libhalve.so"
    subprocess.run(["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-shared", "-fPIC", "-I",
                    os.path.join(PKG_DIR, "csrc"), os.path.join(ROOT, "tests", "halve_check.cpp"), "-o", str(out)],
                   check=True)
    lib = ctypes.CDLL(str(out))
    lib.halve_mismatches.restype = ctypes.c_longlong
    lib.halve_mismatches.argtypes = [ctypes.c_longlong, ctypes.c_ulonglong]
    assert lib.halve_mismatches(3_000_000, 2024) == 0
