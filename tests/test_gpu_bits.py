"""The integer-pipe stand-ins for FP64 instructions (less_ieee for the FP64
compare, half_exact for the multiply by 0.5, product_positive for the sign of
a product, div_small for the face index's integer division) give the
instructions' answers on the GPU for operands of every class: normal,
subnormal, zero, infinite, NaN (tests/bits_check.cu)."""
import json
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CSRC = os.path.join(ROOT, "benchmark-euler-kernels_gb300", "csrc")


@pytest.mark.gpu
def test_integer_pipe_stand_ins(tmp_path):
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    exe = tmp_path / "bits_check"
    subprocess.run([nvcc, "-O3", "-std=c++17", "-gencode", "arch=compute_103a,code=sm_103a", "-I", CSRC,
                    "-I", os.path.join(ROOT, "include"), os.path.join(ROOT, "tests", "bits_check.cu"), "-o", str(exe)],
                   check=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True, timeout=120).stdout
    r = json.loads(out.strip().splitlines()[-1])
    assert r["n"] > 4_000_000
    assert r["less_ieee"] == 0 and r["half_exact"] == 0 and r["product_positive"] == 0 and r["div_small"] == 0, r
