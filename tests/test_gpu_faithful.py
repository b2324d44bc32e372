"""The faithful FP64 reciprocal and square root of the fused step and the
adjoint (csrc/euler_device.cuh: rcp_faithful, sqrt_faithful) against CUDA's
correctly rounded __drcp_rn / __dsqrt_rn on 4M arguments spanning 2^+-100:
each result within one ulp of the correctly rounded one; the load kernel's
sound speed sqrt(x/d) from one reciprocal square root
(sqrt_quotient_faithful) within two ulps of __dsqrt_rn(__ddiv_rn(x, d)) on 4M
argument pairs; and the PTX
approximations they refine (rcp.approx.ftz.f64, rsqrt.approx.ftz.f64) within
the 2^-19.5 relative error the third-order refinement is sized for."""
import json
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CSRC = os.path.join(ROOT, "benchmark-euler-kernels_gb300", "csrc")


@pytest.mark.gpu
def test_faithful_reciprocal_and_sqrt(tmp_path):
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    exe = tmp_path / "faithful_check"
    subprocess.run([nvcc, "-O3", "-std=c++17", "-gencode", "arch=compute_103a,code=sm_103a", "-I", CSRC,
                    os.path.join(ROOT, "tests", "faithful_check.cu"), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True, timeout=120).stdout
    r = json.loads(out.strip().splitlines()[-1])
    assert r["rcp_max_ulp"] <= 1 and r["sqrt_max_ulp"] <= 1, r
    assert r["quot_max_ulp"] <= 2, r
    assert r["rcp_approx_rel"] <= 2.0 ** -19.5 and r["rsqrt_approx_rel"] <= 2.0 ** -19.5, r
