"""GPU check of the drop-in HLLC functor (include/euler_operators/hllc.hpp)
compiled by nvcc into a CUDA kernel: every flux bit equals the oracle's HLLC
on the same faces (random, supersonic, at rest with ustar == 0, signed
zeros, identical states, strong jumps; gamma 1.4 and spread), f64 and f32."""
import os
import shutil
import subprocess

import numpy as np
import pytest

from conftest import ROOT
from dropin_faces import face_states, oracle_fluxes, read_fluxes, write_faces

pytestmark = pytest.mark.gpu

INC = [os.path.join(ROOT, "include"), os.path.join(ROOT, "include", "euler_operators"),
       os.path.join(ROOT, "include", "euler_operators_kokkos")]


@pytest.fixture(scope="module")
def probe(tmp_path_factory, cuda):
    import importlib

    B = importlib.import_module("euler_gb300.build")

    exe = tmp_path_factory.mktemp("hllc") / "probe"
    cmd = [B.nvcc_path(), "-std=c++20", "-O2", *B.ARCH, *[f"-I{d}" for d in INC],
           os.path.join(ROOT, "tests", "dropin_hllc_probe.cu"), "-o", str(exe)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-4000:]
    return exe


@pytest.mark.parametrize("dtype", ["f64", "f32"])
def test_dropin_hllc_bit_identical_on_device(probe, oracle_lib, tmp_path, dtype):
    npdt = np.float64 if dtype == "f64" else np.float32
    dirs, gamma, qL, qR = face_states(seed=11, dtype=npdt)
    write_faces(tmp_path / "in.bin", dirs, gamma, qL, qR)
    r = subprocess.run([str(probe), dtype, str(tmp_path / "in.bin"), str(tmp_path / "out.bin")],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    got = read_fluxes(tmp_path / "out.bin", len(dirs), npdt)
    want = oracle_fluxes(oracle_lib, dirs, gamma, qL, qR)
    assert np.array_equal(got.view(np.uint8), want.view(np.uint8))
