"""GPU tests of the host applications built over the C ABI and the drop-in
headers: the implosion driver (NPY pressure dumps against the oracle) and the
benchmark set (Google Benchmark JSON in the shape plot.py reads)."""
import json
import os
import subprocess

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def oracle_pressure(O, nx, steps, cfl, dtype=np.float64):
    n = nx + 2
    dx = (1.0 / nx,) * 3
    prim = O.init_implode(n, n, n, dx, dtype=dtype)
    cons = O.prim_to_cons(prim, 1.4)
    out = {}
    done = 0
    for s in steps:
        O.simulate(prim, cons, 1.4, dx, cfl, s - done)
        done = s
        out[s] = prim[1].copy()
    return out


@pytest.mark.parametrize("mode,precision", [("fused", "f64"), ("operators", "f64"), ("exact", "f64"), ("exact", "f32")])
def test_driver_npy_output(cuda, euler, oracle_lib, tmp_path, mode, precision):
    from euler_gb300.build import app_path

    exe = app_path("euler_simulation")
    nx, nt = 24, 20
    r = subprocess.run([exe, "--nx", str(nx), "--nt", str(nt), "--output-freq", "10", "--mode", mode,
                        "--precision", precision, "--out", str(tmp_path)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    lines = r.stdout.strip().splitlines()
    assert lines[0].startswith("Saving ") and lines[0].endswith("done")
    assert float(lines[-1]) > 0  # Mcell/s
    ref = oracle_pressure(oracle_lib, nx, (10, 20), 0.49, np.float32 if precision == "f32" else np.float64)
    for s in (10, 20):
        path = tmp_path / f"test_{s:010d}.npy"
        hdr = open(path, "rb").read(128)
        assert b"'fortran_order': True, 'shape': (26, 26, 26, ), }" in hdr
        p = np.load(path)
        assert p.shape == (26, 26, 26) and p.flags.f_contiguous
        # layout_left file order is (i, j, k); the oracle bundle is [k, j, i]
        got = p.transpose(2, 1, 0)
        if mode == "exact":
            # the reference loop with the bit-identical godunov: every dump
            # equals the oracle's loop bit for bit (real_t = double or float)
            assert got.dtype == ref[s].dtype and np.array_equal(got, ref[s]), (mode, precision, s)
            continue
        err = np.abs(got - ref[s]).max() / np.abs(ref[s]).max()
        assert err <= 1e-11, (mode, s, err)


def test_benchmarks_json_for_plot(cuda, euler, tmp_path):
    from euler_gb300.build import app_path

    out = tmp_path / "bm.json"
    r = subprocess.run([app_path("euler_benchmarks"), f"--benchmark_out={out}", "--benchmark_filter=/16",
                        "--benchmark_min_time=0.01"], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    data = json.load(open(out))
    names = [b["name"] for b in data["benchmarks"]]
    for fam in ("Godunov/16", "TimeStep/16", "ConsToPrim/16", "PrimToCons/16", "EulerSimulation/16",
                "EulerStepFused/16", "EulerStepF32C/16"):
        assert fam in names
    for b in data["benchmarks"]:
        # the fields plot.py:34-50 reads (the substring filter also picks /160)
        assert int(b["name"].split("/")[-1]) in (16, 160)
        assert b["cpu_time"] > 0 and b["cells_per_second"] > 0
        assert b["time_unit"] == "ns"
    g = next(b for b in data["benchmarks"] if b["name"] == "Godunov/16")
    # reference counters: cells = (n+2)^3, bytes = prim + 2 cons bundles
    assert abs(g["bytes_per_second"] / g["cells_per_second"] - 120.0) < 1e-6
