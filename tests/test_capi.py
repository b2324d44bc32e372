"""CPU tests of the C ABI boundary: the library loads, exports every symbol
include/euler_gb300.h declares, and rejects invalid arguments with the
documented status codes before touching the GPU."""
import ctypes
import os
import re
import subprocess

import pytest

from conftest import ROOT

HEADER = os.path.join(ROOT, "include", "euler_gb300.h")


def declared_functions():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(eulr_\w+)\s*\(", text)))


def test_header_declares_entry_points():
    names = declared_functions()
    for n in ("eulr_prim_to_cons_f64", "eulr_cons_to_prim_f64", "eulr_time_step_f64", "eulr_godunov_f64",
              "eulr_init_implode_f64", "eulr_sim_create", "eulr_sim_advance"):
        assert n in names


def test_library_exports_every_declared_symbol(euler):
    lib = ctypes.CDLL(euler.LIB_PATH)
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, missing
    nm = subprocess.run(["nm", "-D", "--defined-only", euler.LIB_PATH], capture_output=True, text=True).stdout
    exported = set(re.findall(r"\bT (eulr_\w+)", nm))
    assert set(declared_functions()) <= exported


def test_python_bindings_cover_header(euler):
    assert set(declared_functions()) == set(euler.EXPORTED)


def test_status_strings(euler):
    lib = euler.load()
    assert lib.eulr_status_string(0) == b"success"
    assert lib.eulr_status_string(-1) == b"invalid argument"
    assert lib.eulr_version() >= 100


def _b(*ptrs):
    from euler_gb300 import Bundle5

    return Bundle5(*ptrs)


def test_invalid_arguments_rejected_without_gpu(euler):
    lib = euler.load()
    ok = _b(8, 16, 24, 32, 40)
    null = _b(None, None, None, None, None)
    # bad extents
    assert lib.eulr_prim_to_cons_f64(ok, ok, 0, 4, 4, 1.4, None) == -1
    assert lib.eulr_prim_to_cons_f64(ok, ok, -3, 4, 4, 1.4, None) == -1
    # more cells than the reference's int index range
    assert lib.eulr_cons_to_prim_f64(ok, ok, 2000, 2000, 2000, 1.4, None) == -6
    # null fields
    assert lib.eulr_prim_to_cons_f64(null, ok, 4, 4, 4, 1.4, None) == -1
    assert b"NULL" in lib.eulr_last_error()
    # misaligned field
    assert lib.eulr_prim_to_cons_f64(_b(8, 16, 25, 32, 40), _b(800, 1600, 2400, 3200, 4000), 4, 4, 4, 1.4,
                                     None) == -3
    # gamma <= 1, non-finite dx, bad dt
    far = _b(10_000, 20_000, 30_000, 40_000, 50_000)
    assert lib.eulr_prim_to_cons_f64(ok, far, 1, 1, 1, 1.0, None) == -2
    assert lib.eulr_time_step_f64(ok, 1, 1, 1, 1.4, 0.1, float("nan"), 0.1, 4096, None) == -2
    assert lib.eulr_time_step_f64(ok, 1, 1, 1, 1.4, 0.1, 0.1, 0.1, None, None) == -1
    assert lib.eulr_godunov_f64(ok, far, 1, 1, 1, 1.4, 0.1, 0.1, 0.1, float("inf"), None) == -2
    # overlapping in/out bundles
    assert lib.eulr_godunov_f64(ok, ok, 4, 4, 4, 1.4, 0.1, 0.1, 0.1, 1e-3, None) == -1
    assert b"overlap" in lib.eulr_last_error()
    # simulation handle checks
    h = ctypes.c_void_p()
    assert lib.eulr_sim_create(0, 8, 8, 8, 0.5, 0.1, 0.1, 0.1, 0.4, None, ctypes.byref(h)) == -2
    assert lib.eulr_sim_create(0, 8, 8, 8, 1.4, 0.1, 0.1, 0.1, -1.0, None, ctypes.byref(h)) == -2
    assert lib.eulr_sim_create(7, 8, 8, 8, 1.4, 0.1, 0.1, 0.1, 0.4, None, ctypes.byref(h)) in (-1, -9)
    assert lib.eulr_sim_advance(None, 1) == -1
    assert lib.eulr_sim_destroy(None) == 0


def test_missing_library_fails_loudly(euler, tmp_path):
    with pytest.raises(FileNotFoundError):
        euler.load(str(tmp_path / "libeuler_gb300.so"))


@pytest.mark.parametrize("args", [["--mode", "bogus"], ["--nx", "0"], ["--nt", "-1"], ["--unknown"]])
def test_driver_rejects_bad_arguments_without_gpu(euler, args):
    """The implosion driver validates its options before any CUDA call: a bad
    mode, size or flag prints the usage line (which names every mode) and
    exits 2."""
    from euler_gb300.build import app_path

    r = subprocess.run([app_path("euler_simulation"), *args], capture_output=True, text=True, timeout=60)
    assert r.returncode == 2, (args, r.stdout, r.stderr)
    assert "--mode fused|operators|exact" in r.stdout + r.stderr
