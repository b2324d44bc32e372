"""CPU tests of the C++ drop-in layer (include/euler_operators/ with the
Kokkos names of include/euler_operators_kokkos/): the reference's own driver,
simulations/euler_simulation.cpp, compiles and links unmodified against it and
libeuler_gb300.so.  Compile-only here (no GPU); the reference checkout is read
where it exists and the test skips elsewhere."""
import os
import shutil
import subprocess

import pytest

from conftest import ROOT
from oracle import REFERENCE_DIR as REF

INC = [os.path.join(ROOT, "include"), os.path.join(ROOT, "include", "euler_operators"),
       os.path.join(ROOT, "include", "euler_operators_kokkos"), "/usr/local/cuda/include"]


def _need_ref():
    if not os.path.isfile(os.path.join(REF, "simulations", "euler_simulation.cpp")):
        pytest.skip("reference checkout not present")
    if shutil.which("g++") is None:
        pytest.skip("g++ not available")


def test_reference_driver_builds_against_dropin(euler, tmp_path):
    _need_ref()
    lib_dir = os.path.dirname(euler.LIB_PATH)
    exe = tmp_path / "euler_simulation"
    cmd = ["g++", "-std=c++20", "-O1", *[f"-I{d}" for d in INC], f"-I{REF}/simulations",
           f"{REF}/simulations/euler_simulation.cpp", f"{REF}/simulations/save_npy.cpp",
           f"-L{lib_dir}", "-leuler_gb300", f"-Wl,-rpath,{lib_dir}", "-L/usr/local/cuda/lib64", "-lcudart",
           "-o", str(exe)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-4000:]
    assert exe.exists()


@pytest.mark.parametrize("defines", [[], ["-DEULR_GODUNOV_BIT_EXACT"]], ids=["default", "bit_exact_godunov"])
def test_reference_style_calls_compile_against_dropin(euler, tmp_path, defines):
    """The reference's operator call sequence (simulations/euler_simulation.cpp:
    37-67, benchmarks/benchmark_*.cpp) written against the drop-in: every type
    and operator it names is provided, with godunov on the default or the
    bit-exact entry point."""
    _need_ref()
    src = tmp_path / "probe.cpp"
    src.write_text(
        "#include <cons_to_prim.hpp>\n#include <godunov.hpp>\n#include <init_implode.hpp>\n"
        "#include <prim_to_cons.hpp>\n#include <time_step.hpp>\nusing real_t = double; using index_t = int;\n"
        "void f() {\n"
        "  Kokkos::DefaultExecutionSpace const exec_space; int const n = 10;\n"
        "  PerfectGas<real_t> const eos(1.4); UniformMesh3d<real_t> const mesh(1., 1., 1.);\n"
        "  EulerPrimArrays const pa = create_prim_arrays_1d<real_t>(exec_space, n * n * n);\n"
        "  EulerPrimArrays const p = to_mdspan<Kokkos::mdspan<real_t, Kokkos::dextents<index_t, 3>, Kokkos::layout_left>>(pa, n, n, n);\n"
        "  EulerConsArrays const ca = create_cons_arrays_1d<real_t>(exec_space, n * n * n);\n"
        "  EulerConsArrays const c = to_mdspan<Kokkos::mdspan<real_t, Kokkos::dextents<index_t, 3>, Kokkos::layout_left>>(ca, n, n, n);\n"
        "  init_implode(exec_space, p, mesh); prim_to_cons(exec_space, as_const(p), c, eos);\n"
        "  real_t dt = time_step(exec_space, as_const(p), eos, mesh);\n"
        "  godunov(exec_space, as_const(p), c, eos, mesh, hllc(), dt);\n"
        "  cons_to_prim(exec_space, as_const(c), p, eos); exec_space.fence();\n"
        "  (void)size_bytes(p); (void)size(c); (void)load(p, 1, 1, 1);\n"
        "}\n")
    r = subprocess.run(["g++", "-std=c++20", "-fsyntax-only", *defines, *[f"-I{d}" for d in INC], str(src)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-4000:]
