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


def _compile_host(src, exe, extra=()):
    if shutil.which("g++") is None:
        pytest.skip("g++ not available")
    cmd = ["g++", "-std=c++20", "-O2", "-ffp-contract=off", "-x", "c++", *extra, *[f"-I{d}" for d in INC],
           str(src), "-o", str(exe)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-4000:]


@pytest.mark.parametrize("dtype", ["f64", "f32"])
def test_dropin_hllc_bit_identical_on_host(oracle_lib, tmp_path, dtype):
    """hllc{}(dir_t<D>(), eos, qL, qR) of the drop-in header, compiled for
    the host, against the oracle's HLLC (and the reference's own functor
    where the reference build exists): every bit of every flux component,
    on random, supersonic, at-rest (ustar == 0), signed-zero, identical and
    strong-jump faces, gamma 1.4 and spread."""
    import numpy as np

    from dropin_faces import face_states, oracle_fluxes, read_fluxes, write_faces

    O = oracle_lib
    npdt = np.float64 if dtype == "f64" else np.float32
    exe = tmp_path / "probe"
    _compile_host(os.path.join(ROOT, "tests", "dropin_hllc_probe.cu"), exe)
    dirs, gamma, qL, qR = face_states(dtype=npdt)
    write_faces(tmp_path / "in.bin", dirs, gamma, qL, qR)
    r = subprocess.run([str(exe), dtype, str(tmp_path / "in.bin"), str(tmp_path / "out.bin")],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    got = read_fluxes(tmp_path / "out.bin", len(dirs), npdt)
    want = oracle_fluxes(O, dirs, gamma, qL, qR)
    assert np.isfinite(want).all()
    assert np.array_equal(got.view(np.uint64 if dtype == "f64" else np.uint32),
                          want.view(np.uint64 if dtype == "f64" else np.uint32))
    if O.have_ref():
        ref = oracle_fluxes(O, dirs, gamma, qL, qR, impl="ref")
        assert np.array_equal(ref.view(np.uint8), want.view(np.uint8))


def test_dropin_subspan(tmp_path):
    """subspan of a bundle (euler_arrays.hpp:106-117, 257-268) through the
    Kokkos shim's submdspan: index, full_extent and [first, last) slices
    select what numpy's slicing of the same Fortran-ordered arrays selects;
    slices that keep one contiguous block stay layout_left (and so compile
    into the operators' signatures), the others become layout_stride."""
    import numpy as np

    src = tmp_path / "subspan.cpp"
    src.write_text(r'''
#include <cons_to_prim.hpp>
#include <cstdio>
#include <utility>
#include <vector>
using K = Kokkos::mdspan<double, Kokkos::dextents<int, 3>, Kokkos::layout_left>;
template <class V> void dump(char const* name, V const& v) {
    std::printf("%s %d", name, (int)V::rank());
    for (std::size_t r = 0; r < V::rank(); ++r) std::printf(" %d", (int)v.extent(r));
    if constexpr (V::rank() == 3) {
        for (int k = 0; k < v.extent(2); ++k) for (int j = 0; j < v.extent(1); ++j)
            for (int i = 0; i < v.extent(0); ++i) std::printf(" %g", v(i, j, k));
    } else if constexpr (V::rank() == 2) {
        for (int j = 0; j < v.extent(1); ++j) for (int i = 0; i < v.extent(0); ++i) std::printf(" %g", v(i, j));
    } else if constexpr (V::rank() == 1) {
        for (int i = 0; i < v.extent(0); ++i) std::printf(" %g", v(i));
    } else {
        std::printf(" %g", v());
    }
    std::printf("\n");
}
int main() {
    int const n0 = 7, n1 = 5, n2 = 4, n = n0 * n1 * n2;
    std::vector<double> buf(10 * n);
    for (int f = 0; f < 10; ++f) for (int c = 0; c < n; ++c) buf[f * n + c] = 1000 * f + c;
    EulerPrimArrays<K> p {K(&buf[0], n0, n1, n2), K(&buf[n], n0, n1, n2), K(&buf[2 * n], n0, n1, n2),
                          K(&buf[3 * n], n0, n1, n2), K(&buf[4 * n], n0, n1, n2)};
    EulerConsArrays<K> c {K(&buf[5 * n], n0, n1, n2), K(&buf[6 * n], n0, n1, n2), K(&buf[7 * n], n0, n1, n2),
                          K(&buf[8 * n], n0, n1, n2), K(&buf[9 * n], n0, n1, n2)};
    auto const all = Kokkos::full_extent;
    auto a = subspan(p, all, all, std::pair<int, int>(1, 3));
    static_assert(std::is_same_v<decltype(a.d)::layout_type, Kokkos::layout_left>);
    dump("a_d", a.d); dump("a_ux2", a.ux2);
    auto b = subspan(c, std::pair<int, int>(2, 6), 3, all);
    static_assert(std::is_same_v<decltype(b.e)::layout_type, Kokkos::layout_stride>);
    dump("b_e", b.e); dump("b_mx1", b.mx1);
    auto d = subspan(c, all, std::pair<int, int>(1, 4), 2);
    static_assert(std::is_same_v<decltype(d.mx0)::layout_type, Kokkos::layout_left>);
    dump("d_mx0", d.mx0);
    auto e = subspan(p, 4, 1, std::tuple<int, int>(0, 4));
    static_assert(std::is_same_v<decltype(e.p)::layout_type, Kokkos::layout_stride>);
    dump("e_p", e.p);
    auto g = subspan(p, 6, 4, 3);
    dump("g_d", g.d);
    auto h = subspan(p, Kokkos::ALL, Kokkos::make_pair(1, 4), Kokkos::full_extent);
    static_assert(std::is_same_v<decltype(h.d)::layout_type, Kokkos::layout_stride>);
    dump("h_d", h.d);
    // a contiguous slab is still an operator argument
    auto slab_c = subspan(c, all, all, std::pair<int, int>(1, 3));
    auto slab_p = subspan(p, all, all, std::pair<int, int>(1, 3));
    if (false) {
        Kokkos::DefaultExecutionSpace exec;
        cons_to_prim(exec, as_const(slab_c), slab_p, PerfectGas<double>(1.4));
    }
    return 0;
}
''')
    exe = tmp_path / "subspan"
    _compile_host(src, exe)
    r = subprocess.run([str(exe)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    n0, n1, n2 = 7, 5, 4
    n = n0 * n1 * n2
    fields = [(1000 * f + np.arange(n, dtype=float)).reshape((n0, n1, n2), order="F") for f in range(10)]
    want = {"a_d": fields[0][:, :, 1:3], "a_ux2": fields[4][:, :, 1:3], "b_e": fields[6][2:6, 3, :],
            "b_mx1": fields[8][2:6, 3, :], "d_mx0": fields[7][:, 1:4, 2], "e_p": fields[1][4, 1, 0:4],
            "g_d": fields[0][6, 4, 3], "h_d": fields[0][:, 1:4, :]}
    lines = {ln.split()[0]: ln.split()[1:] for ln in r.stdout.strip().splitlines()}
    assert set(lines) == set(want)
    for name, arr in want.items():
        arr = np.asarray(arr)
        vals = lines[name]
        rank = int(vals[0])
        assert rank == arr.ndim, name
        assert [int(v) for v in vals[1:1 + rank]] == list(arr.shape), name
        assert np.array_equal(np.array([float(v) for v in vals[1 + rank:]]), arr.flatten(order="F")), name
