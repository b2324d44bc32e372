// euler_simulation: the implosion driver of the reference
// (simulations/euler_simulation.cpp:20-88) on one GB300.
//
//   euler_simulation [--nx 128] [--nt 200] [--output-freq 10] [--cfl 0.49]
//                    [--gamma 1.4] [--mode fused|operators|exact]
//                    [--precision f64|f32c|f32c_hilo|f32] [--out DIR]
//
// Defaults are the reference driver's hard-coded values (:25-29).  Every
// `output-freq` steps the pressure field (ghosts included, layout_left) is
// written as DIR/test_%010d.npy (:71-79) in the reference's NPY format.  At
// the end it prints the throughput in Mcell-updates/s over nt * nx^3
// interior cells (:84-87).
//
// --mode fused (default) runs the device-resident simulation: one fused
// kernel per step replayed from a CUDA graph, dt kept on the device, and
// the state copied to the host only for output.  --mode operators runs the
// reference's own loop -- time_step, godunov(cfl*dt), cons_to_prim -- through
// the drop-in operator headers (FP64 or FP32 per --precision f64|f32).
// --mode exact runs the same loop with godunov replaced by the bit-identical
// eulr_godunov_exact_{f64,f32}, so that every written pressure field equals
// the reference loop's bit for bit.
#include <euler_gb300.h>

#include <cons_to_prim.hpp>
#include <euler_arrays.hpp>
#include <euler_npy.hpp>
#include <godunov.hpp>
#include <hllc.hpp>
#include <init_implode.hpp>
#include <perfect_gas.hpp>
#include <prim_to_cons.hpp>
#include <time_step.hpp>
#include <uniform_mesh.hpp>

#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <iomanip>
#include <iostream>
#include <sstream>
#include <string>
#include <type_traits>
#include <vector>

namespace {

struct Options {
    int nx = 128;
    int nt = 200;
    int output_freq = 10;
    double cfl = 0.49;
    double gamma = 1.4;
    std::string mode = "fused";
    std::string precision = "f64";
    std::string out = ".";
};

[[noreturn]] void usage(const char* argv0)
{
    std::cerr << "usage: " << argv0
              << " [--nx N] [--nt STEPS] [--output-freq K] [--cfl C] [--gamma G]"
                 " [--mode fused|operators|exact] [--precision f64|f32c|f32c_hilo|f32] [--out DIR]\n";
    std::exit(2);
}

Options parse(int argc, char** argv)
{
    Options o;
    for (int a = 1; a < argc; ++a) {
        std::string const k = argv[a];
        auto next = [&]() -> std::string {
            if (a + 1 >= argc) {
                usage(argv[0]);
            }
            return argv[++a];
        };
        if (k == "--nx") {
            o.nx = std::stoi(next());
        } else if (k == "--nt") {
            o.nt = std::stoi(next());
        } else if (k == "--output-freq") {
            o.output_freq = std::stoi(next());
        } else if (k == "--cfl") {
            o.cfl = std::stod(next());
        } else if (k == "--gamma") {
            o.gamma = std::stod(next());
        } else if (k == "--mode") {
            o.mode = next();
        } else if (k == "--precision") {
            o.precision = next();
        } else if (k == "--out") {
            o.out = next();
        } else {
            usage(argv[0]);
        }
    }
    if (o.nx < 1 || o.nt < 0 || (o.mode != "fused" && o.mode != "operators" && o.mode != "exact")) {
        usage(argv[0]);
    }
    return o;
}

std::string output_name(Options const& o, int it)
{
    std::stringstream ss;
    ss << o.out << "/test_" << std::setfill('0') << std::setw(10) << it << ".npy";
    return ss.str();
}

void check(int st, const char* what)
{
    if (st != EULR_SUCCESS) {
        std::cerr << what << ": " << eulr_status_string(st) << ": " << eulr_last_error() << "\n";
        std::exit(1);
    }
}

int precision_code(std::string const& p)
{
    if (p == "f64") {
        return EULR_PRECISION_F64;
    }
    if (p == "f32c") {
        return EULR_PRECISION_F32C;
    }
    if (p == "f32c_hilo") {
        return EULR_PRECISION_F32C_HILO;
    }
    if (p == "f32") {
        return EULR_PRECISION_F32;
    }
    std::cerr << "unknown precision " << p << "\n";
    std::exit(2);
}

// Device-resident loop: eulr_sim advances output_freq steps at a time.
double run_fused(Options const& o)
{
    int const n = o.nx + 2;
    double const dx = 1.0 / o.nx;
    eulr_sim* sim = nullptr;
    check(eulr_sim_create(precision_code(o.precision), n, n, n, o.gamma, dx, dx, dx, o.cfl, nullptr, &sim),
          "eulr_sim_create");
    check(eulr_sim_init_implode(sim), "eulr_sim_init_implode");
    std::size_t const cells = static_cast<std::size_t>(n) * n * n;
    std::vector<double> p_host(cells);
    eulr_prim_f64 prim_out {nullptr, p_host.data(), nullptr, nullptr, nullptr};
    eulr_cons_f64 no_cons {nullptr, nullptr, nullptr, nullptr, nullptr};
    check(eulr_sim_time(sim, nullptr, nullptr, nullptr), "sync"); // waits for the stream
    auto const start = std::chrono::steady_clock::now();
    int it = 0;
    while (it < o.nt) {
        int const chunk = o.output_freq > 0 ? std::min(o.output_freq - it % o.output_freq, o.nt - it) : o.nt - it;
        check(eulr_sim_advance(sim, chunk), "eulr_sim_advance");
        it += chunk;
        if (o.output_freq > 0 && it % o.output_freq == 0) {
            std::string const name = output_name(o, it);
            std::cout << "Saving " << name << ' ';
            check(eulr_sim_get_state_f64(sim, prim_out, no_cons), "eulr_sim_get_state_f64");
            euler_npy::write_file(name, p_host.data(), {static_cast<std::size_t>(n), static_cast<std::size_t>(n),
                                                        static_cast<std::size_t>(n)},
                                  true);
            std::cout << "done\n" << std::flush;
        }
    }
    check(eulr_sim_time(sim, nullptr, nullptr, nullptr), "sync");
    auto const end = std::chrono::steady_clock::now();
    check(eulr_sim_status(sim), "eulr_sim_status");
    eulr_sim_destroy(sim);
    return std::chrono::duration<double>(end - start).count();
}

// godunov through eulr_godunov_exact_{f64,f32}: the drop-in's arguments,
// the reference's results bit for bit.
template <class P, class C, class real_t>
void godunov_bit_exact(Kokkos::DefaultExecutionSpace const& exec_space, P const& prim_arrays, C const& cons_arrays,
                       PerfectGas<real_t> const& eos, UniformMesh3d<real_t> const& mesh, real_t const dt)
{
    namespace b = euler_gb300_bridge;
    using ty = b::types<real_t>;
    auto const& s = prim_arrays.d;
    int st;
    if constexpr (std::is_same_v<real_t, double>) {
        st = eulr_godunov_exact_f64(b::prim_ptrs<typename ty::cprim>(prim_arrays),
                                    b::cons_ptrs<typename ty::cons>(cons_arrays), b::extent_int(s, 0),
                                    b::extent_int(s, 1), b::extent_int(s, 2), eos.gamma(), mesh.dx0(), mesh.dx1(),
                                    mesh.dx2(), dt, b::stream_of(exec_space));
    } else {
        st = eulr_godunov_exact_f32(b::prim_ptrs<typename ty::cprim>(prim_arrays),
                                    b::cons_ptrs<typename ty::cons>(cons_arrays), b::extent_int(s, 0),
                                    b::extent_int(s, 1), b::extent_int(s, 2), eos.gamma(), mesh.dx0(), mesh.dx1(),
                                    mesh.dx2(), dt, b::stream_of(exec_space));
    }
    b::check(st, "godunov (bit-exact)");
}

// The reference's loop through the drop-in operator headers; with `exact`,
// godunov is the bit-identical one.
template <class real_t>
double run_operators(Options const& o, bool const exact)
{
    using index_t = int;
    using span = Kokkos::mdspan<real_t, Kokkos::dextents<index_t, 3>, Kokkos::layout_left>;
    real_t const dx = real_t(1) / static_cast<real_t>(o.nx);
    int const n = o.nx + 2;
    PerfectGas<real_t> const eos(static_cast<real_t>(o.gamma));
    UniformMesh3d<real_t> const mesh(dx, dx, dx);
    hllc const riemann_solver;
    Kokkos::DefaultExecutionSpace const exec_space;
    auto const prims_alloc = create_prim_arrays_1d<real_t>(exec_space, static_cast<std::size_t>(n) * n * n);
    auto const prim_arrays = to_mdspan<span>(prims_alloc, n, n, n);
    auto const cons_alloc = create_cons_arrays_1d<real_t>(exec_space, static_cast<std::size_t>(n) * n * n);
    auto const cons_arrays = to_mdspan<span>(cons_alloc, n, n, n);
    init_implode(exec_space, prim_arrays, mesh);
    prim_to_cons(exec_space, as_const(prim_arrays), cons_arrays, eos);
    exec_space.fence();
    auto const start = std::chrono::steady_clock::now();
    for (int it = 1; it <= o.nt; ++it) {
        real_t const dt = time_step(exec_space, as_const(prim_arrays), eos, mesh);
        if (exact) {
            godunov_bit_exact(exec_space, as_const(prim_arrays), cons_arrays, eos, mesh,
                              static_cast<real_t>(o.cfl) * dt);
        } else {
            godunov(exec_space, as_const(prim_arrays), cons_arrays, eos, mesh, riemann_solver,
                    static_cast<real_t>(o.cfl) * dt);
        }
        cons_to_prim(exec_space, as_const(cons_arrays), prim_arrays, eos);
        if (o.output_freq > 0 && it % o.output_freq == 0) {
            std::string const name = output_name(o, it);
            std::cout << "Saving " << name << ' ';
            exec_space.fence(); // the arrays are managed memory: read on the host after the stream drains
            euler_npy::write_file(name, prim_arrays.p.data_handle(),
                                  {static_cast<std::size_t>(n), static_cast<std::size_t>(n),
                                   static_cast<std::size_t>(n)},
                                  true);
            std::cout << "done\n" << std::flush;
        }
    }
    exec_space.fence();
    auto const end = std::chrono::steady_clock::now();
    return std::chrono::duration<double>(end - start).count();
}

} // namespace

int main(int argc, char** argv)
{
    Options const o = parse(argc, argv);
    double seconds = 0;
    if (o.mode == "fused") {
        seconds = run_fused(o);
    } else if (o.precision == "f32") {
        seconds = run_operators<float>(o, o.mode == "exact");
    } else {
        seconds = run_operators<double>(o, o.mode == "exact");
    }
    double const cells_updated = o.nt * static_cast<double>(o.nx) * o.nx * o.nx;
    std::cout << cells_updated / seconds * 1e-6 << '\n';
    return 0;
}
