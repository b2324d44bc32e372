// euler_benchmarks: the reference's benchmark set (benchmarks/*.cpp) on one
// GB300, emitting Google Benchmark's JSON so plot.py (:34-50) reads it as is.
//
//   euler_benchmarks [--benchmark_out=FILE] [--benchmark_filter=SUBSTR]
//                    [--benchmark_min_time=SECONDS]
//
// Families, sizes, states and counters follow the reference:
//   Godunov/<n>        n+2 cells per axis, prim (1,1,0,0,0), dt 1e-9, dx 1
//                      (benchmark_godunov.cpp:16-57)
//   TimeStep/<n>       n cells per axis (benchmark_time_step.cpp:15-42)
//   ConsToPrim/<n>     cons (1, 1/0.4, 0,0,0) (benchmark_cons_to_prim.cpp:14-45)
//   PrimToCons/<n>     prim (1,1,0,0,0) (benchmark_prim_to_cons.cpp:14-45)
//   EulerSimulation/<nx> implosion, one time_step/godunov/cons_to_prim step per
//                      iteration, CFL 0.49 (benchmark_euler_simulation.cpp:20-67)
// with n in 8,16,24,32..320 step 32 and nx in 16..304 step 32, counters
// cells_per_second and bytes_per_second as iteration-invariant rates
// (benchmark_utils.cpp:5-15).  Two extra families time the device-resident
// fused step: EulerStepFused/<nx> (FP64) and EulerStepF32C/<nx>.
//
// Each iteration is the operator call followed by a fence, as in the
// reference; iterations repeat until min_time seconds have passed.  Times
// are wall clock per iteration; real_time and cpu_time carry the same value.
#include <euler_gb300.h>

#include <cons_to_prim.hpp>
#include <euler_arrays.hpp>
#include <godunov.hpp>
#include <hllc.hpp>
#include <init_implode.hpp>
#include <perfect_gas.hpp>
#include <prim_to_cons.hpp>
#include <time_step.hpp>
#include <uniform_mesh.hpp>

#include <unistd.h>

#include <algorithm>
#include <chrono>
#include <cstdio>
#include <ctime>
#include <fstream>
#include <functional>
#include <iomanip>
#include <iostream>
#include <sstream>
#include <string>
#include <thread>
#include <vector>

namespace {

using real_t = double;
using index_t = int;
using span = Kokkos::mdspan<real_t, Kokkos::dextents<index_t, 3>, Kokkos::layout_left>;

struct Result {
    std::string name;
    long long iterations;
    double ns_per_iter;
    double cells;
    double bytes;
};

double g_min_time = 0.5;

// Runs fn (which must end with a fence) until g_min_time seconds have passed.
Result measure(std::string name, double cells, double bytes, std::function<void()> const& fn)
{
    fn(); // warm-up
    long long iters = 0;
    auto const t0 = std::chrono::steady_clock::now();
    double el = 0;
    do {
        fn();
        ++iters;
        el = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    } while (el < g_min_time && iters < 1000000);
    return {std::move(name), iters, el * 1e9 / static_cast<double>(iters), cells, bytes};
}

template <class A>
void fill(A const& a, real_t v)
{
    std::fill(a.data(), a.data() + a.size(), v);
}

void fill_prim(EulerPrimArrays<Kokkos::View<real_t*>> const& p, EulerPrim<real_t> const& q)
{
    fill(p.d, q.d);
    fill(p.p, q.p);
    fill(p.ux0, q.ux0);
    fill(p.ux1, q.ux1);
    fill(p.ux2, q.ux2);
}

void fill_cons(EulerConsArrays<Kokkos::View<real_t*>> const& c, EulerCons<real_t> const& u)
{
    fill(c.d, u.d);
    fill(c.e, u.e);
    fill(c.mx0, u.mx0);
    fill(c.mx1, u.mx1);
    fill(c.mx2, u.mx2);
}

Result bench_godunov(int range)
{
    int const n = range + 2;
    PerfectGas<real_t> const eos(1.4);
    UniformMesh3d<real_t> const mesh(1., 1., 1.);
    Kokkos::DefaultExecutionSpace const exec;
    auto const pa = create_prim_arrays_1d<real_t>(exec, static_cast<std::size_t>(n) * n * n);
    auto const ca = create_cons_arrays_1d<real_t>(exec, static_cast<std::size_t>(n) * n * n);
    EulerPrim<real_t> const q {1, 1, 0, 0, 0};
    fill_prim(pa, q);
    fill_cons(ca, to_cons(q, eos.internal_energy(q.d, q.p)));
    auto const p = to_mdspan<span>(pa, n, n, n);
    auto const c = to_mdspan<span>(ca, n, n, n);
    return measure("Godunov/" + std::to_string(range), static_cast<double>(size(c)),
                   static_cast<double>(size_bytes(p) + 2 * size_bytes(c)), [&] {
                       godunov(exec, as_const(p), c, eos, mesh, hllc(), 1e-9);
                       exec.fence();
                   });
}

Result bench_time_step(int range)
{
    int const n = range;
    PerfectGas<real_t> const eos(1.4);
    UniformMesh3d<real_t> const mesh(1., 1., 1.);
    Kokkos::DefaultExecutionSpace const exec;
    auto const pa = create_prim_arrays_1d<real_t>(exec, static_cast<std::size_t>(n) * n * n);
    fill_prim(pa, {1, 1, 0, 0, 0});
    auto const p = to_mdspan<span>(pa, n, n, n);
    return measure("TimeStep/" + std::to_string(range), static_cast<double>(size(p)),
                   static_cast<double>(size_bytes(p)), [&] {
                       volatile real_t dt = time_step(exec, as_const(p), eos, mesh);
                       (void)dt;
                       exec.fence();
                   });
}

Result bench_cons_to_prim(int range)
{
    int const n = range;
    PerfectGas<real_t> const eos(1.4);
    Kokkos::DefaultExecutionSpace const exec;
    auto const pa = create_prim_arrays_1d<real_t>(exec, static_cast<std::size_t>(n) * n * n);
    auto const ca = create_cons_arrays_1d<real_t>(exec, static_cast<std::size_t>(n) * n * n);
    fill_cons(ca, {1, 1 / 0.4, 0, 0, 0});
    auto const p = to_mdspan<span>(pa, n, n, n);
    auto const c = to_mdspan<span>(ca, n, n, n);
    return measure("ConsToPrim/" + std::to_string(range), static_cast<double>(size(p)),
                   static_cast<double>(size_bytes(p) + size_bytes(c)), [&] {
                       cons_to_prim(exec, as_const(c), p, eos);
                       exec.fence();
                   });
}

Result bench_prim_to_cons(int range)
{
    int const n = range;
    PerfectGas<real_t> const eos(1.4);
    Kokkos::DefaultExecutionSpace const exec;
    auto const pa = create_prim_arrays_1d<real_t>(exec, static_cast<std::size_t>(n) * n * n);
    auto const ca = create_cons_arrays_1d<real_t>(exec, static_cast<std::size_t>(n) * n * n);
    fill_prim(pa, {1, 1, 0, 0, 0});
    auto const p = to_mdspan<span>(pa, n, n, n);
    auto const c = to_mdspan<span>(ca, n, n, n);
    return measure("PrimToCons/" + std::to_string(range), static_cast<double>(size(c)),
                   static_cast<double>(size_bytes(p) + size_bytes(c)), [&] {
                       prim_to_cons(exec, as_const(p), c, eos);
                       exec.fence();
                   });
}

Result bench_euler_simulation(int nx)
{
    real_t const cfl = 0.49;
    real_t const dx = 1. / static_cast<real_t>(nx);
    int const n = nx + 2;
    PerfectGas<real_t> const eos(1.4);
    UniformMesh3d<real_t> const mesh(dx, dx, dx);
    Kokkos::DefaultExecutionSpace const exec;
    auto const pa = create_prim_arrays_1d<real_t>(exec, static_cast<std::size_t>(n) * n * n);
    auto const ca = create_cons_arrays_1d<real_t>(exec, static_cast<std::size_t>(n) * n * n);
    auto const p = to_mdspan<span>(pa, n, n, n);
    auto const c = to_mdspan<span>(ca, n, n, n);
    init_implode(exec, p, mesh);
    prim_to_cons(exec, as_const(p), c, eos);
    exec.fence();
    return measure("EulerSimulation/" + std::to_string(nx), static_cast<double>(size(c)), 0.0, [&] {
        real_t const dt = time_step(exec, as_const(p), eos, mesh);
        godunov(exec, as_const(p), c, eos, mesh, hllc(), cfl * dt);
        cons_to_prim(exec, as_const(c), p, eos);
        exec.fence();
    });
}

Result bench_fused(int nx, int precision, const char* family)
{
    int const n = nx + 2;
    double const dx = 1.0 / nx;
    eulr_sim* sim = nullptr;
    if (eulr_sim_create(precision, n, n, n, 1.4, dx, dx, dx, 0.49, nullptr, &sim) != EULR_SUCCESS ||
        eulr_sim_init_implode(sim) != EULR_SUCCESS) {
        throw std::runtime_error(eulr_last_error());
    }
    Result r = measure(std::string(family) + "/" + std::to_string(nx), static_cast<double>(n) * n * n, 0.0, [&] {
        eulr_sim_advance(sim, 1);
        eulr_sim_time(sim, nullptr, nullptr, nullptr); // fence
    });
    eulr_sim_destroy(sim);
    return r;
}

std::string json_escape(std::string const& s)
{
    std::string o;
    for (char ch : s) {
        if (ch == '"' || ch == '\\') {
            o += '\\';
        }
        o += ch;
    }
    return o;
}

void write_json(std::ostream& os, std::vector<Result> const& rs, std::string const& exe)
{
    char host[256] = {};
    gethostname(host, sizeof(host) - 1);
    std::time_t const now = std::time(nullptr);
    char date[64];
    std::strftime(date, sizeof(date), "%Y-%m-%dT%H:%M:%S%z", std::localtime(&now));
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceProp prop {};
    cudaGetDeviceProperties(&prop, dev);
    os.precision(17);
    os << "{\n  \"context\": {\n"
       << "    \"date\": \"" << date << "\",\n"
       << "    \"host_name\": \"" << json_escape(host) << "\",\n"
       << "    \"executable\": \"" << json_escape(exe) << "\",\n"
       << "    \"num_cpus\": " << std::thread::hardware_concurrency() << ",\n"
       << "    \"mhz_per_cpu\": 0,\n    \"cpu_scaling_enabled\": false,\n"
       << "    \"device\": \"" << json_escape(prop.name) << "\",\n"
       << "    \"library_version\": \"euler_gb300 " << eulr_version() << "\",\n"
       << "    \"library_build_type\": \"release\",\n    \"caches\": []\n  },\n  \"benchmarks\": [\n";
    std::string family;
    int fam = -1, inst = 0;
    for (std::size_t i = 0; i < rs.size(); ++i) {
        Result const& r = rs[i];
        std::string const f = r.name.substr(0, r.name.find('/'));
        if (f != family) {
            family = f;
            ++fam;
            inst = 0;
        }
        double const sec = r.ns_per_iter * 1e-9;
        os << "    {\n      \"name\": \"" << r.name << "\",\n"
           << "      \"family_index\": " << fam << ",\n      \"per_family_instance_index\": " << inst++ << ",\n"
           << "      \"run_name\": \"" << r.name << "\",\n      \"run_type\": \"iteration\",\n"
           << "      \"repetitions\": 1,\n      \"repetition_index\": 0,\n      \"threads\": 1,\n"
           << "      \"iterations\": " << r.iterations << ",\n"
           << "      \"real_time\": " << r.ns_per_iter << ",\n      \"cpu_time\": " << r.ns_per_iter << ",\n"
           << "      \"time_unit\": \"ns\"";
        if (r.bytes > 0) {
            os << ",\n      \"bytes_per_second\": " << r.bytes / sec;
        }
        os << ",\n      \"cells_per_second\": " << r.cells / sec << "\n    }" << (i + 1 < rs.size() ? "," : "")
           << "\n";
    }
    os << "  ]\n}\n";
}

} // namespace

int main(int argc, char** argv)
{
    std::string out, filter;
    for (int a = 1; a < argc; ++a) {
        std::string const k = argv[a];
        if (k.rfind("--benchmark_out=", 0) == 0) {
            out = k.substr(16);
        } else if (k.rfind("--benchmark_filter=", 0) == 0) {
            filter = k.substr(19);
        } else if (k.rfind("--benchmark_min_time=", 0) == 0) {
            g_min_time = std::stod(k.substr(21));
        } else if (k.rfind("--benchmark_format=", 0) == 0) {
            // JSON is the only format
        } else {
            std::cerr << "usage: " << argv[0]
                      << " [--benchmark_out=FILE] [--benchmark_filter=SUBSTR] [--benchmark_min_time=SECONDS]\n";
            return 2;
        }
    }
    std::vector<int> ranges;
    for (int r = 8; r <= 31; r += 8) {
        ranges.push_back(r);
    }
    for (int r = 32; r <= 320; r += 32) {
        ranges.push_back(r);
    }
    std::vector<int> sim_sizes;
    for (int r = 16; r <= 320; r += 32) {
        sim_sizes.push_back(r);
    }
    auto selected = [&](std::string const& name) { return filter.empty() || name.find(filter) != std::string::npos; };
    std::vector<Result> rs;
    auto run = [&](std::string const& family, std::vector<int> const& sizes, auto&& fn) {
        for (int s : sizes) {
            std::string const name = family + "/" + std::to_string(s);
            if (selected(name)) {
                rs.push_back(fn(s));
                std::cerr << name << " " << rs.back().ns_per_iter << " ns\n";
            }
        }
    };
    run("Godunov", ranges, bench_godunov);
    run("TimeStep", ranges, bench_time_step);
    run("ConsToPrim", ranges, bench_cons_to_prim);
    run("PrimToCons", ranges, bench_prim_to_cons);
    run("EulerSimulation", sim_sizes, bench_euler_simulation);
    run("EulerStepFused", sim_sizes, [](int nx) { return bench_fused(nx, EULR_PRECISION_F64, "EulerStepFused"); });
    run("EulerStepF32C", sim_sizes, [](int nx) { return bench_fused(nx, EULR_PRECISION_F32C, "EulerStepF32C"); });
    if (out.empty()) {
        write_json(std::cout, rs, argv[0]);
    } else {
        std::ofstream f(out);
        write_json(f, rs, argv[0]);
    }
    return 0;
}
