// Algorithmic FLOP count of the reference operators (test/measurement tool).
//
// Instantiates the reference's own templates (euler_operators/*.hpp, compiled
// unmodified through the test-only Kokkos shim) with a scalar type that
// counts every +, -, *, / and sqrt (min, max, abs, comparisons and selects
// count 0), on grids of one and two interior cells.  The difference gives
// the per-cell cost without per-call constants.  Prints JSON; the committed
// result is oracle/flops_per_cell.json, read by bench.py for the roofline.
//
//   make -C oracle flops && oracle/_ref/count_flops > oracle/flops_per_cell.json

#include <Kokkos_Core.hpp>

#include <cmath>
#include <cstdio>
#include <limits>
#include <vector>

struct Counted;

struct Tally {
    long long add = 0, sub = 0, mul = 0, div = 0, sqrt = 0;
    long long total() const { return add + sub + mul + div + sqrt; }
};
static Tally g_tally;

struct Counted {
    double v = 0;
    Counted() = default;
    Counted(double x) : v(x) {} // NOLINT: implicit, like a real scalar
};

inline Counted operator+(Counted a, Counted b) { ++g_tally.add; return {a.v + b.v}; }
inline Counted operator-(Counted a, Counted b) { ++g_tally.sub; return {a.v - b.v}; }
inline Counted operator*(Counted a, Counted b) { ++g_tally.mul; return {a.v * b.v}; }
inline Counted operator/(Counted a, Counted b) { ++g_tally.div; return {a.v / b.v}; }
inline Counted operator-(Counted a) { return {-a.v}; }
inline Counted operator+(Counted a, int b) { return a + Counted(b); }
inline Counted operator-(Counted a, int b) { return a - Counted(b); }
inline Counted operator*(Counted a, int b) { return a * Counted(b); }
inline Counted operator/(Counted a, int b) { return a / Counted(b); }
inline Counted operator+(int a, Counted b) { return Counted(a) + b; }
inline Counted operator-(int a, Counted b) { return Counted(a) - b; }
inline Counted operator*(int a, Counted b) { return Counted(a) * b; }
inline Counted operator/(int a, Counted b) { return Counted(a) / b; }
inline Counted& operator+=(Counted& a, Counted b) { a = a + b; return a; }
inline Counted& operator-=(Counted& a, Counted b) { a = a - b; return a; }
inline bool operator<(Counted a, Counted b) { return a.v < b.v; }
inline bool operator>(Counted a, Counted b) { return a.v > b.v; }
inline bool operator<(Counted a, int b) { return a.v < b; }
inline bool operator>(Counted a, int b) { return a.v > b; }

namespace std {
template <>
class numeric_limits<Counted> : public numeric_limits<double> {
public:
    static Counted max() noexcept { return Counted(numeric_limits<double>::max()); }
};
} // namespace std

namespace Kokkos {
inline Counted sqrt(Counted a) { ++g_tally.sqrt; return {std::sqrt(a.v)}; }
inline Counted abs(Counted a) { return {std::fabs(a.v)}; }
} // namespace Kokkos

#include <cons_to_prim.hpp>
#include <euler_arrays.hpp>
#include <godunov.hpp>
#include <hllc.hpp>
#include <perfect_gas.hpp>
#include <prim_to_cons.hpp>
#include <time_step.hpp>
#include <uniform_mesh.hpp>

namespace {

using span3 = Kokkos::mdspan<Counted, Kokkos::dextents<int, 3>, Kokkos::layout_left>;

struct Grid {
    int n0, n1, n2;
    std::vector<Counted> f[10];
    explicit Grid(int a, int b, int c) : n0(a), n1(b), n2(c)
    {
        for (auto& v : f) {
            v.assign(static_cast<size_t>(a) * b * c, Counted(1.0));
        }
        // a non-trivial subsonic state: unequal pressures and velocities
        for (size_t i = 0; i < f[0].size(); ++i) {
            f[0][i] = Counted(1.0 + 0.1 * static_cast<double>(i % 3));
            f[1][i] = Counted(1.0 + 0.2 * static_cast<double>(i % 5));
            f[2][i] = Counted(0.1 * static_cast<double>(i % 2));
            f[3][i] = Counted(-0.05 * static_cast<double>(i % 3));
            f[4][i] = Counted(0.02);
        }
    }
    EulerPrimArrays<span3> prim()
    {
        return {span3(f[0].data(), n0, n1, n2), span3(f[1].data(), n0, n1, n2), span3(f[2].data(), n0, n1, n2),
                span3(f[3].data(), n0, n1, n2), span3(f[4].data(), n0, n1, n2)};
    }
    EulerConsArrays<span3> cons()
    {
        return {span3(f[5].data(), n0, n1, n2), span3(f[6].data(), n0, n1, n2), span3(f[7].data(), n0, n1, n2),
                span3(f[8].data(), n0, n1, n2), span3(f[9].data(), n0, n1, n2)};
    }
};

template <class F>
Tally count(F&& fn)
{
    g_tally = Tally {};
    fn();
    return g_tally;
}

Tally diff(Tally a, Tally b)
{
    return {a.add - b.add, a.sub - b.sub, a.mul - b.mul, a.div - b.div, a.sqrt - b.sqrt};
}

void print(const char* name, Tally t, bool comma = true)
{
    std::printf("  \"%s\": {\"total\": %lld, \"add\": %lld, \"sub\": %lld, \"mul\": %lld, \"div\": %lld, \"sqrt\": %lld}%s\n",
                name, t.total(), t.add, t.sub, t.mul, t.div, t.sqrt, comma ? "," : "");
}

} // namespace

int main()
{
    Kokkos::DefaultExecutionSpace const exec;
    PerfectGas<Counted> const eos(Counted(1.4));
    UniformMesh3d<Counted> const mesh(Counted(0.1), Counted(0.1), Counted(0.1));

    // one HLLC face
    EulerPrim<Counted> const qL {Counted(1.0), Counted(1.0), Counted(0.1), Counted(0.0), Counted(0.0)};
    EulerPrim<Counted> const qR {Counted(0.5), Counted(0.3), Counted(-0.1), Counted(0.0), Counted(0.0)};
    Tally const face = count([&] { (void)hllc()(std::integral_constant<std::size_t, 0>(), eos, qL, qR); });

    // per-cell costs: grids with one and with two interior cells
    Grid g1(3, 3, 3), g2(4, 3, 3);
    auto per_cell = [&](auto&& op) { return diff(count([&] { op(g2); }), count([&] { op(g1); })); };

    Tally const godunov_cell = per_cell([&](Grid& g) {
        godunov(exec, as_const(g.prim()), g.cons(), eos, mesh, hllc(), Counted(1e-3));
    });
    // all-cell operators: 27 vs 36 cells -> divide the difference by 9
    auto per_cell_all = [&](auto&& op) {
        Tally t = diff(count([&] { op(g2); }), count([&] { op(g1); }));
        return Tally {t.add / 9, t.sub / 9, t.mul / 9, t.div / 9, t.sqrt / 9};
    };
    Tally const p2c = per_cell_all([&](Grid& g) { prim_to_cons(exec, as_const(g.prim()), g.cons(), eos); });
    Tally const c2p = per_cell_all([&](Grid& g) { cons_to_prim(exec, as_const(g.cons()), g.prim(), eos); });
    Tally const ts = per_cell_all([&](Grid& g) { (void)time_step(exec, as_const(g.prim()), eos, mesh); });

    // The reference godunov solves 6 faces per cell; the remainder is the
    // per-cell accumulation and update.
    Tally const six {face.add * 6, face.sub * 6, face.mul * 6, face.div * 6, face.sqrt * 6};
    Tally const update = diff(godunov_cell, six);
    Tally const three {face.add * 3, face.sub * 3, face.mul * 3, face.div * 3, face.sqrt * 3};
    Tally fused {three.add + update.add + c2p.add + ts.add, three.sub + update.sub + c2p.sub + ts.sub,
                 three.mul + update.mul + c2p.mul + ts.mul, three.div + update.div + c2p.div + ts.div,
                 three.sqrt + update.sqrt + c2p.sqrt + ts.sqrt};

    std::printf("{\n");
    std::printf("  \"convention\": \"+,-,*,/,sqrt count 1 each; min, max, abs, compare and select count 0; "
                "counted by instantiating the reference templates (euler_operators/*.hpp) with a counting scalar\",\n");
    print("hllc_face", face);
    print("godunov_reference_per_cell", godunov_cell);
    print("godunov_update_per_cell", update);
    print("prim_to_cons_per_cell", p2c);
    print("cons_to_prim_per_cell", c2p);
    print("time_step_per_cell", ts);
    print("fused_step_per_cell_detail", fused);
    std::printf("  \"fused_step_fp64\": %lld,\n", fused.total());
    std::printf("  \"fused_step_note\": \"3 HLLC faces (each face solved once) + godunov accumulation/update + "
                "cons_to_prim + time_step wavespeed, per interior cell\"\n");
    std::printf("}\n");
    return 0;
}
