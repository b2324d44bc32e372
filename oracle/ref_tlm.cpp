// Forward-mode derivative of the reference's own operators (test only).
//
// Instantiates the reference headers (euler_operators/{godunov,hllc,
// prim_to_cons,cons_to_prim,perfect_gas,uniform_mesh,euler_arrays}.hpp,
// UNMODIFIED, through the test-only Kokkos shim) with a dual-number scalar,
// so every value carries its derivative through the reference's exact
// expression sequence.  It pins the C tangent-linear restatement
// (oracle/euler_tlm.c) at states without ties (at a tie the reference's
// min/max and branch pick one side, where the restatement takes the mean).
// Built by `make -C oracle ref` into oracle/_ref/libeuler_ref_tlm.so.

#include <Kokkos_Core.hpp>

#include <cmath>
#include <limits>
#include <vector>

struct Dual {
    double v = 0, d = 0;
    Dual() = default;
    Dual(double x) : v(x) {} // NOLINT: implicit, like a real scalar
    Dual(double x, double dx) : v(x), d(dx) {}
};

inline Dual operator+(Dual a, Dual b) { return {a.v + b.v, a.d + b.d}; }
inline Dual operator-(Dual a, Dual b) { return {a.v - b.v, a.d - b.d}; }
inline Dual operator*(Dual a, Dual b) { return {a.v * b.v, a.d * b.v + a.v * b.d}; }
inline Dual operator/(Dual a, Dual b) { return {a.v / b.v, (a.d * b.v - a.v * b.d) / (b.v * b.v)}; }
inline Dual operator-(Dual a) { return {-a.v, -a.d}; }
inline Dual operator+(Dual a, int b) { return a + Dual(b); }
inline Dual operator-(Dual a, int b) { return a - Dual(b); }
inline Dual operator*(Dual a, int b) { return a * Dual(b); }
inline Dual operator/(Dual a, int b) { return a / Dual(b); }
inline Dual operator+(int a, Dual b) { return Dual(a) + b; }
inline Dual operator-(int a, Dual b) { return Dual(a) - b; }
inline Dual operator*(int a, Dual b) { return Dual(a) * b; }
inline Dual operator/(int a, Dual b) { return Dual(a) / b; }
inline Dual& operator+=(Dual& a, Dual b) { a = a + b; return a; }
inline Dual& operator-=(Dual& a, Dual b) { a = a - b; return a; }
inline bool operator<(Dual a, Dual b) { return a.v < b.v; }
inline bool operator>(Dual a, Dual b) { return a.v > b.v; }
inline bool operator<(Dual a, int b) { return a.v < b; }
inline bool operator>(Dual a, int b) { return a.v > b; }

namespace std {
template <>
class numeric_limits<Dual> : public numeric_limits<double> {
public:
    static Dual max() noexcept { return Dual(numeric_limits<double>::max()); }
};
} // namespace std

namespace Kokkos {
inline Dual sqrt(Dual a)
{
    double const s = std::sqrt(a.v);
    return {s, a.d / (2.0 * s)};
}
inline Dual abs(Dual a) { return a.v < 0 ? -a : a; }
} // namespace Kokkos

#include <cons_to_prim.hpp>
#include <euler_arrays.hpp>
#include <godunov.hpp>
#include <hllc.hpp>
#include <perfect_gas.hpp>
#include <prim_to_cons.hpp>
#include <uniform_mesh.hpp>

namespace {

using span3 = Kokkos::mdspan<Dual, Kokkos::dextents<int, 3>, Kokkos::layout_left>;

struct Fields {
    std::vector<Dual> f[5];
    int n0, n1, n2;
    Fields(double const* const* v, double const* const* d, int a, int b, int c) : n0(a), n1(b), n2(c)
    {
        size_t const n = static_cast<size_t>(a) * b * c;
        for (int k = 0; k < 5; ++k) {
            f[k].resize(n);
            for (size_t i = 0; i < n; ++i) {
                f[k][i] = Dual(v[k][i], d[k][i]);
            }
        }
    }
    void store(double* const* v, double* const* d) const
    {
        for (int k = 0; k < 5; ++k) {
            for (size_t i = 0; i < f[k].size(); ++i) {
                v[k][i] = f[k][i].v;
                d[k][i] = f[k][i].d;
            }
        }
    }
    span3 s(int k) { return span3(f[k].data(), n0, n1, n2); }
    EulerPrimArrays<span3> prim() { return {s(0), s(1), s(2), s(3), s(4)}; }
    EulerConsArrays<span3> cons() { return {s(0), s(1), s(2), s(3), s(4)}; }
};

} // namespace

extern "C" {

void ref_tlm_prim_to_cons_f64(double const* const* prim, double const* const* dprim, double* const* cons,
                              double* const* dcons, int n0, int n1, int n2, double gamma)
{
    Fields p(prim, dprim, n0, n1, n2);
    Fields c(prim, dprim, n0, n1, n2);
    prim_to_cons(Kokkos::DefaultExecutionSpace(), as_const(p.prim()), c.cons(), PerfectGas<Dual>(Dual(gamma)));
    c.store(cons, dcons);
}

void ref_tlm_cons_to_prim_f64(double const* const* cons, double const* const* dcons, double* const* prim,
                              double* const* dprim, int n0, int n1, int n2, double gamma)
{
    Fields c(cons, dcons, n0, n1, n2);
    Fields p(cons, dcons, n0, n1, n2);
    cons_to_prim(Kokkos::DefaultExecutionSpace(), as_const(c.cons()), p.prim(), PerfectGas<Dual>(Dual(gamma)));
    p.store(prim, dprim);
}

void ref_tlm_godunov_f64(double const* const* prim, double const* const* dprim, double* const* cons,
                         double* const* dcons, int n0, int n1, int n2, double gamma, double dx0, double dx1, double dx2,
                         double dt)
{
    Fields p(prim, dprim, n0, n1, n2);
    Fields c(cons, dcons, n0, n1, n2);
    godunov(Kokkos::DefaultExecutionSpace(), as_const(p.prim()), c.cons(), PerfectGas<Dual>(Dual(gamma)),
            UniformMesh3d<Dual>(Dual(dx0), Dual(dx1), Dual(dx2)), hllc(), Dual(dt));
    c.store(cons, dcons);
}

} // extern "C"
