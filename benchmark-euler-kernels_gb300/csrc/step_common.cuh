// Device helpers shared by the FP64/FP32 tile engine (flux.cu) and the FP32
// column engine (flux_f32.cu).  Internal to the library.
#pragma once

#include "euler_device.cuh"
#include "kernels.h"

#include <cfloat>

namespace eulr {
namespace {

constexpr int kFields = 7; // face inputs of a staged cell: d, p, u0, u1, u2, c, e
constexpr long long kInfBits = 0x7ff0000000000000LL;

// g / D for 0 <= g < 2^12 and a compile-time 0 < D < 256, as one product and
// a shift: floor(g (floor(2^20/D) + 1) / 2^20) exceeds g/D by less than
// g/2^20 < 2^-8, which stays below the gap 1/D to the next integer.  The
// tile engine's face index takes one of two constant divisors by a select,
// which the compiler otherwise turned into a runtime integer division.
template <int D>
__device__ __forceinline__ int div_small(int g)
{
    static_assert(D > 0 && D < 256, "divisor range");
    constexpr unsigned kM = (1u << 20) / D + 1u;
    return static_cast<int>((static_cast<unsigned>(g) * kM) >> 20);
}

__device__ __forceinline__ unsigned smem_u32(const void* p)
{
    return static_cast<unsigned>(__cvta_generic_to_shared(p));
}

// Pressure of an FP32 conservative state: compensated states rescue the
// low-pressure cells in FP64 (pressure_f32c), plain FP32 does not.
template <int COMP>
__device__ __forceinline__ float cons_pressure(float d, float e, float m0, float m1, float m2, float r, float gm1,
                                               const float* lo)
{
    if (COMP != kCompNone) {
        return pressure_f32c(d, e, m0, m1, m2, r, gm1, lo);
    }
    return gm1 * (e - (0.5f * r) * (m0 * m0 + m1 * m1 + m2 * m2));
}
template <int COMP>
__device__ __forceinline__ double cons_pressure(double, double, double, double, double, double, double, const double*)
{
    return 0.0;
}

// Sound speed sqrt(gamma p / rho), faithful: fewer FP64 instructions than a
// correctly rounded sqrt, within one ulp of it.
__device__ __forceinline__ double fast_sound_speed(double c2) { return sqrt_faithful(c2); }
__device__ __forceinline__ float fast_sound_speed(float c2) { return c2 * rsqrt_approx(c2); }

__device__ __forceinline__ long long wave_key(double v)
{
    long long const b = dbits(v);
    return b <= kInfBits ? b : 0LL; // NaN never wins (the reference skips it)
}
__device__ __forceinline__ long long wave_key(float v) { return wave_key(static_cast<double>(v)); }

__device__ __forceinline__ bool cell_ok(double d, double pr, double invdt)
{
    return finite_positive(d) && finite_positive(pr) && dbits(invdt) < kInfBits;
}
__device__ __forceinline__ bool cell_ok(float d, float pr, float invdt)
{
    return d > 0.0f && pr > 0.0f && invdt <= 3.0e38f;
}

// sum + err += k*f without rounding error in the product (TwoProduct via
// FMA) or in the running sum (Knuth's TwoSum); the errors collect in err.
__device__ __forceinline__ void compensated_add(float& sum, float& err, float k, float f)
{
    float const prod = k * f;
    float const prod_err = fmaf(k, f, -prod);
    float const s = sum + prod;
    float const bb = s - sum;
    float const sum_err = (sum - (s - bb)) + (prod - bb);
    sum = s;
    err += sum_err + prod_err;
}
__device__ __forceinline__ void compensated_add(double&, double&, double, double) {}

// dt/dv, from the device dt when there is one (godunov.hpp:37 with the
// cfl * dt of euler_simulation.cpp:65), evaluated in double.
template <class T>
__device__ __forceinline__ T dt_over_dv(FluxParams<T> const& p)
{
    if (p.dt_seq != nullptr) {
        return static_cast<T>(p.dt_seq[*p.step_dev] / p.dv);
    }
    if (p.dt_dev != nullptr) {
        return static_cast<T>((p.cfl * *p.dt_dev) / p.dv);
    }
    return p.dtodv;
}

// Turns the max-wavespeed accumulator into the next step's dt
// (time_step.hpp:34-39: min over cells of 1/invdt == 1/max invdt), adds the
// step just taken to the simulated time and clears the accumulator.  The
// accumulator is read with a volatile load: other CTAs of the same launch
// raised it by atomics, and a cached copy must not answer.
template <class T>
__device__ __forceinline__ void finalize_one(SimScalars* s, T cfl, int add_time, const double* dt_seq = nullptr)
{
    if (add_time) {
        // the step just taken, cfl*dt (or the fixed dt), added with separate
        // roundings (no FMA) so every kernel that inlines this agrees bit for bit
        double const step = dt_seq != nullptr ? dt_seq[s->steps]
                                              : (sizeof(T) == 8 ? __dmul_rn(static_cast<double>(cfl), s->dt)
                                                                : static_cast<double>(cfl * static_cast<T>(s->dt)));
        s->t = __dadd_rn(s->t, step);
        s->steps += 1;
    }
    unsigned long long const w = *reinterpret_cast<volatile unsigned long long*>(&s->wmax);
    unsigned long long const wk = w > s->ghost_wmax ? w : s->ghost_wmax;
    T const m = static_cast<T>(__longlong_as_double(static_cast<long long>(wk)));
    T const dt = (m > T(0)) ? rcp_rn(m) : (sizeof(T) == 8 ? T(DBL_MAX) : T(FLT_MAX));
    s->dt = static_cast<double>(dt);
    s->wmax = 0ull;
}

// The step's own finalize, so that a step is one launch.  Called by thread 0
// of every CTA of a single-grid step launch after its wavespeed flush (the
// atomicMax precedes it in the same thread): the fence orders that flush
// before the count, and the CTA that counts last -- every other CTA has
// flushed and read this step's dt by then -- finalizes the step and rewinds
// the counter for the next launch.
template <class T>
__device__ __forceinline__ void step_done(FluxParams<T> const& p)
{
    if (p.fin == nullptr || threadIdx.x != 0) {
        return;
    }
    __threadfence();
    if (atomicAdd(&p.fin->done, 1u) == gridDim.x - 1) {
        __threadfence();
        finalize_one(p.fin, static_cast<T>(p.cfl), 1, p.dt_seq);
        p.fin->done = 0u;
    }
}

// The same for one work item of a batch launch: the grid's last item to
// finish finalizes that grid (its items were all taken from the queue before,
// so no CTA reads the grid's dt afterwards in this launch).  Thread 0, after
// the item's flush.
template <class T>
__device__ __forceinline__ void item_done(FluxParams<T> const& gp)
{
    if (gp.fin == nullptr || threadIdx.x != 0) {
        return;
    }
    __threadfence();
    if (atomicAdd(&gp.fin->done, 1u) == static_cast<unsigned>(gp.grid_items) - 1u) {
        __threadfence();
        finalize_one(gp.fin, static_cast<T>(gp.cfl), 1, gp.dt_seq);
        gp.fin->done = 0u;
    }
}

// A batch CTA leaving (the queue is empty for it).  Thread 0.  The last CTA
// to leave rewinds the queue head for the next launch -- every CTA has made
// its last pop by then -- and finalizes the grids that have no work item.
template <class T>
__device__ __forceinline__ void batch_cta_done(BatchParams<T> const& b)
{
    if (b.exited == nullptr || threadIdx.x != 0) {
        return;
    }
    __threadfence();
    if (atomicAdd(b.exited, 1u) == gridDim.x - 1) {
        __threadfence();
        for (int i = 0; i < b.nidle; ++i) {
            FluxParams<T> const& g = b.grids[b.idle[i]];
            if (g.fin != nullptr) {
                finalize_one(g.fin, static_cast<T>(g.cfl), 1, g.dt_seq);
            }
        }
        *b.head = 0u;
        *b.exited = 0u;
    }
}

// Chunk length (planes per work item) that balances the persistent grid:
// the step lasts as long as its busiest CTA, while each extra chunk costs
// one more z face row and two more staged planes (about 1/(3 kchunk) of a
// chunk's work).  Scores every length from 8 to 64 by
//   (planes / (resident CTAs x planes of the busiest CTA)) x (1 - 1/(3 kchunk))
// and keeps the best.
inline int choose_kchunk(int columns, int iz, long long slots)
{
    int best = 64;
    double best_score = -1.0;
    for (int kc = 8; kc <= 64; ++kc) {
        long long const chunks = (iz + kc - 1) / kc;
        long long const items = chunks * columns;
        long long const rounds = (items + slots - 1) / slots; // items of the busiest CTA
        double const busiest = static_cast<double>(rounds) * kc;
        double const score = (static_cast<double>(iz) * columns / (static_cast<double>(slots) * busiest)) *
                             (1.0 - 1.0 / (3.0 * kc));
        if (score > best_score + 1e-9) {
            best_score = score;
            best = kc;
        }
    }
    return best;
}

// ------------------------------------------ exact max wavespeed, screened
// The CFL step needs the max over cells of the reference's wavespeed
// (time_step.hpp:28-33; cell_invdt_exact: a correctly rounded FP64 division
// and square root per cell, about 25 FP64 issue slots), exactly.  But the
// exact value is needed only where it can be the max, so an FP32 estimate
// screens the cells, with no FP64 instruction at all: its inputs are built
// from the doubles' high words on the integer pipe (the mantissa truncated to
// 20 bits, a relative error in (-2^-20, 0]) and the rest runs on the FP32
// pipe.  Where rho, p and gamma p/rho lie in [1e-30, 1e30] and the estimate
// is at most 1e30, its relative error is below 2^-20 + 5 * 2^-24 to first
// order: p/rho carries under 2^-20 (both truncations go toward zero), the
// square root halves it, |u| carries under 2^-20, and gamma, 1/dx and eight
// FP32 operations add 2^-24 each along any path.  Two estimates can thus
// misorder cells by at most 2.7 * 2^-20 relative, 42 FP32 ulps; a cell is
// evaluated exactly when its estimate is within 128 ulps of the warp's
// running max of estimates.  Every other cell -- NaN, infinite or
// out-of-range values -- is always evaluated exactly.  So the cell holding
// the exact max is always evaluated, and the max of the exact values over
// the evaluated cells is the exact max.  The evaluated cells are essentially
// each warp's running-max records: a few per ten thousand on random states.
struct WaveScreen {
    float g, ix0, ix1, ix2;
    bool on;        // gamma and 1/dx in FP32's safe range: screening is sound
    unsigned run;   // the warp's running max of the estimates' bit patterns

    __device__ __forceinline__ static bool in_range(float x) { return x >= 1e-30f && x <= 1e30f; }

    // x with its mantissa truncated to 20 bits, from the high word alone: 0
    // below FP32's normal range, infinity above it (and for NaN).
    __device__ __forceinline__ static float high_word_float(double x)
    {
        unsigned const hi = static_cast<unsigned>(static_cast<unsigned long long>(__double_as_longlong(x)) >> 32);
        int const e = static_cast<int>((hi >> 20) & 0x7ffu) - (1023 - 127);
        unsigned const mag = e <= 0 ? 0u : (e >= 255 ? 0x7f800000u : (static_cast<unsigned>(e) << 23) | ((hi & 0xfffffu) << 3));
        return __uint_as_float((hi & 0x80000000u) | mag);
    }

    __device__ __forceinline__ WaveScreen(double gamma, double x0, double x1, double x2)
        : g(static_cast<float>(gamma)), ix0(static_cast<float>(x0)), ix1(static_cast<float>(x1)),
          ix2(static_cast<float>(x2)), run(0u)
    {
        on = in_range(g) && in_range(ix0) && in_range(ix1) && in_range(ix2);
    }

    // Warp-collective (all 32 lanes call it together): true when this lane's
    // cell (if valid) needs its exact wavespeed.
    __device__ __forceinline__ bool exact_needed(bool valid, double d, double p, double u0, double u1, double u2)
    {
        float const d32 = high_word_float(d);
        float const p32 = high_word_float(p);
        float const x32 = __fdiv_rn(g * p32, d32);
        float const c32 = __fsqrt_rn(x32);
        float const v32 = (c32 + fabsf(high_word_float(u0))) * ix0 + (c32 + fabsf(high_word_float(u1))) * ix1 +
                          (c32 + fabsf(high_word_float(u2))) * ix2;
        bool const sure = on && in_range(d32) && in_range(p32) && in_range(x32) && v32 <= 1e30f;
        unsigned const key = (valid && sure) ? __float_as_uint(v32) : 0u;
        unsigned const m = __reduce_max_sync(0xffffffffu, key);
        run = m > run ? m : run;
        return valid && (!sure || key + 128u >= run);
    }

    // The fused FP64 step's form (warp-collective as well).  The step has the
    // new state's faithful sound speed cs and its velocities, and its
    // wavespeed is (3 cs + |v0| + |v1| + |v2|) / dx on cubic cells, else
    // sum_d (cs + |v_d|) / dx_d.  The estimate truncates cs and |v_d| (each
    // under 2^-20) and adds at most six FP32 roundings and 1/dx's own, so
    // its relative error is below 2^-20 + 6 * 2^-24, and two estimates
    // misorder by at most 44 ulps: the 128-ulp band holds here too.
    // Velocities below FP32's normal range read as zero: an error under
    // 2^-26 relative to cs >= 1e-30, far inside the band.
    __device__ __forceinline__ bool step_exact_needed(bool valid, double cs, double v0, double v1, double v2, bool cubic)
    {
        float const c32 = high_word_float(cs);
        float const a0 = fabsf(high_word_float(v0));
        float const a1 = fabsf(high_word_float(v1));
        float const a2 = fabsf(high_word_float(v2));
        float const v32 = cubic ? (3.0f * c32 + a0 + a1 + a2) * ix0
                                : (c32 + a0) * ix0 + (c32 + a1) * ix1 + (c32 + a2) * ix2;
        bool const sure = on && in_range(c32) && v32 <= 1e30f;
        unsigned const key = (valid && sure) ? __float_as_uint(v32) : 0u;
        unsigned const m = __reduce_max_sync(0xffffffffu, key);
        run = m > run ? m : run;
        return valid && (!sure || key + 128u >= run);
    }
};

} // namespace
} // namespace eulr
