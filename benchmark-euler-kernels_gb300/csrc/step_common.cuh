// Device helpers shared by the FP64/FP32 tile engine (flux.cu) and the FP32
// column engine (flux_f32.cu).  Internal to the library.
#pragma once

#include "euler_device.cuh"
#include "kernels.h"

namespace eulr {
namespace {

constexpr int kFields = 7; // face inputs of a staged cell: d, p, u0, u1, u2, c, e
constexpr long long kInfBits = 0x7ff0000000000000LL;

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
__device__ __forceinline__ float fast_sound_speed(float c2) { return c2 * rsqrtf(c2); }

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

} // namespace
} // namespace eulr
