// x * 0.5 in binary64 from the bit pattern alone, on the integer pipe.
//
// GB300 runs FP64 arithmetic at 1/64 of its FP32 rate, and the FP64 kernels
// here are bound by their FP64 instruction count.  Halving is exact for
// every normal result -- the exponent field drops by one -- so a DMUL by 0.5
// can be replaced by integer operations with the same bits: an exponent
// decrement for normal results, a one-bit right shift of the significand
// rounded to nearest even for subnormal results, the input itself for
// infinities and NaN (NaN stays NaN; its payload is passed through).
// Plain integer C++, compiled for the host too and checked there against
// x * 0.5 bit for bit.
#pragma once

#include <cstdint>

#if defined(__CUDACC__)
#define EULR_HALVE_FN __host__ __device__ __forceinline__
#else
#define EULR_HALVE_FN inline
#endif

namespace eulr {

EULR_HALVE_FN uint64_t halve_bits(uint64_t b)
{
    uint64_t const sign = b & 0x8000000000000000ull;
    unsigned const e = static_cast<unsigned>(b >> 52) & 0x7ffu;
    uint64_t const mant = b & 0x000fffffffffffffull;
    // exponent field 0 or 1: the result is subnormal (or zero); the
    // significand shifts right by one and the bit shifted out, exactly half
    // a unit, rounds to even
    uint64_t const s = e == 1u ? (mant | 0x0010000000000000ull) : mant;
    uint64_t const q = (s >> 1) + (s & (s >> 1) & 1u);
    return e >= 2u ? (e == 0x7ffu ? b : b - 0x0010000000000000ull) : (sign | q);
}

} // namespace eulr
