// Host check of halve_bits (csrc/halve.cuh), the integer form of x * 0.5
// that the FP64 kernels use in place of a DMUL: every result equal to the
// host's IEEE product x * 0.5 bit for bit (NaN stays NaN).  Exported for
// ctypes: returns the number of mismatches over `count` seeded bit patterns,
// a third of them with exponent field 0 or 1 (subnormal results, ties).
#include "halve.cuh"

#include <cmath>
#include <cstdint>
#include <cstring>
#include <random>

extern "C" long long halve_mismatches(long long count, unsigned long long seed)
{
    std::mt19937_64 g(seed);
    long long bad = 0;
    for (long long i = 0; i < count; ++i) {
        uint64_t b = g();
        if (i % 3 == 1) {
            b &= 0x801fffffffffffffull; // exponent field 0 or 1
        } else if (i % 3 == 2) {
            b = (b & 0x800fffffffffffffull) | (static_cast<uint64_t>(g() % 4) << 52);
        }
        double x;
        std::memcpy(&x, &b, 8);
        double const r = x * 0.5;
        uint64_t rb;
        std::memcpy(&rb, &r, 8);
        uint64_t const h = eulr::halve_bits(b);
        double hx;
        std::memcpy(&hx, &h, 8);
        if (std::isnan(x) ? !std::isnan(hx) : h != rb) {
            ++bad;
        }
    }
    return bad;
}
