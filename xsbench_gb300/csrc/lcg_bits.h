/* lcg_bits.h -- the reference's LCG draw in integer arithmetic.
 *
 * The reference turns the 63-bit LCG state s into a double as
 * (double)s / 9223372036854775808.0 (Simulation.c:462-470, GridInit.c:34-47):
 * s rounded to 53 significant bits (to nearest, ties to even), scaled by
 * 2^-63 exactly.  On GB300 the conversion and the scaling both run on the
 * FP64 pipe, which the lookups already saturate; the same value is assembled
 * here with integer instructions, bit for bit.  A material roll compares the
 * state itself with integer thresholds (the draw is a non-decreasing function
 * of the state, so `draw < x` is `s < T` for one T per threshold x), and an
 * energy bucket floor(draw * 2^k) is the rounded state shifted right.
 *
 * Plain C (also compiled by the CPU tests); CUDA device code includes it
 * through device_common.cuh.
 */
#ifndef XSGB_LCG_BITS_H
#define XSGB_LCG_BITS_H

#include <stdint.h>
#include <string.h>

#ifdef __CUDACC__
#define XSGB_LCG_HD __host__ __device__ __forceinline__
#define XSGB_LCG_HOST __host__ static inline
#else
#define XSGB_LCG_HD static inline
#define XSGB_LCG_HOST static inline
#endif

/* leading zeros of a non-zero 64-bit value */
XSGB_LCG_HD int xsgb_clz64(uint64_t x)
{
#ifdef __CUDA_ARCH__
    return __clzll((long long)x);
#else
    return __builtin_clzll(x);
#endif
}

/* s (below 2^63) rounded to 53 significant bits, to nearest, ties to even:
 * the integer value of (double)s.  Can be 2^63. */
XSGB_LCG_HD uint64_t xsgb_round53(uint64_t s)
{
    if (s < (1ULL << 53)) return s;
    const int sh = 11 - xsgb_clz64(s);   /* bits below the 53 kept, 1..10 */
    const uint64_t q = s >> sh;
    const uint64_t rem = s & ((1ULL << sh) - 1ULL);
    const uint64_t half = 1ULL << (sh - 1);
    const uint64_t up = (rem > half || (rem == half && (q & 1ULL))) ? 1ULL : 0ULL;
    return (q + up) << sh;
}

/* (double)s * 2^-63 for a state s below 2^63 */
XSGB_LCG_HD double xsgb_lcg_value(uint64_t s)
{
    const uint64_t r = xsgb_round53(s);
    if (r == 0) return 0.0;
    const int lz = xsgb_clz64(r);
    const uint64_t mant = (lz == 63) ? 0ULL : ((r << (lz + 1)) >> 12);
    const uint64_t bits = ((uint64_t)(1023 - lz) << 52) | mant;  /* exponent (63 - lz) - 63 */
#ifdef __CUDA_ARCH__
    return __longlong_as_double((long long)bits);
#else
    double d;
    memcpy(&d, &bits, 8);
    return d;
#endif
}

/* floor(xsgb_lcg_value(s) * 2^k), clamped to 2^k - 1 (k <= 31) */
XSGB_LCG_HD int xsgb_lcg_bucket(uint64_t s, int k)
{
    const uint64_t b = xsgb_round53(s) >> (63 - k);
    const uint64_t top = (1ULL << k) - 1ULL;
    return (int)(b < top ? b : top);
}

/* The smallest state s in [0, 2^63] whose draw is >= x, by bisection over the
 * monotone draw (host only; x in [0, 1]). */
XSGB_LCG_HOST uint64_t xsgb_lcg_threshold(double x)
{
    uint64_t lo = 0, hi = 1ULL << 63;   /* draw(hi) = 1.0 >= x */
    while (lo < hi) {
        const uint64_t mid = lo + (hi - lo) / 2;
        const double v = (mid == (1ULL << 63)) ? 1.0 : (double)mid * 0x1p-63;
        if (v >= x) hi = mid;
        else lo = mid + 1;
    }
    return lo;
}

#endif
