/* bin_bits.h -- energy bins of the unionized and hash grids in integer
 * arithmetic.
 *
 * Unionized grid: the bin floor(E * 2^k) of an energy in [0, 1) is exact in
 * integers (E's significand shifted by its exponent), so it needs none of the
 * FP64 pipe's multiply and conversion.
 *
 * Hash grid: the reference's bin is (long)(E / du) with du = 1.0 / bins, an
 * FP64 division (openmp-threading/Simulation.c:350-351).  E / du differs from
 * the exact E * bins by at most bins * 2^-52 (du carries one rounding, the
 * quotient another), so wherever E * bins lies farther than bins * 2^-50 from
 * an integer, the reference's bin is floor(E * bins), which is exact in
 * integers (a 53-bit significand times bins, shifted).  Closer to a bin edge
 * (a fraction of about 1e-11 of the energies for 10,000 bins) the caller
 * takes the division.
 *
 * Plain C (also compiled by the CPU tests); CUDA device code includes it
 * through device_common.cuh.
 */
#ifndef XSGB_BIN_BITS_H
#define XSGB_BIN_BITS_H

#include <stdint.h>
#include <string.h>

#ifdef __CUDACC__
#define XSGB_BIN_HD __host__ __device__ __forceinline__
#define XSGB_BIN_HOST __host__ static inline
#else
#define XSGB_BIN_HD static inline
#define XSGB_BIN_HOST static inline
#endif

XSGB_BIN_HD uint64_t xsgb_double_bits(double x)
{
#ifdef __CUDA_ARCH__
    return (uint64_t)__double_as_longlong(x);
#else
    uint64_t b;
    memcpy(&b, &x, 8);
    return b;
#endif
}

/* floor(E * 2^k) for E in [0, 1) (k <= 31) */
XSGB_BIN_HD int xsgb_floor_scaled_pow2(double E, int k)
{
    const uint64_t bits = xsgb_double_bits(E);
    const int ex = (int)((bits >> 52) & 0x7FF);
    if (ex == 0) return 0;                         /* zero or subnormal */
    const uint64_t m = (bits & ((1ULL << 52) - 1ULL)) | (1ULL << 52);
    const int sh = 1075 - ex - k;                  /* E * 2^k = m * 2^-sh, sh >= 53 - k */
    return sh >= 64 ? 0 : (int)(m >> sh);
}

/* bits [k, k + 64) of the 128-bit value (hi, lo), k >= 0 */
XSGB_BIN_HD uint64_t xsgb_shr128(uint64_t hi, uint64_t lo, int k)
{
    if (k >= 128) return 0;
    if (k >= 64) return hi >> (k - 64);
    if (k == 0) return lo;
    return (lo >> k) | (hi << (64 - k));
}

/* The hash grid's bin of E when it is certain without the division: returns
 * 1 and *bin = floor(E * bins) for E in (0, 1) whose E * bins lies at least
 * 2^-margin_bits from an integer; returns 0 otherwise (E outside (0, 1), NaN,
 * or near a bin edge).  margin_bits = 50 - ceil(log2(bins)), at least 1. */
XSGB_BIN_HD int xsgb_hash_bin(double E, uint32_t bins, int margin_bits, long *bin)
{
    const uint64_t bits = xsgb_double_bits(E);
    const int ex = (int)(bits >> 52);              /* sign bit included */
    if (ex == 0 || ex >= 1023) return 0;           /* zero, subnormal, >= 1, negative, NaN */
    const uint64_t m = (bits & ((1ULL << 52) - 1ULL)) | (1ULL << 52);
    uint64_t hi, lo;
#ifdef __CUDA_ARCH__
    hi = __umul64hi(m, (uint64_t)bins);
    lo = m * (uint64_t)bins;
#else
    const unsigned __int128 p = (unsigned __int128)m * bins;
    hi = (uint64_t)(p >> 64);
    lo = (uint64_t)p;
#endif
    const int sh = 1075 - ex;                      /* E * bins = (hi, lo) * 2^-sh, sh >= 53 */
    const uint64_t mask = (1ULL << margin_bits) - 1ULL;
    const uint64_t top = xsgb_shr128(hi, lo, sh - margin_bits) & mask;  /* leading fraction bits */
    if (top == 0 || top == mask) return 0;         /* within 2^-margin_bits of an integer */
    *bin = (long)xsgb_shr128(hi, lo, sh);
    return 1;
}

/* margin_bits for a hash grid of `bins` bins: 50 - ceil(log2(bins)) */
XSGB_BIN_HOST int xsgb_hash_margin_bits(long bins)
{
    int L = 0;
    while (L < 62 && (1L << L) < bins) L++;
    return L >= 49 ? 1 : 50 - L;
}

#endif
