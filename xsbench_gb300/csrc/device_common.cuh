// device_common.cuh -- per-lookup device code shared by the lookup kernels.
//
// One thread computes one macroscopic lookup (the body of the reference's
// event loop, openmp-threading/Simulation.c:62-110): sample, locate the energy
// in the acceleration structure, interpolate every nuclide of the material and
// accumulate in list order.  The kernels around it arrange for the 32 lanes of
// a warp to share the material, so the nuclide loop does not diverge.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "bin_bits.h"
#include "lcg_bits.h"
#include "xsgb_internal.h"

namespace xsgb {

// ------------------------------------------------------------------- LCG ---
// Simulation.c:462-499: x <- (a x + 1) mod 2^63, value x / 2^63.
constexpr unsigned long long kLcgMul = 2806196910506780709ULL;
constexpr unsigned long long kLcgMask = (1ULL << 63) - 1ULL;

__host__ __device__ __forceinline__ unsigned long long lcg_step(unsigned long long s)
{
    return (kLcgMul * s + 1ULL) & kLcgMask;
}

__host__ __device__ __forceinline__ double lcg_next(unsigned long long &s)
{
    s = lcg_step(s);
#ifdef __CUDA_ARCH__
    return xsgb_lcg_value(s);   // the same bits, on the integer pipe
#else
    return (double)s * 0x1p-63;
#endif
}

__host__ __device__ __forceinline__ unsigned long long lcg_skip(unsigned long long seed,
                                                                unsigned long long n)
{
    unsigned long long mul = kLcgMul, inc = 1ULL, am = 1ULL, ai = 0ULL;
    n &= kLcgMask;
    while (n) {
        if (n & 1ULL) {
            am *= mul;
            ai = ai * mul + inc;
        }
        inc *= (mul + 1ULL);
        mul *= mul;
        n >>= 1;
    }
    return (am * seed + ai) & kLcgMask;
}

// Simulation.c:426-460: the first material whose running sum exceeds the roll;
// the running sums are precomputed on the host in the reference's order, and
// `roll < sum` is compared as `state < mat_tseed` (the smallest state whose
// draw reaches the sum), which gives the same material without forming the roll.
__device__ __forceinline__ int pick_mat(const Tables &t, unsigned long long &s)
{
    s = lcg_step(s);
#pragma unroll
    for (int m = 1; m < kMaterials; m++)
        if (s < t.mat_tseed[m]) return m;
    return 0;
}

// ----------------------------------------------------------- order keys ---
// Signed 64-bit keys that order like the doubles they come from (-0 == +0).
__host__ __device__ __forceinline__ long long order_key(double x)
{
#ifdef __CUDA_ARCH__
    long long b = __double_as_longlong(x);
#else
    long long b;
    __builtin_memcpy(&b, &x, 8);
#endif
    if (b < 0) b = (b == (long long)0x8000000000000000ULL) ? 0 : (b ^ 0x7FFFFFFFFFFFFFFFLL);
    return b;
}

template <typename T>
__device__ __forceinline__ T ldg(const T *p)
{
    return __ldg(p);
}

// A material row entry: from shared memory (S, rows staged by the block) or
// through the read-only cache.
template <bool S, typename T>
__device__ __forceinline__ T rd(const T *p)
{
    if constexpr (S) return *p;
    else return __ldg(p);
}

// The materials' nuclide lists and concentrations staged in shared memory:
// material m's row is mats[off[m] .. off[m+1]), concs likewise.
struct SRows {
    const int *mats = nullptr;
    const double *concs = nullptr;
    const int *off = nullptr;
};

// Error reporting from checked kernels: first error wins.
__device__ __forceinline__ void report(int *err, int code, long a, long b)
{
    if (atomicCAS(err, 0, code) == 0) {
        err[1] = (int)a;
        err[2] = (int)b;
    }
}

// ------------------------------------------------------- union-grid row ---
// grid_search (Simulation.c:380-400) returns clamp(#{A <= E} - 1, 0, n - 2) on
// a sorted array; the accelerator narrows #{A <= E} to one bin of [0,1).
__device__ __forceinline__ long union_row(const Tables &t, double E)
{
    const long n = t.n_union;
    long c;
    const long long q = order_key(E);
    if (q >= 0 && q < 0x3FF0000000000000LL) {   // E in [0, 1) (-0 included, NaN not)
        const int b = xsgb_floor_scaled_pow2(E, t.union_bin_log2);   // floor(E * 2^k)
        long lo = ldg(&t.union_bins[b]), hi = ldg(&t.union_bins[b + 1]);
        while (lo < hi) {
            long mid = (lo + hi) >> 1;
            if (ldg(&t.union_keys[mid]) <= q) lo = mid + 1; else hi = mid;
        }
        c = lo;
    } else {
        // outside [0,1) or NaN: the reference loop with its own comparison
        long lo = 0, hi = n - 1;
        while (hi - lo > 1) {
            long mid = lo + (hi - lo) / 2;
            if (ldg(&t.union_e[mid]) > E) hi = mid; else lo = mid;
        }
        return lo;
    }
    c -= 1;
    if (c < 0) c = 0;
    if (c > n - 2) c = n - 2;
    return c;
}

// ------------------------------------------------ per-nuclide intervals ---
// Each returns the index k of the lower gridpoint, already clamped to
// [0, n_gp-2] the way calculate_micro_xs does it (Simulation.c:259-262,
// :268-271, :298-301).

// UNIONIZED (Simulation.c:264-272)
template <bool CHECKED>
__device__ __forceinline__ long interval_unionized(const Tables &t, long row, int nuc, int *err)
{
    long k = ldg(&t.index_grid[row * t.n_iso + nuc]);
    if (CHECKED && (k < 0 || k > t.n_gp - 1)) {
        report(err, XS_ERR_DATA, row, nuc);
        k = 0;
    }
    return (k == t.n_gp - 1) ? k - 1 : k;
}

// NUCLIDE (Simulation.c:252-263): clamp(#{E_j <= E} - 1, 0, n_gp-2), found in a
// coarse key array (every 16th energy) and then inside one 128-byte line.
__device__ __forceinline__ long interval_nuclide(const Tables &t, int nuc, long long q)
{
    const long long *ck = t.coarse + (long)nuc * t.n_coarse;
    long lo = 0, hi = t.n_coarse;
    while (lo < hi) {
        long mid = (lo + hi) >> 1;
        if (ldg(&ck[mid]) <= q) lo = mid + 1; else hi = mid;
    }
    long ub;
    if (lo == 0) {
        ub = 0;
    } else {
        const long long *k = t.ekeys + (long)nuc * t.n_gp;
        long a = (lo - 1) * kCoarseStride + 1;
        long b = lo * kCoarseStride;
        if (b > t.n_gp) b = t.n_gp;
        while (a < b) {
            long mid = (a + b) >> 1;
            if (ldg(&k[mid]) <= q) a = mid + 1; else b = mid;
        }
        ub = a;
    }
    long kk = ub - 1;
    if (kk < 0) kk = 0;
    if (kk > t.n_gp - 2) kk = t.n_gp - 2;
    return kk;
}

// Warp-cooperative form of the same count, for a batch whose warp holds
// lookups of one material within a narrow energy range (the batched kernel):
// #{ek[0..n) <= q} for a warp-uniform q by a 32-ary search (each round the 32
// lanes probe 32 evenly spaced keys and a ballot keeps one of the 32 pieces),
// 4 dependent loads for 238,847 keys instead of 18.  Every lane must call it.
__device__ __forceinline__ long warp_count_le(const long long *ek, long lo, long hi, long long q,
                                              int lane)
{
    // the count lies in [lo, hi]
    while (hi - lo > 32) {
        const long step = (hi - lo + 31) >> 5;
        const long p = lo + (long)(lane + 1) * step - 1;
        const bool le = p < hi && ldg(&ek[p]) <= q;
        const long c = __popc(__ballot_sync(0xffffffffu, le));
        const long nhi = lo + (c + 1) * step - 1;
        hi = nhi < hi ? nhi : hi;
        lo = lo + c * step;
    }
    const long p = lo + lane;
    const bool le = p < hi && ldg(&ek[p]) <= q;
    return lo + __popc(__ballot_sync(0xffffffffu, le));
}

// NUCLIDE interval of each lane's key q (live lanes' keys in [qmin, qmax],
// warp-uniform bounds): the count for qmin cooperatively, then the 32 keys
// from there held one per lane; when they cover qmax every lane finds its own
// count by binary lifting over the window with shuffles, otherwise by its own
// binary search past that count (no coarse keys: every grid type has ekeys).
// The same interval as interval_nuclide.
//
// bin_min >= 0 (hash grid): qmin's energy lies in hash bin bin_min, so its
// count lies between the bin's index entries (the warp-cooperative hash-bin
// search: one ballot over the bin's keys); -1: search all n keys.  `eq`
// returns whether the key below the count equals q (the hash edge rule).
__device__ __forceinline__ long interval_nuclide_warp(const Tables &t, int nuc, long long q,
                                                      long long qmin, long long qmax, int lane,
                                                      long bin_min, bool &eq)
{
    const long n = t.n_gp;
    const long long *ek = t.ekeys + (long)nuc * n;
    long lo = 0, hi = n;
    if (bin_min >= 0) {
        // u_low = clamp(#{E_j <= bin edge} - 1, 0, n - 2) <= the count; the count
        // is at most #{E_j <= next edge} = next entry + 1 unless that entry is clamped
        lo = ldg(&t.index_grid[bin_min * t.n_iso + nuc]);
        if (bin_min < t.hash_bins - 1) {
            const long nx = ldg(&t.index_grid[(bin_min + 1) * t.n_iso + nuc]);
            if (nx < n - 2) hi = nx + 1;
        }
    }
    const long c0 = warp_count_le(ek, lo, hi, qmin, lane);
    const long long below = c0 > 0 ? ldg(&ek[c0 - 1]) : (-0x7FFFFFFFFFFFFFFFLL - 1);
    const long wi = c0 + lane;
    const long long wkey = wi < n ? ldg(&ek[wi]) : 0x7FFFFFFFFFFFFFFFLL;
    const long long cap = c0 + 32 < n ? ldg(&ek[c0 + 32]) : 0x7FFFFFFFFFFFFFFFLL;
    long cnt;
    if (cap > qmax) {   // every live lane's count is in [c0, c0 + 32]
        int pos = 0;
#pragma unroll
        for (int step = 32; step >= 1; step >>= 1) {
            const int probe = pos + step;
            const long long key = __shfl_sync(0xffffffffu, wkey, (probe - 1) & 31);
            if (probe <= 32 && key <= q) pos = probe;
        }
        const long long kb = __shfl_sync(0xffffffffu, wkey, (pos - 1) & 31);
        eq = (pos > 0 ? kb : below) == q;
        cnt = c0 + pos;
    } else {   // the warp's energies span more than 32 keys: each lane searches past c0
        long a = c0, b = n;
        while (a < b) {
            const long mid = (a + b) >> 1;
            if (ldg(&ek[mid]) <= q) a = mid + 1; else b = mid;
        }
        cnt = a;
        eq = (cnt > c0 ? ldg(&ek[cnt - 1]) : below) == q;
    }
    long kk = cnt - 1;
    if (kk < 0) kk = 0;
    if (kk > n - 2) kk = n - 2;
    return kk;
}

// HASH (Simulation.c:273-302), including its edge rules: E <= e_low gives
// gridpoint 0, E >= e_high gives the last interval.
template <bool CHECKED>
__device__ __forceinline__ long interval_hash(const Tables &t, long bin, int nuc, long long q,
                                              int *err)
{
    const long n_gp = t.n_gp;
    long u_low = ldg(&t.index_grid[bin * t.n_iso + nuc]);
    long u_high = (bin == t.hash_bins - 1) ? n_gp - 1
                                           : (long)ldg(&t.index_grid[(bin + 1) * t.n_iso + nuc]) + 1;
    if (CHECKED && (u_low < 0 || u_low > n_gp - 1 || u_high < 0 || u_high > n_gp - 1)) {
        report(err, XS_ERR_DATA, bin, nuc);
        u_low = 0;
        u_high = n_gp - 1;
    }
    const long long *k = t.ekeys + (long)nuc * n_gp;
    long lower;
    if (q <= ldg(&k[u_low])) {
        lower = 0;
    } else if (q >= ldg(&k[u_high])) {
        lower = n_gp - 1;
    } else {
        long lo = u_low, hi = u_high;
        while (hi - lo > 1) {
            long mid = lo + (hi - lo) / 2;
            if (ldg(&k[mid]) > q) hi = mid; else lo = mid;
        }
        lower = lo;
    }
    return (lower == n_gp - 1) ? lower - 1 : lower;
}

// ------------------------------------------------------- L2 residency ---
// Records of the nuclides most lookups touch are loaded and prefetched with an
// evict_last policy so they stay in L2; the rest (the fuel-only nuclides'
// records, the index rows) are streamed with evict_first.
__device__ __forceinline__ unsigned long long policy_last()
{
    unsigned long long p;
    asm("createpolicy.fractional.L2::evict_last.b64 %0, 1.0;" : "=l"(p));
    return p;
}
__device__ __forceinline__ unsigned long long policy_first()
{
    unsigned long long p;
    asm("createpolicy.fractional.L2::evict_first.b64 %0, 1.0;" : "=l"(p));
    return p;
}
__device__ __forceinline__ bool is_hot(const Tables &t, int nuc)
{
    return nuc < 512 && ((t.hot[nuc >> 5] >> (nuc & 31)) & 1u);
}
__device__ __forceinline__ unsigned long long record_policy(const Tables &t, int nuc)
{
    return is_hot(t, nuc) ? policy_last() : policy_first();
}
// Policy of the L2 prefetch of a record that the lane reads one nuclide later:
// evict_last, so the line survives until that load, which reads it with
// record_policy (evict_first for the cold records) and so releases it
// (2.5 % less DRAM traffic than prefetching under record_policy).
__device__ __forceinline__ unsigned long long prefetch_policy(const Tables &, int)
{
    return policy_last();
}

// ------------------------------------------------------------- prefetch ---
// TMA bulk prefetch of [p, p+bytes) into L2 under an L2 policy; p 16-byte
// aligned, bytes a multiple of 16 (one instruction per 96-byte record or
// index-row span).
__device__ __forceinline__ void prefetch_l2(const void *p, unsigned bytes, unsigned long long pol)
{
    asm volatile("cp.async.bulk.prefetch.L2.global.L2::cache_hint [%0], %1, %2;" ::"l"(
                     __cvta_generic_to_global(p)),
                 "r"(bytes), "l"(pol)
                 : "memory");
}

// --------------------------------------------------------- interpolation ---
// 32-byte read-only load that does not allocate in L1 (the records are
// streamed; the material tables and index rows keep L1 to themselves).
__device__ __forceinline__ void ld_v4(const double *p, double &a, double &b, double &c, double &d,
                                      unsigned long long pol)
{
    asm volatile("ld.global.nc.L1::no_allocate.L2::cache_hint.v4.f64 {%0,%1,%2,%3}, [%4], %5;"
                 : "=d"(a), "=d"(b), "=d"(c), "=d"(d)
                 : "l"(p), "l"(pol));
}

// 16-byte streaming load (no L1 allocation) under an L2 policy.
__device__ __forceinline__ double2 ld_v2(const double2 *p, unsigned long long pol)
{
    double2 v;
    asm volatile("ld.global.nc.L1::no_allocate.L2::cache_hint.v2.f64 {%0,%1}, [%2], %3;"
                 : "=d"(v.x), "=d"(v.y)
                 : "l"(p), "l"(pol));
    return v;
}

// FAST: xs = hi - (E_hi - E) * slope from the 96-byte interval record (in its
// 128-byte slot), read
// with three 32-byte loads (a record is three aligned sectors).
template <bool DE = false>
__device__ __forceinline__ void accumulate_fast(const Tables &t, int nuc, long k, double E,
                                                double conc, double macro[5], double *S = nullptr)
{
    const double *r = reinterpret_cast<const double *>(t.records + ((long)nuc * (t.n_gp - 1) + k) * kRecordPairs);
    const unsigned long long pol = record_policy(t, nuc);
    double e_hi, h0, h1, h2, h3, h4, s0, s1, s2, s3, s4, e_lo;
    ld_v4(r, e_hi, h0, h1, h2, pol);
    ld_v4(r + 4, h3, h4, s0, s1, pol);
    ld_v4(r + 8, s2, s3, s4, e_lo, pol);
    (void)e_lo;
    const double d = e_hi - E;
    macro[0] = fma(fma(-d, s0, h0), conc, macro[0]);
    macro[1] = fma(fma(-d, s1, h1), conc, macro[1]);
    macro[2] = fma(fma(-d, s2, h2), conc, macro[2]);
    macro[3] = fma(fma(-d, s3, h3), conc, macro[3]);
    macro[4] = fma(fma(-d, s4, h4), conc, macro[4]);
    if (DE) {  // d macro / dE = sum over nuclides of conc * slope
        S[0] = fma(conc, s0, S[0]);
        S[1] = fma(conc, s1, S[1]);
        S[2] = fma(conc, s2, S[2]);
        S[3] = fma(conc, s3, S[3]);
        S[4] = fma(conc, s4, S[4]);
    }
}

// EXACT: the reference's operations in its order (Simulation.c:304-322,
// :372-373), no contraction, IEEE division.
__device__ __forceinline__ void accumulate_exact(const Tables &t, int nuc, long k, double E,
                                                 double conc, double macro[5])
{
    const double2 *g = reinterpret_cast<const double2 *>(t.grid + (long)nuc * t.n_gp + k);
    const double2 l0 = ldg(g + 0), l1 = ldg(g + 1), l2 = ldg(g + 2);
    const double2 h0 = ldg(g + 3), h1 = ldg(g + 4), h2 = ldg(g + 5);
    const double f = __ddiv_rn(__dsub_rn(h0.x, E), __dsub_rn(h0.x, l0.x));
    const double lo[5] = {l0.y, l1.x, l1.y, l2.x, l2.y};
    const double hi[5] = {h0.y, h1.x, h1.y, h2.x, h2.y};
#pragma unroll
    for (int c = 0; c < 5; c++) {
        double xs = __dsub_rn(hi[c], __dmul_rn(f, __dsub_rn(hi[c], lo[c])));
        macro[c] = __dadd_rn(macro[c], __dmul_rn(xs, conc));
    }
}

// Simulation.c:100-110
__device__ __forceinline__ int argmax5(const double m[5])
{
    double best = -1.0;
    int arg = 0;
#pragma unroll
    for (int c = 0; c < 5; c++)
        if (m[c] > best) {
            best = m[c];
            arg = c;
        }
    return arg;
}

// Address of the 96 bytes a lookup reads for interval k of nuclide nuc.
template <int ARITH>
__device__ __forceinline__ const void *interval_bytes(const Tables &t, int nuc, long k)
{
    if (ARITH == XS_ARITH_EXACT) return t.grid + (long)nuc * t.n_gp + k;
    return t.records + ((long)nuc * (t.n_gp - 1) + k) * kRecordPairs;
}

#ifndef XSGB_PIPE_P
#define XSGB_PIPE_P 1   // records prefetched this many nuclides ahead (unionized loop);
#endif                  // 2 and 3 measured 4 % and 14 % slower (records evicted before use)

// UNIONIZED nuclide loop, software-pipelined: the index entry of nuclide j+2P
// is loaded and the 96-byte interval of nuclide j+P is prefetched into L2 while
// nuclide j is interpolated, so a lane keeps three gathers in flight instead
// of waiting on each dependent pair.  The lane runs the nuclides
// j = q0, q0 + S, q0 + 2S, ... of the material (S = 1: all of them, in the
// reference's order).
//
// TABLE (FAST arithmetic, union table built): the lane reads its nuclides'
// entries of the row instead of index entries and interval records.
template <int ARITH, bool CHECKED, bool DE, bool TABLE = false, bool SROW = false>
__device__ __forceinline__ void macro_xs_unionized(const Tables &t, double E, int mat, int n,
                                                   const int *mrow, const double *crow,
                                                   double macro[5], int *err, double *S,
                                                   int q0 = 0, int stride = 1)
{
    const long row = union_row(t, E);
    if (TABLE) {
        // the material's entries of this row are contiguous, 80 bytes per
        // nuclide (five pairs (v, s)); xs = v + s * (E - u_row), the
        // interval's line evaluated at E
        const double dl = E - ldg(&t.union_e[row]);
        const double2 *blk = t.utab[mat] + row * n * 5;
        const unsigned long long pol = policy_first();
        if constexpr (DE) {
            // with the energy derivative: macro = sum conc * v + dl * S, where
            // S = sum conc * s is the derivative itself, so 10 FP64 operations
            // per nuclide instead of 15 (every |s * dl| is at most the
            // interval's rise, so the product adds no cancellation)
#pragma unroll 4
            for (int j = q0; j < n; j += stride) {
                const double2 *p = blk + (long)j * 5;
                const double2 a0 = ld_v2(p, pol), a1 = ld_v2(p + 1, pol), a2 = ld_v2(p + 2, pol);
                const double2 a3 = ld_v2(p + 3, pol), a4 = ld_v2(p + 4, pol);
                const double conc = rd<SROW>(&crow[j]);
                macro[0] = fma(conc, a0.x, macro[0]);
                macro[1] = fma(conc, a1.x, macro[1]);
                macro[2] = fma(conc, a2.x, macro[2]);
                macro[3] = fma(conc, a3.x, macro[3]);
                macro[4] = fma(conc, a4.x, macro[4]);
                S[0] = fma(conc, a0.y, S[0]);
                S[1] = fma(conc, a1.y, S[1]);
                S[2] = fma(conc, a2.y, S[2]);
                S[3] = fma(conc, a3.y, S[3]);
                S[4] = fma(conc, a4.y, S[4]);
            }
#pragma unroll
            for (int k = 0; k < 5; k++) macro[k] = fma(dl, S[k], macro[k]);
        } else {
#pragma unroll 4
        for (int j = q0; j < n; j += stride) {
            const double2 *p = blk + (long)j * 5;
            const double2 a0 = ld_v2(p, pol), a1 = ld_v2(p + 1, pol), a2 = ld_v2(p + 2, pol);
            const double2 a3 = ld_v2(p + 3, pol), a4 = ld_v2(p + 4, pol);
            const double conc = rd<SROW>(&crow[j]);
            macro[0] = fma(fma(a0.y, dl, a0.x), conc, macro[0]);
            macro[1] = fma(fma(a1.y, dl, a1.x), conc, macro[1]);
            macro[2] = fma(fma(a2.y, dl, a2.x), conc, macro[2]);
            macro[3] = fma(fma(a3.y, dl, a3.x), conc, macro[3]);
            macro[4] = fma(fma(a4.y, dl, a4.x), conc, macro[4]);
        }
        }
        return;
    }
    constexpr int P = XSGB_PIPE_P;
    const int *irow = t.index_grid + row * t.n_iso;
    if (q0 == 0) {
        // the material's span of the index row, 16-byte aligned
        const uintptr_t a = (uintptr_t)(irow + t.mat_lo[mat]) & ~(uintptr_t)15;
        const uintptr_t b = ((uintptr_t)(irow + t.mat_hi[mat] + 1) + 15) & ~(uintptr_t)15;
        prefetch_l2((const void *)a, (unsigned)(b - a), policy_first());
    }
    // this lane's nuclides: positions q0 + stride * i, i < nl
    const int nl = n > q0 ? (n - q0 + stride - 1) / stride : 0;
    mrow += q0;
    crow += q0;
    const long top = t.n_gp - 1;
    int kr[2 * P];
#pragma unroll
    for (int q = 0; q < 2 * P; q++) kr[q] = (q < nl) ? ldg(&irow[rd<SROW>(&mrow[q * stride])]) : 0;
#pragma unroll
    for (int q = 0; q < P; q++)
        if (q < nl) {
            long k = kr[q];
            if (CHECKED && (k < 0 || k > top)) k = 0;
            const int nq = rd<SROW>(&mrow[q * stride]);
            prefetch_l2(interval_bytes<ARITH>(t, nq, k == top ? k - 1 : k), 96, prefetch_policy(t, nq));
        }
    for (int j0 = 0; j0 < nl; j0 += 2 * P) {
#pragma unroll
        for (int q = 0; q < 2 * P; q++) {
            const int j = j0 + q;
            if (j < nl) {
                long k = kr[q];
                if (CHECKED && (k < 0 || k > top)) {
                    report(err, XS_ERR_DATA, row, rd<SROW>(&mrow[j * stride]));
                    k = 0;
                }
                if (k == top) k -= 1;
                const int jn = j + 2 * P;
                if (jn < nl) kr[q] = ldg(&irow[rd<SROW>(&mrow[jn * stride])]);
                const int jp = j + P;
                if (jp < nl) {
                    long kp = kr[(q + P) % (2 * P)];
                    if (CHECKED && (kp < 0 || kp > top)) kp = 0;
                    const int np = rd<SROW>(&mrow[jp * stride]);
                    prefetch_l2(interval_bytes<ARITH>(t, np, kp == top ? kp - 1 : kp), 96,
                                prefetch_policy(t, np));
                }
                const int nuc = rd<SROW>(&mrow[j * stride]);
                const double conc = rd<SROW>(&crow[j * stride]);
                if (ARITH == XS_ARITH_EXACT)
                    accumulate_exact(t, nuc, k, E, conc, macro);
                else
                    accumulate_fast<DE>(t, nuc, k, E, conc, macro, S);
            }
        }
    }
}

// NUCLIDE (or HASH) lookup of one warp of a batch (every lane calls; `live`
// lanes accumulate; qmin / qmax bound the live lanes' keys, warp-uniform; no
// NaN).  The cooperative search gives the bracketing interval.  The hash
// lookup (Simulation.c:273-301) gives the same interval whenever E lies in
// its bin, [bin*du, (bin+1)*du), except by its edge rule E <= E[u_low] ->
// gridpoint 0, which then holds only when E equals a gridpoint: that case
// loads u_low and applies the rule.  A lookup whose E / du rounded it into a
// neighbouring bin (E within an ulp of a bin edge) takes the hash search
// itself (interval_hash) for every nuclide.
template <int ARITH, bool CHECKED, bool HASHQ = false>
__device__ __forceinline__ void macro_xs_nuclide_warp(const Tables &t, double E, int mat, bool live,
                                                      long long qmin, long long qmax,
                                                      double macro[5], int *err)
{
#pragma unroll
    for (int c = 0; c < 5; c++) macro[c] = 0.0;
    const int n = ldg(&t.num_nucs[mat]);
    const int *mrow = t.mats + mat * t.max_nucs;
    const double *crow = t.concs + mat * t.max_nucs;
    const long long q = order_key(E);
    const int lane = threadIdx.x & 31;
    long bin = 0, bin_min = -1;
    bool outside = false;   // E not in [bin*du, (bin+1)*du)
    if (HASHQ) {
        // Simulation.c:350-351; away from bin edges the bin is exact in
        // integers, and E then lies inside it
        if (!xsgb_hash_bin(E, (uint32_t)t.hash_bins, t.hash_margin, &bin)) {
            bin = (long)(E / t.hash_du);
            if (bin < 0) bin = 0;
            if (bin > t.hash_bins - 1) bin = t.hash_bins - 1;
            outside = (double)bin * t.hash_du > E ||
                      (bin < t.hash_bins - 1 && (double)(bin + 1) * t.hash_du <= E);
        }
        // the bin of the warp's lowest live energy, when that energy lies in it
        const bool is_min = live && q == qmin;
        const unsigned owners = __ballot_sync(0xffffffffu, is_min);
        const int src = __ffs(owners) - 1;
        const long b0 = __shfl_sync(0xffffffffu, bin, src < 0 ? 0 : src);
        const bool out0 = __shfl_sync(0xffffffffu, outside, src < 0 ? 0 : src);
        bin_min = (src >= 0 && !out0) ? b0 : -1;
    }
    for (int j = 0; j < n; j++) {
        const int nuc = ldg(&mrow[j]);
        const double conc = ldg(&crow[j]);
        bool eq = false;
        long k = interval_nuclide_warp(t, nuc, q, qmin, qmax, lane, bin_min, eq);
        if (HASHQ && live) {
            if (outside) {
                k = interval_hash<false>(t, bin, nuc, q, err);
            } else if (eq && k > 0) {
                const long ul = ldg(&t.index_grid[bin * t.n_iso + nuc]);
                if (q <= ldg(&t.ekeys[(long)nuc * t.n_gp + ul])) k = 0;
            }
        }
        if (live) {
            if (ARITH == XS_ARITH_EXACT)
                accumulate_exact(t, nuc, k, E, conc, macro);
            else
                accumulate_fast<false>(t, nuc, k, E, conc, macro, nullptr);
        }
    }
}

// ------------------------------------------------- guided interval search ---
// The hash and nuclide grids both give nuclide nuc the interval
// k = clamp(#{E_j <= E} - 1, 0, n_gp - 2) (Simulation.c:252-263; the hash grid's
// exceptions are below).  The guide (Tables::guide) holds
// g = #{E_j < b 2^-K} for the bin b = floor(E 2^K) of E, so the interval is
// k = clamp(g - 1 + #{j >= g : E_j <= E}, 0, n_gp - 2); with about four bins
// per gridpoint most bins hold no gridpoint and the count is 0.  The lookup
// starts at k = clamp(g - 1, 0, n_gp - 2) -- E_k < b 2^-K <= E, so k is not
// past the interval -- reads interval k's 96 bytes (FAST: its record; EXACT:
// its two gridpoints), whose upper energy says whether E lies below it, and
// steps up while E >= E_{k+1}: one guide entry and, for ~90 % of the
// nuclides, one interval read, where a binary search makes ~14-18 dependent
// reads.
//
// HASH (Simulation.c:273-302): for E strictly inside its hash bin
// (xsgb_hash_bin certain, i.e. more than 2^-50 from both edges) the
// reference's search gives the same k except by its edge rule
// `E <= E[u_low] -> gridpoint 0`, which can then hold only if E equals a
// gridpoint (the lower gridpoint of the interval found, E_k == E); that case
// takes the reference's hash search (interval_hash).  E_high's rule
// `E >= E[u_high] -> n_gp - 1` holds only when u_high = n_gp - 1, where the
// clamp gives the same interval.
//
// Loads: the guide entries through L1-bypassing evict_first loads (the guide
// of the XL grid is 1.5 GB, read at random); the interval through the same
// loads and L2 policy as accumulate_fast / accumulate_exact.

__device__ __forceinline__ int ld_guide(const int *p)
{
    int v;
    asm volatile("ld.global.nc.L1::no_allocate.L2::cache_hint.b32 %0, [%1], %2;"
                 : "=r"(v)
                 : "l"(p), "l"(policy_first()));
    return v;
}

// The 96 bytes of interval k: FAST, the record [E_hi, hi[5], slope[5], E_lo];
// EXACT, the gridpoints k and k+1 [E_lo, lo[5], E_hi, hi[5]].
template <int ARITH>
__device__ __forceinline__ void load_interval(const Tables &t, int nuc, long k, double v[12])
{
    if (ARITH == XS_ARITH_EXACT) {
        const double2 *g = reinterpret_cast<const double2 *>(t.grid + (long)nuc * t.n_gp + k);
#pragma unroll
        for (int i = 0; i < 6; i++) {
            const double2 x = ldg(g + i);
            v[2 * i] = x.x;
            v[2 * i + 1] = x.y;
        }
    } else {
        const double *r = reinterpret_cast<const double *>(t.records + ((long)nuc * (t.n_gp - 1) + k) * kRecordPairs);
        const unsigned long long pol = record_policy(t, nuc);
        ld_v4(r, v[0], v[1], v[2], v[3], pol);
        ld_v4(r + 4, v[4], v[5], v[6], v[7], pol);
        ld_v4(r + 8, v[8], v[9], v[10], v[11], pol);
    }
}

template <int ARITH>
__device__ __forceinline__ double interval_e_hi(const double v[12])
{
    return ARITH == XS_ARITH_EXACT ? v[6] : v[0];
}

template <int ARITH>
__device__ __forceinline__ double interval_e_lo(const double v[12])
{
    return ARITH == XS_ARITH_EXACT ? v[0] : v[11];
}

// accumulate_fast / accumulate_exact on an interval already loaded
template <int ARITH, bool DE>
__device__ __forceinline__ void accumulate_loaded(const double v[12], double E, double conc,
                                                  double macro[5], double *S)
{
    if (ARITH == XS_ARITH_EXACT) {
        const double f = __ddiv_rn(__dsub_rn(v[6], E), __dsub_rn(v[6], v[0]));
#pragma unroll
        for (int c = 0; c < 5; c++) {
            double xs = __dsub_rn(v[7 + c], __dmul_rn(f, __dsub_rn(v[7 + c], v[1 + c])));
            macro[c] = __dadd_rn(macro[c], __dmul_rn(xs, conc));
        }
    } else {
        const double d = v[0] - E;
#pragma unroll
        for (int c = 0; c < 5; c++) macro[c] = fma(fma(-d, v[6 + c], v[1 + c]), conc, macro[c]);
        if (DE) {
#pragma unroll
            for (int c = 0; c < 5; c++) S[c] = fma(conc, v[6 + c], S[c]);
        }
    }
}

// The lane's nuclides j = q0, q0 + stride, ... of the material through the
// guide, software-pipelined like the unionized loop: the guide entry of
// nuclide j+2 is loaded and interval j+1's first guess prefetched into L2
// while nuclide j is interpolated.  Returns false, touching nothing, when E
// is not eligible (outside [0, 1), NaN, or for HASH within 2^-50 of a hash bin
// edge); the caller then runs its own search.
template <int GRID, int ARITH, bool CHECKED, bool DE, bool SROW>
__device__ __forceinline__ bool macro_xs_guided(const Tables &t, double E, int n, const int *mrow,
                                                const double *crow, double macro[5], int *err,
                                                double *S, int q0, int stride)
{
    const long long q = order_key(E);
    if (!(q >= 0 && q < 0x3FF0000000000000LL)) return false;   // E in [0, 1)
    long bin = 0;
    if (GRID == XS_HASH && !xsgb_hash_bin(E, (uint32_t)t.hash_bins, t.hash_margin, &bin)) return false;
    const int b = xsgb_floor_scaled_pow2(E, t.guide_log2);
    const long gstride = (1L << t.guide_log2) + 1;
    const int *gcol = t.guide + b;
    const long top = t.n_gp - 2;
    const int nl = n > q0 ? (n - q0 + stride - 1) / stride : 0;
    mrow += q0;
    crow += q0;
    int gr[2];
#pragma unroll
    for (int i = 0; i < 2; i++) gr[i] = (i < nl) ? ld_guide(&gcol[(long)rd<SROW>(&mrow[i * stride]) * gstride]) : 0;
    if (nl > 0) {
        const long k0 = min(max((long)gr[0] - 1, 0L), top);
        const int n0 = rd<SROW>(&mrow[0]);
        prefetch_l2(interval_bytes<ARITH>(t, n0, k0), 96, prefetch_policy(t, n0));
    }
    for (int j0 = 0; j0 < nl; j0 += 2) {
#pragma unroll
        for (int i = 0; i < 2; i++) {
            const int j = j0 + i;
            if (j < nl) {
                long k = min(max((long)gr[i] - 1, 0L), top);
                if (j + 2 < nl) gr[i] = ld_guide(&gcol[(long)rd<SROW>(&mrow[(j + 2) * stride]) * gstride]);
                if (j + 1 < nl) {
                    const long kp = min(max((long)gr[i ^ 1] - 1, 0L), top);
                    const int np = rd<SROW>(&mrow[(j + 1) * stride]);
                    prefetch_l2(interval_bytes<ARITH>(t, np, kp), 96, prefetch_policy(t, np));
                }
                const int nuc = rd<SROW>(&mrow[j * stride]);
                const double conc = rd<SROW>(&crow[j * stride]);
                double v[12];
                load_interval<ARITH>(t, nuc, k, v);
                while (k < top && !(E < interval_e_hi<ARITH>(v))) {
                    k++;
                    load_interval<ARITH>(t, nuc, k, v);
                }
                if (GRID == XS_HASH && interval_e_lo<ARITH>(v) == E) {
                    // E on a gridpoint: the reference's own hash search and edge rule
                    const long kh = interval_hash<CHECKED>(t, bin, nuc, q, err);
                    if (kh != k) {
                        k = kh;
                        load_interval<ARITH>(t, nuc, k, v);
                    }
                }
                accumulate_loaded<ARITH, DE>(v, E, conc, macro, S);
            }
        }
    }
    return true;
}

// The same intervals through the bin records (Tables::binrec, FAST): slot
// (nuc, b) already holds the record of the interval the guided search starts
// at, so the lane reads it at an address it knows without a load -- no
// dependent read precedes the record -- and walks on from that interval's
// index (kept in the slot's fourth sector) only when E lies at or past its
// upper gridpoint (about one nuclide in ten with four bins per gridpoint).  The bin records of the nuclides
// t.bin_prefetch ahead are prefetched into L2.
__device__ __forceinline__ const double *binrec_at(const Tables &t, int nuc, int b)
{
    return reinterpret_cast<const double *>(t.binrec + (((long)nuc << t.guide_log2) + b) * kRecordPairs);
}

template <int GRID, bool CHECKED, bool DE, bool SROW>
__device__ __forceinline__ bool macro_xs_binned(const Tables &t, double E, int n, const int *mrow,
                                                const double *crow, double macro[5], int *err,
                                                double *S, int q0, int stride)
{
    const long long q = order_key(E);
    if (!(q >= 0 && q < 0x3FF0000000000000LL)) return false;   // E in [0, 1)
    long bin = 0;
    if (GRID == XS_HASH && !xsgb_hash_bin(E, (uint32_t)t.hash_bins, t.hash_margin, &bin)) return false;
    const int b = xsgb_floor_scaled_pow2(E, t.guide_log2);
    const long top = t.n_gp - 2;
    const int nl = n > q0 ? (n - q0 + stride - 1) / stride : 0;
    mrow += q0;
    crow += q0;
    const int P = t.bin_prefetch;
    const unsigned long long pol = policy_first();
    for (int j = 0; j < P && j < nl; j++)
        prefetch_l2(binrec_at(t, rd<SROW>(&mrow[j * stride]), b), 96, policy_last());
#pragma unroll 2
    for (int j = 0; j < nl; j++) {
        if (j + P < nl) prefetch_l2(binrec_at(t, rd<SROW>(&mrow[(j + P) * stride]), b), 96, policy_last());
        const int nuc = rd<SROW>(&mrow[j * stride]);
        const double conc = rd<SROW>(&crow[j * stride]);
        const double *r = binrec_at(t, nuc, b);
        double v[12];
        ld_v4(r, v[0], v[1], v[2], v[3], pol);
        ld_v4(r + 4, v[4], v[5], v[6], v[7], pol);
        ld_v4(r + 8, v[8], v[9], v[10], v[11], pol);
        if (!(E < v[0])) {
            // E at or past the bin's first interval: walk on from its index,
            // kept in the slot's fourth sector (same 128-byte line)
            long k = (long)ldg(reinterpret_cast<const long long *>(r + 12));
            while (k < top && !(E < v[0])) {
                k++;
                load_interval<XS_ARITH_FAST>(t, nuc, k, v);
            }
        }
        if (GRID == XS_HASH && v[11] == E) {
            // E on a gridpoint: the reference's own hash search and edge rule
            load_interval<XS_ARITH_FAST>(t, nuc, interval_hash<CHECKED>(t, bin, nuc, q, err), v);
        }
        accumulate_loaded<XS_ARITH_FAST, DE>(v, E, conc, macro, S);
    }
    return true;
}

// ------------------------------------------------------------ one lookup ---
// calculate_macro_xs (Simulation.c:326-375) for one (E, mat).
// With DE, S[5] receives d macro_xs / dE (the adjoint's energy derivative).
// With stride > 1 the call computes the partial sum over the nuclides
// j = q0, q0 + stride, ... only (one of `stride` lanes sharing the lookup).
//
// SROW: the material's row is read from the block's staged copy `sr`.
template <int GRID, int ARITH, bool CHECKED, bool DE = false, bool TABLE = false, bool SROW = false>
__device__ __forceinline__ void macro_xs(const Tables &t, double E, int mat, double macro[5],
                                         int *err, double *S = nullptr, int q0 = 0,
                                         int stride = 1, SRows sr = SRows())
{
#pragma unroll
    for (int c = 0; c < 5; c++) macro[c] = 0.0;
    if (DE) {
#pragma unroll
        for (int c = 0; c < 5; c++) S[c] = 0.0;
    }
    int n;
    const int *mrow;
    const double *crow;
    if constexpr (SROW) {
        const int o = sr.off[mat];
        n = sr.off[mat + 1] - o;
        mrow = sr.mats + o;
        crow = sr.concs + o;
    } else {
        n = ldg(&t.num_nucs[mat]);
        mrow = t.mats + mat * t.max_nucs;
        crow = t.concs + mat * t.max_nucs;
    }
    if (GRID == XS_UNIONIZED) {
        macro_xs_unionized<ARITH, CHECKED, DE, TABLE, SROW>(t, E, mat, n, mrow, crow, macro, err,
                                                            S, q0, stride);
        return;
    }
    if (ARITH == XS_ARITH_FAST && t.binrec &&
        macro_xs_binned<GRID, CHECKED, DE, SROW>(t, E, n, mrow, crow, macro, err, S, q0, stride))
        return;
    // (FAST arithmetic without bin records -- a device short of memory for
    // them -- keeps the grid's own search: one register set less in the
    // FAST kernels)
    if (ARITH == XS_ARITH_EXACT && t.guide &&
        macro_xs_guided<GRID, ARITH, CHECKED, DE, SROW>(t, E, n, mrow, crow, macro, err, S, q0,
                                                        stride))
        return;
    long row = 0;
    long long q = 0;
    const bool keyed = !(E != E);   // NaN energies use the double-compare path
    if (GRID == XS_UNIONIZED) {
        row = union_row(t, E);
    } else if (GRID == XS_HASH) {
        // Simulation.c:350-351 (away from bin edges exact in integers)
        if (!xsgb_hash_bin(E, (uint32_t)t.hash_bins, t.hash_margin, &row)) {
            row = (long)(E / t.hash_du);
            if (row < 0 || row > t.hash_bins - 1) {
                // the reference reads outside its table here; clamp instead
                if (CHECKED) report(err, XS_ERR_DATA, row, -1);
                row = row < 0 ? 0 : t.hash_bins - 1;
            }
        }
        q = order_key(E);
    } else {
        q = order_key(E);
    }
#pragma unroll 2
    for (int j = q0; j < n; j += stride) {
        const int nuc = rd<SROW>(&mrow[j]);
        const double conc = rd<SROW>(&crow[j]);
        long k;
        if (GRID == XS_UNIONIZED) {
            k = interval_unionized<CHECKED>(t, row, nuc, err);
        } else if (GRID == XS_NUCLIDE) {
            if (keyed) {
                k = interval_nuclide(t, nuc, q);
            } else {
                k = t.n_gp - 2;  // NaN compares false: the search ends at the top
            }
        } else {
            if (keyed) {
                k = interval_hash<CHECKED>(t, row, nuc, q, err);
            } else {
                long u_high = (row == t.hash_bins - 1)
                                  ? t.n_gp - 1
                                  : (long)ldg(&t.index_grid[(row + 1) * t.n_iso + nuc]) + 1;
                k = u_high - 1;
                if (k < 0) k = 0;
                if (k > t.n_gp - 2) k = t.n_gp - 2;
            }
        }
        if (ARITH == XS_ARITH_EXACT)
            accumulate_exact(t, nuc, k, E, conc, macro);
        else
            accumulate_fast<DE>(t, nuc, k, E, conc, macro, S);
    }
}

}  // namespace xsgb
