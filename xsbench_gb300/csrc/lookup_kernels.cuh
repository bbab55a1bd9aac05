// lookup_kernels.cuh -- the lookup kernels, templated on grid type and
// arithmetic.  Instantiated once per grid type (lookup_<grid>.cu) so the
// three translation units compile in parallel.
#pragma once

#include "device_common.cuh"

namespace xsgb {

constexpr int kBlock = 256;          // threads per block of the lookup kernels (the plain and
                                     // list kernels also come in 128 and 512; the tuner picks)
constexpr int kWarps = kBlock / 32;
#ifndef XSGB_PLAIN_MIN_BLOCKS
#define XSGB_PLAIN_MIN_BLOCKS 4      // resident blocks per SM the compiler must allow
#endif


// Arguments of the plain (tiled) lookup kernel.
struct PlainArgs {
    long first, count;
    int tile;
    const double *in_E;          // caller samples, or null: in-kernel LCG sampling
    const int *in_mat;
    double *out_macro;           // count*5 or null
    unsigned char *out_idx;      // count or null
    unsigned long long *verif;
    int *err;
    // overflow queues: each block runs only whole 32-lookup chunks and appends
    // the rest of each material (< 32 lookups) here; null: run them padded
    int *ovf_cnt;                // [12]
    double *ovf_E;               // [12 * ovf_cap]
    int *ovf_id;                 // [12 * ovf_cap]
    int ovf_cap;                 // entries per material
    // lanes per fuel (material 0) lookup: 1, or with FAST arithmetic 2 or 4,
    // each lane summing every fuel_lanes-th nuclide (the partial sums are
    // added in a fixed tree), so a fuel chunk is 32 / fuel_lanes lookups and
    // the block's warps finish their tile together
    int fuel_lanes;
    // 1: the block stages every material's nuclide list and concentrations
    // (rows_total entries in all) in shared memory
    int stage_rows;
    int rows_total;
    int block;                   // threads per block: 128, 256 or 512 (tile a multiple of it)
    // 1: within each material the tile's lookups are also ordered by energy
    // (kTileBuckets buckets over [0, 1)), so a warp's lookups lie in a narrow
    // energy window and its loads of a nuclide's table touch few pages
    int esort;
};

constexpr int kTileBucketsLog2 = 6;
constexpr int kTileBuckets = 1 << kTileBucketsLog2;   // energy buckets of the in-tile sort

// Energy bucket of the in-tile sort: floor(E * kTileBuckets) on [0, 1), the
// end buckets outside it (NaN: 0).
__device__ __forceinline__ int tile_bucket(double E)
{
    if (E >= 0.0 && E < 1.0) return xsgb_floor_scaled_pow2(E, kTileBucketsLog2);
    return E >= 1.0 ? kTileBuckets - 1 : 0;
}

// A material-segmented list of lookups (the batched sort, or the plain
// kernel's overflow).  Chunk c covers virtual positions [32c, 32c+32); the
// chunk's material m satisfies seg_v[m] <= 32c < seg_v[m+1] (each seg_v a
// multiple of 32); entry p_v of material m sits at base[m] + (p_v - seg_v[m])
// (base null: at p_v) and exists when p_v < seg_v[m] + cnt[m].
struct ListArgs {
    const int *seg_v;            // [13]
    const int *cnt;              // [12]
    const int *base;             // [12] or null
    const double *E;
    const int *id;
    unsigned int *queue;
    double *out_macro;
    unsigned char *out_idx;
    unsigned long long *verif;
    int *err;
    int fuel_lanes;              // lanes per fuel lookup (PlainArgs::fuel_lanes)
    int table;                   // 1: read the union table when there is one (FAST)
    int sorted;                  // 1: entries sorted by energy bucket (warp searches pay)
    int block;                   // threads per block of the persistent kernel: 128, 256 or 512
};

// Adds the per-lane verification counts of a block into *verif (one atomic).
__device__ __forceinline__ void block_verification(unsigned long long mine,
                                                   unsigned long long *s_acc,
                                                   unsigned long long *verif)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) mine += __shfl_xor_sync(0xffffffffu, mine, o);
    if ((threadIdx.x & 31) == 0 && mine) atomicAdd(s_acc, mine);
    __syncthreads();
    if (threadIdx.x == 0 && *s_acc) atomicAdd(verif, *s_acc);
}

// Event sample of a lookup: either the caller's arrays or the reference LCG
// (Simulation.c:62-70).  Returns false for a material outside 0..11.
template <bool SAMPLES>
__device__ __forceinline__ bool sample_at(const Tables &t, const double *in_E, const int *in_mat,
                                          long i, unsigned long long &seed, double &E, int &m,
                                          int *err)
{
    if (SAMPLES) {
        E = ldg(&in_E[i]);
        m = ldg(&in_mat[i]);
        if (m < 0 || m >= kMaterials) {
            report(err, XS_ERR_DATA, i, m);
            return false;
        }
        return true;
    } else {
        E = lcg_next(seed);
        m = pick_mat(t, seed);
        return true;
    }
}

// A lookup's outputs, written with the streaming (evict-first) store: they
// are not read again by the kernel, and the sorted lists of the batched form
// write them at scattered addresses.
__device__ __forceinline__ void store_result(double *out_macro, unsigned char *out_idx, long o,
                                             const double macro[5], int arg)
{
    if (out_macro) {
#pragma unroll
        for (int k = 0; k < 5; k++) __stcs(&out_macro[o * 5 + k], macro[k]);
    }
    if (out_idx) __stcs(reinterpret_cast<signed char *>(&out_idx[o]), (signed char)arg);
}

// One lookup of the event batch: macro_xs, argmax, outputs.
template <int GRID, int ARITH, bool CHECKED, bool TABLE, bool SROW = false>
__device__ __forceinline__ unsigned lookup_and_store(const Tables &t, double E, int m, long o,
                                                     double *out_macro, unsigned char *out_idx,
                                                     int *err, SRows sr = SRows())
{
    double macro[5];
    macro_xs<GRID, ARITH, CHECKED, false, TABLE, SROW>(t, E, m, macro, err, nullptr, 0, 1, sr);
    const int arg = argmax5(macro);
    store_result(out_macro, out_idx, o, macro, arg);
    return (unsigned)(arg + 1);
}

// One lookup of material m (the fuel, or a tile's partial chunk) spread over
// L lanes, FAST arithmetic: lane q sums the nuclides j = q, q + L, ...; the
// partial sums are added in the fixed tree (q0 + q1) + (q2 + q3), which gives
// the same bits on every lane of the lookup.  Every lane of the warp calls
// this (shuffles); `live` is the same on the L lanes of a lookup.  Returns
// argmax+1 on the lookup's lane q == 0.
template <int GRID, bool CHECKED, bool TABLE, bool SROW = false>
__device__ __forceinline__ unsigned split_lookup_and_store(const Tables &t, bool live, double E,
                                                           long o, int q, int L,
                                                           double *out_macro,
                                                           unsigned char *out_idx, int *err,
                                                           SRows sr = SRows(), int m = 0)
{
    double macro[5] = {0.0, 0.0, 0.0, 0.0, 0.0};
    if (live)
        macro_xs<GRID, XS_ARITH_FAST, CHECKED, false, TABLE, SROW>(t, E, m, macro, err, nullptr, q,
                                                                   L, sr);
    for (int s = 1; s < L; s <<= 1) {
#pragma unroll
        for (int k = 0; k < 5; k++) macro[k] += __shfl_xor_sync(0xffffffffu, macro[k], s);
    }
    if (!live || q != 0) return 0;
    const int arg = argmax5(macro);
    store_result(out_macro, out_idx, o, macro, arg);
    return (unsigned)(arg + 1);
}

// A warp's 32 entries of one material on the NUCLIDE or HASH grid, sorted by
// energy bucket: the warp-cooperative interval search (macro_xs_nuclide_warp)
// when no live energy is NaN, else each lane's own lookup.  Every lane calls
// this.
template <int GRID, int ARITH, bool CHECKED>
__device__ __forceinline__ unsigned nuclide_warp_lookup_and_store(const Tables &t, bool live,
                                                                  double E, int m, long o,
                                                                  double *out_macro,
                                                                  unsigned char *out_idx,
                                                                  int *err)
{
    const unsigned full = 0xffffffffu;
    const bool keyed = !(E != E);
    if (!__any_sync(full, live)) return 0;
    if (!__all_sync(full, !live || keyed)) {
        if (!live) return 0;
        return lookup_and_store<GRID, ARITH, CHECKED, false>(t, E, m, o, out_macro, out_idx, err);
    }
    const long long q = order_key(E);
    long long qmin = live ? q : 0x7FFFFFFFFFFFFFFFLL, qmax = live ? q : (-0x7FFFFFFFFFFFFFFFLL - 1);
#pragma unroll
    for (int s = 16; s > 0; s >>= 1) {
        const long long a = __shfl_xor_sync(full, qmin, s), b = __shfl_xor_sync(full, qmax, s);
        qmin = a < qmin ? a : qmin;
        qmax = b > qmax ? b : qmax;
    }
    double macro[5];
    macro_xs_nuclide_warp<ARITH, CHECKED, GRID == XS_HASH>(t, E, m, live, qmin, qmax, macro, err);
    if (!live) return 0;
    const int arg = argmax5(macro);
    store_result(out_macro, out_idx, o, macro, arg);
    return (unsigned)(arg + 1);
}

// ---------------------------------------------------------------- PLAIN ---
// One block = one tile of `tile` consecutive lookups.  The block samples them,
// counting-sorts their ids by material in shared memory, then its warps pull
// chunks, fuel first, from a shared-memory queue, so a warp never mixes
// materials: a chunk of another material is 32 lookups, one per lane; a fuel
// chunk is 32 / fuel_lanes lookups with fuel_lanes lanes each.  With overflow
// queues the last, partial 32 lookups of every material go to the queue
// instead of running with idle lanes.
//
// The plain kernel reads index entries and interval records, never the union
// table: its lookups are in random energy order, so each lane would stream a
// different row of a table of ~155 GB, and the page-translation misses of that
// pattern cost more than the bytes it saves (the batched kernel, whose warps
// read neighbouring rows, uses it).
template <int GRID, int ARITH, bool CHECKED, bool SAMPLES, bool SROW = false, int BLOCK = kBlock>
__global__ void __launch_bounds__(BLOCK, XSGB_PLAIN_MIN_BLOCKS * kBlock / BLOCK) k_plain(Tables t, PlainArgs a)
{
    extern __shared__ __align__(16) unsigned char smem[];
    const int tile = a.tile;
    double *sE = reinterpret_cast<double *>(smem);
    int *perm = reinterpret_cast<int *>(sE + tile);
    unsigned char *sMat = reinterpret_cast<unsigned char *>(perm + tile + kMaterials * 32);
    __shared__ int cnt[kMaterials], cur[kMaterials], seg[kMaterials + 1], obase[kMaterials];
    __shared__ int roff[kMaterials + 1];
    __shared__ unsigned int qhead;
    __shared__ unsigned long long s_acc;
    SRows sr;
    if constexpr (SROW) {
        // after the tile's arrays, 8-byte aligned: concs, then nuclide ids
        const size_t o = ((size_t)tile * 13 + kMaterials * 128 + 7) & ~(size_t)7;
        double *sc = reinterpret_cast<double *>(smem + o);
        int *sm = reinterpret_cast<int *>(sc + a.rows_total);
        if (threadIdx.x == 0) {
            int s = 0;
            for (int m = 0; m < kMaterials; m++) {
                roff[m] = s;
                s += ldg(&t.num_nucs[m]);
            }
            roff[kMaterials] = s;
        }
        __syncthreads();
        for (int m = 0; m < kMaterials; m++) {
            const int o0 = roff[m], n = roff[m + 1] - o0;
            for (int j = threadIdx.x; j < n; j += BLOCK) {
                sc[o0 + j] = ldg(&t.concs[m * t.max_nucs + j]);
                sm[o0 + j] = ldg(&t.mats[m * t.max_nucs + j]);
            }
        }
        sr.mats = sm;
        sr.concs = sc;
        sr.off = roff;
    }

    const int tid = threadIdx.x;
    const long base = (long)blockIdx.x * tile;
    const int ntile = (int)min((long)tile, a.count - base);
    // the in-tile energy sort's counts and cursors, after everything else
    int *hcnt = nullptr;
    if (a.esort) {
        const size_t o_rows = ((size_t)tile * 13 + kMaterials * 128 + 7) & ~(size_t)7;
        hcnt = reinterpret_cast<int *>(smem + ((o_rows + (SROW ? (size_t)a.rows_total * 12 : 0) + 3) &
                                               ~(size_t)3));
        for (int i = tid; i < kMaterials * kTileBuckets; i += BLOCK) hcnt[i] = 0;
    }
    if (tid < kMaterials) cnt[tid] = 0;
    if (tid == 0) {
        qhead = 0;
        s_acc = 0;
    }
    __syncthreads();

    // sample: LCG threads take consecutive lookups (one skip-ahead each);
    // caller samples are read with a coalesced stride.
    const int lpt = tile / BLOCK;
    if (SAMPLES) {
        for (int l = tid; l < ntile; l += BLOCK) {
            unsigned long long seed = 0;
            double E;
            int m;
            bool ok = sample_at<true>(t, a.in_E, a.in_mat, base + l, seed, E, m, a.err);
            sE[l] = E;
            sMat[l] = ok ? (unsigned char)m : 0xFF;
            if (ok) {
                atomicAdd(&cnt[m], 1);
                if (hcnt) atomicAdd(&hcnt[m * kTileBuckets + tile_bucket(E)], 1);
            }
        }
    } else {
        const int l0 = tid * lpt;
        if (l0 < ntile) {
            unsigned long long seed =
                lcg_skip(kStartingSeed, 2ULL * (unsigned long long)(a.first + base + l0));
            for (int q = 0; q < lpt && l0 + q < ntile; q++) {
                double E;
                int m;
                sample_at<false>(t, nullptr, nullptr, 0, seed, E, m, a.err);
                sE[l0 + q] = E;
                sMat[l0 + q] = (unsigned char)m;
                atomicAdd(&cnt[m], 1);
                if (hcnt) atomicAdd(&hcnt[m * kTileBuckets + tile_bucket(E)], 1);
            }
        }
    }
    __syncthreads();
    const bool overflow = a.ovf_cnt != nullptr;
    if (tid == 0) {
        int s = 0;
        for (int m = 0; m < kMaterials; m++) {
            seg[m] = s;
            cur[m] = s;
            s += (cnt[m] + 31) & ~31;
        }
        seg[kMaterials] = s;
    }
    if (overflow && tid < kMaterials) {
        const int rem = cnt[tid] & 31;
        obase[tid] = rem ? atomicAdd(&a.ovf_cnt[tid], rem) : 0;
    }
    __syncthreads();
    if (hcnt) {
        // each material's buckets start where the previous one's end
        if (tid < kMaterials) {
            int run = seg[tid];
            for (int b = 0; b < kTileBuckets; b++) {
                const int c = hcnt[tid * kTileBuckets + b];
                hcnt[tid * kTileBuckets + b] = run;
                run += c;
            }
        }
        __syncthreads();
        for (int l = tid; l < ntile; l += BLOCK) {
            int m = sMat[l];
            if (m != 0xFF) perm[atomicAdd(&hcnt[m * kTileBuckets + tile_bucket(sE[l])], 1)] = l;
        }
    } else {
        for (int l = tid; l < ntile; l += BLOCK) {
            int m = sMat[l];
            if (m != 0xFF) perm[atomicAdd(&cur[m], 1)] = l;
        }
    }
    __syncthreads();
    if (overflow) {
        // remainders: positions [seg+full, seg+cnt) of each material
        for (int r = tid; r < kMaterials * 32; r += BLOCK) {
            const int m = r >> 5, q = r & 31;
            const int full = cnt[m] & ~31;
            if (q < (cnt[m] & 31)) {
                const int l = perm[seg[m] + full + q];
                const long slot = (long)m * a.ovf_cap + obase[m] + q;
                a.ovf_E[slot] = sE[l];
                a.ovf_id[slot] = (int)(base + l);
            }
        }
    }

    unsigned long long mine = 0;
    const int lane = tid & 31;
    // fuel chunks of 32 / L lookups first, then 32-lookup chunks of the rest
    const int L = (ARITH == XS_ARITH_FAST) ? a.fuel_lanes : 1;
    const int fuel_v = L > 1 ? seg[1] : 0;
    const int nfuel = fuel_v / (32 / L);
    const int nchunks = nfuel + ((seg[kMaterials] - fuel_v) >> 5);
    for (;;) {
        unsigned int c = 0;
        if (lane == 0) c = atomicAdd(&qhead, 1u);
        c = __shfl_sync(0xffffffffu, c, 0);
        if ((int)c >= nchunks) break;
        if (ARITH == XS_ARITH_FAST && (int)c < nfuel) {
            const int q = lane & (L - 1);
            const int p = (int)c * (32 / L) + lane / L;
            const bool live = p < (overflow ? (cnt[0] & ~31) : cnt[0]);
            const int l = live ? perm[p] : 0;
            mine += split_lookup_and_store<GRID, CHECKED, false, SROW>(
                t, live, sE[l], base + l, q, L, a.out_macro, a.out_idx, a.err, sr);
            continue;
        }
        const int cv = (int)c - nfuel + (fuel_v >> 5);
        const int p = cv * 32 + lane;
        int m = 0;
        while (seg[m + 1] <= cv * 32) m++;
        const int limit = seg[m] + (overflow ? (cnt[m] & ~31) : cnt[m]);
        if constexpr (SAMPLES && ARITH == XS_ARITH_FAST) {
            // Without the overflow pass (the chunked pipelines of caller
            // samples), a material's last chunk is partial: its lookups take
            // 2 or 4 lanes each, so the chunk's warp does not idle half its
            // lanes through the nuclide loop.
            const int live_n = limit - cv * 32;   // warp-uniform
            if (!overflow && live_n < 16) {
                const int Lp = live_n <= 8 ? 4 : 2;
                const int q = lane & (Lp - 1), pl = lane / Lp;
                const bool live = pl < live_n;
                const int l = live ? perm[cv * 32 + pl] : 0;
                mine += split_lookup_and_store<GRID, CHECKED, false, SROW>(
                    t, live, sE[l], base + l, q, Lp, a.out_macro, a.out_idx, a.err, sr, m);
                continue;
            }
        }
        if (p < limit) {
            const int l = perm[p];
            mine += lookup_and_store<GRID, ARITH, CHECKED, false, SROW>(
                t, sE[l], m, base + l, a.out_macro, a.out_idx, a.err, sr);
        }
    }
    block_verification(mine, &s_acc, a.verif);
}

// ------------------------------------------------------ segmented lists ---
// Persistent lookup over a material-segmented list (ListArgs).  Warps pull
// 32-entry chunks from a global queue; fuel (material 0) comes first, so the
// longest chunks start first.  No waits: a warp reads the queue once per chunk.
template <int GRID, int ARITH, bool CHECKED, bool TABLE>
__device__ __forceinline__ void list_lookup_body(const Tables &t, const ListArgs &a)
{
    __shared__ int seg[kMaterials + 1], cnt[kMaterials], bas[kMaterials];
    __shared__ unsigned long long s_acc;
    const int tid = threadIdx.x;
    if (tid <= kMaterials) seg[tid] = a.seg_v[tid];
    if (tid < kMaterials) {
        cnt[tid] = a.cnt[tid];
        bas[tid] = a.base ? a.base[tid] : a.seg_v[tid];
    }
    if (tid == 0) s_acc = 0;
    __syncthreads();
    const int lane = tid & 31;
    // fuel chunks of 32 / L entries first (the fuel segment is [seg[0], seg[1])),
    // then 32-entry chunks of the rest
    const int L = (ARITH == XS_ARITH_FAST) ? a.fuel_lanes : 1;
    const int nfuel = L > 1 ? (seg[1] - seg[0]) / (32 / L) : 0;
    const int skip = L > 1 ? (seg[1] >> 5) : 0;
    const int nchunks = nfuel + (seg[kMaterials] >> 5) - skip;
    unsigned long long mine = 0;
    for (;;) {
        unsigned int c = 0;
        if (lane == 0) c = atomicAdd(a.queue, 1u);
        c = __shfl_sync(0xffffffffu, c, 0);
        if ((int)c >= nchunks) break;
        if (ARITH == XS_ARITH_FAST && (int)c < nfuel) {
            const int q = lane & (L - 1);
            const int pv = seg[0] + (int)c * (32 / L) + lane / L;
            const bool live = pv < seg[0] + cnt[0];
            const long p = live ? (long)bas[0] + (pv - seg[0]) : 0;
            mine += split_lookup_and_store<GRID, CHECKED, TABLE>(t, live, live ? a.E[p] : 0.0,
                                                                 live ? a.id[p] : 0, q, L,
                                                                 a.out_macro, a.out_idx, a.err);
            continue;
        }
        const int cv = (int)c - nfuel + skip;
        const int pv = cv * 32 + lane;
        int m = 0;
        while (seg[m + 1] <= cv * 32) m++;
        if constexpr (GRID == XS_NUCLIDE || GRID == XS_HASH) {
            if (a.sorted && !CHECKED) {
                const bool live = pv < seg[m] + cnt[m];
                const long p = live ? (long)bas[m] + (pv - seg[m]) : 0;
                mine += nuclide_warp_lookup_and_store<GRID, ARITH, CHECKED>(
                    t, live, live ? a.E[p] : 0.0, m, live ? (long)a.id[p] : 0, a.out_macro,
                    a.out_idx, a.err);
                continue;
            }
        }
        if (pv < seg[m] + cnt[m]) {
            const long p = (long)bas[m] + (pv - seg[m]);
            mine += lookup_and_store<GRID, ARITH, CHECKED, TABLE>(t, a.E[p], m, a.id[p], a.out_macro,
                                                                  a.out_idx, a.err);
        }
    }
    block_verification(mine, &s_acc, a.verif);
}

// Resident threads per SM held to those of four 256-thread blocks (three on
// the hash grid, whose search needs more registers): the sorted batches'
// warp-cooperative searches are latency-bound (the hash grid's at 96
// registers, two blocks per SM, ran 11-17 % slower; the nuclide grid's at 78,
// three blocks, 17 % slower than at 64, four).
constexpr int list_min_blocks(int grid, int block)
{
    return ((grid == XS_HASH ? 3 : 4) * kBlock + block - 1) / block;
}

template <int GRID, int ARITH, bool CHECKED, int BLOCK = kBlock>
__global__ void __launch_bounds__(BLOCK, list_min_blocks(GRID, BLOCK)) k_list_lookup(Tables t, ListArgs a)
{
    list_lookup_body<GRID, ARITH, CHECKED, false>(t, a);
}

// The union-table variant (FAST): more registers for loads in flight.
template <int GRID, int BLOCK = kBlock>
__global__ void __launch_bounds__(BLOCK, 2 * kBlock / BLOCK) k_list_lookup_table(Tables t, ListArgs a)
{
    list_lookup_body<GRID, XS_ARITH_FAST, false, true>(t, a);
}

// ------------------------------------------------------- adjoint, energy ---
// Over the adjoint's sorted list: the forward macro_xs (FAST arithmetic) and
// dL/dE = sum_c gbar_c * sum_j conc_j * slope_jc, per lookup.  gbar holds the
// upstream gradients by lookup index; each lookup's five are also written to
// sg in sorted order (5 per position, zeros on padding positions) for the
// interval sums, so no separate gather pass runs.
template <int GRID, bool TABLE = false>
__global__ void __launch_bounds__(kBlock) k_list_adjoint(Tables t, ListArgs a, const double *gbar,
                                                         double *sg, double *d_energy)
{
    __shared__ int seg[kMaterials + 1], cnt[kMaterials];
    __shared__ unsigned long long s_acc;
    const int tid = threadIdx.x;
    if (tid <= kMaterials) seg[tid] = a.seg_v[tid];
    if (tid < kMaterials) cnt[tid] = a.cnt[tid];
    if (tid == 0) s_acc = 0;
    __syncthreads();
    const int nchunks = seg[kMaterials] >> 5;
    const int lane = tid & 31;
    unsigned long long mine = 0;
    for (;;) {
        unsigned int c = 0;
        if (lane == 0) c = atomicAdd(a.queue, 1u);
        c = __shfl_sync(0xffffffffu, c, 0);
        if ((int)c >= nchunks) break;
        const int p = (int)c * 32 + lane;
        int m = 0;
        while (seg[m + 1] <= (int)c * 32) m++;
        if (p < seg[m] + cnt[m]) {
            const long id = a.id[p];
            double macro[5], S[5];
            macro_xs<GRID, XS_ARITH_FAST, false, true, TABLE>(t, a.E[p], m, macro, a.err, S);
            const int arg = argmax5(macro);
            mine += (unsigned)(arg + 1);
            if (a.out_macro) {
#pragma unroll
                for (int k = 0; k < 5; k++) a.out_macro[id * 5 + k] = macro[k];
            }
            double g[5];
#pragma unroll
            for (int k = 0; k < 5; k++) {
                g[k] = ldg(&gbar[id * 5 + k]);
                sg[(long)p * 5 + k] = g[k];
            }
            if (d_energy) {
                double dE = 0.0;
#pragma unroll
                for (int k = 0; k < 5; k++) dE = fma(g[k], S[k], dE);
                d_energy[id] = dE;
            }
        } else {
#pragma unroll
            for (int k = 0; k < 5; k++) sg[(long)p * 5 + k] = 0.0;
        }
    }
    block_verification(mine, &s_acc, a.verif);
}

// -------------------------------------------------------------- HISTORY ---
// Simulation.c:116-238: one thread per particle, `nl` dependent lookups; the
// next sample's seed skips one step per macro_xs channel above 1.0.
template <int GRID, int ARITH>
__global__ void __launch_bounds__(kBlock) k_history(Tables t, long first, long count, int nl,
                                                    unsigned long long *verif, int *err)
{
    __shared__ unsigned long long s_acc;
    if (threadIdx.x == 0) s_acc = 0;
    __syncthreads();
    unsigned long long mine = 0;
    const long tpos = (long)blockIdx.x * kBlock + threadIdx.x;
    if (tpos < count) {
        const long p = first + tpos;
        // Simulation.c:167 multiplies in int
        const int skip = (int)((unsigned)(int)p * (unsigned)nl * 2u * 5u);
        unsigned long long seed = lcg_skip(kStartingSeed, (unsigned long long)(long long)skip);
        double E = lcg_next(seed);
        int m = pick_mat(t, seed);
        for (int i = 0; i < nl; i++) {
            double macro[5];
            macro_xs<GRID, ARITH, false>(t, E, m, macro, err);
            mine += (unsigned long long)(argmax5(macro) + 1);
            unsigned long long nf = 0;
#pragma unroll
            for (int k = 0; k < 5; k++) nf += macro[k] > 1.0;
            if (nf) seed = lcg_skip(seed, nf);
            E = lcg_next(seed);
            m = pick_mat(t, seed);
        }
    }
    block_verification(mine, &s_acc, verif);
}

// ------------------------------------------------------------ launchers ---
inline size_t plain_smem_bytes(int tile, int rows_total = 0, bool esort = false)
{
    // the kernel's layout: tile arrays (b bytes); from the next 8-byte
    // boundary the staged rows (rows_total entries); from the next 4-byte
    // boundary the sort histogram
    const size_t b = (size_t)tile * 8 + (size_t)(tile + kMaterials * 32) * 4 + tile;
    const size_t o_rows = (b + 7) & ~(size_t)7;
    if (esort)
        return ((o_rows + (size_t)rows_total * 12 + 3) & ~(size_t)3) +
               (size_t)kMaterials * kTileBuckets * 4;
    return rows_total ? o_rows + (size_t)rows_total * 12 : b;
}

template <int GRID>
struct GridLaunch {
    static cudaError_t plain(const Tables &t, cudaStream_t st, int arith, int checked,
                             bool samples, const PlainArgs &a)
    {
        const long blocks = (a.count + a.tile - 1) / a.tile;
        // staged rows: FAST, unchecked (the variants instantiated with them);
        // the others keep the smaller shared-memory carveout (and their L1)
        const bool srow = a.stage_rows && a.rows_total > 0 && !checked &&
                          arith != XS_ARITH_EXACT &&
                          plain_smem_bytes(a.tile, a.rows_total, a.esort) <= 96 * 1024;
        const size_t sm = plain_smem_bytes(a.tile, srow ? a.rows_total : 0, a.esort);
        // shared-memory share of the SM's 228 KB that holds the resident
        // blocks (each with its static arrays and 1 KB reserved), L1 the rest
        // (the resident blocks: XSGB_PLAIN_MIN_BLOCKS of 256 threads, or as
        // many threads in blocks of a.block)
        const int blk = (!checked && (a.block == 128 || a.block == 512)) ? a.block : kBlock;
        const size_t resident = (size_t)XSGB_PLAIN_MIN_BLOCKS * kBlock / blk;
        const int need = (int)((resident * (sm + 1280) * 100 + 233471) / 233472);
        const int carve = srow ? need : (need > 25 ? need : 25);
#define XSGB_PLAIN_RB(A, C, S, R, B)                                                          \
    do {                                                                                      \
        auto k = k_plain<GRID, A, C, S, R, B>;                                                \
        cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize,  \
                                             (int)sm);                                        \
        if (e == cudaSuccess)                                                                 \
            e = cudaFuncSetAttribute(k, cudaFuncAttributePreferredSharedMemoryCarveout,       \
                                     carve < 100 ? carve : 100);                              \
        if (e != cudaSuccess) return e;                                                       \
        k<<<(unsigned)blocks, B, sm, st>>>(t, a);                                             \
        return cudaGetLastError();                                                            \
    } while (0)
        // unchecked variants in three block sizes; checked runs use 256
#define XSGB_PLAIN_R(A, C, S, R)                                       \
    do {                                                               \
        if (!(C) && a.block == 128) XSGB_PLAIN_RB(A, C, S, R, 128);    \
        if (!(C) && a.block == 512) XSGB_PLAIN_RB(A, C, S, R, 512);    \
        XSGB_PLAIN_RB(A, C, S, R, kBlock);                             \
    } while (0)
#define XSGB_PLAIN(A, C, S) XSGB_PLAIN_R(A, C, S, false)
        if (srow) {
            if (samples) XSGB_PLAIN_R(XS_ARITH_FAST, false, true, true);
            XSGB_PLAIN_R(XS_ARITH_FAST, false, false, true);
        }
        if (checked) {
            if (samples) XSGB_PLAIN(XS_ARITH_FAST, true, true);
            XSGB_PLAIN(XS_ARITH_FAST, true, false);
        }
        if (arith == XS_ARITH_EXACT) {
            if (samples) XSGB_PLAIN(XS_ARITH_EXACT, false, true);
            XSGB_PLAIN(XS_ARITH_EXACT, false, false);
        }
        if (samples) XSGB_PLAIN(XS_ARITH_FAST, false, true);
        XSGB_PLAIN(XS_ARITH_FAST, false, false);
#undef XSGB_PLAIN
#undef XSGB_PLAIN_R
#undef XSGB_PLAIN_RB
    }

    static cudaError_t list(const Tables &t, cudaStream_t st, int arith, int checked, int blocks,
                            const ListArgs &a)
    {
        // `blocks` persistent blocks of a.block threads (checked runs: 256)
#define XSGB_LIST_B(A, C, B)                                                 \
    do {                                                                     \
        k_list_lookup<GRID, A, C, B><<<blocks, B, 0, st>>>(t, a);            \
        return cudaGetLastError();                                           \
    } while (0)
#define XSGB_LIST(A, C)                                     \
    do {                                                    \
        if (!(C) && a.block == 128) XSGB_LIST_B(A, C, 128); \
        if (!(C) && a.block == 512) XSGB_LIST_B(A, C, 512); \
        XSGB_LIST_B(A, C, kBlock);                          \
    } while (0)
        if (checked) XSGB_LIST(XS_ARITH_FAST, true);
        if (arith == XS_ARITH_EXACT) XSGB_LIST(XS_ARITH_EXACT, false);
        if constexpr (GRID == XS_UNIONIZED) {
            if (a.table && t.utab[0] != nullptr) {
                if (a.block == 128)
                    k_list_lookup_table<GRID, 128><<<blocks, 128, 0, st>>>(t, a);
                else if (a.block == 512)
                    k_list_lookup_table<GRID, 512><<<blocks, 512, 0, st>>>(t, a);
                else
                    k_list_lookup_table<GRID><<<blocks, kBlock, 0, st>>>(t, a);
                return cudaGetLastError();
            }
        }
        XSGB_LIST(XS_ARITH_FAST, false);
#undef XSGB_LIST
#undef XSGB_LIST_B
    }

    static cudaError_t adjoint(const Tables &t, cudaStream_t st, int blocks, const ListArgs &a,
                               const double *gbar, double *sg, double *d_energy)
    {
        if constexpr (GRID == XS_UNIONIZED) {
            if (a.table && t.utab[0] != nullptr) {
                k_list_adjoint<GRID, true><<<blocks, kBlock, 0, st>>>(t, a, gbar, sg, d_energy);
                return cudaGetLastError();
            }
        }
        k_list_adjoint<GRID><<<blocks, kBlock, 0, st>>>(t, a, gbar, sg, d_energy);
        return cudaGetLastError();
    }

    static cudaError_t history(const Tables &t, cudaStream_t st, int arith, long first,
                               long count, int nl, unsigned long long *verif, int *err)
    {
        const unsigned blocks = (unsigned)((count + kBlock - 1) / kBlock);
        if (arith == XS_ARITH_EXACT)
            k_history<GRID, XS_ARITH_EXACT><<<blocks, kBlock, 0, st>>>(t, first, count, nl, verif, err);
        else
            k_history<GRID, XS_ARITH_FAST><<<blocks, kBlock, 0, st>>>(t, first, count, nl, verif, err);
        return cudaGetLastError();
    }
};

// Per-grid entry points (defined in lookup_<grid>.cu).
#define XSGB_DECLARE_GRID(NAME)                                                               \
    cudaError_t NAME##_plain(const Tables &t, cudaStream_t st, int arith, int checked,          \
                             bool samples, const PlainArgs &a);                                 \
    cudaError_t NAME##_list(const Tables &t, cudaStream_t st, int arith, int checked,           \
                            int blocks, const ListArgs &a);                                     \
    cudaError_t NAME##_history(const Tables &t, cudaStream_t st, int arith, long first,         \
                               long count, int nl, unsigned long long *verif, int *err);        \
    cudaError_t NAME##_adjoint(const Tables &t, cudaStream_t st, int blocks, const ListArgs &a, \
                               const double *gbar, double *sg, double *d_energy);
XSGB_DECLARE_GRID(unionized)
XSGB_DECLARE_GRID(nuclide)
XSGB_DECLARE_GRID(hash)

#define XSGB_DEFINE_GRID(NAME, GRID)                                                            \
    cudaError_t NAME##_plain(const Tables &t, cudaStream_t st, int arith, int checked,          \
                             bool samples, const PlainArgs &a)                                  \
    {                                                                                           \
        return GridLaunch<GRID>::plain(t, st, arith, checked, samples, a);                      \
    }                                                                                           \
    cudaError_t NAME##_list(const Tables &t, cudaStream_t st, int arith, int checked,           \
                            int blocks, const ListArgs &a)                                      \
    {                                                                                           \
        return GridLaunch<GRID>::list(t, st, arith, checked, blocks, a);                        \
    }                                                                                           \
    cudaError_t NAME##_history(const Tables &t, cudaStream_t st, int arith, long first,         \
                               long count, int nl, unsigned long long *verif, int *err)          \
    {                                                                                           \
        return GridLaunch<GRID>::history(t, st, arith, first, count, nl, verif, err);           \
    }                                                                                           \
    cudaError_t NAME##_adjoint(const Tables &t, cudaStream_t st, int blocks, const ListArgs &a, \
                               const double *gbar, double *sg, double *d_energy)                \
    {                                                                                           \
        return GridLaunch<GRID>::adjoint(t, st, blocks, a, gbar, sg, d_energy);                 \
    }

}  // namespace xsgb
