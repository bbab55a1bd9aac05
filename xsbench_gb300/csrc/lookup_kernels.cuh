// lookup_kernels.cuh -- the lookup kernels, templated on grid type and
// arithmetic.  Instantiated once per grid type (lookup_<grid>.cu) so the
// three translation units compile in parallel.
#pragma once

#include "device_common.cuh"

namespace xsgb {

constexpr int kBlock = 256;          // threads per block of every lookup kernel
constexpr int kWarps = kBlock / 32;

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

// ---------------------------------------------------------------- PLAIN ---
// One block = one tile of `tile` consecutive lookups.  The block samples them,
// counting-sorts their ids by material in shared memory (each material's run
// padded to a multiple of 32 so a warp never mixes materials), then its warps
// pull 32-lookup chunks, fuel first, from a shared-memory queue and run one
// lookup per lane.
template <int GRID, int ARITH, bool CHECKED, bool SAMPLES>
__global__ void __launch_bounds__(kBlock) k_plain(Tables t, long first, long count, int tile,
                                                  const double *in_E, const int *in_mat,
                                                  double *out_macro, unsigned char *out_idx,
                                                  unsigned long long *verif, int *err)
{
    extern __shared__ __align__(16) unsigned char smem[];
    double *sE = reinterpret_cast<double *>(smem);
    int *perm = reinterpret_cast<int *>(sE + tile);
    unsigned char *sMat = reinterpret_cast<unsigned char *>(perm + tile + kMaterials * 32);
    __shared__ int cnt[kMaterials], cur[kMaterials], seg[kMaterials + 1];
    __shared__ unsigned int qhead;
    __shared__ unsigned long long s_acc;

    const int tid = threadIdx.x;
    const long base = (long)blockIdx.x * tile;
    const int ntile = (int)min((long)tile, count - base);
    if (tid < kMaterials) cnt[tid] = 0;
    if (tid == 0) {
        qhead = 0;
        s_acc = 0;
    }
    __syncthreads();

    // sample: LCG threads take consecutive lookups (one skip-ahead each);
    // caller samples are read with a coalesced stride.
    const int lpt = tile / kBlock;
    if (SAMPLES) {
        for (int l = tid; l < ntile; l += kBlock) {
            unsigned long long seed = 0;
            double E;
            int m;
            bool ok = sample_at<true>(t, in_E, in_mat, base + l, seed, E, m, err);
            sE[l] = E;
            sMat[l] = ok ? (unsigned char)m : 0xFF;
            if (ok) atomicAdd(&cnt[m], 1);
        }
    } else {
        const int l0 = tid * lpt;
        if (l0 < ntile) {
            unsigned long long seed = lcg_skip(kStartingSeed, 2ULL * (unsigned long long)(first + base + l0));
            for (int q = 0; q < lpt && l0 + q < ntile; q++) {
                double E;
                int m;
                sample_at<false>(t, nullptr, nullptr, 0, seed, E, m, err);
                sE[l0 + q] = E;
                sMat[l0 + q] = (unsigned char)m;
                atomicAdd(&cnt[m], 1);
            }
        }
    }
    __syncthreads();
    if (tid == 0) {
        int s = 0;
        for (int m = 0; m < kMaterials; m++) {
            seg[m] = s;
            cur[m] = s;
            s += (cnt[m] + 31) & ~31;
        }
        seg[kMaterials] = s;
    }
    __syncthreads();
    for (int l = tid; l < ntile; l += kBlock) {
        int m = sMat[l];
        if (m != 0xFF) perm[atomicAdd(&cur[m], 1)] = l;
    }
    __syncthreads();

    unsigned long long mine = 0;
    const int lane = tid & 31;
    const int nchunks = seg[kMaterials] >> 5;
    for (;;) {
        unsigned int c = 0;
        if (lane == 0) c = atomicAdd(&qhead, 1u);
        c = __shfl_sync(0xffffffffu, c, 0);
        if ((int)c >= nchunks) break;
        const int p = (int)c * 32 + lane;
        int m = 0;
        while (seg[m + 1] <= (int)c * 32) m++;
        if (p < seg[m] + cnt[m]) {
            const int l = perm[p];
            const double E = sE[l];
            double macro[5];
            macro_xs<GRID, ARITH, CHECKED>(t, E, m, macro, err);
            const int arg = argmax5(macro);
            mine += (unsigned long long)(arg + 1);
            const long o = base + l;
            if (out_macro) {
#pragma unroll
                for (int k = 0; k < 5; k++) out_macro[o * 5 + k] = macro[k];
            }
            if (out_idx) out_idx[o] = (unsigned char)arg;
        }
    }
    block_verification(mine, &s_acc, verif);
}

// -------------------------------------------------------------- BATCHED ---
// Persistent lookup over the (material, energy-bucket)-sorted list.  Warps pull
// 32-entry chunks from a global queue; the sorted order puts the fuel
// material first, so the longest chunks start first.
template <int GRID, int ARITH, bool CHECKED>
__global__ void __launch_bounds__(kBlock) k_batched_lookup(Tables t, const int *seg_g,
                                                           const int *cnt_g, const double *sE,
                                                           const int *sid, unsigned int *queue,
                                                           double *out_macro,
                                                           unsigned char *out_idx,
                                                           unsigned long long *verif, int *err)
{
    __shared__ int seg[kMaterials + 1], cnt[kMaterials];
    __shared__ unsigned long long s_acc;
    const int tid = threadIdx.x;
    if (tid <= kMaterials) seg[tid] = seg_g[tid];
    if (tid < kMaterials) cnt[tid] = cnt_g[tid];
    if (tid == 0) s_acc = 0;
    __syncthreads();
    const int nchunks = seg[kMaterials] >> 5;
    const int lane = tid & 31;
    unsigned long long mine = 0;
    for (;;) {
        unsigned int c = 0;
        if (lane == 0) c = atomicAdd(queue, 1u);
        c = __shfl_sync(0xffffffffu, c, 0);
        if ((int)c >= nchunks) break;
        const int p = (int)c * 32 + lane;
        int m = 0;
        while (seg[m + 1] <= (int)c * 32) m++;
        if (p < seg[m] + cnt[m]) {
            const double E = sE[p];
            const int id = sid[p];
            double macro[5];
            macro_xs<GRID, ARITH, CHECKED>(t, E, m, macro, err);
            const int arg = argmax5(macro);
            mine += (unsigned long long)(arg + 1);
            if (out_macro) {
#pragma unroll
                for (int k = 0; k < 5; k++) out_macro[(long)id * 5 + k] = macro[k];
            }
            if (out_idx) out_idx[id] = (unsigned char)arg;
        }
    }
    block_verification(mine, &s_acc, verif);
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
template <int GRID>
struct GridLaunch {
    static cudaError_t plain(const Tables &t, cudaStream_t st, int arith, int checked,
                             bool samples, long first, long count, int tile, const double *in_E,
                             const int *in_mat, double *out_macro, unsigned char *out_idx,
                             unsigned long long *verif, int *err)
    {
        const long blocks = (count + tile - 1) / tile;
        const size_t sm = (size_t)tile * 8 + (size_t)(tile + kMaterials * 32) * 4 + tile;
#define XSGB_PLAIN(A, C, S)                                                               \
    do {                                                                                  \
        auto k = k_plain<GRID, A, C, S>;                                                  \
        cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, \
                                             (int)sm);                                    \
        if (e != cudaSuccess) return e;                                                   \
        k<<<(unsigned)blocks, kBlock, sm, st>>>(t, first, count, tile, in_E, in_mat,      \
                                                out_macro, out_idx, verif, err);          \
        return cudaGetLastError();                                                        \
    } while (0)
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
    }

    static cudaError_t batched(const Tables &t, cudaStream_t st, int arith, int checked,
                               int blocks, const int *seg, const int *cnt, const double *sE,
                               const int *sid, unsigned int *queue, double *out_macro,
                               unsigned char *out_idx, unsigned long long *verif, int *err)
    {
#define XSGB_BATCHED(A, C)                                                                    \
    do {                                                                                      \
        k_batched_lookup<GRID, A, C><<<blocks, kBlock, 0, st>>>(t, seg, cnt, sE, sid, queue,  \
                                                                out_macro, out_idx, verif,    \
                                                                err);                         \
        return cudaGetLastError();                                                            \
    } while (0)
        if (checked) XSGB_BATCHED(XS_ARITH_FAST, true);
        if (arith == XS_ARITH_EXACT) XSGB_BATCHED(XS_ARITH_EXACT, false);
        XSGB_BATCHED(XS_ARITH_FAST, false);
#undef XSGB_BATCHED
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
                             bool samples, long first, long count, int tile, const double *in_E, \
                             const int *in_mat, double *out_macro, unsigned char *out_idx,       \
                             unsigned long long *verif, int *err);                               \
    cudaError_t NAME##_batched(const Tables &t, cudaStream_t st, int arith, int checked,        \
                               int blocks, const int *seg, const int *cnt, const double *sE,     \
                               const int *sid, unsigned int *queue, double *out_macro,           \
                               unsigned char *out_idx, unsigned long long *verif, int *err);     \
    cudaError_t NAME##_history(const Tables &t, cudaStream_t st, int arith, long first,         \
                               long count, int nl, unsigned long long *verif, int *err);
XSGB_DECLARE_GRID(unionized)
XSGB_DECLARE_GRID(nuclide)
XSGB_DECLARE_GRID(hash)

#define XSGB_DEFINE_GRID(NAME, GRID)                                                            \
    cudaError_t NAME##_plain(const Tables &t, cudaStream_t st, int arith, int checked,          \
                             bool samples, long first, long count, int tile, const double *in_E, \
                             const int *in_mat, double *out_macro, unsigned char *out_idx,       \
                             unsigned long long *verif, int *err)                                \
    {                                                                                           \
        return GridLaunch<GRID>::plain(t, st, arith, checked, samples, first, count, tile, in_E, \
                                       in_mat, out_macro, out_idx, verif, err);                  \
    }                                                                                           \
    cudaError_t NAME##_batched(const Tables &t, cudaStream_t st, int arith, int checked,        \
                               int blocks, const int *seg, const int *cnt, const double *sE,     \
                               const int *sid, unsigned int *queue, double *out_macro,           \
                               unsigned char *out_idx, unsigned long long *verif, int *err)      \
    {                                                                                           \
        return GridLaunch<GRID>::batched(t, st, arith, checked, blocks, seg, cnt, sE, sid, queue, \
                                         out_macro, out_idx, verif, err);                        \
    }                                                                                           \
    cudaError_t NAME##_history(const Tables &t, cudaStream_t st, int arith, long first,         \
                               long count, int nl, unsigned long long *verif, int *err)          \
    {                                                                                           \
        return GridLaunch<GRID>::history(t, st, arith, first, count, nl, verif, err);           \
    }

}  // namespace xsgb
