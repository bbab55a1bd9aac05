// lookup.cu -- orchestration of the lookup kernels and the on-device
// counting sort of the batched form.
//
// The batched form replaces the reference's optimisation 6
// (cuda/Simulation.cu:1024-1099: sampling_kernel, 12 thrust::count, a
// thrust::sort_by_key by material and 12 by energy, 12 launches of
// xs_lookup_kernel_optimization_4, thrust::reduce) by four kernels captured in
// one CUDA graph: histogram of (material, energy bucket) keys, one-block scan,
// scatter, and one persistent lookup kernel whose block sums are added into the
// verification counter.
#include <cstdio>
#include <cstring>

#include <algorithm>

#include "lookup_kernels.cuh"

namespace xsgb {

// ------------------------------------------------------------ sort pass ---
constexpr int kSortLpt = 8;  // lookups per thread in the sampling passes

// floor(E * 2^nb_log2) for E in [0, 1), on the integer pipe
__device__ __forceinline__ int energy_bucket(double E, int nb_log2)
{
    const long long q = order_key(E);
    if (q >= 0 && q < 0x3FF0000000000000LL) return xsgb_floor_scaled_pow2(E, nb_log2);
    return (q >= 0x3FF0000000000000LL && q <= 0x7FF0000000000000LL) ? (1 << nb_log2) - 1
                                                                   : 0;  // NaN and negatives: 0
}

template <bool SAMPLES, bool SCATTER>
__global__ void __launch_bounds__(kBlock) k_sort_pass(Tables t, long first, long count,
                                                      int nb_log2, const double *in_E,
                                                      const int *in_mat, int *offs, double *sE,
                                                      int *sid, int *err)
{
    const long g = (long)blockIdx.x * kBlock + threadIdx.x;
    if (SAMPLES) {
        // coalesced stride over the caller's arrays
        const long stride = (long)gridDim.x * kBlock;
        for (long i = g; i < count; i += stride) {
            unsigned long long seed = 0;
            double E;
            int m;
            if (!sample_at<true>(t, in_E, in_mat, i, seed, E, m, err)) continue;
            const int key = (m << nb_log2) + energy_bucket(E, nb_log2);
            if (SCATTER) {
                const int pos = atomicAdd(&offs[key], 1);
                sE[pos] = E;
                sid[pos] = (int)i;
            } else {
                atomicAdd(&offs[key], 1);
            }
        }
    } else {
        const long i0 = g * kSortLpt;
        if (i0 >= count) return;
        unsigned long long seed = lcg_skip(kStartingSeed, 2ULL * (unsigned long long)(first + i0));
        for (int q = 0; q < kSortLpt && i0 + q < count; q++) {
            // the energy draw's state; its bucket floor(E * nb) and (when
            // scattering) E itself come from it on the integer pipe
            seed = lcg_step(seed);
            const unsigned long long es = seed;
            const int m = pick_mat(t, seed);
            const int key = (m << nb_log2) + xsgb_lcg_bucket(es, nb_log2);
            if (SCATTER) {
                const int pos = atomicAdd(&offs[key], 1);
                sE[pos] = xsgb_lcg_value(es);
                sid[pos] = (int)(i0 + q);
            } else {
                atomicAdd(&offs[key], 1);
            }
        }
    }
}

// One block turns the (material, bucket) histogram into scatter offsets.
// Each material's run starts on a multiple of 32 entries, so every 32-entry
// chunk of the sorted list holds one material only.
constexpr int kScanThreads = 1024;
__global__ void __launch_bounds__(kScanThreads) k_sort_scan(int *offs, int nb_log2, int *seg,
                                                            int *cnt)
{
    __shared__ int warp_tot[32];
    __shared__ int base;
    const int nb = 1 << nb_log2;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int per = (nb + kScanThreads - 1) / kScanThreads;
    if (tid == 0) base = 0;
    __syncthreads();
    for (int m = 0; m < kMaterials; m++) {
        int *h = offs + (m << nb_log2);
        const int b0 = tid * per, b1 = min(nb, b0 + per);
        int s = 0;
        for (int b = b0; b < b1; b++) s += h[b];
        // inclusive warp scan
        int v = s;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            int y = __shfl_up_sync(0xffffffffu, v, o);
            if (lane >= o) v += y;
        }
        if (lane == 31) warp_tot[warp] = v;
        __syncthreads();
        if (warp == 0) {
            int w = warp_tot[lane];
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                int y = __shfl_up_sync(0xffffffffu, w, o);
                if (lane >= o) w += y;
            }
            warp_tot[lane] = w;  // inclusive over warps
        }
        __syncthreads();
        const int total = warp_tot[31];
        int run = base + (v - s) + (warp ? warp_tot[warp - 1] : 0);
        for (int b = b0; b < b1; b++) {
            int c = h[b];
            h[b] = run;
            run += c;
        }
        __syncthreads();
        if (tid == 0) {
            cnt[m] = total;
            seg[m] = base;
            base += (total + 31) & ~31;
        }
        __syncthreads();
    }
    if (tid == 0) seg[kMaterials] = base;
}

// Simulation.c:735-750: the samples alone, one thread per 8 consecutive lookups
__global__ void __launch_bounds__(kBlock) k_sample(Tables t, long first, long count, double *E,
                                                   int *mat)
{
    const long i0 = ((long)blockIdx.x * kBlock + threadIdx.x) * kSortLpt;
    if (i0 >= count) return;
    unsigned long long seed = lcg_skip(kStartingSeed, 2ULL * (unsigned long long)(first + i0));
    for (int q = 0; q < kSortLpt && i0 + q < count; q++) {
        E[i0 + q] = lcg_next(seed);
        mat[i0 + q] = pick_mat(t, seed);
    }
}

xs_status launch_sample(xs_ctx *ctx, cudaStream_t st, long first, long count, double *E, int *mat)
{
    const unsigned blocks = (unsigned)((count + (long)kBlock * kSortLpt - 1) / ((long)kBlock * kSortLpt));
    k_sample<<<blocks, kBlock, 0, st>>>(ctx->t, first, count, E, mat);
    XS_CUDA(cudaGetLastError());
    return XS_OK;
}

size_t batched_scratch_bytes(long count, int buckets)
{
    const size_t padded = (size_t)count + kMaterials * 32;
    size_t b = (size_t)kMaterials * buckets * 4;   // offsets
    b = (b + 255) & ~(size_t)255;
    b += 256;                                       // seg[13] + cnt[12]
    b += padded * 8;                                // sorted energies
    b = (b + 255) & ~(size_t)255;
    b += padded * 4;                                // original ids
    return b + 256;
}

static int ilog2(int x)
{
    int l = 0;
    while ((1 << l) < x) l++;
    return l;
}

typedef cudaError_t (*PlainFn)(const Tables &, cudaStream_t, int, int, bool, const PlainArgs &);
typedef cudaError_t (*ListFn)(const Tables &, cudaStream_t, int, int, int, const ListArgs &);
typedef cudaError_t (*HistoryFn)(const Tables &, cudaStream_t, int, long, long, int,
                                 unsigned long long *, int *);

static PlainFn plain_fn(int g)
{
    return g == XS_UNIONIZED ? unionized_plain : g == XS_NUCLIDE ? nuclide_plain : hash_plain;
}
static ListFn list_fn(int g)
{
    return g == XS_UNIONIZED ? unionized_list : g == XS_NUCLIDE ? nuclide_list : hash_list;
}
static HistoryFn history_fn(int g)
{
    return g == XS_UNIONIZED ? unionized_history : g == XS_NUCLIDE ? nuclide_history : hash_history;
}

// Packed chunk layout of the overflow queues: material m's entries sit at
// [m*cap, m*cap + cnt[m]); its chunks start at the running sum of the
// 32-rounded counts.
__global__ void k_overflow_seg(const int *cnt, int cap, int *seg_v, int *base)
{
    if (threadIdx.x == 0) {
        int s = 0;
        for (int m = 0; m < kMaterials; m++) {
            seg_v[m] = s;
            base[m] = m * cap;
            s += (cnt[m] + 31) & ~31;
        }
        seg_v[kMaterials] = s;
    }
}

static int overflow_cap(long count, int tile)
{
    const long tiles = (count + tile - 1) / tile;
    return (int)(((tiles * 31) + 31) & ~31L);
}

size_t plain_scratch_bytes(long count, int tile)
{
    const size_t cap = (size_t)overflow_cap(count, tile);
    return 1024 + (size_t)kMaterials * cap * 12 + 256;
}

PlainScratch carve_plain_scratch(void *buf, long count, int tile)
{
    PlainScratch p;
    char *b = (char *)buf;
    p.cap = overflow_cap(count, tile);
    p.cnt = (int *)b;            // [12]
    p.seg_v = (int *)(b + 64);   // [13]
    p.base = (int *)(b + 128);   // [12]
    p.queue = (unsigned int *)(b + 192);
    p.E = (double *)(b + 1024);
    p.id = (int *)(b + 1024 + (size_t)kMaterials * p.cap * 8);
    return p;
}

int list_blocks(const xs_ctx *ctx, int block)
{
    if (block <= 0) block = ctx->batched_block;
    const int b = ctx->sm_count * ctx->batched_blocks_per_sm * kBlock / block;
    return b > 0 ? b : 1;
}

xs_status launch_plain(xs_ctx *ctx, cudaStream_t st, int arith, int checked, long first,
                       long count, int tile, int block, const SampleInput &in,
                       const Outputs &out, const PlainScratch *ps, int *launches,
                       const OverflowStream *os)
{
    if (block == 0) {
        block = ctx->plain_block;
        while (block > tile && block > 128) block >>= 1;
    }
    if (block != 128 && block != 256 && block != 512)
        return fail(XS_ERR_INVALID_ARGUMENT, "block_threads %d: 128, 256 or 512", block);
    if (tile < block || tile % block)
        return fail(XS_ERR_INVALID_ARGUMENT, "tile_lookups %d must be a multiple of the block size %d", tile, block);
    if (tile > 8192) return fail(XS_ERR_INVALID_ARGUMENT, "tile_lookups %d above 8192", tile);
    PlainArgs a;
    a.block = block;
    a.esort = ctx->tile_sort >= 0 ? ctx->tile_sort : ctx->t.grid_type != XS_UNIONIZED;
    a.first = first;
    a.count = count;
    a.tile = tile;
    a.in_E = in.energy;
    a.in_mat = in.mat;
    a.out_macro = out.macro;
    a.out_idx = out.max_idx;
    a.verif = ctx->s.verification;
    a.err = ctx->s.error;
    a.ovf_cnt = ps ? ps->cnt : nullptr;
    a.ovf_E = ps ? ps->E : nullptr;
    a.ovf_id = ps ? ps->id : nullptr;
    a.ovf_cap = ps ? ps->cap : 0;
    a.fuel_lanes = ctx->fuel_lanes;
    a.stage_rows = ctx->stage_rows >= 0 ? ctx->stage_rows : ctx->t.grid_type == XS_UNIONIZED;
    a.rows_total = 0;
    for (int m = 0; m < kMaterials; m++) a.rows_total += ctx->num_nucs_host[m];
    if (ps) {
        XS_CUDA(cudaMemsetAsync(ps->cnt, 0, 256, st));  // counts, layout, queue
    }
    XS_CUDA(plain_fn(ctx->t.grid_type)(ctx->t, st, arith, checked, in.energy != nullptr, a));
    if (launches) *launches += 1;
    if (ps) {
        cudaStream_t tiles = st;
        if (os) {
            XS_CUDA(cudaEventRecord(os->ready, tiles));
            XS_CUDA(cudaStreamWaitEvent(os->st, os->ready, 0));
            st = os->st;
        }
        k_overflow_seg<<<1, 32, 0, st>>>(ps->cnt, ps->cap, ps->seg_v, ps->base);
        XS_CUDA(cudaGetLastError());
        ListArgs l;
        l.seg_v = ps->seg_v;
        l.cnt = ps->cnt;
        l.base = ps->base;
        l.E = ps->E;
        l.id = ps->id;
        l.queue = ps->queue;
        l.out_macro = out.macro;
        l.out_idx = out.max_idx;
        l.verif = ctx->s.verification;
        l.err = ctx->s.error;
        l.fuel_lanes = ctx->fuel_lanes;  // the plain kernel's arithmetic, lookup for lookup
        l.table = 0;
        l.sorted = 0;
        l.block = ctx->batched_block;
        XS_CUDA(list_fn(ctx->t.grid_type)(ctx->t, st, arith, checked, list_blocks(ctx, l.block), l));
        if (launches) *launches += 2;
        if (os) {
            XS_CUDA(cudaEventRecord(os->done, st));
            XS_CUDA(cudaStreamWaitEvent(tiles, os->done, 0));
        }
    }
    return XS_OK;
}

// Enqueues the batched pipeline on `st` (used directly or under capture).
BatchedScratch carve_batched_scratch(void *buf, long count, int nb_log2)
{
    const int nb = 1 << nb_log2;
    char *b = (char *)buf;
    BatchedScratch r;
    r.offs = (int *)b;
    size_t off = ((size_t)kMaterials * nb * 4 + 255) & ~(size_t)255;
    r.seg = (int *)(b + off);         // [13]
    r.cnt = r.seg + 16;               // [12]
    r.queue = (unsigned int *)(r.seg + 32);
    off += 256;
    r.sE = (double *)(b + off);
    off += ((size_t)count + kMaterials * 32) * 8;
    off = (off + 255) & ~(size_t)255;
    r.sid = (int *)(b + off);
    r.verification = nullptr;
    r.error = nullptr;
    return r;
}

// The batched run on explicit buffers (b.verification / b.error set): clears
// the bucket offsets and the queue, sorts, runs the lookups.  Four launches.
xs_status enqueue_batched_buf(xs_ctx *ctx, cudaStream_t st, int arith, int checked, long first,
                              long count, int nb_log2, int block, const SampleInput &in,
                              const Outputs &out, const BatchedScratch &b, int *launches)
{
    if (block <= 0) block = ctx->batched_block;
    const int nb = 1 << nb_log2;
    XS_CUDA(cudaMemsetAsync(b.offs, 0, (size_t)kMaterials * nb * 4, st));
    XS_CUDA(cudaMemsetAsync(b.queue, 0, sizeof(unsigned int), st));
    const bool samples = in.energy != nullptr;
    unsigned blocks;
    if (samples) {
        long want = (count + kBlock - 1) / kBlock;
        long cap = (long)ctx->sm_count * 8;
        blocks = (unsigned)(want < cap ? want : cap);
        if (blocks == 0) blocks = 1;
        k_sort_pass<true, false><<<blocks, kBlock, 0, st>>>(ctx->t, first, count, nb_log2, in.energy, in.mat, b.offs, b.sE, b.sid, b.error);
    } else {
        blocks = (unsigned)((count + (long)kBlock * kSortLpt - 1) / ((long)kBlock * kSortLpt));
        k_sort_pass<false, false><<<blocks, kBlock, 0, st>>>(ctx->t, first, count, nb_log2, nullptr, nullptr, b.offs, b.sE, b.sid, b.error);
    }
    XS_CUDA(cudaGetLastError());
    k_sort_scan<<<1, kScanThreads, 0, st>>>(b.offs, nb_log2, b.seg, b.cnt);
    XS_CUDA(cudaGetLastError());
    if (samples)
        k_sort_pass<true, true><<<blocks, kBlock, 0, st>>>(ctx->t, first, count, nb_log2, in.energy, in.mat, b.offs, b.sE, b.sid, b.error);
    else
        k_sort_pass<false, true><<<blocks, kBlock, 0, st>>>(ctx->t, first, count, nb_log2, nullptr, nullptr, b.offs, b.sE, b.sid, b.error);
    XS_CUDA(cudaGetLastError());
    ListArgs l;
    l.seg_v = b.seg;
    l.cnt = b.cnt;
    l.base = nullptr;
    l.E = b.sE;
    l.id = b.sid;
    l.queue = b.queue;
    l.out_macro = out.macro;
    l.out_idx = out.max_idx;
    l.verif = b.verification;
    l.err = b.error;
    l.fuel_lanes = ctx->batched_fuel_lanes;
    l.table = 1;
    l.sorted = 1;
    l.block = block;
    XS_CUDA(list_fn(ctx->t.grid_type)(ctx->t, st, arith, checked, list_blocks(ctx, block), l));
    if (launches) *launches += 4;
    return XS_OK;
}

static xs_status enqueue_batched(xs_ctx *ctx, cudaStream_t st, int arith, int checked, long first,
                                 long count, int nb_log2, int block, const SampleInput &in,
                                 const Outputs &out, int *launches)
{
    BatchedScratch b = carve_batched_scratch(ctx->s.sort_buf, count, nb_log2);
    b.queue = ctx->s.queue;
    b.verification = ctx->s.verification;
    b.error = ctx->s.error;
    return enqueue_batched_buf(ctx, st, arith, checked, first, count, nb_log2, block, in, out, b,
                               launches);
}

// The (material, energy-bucket) counting sort alone, for the adjoint: fills
// starts (bucket starts, before the scatter), offs (bucket ends, after it),
// seg/cnt (padded material segments), sE and sid.
xs_status enqueue_sort_only(xs_ctx *ctx, cudaStream_t st, long first, long count, int nb_log2,
                            const SampleInput &in, int *offs, int *starts, int *seg, int *cnt,
                            double *sE, int *sid)
{
    const int nb = 1 << nb_log2;
    XS_CUDA(cudaMemsetAsync(offs, 0, (size_t)kMaterials * nb * 4, st));
    const bool samples = in.energy != nullptr;
    unsigned blocks;
    if (samples) {
        long want = (count + kBlock - 1) / kBlock;
        long cap = (long)ctx->sm_count * 8;
        blocks = (unsigned)(want < cap ? want : cap);
        if (blocks == 0) blocks = 1;
        k_sort_pass<true, false><<<blocks, kBlock, 0, st>>>(ctx->t, first, count, nb_log2, in.energy, in.mat, offs, sE, sid, ctx->s.error);
    } else {
        blocks = (unsigned)((count + (long)kBlock * kSortLpt - 1) / ((long)kBlock * kSortLpt));
        k_sort_pass<false, false><<<blocks, kBlock, 0, st>>>(ctx->t, first, count, nb_log2, nullptr, nullptr, offs, sE, sid, ctx->s.error);
    }
    XS_CUDA(cudaGetLastError());
    k_sort_scan<<<1, kScanThreads, 0, st>>>(offs, nb_log2, seg, cnt);
    XS_CUDA(cudaGetLastError());
    XS_CUDA(cudaMemcpyAsync(starts, offs, (size_t)kMaterials * nb * 4, cudaMemcpyDeviceToDevice, st));
    if (samples)
        k_sort_pass<true, true><<<blocks, kBlock, 0, st>>>(ctx->t, first, count, nb_log2, in.energy, in.mat, offs, sE, sid, ctx->s.error);
    else
        k_sort_pass<false, true><<<blocks, kBlock, 0, st>>>(ctx->t, first, count, nb_log2, nullptr, nullptr, offs, sE, sid, ctx->s.error);
    XS_CUDA(cudaGetLastError());
    return XS_OK;
}

xs_status launch_adjoint_energy(xs_ctx *ctx, cudaStream_t st, const ListArgs &l,
                                const double *gbar, double *sg, double *d_energy)
{
    typedef cudaError_t (*AdjFn)(const Tables &, cudaStream_t, int, const ListArgs &,
                                 const double *, double *, double *);
    const int g = ctx->t.grid_type;
    AdjFn f = g == XS_UNIONIZED ? unionized_adjoint : g == XS_NUCLIDE ? nuclide_adjoint : hash_adjoint;
    XS_CUDA(f(ctx->t, st, ctx->sm_count * ctx->batched_blocks_per_sm, l, gbar, sg, d_energy));
    return XS_OK;
}

// The batched pipeline over caller-provided scratch: the same four kernels
// as enqueue_batched, launched directly (no graph), for the entry point whose
// scratch is a static device array (static_scratch.cu).
xs_status enqueue_batched_in(xs_ctx *ctx, cudaStream_t st, int arith, long first, long count,
                             int nb_log2, const BatchedScratch &b, const Outputs &out)
{
    const unsigned blocks =
        (unsigned)((count + (long)kBlock * kSortLpt - 1) / ((long)kBlock * kSortLpt));
    k_sort_pass<false, false><<<blocks, kBlock, 0, st>>>(ctx->t, first, count, nb_log2, nullptr,
                                                          nullptr, b.offs, b.sE, b.sid, b.error);
    XS_CUDA(cudaGetLastError());
    k_sort_scan<<<1, kScanThreads, 0, st>>>(b.offs, nb_log2, b.seg, b.cnt);
    XS_CUDA(cudaGetLastError());
    k_sort_pass<false, true><<<blocks, kBlock, 0, st>>>(ctx->t, first, count, nb_log2, nullptr,
                                                         nullptr, b.offs, b.sE, b.sid, b.error);
    XS_CUDA(cudaGetLastError());
    ListArgs l;
    l.seg_v = b.seg;
    l.cnt = b.cnt;
    l.base = nullptr;
    l.E = b.sE;
    l.id = b.sid;
    l.queue = b.queue;
    l.out_macro = out.macro;
    l.out_idx = out.max_idx;
    l.verif = b.verification;
    l.err = b.error;
    l.fuel_lanes = ctx->batched_fuel_lanes;
    l.table = 1;
    l.sorted = 1;
    l.block = ctx->batched_block;
    XS_CUDA(list_fn(ctx->t.grid_type)(ctx->t, st, arith, 0, list_blocks(ctx, l.block), l));
    return XS_OK;
}

xs_status launch_batched(xs_ctx *ctx, cudaStream_t st, int arith, int checked, long first,
                         long count, int block, int buckets, const SampleInput &in,
                         const Outputs &out, int *launches)
{
    if (block <= 0) block = ctx->batched_block;
    if (block != 128 && block != 256 && block != 512)
        return fail(XS_ERR_INVALID_ARGUMENT, "block_threads %d: 128, 256 or 512", block);
    if (buckets < 1 || (buckets & (buckets - 1)) || buckets > 65536)
        return fail(XS_ERR_INVALID_ARGUMENT, "energy_buckets %d must be a power of two <= 65536", buckets);
    if (count > 0x7FFFFFFFL - kMaterials * 32)
        return fail(XS_ERR_INVALID_ARGUMENT, "batched runs take at most 2^31 - 385 lookups");
    const int nb_log2 = ilog2(buckets);
    const size_t need = batched_scratch_bytes(count, buckets);
    if (ctx->s.sort_bytes < need) {
        for (auto &kv : ctx->graphs) cudaGraphExecDestroy(kv.second.exec);
        ctx->graphs.clear();
        if (ctx->s.sort_buf) {
            cudaFree(ctx->s.sort_buf);
            ctx->device_bytes -= ctx->s.sort_bytes;
            ctx->s.sort_buf = nullptr;
            ctx->s.sort_bytes = 0;
        }
        cudaError_t e = cudaMalloc(&ctx->s.sort_buf, need);
        if (e != cudaSuccess) {
            cudaGetLastError();
            return fail(XS_ERR_OUT_OF_MEMORY, "device allocation of %zu bytes for the batched sort failed", need);
        }
        ctx->s.sort_bytes = need;
        ctx->device_bytes += need;
    }
    char key[256];
    // everything the captured launches bake in: options, pointers, grid view
    snprintf(key, sizeof key, "%d/%d/%ld/%ld/%d/%p/%p/%p/%p/%p/%d/%d/%d/%p/%p/%d/%d", arith, checked,
             first, count, nb_log2, (const void *)in.energy, (const void *)in.mat,
             (void *)out.macro, (void *)out.max_idx, (void *)st, ctx->batched_blocks_per_sm, block,
             ctx->t.grid_type, (const void *)ctx->t.index_grid, (const void *)ctx->t.coarse,
             ctx->t.hash_bins, ctx->batched_fuel_lanes * 2 + (ctx->t.utab[0] != nullptr));
    auto it = ctx->graphs.find(key);
    if (it == ctx->graphs.end()) {
        cudaStream_t cap;
        XS_CUDA(cudaStreamCreateWithFlags(&cap, cudaStreamNonBlocking));
        cudaGraph_t g = nullptr;
        cudaError_t e = cudaStreamBeginCapture(cap, cudaStreamCaptureModeThreadLocal);
        if (e != cudaSuccess) {
            cudaStreamDestroy(cap);
            return cuda_fail(e, "cudaStreamBeginCapture");
        }
        int n = 0;
        xs_status s = enqueue_batched(ctx, cap, arith, checked, first, count, nb_log2, block, in, out,
                                      &n);
        e = cudaStreamEndCapture(cap, &g);
        cudaStreamDestroy(cap);
        if (s != XS_OK) {
            if (g) cudaGraphDestroy(g);
            return s;
        }
        if (e != cudaSuccess) return cuda_fail(e, "cudaStreamEndCapture");
        BatchedGraph bg;
        e = cudaGraphInstantiate(&bg.exec, g, 0);
        cudaGraphDestroy(g);
        if (e != cudaSuccess) return cuda_fail(e, "cudaGraphInstantiate");
        bg.launches = n;
        if (ctx->graphs.size() > 64) {
            for (auto &kv : ctx->graphs) cudaGraphExecDestroy(kv.second.exec);
            ctx->graphs.clear();
        }
        it = ctx->graphs.emplace(key, bg).first;
    }
    XS_CUDA(cudaGraphLaunch(it->second.exec, st));
    if (launches) *launches += it->second.launches;
    return XS_OK;
}

// Stepped history: particle p's state (seed, energy, material) before its
// first lookup (Simulation.c:160-175; the skip is multiplied in int there).
__global__ void k_history_init(Tables t, long first, long count, int nl,
                               unsigned long long *seed, double *E, int *mat)
{
    for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < count;
         i += (long)gridDim.x * blockDim.x) {
        const long p = first + i;
        const int skip = (int)((unsigned)(int)p * (unsigned)nl * 2u * 5u);
        unsigned long long s = lcg_skip(kStartingSeed, (unsigned long long)(long long)skip);
        E[i] = lcg_next(s);
        mat[i] = pick_mat(t, s);
        seed[i] = s;
    }
}

// The state after a lookup (Simulation.c:205-224): one skip per macro_xs
// channel above 1.0, then the next energy and material.
__global__ void k_history_advance(Tables t, long count, const double *macro,
                                  unsigned long long *seed, double *E, int *mat)
{
    for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < count;
         i += (long)gridDim.x * blockDim.x) {
        unsigned long long nf = 0;
#pragma unroll
        for (int k = 0; k < 5; k++) nf += macro[i * 5 + k] > 1.0;
        unsigned long long s = seed[i];
        if (nf) s = lcg_skip(s, nf);
        E[i] = lcg_next(s);
        mat[i] = pick_mat(t, s);
        seed[i] = s;
    }
}

xs_status launch_history_stepped(xs_ctx *ctx, cudaStream_t st, int arith, long first, long count,
                                 int tile, int *launches)
{
    const int nl = ctx->inputs.lookups;
    // A step is one batch of `count` lookups (500,000 at the default size),
    // too few to fill the GPU, so a step lasts about as long as its longest
    // fuel lookups; the overflow pass would add one more such chain per step
    // (EXACT 172 M lookups/s against 115-130 M with the pass, one group).
    // Tiles measured with four groups (large problem, unionized / hash /
    // nuclide grid): FAST 256: 762 / 610 / 591 M, 512: 824 / 619 / 648 M,
    // 1,024: 725 / 594 / 565 M; EXACT 1,024: 219 / 210 / 202 M, 2,048:
    // 183 / 169 / 164 M.
    if (tile <= 0) tile = arith == XS_ARITH_EXACT ? 1024 : 512;
    const size_t need = (size_t)count * (8 + 8 + 4 + 40) + 4096;
    if (ctx->s.hist_bytes < need) {
        if (ctx->s.hist_buf) {
            cudaFree(ctx->s.hist_buf);
            ctx->device_bytes -= ctx->s.hist_bytes;
            ctx->s.hist_buf = nullptr;
            ctx->s.hist_bytes = 0;
        }
        cudaError_t e = cudaMalloc(&ctx->s.hist_buf, need);
        if (e != cudaSuccess) {
            cudaGetLastError();
            return fail(XS_ERR_OUT_OF_MEMORY, "history particle states (%zu bytes)", need);
        }
        ctx->s.hist_bytes = need;
        ctx->device_bytes += need;
    }
    char *b = (char *)ctx->s.hist_buf;
    auto take = [&](size_t bytes) { char *r = b; b += (bytes + 255) & ~(size_t)255; return r; };
    unsigned long long *seed = (unsigned long long *)take((size_t)count * 8);
    double *E = (double *)take((size_t)count * 8);
    int *mat = (int *)take((size_t)count * 4);
    double *macro = (double *)take((size_t)count * 40);
    const unsigned blocks = (unsigned)std::min<long>((count + 255) / 256, (long)ctx->sm_count * 16);
    k_history_init<<<blocks, 256, 0, st>>>(ctx->t, first, count, nl, seed, E, mat);
    XS_CUDA(cudaGetLastError());
    int n = 1;
    // The particles in up to eight contiguous groups (of at least 65,536),
    // each on a stream of its own through all its steps: a group's step ends
    // in a tail (its longest fuel lookups), which the other groups' steps
    // fill.  Particles are independent, so the groups' steps need no order
    // among themselves.  Large problem, unionized grid, one / four / eight
    // groups: FAST 654 / 823 / 825 M lookups/s, EXACT 172 / 220 / 229 M.
    const int groups = (int)std::max<long>(1, std::min<long>(ctx->hist_groups, count / 65536));
    cudaStream_t gs[xs_ctx::kPipeSlots];
    long lo[xs_ctx::kPipeSlots + 1];
    for (int g = 0; g <= groups; g++) lo[g] = count * g / groups;
    if (groups > 1) {
        XS_CUDA(cudaEventRecord(ctx->fork_event, st));
        for (int g = 0; g < groups; g++) {
            gs[g] = ctx->pipe_stream[g];
            XS_CUDA(cudaStreamWaitEvent(gs[g], ctx->fork_event, 0));
        }
    } else {
        gs[0] = st;
    }
    for (int step = 0; step < nl; step++) {
        for (int g = 0; g < groups; g++) {
            const long m = lo[g + 1] - lo[g];
            SampleInput in;
            in.energy = E + lo[g];
            in.mat = mat + lo[g];
            Outputs out;
            out.macro = macro + lo[g] * 5;
            xs_status s = launch_plain(ctx, gs[g], arith, 0, 0, m, tile, 0, in, out, nullptr, &n);
            if (s != XS_OK) return s;
            if (step + 1 < nl) {
                const unsigned b = (unsigned)std::min<long>((m + 255) / 256, (long)ctx->sm_count * 16);
                k_history_advance<<<b, 256, 0, gs[g]>>>(ctx->t, m, macro + lo[g] * 5, seed + lo[g],
                                                        E + lo[g], mat + lo[g]);
                XS_CUDA(cudaGetLastError());
                n++;
            }
        }
    }
    if (groups > 1) {
        for (int g = 0; g < groups; g++) {
            XS_CUDA(cudaEventRecord(ctx->pipe_event[g], gs[g]));
            XS_CUDA(cudaStreamWaitEvent(st, ctx->pipe_event[g], 0));
        }
    }
    if (launches) *launches += n;
    return XS_OK;
}

xs_status launch_history(xs_ctx *ctx, cudaStream_t st, int arith, long first, long count,
                         int *launches)
{
    XS_CUDA(history_fn(ctx->t.grid_type)(ctx->t, st, arith, first, count, ctx->inputs.lookups,
                                         ctx->s.verification, ctx->s.error));
    if (launches) *launches += 1;
    return XS_OK;
}

}  // namespace xsgb
