// setup_device.cu -- the problem built on the GPU (xs_ctx_create_on_device):
// the same arrays as grid_init_do_not_profile (openmp-threading/GridInit.c:3-230)
// bit for bit, with no host-side grid and no upload of it.
//
//   gridpoints  point p draws its six values from the LCG state skipped to 6p
//               from seed 42 (the one sequential stream of GridInit.c:34-47);
//   per-nuclide sort by energy, stable (GridInit.c:50-51 with ties kept in
//               draw order): a counting sort into energy buckets, then each
//               bucket sorted by (energy, draw index);
//   union grid  all energies sorted the same way (GridInit.c:84-89);
//   index grid  index[e][i] = min(n_gp - 2, #{j >= 1 : E_ij <= u_e}), which is
//               what the sweep of GridInit.c:106-122 leaves when a nuclide's
//               energies are strictly increasing (checked; otherwise the call
//               reports XS_ERR_UNSUPPORTED);
//   hash grid   the search of GridInit.c:137-150 per (bin, nuclide);
//   materials   the 12 lists and the concentration stream, built on the host
//               (46 KB) and uploaded.
#include <algorithm>
#include <cstring>
#include <vector>

#include "device_common.cuh"

namespace xsgb {

constexpr int kGenPerThread = 64;

__global__ void k_gen_points(long n_pts, xs_gridpoint *g)
{
    const long p0 = ((long)blockIdx.x * blockDim.x + threadIdx.x) * kGenPerThread;
    if (p0 >= n_pts) return;
    unsigned long long s = lcg_skip(42ULL, 6ULL * (unsigned long long)p0);
    for (long p = p0; p < p0 + kGenPerThread && p < n_pts; p++) {
        xs_gridpoint v;
        v.energy = lcg_next(s);
        v.total_xs = lcg_next(s);
        v.elastic_xs = lcg_next(s);
        v.absorbtion_xs = lcg_next(s);
        v.fission_xs = lcg_next(s);
        v.nu_fission_xs = lcg_next(s);
        g[p] = v;
    }
}

__device__ __forceinline__ long energy_bucket_of(double E, int nb)
{
    if (!(E > 0.0)) return 0;
    long b = (long)(E * (double)nb);
    return b >= nb ? nb - 1 : b;
}

// histogram (or scatter) of values into (segment, energy bucket) keys;
// segment = p / seg_len
template <bool SCATTER>
__global__ void k_bucket_pass(const double *vals, long stride, long n, long seg_len, int nb,
                              int *offs, double *outE, int *outId)
{
    for (long p = (long)blockIdx.x * blockDim.x + threadIdx.x; p < n;
         p += (long)gridDim.x * blockDim.x) {
        const double E = vals[p * stride];
        const long key = (p / seg_len) * nb + energy_bucket_of(E, nb);
        if (SCATTER) {
            const int pos = atomicAdd(&offs[key], 1);
            outE[pos] = E;
            outId[pos] = (int)(p % seg_len);
        } else {
            atomicAdd(&offs[key], 1);
        }
    }
}

// exclusive scan of n ints in place, three phases with a fixed shape
constexpr int kIScan = 1024;
__global__ void __launch_bounds__(kIScan) k_iscan_blocks(const int *a, long n, long long *bsum)
{
    __shared__ long long red[kIScan];
    const long nb = (n + kIScan - 1) / kIScan;
    for (long b = blockIdx.x; b < nb; b += gridDim.x) {
        const long i = b * kIScan + threadIdx.x;
        red[threadIdx.x] = i < n ? a[i] : 0;
        __syncthreads();
        for (int w = kIScan / 2; w > 0; w >>= 1) {
            if (threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
            __syncthreads();
        }
        if (threadIdx.x == 0) bsum[b] = red[0];
        __syncthreads();
    }
}

__global__ void __launch_bounds__(kIScan) k_iscan_top(long nb, long long *bsum)
{
    __shared__ long long part[kIScan];
    const long per = (nb + kIScan - 1) / kIScan;
    const long a = threadIdx.x * per, e = min(nb, a + per);
    long long s = 0;
    for (long b = a; b < e; b++) s += bsum[b];
    part[threadIdx.x] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
        long long run = 0;
        for (int t = 0; t < kIScan; t++) {
            long long v = part[t];
            part[t] = run;
            run += v;
        }
    }
    __syncthreads();
    long long run = part[threadIdx.x];
    for (long b = a; b < e; b++) {
        long long v = bsum[b];
        bsum[b] = run;
        run += v;
    }
}

__global__ void __launch_bounds__(kIScan) k_iscan_local(int *a, long n, const long long *bsum)
{
    __shared__ long long buf[kIScan];
    const long nb = (n + kIScan - 1) / kIScan;
    for (long b = blockIdx.x; b < nb; b += gridDim.x) {
        const long i = b * kIScan + threadIdx.x;
        const long long v = i < n ? a[i] : 0;
        buf[threadIdx.x] = v;
        __syncthreads();
        for (int o = 1; o < kIScan; o <<= 1) {
            const long long x = threadIdx.x >= o ? buf[threadIdx.x - o] : 0;
            __syncthreads();
            buf[threadIdx.x] += x;
            __syncthreads();
        }
        if (i < n) a[i] = (int)(bsum[b] + buf[threadIdx.x] - v);
        __syncthreads();
    }
}

// bucket starts from the ends the scatter left: start = end - count
__global__ void k_bucket_starts(const int *ends, const int *counts, long n, int *starts)
{
    for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x)
        starts[i] = ends[i] - counts[i];
}

// sorted gridpoints of each nuclide, and a flag if any nuclide repeats an energy
// sorted gridpoints of each nuclide: dst[n][j] = src[n][sid[n][j]]
__global__ void k_permute_points(const xs_gridpoint *src, const int *sid, long n_iso, long n_gp,
                                 xs_gridpoint *dst)
{
    for (long p = (long)blockIdx.x * blockDim.x + threadIdx.x; p < n_iso * n_gp;
         p += (long)gridDim.x * blockDim.x) {
        const long nuc = p / n_gp;
        dst[p] = src[nuc * n_gp + sid[p]];
    }
}

// flag (*dup = 1) when some nuclide's energies are not strictly increasing
__global__ void k_check_strict(const xs_gridpoint *g, long n_iso, long n_gp, int *dup)
{
    for (long p = (long)blockIdx.x * blockDim.x + threadIdx.x; p < n_iso * n_gp;
         p += (long)gridDim.x * blockDim.x) {
        if (p % n_gp == 0) continue;
        if (!(g[p - 1].energy < g[p].energy)) *dup = 1;
    }
}

// unionized index grid: thread = (chunk of kRows union rows, nuclide); nuclide
// fastest so a warp writes consecutive entries of a row
constexpr int kRows = 32;
__global__ void k_union_index(const xs_gridpoint *g, const double *u, long n_union, long n_iso,
                              long n_gp, int *index)
{
    const long nchunks = (n_union + kRows - 1) / kRows;
    for (long w = (long)blockIdx.x * blockDim.x + threadIdx.x; w < nchunks * n_iso;
         w += (long)gridDim.x * blockDim.x) {
        const long chunk = w / n_iso, i = w - chunk * n_iso;
        const xs_gridpoint *A = g + i * n_gp;
        const long e0 = chunk * kRows;
        // c = #{j >= 1 : E_j <= u[e0]}
        const double q = u[e0];
        long lo = 1, hi = n_gp;
        while (lo < hi) {
            long mid = (lo + hi) >> 1;
            if (A[mid].energy <= q) lo = mid + 1; else hi = mid;
        }
        long c = lo - 1;
        const long e1 = min(n_union, e0 + kRows);
        for (long e = e0; e < e1; e++) {
            const double ue = u[e];
            while (c + 1 <= n_gp - 1 && A[c + 1].energy <= ue) c++;
            index[e * n_iso + i] = (int)min(c, n_gp - 2);
        }
    }
}

static int pow2_at_least(long x)
{
    int p = 1;
    while (p < x && p < (1 << 26)) p <<= 1;
    return p;
}

// Sorts values (stride apart) into segments of seg_len; outputs the sorted
// values and, per position, the value's index within its segment.
static xs_status segmented_sort(xs_ctx *ctx, cudaStream_t st, const double *vals, long stride,
                                long n, long seg_len, double *outE, int *outId)
{
    const long nseg = n / seg_len;
    const int nb = pow2_at_least(std::max<long>(1, seg_len / 16));  // ~16 values per bucket
    const long nkeys = nseg * nb;
    const long nblk = (nkeys + kIScan - 1) / kIScan;
    void *tmp = nullptr;
    const size_t bytes = (size_t)nkeys * 4 * 3 + (size_t)nblk * 8 + 1024;
    cudaError_t e = cudaMalloc(&tmp, bytes);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return fail(XS_ERR_OUT_OF_MEMORY, "device setup: %zu bytes of sort scratch", bytes);
    }
    int *counts = (int *)tmp, *offs = counts + nkeys, *starts = offs + nkeys;
    long long *bsum = (long long *)(starts + nkeys + 2);
    bsum = (long long *)(((uintptr_t)bsum + 7) & ~(uintptr_t)7);
    const int sm = ctx->sm_count;
    xs_status s = XS_OK;
    do {
        if ((e = cudaMemsetAsync(counts, 0, (size_t)nkeys * 4, st)) != cudaSuccess) break;
        k_bucket_pass<false><<<sm * 16, 256, 0, st>>>(vals, stride, n, seg_len, nb, counts, nullptr, nullptr);
        if ((e = cudaMemcpyAsync(offs, counts, (size_t)nkeys * 4, cudaMemcpyDeviceToDevice, st)) != cudaSuccess) break;
        k_iscan_blocks<<<std::min<long>(nblk, sm * 8), kIScan, 0, st>>>(offs, nkeys, bsum);
        k_iscan_top<<<1, kIScan, 0, st>>>(nblk, bsum);
        k_iscan_local<<<std::min<long>(nblk, sm * 8), kIScan, 0, st>>>(offs, nkeys, bsum);
        k_bucket_pass<true><<<sm * 16, 256, 0, st>>>(vals, stride, n, seg_len, nb, offs, outE, outId);
        k_bucket_starts<<<sm * 8, 256, 0, st>>>(offs, counts, nkeys, starts);
        if ((e = launch_bucket_sort(starts, offs, (int)nkeys, outE, outId,
                                    (int)std::min<long>(nkeys, (long)sm * 16), st)) != cudaSuccess)
            break;
        e = cudaStreamSynchronize(st);
    } while (0);
    cudaFree(tmp);
    if (e != cudaSuccess) s = cuda_fail(e, "device setup sort");
    return s;
}

}  // namespace xsgb

using namespace xsgb;

extern "C" xs_status xs_ctx_create_on_device(const xs_inputs *in, int device, xs_ctx **out)
{
    if (!out) return fail(XS_ERR_INVALID_ARGUMENT, "xs_ctx_create_on_device: out is NULL");
    *out = nullptr;
    if (!in || in->n_isotopes < 1 || in->n_gridpoints < 2)
        return fail(XS_ERR_INVALID_ARGUMENT, "need n_isotopes >= 1 and n_gridpoints >= 2");
    if (in->grid_type < 0 || in->grid_type > 2) return fail(XS_ERR_INVALID_ARGUMENT, "grid_type %d", in->grid_type);
    if (in->grid_type == XS_HASH && in->hash_bins < 1) return fail(XS_ERR_INVALID_ARGUMENT, "hash_bins %d", in->hash_bins);
    const long n_iso = in->n_isotopes, n_gp = in->n_gridpoints, n_pts = n_iso * n_gp;
    if (n_pts > 0x7FFFFFFFL) return fail(XS_ERR_INVALID_ARGUMENT, "n_isotopes*n_gridpoints above 2^31-1");
    if (in->grid_type == XS_UNIONIZED && n_pts * n_iso > (1L << 40))
        return fail(XS_ERR_INVALID_ARGUMENT, "unionized index grid of %ld entries", n_pts * n_iso);
    // the material tables (host, 46 KB)
    xs_simdata mats;
    std::memset(&mats, 0, sizeof mats);
    xs_status s = load_materials(n_iso, &mats);
    if (s != XS_OK) {
        xs_simdata_free(&mats);
        return s;
    }
    xs_ctx *ctx = nullptr;
    s = ctx_open(in, device, &ctx);
    if (s != XS_OK) {
        xs_simdata_free(&mats);
        return s;
    }
    Tables &t = ctx->t;
    cudaStream_t st = ctx->stream;
    const int sm = ctx->sm_count;
    void *gen = nullptr, *tmpE = nullptr, *tmpId = nullptr;
    int *dup = ctx->s.error + 3;
    cudaError_t e = cudaSuccess;
    do {
        s = install_materials(ctx, in, &mats);
        if (s != XS_OK) break;
        // gridpoints in draw order, then sorted per nuclide into the context's grid
        e = cudaMalloc(&gen, (size_t)n_pts * sizeof(xs_gridpoint));
        if (e == cudaSuccess) e = cudaMalloc(&tmpE, (size_t)n_pts * 8);
        if (e == cudaSuccess) e = cudaMalloc(&tmpId, (size_t)n_pts * 4);
        if (e != cudaSuccess) {
            cudaGetLastError();
            s = fail(XS_ERR_OUT_OF_MEMORY, "device setup scratch (%ld points)", n_pts);
            break;
        }
        const long gthreads = (n_pts + kGenPerThread - 1) / kGenPerThread;
        k_gen_points<<<(unsigned)((gthreads + 255) / 256), 256, 0, st>>>(n_pts, (xs_gridpoint *)gen);
        s = segmented_sort(ctx, st, (const double *)gen, 6, n_pts, n_gp, (double *)tmpE, (int *)tmpId);
        if (s != XS_OK) break;
        void *grid = nullptr;
        s = ctx_alloc(ctx, &grid, (size_t)n_pts * sizeof(xs_gridpoint));
        if (s != XS_OK) break;
        t.grid = (const xs_gridpoint *)grid;
        k_permute_points<<<sm * 16, 256, 0, st>>>((const xs_gridpoint *)gen, (const int *)tmpId, n_iso, n_gp,
                                                   (xs_gridpoint *)grid);
        if (in->grid_type == XS_UNIONIZED) {
            e = cudaMemsetAsync(dup, 0, 4, st);
            if (e != cudaSuccess) break;
            k_check_strict<<<sm * 16, 256, 0, st>>>(t.grid, n_iso, n_gp, dup);
            int *hdup = (int *)ctx->h_result;
            e = cudaMemcpyAsync(hdup, dup, 4, cudaMemcpyDeviceToHost, st);
            if (e == cudaSuccess) e = cudaStreamSynchronize(st);
            if (e != cudaSuccess) break;
            if (*hdup) {
                s = fail(XS_ERR_UNSUPPORTED, "a nuclide repeats an energy: build this problem on the host (xs_grid_init)");
                break;
            }
            // union energies: every energy, sorted (one segment)
            s = segmented_sort(ctx, st, (const double *)grid, 6, n_pts, n_pts, (double *)tmpE, (int *)tmpId);
            if (s != XS_OK) break;
            void *u = nullptr, *idx = nullptr;
            s = ctx_alloc(ctx, &u, (size_t)n_pts * 8);
            if (s == XS_OK) s = ctx_alloc(ctx, &idx, (size_t)n_pts * n_iso * 4);
            if (s != XS_OK) break;
            e = cudaMemcpyAsync(u, tmpE, (size_t)n_pts * 8, cudaMemcpyDeviceToDevice, st);
            if (e != cudaSuccess) break;
            t.union_e = (const double *)u;
            t.n_union = n_pts;
            const long work = ((n_pts + kRows - 1) / kRows) * n_iso;
            k_union_index<<<(unsigned)std::min<long>((work + 255) / 256, (long)sm * 64), 256, 0, st>>>(
                t.grid, t.union_e, n_pts, n_iso, n_gp, (int *)idx);
            t.index_grid = (const int *)idx;
        } else if (in->grid_type == XS_HASH) {
            void *idx = nullptr;
            s = ctx_alloc(ctx, &idx, (size_t)in->hash_bins * n_iso * 4);
            if (s != XS_OK) break;
            if ((e = launch_hash_grid(t.grid, n_iso, n_gp, in->hash_bins, (int *)idx, sm, st)) != cudaSuccess)
                break;
            t.index_grid = (const int *)idx;
        }
        if ((e = cudaGetLastError()) != cudaSuccess) break;
        if ((e = cudaMemsetAsync(ctx->s.error, 0, 16, st)) != cudaSuccess) break;
        if ((e = cudaStreamSynchronize(st)) != cudaSuccess) break;
        ctx->own_index = t.index_grid;
        s = build_derived_tables(ctx);
        if (s == XS_OK) s = build_union_table(ctx);
    } while (0);
    if (s == XS_OK && e != cudaSuccess) s = cuda_fail(e, "device setup");
    cudaStreamSynchronize(st);
    if (gen) cudaFree(gen);
    if (tmpE) cudaFree(tmpE);
    if (tmpId) cudaFree(tmpId);
    xs_simdata_free(&mats);
    if (s != XS_OK) {
        xs_ctx_destroy(ctx);
        return s;
    }
    ctx->base_coarse = t.coarse;
    ctx->base_n_coarse = t.n_coarse;
    ctx->own_guide = t.guide;
    ctx->own_binrec = t.binrec;
    ctx->base_guided = t.guide != nullptr;
    *out = ctx;
    return XS_OK;
}
