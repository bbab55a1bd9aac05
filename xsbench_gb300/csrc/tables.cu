// tables.cu -- device-side tables derived from the reference arrays at
// context creation, and the validation pass that lets the lookup kernels
// index without bounds checks.
//
//   records     per nuclide interval k: E_hi, the five xs at k+1, the five
//               slopes (xs_{k+1}-xs_k)/(E_{k+1}-E_k) and E_lo (96 bytes in a
//               128-byte slot)
//   ekeys       order keys of every gridpoint energy (HASH / NUCLIDE searches)
//   coarse      every 16th key of each nuclide (NUCLIDE search, first level)
//   union_keys  order keys of the unionized energies
//   union_bins  for b = 0..2^L: #{union energies < b / 2^L}
//   union table per material m and union row e, one 80-byte entry per
//               nuclide j of m: the five pairs (v, s), v = the channel of
//               nuclide j's interval line at u_e, s its slope; stored [e][j][c]
//               (the unionized grid with every nuclide's cross sections
//               reconstructed on it)
#include <cstdlib>

#include "device_common.cuh"

namespace xsgb {

__global__ void k_records(const xs_gridpoint *grid, long n_iso, long n_gp, double2 *rec)
{
    const long n_int = n_gp - 1;
    for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < n_iso * n_int;
         i += (long)gridDim.x * blockDim.x) {
        const long nuc = i / n_int, k = i - nuc * n_int;
        const xs_gridpoint lo = grid[nuc * n_gp + k];
        const xs_gridpoint hi = grid[nuc * n_gp + k + 1];
        const double dE = hi.energy - lo.energy;
        double2 *r = rec + i * kRecordPairs;
        r[0] = make_double2(hi.energy, hi.total_xs);
        r[1] = make_double2(hi.elastic_xs, hi.absorbtion_xs);
        r[2] = make_double2(hi.fission_xs, hi.nu_fission_xs);
        r[3] = make_double2((hi.total_xs - lo.total_xs) / dE, (hi.elastic_xs - lo.elastic_xs) / dE);
        r[4] = make_double2((hi.absorbtion_xs - lo.absorbtion_xs) / dE,
                            (hi.fission_xs - lo.fission_xs) / dE);
        r[5] = make_double2((hi.nu_fission_xs - lo.nu_fission_xs) / dE, lo.energy);
        r[6] = make_double2(0.0, 0.0);   // slot padding
        r[7] = make_double2(0.0, 0.0);
    }
}

__global__ void k_grid_keys(const xs_gridpoint *grid, long n, long long *keys)
{
    for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += (long)gridDim.x * blockDim.x)
        keys[i] = order_key(grid[i].energy);
}

__global__ void k_coarse(const long long *ekeys, long n_iso, long n_gp, int n_coarse,
                         long long *coarse)
{
    for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < n_iso * n_coarse;
         i += (long)gridDim.x * blockDim.x) {
        const long nuc = i / n_coarse, c = i - nuc * n_coarse;
        coarse[i] = ekeys[nuc * n_gp + c * kCoarseStride];
    }
}

// Hash grid of GridInit.c:128-151: index[e][nuc] = grid_search_nuclide of the
// bin edge e * du over the nuclide's whole grid (Simulation.c:403-423).
__global__ void k_hash_grid(const xs_gridpoint *grid, long n_iso, long n_gp, int bins, double du,
                            int *index)
{
    for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < (long)bins * n_iso;
         i += (long)gridDim.x * blockDim.x) {
        const long e = i / n_iso, nuc = i - e * n_iso;
        const double energy = e * du;
        const xs_gridpoint *A = grid + nuc * n_gp;
        long lo = 0, hi = n_gp - 1;
        while (hi - lo > 1) {
            long mid = lo + (hi - lo) / 2;
            if (A[mid].energy > energy) hi = mid; else lo = mid;
        }
        index[i] = (int)lo;
    }
}

// Energy-bin guide of each nuclide: for 2^k bins over [0, 1),
// guide[nuc][b] = #{j : E_j < b / 2^k}.  Thread (nuc, j) for j = 0 .. n_gp
// writes j into the bins b with E_{j-1} < b / 2^k <= E_j (E_{-1} = -inf,
// E_{n_gp} = +inf): on a sorted grid these ranges partition 0 .. 2^k, so
// every entry is written exactly once.  b / 2^k <= E  <=>  b <= floor(E 2^k),
// exact in integers for E in [0, 1).
__device__ __forceinline__ long guide_floor(double E, int k)
{
    if (!(E >= 0.0)) return -1;                 // negative (or NaN: ordered last by the sort)
    if (E >= 1.0) return 1L << k;
    return xsgb_floor_scaled_pow2(E, k);
}

__global__ void k_guide(const xs_gridpoint *grid, long n_iso, long n_gp, int k, int *guide)
{
    const long nb = (1L << k) + 1;
    for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < n_iso * (n_gp + 1);
         i += (long)gridDim.x * blockDim.x) {
        const long nuc = i / (n_gp + 1), j = i - nuc * (n_gp + 1);
        const xs_gridpoint *A = grid + nuc * n_gp;
        long lo = j == 0 ? 0 : guide_floor(A[j - 1].energy, k) + 1;
        long hi = j == n_gp ? nb - 1 : guide_floor(A[j].energy, k);
        if (lo < 0) lo = 0;
        if (hi > nb - 1) hi = nb - 1;
        int *g = guide + nuc * nb;
        for (long b = lo; b <= hi; b++) g[b] = (int)j;
    }
}

// Bin records: slot (nuc, b) = the record of interval
// k0 = clamp(guide[nuc][b] - 1, 0, n_gp - 2), and in the slot's fourth
// sector (double 12, as integer bits) k0 itself, which the lookup reads only
// when E lies past that interval: the sector comes with the slot's 128-byte
// line, so the walk starts without a guide read.
__global__ void k_bin_records(const double2 *rec, const int *guide, long n_iso, long n_gp, int k,
                              double2 *out)
{
    const long nb = 1L << k;
    for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < n_iso * nb;
         i += (long)gridDim.x * blockDim.x) {
        const long nuc = i >> k, b = i & (nb - 1);
        long k0 = (long)guide[nuc * (nb + 1) + b] - 1;
        if (k0 < 0) k0 = 0;
        if (k0 > n_gp - 2) k0 = n_gp - 2;
        const double2 *src = rec + (nuc * (n_gp - 1) + k0) * kRecordPairs;
        double2 *dst = out + i * kRecordPairs;
#pragma unroll
        for (int q = 0; q < 6; q++) dst[q] = src[q];
        dst[6] = make_double2(__longlong_as_double((long long)k0), 0.0);
        dst[7] = make_double2(0.0, 0.0);
    }
}

cudaError_t launch_hash_grid(const xs_gridpoint *grid, long n_iso, long n_gp, int bins, int *index,
                             int sm_count, cudaStream_t st)
{
    k_hash_grid<<<sm_count * 8, 256, 0, st>>>(grid, n_iso, n_gp, bins, 1.0 / bins, index);
    return cudaGetLastError();
}

cudaError_t launch_coarse_keys(const long long *ekeys, long n_iso, long n_gp, int n_coarse,
                               long long *coarse, int sm_count, cudaStream_t st)
{
    k_coarse<<<sm_count * 8, 256, 0, st>>>(ekeys, n_iso, n_gp, n_coarse, coarse);
    return cudaGetLastError();
}

__global__ void k_double_keys(const double *v, long n, long long *keys)
{
    for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += (long)gridDim.x * blockDim.x)
        keys[i] = order_key(v[i]);
}

__global__ void k_union_bins(const long long *keys, long n, int log2b, int *bins)
{
    const long nb = 1L << log2b;
    for (long b = (long)blockIdx.x * blockDim.x + threadIdx.x; b <= nb;
         b += (long)gridDim.x * blockDim.x) {
        const long long q = order_key((double)b / (double)nb);
        long lo = 0, hi = n;  // first index with key >= q
        while (lo < hi) {
            long mid = (lo + hi) >> 1;
            if (keys[mid] < q) lo = mid + 1; else hi = mid;
        }
        bins[b] = (int)lo;
    }
}

// Range checks of caller-supplied tables; err[0] = 1 on the first failure.
__global__ void k_check_index(const int *idx, long n, int lo, int hi, int *err)
{
    for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += (long)gridDim.x * blockDim.x) {
        const int v = idx[i];
        if (v < lo || v > hi) report(err, XS_ERR_DATA, i, v);
    }
}

static unsigned grid_for(long n, int sm)
{
    long b = (n + 255) / 256;
    long cap = (long)sm * 32;
    if (b > cap) b = cap;
    return (unsigned)(b < 1 ? 1 : b);
}

// Entry (e, j) of material m's union table.  The interval is the one the
// reference's unionized lookup reads for (u_e, nuclide) (Simulation.c:264-272):
// index_grid[e][nuc], moved down one at the top gridpoint.
__global__ void k_union_table(Tables t, int m, int n_m, double2 *out)
{
    const long total = t.n_union * n_m;
    const long top = t.n_gp - 1;
    for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < total;
         i += (long)gridDim.x * blockDim.x) {
        const long e = i / n_m;
        const int j = (int)(i - e * n_m);
        const int nuc = t.mats[m * t.max_nucs + j];
        long k = t.index_grid[e * t.n_iso + nuc];
        if (k == top) k -= 1;
        const double *r = reinterpret_cast<const double *>(t.records + ((long)nuc * (t.n_gp - 1) + k) * kRecordPairs);
        const double d = t.union_e[e] - r[0];
        double2 *o = out + i * 5;
#pragma unroll
        for (int c = 0; c < 5; c++) o[c] = make_double2(fma(r[6 + c], d, r[1 + c]), r[6 + c]);
    }
}

xs_status build_union_table(xs_ctx *ctx)
{
    Tables &t = ctx->t;
    for (int m = 0; m < kMaterials; m++) t.utab[m] = nullptr;
    ctx->union_table_bytes = 0;
    if (t.grid_type != XS_UNIONIZED) return XS_OK;
    if (const char *env = getenv("XSGB_UNION_TABLE"))
        if (atoi(env) == 0) return XS_OK;
    size_t need = 0;
    for (int m = 0; m < kMaterials; m++) need += (size_t)t.n_union * ctx->num_nucs_host[m] * 80 + 256;
    // built only when it leaves room for the runs' own buffers
    size_t free_b = 0, total_b = 0;
    if (cudaMemGetInfo(&free_b, &total_b) != cudaSuccess) {
        cudaGetLastError();
        return XS_OK;
    }
    const size_t reserve = (size_t)24 << 30;
    if (free_b < need + reserve) return XS_OK;
    const int sm = ctx->sm_count;
    for (int m = 0; m < kMaterials; m++) {
        const int n_m = ctx->num_nucs_host[m];
        if (n_m == 0) continue;
        void *p = nullptr;
        xs_status s = ctx_alloc(ctx, &p, (size_t)t.n_union * n_m * 80);
        if (s != XS_OK) return s;
        k_union_table<<<(unsigned)sm * 16, 256, 0, ctx->stream>>>(t, m, n_m, (double2 *)p);
        XS_CUDA(cudaGetLastError());
        t.utab[m] = (const double2 *)p;
    }
    XS_CUDA(cudaStreamSynchronize(ctx->stream));
    ctx->union_table_bytes = need;
    if (!getenv("XSGB_BATCHED_FUEL_LANES")) ctx->batched_fuel_lanes = ctx->num_nucs_host[0] >= 64 ? 2 : 1;
    return XS_OK;
}

// The energy-bin guide (Tables::guide) and the bin records
// (Tables::binrec): about four bins per gridpoint (2^(ceil(log2 n_gp) + 2),
// at most 2^26 per nuclide; two where the device lacks the room), so most
// bins hold no gridpoint and a lookup's interval is the bin's first one.
// Measured on 355 x 238,847 points: hash grid 592 / 649 / 665-670 M
// lookups/s at two / four / eight bins per gridpoint, nuclide grid 704 M at
// four and 679 M at eight (on 355 x 11,303 points: 746 M at four, 666 M at
// eight); four holds up on both grids at half the memory of eight.  Built for the hash and nuclide grids (and
// by the autotuner when it serves a unionized context from those);
// XSGB_GUIDE=0 in the environment leaves both out, and so does a device
// without room for them (the searches then run without them).
xs_status build_guide(xs_ctx *ctx)
{
    Tables &t = ctx->t;
    t.guide = nullptr;
    t.guide_log2 = 0;
    t.binrec = nullptr;
    size_t free_b = 0, total_b = 0;
    if (cudaMemGetInfo(&free_b, &total_b) != cudaSuccess) {
        cudaGetLastError();
        return XS_OK;
    }
    // four bins per gridpoint where the device has room for their bin
    // records (16 GiB kept free), else two
    int lg = 0;
    while (lg < 26 && (1L << lg) < t.n_gp) lg++;
    int k = lg + 2 < 26 ? lg + 2 : 26;
    auto need = [&](int kk) {
        return (size_t)t.n_iso * (((size_t)1 << kk) * (kRecordDoubles * 8 + 4) + 4) + ((size_t)16 << 30);
    };
    while (k > lg + 1 && need(k) > free_b) k--;
    if (const char *env = getenv("XSGB_GUIDE_LOG2")) {
        const int v = atoi(env);
        if (v >= 1 && v <= 26) k = v;
    }
    const size_t bytes = (size_t)t.n_iso * (((size_t)1 << k) + 1) * 4;
    if (free_b < bytes + ((size_t)4 << 30)) return XS_OK;
    void *p = nullptr;
    xs_status s = ctx_alloc(ctx, &p, bytes);
    if (s != XS_OK) return s;
    k_guide<<<grid_for((long)t.n_iso * (t.n_gp + 1), ctx->sm_count), 256, 0, ctx->stream>>>(
        t.grid, t.n_iso, t.n_gp, k, (int *)p);
    XS_CUDA(cudaGetLastError());
    t.guide = (const int *)p;
    t.guide_log2 = k;

    // bin records: 128 bytes per (nuclide, bin), when the device keeps 16 GiB
    // beside them; XSGB_BIN_RECORDS=0 leaves them out
    t.binrec = nullptr;
    t.bin_prefetch = 1;
    if (const char *env = getenv("XSGB_BIN_PREFETCH")) {
        const int v = atoi(env);
        if (v >= 0 && v <= 4) t.bin_prefetch = v;
    }
    if (const char *env = getenv("XSGB_BIN_RECORDS"))
        if (atoi(env) == 0) return XS_OK;
    const size_t rbytes = (size_t)t.n_iso * ((size_t)1 << k) * kRecordDoubles * 8;
    if (cudaMemGetInfo(&free_b, &total_b) != cudaSuccess) {
        cudaGetLastError();
        return XS_OK;
    }
    if (free_b < rbytes + ((size_t)16 << 30)) return XS_OK;
    s = ctx_alloc(ctx, &p, rbytes);
    if (s != XS_OK) return s;
    k_bin_records<<<grid_for((long)t.n_iso << k, ctx->sm_count), 256, 0, ctx->stream>>>(
        t.records, t.guide, t.n_iso, t.n_gp, k, (double2 *)p);
    XS_CUDA(cudaGetLastError());
    t.binrec = (const double2 *)p;
    return XS_OK;
}

xs_status build_derived_tables(xs_ctx *ctx)
{
    Tables &t = ctx->t;
    cudaStream_t st = ctx->stream;
    const int sm = ctx->sm_count;
    const long n_points = (long)t.n_iso * t.n_gp;

    // validation of the integer tables the kernels index with
    XS_CUDA(cudaMemsetAsync(ctx->s.error, 0, 4 * sizeof(int), st));
    if (t.grid_type == XS_UNIONIZED)
        k_check_index<<<grid_for((long)t.n_union * t.n_iso, sm), 256, 0, st>>>(
            t.index_grid, (long)t.n_union * t.n_iso, 0, (int)(t.n_gp - 1), ctx->s.error);
    if (t.grid_type == XS_HASH)
        k_check_index<<<grid_for((long)t.hash_bins * t.n_iso, sm), 256, 0, st>>>(
            t.index_grid, (long)t.hash_bins * t.n_iso, 0, (int)(t.n_gp - 2), ctx->s.error);
    XS_CUDA(cudaGetLastError());

    // interval records for the fast arithmetic
    void *p = nullptr;
    xs_status s = ctx_alloc(ctx, &p, (size_t)t.n_iso * (t.n_gp - 1) * kRecordDoubles * 8);
    if (s != XS_OK) return s;
    t.records = (const double2 *)p;
    k_records<<<grid_for(t.n_iso * (t.n_gp - 1), sm), 256, 0, st>>>(t.grid, t.n_iso, t.n_gp, (double2 *)p);
    XS_CUDA(cudaGetLastError());

    {   // every grid type: the searches of the hash / nuclide grids and the adjoint
        s = ctx_alloc(ctx, &p, (size_t)n_points * 8);
        if (s != XS_OK) return s;
        t.ekeys = (const long long *)p;
        k_grid_keys<<<grid_for(n_points, sm), 256, 0, st>>>(t.grid, n_points, (long long *)p);
        XS_CUDA(cudaGetLastError());
    }
    if (t.grid_type == XS_NUCLIDE) {
        t.n_coarse = (int)((t.n_gp + kCoarseStride - 1) / kCoarseStride);
        s = ctx_alloc(ctx, &p, (size_t)t.n_iso * t.n_coarse * 8);
        if (s != XS_OK) return s;
        t.coarse = (const long long *)p;
        k_coarse<<<grid_for((long)t.n_iso * t.n_coarse, sm), 256, 0, st>>>(t.ekeys, t.n_iso, t.n_gp, t.n_coarse, (long long *)p);
        XS_CUDA(cudaGetLastError());
    }
    // the guided searches: on the nuclide grid always; on the hash grid when
    // its energy keys exceed L2 (below that the hash grid's own search, its
    // index rows and keys held in L2, is faster: 722 against 665 M lookups/s
    // on 355 x 11,303 points; 616 against 370 M on 355 x 238,847).
    // XSGB_GUIDE=1 / 0 forces either.
    bool guided = t.grid_type == XS_NUCLIDE;
    if (t.grid_type == XS_HASH) {
        int l2 = 0;
        if (cudaDeviceGetAttribute(&l2, cudaDevAttrL2CacheSize, ctx->device) != cudaSuccess) {
            cudaGetLastError();
            l2 = 0;
        }
        guided = (size_t)n_points * 8 > (size_t)l2;
    }
    if (const char *env = getenv("XSGB_GUIDE")) guided = atoi(env) != 0 && t.grid_type != XS_UNIONIZED;
    if (guided) {
        s = build_guide(ctx);
        if (s != XS_OK) return s;
    }
    // with the in-tile energy order (the hash and nuclide grids) the plain
    // kernel runs best in tiles of 2,048 (XL, guided: 616 against 518 M
    // lookups/s at 1,024; large hash grid, its own search: 754 against 738 M)
    // plain tiles: 2,048 lookups on the hash grid, 1,536 on the nuclide grid
    // (large problem: 749 against 745 M lookups/s, 727 against 715 M end to
    // end; the hash grid 752 against 745 M at 1,536), 3,072 on long grids
    // (the XL problem), whose bin-record reads gain from the denser energy
    // order of a bigger tile while four blocks still share an SM (XL, hash /
    // nuclide grid: 660 / 704 M at 2,048, 707 / 755 M at 3,072, 685 / 737 M at
    // 3,584; 597 M at 4,096, three blocks per SM)
    if (t.grid_type != XS_UNIONIZED)
        ctx->plain_tile = t.n_gp > 65536 ? 3072 : t.grid_type == XS_NUCLIDE ? 1536 : 2048;
    if (t.grid_type == XS_UNIONIZED) {
        s = ctx_alloc(ctx, &p, (size_t)t.n_union * 8);
        if (s != XS_OK) return s;
        t.union_keys = (const long long *)p;
        k_double_keys<<<grid_for(t.n_union, sm), 256, 0, st>>>(t.union_e, t.n_union, (long long *)p);
        XS_CUDA(cudaGetLastError());
        // about one union energy per bin, at least 2^10 and at most 2^26 bins
        int lb = 10;
        while (lb < 26 && (1L << lb) < t.n_union) lb++;
        t.union_bin_log2 = lb;
        s = ctx_alloc(ctx, &p, ((size_t)(1L << lb) + 1) * 4);
        if (s != XS_OK) return s;
        t.union_bins = (const int *)p;
        k_union_bins<<<grid_for((1L << lb) + 1, sm), 256, 0, st>>>(t.union_keys, t.n_union, lb, (int *)p);
        XS_CUDA(cudaGetLastError());
    }
    int herr[4] = {0, 0, 0, 0};
    XS_CUDA(cudaMemcpyAsync(herr, ctx->s.error, sizeof herr, cudaMemcpyDeviceToHost, st));
    XS_CUDA(cudaStreamSynchronize(st));
    if (herr[0])
        return fail(XS_ERR_DATA, "table entry out of range (position %d, value %d)", herr[1], herr[2]);
    return XS_OK;
}

}  // namespace xsgb
