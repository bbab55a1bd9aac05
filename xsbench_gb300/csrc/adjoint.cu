// adjoint.cu -- gradients of the macroscopic lookup.
//
// For a scalar loss L with upstream gradients g_i = dL/dmacro_xs_i (5 per
// lookup), lookup i of material m in interval k of nuclide n (conc c) has
//   xs_c = hi_c - f (hi_c - lo_c),  f = (E_hi - E_i) / (E_hi - E_lo)
// so that
//   dL/dE_i        = sum_c g_ic * sum_j c_j slope_jc          (per lookup)
//   dL/dlo_kc     += c * sum_{i in k} g_ic f_i                (gridpoint k)
//   dL/dhi_kc     += c * sum_{i in k} g_ic (1 - f_i)          (gridpoint k+1)
//   dL/dc_mj       = sum_k sum_c [hi_kc G_kc - (hi_kc - lo_kc) F_kc]
// with G_kc = sum_{i in k} g_ic and F_kc = sum_{i in k} g_ic f_i.
//
// Pipeline (one stream, every sum in a fixed order, so results are
// bit-reproducible):
//   1. counting sort by (material, energy bucket), then each bucket sorted by
//      (energy, index) -- a deterministic total order per material;
//   2. the upstream gradients gathered into that order;
//   3. per lookup: forward macro_xs and dL/dE (interval search recomputed);
//   4. transposed pass: a warp takes a chunk of one material's sorted lookups
//      and lanes take that material's nuclides; each lane walks its nuclide's
//      intervals alongside the rising energies and accumulates
//      A_kc = sum g_ic (E_hi - E_i) and G_kc per interval; intervals inside the
//      chunk are stored, the first and last go to per-chunk boundary slots;
//   5. boundary slots added into the interval table chunk by chunk, in order;
//   6. dL/dxs per gridpoint (materials in order) and dL/dconcs per (m, j)
//      (fixed-shape tree), added into the caller's arrays.
#include <algorithm>
#include <cstring>

#include "lookup_kernels.cuh"

namespace xsgb {

constexpr int kAdjChunk = 2048;        // sorted lookups per transposed chunk
constexpr int kAdjBucketLog2 = 12;     // energy buckets per material
constexpr int kSortCap = 2048;         // largest bucket sorted in shared memory
constexpr int kTbl = 10;               // doubles per (pair, interval): A[5], G[5]
constexpr int kSlot = 12;              // doubles per boundary slot: k, A[5], G[5], pad

__device__ __forceinline__ bool pair_less(long long ka, int ia, long long kb, int ib)
{
    return ka < kb || (ka == kb && ia < ib);
}

// ---------------------------------------------------------- bucket sort ---
// One block per bucket: sort the bucket's (energy, id) entries by (order key
// of the energy, id).  Buckets up to kSortCap entries sort in shared memory;
// larger ones in place in global memory.  Both use the bitonic network in its
// all-ascending form (first step of each merge pairs i with i ^ (k-1)), so
// positions past the bucket act as +infinity and never move.
__global__ void __launch_bounds__(256) k_bucket_sort(const int *starts, const int *ends,
                                                     int nbuckets, double *sE, int *sid)
{
    __shared__ long long key[kSortCap];
    __shared__ int id[kSortCap];
    __shared__ double ev[kSortCap];
    for (int b = blockIdx.x; b < nbuckets; b += gridDim.x) {
        const int a = starts[b], n = ends[b] - a;
        if (n <= 1) continue;
        int P = 1;
        while (P < n) P <<= 1;
        if (n <= kSortCap) {
            for (int i = threadIdx.x; i < P; i += blockDim.x) {
                if (i < n) {
                    ev[i] = sE[a + i];
                    key[i] = order_key(ev[i]);
                    id[i] = sid[a + i];
                } else {
                    key[i] = 0x7FFFFFFFFFFFFFFFLL;
                    id[i] = 0x7FFFFFFF;
                    ev[i] = 0.0;
                }
            }
            __syncthreads();
            for (int k = 2; k <= P; k <<= 1) {
                for (int j = k >> 1; j > 0; j >>= 1) {
                    for (int i = threadIdx.x; i < P; i += blockDim.x) {
                        const int q = (j == (k >> 1)) ? (i ^ (k - 1)) : (i ^ j);
                        if (q > i && pair_less(key[q], id[q], key[i], id[i])) {
                            long long tk = key[i]; key[i] = key[q]; key[q] = tk;
                            int ti = id[i]; id[i] = id[q]; id[q] = ti;
                            double te = ev[i]; ev[i] = ev[q]; ev[q] = te;
                        }
                    }
                    __syncthreads();
                }
            }
            for (int i = threadIdx.x; i < n; i += blockDim.x) {
                sE[a + i] = ev[i];
                sid[a + i] = id[i];
            }
            __syncthreads();
        } else {
            double *ge = sE + a;
            int *gi = sid + a;
            for (int k = 2; k <= P; k <<= 1) {
                for (int j = k >> 1; j > 0; j >>= 1) {
                    for (int i = threadIdx.x; i < P; i += blockDim.x) {
                        const int q = (j == (k >> 1)) ? (i ^ (k - 1)) : (i ^ j);
                        if (q > i && q < n) {
                            const long long ki = order_key(ge[i]), kq = order_key(ge[q]);
                            if (pair_less(kq, gi[q], ki, gi[i])) {
                                double te = ge[i]; ge[i] = ge[q]; ge[q] = te;
                                int ti = gi[i]; gi[i] = gi[q]; gi[q] = ti;
                            }
                        }
                    }
                    __syncthreads();
                }
            }
        }
    }
}

// gradients into sorted order (zeros on padding positions)
__global__ void k_gather_gbar(const int *seg, const int *cnt, const int *sid, const double *gbar,
                              double *sg)
{
    const int total = seg[kMaterials];
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < total; p += gridDim.x * blockDim.x) {
        int m = 0;
        while (seg[m + 1] <= p) m++;
        const bool valid = p < seg[m] + cnt[m];
        const long id = valid ? sid[p] : 0;
#pragma unroll
        for (int c = 0; c < 5; c++) sg[(long)p * 5 + c] = valid ? gbar[id * 5 + c] : 0.0;
    }
}

// ------------------------------------------------------- prefix of gbar ---
// EP[p] = sum_{q < p} sg[q] per channel, over all P positions (padding holds
// zeros), by a three-phase scan with a fixed shape (the same additions in the
// same order on every run): tile sums, a one-block scan of the tile sums, a
// tile-local scan plus the tile's offset.  A tile is 1,024 positions x 5
// channels, staged through shared memory so that every global access is
// coalesced; each of the 256 threads owns 4 consecutive positions.
constexpr int kScanBlock = 1024;               // positions per tile
constexpr int kScanThreads2 = 256;
constexpr int kScanPer = kScanBlock / kScanThreads2;

// the tile's 5120 doubles into shared memory (zeros past `total`)
__device__ __forceinline__ void scan_stage(const double *sg, long tile0, int total, double *sh)
{
    const long base = tile0 * 5;
    const long end = (long)total * 5;
    for (int i = threadIdx.x; i < kScanBlock * 5; i += kScanThreads2)
        sh[i] = base + i < end ? sg[base + i] : 0.0;
}

// inclusive scan of v over the warp's lanes (fixed shape)
__device__ __forceinline__ double warp_incl(double v, int lane)
{
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const double u = __shfl_up_sync(0xffffffffu, v, o);
        if (lane >= o) v += u;
    }
    return v;
}

__global__ void __launch_bounds__(kScanThreads2) k_scan_blocks(const int *seg, const double *sg,
                                                               double *bsum)
{
    __shared__ double sh[kScanBlock * 5];
    __shared__ double wsum[kScanThreads2 / 32][5];
    const int total = seg[kMaterials];
    const int nblocks = (total + kScanBlock - 1) / kScanBlock;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int b = blockIdx.x; b < nblocks; b += gridDim.x) {
        scan_stage(sg, (long)b * kScanBlock, total, sh);
        __syncthreads();
        double v[5] = {0.0, 0.0, 0.0, 0.0, 0.0};
        for (int i = 0; i < kScanPer; i++) {
            const double *x = sh + (threadIdx.x * kScanPer + i) * 5;
#pragma unroll
            for (int c = 0; c < 5; c++) v[c] += x[c];
        }
#pragma unroll
        for (int c = 0; c < 5; c++) {
            const double w = warp_incl(v[c], lane);
            if (lane == 31) wsum[warp][c] = w;
        }
        __syncthreads();
        if (threadIdx.x < 5) {
            double t = 0.0;
            for (int w = 0; w < kScanThreads2 / 32; w++) t += wsum[w][threadIdx.x];
            bsum[(long)b * 5 + threadIdx.x] = t;
        }
        __syncthreads();
    }
}

// exclusive scan of the tile sums in one block: each thread a contiguous run
// of tiles, then a scan of the threads' totals
__global__ void __launch_bounds__(1024) k_scan_bsums(const int *seg, double *bsum)
{
    __shared__ double wtot[32][5];
    const int nblocks = (seg[kMaterials] + kScanBlock - 1) / kScanBlock;
    const int per = (nblocks + 1023) / 1024;
    const int a = threadIdx.x * per, e = min(nblocks, a + per);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    double tot[5] = {0.0, 0.0, 0.0, 0.0, 0.0};
    for (int b = a; b < e; b++)
#pragma unroll
        for (int c = 0; c < 5; c++) tot[c] += bsum[(long)b * 5 + c];
    double incl[5];
#pragma unroll
    for (int c = 0; c < 5; c++) {
        incl[c] = warp_incl(tot[c], lane);
        if (lane == 31) wtot[warp][c] = incl[c];
    }
    __syncthreads();
    if (threadIdx.x < 5) {   // exclusive scan of the 32 warp totals, in order
        double run = 0.0;
        for (int w = 0; w < 32; w++) {
            const double v = wtot[w][threadIdx.x];
            wtot[w][threadIdx.x] = run;
            run += v;
        }
    }
    __syncthreads();
    double run[5];
#pragma unroll
    for (int c = 0; c < 5; c++) run[c] = wtot[warp][c] + (incl[c] - tot[c]);
    for (int b = a; b < e; b++)
#pragma unroll
        for (int c = 0; c < 5; c++) {
            const double v = bsum[(long)b * 5 + c];
            bsum[(long)b * 5 + c] = run[c];
            run[c] += v;
        }
}

__global__ void __launch_bounds__(kScanThreads2) k_scan_local(const int *seg, const double *sg,
                                                              const double *bsum, double *ep)
{
    __shared__ double sh[kScanBlock * 5];
    __shared__ double woff[kScanThreads2 / 32][5];
    const int total = seg[kMaterials];
    const int nblocks = (total + kScanBlock - 1) / kScanBlock;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int b = blockIdx.x; b < nblocks; b += gridDim.x) {
        const long tile0 = (long)b * kScanBlock;
        scan_stage(sg, tile0, total, sh);
        __syncthreads();
        double v[5] = {0.0, 0.0, 0.0, 0.0, 0.0};
        for (int i = 0; i < kScanPer; i++) {
            const double *x = sh + (threadIdx.x * kScanPer + i) * 5;
#pragma unroll
            for (int c = 0; c < 5; c++) v[c] += x[c];
        }
        double incl[5];
#pragma unroll
        for (int c = 0; c < 5; c++) {
            incl[c] = warp_incl(v[c], lane);
            if (lane == 31) woff[warp][c] = incl[c];
        }
        __syncthreads();
        if (threadIdx.x < 5) {   // exclusive offsets of the 8 warps, plus the tile's
            double run = bsum[(long)b * 5 + threadIdx.x];
            for (int w = 0; w < kScanThreads2 / 32; w++) {
                const double t = woff[w][threadIdx.x];
                woff[w][threadIdx.x] = run;
                run += t;
            }
        }
        __syncthreads();
        double run[5];
#pragma unroll
        for (int c = 0; c < 5; c++) run[c] = woff[warp][c] + (incl[c] - v[c]);
        // exclusive prefix of each of the thread's positions, in place
        for (int i = 0; i < kScanPer; i++) {
            double *x = sh + (threadIdx.x * kScanPer + i) * 5;
#pragma unroll
            for (int c = 0; c < 5; c++) {
                const double t = x[c];
                x[c] = run[c];
                run[c] += t;
            }
        }
        // the prefix after the last position
        const int last = total - 1 - (int)tile0;
        if (last >= 0 && last / kScanPer == (int)threadIdx.x) {
            // run[] now holds the inclusive prefix of this thread's last position;
            // past the end of the data the staged zeros kept it unchanged
#pragma unroll
            for (int c = 0; c < 5; c++) ep[(long)total * 5 + c] = run[c];
        }
        __syncthreads();
        const long base = tile0 * 5, end = (long)total * 5;
        for (int i = threadIdx.x; i < kScanBlock * 5; i += kScanThreads2)
            if (base + i < end) ep[base + i] = sh[i];
        __syncthreads();
    }
}

// ---------------------------------------------------- transposed layout ---
struct AdjLayout {
    int nchunks[kMaterials];
    int group[kMaterials];     // lanes per chunk (power of two >= num_nucs, <= 32)
    int task_off[kMaterials + 1];
    long slot_base[kMaterials];
};

__global__ void k_adj_layout(Tables t, const int *cnt, AdjLayout *L)
{
    if (threadIdx.x != 0) return;
    int task = 0;
    long slot = 0;
    for (int m = 0; m < kMaterials; m++) {
        const int nn = t.num_nucs[m];
        int G = 1;
        while (G < nn && G < 32) G <<= 1;
        const int ngroups = (nn + G - 1) / G;
        const int S = 32 / G;
        const int nch = (cnt[m] + kAdjChunk - 1) / kAdjChunk;
        L->nchunks[m] = nch;
        L->group[m] = G;
        L->task_off[m] = task;
        L->slot_base[m] = slot;
        task += nn ? ngroups * ((nch + S - 1) / S) : 0;
        slot += (long)nn * nch * 2;
    }
    L->task_off[kMaterials] = task;
}

__device__ __forceinline__ void store10(double *dst, const double A[5], const double G[5])
{
#pragma unroll
    for (int c = 0; c < 5; c++) {
        dst[c] = A[c];
        dst[5 + c] = G[c];
    }
}

// The transposed pass (see the file comment, step 4).
__global__ void __launch_bounds__(256) k_adj_transposed(Tables t, const int *seg, const int *cnt,
                                                        const double *sE, const double *sg,
                                                        const double *ep, const AdjLayout *L,
                                                        unsigned int *queue, double *table,
                                                        double *slots)
{
    __shared__ AdjLayout lay;
    __shared__ int s_seg[kMaterials + 1], s_cnt[kMaterials];
    if (threadIdx.x == 0) lay = *L;
    if (threadIdx.x <= kMaterials) s_seg[threadIdx.x] = seg[threadIdx.x];
    if (threadIdx.x < kMaterials) s_cnt[threadIdx.x] = cnt[threadIdx.x];
    __syncthreads();
    const int lane = threadIdx.x & 31;
    const long n_int = t.n_gp - 1;
    for (;;) {
        unsigned int task = 0;
        if (lane == 0) task = atomicAdd(queue, 1u);
        task = __shfl_sync(0xffffffffu, task, 0);
        if ((int)task >= lay.task_off[kMaterials]) break;
        int m = 0;
        while (lay.task_off[m + 1] <= (int)task) m++;
        const int nn = t.num_nucs[m];
        const int G = lay.group[m], S = 32 / G;
        const int ngroups = (nn + G - 1) / G;
        const int lt = (int)task - lay.task_off[m];
        const int grp = lt % ngroups, cb = lt / ngroups;
        const int s = lane / G, jl = lane % G;
        const int j = grp * G + jl;
        const int c = cb * S + s;
        if (j < nn && c < lay.nchunks[m]) {
        const long a = s_seg[m] + (long)c * kAdjChunk;
        const long b = min((long)s_seg[m] + s_cnt[m], a + kAdjChunk);
        const int nuc = t.mats[m * t.max_nucs + j];
        const long long *ek = t.ekeys + (long)nuc * t.n_gp;
        double *tab = table + ((long)(t.pair_base[m] + j) * n_int) * kTbl;
        double *slot = slots + (lay.slot_base[m] + ((long)j * lay.nchunks[m] + c) * 2) * kSlot;

        // interval of the first energy: clamp(#{E_j <= E} - 1, 0, n_gp - 2)
        long k;
        {
            const long long q = order_key(sE[a]);
            long lo = 0, hi = t.n_gp;
            while (lo < hi) {
                long mid = (lo + hi) >> 1;
                if (ek[mid] <= q) lo = mid + 1; else hi = mid;
            }
            k = lo - 1;
            if (k < 0) k = 0;
            if (k > t.n_gp - 2) k = t.n_gp - 2;
        }
        const long k_first = k;
        long long next_key = (k + 1 <= t.n_gp - 2) ? ek[k + 1] : 0x7FFFFFFFFFFFFFFFLL;
        double e_hi = t.grid[(long)nuc * t.n_gp + k + 1].energy;
        double A[5] = {0, 0, 0, 0, 0}, Gs[5];
        long i_start = a;   // first position of the current interval in this chunk
        for (long i = a; i < b; i++) {
            const double E = sE[i];
            const long long q = order_key(E);
            if (q >= next_key) {
                // G over [i_start, i) from the prefix of gbar
#pragma unroll
                for (int cc = 0; cc < 5; cc++) Gs[cc] = ep[i * 5 + cc] - ep[i_start * 5 + cc];
                i_start = i;
                // leave interval k: the first one goes to slot 0, later ones into the table
                if (k == k_first) {
                    slot[0] = __longlong_as_double(k);
                    store10(slot + 1, A, Gs);
                } else {
                    store10(tab + k * kTbl, A, Gs);
                }
                do {
                    k++;
                    next_key = (k + 1 <= t.n_gp - 2) ? ek[k + 1] : 0x7FFFFFFFFFFFFFFFLL;
                } while (q >= next_key);
                e_hi = t.grid[(long)nuc * t.n_gp + k + 1].energy;
#pragma unroll
                for (int cc = 0; cc < 5; cc++) A[cc] = 0.0;
            }
            const double d = e_hi - E;
            const double *g = sg + i * 5;
#pragma unroll
            for (int cc = 0; cc < 5; cc++) A[cc] = fma(g[cc], d, A[cc]);
        }
#pragma unroll
        for (int cc = 0; cc < 5; cc++) Gs[cc] = ep[b * 5 + cc] - ep[i_start * 5 + cc];
        if (k == k_first) {
            slot[0] = __longlong_as_double(k);
            store10(slot + 1, A, Gs);
            slot[kSlot] = __longlong_as_double(-1LL);
        } else {
            slot[kSlot] = __longlong_as_double(k);
            store10(slot + kSlot + 1, A, Gs);
        }
        }
    }
}

// Boundary slots into the table.  Interval k's boundary pieces sit in
// consecutive chunks (the last interval of chunk c, the first of chunk c+1,
// and onwards while a chunk holds k only).  The chunk holding the first piece
// owns k and adds the pieces in chunk order, so the sum is deterministic;
// owners work in parallel over (pair, chunk, side).
__global__ void k_adj_fixup(Tables t, const AdjLayout *L, const double *slots, double *table)
{
    const long n_int = t.n_gp - 1;
    long total = 0;
    for (int m = 0; m < kMaterials; m++) total += (long)t.num_nucs[m] * L->nchunks[m] * 2;
    for (long w = (long)blockIdx.x * blockDim.x + threadIdx.x; w < total;
         w += (long)gridDim.x * blockDim.x) {
        int m = 0;
        while (m + 1 < kMaterials && L->slot_base[m + 1] <= w) m++;
        const long local = w - L->slot_base[m];
        const int nch = L->nchunks[m];
        const int j = (int)(local / (2L * nch));
        const int c = (int)((local / 2) % nch);
        const int side = (int)(local & 1);
        const double *base = slots + (L->slot_base[m] + (long)j * nch * 2) * kSlot;
        const double *sl = base + ((long)c * 2 + side) * kSlot;
        const long k = __double_as_longlong(sl[0]);
        if (k < 0) continue;
        if (side == 0 && c > 0) {
            // a chain started earlier owns k if the previous piece holds it
            const double *prev = base + ((long)(c - 1) * 2) * kSlot;
            const long k1 = __double_as_longlong(prev[kSlot]);
            const long kp = k1 >= 0 ? k1 : __double_as_longlong(prev[0]);
            if (kp == k) continue;
        }
        double acc[kTbl];
#pragma unroll
        for (int v = 0; v < kTbl; v++) acc[v] = sl[1 + v];
        // later chunks: their first piece continues the chain while it holds k
        for (int cc = c + 1; cc < nch; cc++) {
            const double *nx = base + ((long)cc * 2) * kSlot;
            if (__double_as_longlong(nx[0]) != k) break;
#pragma unroll
            for (int v = 0; v < kTbl; v++) acc[v] += nx[1 + v];
            if (__double_as_longlong(nx[kSlot]) >= 0) break;  // the chunk moved past k
        }
        double *dst = table + ((long)(t.pair_base[m] + j) * n_int + k) * kTbl;
#pragma unroll
        for (int v = 0; v < kTbl; v++) dst[v] += acc[v];
    }
}

// dL/dxs, one thread per (nuclide, gridpoint): the pairs holding the nuclide
// in material order; gridpoint p is the low end of interval p and the high
// end of interval p-1.
__global__ void k_adj_dxs(Tables t, const double *table, double *d_xs)
{
    const long npts = (long)t.n_iso * t.n_gp;
    const long n_int = t.n_gp - 1;
    for (long idx = (long)blockIdx.x * blockDim.x + threadIdx.x; idx < npts;
         idx += (long)gridDim.x * blockDim.x) {
        const int n = (int)(idx / t.n_gp);
        const long p = idx - (long)n * t.n_gp;
        const xs_gridpoint *g = t.grid + (long)n * t.n_gp;
        double inv_lo = 0.0, inv_hi = 0.0;  // 1 / width of intervals p and p-1
        if (p <= t.n_gp - 2) inv_lo = 1.0 / (g[p + 1].energy - g[p].energy);
        if (p >= 1) inv_hi = 1.0 / (g[p].energy - g[p - 1].energy);
        double out[5] = {0, 0, 0, 0, 0};
        for (int q = t.inv_off[n]; q < t.inv_off[n + 1]; q++) {
            const int mj = t.inv_pair[q];
            const int m = mj / t.max_nucs, j = mj - m * t.max_nucs;
            const double conc = t.concs[mj];
            const double *tab = table + (long)(t.pair_base[m] + j) * n_int * kTbl;
            if (p <= t.n_gp - 2) {
                const double *e = tab + p * kTbl;   // interval p: gridpoint p is its low end
#pragma unroll
                for (int c = 0; c < 5; c++) out[c] = fma(conc, e[c] * inv_lo, out[c]);
            }
            if (p >= 1) {
                const double *e = tab + (p - 1) * kTbl;   // interval p-1: high end
#pragma unroll
                for (int c = 0; c < 5; c++) out[c] = fma(conc, e[5 + c] - e[c] * inv_hi, out[c]);
            }
        }
#pragma unroll
        for (int c = 0; c < 5; c++) d_xs[idx * 5 + c] += out[c];
    }
}

// dL/dconcs, one block per pair: threads stride over intervals, then a
// fixed-shape tree.
__global__ void __launch_bounds__(256) k_adj_dconc(Tables t, const double *table, double *d_concs)
{
    __shared__ double red[256];
    const int pair = blockIdx.x;
    int m = 0;
    while (t.pair_base[m + 1] <= pair) m++;
    const int j = pair - t.pair_base[m];
    const int nuc = t.mats[m * t.max_nucs + j];
    const xs_gridpoint *g = t.grid + (long)nuc * t.n_gp;
    const long n_int = t.n_gp - 1;
    const double *tab = table + (long)pair * n_int * kTbl;
    double acc = 0.0;
    for (long k = threadIdx.x; k < n_int; k += blockDim.x) {
        const xs_gridpoint lo = g[k], hi = g[k + 1];
        const double inv = 1.0 / (hi.energy - lo.energy);
        const double hv[5] = {hi.total_xs, hi.elastic_xs, hi.absorbtion_xs, hi.fission_xs, hi.nu_fission_xs};
        const double lv[5] = {lo.total_xs, lo.elastic_xs, lo.absorbtion_xs, lo.fission_xs, lo.nu_fission_xs};
        const double *e = tab + k * kTbl;
#pragma unroll
        for (int c = 0; c < 5; c++) acc += hv[c] * e[5 + c] - (hv[c] - lv[c]) * (e[c] * inv);
    }
    red[threadIdx.x] = acc;
    __syncthreads();
    for (int w = 128; w > 0; w >>= 1) {
        if (threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
        __syncthreads();
    }
    if (threadIdx.x == 0) d_concs[m * t.max_nucs + j] += red[0];
}

static size_t align256(size_t b) { return (b + 255) & ~(size_t)255; }

xs_status launch_adjoint(xs_ctx *ctx, cudaStream_t st, long first, long count,
                         const SampleInput &in, const double *gbar, double *macro_out,
                         double *d_concs, double *d_xs, double *d_energy, int *launches)
{
    const Tables &t = ctx->t;
    if (count > 0x7FFFFFFFL - kMaterials * 32)
        return fail(XS_ERR_INVALID_ARGUMENT, "the adjoint takes at most 2^31 - 385 lookups per call");
    if (!t.ekeys || !t.inv_off) return fail(XS_ERR_UNSUPPORTED, "adjoint tables missing");
    const int nb = 1 << kAdjBucketLog2;
    const size_t padded = (size_t)count + kMaterials * 32;
    const long n_int = t.n_gp - 1;
    const int pairs = t.pair_base[kMaterials];
    long max_nn = 0;
    for (int m = 0; m < kMaterials; m++) max_nn = std::max<long>(max_nn, t.pair_base[m + 1] - t.pair_base[m]);
    const size_t slot_count = (size_t)(max_nn * (count / kAdjChunk + 1) + pairs) * 2 + 2 * kMaterials;
    size_t off = 0;
    const size_t o_offs = off; off = align256(off + (size_t)kMaterials * nb * 4);
    const size_t o_starts = off; off = align256(off + (size_t)kMaterials * nb * 4);
    const size_t o_seg = off; off = align256(off + 256);
    const size_t o_layout = off; off = align256(off + sizeof(AdjLayout));
    const size_t o_queue = off; off = align256(off + 64);
    const size_t o_sE = off; off = align256(off + padded * 8);
    const size_t o_sid = off; off = align256(off + padded * 4);
    const size_t o_sg = off; off = align256(off + padded * 40);
    const size_t o_ep = off; off = align256(off + (padded + 1) * 40);
    const size_t o_bsum = off; off = align256(off + (padded / kScanBlock + 2) * 40);
    const size_t o_table = off; off = align256(off + (size_t)pairs * n_int * kTbl * 8);
    const size_t o_slots = off; off = align256(off + slot_count * kSlot * 8);
    const size_t need = off;
    if (ctx->s.adj_bytes < need) {
        if (ctx->s.adj_buf) {
            cudaFree(ctx->s.adj_buf);
            ctx->device_bytes -= ctx->s.adj_bytes;
            ctx->s.adj_buf = nullptr;
            ctx->s.adj_bytes = 0;
        }
        cudaError_t e = cudaMalloc(&ctx->s.adj_buf, need);
        if (e != cudaSuccess) {
            cudaGetLastError();
            return fail(XS_ERR_OUT_OF_MEMORY, "adjoint scratch of %zu bytes", need);
        }
        ctx->s.adj_bytes = need;
        ctx->device_bytes += need;
    }
    char *B = (char *)ctx->s.adj_buf;
    int *offs = (int *)(B + o_offs), *starts = (int *)(B + o_starts);
    int *seg = (int *)(B + o_seg), *cnt = seg + 16;
    AdjLayout *L = (AdjLayout *)(B + o_layout);
    unsigned int *queue = (unsigned int *)(B + o_queue);
    double *sE = (double *)(B + o_sE);
    int *sid = (int *)(B + o_sid);
    double *sg = (double *)(B + o_sg);
    double *ep = (double *)(B + o_ep);
    double *bsum = (double *)(B + o_bsum);
    double *table = (double *)(B + o_table);
    double *slots = (double *)(B + o_slots);

    xs_status s = enqueue_sort_only(ctx, st, first, count, kAdjBucketLog2, in, offs, starts, seg,
                                    cnt, sE, sid);
    if (s != XS_OK) return s;
    const int nbuckets = kMaterials * nb;
    k_bucket_sort<<<std::min(nbuckets, ctx->sm_count * 8), 256, 0, st>>>(starts, offs, nbuckets, sE, sid);
    XS_CUDA(cudaGetLastError());
    k_gather_gbar<<<ctx->sm_count * 8, 256, 0, st>>>(seg, cnt, sid, gbar, sg);
    XS_CUDA(cudaGetLastError());

    // forward and dL/dE per lookup
    XS_CUDA(cudaMemsetAsync(queue, 0, 64, st));
    ListArgs l;
    l.seg_v = seg;
    l.cnt = cnt;
    l.base = nullptr;
    l.E = sE;
    l.id = sid;
    l.queue = queue;
    l.out_macro = macro_out;
    l.out_idx = nullptr;
    l.verif = ctx->s.verification;
    l.err = ctx->s.error;
    l.fuel_lanes = 1;
    l.table = 1;   // the forward reads the union table when there is one
    s = launch_adjoint_energy(ctx, st, l, sg, d_energy);
    if (s != XS_OK) return s;

    int n = 7;
    if (d_xs || d_concs) {
        XS_CUDA(cudaMemsetAsync(table, 0, (size_t)pairs * n_int * kTbl * 8, st));
        XS_CUDA(cudaMemsetAsync(queue + 4, 0, 4, st));
        k_adj_layout<<<1, 32, 0, st>>>(t, cnt, L);
        XS_CUDA(cudaGetLastError());
        k_scan_blocks<<<ctx->sm_count * 4, kScanThreads2, 0, st>>>(seg, sg, bsum);
        k_scan_bsums<<<1, 1024, 0, st>>>(seg, bsum);
        k_scan_local<<<ctx->sm_count * 4, kScanThreads2, 0, st>>>(seg, sg, bsum, ep);
        XS_CUDA(cudaGetLastError());
        k_adj_transposed<<<ctx->sm_count * 4, 256, 0, st>>>(t, seg, cnt, sE, sg, ep, L, queue + 4, table, slots);
        XS_CUDA(cudaGetLastError());
        k_adj_fixup<<<ctx->sm_count * 8, 256, 0, st>>>(t, L, slots, table);
        XS_CUDA(cudaGetLastError());
        n += 6;
        if (d_xs) {
            const long npts = (long)t.n_iso * t.n_gp;
            const long want = (npts + 255) / 256;
            k_adj_dxs<<<(unsigned)std::min<long>(want, (long)ctx->sm_count * 32), 256, 0, st>>>(t, table, d_xs);
            XS_CUDA(cudaGetLastError());
            n++;
        }
        if (d_concs) {
            k_adj_dconc<<<pairs, 256, 0, st>>>(t, table, d_concs);
            XS_CUDA(cudaGetLastError());
            n++;
        }
    }
    if (launches) *launches += n;
    return XS_OK;
}

}  // namespace xsgb
