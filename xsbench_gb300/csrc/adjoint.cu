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
//   2-3. per lookup: forward macro_xs and dL/dE (interval search
//      recomputed), the upstream gradients gathered into sorted order on
//      the way;
//   4. chunk-local prefixes of g and g (E - Eref) over each chunk of 2,048
//      sorted lookups; transposed pass: lanes take a chunk's nuclides, and each
//      lane walks its nuclide's intervals across the chunk, finding the end of
//      each interval's run of lookups by a galloping search and taking
//      G_kc = sum g_ic and A_kc = sum g_ic (E_hi - E_i) from the prefixes;
//      intervals inside the chunk are stored, the first and last go to
//      per-chunk boundary slots;
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
constexpr int kSubRun = 32;            // longest sub-bucket sorted by insertion

// Sub-bucket of order key k among nsub equal key ranges of [kmin, kmax]: a
// non-decreasing function of k (the conversion to double, the product with a
// positive scale and the truncation are each monotone).
__device__ __forceinline__ int sub_of(long long k, long long kmin, double scale, int nsub)
{
    const int s = (int)((double)((unsigned long long)k - (unsigned long long)kmin) * scale);
    return s < nsub - 1 ? s : nsub - 1;
}

// Block-wide min and max (256 threads); every thread gets the results.
__device__ __forceinline__ void block_minmax(long long &lo, long long &hi, long long *red)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        const long long a = __shfl_xor_sync(0xffffffffu, lo, o), b = __shfl_xor_sync(0xffffffffu, hi, o);
        lo = a < lo ? a : lo;
        hi = b > hi ? b : hi;
    }
    const int w = threadIdx.x >> 5;
    if ((threadIdx.x & 31) == 0) {
        red[w] = lo;
        red[8 + w] = hi;
    }
    __syncthreads();
    lo = red[0];
    hi = red[8];
    for (int i = 1; i < 8; i++) {
        lo = red[i] < lo ? red[i] : lo;
        hi = red[8 + i] > hi ? red[8 + i] : hi;
    }
    __syncthreads();
}

// Exclusive scan of c[0, n) in place, n <= 1024 (256 threads, four each).
__device__ __forceinline__ void block_scan_1024(int *c, int n, long long *red)
{
    const int t = threadIdx.x;
    int v[4], sum = 0;
#pragma unroll
    for (int q = 0; q < 4; q++) {
        v[q] = (4 * t + q < n) ? c[4 * t + q] : 0;
        sum += v[q];
    }
    int inc = sum;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int x = __shfl_up_sync(0xffffffffu, inc, o);
        if ((t & 31) >= o) inc += x;
    }
    int *wsum = reinterpret_cast<int *>(red);
    if ((t & 31) == 31) wsum[t >> 5] = inc;
    __syncthreads();
    int base = 0;
    for (int i = 0; i < (t >> 5); i++) base += wsum[i];
    int run = base + inc - sum;
#pragma unroll
    for (int q = 0; q < 4; q++) {
        if (4 * t + q < n) c[4 * t + q] = run;
        run += v[q];
    }
    __syncthreads();
}

// One block per bucket: sort the bucket's (energy, id) entries by (order key
// of the energy, id).  A bucket of up to kSortCap entries is loaded into
// shared memory and spread over n/2 sub-buckets, equal ranges of its keys
// (the keys of one bucket are close to uniform): a counting pass, a scan,
// a scatter of entry indices, then each thread sorts one sub-bucket (about
// two entries) by insertion on (key, id).  The order is the unique (key, id)
// order whatever the scatter's arrival order, so the result is deterministic.
// A bucket whose keys crowd one sub-bucket (more than kSubRun entries, e.g.
// repeated energies) takes the bitonic network in shared memory instead, and
// a bucket larger than kSortCap the same network in place in global memory;
// both use its all-ascending form (first step of each merge pairs i with
// i ^ (k-1)), so positions past the bucket act as +infinity and never move.
// Dynamic shared memory: bucket_sort_smem_bytes().
__global__ void __launch_bounds__(256) k_bucket_sort(const int *starts, const int *ends,
                                                     int nbuckets, double *sE, int *sid)
{
    extern __shared__ __align__(16) unsigned char bsm[];
    long long *key = reinterpret_cast<long long *>(bsm);
    double *ev = reinterpret_cast<double *>(key + kSortCap);
    int *id = reinterpret_cast<int *>(ev + kSortCap);
    int *cur = id + kSortCap;                                            // [kSortCap / 2]
    unsigned short *perm = reinterpret_cast<unsigned short *>(cur + kSortCap / 2);
    __shared__ long long red[16];
    for (int b = blockIdx.x; b < nbuckets; b += gridDim.x) {
        const int a = starts[b], n = ends[b] - a;
        if (n <= 1) continue;
        int P = 1;
        while (P < n) P <<= 1;
        if (n <= kSortCap) {
            long long lo = 0x7FFFFFFFFFFFFFFFLL, hi = -0x7FFFFFFFFFFFFFFFLL - 1;
            for (int i = threadIdx.x; i < P; i += blockDim.x) {
                if (i < n) {
                    ev[i] = sE[a + i];
                    key[i] = order_key(ev[i]);
                    id[i] = sid[a + i];
                    lo = key[i] < lo ? key[i] : lo;
                    hi = key[i] > hi ? key[i] : hi;
                } else {
                    key[i] = 0x7FFFFFFFFFFFFFFFLL;
                    id[i] = 0x7FFFFFFF;
                    ev[i] = 0.0;
                }
            }
            block_minmax(lo, hi, red);   // (its barriers also publish the loads)
            const int nsub = n >> 1;
            const double scale =
                (double)nsub / ((double)((unsigned long long)hi - (unsigned long long)lo) + 1.0);
            for (int s = threadIdx.x; s < nsub; s += blockDim.x) cur[s] = 0;
            __syncthreads();
            for (int i = threadIdx.x; i < n; i += blockDim.x)
                atomicAdd(&cur[sub_of(key[i], lo, scale, nsub)], 1);
            __syncthreads();
            long long most = 0, unused = 0;
            for (int s = threadIdx.x; s < nsub; s += blockDim.x) most = cur[s] > most ? cur[s] : most;
            block_minmax(unused, most, red);
            if (most <= kSubRun) {
                block_scan_1024(cur, nsub, red);
                for (int i = threadIdx.x; i < n; i += blockDim.x)
                    perm[atomicAdd(&cur[sub_of(key[i], lo, scale, nsub)], 1)] = (unsigned short)i;
                __syncthreads();
                // cur[s] is now the end of sub-bucket s
                for (int s = threadIdx.x; s < nsub; s += blockDim.x) {
                    const int s0 = s ? cur[s - 1] : 0, s1 = cur[s];
                    for (int i = s0 + 1; i < s1; i++) {
                        const unsigned short x = perm[i];
                        const long long kx = key[x];
                        const int ix = id[x];
                        int j = i - 1;
                        while (j >= s0 && pair_less(kx, ix, key[perm[j]], id[perm[j]])) {
                            perm[j + 1] = perm[j];
                            j--;
                        }
                        perm[j + 1] = x;
                    }
                }
                __syncthreads();
                for (int i = threadIdx.x; i < n; i += blockDim.x) {
                    const int x = perm[i];
                    sE[a + i] = ev[x];
                    sid[a + i] = id[x];
                }
                __syncthreads();
                continue;
            }
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

size_t bucket_sort_smem_bytes()
{
    return (size_t)kSortCap * (8 + 8 + 4 + 2) + (size_t)(kSortCap / 2) * 4;
}

cudaError_t launch_bucket_sort(const int *starts, const int *ends, int nbuckets, double *sE,
                               int *sid, int blocks, cudaStream_t st)
{
    const size_t sm = bucket_sort_smem_bytes();
    cudaError_t e = cudaFuncSetAttribute(k_bucket_sort, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)sm);
    if (e != cudaSuccess) return e;
    k_bucket_sort<<<blocks, 256, sm, st>>>(starts, ends, nbuckets, sE, sid);
    return cudaGetLastError();
}

// ---------------------------------------------------- transposed layout ---
struct AdjLayout {
    int nchunks[kMaterials];
    int group[kMaterials];     // lanes per chunk (power of two >= num_nucs, <= 32)
    int task_off[kMaterials + 1];
    long slot_base[kMaterials];
    int chunk_off[kMaterials + 1];  // global number of each material's first chunk
};

__global__ void k_adj_layout(Tables t, const int *cnt, AdjLayout *L)
{
    if (threadIdx.x != 0) return;
    int task = 0, chunks = 0;
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
        L->chunk_off[m] = chunks;
        task += nn ? ngroups * ((nch + S - 1) / S) : 0;
        slot += (long)nn * nch * 2;
        chunks += nch;
    }
    L->task_off[kMaterials] = task;
    L->chunk_off[kMaterials] = chunks;
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

// ------------------------------------------------- chunk-local prefixes ---
// For chunk (m, c) = sorted positions [a, b) with Eref = sE[a]: at entry
// a + gc + (i - a), i in [a, b], the exclusive prefixes over [a, i) of
//   g_c             (5 doubles)  and   g_c * (E - Eref)   (5 doubles),
// gc being the chunk's global number (one extra entry per chunk).  Local
// prefixes keep the terms and the differences taken from them small; one
// block per chunk, 8 consecutive positions per thread, a fixed-shape scan.
constexpr int kPreThreads = kAdjChunk / 8;

__global__ void __launch_bounds__(kPreThreads) k_adj_prefix(const int *seg, const int *cnt,
                                                            const AdjLayout *L, const double *sE,
                                                            const double *sg, double *pre)
{
    __shared__ double woff[kPreThreads / 32][10];
    const int total = L->chunk_off[kMaterials];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int gc = blockIdx.x; gc < total; gc += gridDim.x) {
        int m = 0;
        while (L->chunk_off[m + 1] <= gc) m++;
        const int c = gc - L->chunk_off[m];
        const long a = seg[m] + (long)c * kAdjChunk;
        const long b = min((long)seg[m] + cnt[m], a + kAdjChunk);
        const double eref = sE[a];
        const long i0 = a + (long)threadIdx.x * 8, i1 = min(b, i0 + 8);
        double v[10];
#pragma unroll
        for (int k = 0; k < 10; k++) v[k] = 0.0;
        for (long i = i0; i < i1; i++) {
            const double de = sE[i] - eref;
#pragma unroll
            for (int k = 0; k < 5; k++) {
                const double g = sg[i * 5 + k];
                v[k] += g;
                v[5 + k] = fma(g, de, v[5 + k]);
            }
        }
        double incl[10];
#pragma unroll
        for (int k = 0; k < 10; k++) {
            incl[k] = warp_incl(v[k], lane);
            if (lane == 31) woff[warp][k] = incl[k];
        }
        __syncthreads();
        if (threadIdx.x < 10) {
            double run = 0.0;
            for (int w = 0; w < kPreThreads / 32; w++) {
                const double t = woff[w][threadIdx.x];
                woff[w][threadIdx.x] = run;
                run += t;
            }
        }
        __syncthreads();
        double run[10];
#pragma unroll
        for (int k = 0; k < 10; k++) run[k] = woff[warp][k] + (incl[k] - v[k]);
        double *out = pre + (a + gc) * 10;
        for (long i = i0; i < i1; i++) {
            double *o = out + (i - a) * 10;
            const double de = sE[i] - eref;
#pragma unroll
            for (int k = 0; k < 10; k++) o[k] = run[k];
#pragma unroll
            for (int k = 0; k < 5; k++) {
                const double g = sg[i * 5 + k];
                run[k] += g;
                run[5 + k] = fma(g, de, run[5 + k]);
            }
        }
        if (i1 == b && i0 < b) {
#pragma unroll
            for (int k = 0; k < 10; k++) out[(b - a) * 10 + k] = run[k];
        }
        __syncthreads();
    }
}

__device__ __forceinline__ void store10(double *dst, const double A[5], const double G[5])
{
#pragma unroll
    for (int c = 0; c < 5; c++) {
        dst[c] = A[c];
        dst[5 + c] = G[c];
    }
}

// The transposed pass (see the file comment, step 4).  A lane takes one
// nuclide of the chunk's material and walks the nuclide's intervals across
// the chunk's sorted energies: the end of each interval's run of lookups is
// found by a galloping search, and its sums come from the chunk-local
// prefixes: G = dP_g, A = sum g (E_hi - E) = (E_hi - Eref) G - dP_gE.
__global__ void __launch_bounds__(256) k_adj_transposed(Tables t, const int *seg, const int *cnt,
                                                        const double *sE, const double *pre,
                                                        const AdjLayout *L, unsigned int *queue,
                                                        double *table, double *slots)
{
    __shared__ AdjLayout lay;
    __shared__ int s_seg[kMaterials + 1], s_cnt[kMaterials];
    if (threadIdx.x == 0) lay = *L;
    if (threadIdx.x <= kMaterials) s_seg[threadIdx.x] = seg[threadIdx.x];
    if (threadIdx.x < kMaterials) s_cnt[threadIdx.x] = cnt[threadIdx.x];
    __syncthreads();
    const int lane = threadIdx.x & 31;
    const long n_int = t.n_gp - 1;
    const long top = t.n_gp - 2;   // last interval
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
        if (j >= nn || c >= lay.nchunks[m]) continue;
        const long a = s_seg[m] + (long)c * kAdjChunk;
        const long b = min((long)s_seg[m] + s_cnt[m], a + kAdjChunk);
        const double eref = sE[a];
        const double *P = pre + (a + lay.chunk_off[m] + c) * 10;   // entry of position i: P[(i-a)*10]
        const int nuc = t.mats[m * t.max_nucs + j];
        const long long *ek = t.ekeys + (long)nuc * t.n_gp;
        const xs_gridpoint *gp = t.grid + (long)nuc * t.n_gp;
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
            if (k > top) k = top;
        }
        const long k_first = k;
        long pos = a;
        for (;;) {
            // the run of interval k: [pos, end), end = first i with key(E_i) >= ek[k+1]
            long end = b;
            if (k < top) {
                const long long nk = ek[k + 1];
                long lo = pos, step = 1;   // key(E_lo) < nk
                long hi = b;
                for (;;) {
                    const long probe = lo + step;
                    if (probe >= b) break;
                    if (order_key(sE[probe]) >= nk) {
                        hi = probe;
                        break;
                    }
                    lo = probe;
                    step <<= 1;
                }
                while (hi - lo > 1) {
                    const long mid = lo + ((hi - lo) >> 1);
                    if (order_key(sE[mid]) >= nk) hi = mid; else lo = mid;
                }
                end = hi;
            }
            const double *p0 = P + (pos - a) * 10, *p1 = P + (end - a) * 10;
            const double dh = gp[k + 1].energy - eref;
            double A[5], Gs[5];
#pragma unroll
            for (int cc = 0; cc < 5; cc++) {
                Gs[cc] = p1[cc] - p0[cc];
                A[cc] = fma(dh, Gs[cc], -(p1[5 + cc] - p0[5 + cc]));
            }
            if (end == b) {   // the chunk's last interval (possibly also its first)
                if (k == k_first) {
                    slot[0] = __longlong_as_double(k);
                    store10(slot + 1, A, Gs);
                    slot[kSlot] = __longlong_as_double(-1LL);
                } else {
                    slot[kSlot] = __longlong_as_double(k);
                    store10(slot + kSlot + 1, A, Gs);
                }
                break;
            }
            if (k == k_first) {
                slot[0] = __longlong_as_double(k);
                store10(slot + 1, A, Gs);
            } else {
                store10(tab + k * kTbl, A, Gs);
            }
            // the interval of E_end: the largest j > k with ek[j] <= key(E_end),
            // capped at the last interval (ek[k+1] <= key(E_end) here)
            const long long q = order_key(sE[end]);
            const long last = t.n_gp - 1;
            long lo = k + 1, step = 1;   // ek[lo] <= q
            while (lo + step <= last && ek[lo + step] <= q) {
                lo += step;
                step <<= 1;
            }
            long hi = min(lo + step, last + 1);   // ek[hi] > q, or hi == n_gp
            while (hi - lo > 1) {
                const long mid = lo + ((hi - lo) >> 1);
                if (ek[mid] <= q) lo = mid; else hi = mid;
            }
            k = lo < top ? lo : top;
            pos = end;
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
    const size_t o_pre = off; off = align256(off + (padded + count / kAdjChunk + kMaterials + 1) * 80);
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
    double *pre = (double *)(B + o_pre);
    double *table = (double *)(B + o_table);
    double *slots = (double *)(B + o_slots);

    xs_status s = enqueue_sort_only(ctx, st, first, count, kAdjBucketLog2, in, offs, starts, seg,
                                    cnt, sE, sid);
    if (s != XS_OK) return s;
    const int nbuckets = kMaterials * nb;
    XS_CUDA(launch_bucket_sort(starts, offs, nbuckets, sE, sid, std::min(nbuckets, ctx->sm_count * 8), st));

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
    l.sorted = 1;
    l.block = 256;
    s = launch_adjoint_energy(ctx, st, l, gbar, sg, d_energy);
    if (s != XS_OK) return s;

    int n = 6;
    if (d_xs || d_concs) {
        XS_CUDA(cudaMemsetAsync(table, 0, (size_t)pairs * n_int * kTbl * 8, st));
        XS_CUDA(cudaMemsetAsync(queue + 4, 0, 4, st));
        k_adj_layout<<<1, 32, 0, st>>>(t, cnt, L);
        XS_CUDA(cudaGetLastError());
        k_adj_prefix<<<ctx->sm_count * 8, kPreThreads, 0, st>>>(seg, cnt, L, sE, sg, pre);
        XS_CUDA(cudaGetLastError());
        k_adj_transposed<<<ctx->sm_count * 4, 256, 0, st>>>(t, seg, cnt, sE, pre, L, queue + 4, table, slots);
        XS_CUDA(cudaGetLastError());
        k_adj_fixup<<<ctx->sm_count * 8, 256, 0, st>>>(t, L, slots, table);
        XS_CUDA(cudaGetLastError());
        n += 4;
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
