// capi.cu -- the extern "C" entry points of include/xsgb.h: contexts,
// runs, the caller-sample pipeline, and error reporting.
#include <algorithm>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "device_common.cuh"
#include "pipeline_chunks.h"

namespace xsgb {

static thread_local std::string g_last_error;

xs_status fail(xs_status s, const char *fmt, ...)
{
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    g_last_error = buf;
    return s;
}

xs_status cuda_fail(cudaError_t e, const char *what)
{
    cudaGetLastError();  // clear a sticky launch error where it is not fatal
    if (e == cudaErrorMemoryAllocation)
        return fail(XS_ERR_OUT_OF_MEMORY, "%s: %s", what, cudaGetErrorString(e));
    return fail(XS_ERR_CUDA, "%s: %s", what, cudaGetErrorString(e));
}

xs_status ctx_alloc(xs_ctx *ctx, void **p, size_t bytes)
{
    *p = nullptr;
    // whole 256-byte units, so a 16-byte-rounded bulk prefetch of the last
    // entries stays inside the allocation
    bytes = (bytes + 255) & ~(size_t)255;
    if (bytes == 0) bytes = 256;
    cudaError_t e = cudaMalloc(p, bytes);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return fail(XS_ERR_OUT_OF_MEMORY, "device allocation of %zu bytes failed (%s)", bytes,
                    cudaGetErrorString(e));
    }
    ctx->allocations.push_back(*p);
    ctx->device_bytes += bytes;
    return XS_OK;
}

template <typename T>
static xs_status upload(xs_ctx *ctx, const T *host, size_t n, const T **dev)
{
    void *p = nullptr;
    xs_status s = ctx_alloc(ctx, &p, n * sizeof(T));
    if (s != XS_OK) return s;
    if (n) XS_CUDA(cudaMemcpyAsync(p, host, n * sizeof(T), cudaMemcpyHostToDevice, ctx->stream));
    *dev = (const T *)p;
    return XS_OK;
}

static bool is_device_pointer(const void *p)
{
    if (!p) return false;
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged;
}

static xs_status ensure_stage(xs_ctx *ctx, size_t bytes)
{
    if (ctx->s.stage_bytes >= bytes) return XS_OK;
    if (ctx->s.stage) {
        cudaFree(ctx->s.stage);
        ctx->device_bytes -= ctx->s.stage_bytes;
        ctx->s.stage = nullptr;
        ctx->s.stage_bytes = 0;
        for (auto &kv : ctx->graphs) cudaGraphExecDestroy(kv.second.exec);
        ctx->graphs.clear();
    }
    cudaError_t e = cudaMalloc(&ctx->s.stage, bytes);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return fail(XS_ERR_OUT_OF_MEMORY, "staging buffer of %zu bytes", bytes);
    }
    ctx->s.stage_bytes = bytes;
    ctx->device_bytes += bytes;
    return XS_OK;
}

static xs_status ensure_plain(xs_ctx *ctx, size_t bytes)
{
    if (ctx->s.plain_bytes >= bytes) return XS_OK;
    if (ctx->s.plain_buf) {
        cudaFree(ctx->s.plain_buf);
        ctx->device_bytes -= ctx->s.plain_bytes;
        ctx->s.plain_buf = nullptr;
        ctx->s.plain_bytes = 0;
    }
    cudaError_t e = cudaMalloc(&ctx->s.plain_buf, bytes);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return fail(XS_ERR_OUT_OF_MEMORY, "overflow queues of %zu bytes", bytes);
    }
    ctx->s.plain_bytes = bytes;
    ctx->device_bytes += bytes;
    return XS_OK;
}

// Plain runs of more than a few tiles send each tile's partial chunks to the
// overflow queues (two more launches); short runs keep them in the tile.  On
// the nuclide grid the queued lookups cost more (long unsorted searches in
// fewer resident warps) than the idle lanes they save, so it keeps them too.
static bool use_overflow(const xs_ctx *ctx, long count, int tile)
{
    if (ctx->overflow >= 0) return ctx->overflow && count > 8L * tile;
    // with the guided searches the nuclide grid gains from the pass too
    // (XL: 626 -> 664 M lookups/s); its own binary search does not
    return (ctx->t.grid_type != XS_NUCLIDE || ctx->t.binrec) && count > 8L * tile;
}

static xs_status resolve(const xs_ctx *ctx, const xs_run_opts *o, long total, xs_run_opts *r)
{
    xs_run_opts_init(r);
    if (o) *r = *o;
    if (r->kernel != XS_KERNEL_PLAIN && r->kernel != XS_KERNEL_BATCHED)
        return fail(XS_ERR_INVALID_ARGUMENT, "unknown kernel %d", r->kernel);
    if (r->arith != XS_ARITH_FAST && r->arith != XS_ARITH_EXACT)
        return fail(XS_ERR_INVALID_ARGUMENT, "unknown arithmetic %d", r->arith);
    if (r->first < 0) return fail(XS_ERR_INVALID_ARGUMENT, "first %ld < 0", r->first);
    if (r->count <= 0) r->count = total - r->first;
    if (r->count <= 0) return fail(XS_ERR_INVALID_ARGUMENT, "no lookups in range");
    if (r->tile_lookups <= 0) r->tile_lookups = ctx->plain_tile;
    if (r->energy_buckets <= 0) r->energy_buckets = ctx->batched_buckets;
    if (r->block_threads != 0 && r->block_threads != 128 && r->block_threads != 256 &&
        r->block_threads != 512)
        return fail(XS_ERR_INVALID_ARGUMENT, "block_threads %d: 0 (tuned), 128, 256 or 512",
                    r->block_threads);
    return XS_OK;
}

static xs_status read_back(xs_ctx *ctx, cudaStream_t st, xs_run_result *res)
{
    unsigned long long *h = (unsigned long long *)ctx->h_result;
    XS_CUDA(cudaMemcpyAsync(h, ctx->s.verification, 8, cudaMemcpyDeviceToHost, st));
    XS_CUDA(cudaMemcpyAsync(h + 1, ctx->s.error, 16, cudaMemcpyDeviceToHost, st));
    XS_CUDA(cudaStreamSynchronize(st));
    const int *err = (const int *)(h + 1);
    float ms = 0.f;
    if (cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1) != cudaSuccess) {
        cudaGetLastError();
        ms = 0.f;
    }
    if (res) {
        res->verification = h[0];
        res->device_ms = ms;
    }
    if (err[0])
        return fail((xs_status)err[0], "device check failed: entry %d, value %d", err[1], err[2]);
    return XS_OK;
}

}  // namespace xsgb

using namespace xsgb;

extern "C" {

const char *xs_status_str(xs_status s)
{
    switch (s) {
    case XS_OK: return "ok";
    case XS_ERR_INVALID_ARGUMENT: return "invalid argument";
    case XS_ERR_OUT_OF_MEMORY: return "out of memory";
    case XS_ERR_CUDA: return "CUDA error";
    case XS_ERR_NO_DEVICE: return "no usable device";
    case XS_ERR_TIMEOUT: return "device wait timed out";
    case XS_ERR_DATA: return "table or sample out of range";
    case XS_ERR_UNSUPPORTED: return "unsupported";
    case XS_ERR_IO: return "I/O error";
    }
    return "unknown status";
}

const char *xs_last_error(void) { return g_last_error.c_str(); }

void xs_run_opts_init(xs_run_opts *o)
{
    if (!o) return;
    std::memset(o, 0, sizeof *o);
    o->kernel = XS_KERNEL_PLAIN;
    o->arith = XS_ARITH_FAST;
}

size_t xs_ctx_device_bytes(const xs_ctx *ctx) { return ctx ? ctx->device_bytes : 0; }

size_t xs_ctx_union_table_bytes(const xs_ctx *ctx) { return ctx ? ctx->union_table_bytes : 0; }

void xs_ctx_destroy(xs_ctx *ctx)
{
    if (!ctx) return;
    cudaSetDevice(ctx->device);
    if (ctx->stream) cudaStreamSynchronize(ctx->stream);
    for (auto &kv : ctx->graphs) cudaGraphExecDestroy(kv.second.exec);
    for (void *p : ctx->allocations) cudaFree(p);
    if (ctx->s.sort_buf) cudaFree(ctx->s.sort_buf);
    if (ctx->s.stage) cudaFree(ctx->s.stage);
    if (ctx->pipe_buf) cudaFree(ctx->pipe_buf);
    if (ctx->s.plain_buf) cudaFree(ctx->s.plain_buf);
    if (ctx->s.adj_buf) cudaFree(ctx->s.adj_buf);
    if (ctx->s.hist_buf) cudaFree(ctx->s.hist_buf);
    if (ctx->h_result) cudaFreeHost(ctx->h_result);
    if (ctx->ev0) cudaEventDestroy(ctx->ev0);
    if (ctx->ev1) cudaEventDestroy(ctx->ev1);
    for (int i = 0; i < xs_ctx::kPipeSlots; i++) {
        if (ctx->pipe_stream[i]) cudaStreamDestroy(ctx->pipe_stream[i]);
        if (ctx->pipe_event[i]) cudaEventDestroy(ctx->pipe_event[i]);
        if (ctx->ovf_ready[i]) cudaEventDestroy(ctx->ovf_ready[i]);
        if (ctx->ovf_done[i]) cudaEventDestroy(ctx->ovf_done[i]);
    }
    if (ctx->ovf_stream) cudaStreamDestroy(ctx->ovf_stream);
    if (ctx->fork_event) cudaEventDestroy(ctx->fork_event);
    if (ctx->stream) cudaStreamDestroy(ctx->stream);
    delete ctx;
}

static xs_status check_problem(const xs_inputs *in, const xs_simdata *sd)
{
    if (!in || !sd) return fail(XS_ERR_INVALID_ARGUMENT, "NULL inputs or simulation data");
    if (in->n_isotopes < 1 || in->n_gridpoints < 2)
        return fail(XS_ERR_INVALID_ARGUMENT, "need n_isotopes >= 1 and n_gridpoints >= 2");
    if (in->grid_type < 0 || in->grid_type > 2) return fail(XS_ERR_INVALID_ARGUMENT, "grid_type %d", in->grid_type);
    const long n_pts = in->n_isotopes * in->n_gridpoints;
    if (!sd->nuclide_grid || sd->length_nuclide_grid != n_pts)
        return fail(XS_ERR_INVALID_ARGUMENT, "nuclide grid length %d, expected %ld", sd->length_nuclide_grid, n_pts);
    if (!sd->num_nucs || !sd->mats || !sd->concs || sd->length_num_nucs != kMaterials || sd->max_num_nucs < 1 ||
        sd->length_mats != kMaterials * sd->max_num_nucs || sd->length_concs != sd->length_mats)
        return fail(XS_ERR_INVALID_ARGUMENT, "material tables malformed");
    for (int m = 0; m < kMaterials; m++) {
        if (sd->num_nucs[m] < 0 || sd->num_nucs[m] > sd->max_num_nucs)
            return fail(XS_ERR_DATA, "num_nucs[%d] = %d outside 0..%d", m, sd->num_nucs[m], sd->max_num_nucs);
        for (int j = 0; j < sd->num_nucs[m]; j++) {
            const int nuc = sd->mats[m * sd->max_num_nucs + j];
            if (nuc < 0 || nuc >= in->n_isotopes)
                return fail(XS_ERR_DATA, "mats[%d][%d] = %d outside 0..%ld", m, j, nuc, in->n_isotopes - 1);
        }
    }
    if (in->grid_type == XS_UNIONIZED) {
        if (!sd->unionized_energy_array || !sd->index_grid || sd->length_unionized_energy_array < 2 ||
            sd->length_index_grid != (long)sd->length_unionized_energy_array * in->n_isotopes)
            return fail(XS_ERR_INVALID_ARGUMENT, "unionized grid malformed");
        if (sd->length_unionized_energy_array > 0x7FFFFFFFL)
            return fail(XS_ERR_INVALID_ARGUMENT, "unionized grid too long");
    }
    if (in->grid_type == XS_HASH) {
        if (in->hash_bins < 1 || !sd->index_grid || sd->length_index_grid != (long)in->hash_bins * in->n_isotopes)
            return fail(XS_ERR_INVALID_ARGUMENT, "hash grid malformed");
    }
    return XS_OK;
}

}  // extern "C"

namespace xsgb {

// A context with streams, events and run scratch, and no problem yet.
xs_status ctx_open(const xs_inputs *in, int device, xs_ctx **out)
{
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev < 1) {
        cudaGetLastError();
        return fail(XS_ERR_NO_DEVICE, "no CUDA device");
    }
    if (device < 0 || device >= ndev) return fail(XS_ERR_NO_DEVICE, "device %d of %d", device, ndev);
    cudaDeviceProp prop;
    XS_CUDA(cudaGetDeviceProperties(&prop, device));
    if (prop.major != 10 || prop.minor != 3)
        return fail(XS_ERR_NO_DEVICE, "device %d is sm_%d%d; this library is built for sm_103a only", device, prop.major, prop.minor);
    XS_CUDA(cudaSetDevice(device));
    xs_ctx *ctx = new xs_ctx();
    ctx->device = device;
    ctx->inputs = *in;
    ctx->hm = in->HM ? in->HM : "";
    ctx->inputs.HM = (char *)ctx->hm.c_str();
    ctx->sm_count = prop.multiProcessorCount;
    cudaError_t e = cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaEventCreate(&ctx->ev0);
    if (e == cudaSuccess) e = cudaEventCreate(&ctx->ev1);
    for (int i = 0; i < xs_ctx::kPipeSlots && e == cudaSuccess; i++) {
        e = cudaStreamCreateWithFlags(&ctx->pipe_stream[i], cudaStreamNonBlocking);
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&ctx->pipe_event[i], cudaEventDisableTiming);
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&ctx->ovf_ready[i], cudaEventDisableTiming);
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&ctx->ovf_done[i], cudaEventDisableTiming);
    }
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&ctx->fork_event, cudaEventDisableTiming);
    if (e == cudaSuccess) {
        int least = 0, greatest = 0;
        e = cudaDeviceGetStreamPriorityRange(&least, &greatest);
        if (e == cudaSuccess) e = cudaStreamCreateWithPriority(&ctx->ovf_stream, cudaStreamNonBlocking, greatest);
    }
    if (e == cudaSuccess) e = cudaMallocHost(&ctx->h_result, 64);
    if (e != cudaSuccess) {
        xs_ctx_destroy(ctx);
        return cuda_fail(e, "context streams");
    }
    void *p;
    xs_status s = ctx_alloc(ctx, &p, 256);
    if (s != XS_OK) {
        xs_ctx_destroy(ctx);
        return s;
    }
    ctx->s.verification = (unsigned long long *)p;
    ctx->s.error = (int *)((char *)p + 64);
    ctx->s.queue = (unsigned int *)((char *)p + 128);
    Tables &t = ctx->t;
    t.n_iso = (int)in->n_isotopes;
    t.n_gp = in->n_gridpoints;
    t.grid_type = in->grid_type;
    t.hash_bins = in->hash_bins;
    t.hash_du = in->hash_bins > 0 ? 1.0 / in->hash_bins : 0.0;
    t.hash_margin = xsgb_hash_margin_bits(in->hash_bins);
    pick_mat_thresholds(t.mat_thresh);
    for (int m = 0; m < kMaterials; m++) t.mat_tseed[m] = xsgb_lcg_threshold(t.mat_thresh[m]);
    *out = ctx;
    return XS_OK;
}

// The material tables of a problem into an open context: the three arrays,
// the nuclide span of each material, the nuclides whose records stay in L2
// and the map nuclide -> (material, position) pairs.
xs_status install_materials(xs_ctx *ctx, const xs_inputs *in, const xs_simdata *sd)
{
    xs_status s = XS_OK;
    Tables &t = ctx->t;
    t.max_nucs = sd->max_num_nucs;
    for (int m = 0; m < kMaterials; m++) {
        int lo = (int)in->n_isotopes - 1, hi = 0;
        for (int j = 0; j < sd->num_nucs[m]; j++) {
            const int nuc = sd->mats[m * sd->max_num_nucs + j];
            lo = nuc < lo ? nuc : lo;
            hi = nuc > hi ? nuc : hi;
        }
        if (lo > hi) lo = hi = 0;
        t.mat_lo[m] = lo;
        t.mat_hi[m] = hi;
    }
    {   // hot nuclides: most expected record accesses per lookup, within a quarter of L2
        double thr[kMaterials], prob[kMaterials];
        pick_mat_thresholds(thr);
        for (int m = 1; m < kMaterials; m++) prob[m] = thr[m] - thr[m - 1];
        prob[0] = 1.0 - thr[kMaterials - 1];
        std::vector<double> freq((size_t)in->n_isotopes, 0.0);
        for (int m = 0; m < kMaterials; m++)
            for (int j = 0; j < sd->num_nucs[m]; j++) freq[(size_t)sd->mats[m * sd->max_num_nucs + j]] += prob[m];
        std::vector<int> order((size_t)in->n_isotopes);
        for (size_t i = 0; i < order.size(); i++) order[i] = (int)i;
        std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return freq[(size_t)a] > freq[(size_t)b]; });
        cudaDeviceProp prop;
        size_t l2 = 64u << 20;
        if (cudaGetDeviceProperties(&prop, ctx->device) == cudaSuccess && prop.l2CacheSize > 0) l2 = (size_t)prop.l2CacheSize;
        // a quarter of L2: measured from 0 to a half, the budget changes the
        // plain step's DRAM traffic by under 1 %
        const size_t per = (size_t)(in->n_gridpoints - 1) * kRecordDoubles * 8, budget = l2 / 4;
        size_t used = 0;
        std::memset(t.hot, 0, sizeof t.hot);
        for (int n : order) {
            if (n >= 512 || freq[(size_t)n] <= 0.0 || used + per > budget) continue;
            t.hot[n >> 5] |= 1u << (n & 31);
            used += per;
        }
    }
    {   // (material, position) pairs, and for each nuclide the pairs holding it
        t.pair_base[0] = 0;
        for (int m = 0; m < kMaterials; m++) t.pair_base[m + 1] = t.pair_base[m] + sd->num_nucs[m];
        std::vector<int> off((size_t)in->n_isotopes + 1, 0), pairs((size_t)t.pair_base[kMaterials] + 1, 0);
        for (int m = 0; m < kMaterials; m++)
            for (int j = 0; j < sd->num_nucs[m]; j++) off[(size_t)sd->mats[m * sd->max_num_nucs + j] + 1]++;
        for (long n = 0; n < in->n_isotopes; n++) off[(size_t)n + 1] += off[(size_t)n];
        std::vector<int> fill(off.begin(), off.end() - 1);
        for (int m = 0; m < kMaterials; m++)
            for (int j = 0; j < sd->num_nucs[m]; j++) {
                const int nuc = sd->mats[m * sd->max_num_nucs + j];
                pairs[(size_t)fill[(size_t)nuc]++] = m * sd->max_num_nucs + j;
            }
        if (s == XS_OK) s = upload(ctx, off.data(), off.size(), &t.inv_off);
        if (s == XS_OK) s = upload(ctx, pairs.data(), pairs.size(), &t.inv_pair);
        if (s == XS_OK) {  // the host vectors go out of scope
            cudaError_t e = cudaStreamSynchronize(ctx->stream);
            if (e != cudaSuccess) s = cuda_fail(e, "cudaStreamSynchronize");
        }
    }
    // a long fuel list is split over 4 lanes per lookup in the plain kernel
    // (FAST arithmetic) and over 2 in the batched kernel when it reads the
    // union table (set by build_union_table); xs_autotune measures 1, 2 and 4;
    // XSGB_FUEL_LANES and XSGB_BATCHED_FUEL_LANES = 1, 2 or 4 override
    for (int m = 0; m < kMaterials; m++) ctx->num_nucs_host[m] = sd->num_nucs[m];
    // energy buckets of the batched sort: at least one per 8 gridpoints of a
    // nuclide, so that a warp's 32 sorted lookups span few intervals (the
    // warp-cooperative nuclide search holds 32 keys)
    ctx->batched_buckets = 4096;
    while (ctx->batched_buckets < 65536 && (long)ctx->batched_buckets * 8 < in->n_gridpoints)
        ctx->batched_buckets <<= 1;
    // (measured: 4 lanes win up to ~11,000 gridpoints per nuclide and lose on
    // the 238,847-point XL grid)
    ctx->fuel_lanes = (sd->num_nucs[0] >= 64 && in->n_gridpoints <= 65536) ? 4 : 1;
    if (const char *env = getenv("XSGB_FUEL_LANES")) {
        const int v = atoi(env);
        if (v == 1 || v == 2 || v == 4) ctx->fuel_lanes = v;
    }
    if (const char *env = getenv("XSGB_STAGE_ROWS")) ctx->stage_rows = atoi(env) != 0 ? 1 : 0;
    if (const char *env = getenv("XSGB_TILE_SORT")) ctx->tile_sort = atoi(env) != 0 ? 1 : 0;
    if (const char *env = getenv("XSGB_OVERFLOW")) ctx->overflow = atoi(env) != 0 ? 1 : 0;
    if (const char *env = getenv("XSGB_PIPE_SLOTS")) ctx->pipe_slots = std::min(std::max(atoi(env), 2), xs_ctx::kPipeSlots);
    if (const char *env = getenv("XSGB_PIPE_CHUNK")) ctx->pipe_chunk = atol(env);
    if (const char *env = getenv("XSGB_HIST_GROUPS")) ctx->hist_groups = std::min(std::max(atoi(env), 1), xs_ctx::kPipeSlots);
    if (const char *env = getenv("XSGB_BATCHED_FUEL_LANES")) {
        const int v = atoi(env);
        if (v == 1 || v == 2 || v == 4) ctx->batched_fuel_lanes = v;
    }
    if (s == XS_OK) s = upload(ctx, sd->num_nucs, kMaterials, &t.num_nucs);
    if (s == XS_OK) s = upload(ctx, sd->mats, (size_t)sd->length_mats, &t.mats);
    if (s == XS_OK) s = upload(ctx, sd->concs, (size_t)sd->length_concs, &t.concs);
    return s;
}

}  // namespace xsgb

extern "C" {

xs_status xs_ctx_create(const xs_inputs *in, const xs_simdata *sd, int device, xs_ctx **out)
{
    if (!out) return fail(XS_ERR_INVALID_ARGUMENT, "xs_ctx_create: out is NULL");
    *out = nullptr;
    xs_status s = check_problem(in, sd);
    if (s != XS_OK) return s;
    xs_ctx *ctx = nullptr;
    s = ctx_open(in, device, &ctx);
    if (s != XS_OK) return s;
    Tables &t = ctx->t;
    s = install_materials(ctx, in, sd);
    const long n_pts = in->n_isotopes * in->n_gridpoints;
    if (s == XS_OK) s = upload(ctx, sd->nuclide_grid, (size_t)n_pts, &t.grid);
    if (s == XS_OK && in->grid_type == XS_UNIONIZED) {
        t.n_union = sd->length_unionized_energy_array;
        s = upload(ctx, sd->unionized_energy_array, (size_t)t.n_union, &t.union_e);
    }
    if (s == XS_OK && in->grid_type != XS_NUCLIDE) {
        s = upload(ctx, sd->index_grid, (size_t)sd->length_index_grid, &t.index_grid);
        ctx->own_index = t.index_grid;
    }
    if (s == XS_OK) s = build_derived_tables(ctx);
    if (s == XS_OK) s = build_union_table(ctx);
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

xs_status xs_ctx_download(xs_ctx *ctx, xs_simdata *out)
{
    if (!ctx || !out) return fail(XS_ERR_INVALID_ARGUMENT, "xs_ctx_download: NULL argument");
    XS_CUDA(cudaSetDevice(ctx->device));
    const Tables &t = ctx->t;
    xs_simdata r;
    std::memset(&r, 0, sizeof r);
    const long n_pts = (long)t.n_iso * t.n_gp;
    r.length_num_nucs = kMaterials;
    r.max_num_nucs = t.max_nucs;
    r.length_mats = r.length_concs = kMaterials * t.max_nucs;
    r.length_nuclide_grid = (int)n_pts;
    r.num_nucs = (int *)malloc(sizeof(int) * kMaterials);
    r.mats = (int *)malloc(sizeof(int) * (size_t)r.length_mats);
    r.concs = (double *)malloc(sizeof(double) * (size_t)r.length_concs);
    r.nuclide_grid = (xs_gridpoint *)malloc(sizeof(xs_gridpoint) * (size_t)n_pts);
    long n_index = 0;
    const int gtype = ctx->inputs.grid_type;
    if (gtype == XS_UNIONIZED) {
        r.length_unionized_energy_array = (int)t.n_union;
        r.unionized_energy_array = (double *)malloc(sizeof(double) * (size_t)t.n_union);
        n_index = t.n_union * t.n_iso;
    } else if (gtype == XS_HASH) {
        n_index = (long)ctx->inputs.hash_bins * t.n_iso;
    }
    r.length_index_grid = n_index;
    if (n_index) r.index_grid = (int *)malloc(sizeof(int) * (size_t)n_index);
    if (!r.num_nucs || !r.mats || !r.concs || !r.nuclide_grid || (n_index && !r.index_grid) ||
        (gtype == XS_UNIONIZED && !r.unionized_energy_array)) {
        xs_simdata_free(&r);
        return fail(XS_ERR_OUT_OF_MEMORY, "host copies");
    }
    cudaStream_t st = ctx->stream;
    cudaError_t e = cudaMemcpyAsync(r.num_nucs, t.num_nucs, sizeof(int) * kMaterials, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(r.mats, t.mats, sizeof(int) * (size_t)r.length_mats, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(r.concs, t.concs, sizeof(double) * (size_t)r.length_concs, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(r.nuclide_grid, t.grid, sizeof(xs_gridpoint) * (size_t)n_pts, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess && r.unionized_energy_array)
        e = cudaMemcpyAsync(r.unionized_energy_array, t.union_e, sizeof(double) * (size_t)t.n_union, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess && n_index)
        e = cudaMemcpyAsync(r.index_grid, ctx->own_index, sizeof(int) * (size_t)n_index, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) {
        xs_simdata_free(&r);
        return cuda_fail(e, "download");
    }
    *out = r;
    return XS_OK;
}

xs_status xs_ctx_sync(xs_ctx *ctx, xs_run_result *result)
{
    if (!ctx) return fail(XS_ERR_INVALID_ARGUMENT, "xs_ctx_sync: NULL context");
    XS_CUDA(cudaSetDevice(ctx->device));
    cudaStream_t st = ctx->last_stream ? ctx->last_stream : ctx->stream;
    xs_status s = read_back(ctx, st, result);
    if (result) result->kernel_launches = ctx->last_launches;
    return s;
}

static xs_status run_pipelined(xs_ctx *ctx, const xs_run_opts &o, const double *energy,
                               const int *mat, long n, double *macro_out, unsigned char *idx_out,
                               xs_run_result *result);

// Shared by xs_run_event (samples == NULL) and device-resident xs_lookup_samples.
static xs_status run_once(xs_ctx *ctx, const xs_run_opts &o, const SampleInput &in,
                          double *macro_out, unsigned char *idx_out, xs_run_result *result)
{
    cudaStream_t st = o.stream ? (cudaStream_t)o.stream : ctx->stream;
    const long n = o.count;
    const bool host_macro = macro_out && !is_device_pointer(macro_out);
    const bool host_idx = idx_out && !is_device_pointer(idx_out);
    if (o.async && (host_macro || host_idx))
        return fail(XS_ERR_INVALID_ARGUMENT, "async runs take device (or NULL) output arrays");
    // the event batch's own samples with every output on the host: chunks
    // whose copies out overlap the next chunks' lookups
    if (!in.energy && (host_macro || host_idx) && (!macro_out || host_macro) && (!idx_out || host_idx))
        return run_pipelined(ctx, o, nullptr, nullptr, n, macro_out, idx_out, result);
    Outputs out;
    out.macro = macro_out;
    out.max_idx = idx_out;
    if (host_macro || host_idx) {
        size_t need = (host_macro ? (size_t)n * 40 : 0) + (host_idx ? (size_t)n + 256 : 0);
        xs_status s = ensure_stage(ctx, need);
        if (s != XS_OK) return s;
        char *b = (char *)ctx->s.stage;
        if (host_macro) {
            out.macro = (double *)b;
            b += (size_t)n * 40;
        }
        if (host_idx) out.max_idx = (unsigned char *)b;
    }
    XS_CUDA(cudaMemsetAsync(ctx->s.verification, 0, 8, st));
    XS_CUDA(cudaMemsetAsync(ctx->s.error, 0, 16, st));
    XS_CUDA(cudaEventRecord(ctx->ev0, st));
    int launches = 0;
    xs_status s;
    if (o.kernel == XS_KERNEL_PLAIN) {
        PlainScratch ps;
        const PlainScratch *psp = nullptr;
        if (use_overflow(ctx, n, o.tile_lookups)) {
            s = ensure_plain(ctx, plain_scratch_bytes(n, o.tile_lookups));
            if (s != XS_OK) return s;
            ps = carve_plain_scratch(ctx->s.plain_buf, n, o.tile_lookups);
            psp = &ps;
        }
        s = launch_plain(ctx, st, o.arith, o.checked, o.first, n, o.tile_lookups, o.block_threads,
                         in, out, psp, &launches);
    } else
        s = launch_batched(ctx, st, o.arith, o.checked, o.first, n, o.block_threads,
                           o.energy_buckets, in, out, &launches);
    if (s != XS_OK) return s;
    XS_CUDA(cudaEventRecord(ctx->ev1, st));
    ctx->last_stream = st;
    ctx->last_launches = launches;
    if (o.async) {
        if (result) {
            result->verification = 0;
            result->device_ms = 0.f;
            result->kernel_launches = launches;
        }
        return XS_OK;
    }
    if (host_macro) XS_CUDA(cudaMemcpyAsync(macro_out, out.macro, (size_t)n * 40, cudaMemcpyDeviceToHost, st));
    if (host_idx) XS_CUDA(cudaMemcpyAsync(idx_out, out.max_idx, (size_t)n, cudaMemcpyDeviceToHost, st));
    s = read_back(ctx, st, result);
    if (result) result->kernel_launches = launches;
    return s;
}

xs_status xs_run_event(xs_ctx *ctx, const xs_run_opts *opts, double *macro_xs_out,
                       unsigned char *max_idx_out, xs_run_result *result)
{
    if (!ctx) return fail(XS_ERR_INVALID_ARGUMENT, "xs_run_event: NULL context");
    XS_CUDA(cudaSetDevice(ctx->device));
    xs_run_opts o;
    xs_status s = resolve(ctx, opts, (long)ctx->inputs.lookups, &o);
    if (s != XS_OK) return s;
    return run_once(ctx, o, SampleInput{}, macro_xs_out, max_idx_out, result);
}


// Host-resident samples (energy, mat), or with energy == NULL the event
// batch's own LCG samples of lookups o.first + i (nothing copied in): chunks
// rotate over the pipeline's streams (one buffer set each), so the copies of
// some chunks overlap the lookups of others.
static xs_status run_pipelined(xs_ctx *ctx, const xs_run_opts &o, const double *energy,
                               const int *mat, long n, double *macro_out, unsigned char *idx_out,
                               xs_run_result *result)
{
    const bool host_in = energy != nullptr;
    // Whole chunks of 2^21 lookups (plain) or 2^22 (batched: each chunk is
    // sorted on its own, and its persistent launch ends in a tail); swept end
    // to end on the large problem, four slots: plain 2^20 / 2^21 / 2^22 =
    // 898 / 905 / 898 M lookups/s, batched 2^21 / 2^22 / 2^23 = 920 / 926 /
    // 850 M.  A longer batch takes whole chunks of about n / 8 (at most 2^24):
    // its pipeline's ends cost little beside it, and each chunk has a tail
    // (XL, 100M lookups: hash grid 619 / 625 / 629 / 631 M lookups/s with
    // chunks of 2^21 / 2^22 / 2^23 / 2^24).
    const long chunk = ctx->pipe_chunk > 0 ? std::max<long>(ctx->pipe_chunk, o.tile_lookups)
                                           : xsgb_pipeline_whole(n, o.kernel == XS_KERNEL_BATCHED,
                                                                 o.tile_lookups);
    const size_t in_per = host_in ? 12 : 0;
    const size_t per = in_per + (macro_out ? 40 : 0) + (idx_out ? 1 : 0);
    const size_t io_bytes = ((size_t)chunk * per + 1023) & ~(size_t)255;
    // Plain kernel: each chunk's partial 32-lookup groups go to its own
    // overflow queues, and the chunk's overflow pass runs on the
    // high-priority stream, so its blocks are dispatched as soon as the
    // chunk's tiles end instead of after the other streams' pending tiles
    // (on the tiles' own stream the pass waited behind them and held up the
    // next chunk: 0.77 G lookups/s end to end, against 0.86 G with the
    // partial groups padded in their tiles).  A chunk's buffers are reused
    // by the chunk `slots` places later, which waits for its overflow pass
    // and copy out: with two slots that chain stalled the 1M-lookup chunks
    // (large hash grid, end to end: 665 M lookups/s with two slots of 1M,
    // 723 M with three of 2M, 746 M with four of 2M).
    const bool ovf = o.kernel == XS_KERNEL_PLAIN && use_overflow(ctx, chunk, o.tile_lookups);
    const size_t ovf_bytes = ovf ? ((plain_scratch_bytes(chunk, o.tile_lookups) + 255) & ~(size_t)255) : 0;
    // batched: each slot has its own sort buffers, so the streams overlap
    const bool batched = o.kernel == XS_KERNEL_BATCHED;
    int nb_log2 = 0;
    while ((1 << nb_log2) < o.energy_buckets) nb_log2++;
    if (batched && ((1 << nb_log2) != o.energy_buckets || o.energy_buckets > 65536))
        return fail(XS_ERR_INVALID_ARGUMENT, "energy_buckets %d must be a power of two <= 65536", o.energy_buckets);
    const size_t slot = io_bytes + ovf_bytes +
                        (batched ? ((batched_scratch_bytes(chunk, o.energy_buckets) + 255) & ~(size_t)255) : 0);
    const size_t need = (size_t)ctx->pipe_slots * slot;
    if (ctx->pipe_bytes < need) {
        if (ctx->pipe_buf) {
            cudaFree(ctx->pipe_buf);
            ctx->device_bytes -= ctx->pipe_bytes;
            ctx->pipe_buf = nullptr;
            ctx->pipe_bytes = 0;
            for (auto &kv : ctx->graphs) cudaGraphExecDestroy(kv.second.exec);
            ctx->graphs.clear();
        }
        cudaError_t e = cudaMalloc(&ctx->pipe_buf, need);
        if (e != cudaSuccess) {
            cudaGetLastError();
            return fail(XS_ERR_OUT_OF_MEMORY, "sample pipeline buffers (%zu bytes)", need);
        }
        ctx->pipe_bytes = need;
        ctx->device_bytes += need;
    }
    cudaStream_t main = o.stream ? (cudaStream_t)o.stream : ctx->stream;
    XS_CUDA(cudaMemsetAsync(ctx->s.verification, 0, 8, main));
    XS_CUDA(cudaMemsetAsync(ctx->s.error, 0, 16, main));
    XS_CUDA(cudaEventRecord(ctx->ev0, main));
    const int S = ctx->pipe_slots;
    for (int i = 0; i < S; i++) XS_CUDA(cudaStreamWaitEvent(ctx->pipe_stream[i], ctx->ev0, 0));
    int launches = 0;
    std::vector<long> sizes((size_t)xsgb_pipeline_chunks(n, chunk, o.tile_lookups, nullptr, 0));
    xsgb_pipeline_chunks(n, chunk, o.tile_lookups, sizes.data(), (long)sizes.size());
    long c0 = 0;
    for (size_t k = 0; k < sizes.size(); c0 += sizes[k], k++) {
        const int w = (int)(k % S);
        cudaStream_t st = ctx->pipe_stream[w];
        const long m = sizes[k];
        char *b = (char *)ctx->pipe_buf + (size_t)w * slot;
        double *dE = (double *)b;
        int *dM = (int *)(b + (size_t)chunk * 8);
        double *dMacro = macro_out ? (double *)(b + (size_t)chunk * in_per) : nullptr;
        unsigned char *dIdx = idx_out ? (unsigned char *)(b + (size_t)chunk * (in_per + (macro_out ? 40 : 0))) : nullptr;
        SampleInput in;
        if (host_in) {
            XS_CUDA(cudaMemcpyAsync(dE, energy + c0, (size_t)m * 8, cudaMemcpyHostToDevice, st));
            XS_CUDA(cudaMemcpyAsync(dM, mat + c0, (size_t)m * 4, cudaMemcpyHostToDevice, st));
            in.energy = dE;
            in.mat = dM;
        }
        // lookups sampled in the kernels are numbered from the run's first
        const long first = host_in ? 0 : o.first + c0;
        Outputs out;
        out.macro = dMacro;
        out.max_idx = dIdx;
        xs_status s;
        if (o.kernel == XS_KERNEL_PLAIN) {
            PlainScratch ps;
            OverflowStream os{ctx->ovf_stream, ctx->ovf_ready[w], ctx->ovf_done[w]};
            if (ovf) ps = carve_plain_scratch(b + io_bytes, m, o.tile_lookups);
            s = launch_plain(ctx, st, o.arith, o.checked, first, m, o.tile_lookups, o.block_threads,
                             in, out, ovf ? &ps : nullptr, &launches, ovf ? &os : nullptr);
        } else {
            BatchedScratch bs = carve_batched_scratch(b + io_bytes, chunk, nb_log2);
            bs.verification = ctx->s.verification;
            bs.error = ctx->s.error;
            s = enqueue_batched_buf(ctx, st, o.arith, o.checked, first, m, nb_log2, o.block_threads,
                                    in, out, bs, &launches);
        }
        if (s != XS_OK) return s;
        if (macro_out) XS_CUDA(cudaMemcpyAsync(macro_out + c0 * 5, dMacro, (size_t)m * 40, cudaMemcpyDeviceToHost, st));
        if (idx_out) XS_CUDA(cudaMemcpyAsync(idx_out + c0, dIdx, (size_t)m, cudaMemcpyDeviceToHost, st));
    }
    for (int i = 0; i < S; i++) {
        XS_CUDA(cudaEventRecord(ctx->pipe_event[i], ctx->pipe_stream[i]));
        XS_CUDA(cudaStreamWaitEvent(main, ctx->pipe_event[i], 0));
    }
    XS_CUDA(cudaEventRecord(ctx->ev1, main));
    xs_status s = read_back(ctx, main, result);
    if (result) result->kernel_launches = launches;
    return s;
}

xs_status xs_lookup_samples(xs_ctx *ctx, const xs_run_opts *opts, const double *energy,
                            const int *mat, long n, double *macro_xs_out,
                            unsigned char *max_idx_out, xs_run_result *result)
{
    if (!ctx) return fail(XS_ERR_INVALID_ARGUMENT, "xs_lookup_samples: NULL context");
    if (!energy || !mat || n <= 0) return fail(XS_ERR_INVALID_ARGUMENT, "xs_lookup_samples: need energy, mat and n > 0");
    XS_CUDA(cudaSetDevice(ctx->device));
    xs_run_opts o;
    xs_status s = resolve(ctx, opts, n, &o);
    if (s != XS_OK) return s;
    o.first = 0;
    o.count = n;
    const bool dev_in = is_device_pointer(energy) && is_device_pointer(mat);
    if (dev_in) {
        SampleInput in;
        in.energy = energy;
        in.mat = mat;
        return run_once(ctx, o, in, macro_xs_out, max_idx_out, result);
    }
    if (o.async) return fail(XS_ERR_INVALID_ARGUMENT, "async runs take device sample arrays");
    if (is_device_pointer(energy) || is_device_pointer(mat) ||
        (macro_xs_out && is_device_pointer(macro_xs_out)) || (max_idx_out && is_device_pointer(max_idx_out)))
        return fail(XS_ERR_INVALID_ARGUMENT, "host sample arrays need host output arrays");
    return run_pipelined(ctx, o, energy, mat, n, macro_xs_out, max_idx_out, result);
}

xs_status xs_sample_event(xs_ctx *ctx, long first, long count, double *energy_out, int *mat_out)
{
    if (!ctx || !energy_out || !mat_out || first < 0 || count <= 0)
        return fail(XS_ERR_INVALID_ARGUMENT, "xs_sample_event: bad argument");
    XS_CUDA(cudaSetDevice(ctx->device));
    const bool dev = is_device_pointer(energy_out) && is_device_pointer(mat_out);
    double *E = energy_out;
    int *M = mat_out;
    if (!dev) {
        xs_status s = ensure_stage(ctx, (size_t)count * 12 + 256);
        if (s != XS_OK) return s;
        E = (double *)ctx->s.stage;
        M = (int *)((char *)ctx->s.stage + (size_t)count * 8);
    }
    xs_status s = launch_sample(ctx, ctx->stream, first, count, E, M);
    if (s != XS_OK) return s;
    if (!dev) {
        XS_CUDA(cudaMemcpyAsync(energy_out, E, (size_t)count * 8, cudaMemcpyDeviceToHost, ctx->stream));
        XS_CUDA(cudaMemcpyAsync(mat_out, M, (size_t)count * 4, cudaMemcpyDeviceToHost, ctx->stream));
    }
    XS_CUDA(cudaStreamSynchronize(ctx->stream));
    return XS_OK;
}

xs_status xs_run_history(xs_ctx *ctx, const xs_run_opts *opts, xs_run_result *result)
{
    if (!ctx) return fail(XS_ERR_INVALID_ARGUMENT, "xs_run_history: NULL context");
    XS_CUDA(cudaSetDevice(ctx->device));
    xs_run_opts o;
    xs_status s = resolve(ctx, opts, (long)ctx->inputs.particles, &o);
    if (s != XS_OK) return s;
    if (ctx->inputs.lookups < 1) return fail(XS_ERR_INVALID_ARGUMENT, "lookups per particle < 1");
    cudaStream_t st = o.stream ? (cudaStream_t)o.stream : ctx->stream;
    XS_CUDA(cudaMemsetAsync(ctx->s.verification, 0, 8, st));
    XS_CUDA(cudaMemsetAsync(ctx->s.error, 0, 16, st));
    XS_CUDA(cudaEventRecord(ctx->ev0, st));
    int launches = 0;
    s = o.kernel == XS_KERNEL_BATCHED
            ? launch_history_stepped(ctx, st, o.arith, o.first, o.count,
                                     opts && opts->tile_lookups > 0 ? opts->tile_lookups : 0, &launches)
            : launch_history(ctx, st, o.arith, o.first, o.count, &launches);
    if (s != XS_OK) return s;
    XS_CUDA(cudaEventRecord(ctx->ev1, st));
    s = read_back(ctx, st, result);
    if (result) result->kernel_launches = launches;
    return s;
}

// The adjoint for LCG-sampled (in.energy == NULL) or caller-sampled lookups.
static xs_status adjoint_common(xs_ctx *ctx, const xs_run_opts *opts, const double *energy,
                                const int *mat, long n_samples, const double *gbar,
                                double *macro_out, double *d_concs, double *d_xs,
                                double *d_energy, xs_run_result *result)
{
    if (!ctx) return fail(XS_ERR_INVALID_ARGUMENT, "adjoint: NULL context");
    if (!gbar) return fail(XS_ERR_INVALID_ARGUMENT, "adjoint: gbar is NULL");
    XS_CUDA(cudaSetDevice(ctx->device));
    xs_run_opts o;
    const bool samples = energy != nullptr;
    xs_status s = resolve(ctx, opts, samples ? n_samples : (long)ctx->inputs.lookups, &o);
    if (s != XS_OK) return s;
    if (samples) {
        o.first = 0;
        o.count = n_samples;
    }
    const long n = o.count;
    const Tables &t = ctx->t;
    const size_t nconc = (size_t)kMaterials * t.max_nucs, nxs = (size_t)t.n_iso * t.n_gp * 5;
    const void *ptrs[7] = {energy, mat, gbar, macro_out, d_concs, d_xs, d_energy};
    int ndev = 0, nhost = 0;
    for (const void *p : ptrs) {
        if (!p) continue;
        if (is_device_pointer(p)) ndev++; else nhost++;
    }
    if (ndev && nhost) return fail(XS_ERR_INVALID_ARGUMENT, "adjoint: arrays must be all host or all device memory");
    cudaStream_t st = o.stream ? (cudaStream_t)o.stream : ctx->stream;
    SampleInput in;
    const double *g_dev = gbar;
    double *m_dev = macro_out, *c_dev = d_concs, *x_dev = d_xs, *e_dev = d_energy;
    if (nhost) {
        // one staging block: samples, gbar, outputs, zeroed gradient sums
        const size_t bytes = (samples ? (size_t)n * 12 : 0) + (size_t)n * 40 +
                             (macro_out ? (size_t)n * 40 : 0) + (d_energy ? (size_t)n * 8 : 0) +
                             (d_concs ? nconc * 8 : 0) + (d_xs ? nxs * 8 : 0) + 8 * 256;
        s = ensure_stage(ctx, bytes);
        if (s != XS_OK) return s;
        char *b = (char *)ctx->s.stage;
        auto take = [&](size_t sz) { char *r = b; b += (sz + 255) & ~(size_t)255; return r; };
        if (samples) {
            double *dE = (double *)take((size_t)n * 8);
            int *dM = (int *)take((size_t)n * 4);
            XS_CUDA(cudaMemcpyAsync(dE, energy, (size_t)n * 8, cudaMemcpyHostToDevice, st));
            XS_CUDA(cudaMemcpyAsync(dM, mat, (size_t)n * 4, cudaMemcpyHostToDevice, st));
            in.energy = dE;
            in.mat = dM;
        }
        double *dg = (double *)take((size_t)n * 40);
        XS_CUDA(cudaMemcpyAsync(dg, gbar, (size_t)n * 40, cudaMemcpyHostToDevice, st));
        g_dev = dg;
        m_dev = macro_out ? (double *)take((size_t)n * 40) : nullptr;
        e_dev = d_energy ? (double *)take((size_t)n * 8) : nullptr;
        c_dev = d_concs ? (double *)take(nconc * 8) : nullptr;
        x_dev = d_xs ? (double *)take(nxs * 8) : nullptr;
        if (c_dev) XS_CUDA(cudaMemsetAsync(c_dev, 0, nconc * 8, st));
        if (x_dev) XS_CUDA(cudaMemsetAsync(x_dev, 0, nxs * 8, st));
    } else if (samples) {
        in.energy = energy;
        in.mat = mat;
    }
    XS_CUDA(cudaMemsetAsync(ctx->s.verification, 0, 8, st));
    XS_CUDA(cudaMemsetAsync(ctx->s.error, 0, 16, st));
    XS_CUDA(cudaEventRecord(ctx->ev0, st));
    int launches = 0;
    s = launch_adjoint(ctx, st, o.first, n, in, g_dev, m_dev, c_dev, x_dev, e_dev, &launches);
    if (s != XS_OK) return s;
    XS_CUDA(cudaEventRecord(ctx->ev1, st));
    std::vector<double> hc, hx;
    if (nhost) {
        if (macro_out) XS_CUDA(cudaMemcpyAsync(macro_out, m_dev, (size_t)n * 40, cudaMemcpyDeviceToHost, st));
        if (d_energy) XS_CUDA(cudaMemcpyAsync(d_energy, e_dev, (size_t)n * 8, cudaMemcpyDeviceToHost, st));
        if (d_concs) {
            hc.resize(nconc);
            XS_CUDA(cudaMemcpyAsync(hc.data(), c_dev, nconc * 8, cudaMemcpyDeviceToHost, st));
        }
        if (d_xs) {
            hx.resize(nxs);
            XS_CUDA(cudaMemcpyAsync(hx.data(), x_dev, nxs * 8, cudaMemcpyDeviceToHost, st));
        }
    }
    s = read_back(ctx, st, result);
    if (result) result->kernel_launches = launches;
    if (s != XS_OK) return s;
    for (size_t i = 0; i < hc.size(); i++) d_concs[i] += hc[i];
    for (size_t i = 0; i < hx.size(); i++) d_xs[i] += hx[i];
    return XS_OK;
}

xs_status xs_run_adjoint(xs_ctx *ctx, const xs_run_opts *opts, const double *gbar,
                         double *macro_xs_out, double *d_concs, double *d_xs, double *d_energy,
                         xs_run_result *result)
{
    return adjoint_common(ctx, opts, nullptr, nullptr, 0, gbar, macro_xs_out, d_concs, d_xs,
                          d_energy, result);
}

xs_status xs_adjoint_samples(xs_ctx *ctx, const xs_run_opts *opts, const double *energy,
                             const int *mat, long n, const double *gbar, double *macro_xs_out,
                             double *d_concs, double *d_xs, double *d_energy,
                             xs_run_result *result)
{
    if (!energy || !mat || n <= 0) return fail(XS_ERR_INVALID_ARGUMENT, "xs_adjoint_samples: need energy, mat and n > 0");
    return adjoint_common(ctx, opts, energy, mat, n, gbar, macro_xs_out, d_concs, d_xs, d_energy,
                          result);
}


xs_status xs_run_event_based_simulation(xs_inputs in, xs_simdata sd, int mype,
                                        unsigned long long *verification)
{
    (void)mype;
    if (!verification) return fail(XS_ERR_INVALID_ARGUMENT, "verification is NULL");
    xs_ctx *ctx = nullptr;
    xs_status s = xs_ctx_create(&in, &sd, 0, &ctx);
    if (s != XS_OK) return s;
    xs_run_result r;
    s = xs_run_event(ctx, nullptr, nullptr, nullptr, &r);
    if (s == XS_OK) *verification = r.verification;
    xs_ctx_destroy(ctx);
    return s;
}

}  // extern "C"
