// tune.cu -- the autotuner: times the kernel shapes and the grid types a
// context can serve on a sample of its own event batch, keeps the fastest as
// the context's defaults, and caches the choice in a JSON file keyed by
// (device name, problem).
//
// Grid types: every grid gives each lookup the same nuclide intervals as the
// unionized grid (the hash grid's edge rule E == e_low -> gridpoint 0 is the
// only exception, and needs an energy equal to a tabulated one), so the tuner
// may serve a context from a grid other than the one it was built with: it
// derives a hash grid on the device (GridInit.c:128-151 semantics, 10,000
// bins) and the nuclide grid's coarse keys when they are missing.
#include <algorithm>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "device_common.cuh"

namespace xsgb {

// The fields of Tables that differ between grid types.
struct GridView {
    int grid_type, hash_bins;
    double hash_du;
    const int *index_grid;
    const long long *coarse;
    int n_coarse;
    int guided;          // 1: the guided searches (energy-bin guide and bin records)
};

static GridView view_of(const Tables &t)
{
    return GridView{t.grid_type, t.hash_bins, t.hash_du, t.index_grid, t.coarse, t.n_coarse,
                    t.guide != nullptr};
}

static void apply_view(xs_ctx *ctx, const GridView &v)
{
    Tables &t = ctx->t;
    t.grid_type = v.grid_type;
    t.hash_bins = v.hash_bins;
    t.hash_du = v.hash_du;
    t.hash_margin = xsgb_hash_margin_bits(v.hash_bins);
    t.index_grid = v.index_grid;
    t.coarse = v.coarse;
    t.n_coarse = v.n_coarse;
    t.guide = v.guided ? ctx->own_guide : nullptr;
    t.binrec = v.guided ? ctx->own_binrec : nullptr;
}

static std::string cache_key(const xs_ctx *ctx)
{
    cudaDeviceProp p;
    char name[256] = "unknown";
    if (cudaGetDeviceProperties(&p, ctx->device) == cudaSuccess) snprintf(name, sizeof name, "%s", p.name);
    char key[512];
    snprintf(key, sizeof key, "%s|grid=%d|n_iso=%ld|n_gp=%ld|bins=%d|lookups=%d", name,
             ctx->inputs.grid_type, ctx->inputs.n_isotopes, ctx->inputs.n_gridpoints,
             ctx->inputs.hash_bins, ctx->inputs.lookups);
    return key;
}

struct Choice {
    int grid_type = -1, kernel = 0, tile = 1024, buckets = 4096, blocks_per_sm = 4, lanes = 1;
    double rate = 0;
    int block = 256;   // threads per block of the chosen kernel
    int guided = 0;    // the guided searches (hash / nuclide grids)
    int tile_sort = 0; // plain kernel: energy order within each tile's materials
};

// cache file: one entry per line, {"<key>": {...}} inside a JSON object
static bool cache_read(const char *path, const std::string &key, Choice &c)
{
    FILE *f = fopen(path, "r");
    if (!f) return false;
    char line[2048];
    const std::string want = "\"" + key + "\":";
    bool found = false;
    while (fgets(line, sizeof line, f)) {
        const char *p = strstr(line, want.c_str());
        if (!p) continue;
        p += want.size();
        if (sscanf(p, " {\"grid_type\": %d, \"kernel\": %d, \"tile\": %d, \"buckets\": %d, "
                      "\"blocks_per_sm\": %d, \"fuel_lanes\": %d, \"block\": %d, "
                      "\"guided\": %d, \"tile_sort\": %d, \"lookups_per_s\": %lf",
                   &c.grid_type, &c.kernel, &c.tile, &c.buckets, &c.blocks_per_sm, &c.lanes,
                   &c.block, &c.guided, &c.tile_sort, &c.rate) == 10 &&
            (c.lanes == 1 || c.lanes == 2 || c.lanes == 4) &&
            (c.block == 128 || c.block == 256 || c.block == 512) && c.tile % c.block == 0)
            found = true;
    }
    fclose(f);
    return found;
}

static void cache_write(const char *path, const std::string &key, const Choice &c)
{
    std::vector<std::string> lines;
    if (FILE *f = fopen(path, "r")) {
        char line[2048];
        while (fgets(line, sizeof line, f)) {
            std::string s(line);
            if (s.find("\": {\"grid_type\"") != std::string::npos &&
                s.find("\"" + key + "\":") == std::string::npos) {
                while (!s.empty() && (s.back() == '\n' || s.back() == ',')) s.pop_back();
                lines.push_back(s);
            }
        }
        fclose(f);
    }
    char buf[1024];
    snprintf(buf, sizeof buf,
             "  \"%s\": {\"grid_type\": %d, \"kernel\": %d, \"tile\": %d, \"buckets\": %d, "
             "\"blocks_per_sm\": %d, \"fuel_lanes\": %d, \"block\": %d, \"guided\": %d, "
             "\"tile_sort\": %d, \"lookups_per_s\": %.6g}",
             key.c_str(), c.grid_type, c.kernel, c.tile, c.buckets, c.blocks_per_sm, c.lanes,
             c.block, c.guided, c.tile_sort, c.rate);
    lines.push_back(buf);
    FILE *f = fopen(path, "w");
    if (!f) return;
    fprintf(f, "{\n");
    for (size_t i = 0; i < lines.size(); i++) fprintf(f, "%s%s\n", lines[i].c_str(), i + 1 < lines.size() ? "," : "");
    fprintf(f, "}\n");
    fclose(f);
}

}  // namespace xsgb

using namespace xsgb;

extern "C" xs_status xs_autotune(xs_ctx *ctx, const char *cache_path, xs_run_opts *best)
{
    if (!ctx) return fail(XS_ERR_INVALID_ARGUMENT, "xs_autotune: NULL context");
    XS_CUDA(cudaSetDevice(ctx->device));
    Tables &t = ctx->t;
    // the grid types this context can serve, starting with the one it was built with
    const GridView base{ctx->inputs.grid_type, ctx->inputs.hash_bins,
                        ctx->inputs.hash_bins > 0 ? 1.0 / ctx->inputs.hash_bins : 0.0,
                        ctx->own_index, ctx->base_coarse, ctx->base_n_coarse,
                        ctx->base_guided};
    apply_view(ctx, base);
    std::vector<GridView> views;
    if (!ctx->tune_hash_index && t.grid_type != XS_HASH) {
        void *p = nullptr;
        const int bins = 10000;
        xs_status s = ctx_alloc(ctx, &p, (size_t)bins * t.n_iso * 4);
        if (s != XS_OK) return s;
        XS_CUDA(launch_hash_grid(t.grid, t.n_iso, t.n_gp, bins, (int *)p, ctx->sm_count, ctx->stream));
        ctx->tune_hash_index = (int *)p;
    }
    if (!base.coarse && !ctx->tune_coarse) {
        void *p = nullptr;
        const int nc = (int)((t.n_gp + kCoarseStride - 1) / kCoarseStride);
        xs_status s = ctx_alloc(ctx, &p, (size_t)t.n_iso * nc * 8);
        if (s != XS_OK) return s;
        XS_CUDA(launch_coarse_keys(t.ekeys, t.n_iso, t.n_gp, nc, (long long *)p, ctx->sm_count,
                                   ctx->stream));
        ctx->tune_coarse = (long long *)p;
        ctx->tune_n_coarse = nc;
    }
    if (!ctx->own_guide) {   // the guided searches of the hash and nuclide grids
        xs_status s = build_guide(ctx);
        if (s != XS_OK) return s;
        ctx->own_guide = t.guide;
        ctx->own_binrec = t.binrec;
    }
    // every grid type the context can serve; the hash and nuclide grids both
    // with and without the guided searches (when the guide could be built)
    std::vector<GridView> grids{base};
    if (base.grid_type != XS_HASH)
        grids.push_back(GridView{XS_HASH, 10000, 1.0 / 10000, ctx->tune_hash_index, base.coarse,
                                 base.n_coarse, 0});
    if (base.grid_type != XS_NUCLIDE)
        grids.push_back(GridView{XS_NUCLIDE, base.hash_bins, base.hash_du, base.index_grid,
                                 ctx->tune_coarse, ctx->tune_n_coarse, 0});
    for (GridView v : grids) {
        if (v.grid_type == XS_UNIONIZED || !ctx->own_guide) {
            v.guided = 0;
            views.push_back(v);
            continue;
        }
        v.guided = 1;
        views.push_back(v);
        v.guided = 0;
        views.push_back(v);
    }
    XS_CUDA(cudaStreamSynchronize(ctx->stream));

    const std::string key = cache_key(ctx);
    Choice c;
    bool cached = cache_path && cache_read(cache_path, key, c);
    if (!cached) {
        const long sample = std::min<long>(ctx->inputs.lookups, 4L << 20);
        const GridView original = view_of(t);
        auto time_run = [&](xs_run_opts &o, double *rate) -> xs_status {
            xs_run_result r;
            xs_status s = xs_run_event(ctx, &o, nullptr, nullptr, &r);  // warm-up
            if (s != XS_OK) return s;
            float ms[3];
            for (int i = 0; i < 3; i++) {
                s = xs_run_event(ctx, &o, nullptr, nullptr, &r);
                if (s != XS_OK) return s;
                ms[i] = r.device_ms;
            }
            std::sort(ms, ms + 3);
            *rate = sample / (ms[1] * 1e-3);
            return XS_OK;
        };
        const int saved_bps = ctx->batched_blocks_per_sm;
        const int saved_lanes = ctx->fuel_lanes, saved_blanes = ctx->batched_fuel_lanes;
        const int saved_pblock = ctx->plain_block, saved_bblock = ctx->batched_block;
        const int saved_sort = ctx->tile_sort;
        auto restore = [&]() {
            apply_view(ctx, original);
            ctx->tile_sort = saved_sort;
            ctx->batched_blocks_per_sm = saved_bps;
            ctx->fuel_lanes = saved_lanes;
            ctx->batched_fuel_lanes = saved_blanes;
            ctx->plain_block = saved_pblock;
            ctx->batched_block = saved_bblock;
        };
        // the shapes are searched at 256 threads per block, the block size after
        ctx->plain_block = ctx->batched_block = 256;
        for (const GridView &v : views) {
            apply_view(ctx, v);
            for (int bps : {3, 4}) {
                ctx->batched_blocks_per_sm = bps;
                for (int lanes : {1, 2, 4}) {
                    ctx->fuel_lanes = lanes;
                    ctx->batched_fuel_lanes = lanes;
                    for (int tile : {512, 1024, 1536, 2048, 3072}) {
                        xs_run_opts o;
                        xs_run_opts_init(&o);
                        o.count = sample;
                        o.tile_lookups = tile;
                        double rate = 0;
                        xs_status s = time_run(o, &rate);
                        if (s != XS_OK) {
                            restore();
                            return s;
                        }
                        if (rate > c.rate)
                            c = Choice{v.grid_type, XS_KERNEL_PLAIN, tile, c.buckets, bps, lanes, rate,
                                       256, v.guided, -1};
                    }
                    for (int nb : {256, 1024, 4096, 16384}) {
                        xs_run_opts o;
                        xs_run_opts_init(&o);
                        o.count = sample;
                        o.kernel = XS_KERNEL_BATCHED;
                        o.energy_buckets = nb;
                        double rate = 0;
                        xs_status s = time_run(o, &rate);
                        if (s != XS_OK) {
                            restore();
                            return s;
                        }
                        if (rate > c.rate)
                            c = Choice{v.grid_type, XS_KERNEL_BATCHED, c.tile, nb, bps, lanes, rate,
                                       256, v.guided, -1};
                    }
                }
            }
        }
        // block shape of the chosen kernel, with the rest of the choice in
        // place and the threads per SM unchanged (the plain kernel's blocks
        // divide its tile)
        for (const GridView &v : views)
            if (v.grid_type == c.grid_type && v.guided == c.guided) apply_view(ctx, v);
        ctx->batched_blocks_per_sm = c.blocks_per_sm;
        ctx->fuel_lanes = c.lanes;
        ctx->batched_fuel_lanes = c.lanes;
        for (int block : {128, 512}) {
            if (c.kernel == XS_KERNEL_PLAIN && c.tile % block) continue;
            xs_run_opts o;
            xs_run_opts_init(&o);
            o.count = sample;
            o.kernel = c.kernel;
            o.tile_lookups = c.tile;
            o.energy_buckets = c.buckets;
            o.block_threads = block;
            double rate = 0;
            xs_status s = time_run(o, &rate);
            if (s != XS_OK) {
                restore();
                return s;
            }
            if (rate > c.rate) {
                c.rate = rate;
                c.block = block;
            }
        }
        // the plain kernel's in-tile energy order, on and off (the search
        // above ran the grid type's default)
        if (c.kernel == XS_KERNEL_PLAIN) {
            ctx->plain_block = c.block;
            for (int ts : {0, 1}) {
                ctx->tile_sort = ts;
                xs_run_opts o;
                xs_run_opts_init(&o);
                o.count = sample;
                o.tile_lookups = c.tile;
                double rate = 0;
                xs_status s = time_run(o, &rate);
                if (s != XS_OK) {
                    restore();
                    return s;
                }
                if (rate > c.rate) {
                    c.rate = rate;
                    c.tile_sort = ts;
                }
            }
        }
        restore();
        if (cache_path) cache_write(cache_path, key, c);
    }
    // install the choice
    for (const GridView &v : views)
        if (v.grid_type == c.grid_type && v.guided == c.guided) apply_view(ctx, v);
    ctx->plain_tile = c.tile;
    ctx->batched_buckets = c.buckets;
    ctx->batched_blocks_per_sm = c.blocks_per_sm;
    if (c.kernel == XS_KERNEL_PLAIN) {
        ctx->fuel_lanes = c.lanes;
        ctx->plain_block = c.block;
        if (c.tile_sort >= 0) ctx->tile_sort = c.tile_sort;
    } else {
        ctx->batched_fuel_lanes = c.lanes;
        ctx->batched_block = c.block;
    }
    for (auto &kv : ctx->graphs) cudaGraphExecDestroy(kv.second.exec);
    ctx->graphs.clear();
    if (best) {
        xs_run_opts_init(best);
        best->kernel = c.kernel;
        best->tile_lookups = c.tile;
        best->energy_buckets = c.buckets;
        best->block_threads = c.block;
    }
    return XS_OK;
}

extern "C" int xs_ctx_grid_type(const xs_ctx *ctx) { return ctx ? ctx->t.grid_type : -1; }
