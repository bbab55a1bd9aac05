// setup_host.cu -- host side of the library: command line, problem setup,
// dataset file.
//
// xs_grid_init builds exactly the arrays of the reference's
// grid_init_do_not_profile (openmp-threading/GridInit.c:3-230,
// Materials.c:7-117) with the host's cores:
//   * the one sequential LCG stream of the nuclide grid is split into
//     per-thread ranges with the closed-form skip-ahead, so every draw lands
//     where the serial loop puts it;
//   * per-nuclide sorts, the union sort and the hash grid run in parallel;
//   * the unionized index grid is swept in row ranges.  Within a nuclide whose
//     energies are strictly increasing, the reference's sweep (one step per
//     union energy, capped at n_gp-2) leaves min(n_gp-2, #{j>=1 : E_j <= u})
//     after union energy u, so a range can start from that count; a nuclide
//     with repeated energies falls back to the serial sweep.
#include <algorithm>
#include <atomic>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <functional>
#include <strings.h>
#include <thread>
#include <vector>

#include "device_common.cuh"

namespace xsgb {

// Simulation.c:433-445 material volume fractions
static const double kDist[kMaterials] = {0.140, 0.052, 0.275, 0.134, 0.154, 0.064,
                                         0.066, 0.055, 0.008, 0.015, 0.025, 0.013};

void pick_mat_thresholds(double out[kMaterials])
{
    // Simulation.c:450-457: running sum for material i, from dist[i] down to dist[1]
    for (int i = 0; i < kMaterials; i++) {
        double running = 0;
        for (int j = i; j > 0; j--) running += kDist[j];
        out[i] = running;
    }
}

static int host_threads()
{
    unsigned n = std::thread::hardware_concurrency();
    if (const char *e = getenv("XSGB_HOST_THREADS")) n = (unsigned)atoi(e);
    return n < 1 ? 1 : (int)(n > 64 ? 64 : n);
}

static void parallel_for(long n, int threads, const std::function<void(long, long)> &body)
{
    if (n <= 0) return;
    if (threads > n) threads = (int)n;
    if (threads <= 1) {
        body(0, n);
        return;
    }
    std::vector<std::thread> pool;
    for (int t = 0; t < threads; t++) {
        long a = n * t / threads, b = n * (t + 1) / threads;
        pool.emplace_back([=, &body] { body(a, b); });
    }
    for (auto &th : pool) th.join();
}

// parallel merge sort of doubles (ascending, std::sort order)
static void parallel_sort(double *v, long n, int threads)
{
    int parts = 1;
    while (parts * 2 <= threads && n / (parts * 2) > 65536) parts *= 2;
    std::vector<long> cut(parts + 1);
    for (int p = 0; p <= parts; p++) cut[p] = n * p / parts;
    parallel_for(parts, parts, [&](long a, long b) {
        for (long p = a; p < b; p++) std::sort(v + cut[p], v + cut[p + 1]);
    });
    std::vector<double> tmp((size_t)n);
    double *src = v, *dst = tmp.data();
    for (int w = 1; w < parts; w *= 2) {
        const int pairs = (parts + 2 * w - 1) / (2 * w);
        parallel_for(pairs, pairs, [&](long a, long b) {
            for (long q = a; q < b; q++) {
                long lo = cut[q * 2 * w], mid = cut[std::min<long>(parts, q * 2 * w + w)],
                     hi = cut[std::min<long>(parts, q * 2 * w + 2 * w)];
                std::merge(src + lo, src + mid, src + mid, src + hi, dst + lo);
            }
        });
        std::swap(src, dst);
    }
    if (src != v) std::memcpy(v, src, sizeof(double) * (size_t)n);
}

// Simulation.c:403-423 (lower-bound search, returns the lower index)
static long search_points(const xs_gridpoint *A, double q, long lo, long hi)
{
    while (hi - lo > 1) {
        long mid = lo + (hi - lo) / 2;
        if (A[mid].energy > q) hi = mid; else lo = mid;
    }
    return lo;
}

// Materials.c:7-117
xs_status load_materials(long n_iso, xs_simdata *sd)
{
    static const int rest[11] = {5, 4, 4, 27, 21, 21, 21, 21, 21, 9, 9};
    static const int fuel34[34] = {58, 59, 60, 61, 40, 42, 43, 44, 45, 46, 1,  2,
                                   3,  7,  8,  9,  10, 29, 57, 47, 48, 0,  62, 15,
                                   33, 34, 52, 53, 54, 55, 56, 18, 23, 41};
    static const int clad[5] = {63, 64, 65, 66, 67};
    static const int water[4] = {24, 41, 4, 5};
    static const int rpv[27] = {19, 20, 21, 22, 35, 36, 37, 38, 39, 25, 27, 28, 29, 30,
                                31, 32, 26, 49, 50, 51, 11, 12, 13, 14, 6,  16, 17};
    static const int refl[21] = {24, 41, 4, 5, 19, 20, 21, 22, 35, 36, 37,
                                 38, 39, 25, 49, 50, 51, 11, 12, 13, 14};
    static const int fa_end[9] = {24, 41, 4, 5, 63, 64, 65, 66, 67};
    static const int *const lists[kMaterials] = {nullptr, clad, water, water, rpv,    refl,
                                                 refl,    refl, refl,  refl,  fa_end, fa_end};
    int nn[kMaterials];
    nn[0] = (n_iso == 68) ? 34 : 321;
    for (int m = 1; m < kMaterials; m++) nn[m] = rest[m - 1];
    int mx = 0;
    for (int m = 0; m < kMaterials; m++) mx = std::max(mx, nn[m]);
    // the lists name nuclides up to 67 (small) or 354 (large)
    const int highest = (n_iso == 68) ? 67 : 354;
    if (n_iso <= highest)
        return fail(XS_ERR_INVALID_ARGUMENT, "n_isotopes %ld: the material lists need 68 (small) or at least 355 nuclides", n_iso);
    sd->length_num_nucs = kMaterials;
    sd->max_num_nucs = mx;
    sd->length_mats = kMaterials * mx;
    sd->length_concs = sd->length_mats;
    sd->num_nucs = (int *)malloc(sizeof nn);
    sd->mats = (int *)calloc((size_t)sd->length_mats, sizeof(int));
    sd->concs = (double *)calloc((size_t)sd->length_concs, sizeof(double));
    if (!sd->num_nucs || !sd->mats || !sd->concs) return fail(XS_ERR_OUT_OF_MEMORY, "material tables");
    std::memcpy(sd->num_nucs, nn, sizeof nn);
    for (int j = 0; j < nn[0]; j++) sd->mats[j] = j < 34 ? fuel34[j] : 68 + (j - 34);
    for (int m = 1; m < kMaterials; m++)
        std::memcpy(sd->mats + m * mx, lists[m], sizeof(int) * (size_t)nn[m]);
    unsigned long long seed = kStartingSeed * kStartingSeed;  // Materials.c:101
    for (int m = 0; m < kMaterials; m++)
        for (int j = 0; j < nn[m]; j++) sd->concs[m * mx + j] = lcg_next(seed);
    return XS_OK;
}

}  // namespace xsgb

using namespace xsgb;

extern "C" {

// ----------------------------------------------------------- command line
static xs_status cli_error(const char *what)
{
    return fail(XS_ERR_INVALID_ARGUMENT, "%s (usage: -t threads -g gridpoints -m event|history -l lookups -h hash_bins -p particles -s small|large|XL|XXL -G unionized|nuclide|hash -b read|write -k kernel)", what);
}

xs_status xs_read_cli(int argc, char **argv, xs_inputs *out)
{
    if (!out) return fail(XS_ERR_INVALID_ARGUMENT, "xs_read_cli: out is NULL");
    static char large_name[] = "large";
    xs_inputs in;
    std::memset(&in, 0, sizeof in);
    // defaults: io.c:231-272
    in.simulation_method = XS_HISTORY_BASED;
    in.nthreads = (int)std::thread::hardware_concurrency();
    in.n_isotopes = 355;
    in.n_gridpoints = 11303;
    in.particles = 500000;
    in.lookups = 34;
    in.grid_type = XS_UNIONIZED;
    in.hash_bins = 10000;
    in.binary_mode = XS_BINARY_NONE;
    in.kernel_id = 0;
    in.HM = large_name;
    int user_g = 0, default_lookups = 1, default_particles = 1;
    for (int i = 1; i < argc; i++) {  // io.c:281-412
        const char *a = argv[i];
        auto need = [&](void) -> const char * { return (i + 1 < argc) ? argv[++i] : nullptr; };
        const char *v;
        if (!strcmp(a, "-t")) {
            if (!(v = need())) return cli_error("-t needs a value");
            in.nthreads = atoi(v);
        } else if (!strcmp(a, "-g")) {
            if (!(v = need())) return cli_error("-g needs a value");
            user_g = 1;
            in.n_gridpoints = atol(v);
        } else if (!strcmp(a, "-m")) {
            if (!(v = need())) return cli_error("-m needs a value");
            if (!strcmp(v, "history")) in.simulation_method = XS_HISTORY_BASED;
            else if (!strcmp(v, "event")) {
                in.simulation_method = XS_EVENT_BASED;
                if (default_lookups && default_particles) {  // io.c:319-323
                    in.lookups = in.lookups * in.particles;
                    in.particles = 0;
                }
            } else return cli_error("unknown simulation method");
        } else if (!strcmp(a, "-l")) {
            if (!(v = need())) return cli_error("-l needs a value");
            in.lookups = atoi(v);
            default_lookups = 0;
        } else if (!strcmp(a, "-h")) {
            if (!(v = need())) return cli_error("-h needs a value");
            in.hash_bins = atoi(v);
        } else if (!strcmp(a, "-p")) {
            if (!(v = need())) return cli_error("-p needs a value");
            in.particles = atoi(v);
            default_particles = 0;
        } else if (!strcmp(a, "-s")) {
            if (!(v = need())) return cli_error("-s needs a value");
            in.HM = (char *)v;
        } else if (!strcmp(a, "-G")) {
            if (!(v = need())) return cli_error("-G needs a value");
            if (!strcmp(v, "unionized")) in.grid_type = XS_UNIONIZED;
            else if (!strcmp(v, "nuclide")) in.grid_type = XS_NUCLIDE;
            else if (!strcmp(v, "hash")) in.grid_type = XS_HASH;
            else return cli_error("unknown grid type");
        } else if (!strcmp(a, "-b")) {
            if (!(v = need())) return cli_error("-b needs a value");
            if (!strcmp(v, "read")) in.binary_mode = XS_BINARY_READ;
            else if (!strcmp(v, "write")) in.binary_mode = XS_BINARY_WRITE;
            else return cli_error("unknown binary mode");
        } else if (!strcmp(a, "-k")) {
            if (!(v = need())) return cli_error("-k needs a value");
            in.kernel_id = atoi(v);
        } else {
            return cli_error("unknown argument");
        }
    }
    // io.c:416-441
    if (in.nthreads < 1) return cli_error("threads must be >= 1");
    if (in.n_isotopes < 1) return cli_error("isotopes must be >= 1");
    if (in.n_gridpoints < 1) return cli_error("gridpoints must be >= 1");
    if (in.lookups < 1) return cli_error("lookups must be >= 1");
    if (in.hash_bins < 1) return cli_error("hash bins must be >= 1");
    if (strcasecmp(in.HM, "small") && strcasecmp(in.HM, "large") && strcasecmp(in.HM, "XL") &&
        strcasecmp(in.HM, "XXL"))
        return cli_error("unknown problem size");
    // io.c:445-450
    if (!strcasecmp(in.HM, "small")) in.n_isotopes = 68;
    else if (!strcasecmp(in.HM, "XL") && !user_g) in.n_gridpoints = 238847;
    else if (!strcasecmp(in.HM, "XXL") && !user_g) in.n_gridpoints = (long)(238847 * 2.1);
    *out = in;
    return XS_OK;
}

// ------------------------------------------------------------------- setup
void xs_simdata_free(xs_simdata *sd)
{
    if (!sd) return;
    free(sd->num_nucs);
    free(sd->concs);
    free(sd->mats);
    free(sd->unionized_energy_array);
    free(sd->index_grid);
    free(sd->nuclide_grid);
    free(sd->p_energy_samples);
    free(sd->mat_samples);
    std::memset(sd, 0, sizeof *sd);
}

xs_status xs_grid_init(const xs_inputs *in, xs_simdata *out)
{
    if (!in || !out) return fail(XS_ERR_INVALID_ARGUMENT, "xs_grid_init: NULL argument");
    if (in->n_isotopes < 1 || in->n_gridpoints < 2)
        return fail(XS_ERR_INVALID_ARGUMENT, "need n_isotopes >= 1 and n_gridpoints >= 2");
    if (in->grid_type < 0 || in->grid_type > 2) return fail(XS_ERR_INVALID_ARGUMENT, "grid_type %d", in->grid_type);
    if (in->grid_type == XS_HASH && in->hash_bins < 1) return fail(XS_ERR_INVALID_ARGUMENT, "hash_bins %d", in->hash_bins);
    const long n_iso = in->n_isotopes, n_gp = in->n_gridpoints;
    const long n_pts = n_iso * n_gp;
    if (n_pts > 0x7FFFFFFFL) return fail(XS_ERR_INVALID_ARGUMENT, "n_isotopes*n_gridpoints above 2^31-1 (int lengths of the reference layout)");
    const int T = host_threads();
    xs_simdata sd;
    std::memset(&sd, 0, sizeof sd);

    // GridInit.c:34-47: one stream from seed 42, six draws per point
    sd.length_nuclide_grid = (int)n_pts;
    sd.nuclide_grid = (xs_gridpoint *)malloc(sizeof(xs_gridpoint) * (size_t)n_pts);
    if (!sd.nuclide_grid) return fail(XS_ERR_OUT_OF_MEMORY, "nuclide grid (%ld points)", n_pts);
    parallel_for(n_pts, T, [&](long a, long b) {
        unsigned long long s = lcg_skip(42ULL, 6ULL * (unsigned long long)a);
        for (long p = a; p < b; p++) {
            xs_gridpoint &g = sd.nuclide_grid[p];
            g.energy = lcg_next(s);
            g.total_xs = lcg_next(s);
            g.elastic_xs = lcg_next(s);
            g.absorbtion_xs = lcg_next(s);
            g.fission_xs = lcg_next(s);
            g.nu_fission_xs = lcg_next(s);
        }
    });
    // GridInit.c:50-51: order each nuclide by energy
    parallel_for(n_iso, T, [&](long a, long b) {
        for (long i = a; i < b; i++)
            std::stable_sort(sd.nuclide_grid + i * n_gp, sd.nuclide_grid + (i + 1) * n_gp,
                             [](const xs_gridpoint &x, const xs_gridpoint &y) { return x.energy < y.energy; });
    });

    if (in->grid_type == XS_UNIONIZED) {  // GridInit.c:74-126
        sd.length_unionized_energy_array = (int)n_pts;
        sd.unionized_energy_array = (double *)malloc(sizeof(double) * (size_t)n_pts);
        sd.length_index_grid = n_pts * n_iso;
        sd.index_grid = (int *)malloc(sizeof(int) * (size_t)sd.length_index_grid);
        if (!sd.unionized_energy_array || !sd.index_grid) {
            xs_simdata_free(&sd);
            return fail(XS_ERR_OUT_OF_MEMORY, "unionized grid (%ld x %ld)", n_pts, n_iso);
        }
        double *u = sd.unionized_energy_array;
        parallel_for(n_pts, T, [&](long a, long b) {
            for (long p = a; p < b; p++) u[p] = sd.nuclide_grid[p].energy;
        });
        parallel_sort(u, n_pts, T);
        // strictly increasing energies per nuclide?
        std::vector<char> strict((size_t)n_iso, 1);
        parallel_for(n_iso, T, [&](long a, long b) {
            for (long i = a; i < b; i++)
                for (long j = 1; j < n_gp; j++)
                    if (!(sd.nuclide_grid[i * n_gp + j - 1].energy < sd.nuclide_grid[i * n_gp + j].energy)) {
                        strict[i] = 0;
                        break;
                    }
        });
        int *idx = sd.index_grid;
        // rows in ranges; nuclides with repeated energies are swept serially below
        parallel_for(n_pts, T, [&](long a, long b) {
            std::vector<int> cur((size_t)n_iso);
            std::vector<double> nxt((size_t)n_iso);
            for (long i = 0; i < n_iso; i++) {
                const xs_gridpoint *g = sd.nuclide_grid + i * n_gp;
                long c = 0;
                if (a > 0) {
                    // #{j >= 1 : E_j <= u[a-1]}
                    const double q = u[a - 1];
                    long lo = 1, hi = n_gp;
                    while (lo < hi) {
                        long mid = (lo + hi) / 2;
                        if (g[mid].energy <= q) lo = mid + 1; else hi = mid;
                    }
                    c = std::min(lo - 1, n_gp - 2);
                }
                cur[i] = (int)c;
                nxt[i] = g[c + 1].energy;
            }
            for (long e = a; e < b; e++) {
                const double ue = u[e];
                int *row = idx + e * n_iso;
                for (long i = 0; i < n_iso; i++) {
                    if (!(ue < nxt[i]) && cur[i] != n_gp - 2) {
                        cur[i]++;
                        nxt[i] = sd.nuclide_grid[i * n_gp + cur[i] + 1].energy;
                    }
                    row[i] = cur[i];
                }
            }
        });
        for (long i = 0; i < n_iso; i++) {
            if (strict[i]) continue;
            int c = 0;
            double nx = sd.nuclide_grid[i * n_gp + 1].energy;
            for (long e = 0; e < n_pts; e++) {
                if (!(u[e] < nx) && c != n_gp - 2) {
                    c++;
                    nx = sd.nuclide_grid[i * n_gp + c + 1].energy;
                }
                idx[e * n_iso + i] = c;
            }
        }
    } else if (in->grid_type == XS_HASH) {  // GridInit.c:128-151
        sd.length_index_grid = (long)in->hash_bins * n_iso;
        sd.index_grid = (int *)malloc(sizeof(int) * (size_t)sd.length_index_grid);
        if (!sd.index_grid) {
            xs_simdata_free(&sd);
            return fail(XS_ERR_OUT_OF_MEMORY, "hash grid");
        }
        const double du = 1.0 / in->hash_bins;
        parallel_for(in->hash_bins, T, [&](long a, long b) {
            for (long e = a; e < b; e++) {
                const double energy = e * du;
                for (long i = 0; i < n_iso; i++)
                    sd.index_grid[e * n_iso + i] =
                        (int)search_points(sd.nuclide_grid + i * n_gp, energy, 0, n_gp - 1);
            }
        });
    }
    xs_status s = load_materials(n_iso, &sd);
    if (s != XS_OK) {
        xs_simdata_free(&sd);
        return s;
    }
    *out = sd;
    return XS_OK;
}

// ------------------------------------------------------------ dataset file
// io.c:456-508: struct, then num_nucs, concs, mats, nuclide_grid, index_grid,
// unionized_energy_array.
xs_status xs_binary_write(const char *path, const xs_simdata *sd)
{
    if (!path || !sd) return fail(XS_ERR_INVALID_ARGUMENT, "xs_binary_write: NULL argument");
    FILE *f = fopen(path, "wb");
    if (!f) return fail(XS_ERR_IO, "cannot open %s for writing", path);
    bool ok = fwrite(sd, sizeof *sd, 1, f) == 1;
    ok = ok && fwrite(sd->num_nucs, sizeof(int), (size_t)sd->length_num_nucs, f) == (size_t)sd->length_num_nucs;
    ok = ok && fwrite(sd->concs, sizeof(double), (size_t)sd->length_concs, f) == (size_t)sd->length_concs;
    ok = ok && fwrite(sd->mats, sizeof(int), (size_t)sd->length_mats, f) == (size_t)sd->length_mats;
    ok = ok && fwrite(sd->nuclide_grid, sizeof(xs_gridpoint), (size_t)sd->length_nuclide_grid, f) == (size_t)sd->length_nuclide_grid;
    if (sd->length_index_grid > 0)
        ok = ok && fwrite(sd->index_grid, sizeof(int), (size_t)sd->length_index_grid, f) == (size_t)sd->length_index_grid;
    if (sd->length_unionized_energy_array > 0)
        ok = ok && fwrite(sd->unionized_energy_array, sizeof(double), (size_t)sd->length_unionized_energy_array, f) == (size_t)sd->length_unionized_energy_array;
    ok = (fclose(f) == 0) && ok;
    return ok ? XS_OK : fail(XS_ERR_IO, "short write to %s", path);
}

xs_status xs_binary_read(const char *path, xs_simdata *out)
{
    if (!path || !out) return fail(XS_ERR_INVALID_ARGUMENT, "xs_binary_read: NULL argument");
    FILE *f = fopen(path, "rb");
    if (!f) return fail(XS_ERR_IO, "cannot open %s", path);
    xs_simdata sd;
    if (fread(&sd, sizeof sd, 1, f) != 1) {
        fclose(f);
        return fail(XS_ERR_IO, "%s: truncated header", path);
    }
    if (sd.length_num_nucs != kMaterials || sd.length_mats < 0 || sd.length_concs != sd.length_mats ||
        sd.length_nuclide_grid < 0 || sd.length_index_grid < 0 || sd.length_unionized_energy_array < 0 ||
        sd.max_num_nucs < 1 || (long)sd.length_mats != (long)kMaterials * sd.max_num_nucs) {
        fclose(f);
        return fail(XS_ERR_IO, "%s: header lengths are not those of an XSBench dataset", path);
    }
    xs_simdata r;
    std::memset(&r, 0, sizeof r);
    r.length_num_nucs = sd.length_num_nucs;
    r.length_concs = sd.length_concs;
    r.length_mats = sd.length_mats;
    r.length_unionized_energy_array = sd.length_unionized_energy_array;
    r.length_index_grid = sd.length_index_grid;
    r.length_nuclide_grid = sd.length_nuclide_grid;
    r.max_num_nucs = sd.max_num_nucs;
    r.num_nucs = (int *)malloc(sizeof(int) * kMaterials);
    r.concs = (double *)malloc(sizeof(double) * (size_t)r.length_concs);
    r.mats = (int *)malloc(sizeof(int) * (size_t)r.length_mats);
    r.nuclide_grid = (xs_gridpoint *)malloc(sizeof(xs_gridpoint) * (size_t)std::max(1, r.length_nuclide_grid));
    if (r.length_index_grid > 0) r.index_grid = (int *)malloc(sizeof(int) * (size_t)r.length_index_grid);
    if (r.length_unionized_energy_array > 0)
        r.unionized_energy_array = (double *)malloc(sizeof(double) * (size_t)r.length_unionized_energy_array);
    if (!r.num_nucs || !r.concs || !r.mats || !r.nuclide_grid ||
        (r.length_index_grid > 0 && !r.index_grid) ||
        (r.length_unionized_energy_array > 0 && !r.unionized_energy_array)) {
        fclose(f);
        xs_simdata_free(&r);
        return fail(XS_ERR_OUT_OF_MEMORY, "dataset arrays");
    }
    bool ok = fread(r.num_nucs, sizeof(int), kMaterials, f) == (size_t)kMaterials;
    ok = ok && fread(r.concs, sizeof(double), (size_t)r.length_concs, f) == (size_t)r.length_concs;
    ok = ok && fread(r.mats, sizeof(int), (size_t)r.length_mats, f) == (size_t)r.length_mats;
    ok = ok && fread(r.nuclide_grid, sizeof(xs_gridpoint), (size_t)r.length_nuclide_grid, f) == (size_t)r.length_nuclide_grid;
    if (r.length_index_grid > 0)
        ok = ok && fread(r.index_grid, sizeof(int), (size_t)r.length_index_grid, f) == (size_t)r.length_index_grid;
    if (r.length_unionized_energy_array > 0)
        ok = ok && fread(r.unionized_energy_array, sizeof(double), (size_t)r.length_unionized_energy_array, f) == (size_t)r.length_unionized_energy_array;
    fclose(f);
    if (!ok) {
        xs_simdata_free(&r);
        return fail(XS_ERR_IO, "%s: truncated arrays", path);
    }
    *out = r;
    return XS_OK;
}

}  // extern "C"
