/*
 * xs_oracle.c -- CPU restatement of XSBench's event-based macroscopic
 * cross-section lookup and of the problem setup that feeds it.
 *
 * TEST INFRASTRUCTURE ONLY (the checker, never the product): see xs_oracle.h.
 *
 * Every routine follows the reference file:line cited beside it, with the same
 * floating-point operation order.  It must be compiled with
 * -ffp-contract=off: the reference is built for x86-64 without FMA, so no
 * multiply-add is ever fused there, and aarch64 compilers would otherwise fuse.
 */
#include "xs_oracle.h"

#include <stdlib.h>
#include <string.h>
#include <time.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define OR_STARTING_SEED 1070ULL              /* XSbench_header.h:51 */
#define OR_LCG_MOD (1ULL << 63)               /* Simulation.c:465 */
#define OR_LCG_MUL 2806196910506780709ULL     /* Simulation.c:466 */
#define OR_LCG_INC 1ULL                       /* Simulation.c:467 */

/* ---------------------------------------------------------------- LCG --- */

/* Simulation.c:462-470: one LCG step, value = state / 2^63. */
double or_lcg_double(uint64_t *seed)
{
    *seed = (OR_LCG_MUL * (*seed) + OR_LCG_INC) % OR_LCG_MOD;
    return (double)(*seed) / (double)OR_LCG_MOD;
}

/* Simulation.c:472-499: skip n steps by square-and-multiply of the affine map. */
uint64_t or_lcg_skip(uint64_t seed, uint64_t n)
{
    uint64_t mul = OR_LCG_MUL, inc = OR_LCG_INC;
    uint64_t acc_mul = 1, acc_inc = 0;
    n %= OR_LCG_MOD;
    for (; n > 0; n >>= 1) {
        if (n & 1) {
            acc_mul *= mul;
            acc_inc = acc_inc * mul + inc;
        }
        inc *= (mul + 1);
        mul *= mul;
    }
    return (acc_mul * seed + acc_inc) % OR_LCG_MOD;
}

/* Simulation.c:426-460: material pick.  The running sum for material i is
 * re-accumulated from dist[i] down to dist[1] on every i (order matters). */
int or_pick_mat(uint64_t *seed)
{
    static const double dist[12] = {0.140, 0.052, 0.275, 0.134, 0.154, 0.064,
                                    0.066, 0.055, 0.008, 0.015, 0.025, 0.013};
    double roll = or_lcg_double(seed);
    for (int i = 0; i < 12; i++) {
        double running = 0;
        for (int j = i; j > 0; j--)
            running += dist[j];
        if (roll < running)
            return i;
    }
    return 0;
}

/* Simulation.c:62-70 */
void or_sample_event(long i, double *energy, int *mat)
{
    uint64_t seed = or_lcg_skip(OR_STARTING_SEED, 2 * (uint64_t)i);
    *energy = or_lcg_double(&seed);
    *mat = or_pick_mat(&seed);
}

/* ------------------------------------------------------------ searches --- */

/* Simulation.c:380-400 */
long or_grid_search(long n, double quarry, const double *A)
{
    long lo = 0, hi = n - 1;
    while (hi - lo > 1) {
        long mid = lo + (hi - lo) / 2;
        if (A[mid] > quarry) hi = mid; else lo = mid;
    }
    return lo;
}

/* Simulation.c:403-423 */
long or_grid_search_nuclide(long n, double quarry, const or_gridpoint *A, long low, long high)
{
    (void)n;
    long lo = low, hi = high;
    while (hi - lo > 1) {
        long mid = lo + (hi - lo) / 2;
        if (A[mid].energy > quarry) hi = mid; else lo = mid;
    }
    return lo;
}

/* ------------------------------------------------------------- lookups --- */

/* Simulation.c:241-323: micro XS of one nuclide.  idx is the union-grid index
 * (UNIONIZED) or the hash bin (HASH); unused for NUCLIDE. */
static void or_micro_xs(double E, int nuc, long n_iso, long n_gp, const int *restrict index_data,
                        const or_gridpoint *restrict grids, long idx, double *restrict xs,
                        int grid_type, int hash_bins)
{
    const or_gridpoint *nuc_grid = &grids[nuc * n_gp];
    const or_gridpoint *lo;
    if (grid_type == OR_NUCLIDE) {                                   /* :252-263 */
        long k = or_grid_search_nuclide(n_gp, E, nuc_grid, 0, n_gp - 1);
        lo = (k == n_gp - 1) ? &nuc_grid[k - 1] : &nuc_grid[k];
    } else if (grid_type == OR_UNIONIZED) {                          /* :264-272 */
        long k = index_data[idx * n_iso + nuc];
        lo = (k == n_gp - 1) ? &nuc_grid[k - 1] : &nuc_grid[k];
    } else {                                                         /* :273-302 */
        int u_low = index_data[idx * n_iso + nuc];
        int u_high = (idx == hash_bins - 1) ? (int)(n_gp - 1)
                                            : index_data[(idx + 1) * n_iso + nuc] + 1;
        double e_low = nuc_grid[u_low].energy;
        double e_high = nuc_grid[u_high].energy;
        int k;
        if (E <= e_low) k = 0;
        else if (E >= e_high) k = (int)(n_gp - 1);
        else k = (int)or_grid_search_nuclide(n_gp, E, nuc_grid, u_low, u_high);
        lo = (k == n_gp - 1) ? &nuc_grid[k - 1] : &nuc_grid[k];
    }
    const or_gridpoint *hi = lo + 1;
    double f = (hi->energy - E) / (hi->energy - lo->energy);         /* :307 */
    xs[0] = hi->total_xs - f * (hi->total_xs - lo->total_xs);        /* :310-322 */
    xs[1] = hi->elastic_xs - f * (hi->elastic_xs - lo->elastic_xs);
    xs[2] = hi->absorbtion_xs - f * (hi->absorbtion_xs - lo->absorbtion_xs);
    xs[3] = hi->fission_xs - f * (hi->fission_xs - lo->fission_xs);
    xs[4] = hi->nu_fission_xs - f * (hi->nu_fission_xs - lo->nu_fission_xs);
}

/* Simulation.c:326-375: macro XS = sum over the material's nuclides, in list order. */
void or_macro_xs(const or_inputs *in, const or_simdata *sd, double E, int mat, double *restrict macro)
{
    /* the reference passes these arrays as restrict parameters (Simulation.c:326-332) */
    const int *restrict mats = sd->mats;
    const double *restrict concs = sd->concs;
    const int *restrict index_grid = sd->index_grid;
    const or_gridpoint *restrict grid = sd->nuclide_grid;
    const long n_iso = in->n_isotopes, n_gp = in->n_gridpoints;
    const int grid_type = in->grid_type, hash_bins = in->hash_bins;
    long idx = -1;
    for (int k = 0; k < 5; k++) macro[k] = 0;
    if (grid_type == OR_UNIONIZED)
        idx = or_grid_search(n_iso * n_gp, E, sd->unionized_energy_array);
    else if (grid_type == OR_HASH) {
        double du = 1.0 / hash_bins;
        idx = (long)(E / du);
    }
    const int row = mat * sd->max_num_nucs;
    const int nn = sd->num_nucs[mat];
    for (int j = 0; j < nn; j++) {
        double xs[5];
        int nuc = mats[row + j];
        double conc = concs[row + j];
        or_micro_xs(E, nuc, n_iso, n_gp, index_grid, grid, idx, xs, grid_type, hash_bins);
        for (int k = 0; k < 5; k++) macro[k] += xs[k] * conc;
    }
}

/* Simulation.c:100-110 */
int or_argmax5(const double macro[5])
{
    double best = -1.0;
    int arg = 0;
    for (int k = 0; k < 5; k++)
        if (macro[k] > best) { best = macro[k]; arg = k; }
    return arg;
}

static double or_now(void)
{
    struct timespec ts;
    clock_gettime(CLOCK_MONOTONIC, &ts);
    return (double)ts.tv_sec + 1e-9 * (double)ts.tv_nsec;
}

static void or_set_threads(int nthreads)
{
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#else
    (void)nthreads;
#endif
}

/* Simulation.c:15-114 */
unsigned long long or_run_event(const or_inputs *in, const or_simdata *sd, long first, long n,
                                int nthreads, double *macro_out, unsigned char *maxidx_out,
                                double *energy_out, int *mat_out)
{
    unsigned long long verification = 0;
    or_set_threads(nthreads);
#pragma omp parallel for schedule(dynamic, 100) reduction(+ : verification)
    for (long t = 0; t < n; t++) {
        double E, macro[5];
        int mat;
        or_sample_event(first + t, &E, &mat);
        or_macro_xs(in, sd, E, mat, macro);
        int arg = or_argmax5(macro);
        verification += (unsigned long long)(arg + 1);
        if (macro_out) memcpy(&macro_out[t * 5], macro, sizeof macro);
        if (maxidx_out) maxidx_out[t] = (unsigned char)arg;
        if (energy_out) energy_out[t] = E;
        if (mat_out) mat_out[t] = mat;
    }
    return verification;
}

unsigned long long or_run_event_samples(const or_inputs *in, const or_simdata *sd, long n,
                                        const double *energy, const int *mat, int nthreads,
                                        double *macro_out, unsigned char *maxidx_out)
{
    unsigned long long verification = 0;
    or_set_threads(nthreads);
#pragma omp parallel for schedule(dynamic, 100) reduction(+ : verification)
    for (long t = 0; t < n; t++) {
        double macro[5];
        or_macro_xs(in, sd, energy[t], mat[t], macro);
        int arg = or_argmax5(macro);
        verification += (unsigned long long)(arg + 1);
        if (macro_out) memcpy(&macro_out[t * 5], macro, sizeof macro);
        if (maxidx_out) maxidx_out[t] = (unsigned char)arg;
    }
    return verification;
}

/* ---------------------------------------------- optimisation 1 (k1) --- */
/* Simulation.c:698-871: the sampling loop split from the lookups, the samples
 * sorted by material and then, within each material, by energy, and the
 * lookups run material by material.  The two sorts are parallel quicksorts
 * of (key, payload) pairs, as the reference's are (Simulation.c:565-688:
 * recursion into OpenMP tasks above 10,000 entries, at most 16 threads); the
 * one below is this oracle's own, a Hoare partition around the middle entry. */

#define OR_SORT_TASK_CUTOFF 10000

/* sort (mat key, energy payload) by material */
static void or_qsort_mat(int *key, double *val, long lo, long hi)
{
    while (lo < hi) {
        const int pivot = key[lo + (hi - lo) / 2];
        long a = lo, b = hi;
        while (a <= b) {
            while (key[a] < pivot) a++;
            while (key[b] > pivot) b--;
            if (a <= b) {
                int tk = key[a]; key[a] = key[b]; key[b] = tk;
                double tv = val[a]; val[a] = val[b]; val[b] = tv;
                a++;
                b--;
            }
        }
        if (hi - lo >= OR_SORT_TASK_CUTOFF) {
#pragma omp task
            or_qsort_mat(key, val, lo, b);
#pragma omp task
            or_qsort_mat(key, val, a, hi);
            return;
        }
        if (b - lo < hi - a) {     /* recurse into the shorter side */
            or_qsort_mat(key, val, lo, b);
            lo = a;
        } else {
            or_qsort_mat(key, val, a, hi);
            hi = b;
        }
    }
}

/* sort (energy key, mat payload) by energy */
static void or_qsort_energy(double *key, int *val, long lo, long hi)
{
    while (lo < hi) {
        const double pivot = key[lo + (hi - lo) / 2];
        long a = lo, b = hi;
        while (a <= b) {
            while (key[a] < pivot) a++;
            while (key[b] > pivot) b--;
            if (a <= b) {
                double tk = key[a]; key[a] = key[b]; key[b] = tk;
                int tv = val[a]; val[a] = val[b]; val[b] = tv;
                a++;
                b--;
            }
        }
        if (hi - lo >= OR_SORT_TASK_CUTOFF) {
#pragma omp task
            or_qsort_energy(key, val, lo, b);
#pragma omp task
            or_qsort_energy(key, val, a, hi);
            return;
        }
        if (b - lo < hi - a) {
            or_qsort_energy(key, val, lo, b);
            lo = a;
        } else {
            or_qsort_energy(key, val, a, hi);
            hi = b;
        }
    }
}

static int or_sort_threads(int nthreads)
{
    return nthreads > 16 ? 16 : (nthreads > 0 ? nthreads : 1);   /* Simulation.c:612-613 */
}

unsigned long long or_run_event_k1(const or_inputs *in, const or_simdata *sd, long first, long n,
                                   int nthreads, double phase_s[4])
{
    double *E = (double *)malloc((size_t)(n > 0 ? n : 1) * sizeof(double));
    int *M = (int *)malloc((size_t)(n > 0 ? n : 1) * sizeof(int));
    unsigned long long verification = 0;
    if (!E || !M) {
        free(E);
        free(M);
        return 0;
    }
    or_set_threads(nthreads);
    double t0 = or_now();
#pragma omp parallel for schedule(dynamic, 100)
    for (long t = 0; t < n; t++) or_sample_event(first + t, &E[t], &M[t]);
    double t1 = or_now();
#pragma omp parallel num_threads(or_sort_threads(nthreads))
    {
#pragma omp single nowait
        if (n > 1) or_qsort_mat(M, E, 0, n - 1);
    }
    long count[12] = {0}, offset[12] = {0};
    for (long t = 0; t < n; t++) count[M[t]]++;
    for (int m = 1; m < 12; m++) offset[m] = offset[m - 1] + count[m - 1];
    for (int m = 0; m < 12; m++) {
#pragma omp parallel num_threads(or_sort_threads(nthreads))
        {
#pragma omp single nowait
            if (count[m] > 1) or_qsort_energy(E + offset[m], M + offset[m], 0, count[m] - 1);
        }
    }
    double t2 = or_now();
    for (int m = 0; m < 12; m++) {
#pragma omp parallel for schedule(dynamic, 100) reduction(+ : verification)
        for (long t = offset[m]; t < offset[m] + count[m]; t++) {
            double macro[5];
            or_macro_xs(in, sd, E[t], M[t], macro);
            verification += (unsigned long long)(or_argmax5(macro) + 1);
        }
    }
    double t3 = or_now();
    if (phase_s) {
        phase_s[0] = t1 - t0;   /* sampling */
        phase_s[1] = t2 - t1;   /* material and energy sorts */
        phase_s[2] = t3 - t2;   /* lookups */
        phase_s[3] = t3 - t0;
    }
    free(E);
    free(M);
    return verification;
}

/* Simulation.c:116-238: 'lookups' dependent lookups per particle. */
unsigned long long or_run_history(const or_inputs *in, const or_simdata *sd, long first, long n,
                                  int nthreads)
{
    unsigned long long verification = 0;
    or_set_threads(nthreads);
#pragma omp parallel for schedule(dynamic, 100) reduction(+ : verification)
    for (long t = 0; t < n; t++) {
        long p = first + t;
        /* Simulation.c:167: the skip is computed in int arithmetic there. */
        uint64_t seed = or_lcg_skip(OR_STARTING_SEED,
                                    (uint64_t)(int)((int)p * in->lookups * 2 * 5));
        double E = or_lcg_double(&seed);
        int mat = or_pick_mat(&seed);
        for (int i = 0; i < in->lookups; i++) {
            double macro[5];
            or_macro_xs(in, sd, E, mat, macro);
            verification += (unsigned long long)(or_argmax5(macro) + 1);
            uint64_t n_forward = 0;
            for (int k = 0; k < 5; k++)
                if (macro[k] > 1.0) n_forward++;
            if (n_forward > 0) seed = or_lcg_skip(seed, n_forward);
            E = or_lcg_double(&seed);
            mat = or_pick_mat(&seed);
        }
    }
    return verification;
}

/* --------------------------------------------------------------- setup --- */

/* XSutils.c:16-28 / :3-14: order by energy only. */
static int or_cmp_gridpoint(const void *a, const void *b)
{
    double x = ((const or_gridpoint *)a)->energy, y = ((const or_gridpoint *)b)->energy;
    return (x > y) - (x < y);
}
static int or_cmp_double(const void *a, const void *b)
{
    double x = *(const double *)a, y = *(const double *)b;
    return (x > y) - (x < y);
}

/* Materials.c:7-31 */
static void or_load_num_nucs(long n_iso, int num_nucs[12])
{
    static const int rest[11] = {5, 4, 4, 27, 21, 21, 21, 21, 21, 9, 9};
    num_nucs[0] = (n_iso == 68) ? 34 : 321;
    for (int m = 1; m < 12; m++) num_nucs[m] = rest[m - 1];
}

/* Materials.c:34-96: nuclide lists; the large fuel list extends the small one
 * with nuclides 68..354. */
static void or_load_mats(const int num_nucs[12], long n_iso, int max_nucs, int *mats)
{
    static const int fuel_small[34] = {58, 59, 60, 61, 40, 42, 43, 44, 45, 46, 1,  2,
                                       3,  7,  8,  9,  10, 29, 57, 47, 48, 0,  62, 15,
                                       33, 34, 52, 53, 54, 55, 56, 18, 23, 41};
    static const int cladding[5] = {63, 64, 65, 66, 67};
    static const int water[4] = {24, 41, 4, 5};
    static const int rpv[27] = {19, 20, 21, 22, 35, 36, 37, 38, 39, 25, 27, 28, 29, 30,
                                31, 32, 26, 49, 50, 51, 11, 12, 13, 14, 6,  16, 17};
    static const int reflector[21] = {24, 41, 4,  5,  19, 20, 21, 22, 35, 36, 37,
                                      38, 39, 25, 49, 50, 51, 11, 12, 13, 14};
    static const int assembly_end[9] = {24, 41, 4, 5, 63, 64, 65, 66, 67};
    const int *lists[12] = {NULL,      cladding,  water,     water,     rpv,          reflector,
                            reflector, reflector, reflector, reflector, assembly_end, assembly_end};
    memset(mats, 0, sizeof(int) * 12 * (size_t)max_nucs);
    for (int j = 0; j < num_nucs[0]; j++)
        mats[j] = (j < 34) ? fuel_small[j] : 68 + (j - 34);
    (void)n_iso;
    for (int m = 1; m < 12; m++)
        memcpy(&mats[m * max_nucs], lists[m], sizeof(int) * (size_t)num_nucs[m]);
}

/* Materials.c:99-117: one LCG stream seeded 1070^2, row-major (material, nuclide). */
static void or_load_concs(const int num_nucs[12], int max_nucs, double *concs)
{
    uint64_t seed = OR_STARTING_SEED * OR_STARTING_SEED;
    memset(concs, 0, sizeof(double) * 12 * (size_t)max_nucs);
    for (int m = 0; m < 12; m++)
        for (int j = 0; j < num_nucs[m]; j++)
            concs[m * max_nucs + j] = or_lcg_double(&seed);
}

/* GridInit.c:3-230 (no AML replicas). */
int or_grid_init(const or_inputs *in, or_simdata *sd)
{
    memset(sd, 0, sizeof *sd);
    const long n_iso = in->n_isotopes, n_gp = in->n_gridpoints;

    /* GridInit.c:34-51: one sequential stream from seed 42, six draws per point. */
    sd->length_nuclide_grid = (int)(n_iso * n_gp);
    sd->nuclide_grid = (or_gridpoint *)malloc(sizeof(or_gridpoint) * (size_t)sd->length_nuclide_grid);
    if (!sd->nuclide_grid) return 1;
    uint64_t seed = 42;
    for (long p = 0; p < (long)sd->length_nuclide_grid; p++) {
        or_gridpoint *g = &sd->nuclide_grid[p];
        g->energy = or_lcg_double(&seed);
        g->total_xs = or_lcg_double(&seed);
        g->elastic_xs = or_lcg_double(&seed);
        g->absorbtion_xs = or_lcg_double(&seed);
        g->fission_xs = or_lcg_double(&seed);
        g->nu_fission_xs = or_lcg_double(&seed);
    }
    for (long i = 0; i < n_iso; i++)
        qsort(&sd->nuclide_grid[i * n_gp], (size_t)n_gp, sizeof(or_gridpoint), or_cmp_gridpoint);

    if (in->grid_type == OR_UNIONIZED) {                       /* GridInit.c:74-126 */
        long n_union = n_iso * n_gp;
        sd->length_unionized_energy_array = (int)n_union;
        sd->unionized_energy_array = (double *)malloc(sizeof(double) * (size_t)n_union);
        if (!sd->unionized_energy_array) return 1;
        for (long e = 0; e < n_union; e++)
            sd->unionized_energy_array[e] = sd->nuclide_grid[e].energy;
        qsort(sd->unionized_energy_array, (size_t)n_union, sizeof(double), or_cmp_double);

        sd->length_index_grid = n_union * n_iso;
        sd->index_grid = (int *)malloc(sizeof(int) * (size_t)sd->length_index_grid);
        int *cursor = (int *)calloc((size_t)n_iso, sizeof(int));
        double *next_e = (double *)malloc(sizeof(double) * (size_t)n_iso);
        if (!sd->index_grid || !cursor || !next_e) { free(cursor); free(next_e); return 1; }
        for (long i = 0; i < n_iso; i++) next_e[i] = sd->nuclide_grid[i * n_gp + 1].energy;
        /* GridInit.c:106-122: sweep the union grid, advancing each nuclide's
         * cursor by at most one point per union energy, capped at n_gp-2. */
        for (long e = 0; e < n_union; e++) {
            double u = sd->unionized_energy_array[e];
            int *row = &sd->index_grid[e * n_iso];
            for (long i = 0; i < n_iso; i++) {
                if (!(u < next_e[i]) && cursor[i] != n_gp - 2) {
                    cursor[i]++;
                    next_e[i] = sd->nuclide_grid[i * n_gp + cursor[i] + 1].energy;
                }
                row[i] = cursor[i];
            }
        }
        free(cursor);
        free(next_e);
    } else if (in->grid_type == OR_HASH) {                     /* GridInit.c:128-151 */
        sd->length_unionized_energy_array = 0;
        sd->length_index_grid = (long)in->hash_bins * n_iso;
        sd->index_grid = (int *)malloc(sizeof(int) * (size_t)sd->length_index_grid);
        if (!sd->index_grid) return 1;
        double du = 1.0 / in->hash_bins;
#pragma omp parallel for
        for (long e = 0; e < in->hash_bins; e++) {
            double energy = e * du;
            for (long i = 0; i < n_iso; i++)
                sd->index_grid[e * n_iso + i] = (int)or_grid_search_nuclide(
                    n_gp, energy, &sd->nuclide_grid[i * n_gp], 0, n_gp - 1);
        }
    } else {                                                   /* GridInit.c:68-72 */
        sd->length_unionized_energy_array = 0;
        sd->length_index_grid = 0;
    }

    /* GridInit.c:156-174 */
    int num_nucs[12];
    or_load_num_nucs(n_iso, num_nucs);
    int max_nucs = 0;
    for (int m = 0; m < 12; m++) if (num_nucs[m] > max_nucs) max_nucs = num_nucs[m];
    sd->length_num_nucs = 12;
    sd->num_nucs = (int *)malloc(sizeof num_nucs);
    sd->max_num_nucs = max_nucs;
    sd->length_mats = 12 * max_nucs;
    sd->length_concs = sd->length_mats;
    sd->mats = (int *)malloc(sizeof(int) * (size_t)sd->length_mats);
    sd->concs = (double *)malloc(sizeof(double) * (size_t)sd->length_concs);
    if (!sd->num_nucs || !sd->mats || !sd->concs) return 1;
    memcpy(sd->num_nucs, num_nucs, sizeof num_nucs);
    or_load_mats(num_nucs, n_iso, max_nucs, sd->mats);
    or_load_concs(num_nucs, max_nucs, sd->concs);
    return 0;
}

void or_simdata_free(or_simdata *sd)
{
    free(sd->num_nucs);
    free(sd->concs);
    free(sd->mats);
    free(sd->unionized_energy_array);
    free(sd->index_grid);
    free(sd->nuclide_grid);
    free(sd->p_energy_samples);
    free(sd->mat_samples);
    memset(sd, 0, sizeof *sd);
}
