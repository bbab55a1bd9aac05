/*
 * xs_oracle.h -- CPU restatement of XSBench's event-based cross-section lookup.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the checker for the GB300 kernels:
 * only tests/, __graft_entry__.smoke() and bench.py's cpu_baseline / reference
 * arm may load it.  The product (xsbench_gb300/) never links or calls it.
 *
 * Parity is pinned: the restatement reproduces the reference's published
 * verification hashes (openmp-threading/io.c:89-90) and the per-lookup
 * macro_xs / setup-array digests dumped from the reference built from source
 * (tests/golden/).
 *
 * The struct layouts are those of openmp-threading/XSbench_header.h:54-102
 * (without the AML members), so arrays made by the reference's
 * grid_init_do_not_profile, by this oracle, or by the product's host setup can
 * be passed to any of them.
 */
#ifndef XS_ORACLE_H
#define XS_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* openmp-threading/XSbench_header.h:37-39 */
enum { OR_UNIONIZED = 0, OR_NUCLIDE = 1, OR_HASH = 2 };
/* openmp-threading/XSbench_header.h:42-43 */
enum { OR_HISTORY_BASED = 1, OR_EVENT_BASED = 2 };

typedef struct { /* openmp-threading/XSbench_header.h:54-61 */
    double energy, total_xs, elastic_xs, absorbtion_xs, fission_xs, nu_fission_xs;
} or_gridpoint;

typedef struct { /* openmp-threading/XSbench_header.h:63-75 */
    int nthreads;
    long n_isotopes;
    long n_gridpoints;
    int lookups;
    char *HM;
    int grid_type;
    int hash_bins;
    int particles;
    int simulation_method;
    int binary_mode;
    int kernel_id;
} or_inputs;

typedef struct { /* openmp-threading/XSbench_header.h:77-102 (no AML) */
    int *num_nucs;
    double *concs;
    int *mats;
    double *unionized_energy_array;
    int *index_grid;
    or_gridpoint *nuclide_grid;
    int length_num_nucs;
    int length_concs;
    int length_mats;
    int length_unionized_energy_array;
    long length_index_grid;
    int length_nuclide_grid;
    int max_num_nucs;
    double *p_energy_samples;
    int length_p_energy_samples;
    int *mat_samples;
    int length_mat_samples;
} or_simdata;

/* Problem setup (openmp-threading/GridInit.c:3-230, Materials.c:7-117).
 * Returns 0 on success, non-zero on allocation failure. */
int or_grid_init(const or_inputs *in, or_simdata *sd);
void or_simdata_free(or_simdata *sd);

/* LCG pieces (openmp-threading/Simulation.c:426-499). */
double or_lcg_double(uint64_t *seed);
uint64_t or_lcg_skip(uint64_t seed, uint64_t n);
int or_pick_mat(uint64_t *seed);
/* Sample of event lookup i (Simulation.c:62-70). */
void or_sample_event(long i, double *energy, int *mat);

/* Searches (Simulation.c:380-423). */
long or_grid_search(long n, double quarry, const double *A);
long or_grid_search_nuclide(long n, double quarry, const or_gridpoint *A, long low, long high);

/* One macroscopic lookup (Simulation.c:326-375). */
void or_macro_xs(const or_inputs *in, const or_simdata *sd, double energy, int mat, double *macro);

/* argmax rule of the verification (Simulation.c:100-110): returns max_idx in 0..4. */
int or_argmax5(const double macro[5]);

/* Event-based loop (Simulation.c:15-114) over lookups [first, first+n).
 * Returns the un-modded verification sum.  macro_out (n*5) and maxidx_out (n)
 * may be NULL.  energy_out / mat_out (n) may be NULL. nthreads<=0: OpenMP default. */
unsigned long long or_run_event(const or_inputs *in, const or_simdata *sd, long first, long n,
                                int nthreads, double *macro_out, unsigned char *maxidx_out,
                                double *energy_out, int *mat_out);

/* Event lookups with caller-supplied (energy, material) samples. */
/* Optimisation 1 (Simulation.c:698-871) over lookups [first, first+n): sample,
 * sort by material then by energy, look up material by material.  The same
 * verification sum as or_run_event.  phase_s (nullable) receives the seconds
 * of sampling, sorting, lookups and the total. */
unsigned long long or_run_event_k1(const or_inputs *in, const or_simdata *sd, long first, long n,
                                   int nthreads, double phase_s[4]);
unsigned long long or_run_event_samples(const or_inputs *in, const or_simdata *sd, long n,
                                        const double *energy, const int *mat, int nthreads,
                                        double *macro_out, unsigned char *maxidx_out);

/* History-based loop (Simulation.c:116-238) over particles [first, first+n). */
unsigned long long or_run_history(const or_inputs *in, const or_simdata *sd, long first, long n,
                                  int nthreads);

#ifdef __cplusplus
}
#endif
#endif
