/*
 * ref_harness.c -- dump harness around the reference's own openmp-threading
 * code, compiled from its sources into oracle/_ref/libxsref.so (see
 * oracle/Makefile).  TEST INFRASTRUCTURE ONLY: it exists to generate the
 * golden fixtures under tests/golden/ and to cross-check the oracle in this
 * container; nothing in the product links it.
 *
 * It calls the reference's functions unchanged:
 *   grid_init_do_not_profile  (openmp-threading/GridInit.c:3)
 *   fast_forward_LCG, LCG_random_double, pick_mat, calculate_macro_xs
 *                             (openmp-threading/Simulation.c:472,462,426,326)
 *   run_event_based_simulation / run_history_based_simulation
 *                             (openmp-threading/Simulation.c:15,116)
 *   run_event_based_simulation_optimization_1
 *                             (openmp-threading/Simulation.c:698)
 */
#include "XSbench_header.h"

SimulationData *refh_grid_init(Inputs *in)
{
    SimulationData *sd = (SimulationData *)malloc(sizeof(SimulationData));
    *sd = grid_init_do_not_profile(*in, 1);
    return sd;
}

void refh_free(SimulationData *sd)
{
    free(sd->num_nucs);
    free(sd->concs);
    free(sd->mats);
    if (sd->length_unionized_energy_array > 0) free(sd->unionized_energy_array);
    if (sd->length_index_grid > 0) free(sd->index_grid);
    free(sd->nuclide_grid);
    free(sd);
}

/* Per-lookup dump of the event loop body (Simulation.c:62-110). */
unsigned long long refh_run_event(Inputs *in, SimulationData *sd, long first, long n,
                                  double *macro_out, unsigned char *maxidx_out,
                                  double *energy_out, int *mat_out)
{
    unsigned long long verification = 0;
#pragma omp parallel for schedule(dynamic, 100) reduction(+ : verification)
    for (long t = 0; t < n; t++) {
        uint64_t seed = fast_forward_LCG(STARTING_SEED, 2 * (uint64_t)(first + t));
        double E = LCG_random_double(&seed);
        int mat = pick_mat(&seed);
        double macro[5] = {0};
        calculate_macro_xs(E, mat, in->n_isotopes, in->n_gridpoints, sd->num_nucs, sd->concs,
                           sd->unionized_energy_array, sd->index_grid, sd->nuclide_grid,
                           sd->mats, macro, in->grid_type, in->hash_bins, sd->max_num_nucs);
        double best = -1.0;
        int arg = 0;
        for (int k = 0; k < 5; k++)
            if (macro[k] > best) { best = macro[k]; arg = k; }
        verification += arg + 1;
        if (macro_out) for (int k = 0; k < 5; k++) macro_out[t * 5 + k] = macro[k];
        if (maxidx_out) maxidx_out[t] = (unsigned char)arg;
        if (energy_out) energy_out[t] = E;
        if (mat_out) mat_out[t] = mat;
    }
    return verification;
}

unsigned long long refh_event_simulation(Inputs *in, SimulationData *sd)
{
    return run_event_based_simulation(*in, *sd, 1);
}

/* Optimisation 1 (Simulation.c:698-871) over in->lookups lookups. */
unsigned long long refh_event_k1(Inputs *in, SimulationData *sd)
{
    return run_event_based_simulation_optimization_1(*in, *sd, 1);
}

unsigned long long refh_history_simulation(Inputs *in, SimulationData *sd)
{
    return run_history_based_simulation(*in, *sd, 1);
}

void refh_set_threads(int n)
{
#ifdef OPENMP
    omp_set_num_threads(n);
#endif
}
