// ref_cuda_harness.cu -- times the reference's own CUDA lookup kernels on
// this GPU.  TEST INFRASTRUCTURE ONLY (a comparison measurement).
//
// The reference's cuda/Simulation.cu is compiled from its sources into a
// cubin (oracle/Makefile, target refcuda); its host driver cannot run here,
// so this harness plays that role: it builds the problem (xs_grid_init, bit
// identical to the reference's grid_init_do_not_profile), uploads it the way
// move_simulation_data_to_device does (cuda/GridInit.cu:4-79), loads the
// cubin with the driver API and launches the reference's kernels:
//   -k 0  xs_lookup_kernel_baseline, 256 threads per block
//         (cuda/Simulation.cu:15-38)
//   -k 1..6  sampling_kernel, then the optimisations' lookup launches, 32
//         threads per block: 1 one kernel (:464), 2 one per material over all
//         samples (:576), 3 fuel and non-fuel over all samples (:692), 4 the
//         samples sorted by material, one launch per material (:823), 5 fuel
//         partitioned first, two launches (:960), 6 sorted by material and
//         energy, one launch per material of the optimisation-4 kernel
//         (:1062-1086); the thrust sorts / partition run on the host here and
//         are not timed
// Only the lookup launches are timed (CUDA events); the per-lookup
// verification array is summed on the host afterwards.  Output: one JSON line.
#include <cuda.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <numeric>
#include <string>
#include <vector>

#include "../include/xsgb.h"

// cuda/XSbench_header.cuh:65-89 (the CUDA build's SimulationData)
struct RefCudaSimData {
    int *num_nucs;
    double *concs;
    int *mats;
    double *unionized_energy_array;
    int *index_grid;
    xs_gridpoint *nuclide_grid;
    int length_num_nucs;
    int length_concs;
    int length_mats;
    int length_unionized_energy_array;
    long length_index_grid;
    int length_nuclide_grid;
    int max_num_nucs;
    unsigned long *verification;
    int length_verification;
    double *p_energy_samples;
    int length_p_energy_samples;
    int *mat_samples;
    int length_mat_samples;
};

#define CK(x)                                                                        \
    do {                                                                             \
        cudaError_t e = (x);                                                         \
        if (e != cudaSuccess) {                                                      \
            fprintf(stderr, "%s: %s\n", #x, cudaGetErrorString(e));                  \
            return 2;                                                                \
        }                                                                            \
    } while (0)
#define CKD(x)                                                                       \
    do {                                                                             \
        CUresult r = (x);                                                            \
        if (r != CUDA_SUCCESS) {                                                     \
            const char *msg = nullptr;                                               \
            cuGetErrorString(r, &msg);                                               \
            fprintf(stderr, "%s: %s\n", #x, msg ? msg : "?");                        \
            return 2;                                                                \
        }                                                                            \
    } while (0)

template <typename T>
static int upload(T **dst, const T *src, size_t n)
{
    CK(cudaMalloc((void **)dst, std::max<size_t>(n, 1) * sizeof(T)));
    if (n) CK(cudaMemcpy(*dst, src, n * sizeof(T), cudaMemcpyHostToDevice));
    return 0;
}

int main(int argc, char **argv)
{
    const char *cubin = "oracle/_ref/xsbench_cuda_sim.cubin";
    int kernel = 0, reps = 5;
    std::vector<char *> cli = {argv[0]};
    for (int i = 1; i < argc; i++) {
        if (!strcmp(argv[i], "--cubin") && i + 1 < argc) cubin = argv[++i];
        else if (!strcmp(argv[i], "--reps") && i + 1 < argc) reps = atoi(argv[++i]);
        else if (!strcmp(argv[i], "-k") && i + 1 < argc) kernel = atoi(argv[++i]);
        else cli.push_back(argv[i]);
    }
    xs_inputs in;
    if (xs_read_cli((int)cli.size(), cli.data(), &in) != XS_OK) {
        fprintf(stderr, "bad arguments: %s\n", xs_last_error());
        return 1;
    }
    in.simulation_method = XS_EVENT_BASED;
    xs_simdata sd;
    if (xs_grid_init(&in, &sd) != XS_OK) {
        fprintf(stderr, "grid init: %s\n", xs_last_error());
        return 1;
    }
    CKD(cuInit(0));
    CK(cudaSetDevice(0));
    CK(cudaFree(0));  // primary context
    CUmodule mod;
    CKD(cuModuleLoad(&mod, cubin));

    RefCudaSimData g;
    memset(&g, 0, sizeof g);
    g.length_num_nucs = sd.length_num_nucs;
    g.length_concs = sd.length_concs;
    g.length_mats = sd.length_mats;
    g.length_unionized_energy_array = sd.length_unionized_energy_array;
    g.length_index_grid = sd.length_index_grid;
    g.length_nuclide_grid = sd.length_nuclide_grid;
    g.max_num_nucs = sd.max_num_nucs;
    if (upload(&g.num_nucs, sd.num_nucs, (size_t)sd.length_num_nucs)) return 2;
    if (upload(&g.concs, sd.concs, (size_t)sd.length_concs)) return 2;
    if (upload(&g.mats, sd.mats, (size_t)sd.length_mats)) return 2;
    if (upload(&g.unionized_energy_array, sd.unionized_energy_array,
               (size_t)sd.length_unionized_energy_array)) return 2;
    if (upload(&g.index_grid, sd.index_grid, (size_t)sd.length_index_grid)) return 2;
    if (upload(&g.nuclide_grid, sd.nuclide_grid, (size_t)sd.length_nuclide_grid)) return 2;
    const long N = in.lookups;
    CK(cudaMalloc((void **)&g.verification, N * sizeof(unsigned long)));
    g.length_verification = (int)N;

    cudaEvent_t e0, e1;
    CK(cudaEventCreate(&e0));
    CK(cudaEventCreate(&e1));
    std::vector<float> times;
    const char *what;
    std::vector<int> counts(12, 0);

    if (kernel == 0) {
        what = "xs_lookup_kernel_baseline (cuda/Simulation.cu:44), 256 threads/block";
        CUfunction f;
        CKD(cuModuleGetFunction(&f, mod, "_Z25xs_lookup_kernel_baseline6Inputs14SimulationData"));
        void *params[] = {&in, &g};
        const unsigned blocks = (unsigned)((N + 255) / 256);
        for (int r = 0; r < reps + 1; r++) {
            CK(cudaEventRecord(e0));
            CKD(cuLaunchKernel(f, blocks, 1, 1, 256, 1, 1, 0, 0, params, nullptr));
            CK(cudaEventRecord(e1));
            CK(cudaEventSynchronize(e1));
            float ms;
            CK(cudaEventElapsedTime(&ms, e0, e1));
            if (r) times.push_back(ms);
        }
    } else if (kernel >= 1 && kernel <= 6) {
        // cuda/Simulation.cu:388-1099: sampling_kernel, then per variant
        // (samples reordered on the host where the reference runs thrust;
        // not timed) the lookup launches, 32 threads per block
        static const char *whats[7] = {
            "",
            "sampling_kernel, xs_lookup_kernel_optimization_1 (cuda/Simulation.cu:464); lookups timed",
            "sampling_kernel, 12 x xs_lookup_kernel_optimization_2 (cuda/Simulation.cu:576), one per "
            "material over all samples; lookups timed",
            "sampling_kernel, 2 x xs_lookup_kernel_optimization_3 (cuda/Simulation.cu:692), fuel and "
            "non-fuel over all samples; lookups timed",
            "sampling_kernel, host sort by material, 12 x xs_lookup_kernel_optimization_4 "
            "(cuda/Simulation.cu:823); lookups timed",
            "sampling_kernel, host partition fuel first, 2 x xs_lookup_kernel_optimization_5 "
            "(cuda/Simulation.cu:960); lookups timed",
            "sampling_kernel, host sort by (material, energy), 12 x xs_lookup_kernel_optimization_4 "
            "(cuda/Simulation.cu:823), 32 threads/block; lookups timed"};
        what = whats[kernel];
        CK(cudaMalloc((void **)&g.p_energy_samples, N * sizeof(double)));
        CK(cudaMalloc((void **)&g.mat_samples, N * sizeof(int)));
        g.length_p_energy_samples = g.length_mat_samples = (int)N;
        CUfunction fs, fk;
        CKD(cuModuleGetFunction(&fs, mod, "_Z15sampling_kernel6Inputs14SimulationData"));
        static const char *names[7] = {
            "", "_Z31xs_lookup_kernel_optimization_16Inputs14SimulationData",
            "_Z31xs_lookup_kernel_optimization_26Inputs14SimulationDatai",
            "_Z31xs_lookup_kernel_optimization_36Inputs14SimulationDatai",
            "_Z31xs_lookup_kernel_optimization_46Inputs14SimulationDataiii",
            "_Z31xs_lookup_kernel_optimization_56Inputs14SimulationDataii",
            "_Z31xs_lookup_kernel_optimization_46Inputs14SimulationDataiii"};
        CKD(cuModuleGetFunction(&fk, mod, names[kernel]));
        void *sp[] = {&in, &g};
        const unsigned all_blocks = (unsigned)((N + 31) / 32);
        CKD(cuLaunchKernel(fs, all_blocks, 1, 1, 32, 1, 1, 0, 0, sp, nullptr));
        CK(cudaDeviceSynchronize());
        int n_fuel = 0;
        if (kernel >= 4) {
            std::vector<double> E(N);
            std::vector<int> M(N);
            CK(cudaMemcpy(E.data(), g.p_energy_samples, N * 8, cudaMemcpyDeviceToHost));
            CK(cudaMemcpy(M.data(), g.mat_samples, N * 4, cudaMemcpyDeviceToHost));
            std::vector<long> order(N);
            std::iota(order.begin(), order.end(), 0L);
            if (kernel == 4)       // thrust::sort_by_key on the materials (:797)
                std::stable_sort(order.begin(), order.end(), [&](long a, long b) { return M[a] < M[b]; });
            else if (kernel == 5)  // thrust::partition, fuel first (:936)
                std::stable_partition(order.begin(), order.end(), [&](long a) { return M[a] == 0; });
            else                   // by material, then energy within each (:1067-1076)
                std::sort(order.begin(), order.end(), [&](long a, long b) {
                    return M[a] != M[b] ? M[a] < M[b] : E[a] < E[b];
                });
            std::vector<double> E2(N);
            std::vector<int> M2(N);
            for (long i = 0; i < N; i++) {
                E2[i] = E[order[i]];
                M2[i] = M[order[i]];
                counts[M2[i]]++;
            }
            n_fuel = counts[0];
            CK(cudaMemcpy(g.p_energy_samples, E2.data(), N * 8, cudaMemcpyHostToDevice));
            CK(cudaMemcpy(g.mat_samples, M2.data(), N * 4, cudaMemcpyHostToDevice));
        }
        for (int r = 0; r < reps + 1; r++) {
            CK(cudaEventRecord(e0));
            if (kernel == 1) {
                CKD(cuLaunchKernel(fk, all_blocks, 1, 1, 32, 1, 1, 0, 0, sp, nullptr));
            } else if (kernel == 2 || kernel == 3) {
                for (int m = 0; m < (kernel == 2 ? 12 : 2); m++) {
                    void *p2[] = {&in, &g, &m};
                    CKD(cuLaunchKernel(fk, all_blocks, 1, 1, 32, 1, 1, 0, 0, p2, nullptr));
                }
            } else if (kernel == 5) {
                int n0 = n_fuel, o0 = 0, n1 = (int)N - n_fuel, o1 = n_fuel;
                void *p5a[] = {&in, &g, &n0, &o0};
                void *p5b[] = {&in, &g, &n1, &o1};
                if (n0) CKD(cuLaunchKernel(fk, (unsigned)((n0 + 31) / 32), 1, 1, 32, 1, 1, 0, 0, p5a, nullptr));
                if (n1) CKD(cuLaunchKernel(fk, (unsigned)((n1 + 31) / 32), 1, 1, 32, 1, 1, 0, 0, p5b, nullptr));
            } else {
                int offset = 0;
                for (int m = 0; m < 12; m++) {
                    int n_m = counts[m];
                    void *p4[] = {&in, &g, &m, &n_m, &offset};
                    const unsigned blocks = (unsigned)((n_m + 31) / 32);
                    if (blocks) CKD(cuLaunchKernel(fk, blocks, 1, 1, 32, 1, 1, 0, 0, p4, nullptr));
                    offset += n_m;
                }
            }
            CK(cudaEventRecord(e1));
            CK(cudaEventSynchronize(e1));
            float ms;
            CK(cudaEventElapsedTime(&ms, e0, e1));
            if (r) times.push_back(ms);
        }
    } else {
        fprintf(stderr, "kernel %d: use 0 to 6\n", kernel);
        return 1;
    }
    std::vector<unsigned long> v(N);
    CK(cudaMemcpy(v.data(), g.verification, N * sizeof(unsigned long), cudaMemcpyDeviceToHost));
    unsigned long long sum = 0;
    for (long i = 0; i < N; i++) sum += v[i];
    std::sort(times.begin(), times.end());
    const double ms = times[times.size() / 2];
    printf("{\"impl\": \"reference-cuda\", \"kernel\": %d, \"what\": \"%s\", \"size\": \"%s\", "
           "\"grid_type\": %d, \"lookups\": %ld, \"ms\": %.4f, \"lookups_per_s\": %.6g, "
           "\"verification\": %llu, \"hash\": %llu}\n",
           kernel, what, in.HM, in.grid_type, N, ms, N / (ms * 1e-3), sum, sum % 999983ULL);
    xs_simdata_free(&sd);
    return 0;
}
