/*
 * xsgb.h -- C ABI of the GB300 (sm_103a) event-based macroscopic
 * cross-section lookup: a drop-in for the lookup loop of XSBench.
 *
 * Plain C: pointers, sizes and status codes only, so that C, ctypes, cgo or
 * any other FFI can bind it.  Every call returns an xs_status and never exits
 * the process; xs_last_error() holds the message of the calling thread's last
 * failure.  A context (xs_ctx) owns the device copy of one problem; it is not
 * thread-safe (one context per host thread), and calls on it are ordered on
 * the context's CUDA stream and block until their results are written.
 *
 * The struct layouts xs_gridpoint / xs_inputs / xs_simdata are identical to
 * NuclideGridPoint / Inputs / SimulationData of the reference
 * (openmp-threading/XSbench_header.h:54-102, AML members absent), so arrays made
 * by the reference's grid_init_do_not_profile (openmp-threading/GridInit.c:3)
 * can be passed by pointer cast, and arrays made by xs_grid_init can be passed
 * back to the reference's own functions.
 */
#ifndef XSGB_H
#define XSGB_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define XSGB_VERSION 1

/* ------------------------------------------------------------------ types */

typedef enum {
    XS_OK = 0,
    XS_ERR_INVALID_ARGUMENT = 1, /* bad pointer, size or option (reference: print_CLI_error/exit) */
    XS_ERR_OUT_OF_MEMORY = 2,    /* host or device allocation failed (reference: assert) */
    XS_ERR_CUDA = 3,             /* a CUDA runtime call failed (reference: gpuErrchk abort) */
    XS_ERR_NO_DEVICE = 4,        /* no usable sm_103 device */
    XS_ERR_TIMEOUT = 5,          /* a bounded device-side wait ran out */
    XS_ERR_DATA = 6,             /* a checked run found an out-of-range table index or material */
    XS_ERR_UNSUPPORTED = 7,      /* option not available for this problem */
    XS_ERR_IO = 8                /* file could not be read or written */
} xs_status;

/* Grid types: openmp-threading/XSbench_header.h:37-39 */
enum { XS_UNIONIZED = 0, XS_NUCLIDE = 1, XS_HASH = 2 };
/* Simulation methods: openmp-threading/XSbench_header.h:42-43 */
enum { XS_HISTORY_BASED = 1, XS_EVENT_BASED = 2 };
/* Binary modes: openmp-threading/XSbench_header.h:46-48 */
enum { XS_BINARY_NONE = 0, XS_BINARY_READ = 1, XS_BINARY_WRITE = 2 };

typedef struct { /* = NuclideGridPoint, openmp-threading/XSbench_header.h:54-61 */
    double energy;
    double total_xs;
    double elastic_xs;
    double absorbtion_xs;
    double fission_xs;
    double nu_fission_xs;
} xs_gridpoint;

typedef struct { /* = Inputs, openmp-threading/XSbench_header.h:63-75 */
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
} xs_inputs;

typedef struct { /* = SimulationData, openmp-threading/XSbench_header.h:77-102 */
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
    double *p_energy_samples;
    int length_p_energy_samples;
    int *mat_samples;
    int length_mat_samples;
} xs_simdata;

typedef struct xs_ctx xs_ctx;

/* Lookup kernels.  PLAIN is the drop-in for the event loop
 * (openmp-threading/Simulation.c:15, cuda/Simulation.cu:15): one launch that
 * samples, block-sorts by material and looks up.  BATCHED is the sorted form
 * (cuda/Simulation.cu:1024, optimisation 6): on-device counting sort by
 * (material, energy bucket), then one persistent lookup kernel, all in one
 * CUDA graph. */
typedef enum { XS_KERNEL_PLAIN = 0, XS_KERNEL_BATCHED = 1 } xs_kernel;

/* Arithmetic.  EXACT performs the reference's floating-point operations in the
 * reference's order with no fused multiply-add and IEEE division
 * (openmp-threading/Simulation.c:307-322, :372-373), so every macro_xs is
 * bit-identical to the reference's.  FAST interpolates with per-interval slopes
 * precomputed at context creation (one subtraction and five FMAs per nuclide
 * instead of a division and fifteen operations); its macro_xs stay within
 * 1e-12 relative of the reference's.  Both are FP64 throughout. */
typedef enum { XS_ARITH_FAST = 0, XS_ARITH_EXACT = 1 } xs_arith;

typedef struct {
    int kernel;          /* xs_kernel */
    int arith;           /* xs_arith */
    long first;          /* first event index (lookup i uses seed skip 2*i) */
    long count;          /* number of lookups; <= 0 means inputs.lookups - first */
    int block_threads;   /* 0 = tuned default; else 128, 256 or 512 */
    int tile_lookups;    /* PLAIN: lookups per block tile; 0 = default */
    int energy_buckets;  /* BATCHED: energy buckets per material (power of 2); 0 = default */
    int checked;         /* 1: bounds-check every table index and report XS_ERR_DATA */
    int async;           /* 1: only enqueue (device or NULL outputs); finish with xs_ctx_sync */
    void *stream;        /* cudaStream_t to order on; NULL = the context's own stream
                            (so the legacy default stream cannot be named here) */
} xs_run_opts;

/* Results of one run.  Output arrays may be NULL, host memory or device
 * memory; host arrays are filled through a device staging buffer. */
typedef struct {
    unsigned long long verification; /* un-modded sum of (argmax+1), Simulation.c:110 */
    float device_ms;                 /* CUDA-event time of the lookup work on the stream */
    int kernel_launches;             /* kernels this call launched (graph nodes included) */
} xs_run_result;

/* -------------------------------------------------------- host-side setup */

/* Reads the reference's command line (openmp-threading/io.c:227-454): flags
 * -t -g -m -l -h -p -s -G -b -k with the same defaults and resolution.  Returns
 * XS_ERR_INVALID_ARGUMENT where the reference would print_CLI_error() and exit.
 * out->HM points into argv or at a static string. */
xs_status xs_read_cli(int argc, char **argv, xs_inputs *out);

/* Builds the problem exactly as grid_init_do_not_profile does
 * (openmp-threading/GridInit.c:3-230, Materials.c:7-117): same LCG streams,
 * orders and tables, bit for bit; multi-threaded on the host.
 * Arrays are malloc'd; release them with xs_simdata_free. */
xs_status xs_grid_init(const xs_inputs *in, xs_simdata *out);
void xs_simdata_free(xs_simdata *sd);

/* Dataset file in the reference's format (openmp-threading/io.c:456-508):
 * the raw xs_simdata struct, then num_nucs, concs, mats, nuclide_grid,
 * index_grid, unionized_energy_array. */
xs_status xs_binary_write(const char *path, const xs_simdata *sd);
xs_status xs_binary_read(const char *path, xs_simdata *out);

/* ------------------------------------------------------------ device side */

/* Copies one problem to device `device` and builds the device-side derived
 * tables (slope records, search keys, union-grid bins; on the nuclide grid,
 * and on a hash grid whose energy keys exceed L2, an energy-bin guide and
 * bin records: per nuclide and bin a copy of the interval record the bin's
 * search starts at, 47.6 GB for the XL problem, built when the device keeps
 * 16 GiB free beside them).  Replaces move_simulation_data_to_device
 * (cuda/GridInit.cu:4).  The caller keeps ownership of the host arrays. */
xs_status xs_ctx_create(const xs_inputs *in, const xs_simdata *sd, int device, xs_ctx **out);

/* Builds the problem directly on the device: the same tables as
 * xs_grid_init (bit for bit), with no host arrays and no upload.  Replaces
 * grid_init_do_not_profile (openmp-threading/GridInit.c:3) followed by
 * move_simulation_data_to_device (cuda/GridInit.cu:4).  Returns
 * XS_ERR_UNSUPPORTED for a unionized problem in which a nuclide draws the same
 * energy twice (probability ~n_gridpoints^2 / 2^53; xs_grid_init handles it). */
xs_status xs_ctx_create_on_device(const xs_inputs *in, int device, xs_ctx **out);

/* Copies the context's setup arrays back into host arrays shaped like
 * xs_grid_init's (for checking); release with xs_simdata_free. */
xs_status xs_ctx_download(xs_ctx *ctx, xs_simdata *out);

/* Releases the device memory (cuda/GridInit.cu:81 release_device_memory). */
void xs_ctx_destroy(xs_ctx *ctx);

/* Bytes of device memory the context holds. */
size_t xs_ctx_device_bytes(const xs_ctx *ctx);

/* Bytes of the context's union table (0: not built).  For a unionized problem
 * the context reconstructs every nuclide's cross sections on the union grid:
 * per material and union row, each nuclide's five xs at the row energy and
 * the slopes of its interval (80 bytes), so a FAST lookup reads its
 * material's entries of one row contiguously instead of an index entry and a
 * 96-byte interval per nuclide.  Built at context creation when the device
 * has the room (n_union x sum(num_nucs) x 80 bytes, 155 GB for the large
 * problem, plus 24 GiB to spare); XSGB_UNION_TABLE=0 in the environment
 * disables it.  No reference counterpart. */
size_t xs_ctx_union_table_bytes(const xs_ctx *ctx);

/* Fills opts with defaults (PLAIN, FAST, all lookups, tuned shapes). */
void xs_run_opts_init(xs_run_opts *opts);

/* Event-based lookups [first, first+count) with in-kernel LCG sampling: the
 * drop-in for run_event_based_simulation (openmp-threading/Simulation.c:15;
 * cuda/Simulation.cu:15 and :1024).  macro_xs_out (count*5 doubles) and
 * max_idx_out (count bytes, argmax 0..4) may be NULL, device or host memory;
 * host outputs (every non-NULL one) are filled chunk by chunk, each chunk's
 * copy overlapping the next chunks' lookups (page-locked host memory lets
 * the copies overlap); device_ms then covers the copies too. */
xs_status xs_run_event(xs_ctx *ctx, const xs_run_opts *opts, double *macro_xs_out,
                       unsigned char *max_idx_out, xs_run_result *result);

/* The event samples alone: energy and material of lookups [first,
 * first+count), as the reference's sampling loop / kernel produce them
 * (openmp-threading/Simulation.c:735-750, cuda/Simulation.cu:441).  Output
 * arrays may be host or device memory. */
xs_status xs_sample_event(xs_ctx *ctx, long first, long count, double *energy_out,
                          int *mat_out);

/* Waits for the work enqueued by async runs and returns the last run's
 * verification sum and error state (device_ms covers the last run). */
xs_status xs_ctx_sync(xs_ctx *ctx, xs_run_result *result);

/* Lookups of caller-supplied samples (energy, material) -- the sampling split
 * of optimisation 1 (openmp-threading/Simulation.c:735-750,
 * cuda/Simulation.cu:441) with the samples owned by the caller.  Arrays may be
 * host or device memory; host arrays are streamed through the device in
 * overlapped chunks (their copies overlap the lookups when the host arrays
 * are page-locked, cudaHostAlloc / cudaHostRegister; pageable arrays work,
 * but the driver stages their copies and they serialise).  Materials outside
 * 0..11 give XS_ERR_DATA. */
xs_status xs_lookup_samples(xs_ctx *ctx, const xs_run_opts *opts, const double *energy,
                            const int *mat, long n, double *macro_xs_out,
                            unsigned char *max_idx_out, xs_run_result *result);

/* History-based lookups (openmp-threading/Simulation.c:116-238) for particles
 * [first, first+count) of opts (count <= 0: inputs.particles).  PLAIN: one
 * thread per particle walks its lookups, as the reference does.  BATCHED: the
 * particles advance in lockstep, step by step: the i-th lookups of all
 * particles run as one event batch through the plain lookup kernel, then each
 * particle's next sample is drawn (the same seeds, skips and samples as the
 * reference's loop), so material sorting and load balance apply to history
 * mode too. */
xs_status xs_run_history(xs_ctx *ctx, const xs_run_opts *opts, xs_run_result *result);

/* Adjoint of the lookup (no reference counterpart: the reference has no
 * derivatives; it differentiates calculate_macro_xs, Simulation.c:241-375).
 * For upstream gradients gbar (count*5: dL/dmacro_xs of lookups
 * [first, first+count) for a scalar loss L) it computes
 *   d_energy (count)                      =  dL/d(sampled energy)
 *   d_concs  (12*max_num_nucs)           +=  dL/dconcs
 *   d_xs     (n_isotopes*n_gridpoints*5) +=  dL/d(tabulated xs: total, elastic,
 *                                            absorbtion, fission, nu_fission)
 * and, when macro_xs_out is non-NULL, the forward macro_xs (count*5).  Any
 * output may be NULL.  The search indices are recomputed, not stored.  Every
 * sum runs in a fixed order over a deterministic (material, energy, index)
 * sort, so the results are bit-reproducible.  Arrays may be host or device
 * memory (all of one kind). */
xs_status xs_run_adjoint(xs_ctx *ctx, const xs_run_opts *opts, const double *gbar,
                         double *macro_xs_out, double *d_concs, double *d_xs,
                         double *d_energy, xs_run_result *result);

/* The same for caller-supplied samples (energy, mat: n entries). */
xs_status xs_adjoint_samples(xs_ctx *ctx, const xs_run_opts *opts, const double *energy,
                             const int *mat, long n, const double *gbar, double *macro_xs_out,
                             double *d_concs, double *d_xs, double *d_energy,
                             xs_run_result *result);

/* Autotuner (no reference counterpart).  Times, on a sample of up to 4M of
 * the context's event lookups, the plain kernel's tile sizes, the batched
 * kernel's energy buckets, the persistent kernels' blocks per SM, the lanes
 * per fuel lookup, the chosen kernel's threads per block (128, 256, 512) and every
 * grid type the context can serve (it derives a 10,000-bin hash grid and the
 * nuclide grid's search keys on the device when missing; all grid types give
 * the same intervals), installs the fastest as the context's defaults and
 * returns it in *best (kernel, tile_lookups, energy_buckets, block_threads).  With
 * cache_path non-NULL the choice is read from, or merged into, a JSON file
 * keyed by (device name, problem), and a cached choice is installed without
 * timing. */
xs_status xs_autotune(xs_ctx *ctx, const char *cache_path, xs_run_opts *best);

/* Grid type the context currently looks up with (changes after xs_autotune). */
int xs_ctx_grid_type(const xs_ctx *ctx);

/* Allocation-free batched run.  It has no counterpart in the reference.
 * The same lookups as xs_run_event with the BATCHED kernel, for callers that
 * must not allocate device memory -- e.g. a host thread that drives other GPU
 * work and must not stall it (cudaMalloc/cudaFree can synchronise the device),
 * or a program whose memory manager owns the device budget.  Its sort buffers
 * and counters live in one static device array of 6.5 MB that every GPU
 * loading this library holds until exit; so it takes at most 524,288 lookups
 * (count) and 4,096 energy buckets per call (larger values are rejected with
 * XS_ERR_INVALID_ARGUMENT), and it calls no allocating routine.
 * energy_buckets <= 0 takes the context's batched bucket count, capped at 4,096.
 * Outputs (macro_xs_out count*5, max_idx_out count) must be NULL or device
 * memory of the context's device (or managed memory); *verification (host)
 * receives the un-modded sum; the call is ordered on `stream` (NULL: the
 * context's stream) and returns when it is done.  It runs on the context's
 * device and leaves the calling thread's current device as it found it.
 * The first call on a device (and the first after that device's CUDA context
 * was re-created, e.g. by a cudaDeviceReset) looks up the array's device
 * address (cudaGetSymbolAddress), so make that first call before any stream
 * capture.  All calls share the one array, which keeps the last call's
 * contents (each call clears its counters and histogram first): calls whose
 * work overlaps on the GPU (other streams, other host threads) race on it and
 * must be serialised by the caller. */
xs_status xs_run_event_batched_static(xs_ctx *ctx, long first, long count, int arith,
                                      int energy_buckets, double *macro_xs_out,
                                      unsigned char *max_idx_out, void *stream,
                                      unsigned long long *verification);

/* Full drop-in of the reference seam
 *   unsigned long long run_event_based_simulation(Inputs, SimulationData, int)
 * (openmp-threading/XSbench_header.h:117): creates a context on device 0,
 * runs the plain kernel over in.lookups lookups, destroys the context and
 * stores the un-modded verification sum. */
xs_status xs_run_event_based_simulation(xs_inputs in, xs_simdata sd, int mype,
                                        unsigned long long *verification);

/* ----------------------------------------------------------------- errors */

const char *xs_status_str(xs_status s);
const char *xs_last_error(void);

#ifdef __cplusplus
}
#endif
#endif /* XSGB_H */
