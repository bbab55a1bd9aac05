// xsgb_internal.h -- shared declarations of the GB300 lookup library.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <map>
#include <string>
#include <vector>

#include "../../include/xsgb.h"

namespace xsgb {

constexpr int kMaterials = 12;
constexpr int kRecordDoubles = 16;      // fast-mode interval record: 96 bytes used, 128-byte slot
constexpr int kRecordPairs = kRecordDoubles / 2;
constexpr int kCoarseStride = 16;       // NUCLIDE grid: one coarse key per 16 energies
constexpr unsigned long long kStartingSeed = 1070ULL;  // XSbench_header.h:51

// Record layout of interval k of nuclide n (fast arithmetic):
//   [0] E_hi  [1..5] xs_hi[5]  [6..10] slope[5] = (hi-lo)/(E_hi-E_lo)  [11] E_lo
// 96 bytes = three 32-byte sectors, in a 128-byte-aligned 128-byte slot: a
// record then always lies in two aligned 64-byte DRAM bursts.  At a 96-byte
// stride half the records straddled three bursts' worth of sector requests
// that reached DRAM unmerged (measured 158 B per record read).

// Read-only device view of one problem, passed by value to the kernels.
struct Tables {
    int n_iso;
    int grid_type;
    long n_gp;
    int hash_bins;
    int max_nucs;
    double hash_du;                  // 1.0 / hash_bins, as the reference computes it
    int hash_margin;                 // xsgb_hash_margin_bits(hash_bins)
    long n_union;
    int union_bin_log2;              // union accelerator: 2^b bins over [0,1)
    int n_coarse;                    // coarse keys per nuclide (NUCLIDE grid)
    const int *num_nucs;             // [12]
    const int *mats;                 // [12 * max_nucs]
    const double *concs;             // [12 * max_nucs]
    const xs_gridpoint *grid;        // [n_iso * n_gp]  reference AoS
    const double2 *records;          // [n_iso * (n_gp-1) * kRecordPairs] fast records
    const long long *ekeys;          // [n_iso * n_gp]  order keys of grid energies
    const long long *coarse;         // [n_iso * n_coarse]
    const double *union_e;           // [n_union]
    const long long *union_keys;     // [n_union]
    const int *union_bins;           // [2^b + 1]
    const int *index_grid;           // UEG: [n_union * n_iso]  HASH: [hash_bins * n_iso]
    // energy-bin guide of each nuclide (searches of the hash and nuclide
    // grids): guide[nuc * (2^guide_log2 + 1) + b] = #{j : E_j < b * 2^-guide_log2},
    // b = 0 .. 2^guide_log2; null when not built
    const int *guide;
    int guide_log2;
    // bin records (FAST): for nuclide nuc and guide bin b, a copy of the
    // interval record of interval k0 = clamp(guide[nuc][b] - 1, 0, n_gp - 2) --
    // the interval holding the bin's lower edge -- and k0 itself (double 12
    // of the slot, integer bits), in 128-byte slots, [n_iso][2^guide_log2];
    // null when not built
    const double2 *binrec;
    int bin_prefetch;                // nuclides ahead whose bin record is prefetched into L2
    double mat_thresh[kMaterials];   // pick_mat running sums, Simulation.c:450-457
    unsigned long long mat_tseed[kMaterials];  // smallest LCG state whose draw reaches each sum
    int mat_lo[kMaterials];          // smallest / largest nuclide id of each material
    int mat_hi[kMaterials];          //   (span of the index-row prefetch)
    unsigned hot[16];                // nuclides (< 512) whose records stay in L2 (evict_last)
    int pair_base[kMaterials + 1];   // running sum of num_nucs: (material, position) pairs
    const int *inv_off;              // [n_iso + 1] pairs holding each nuclide (CSR)
    const int *inv_pair;             // [pairs] m * max_nucs + j, by nuclide, m ascending
    // union table (UNIONIZED, FAST): per material m, [n_union][num_nucs[m]]
    // entries of five (v, s) pairs: v = the nuclide's xs at the row's union
    // energy, s = the slope of its interval there; null when not built
    const double2 *utab[kMaterials];
};

// Per-run scratch in device memory (owned by the context).
struct Scratch {
    unsigned long long *verification = nullptr;  // 1 counter
    int *error = nullptr;                        // 1 flag + 3 detail words
    unsigned int *queue = nullptr;               // work-queue counter
    void *sort_buf = nullptr;                    // batched sort buffers
    size_t sort_bytes = 0;
    void *stage = nullptr;                       // staging for host outputs
    size_t stage_bytes = 0;
    void *plain_buf = nullptr;                   // plain-kernel overflow queues
    size_t plain_bytes = 0;
    void *adj_buf = nullptr;                     // adjoint sort, tables and partials
    size_t adj_bytes = 0;
    void *hist_buf = nullptr;                    // stepped history: particle states
    size_t hist_bytes = 0;
};

struct BatchedGraph {
    cudaGraphExec_t exec = nullptr;
    int launches = 0;
};

}  // namespace xsgb

struct xs_ctx {
    int device = 0;
    xs_inputs inputs{};
    std::string hm;
    xsgb::Tables t{};
    cudaStream_t stream = nullptr;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    std::vector<void *> allocations;
    size_t device_bytes = 0;
    xsgb::Scratch s;
    // tuned defaults
    int plain_tile = 1536;                    // unionized grid (2,048 on the others)
    int batched_buckets = 4096;
    int batched_blocks_per_sm = 4;            // in 256-thread blocks (threads per SM / 256)
    int plain_block = 256;                    // threads per block of the plain kernel
    int batched_block = 256;                  // threads per block of the persistent list kernel
    int fuel_lanes = 1;                       // plain kernel, FAST: lanes per fuel lookup
    int batched_fuel_lanes = 1;               // the same for the batched kernel
    // plain kernel: material rows in shared memory (1), through the
    // read-only cache (0), or by grid type (-1: staged on the unionized grid,
    // +0.7 % there; 0.4 % slower on the hash grid, even on the nuclide grid)
    int stage_rows = -1;
    // plain kernel: tile lookups ordered by energy within each material (1),
    // by material only (0), or by grid type (-1: on the hash and nuclide grids)
    int tile_sort = -1;
    // plain kernel over the event batch: the tiles' partial 32-lookup chunks
    // run in a second, packed pass (1), padded in their tiles (0), or by grid
    // type (-1: the pass runs except on the nuclide grid without the guided
    // searches)
    int overflow = -1;
    int num_nucs_host[xsgb::kMaterials] = {}; // host copy of num_nucs
    size_t union_table_bytes = 0;             // 0: no union table
    std::map<std::string, xsgb::BatchedGraph> graphs;
    int sm_count = 0;
    void *h_result = nullptr;                 // pinned: verification + error words
    cudaStream_t last_stream = nullptr;       // stream of the last (async) run
    int last_launches = 0;
    // host-sample pipeline: `pipe_slots` streams with a buffer set each, and
    // the plain kernel's overflow passes on one more, high-priority stream
    static constexpr int kPipeSlots = 8;
    cudaStream_t pipe_stream[kPipeSlots] = {};
    cudaEvent_t pipe_event[kPipeSlots] = {};
    cudaStream_t ovf_stream = nullptr;
    cudaEvent_t ovf_ready[kPipeSlots] = {};
    cudaEvent_t ovf_done[kPipeSlots] = {};
    cudaEvent_t fork_event = nullptr;         // stepped history: the groups' start
    int pipe_slots = 4;                       // buffer sets (and streams) in use
    int hist_groups = 8;                      // stepped history: particle groups (streams)
    long pipe_chunk = 0;                      // lookups per whole chunk (0: by kernel)
    void *pipe_buf = nullptr;
    size_t pipe_bytes = 0;
    // grids the autotuner may switch to (owned through `allocations`)
    const int *own_index = nullptr;           // the index grid the problem came with
    const long long *base_coarse = nullptr;   // coarse keys built with the context
    int base_n_coarse = 0;
    int *tune_hash_index = nullptr;           // derived 10,000-bin hash grid
    long long *tune_coarse = nullptr;         // derived coarse keys (nuclide grid)
    int tune_n_coarse = 0;
    // the guided searches' tables (owned through `allocations`); the tuner
    // may switch them off for a grid view
    const int *own_guide = nullptr;
    const double2 *own_binrec = nullptr;
    int base_guided = 0;                      // built with the context
};

namespace xsgb {

// error helpers (capi.cu)
xs_status fail(xs_status s, const char *fmt, ...);
xs_status cuda_fail(cudaError_t e, const char *what);
#define XS_CUDA(call)                                            \
    do {                                                         \
        cudaError_t e__ = (call);                                \
        if (e__ != cudaSuccess) return ::xsgb::cuda_fail(e__, #call); \
    } while (0)

// device memory owned by a context
xs_status ctx_alloc(xs_ctx *ctx, void **p, size_t bytes);

// derived-table builders (tables.cu)
xs_status build_derived_tables(xs_ctx *ctx);
// the union table, when the grid is unionized and device memory allows
xs_status build_union_table(xs_ctx *ctx);
// the energy-bin guide of the hash / nuclide searches (part of build_derived_tables)
xs_status build_guide(xs_ctx *ctx);
// hash grid of `bins` bins (GridInit.c:128-151) and the nuclide grid's coarse
// keys (every kCoarseStride-th order key), built on the device
cudaError_t launch_hash_grid(const xs_gridpoint *grid, long n_iso, long n_gp, int bins, int *index,
                             int sm_count, cudaStream_t st);
cudaError_t launch_coarse_keys(const long long *ekeys, long n_iso, long n_gp, int n_coarse,
                               long long *coarse, int sm_count, cudaStream_t st);

// lookup launchers (lookup.cu).  Every launcher only enqueues on `st`.
struct Outputs {
    double *macro = nullptr;          // device, count*5, or null
    unsigned char *max_idx = nullptr; // device, count, or null
};
struct SampleInput {
    const double *energy = nullptr;   // device, or null: in-kernel LCG sampling
    const int *mat = nullptr;
};
// Overflow queues of the plain kernel (see PlainArgs in lookup_kernels.cuh).
struct PlainScratch {
    int *cnt;            // [12] entries per material
    int *seg_v;          // [13] packed chunk starts
    int *base;           // [12] m * cap
    unsigned int *queue;
    double *E;           // [12 * cap]
    int *id;             // [12 * cap]
    int cap;
};
size_t plain_scratch_bytes(long count, int tile);
PlainScratch carve_plain_scratch(void *buf, long count, int tile);
// Where the overflow pass runs when it is not on the tiles' stream: `st` (a
// high-priority stream, so the pass's blocks are dispatched ahead of another
// stream's pending tiles), `ready` recorded after the tiles, `done` after the
// pass (the tiles' stream waits on it).
struct OverflowStream {
    cudaStream_t st;
    cudaEvent_t ready, done;
};
// ps == null: each block runs the partial chunks of its tile with idle lanes.
// block: threads per block (128, 256 or 512; 0 = the context's, halved while
// above the tile).  os == null: the overflow pass follows the tiles on `st`.
xs_status launch_plain(xs_ctx *ctx, cudaStream_t st, int arith, int checked, long first,
                       long count, int tile, int block, const SampleInput &in,
                       const Outputs &out, const PlainScratch *ps, int *launches,
                       const OverflowStream *os = nullptr);
xs_status launch_batched(xs_ctx *ctx, cudaStream_t st, int arith, int checked, long first,
                         long count, int block, int buckets, const SampleInput &in,
                         const Outputs &out, int *launches);
xs_status launch_history(xs_ctx *ctx, cudaStream_t st, int arith, long first, long count,
                         int *launches);
// History mode advanced in lockstep: one event batch per lookup step.
xs_status launch_history_stepped(xs_ctx *ctx, cudaStream_t st, int arith, long first, long count,
                                 int tile, int *launches);
size_t batched_scratch_bytes(long count, int buckets);
// Sorts each bucket [starts[b], ends[b]) of (sE, sid) by (energy order key,
// id) in place (adjoint order, device setup); one block per bucket.
cudaError_t launch_bucket_sort(const int *starts, const int *ends, int nbuckets, double *sE,
                               int *sid, int blocks, cudaStream_t st);
// Explicit device buffers of one batched run (every pointer into caller memory).
struct BatchedScratch {
    unsigned long long *verification;
    int *error;
    unsigned int *queue;
    int *offs;   // [12 << nb_log2]
    int *seg;    // [13]
    int *cnt;    // [12]
    double *sE;  // [count + 384]
    int *sid;    // [count + 384]
};
xs_status enqueue_batched_in(xs_ctx *ctx, cudaStream_t st, int arith, long first, long count,
                             int nb_log2, const BatchedScratch &b, const Outputs &out);
// Buffers of one batched run carved from `buf` (batched_scratch_bytes(count,
// 1 << nb_log2) bytes); verification and error are left null for the caller.
BatchedScratch carve_batched_scratch(void *buf, long count, int nb_log2);
xs_status enqueue_batched_buf(xs_ctx *ctx, cudaStream_t st, int arith, int checked, long first,
                              long count, int nb_log2, int block, const SampleInput &in,
                              const Outputs &out, const BatchedScratch &b, int *launches);
// Blocks of the persistent list kernel for `block` threads each (0: the
// context's): batched_blocks_per_sm x 256 threads per SM.
int list_blocks(const xs_ctx *ctx, int block);
xs_status launch_sample(xs_ctx *ctx, cudaStream_t st, long first, long count, double *E, int *mat);

struct ListArgs;
xs_status enqueue_sort_only(xs_ctx *ctx, cudaStream_t st, long first, long count, int nb_log2,
                            const SampleInput &in, int *offs, int *starts, int *seg, int *cnt,
                            double *sE, int *sid);
xs_status launch_adjoint_energy(xs_ctx *ctx, cudaStream_t st, const ListArgs &l,
                                const double *gbar, double *sg, double *d_energy);
// adjoint.cu: the whole adjoint on `st` (all pointers device memory)
xs_status launch_adjoint(xs_ctx *ctx, cudaStream_t st, long first, long count,
                         const SampleInput &in, const double *gbar, double *macro_out,
                         double *d_concs, double *d_xs, double *d_energy, int *launches);

// host setup (setup_host.cu)
void pick_mat_thresholds(double out[kMaterials]);
// the 12 materials of Materials.c:7-117 (host arrays, freed by xs_simdata_free)
xs_status load_materials(long n_iso, xs_simdata *sd);

// context assembly (capi.cu)
xs_status ctx_open(const xs_inputs *in, int device, xs_ctx **out);
xs_status install_materials(xs_ctx *ctx, const xs_inputs *in, const xs_simdata *sd);

}  // namespace xsgb
