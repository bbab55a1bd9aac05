// static_scratch.cu -- the batched lookup with its scratch in a static
// device array, for callers that must not allocate device memory.
//
// Who needs it: a host thread that drives other work on the GPU and must not
// stall it -- cudaMalloc and cudaFree can synchronise the whole device -- or a
// host program whose memory manager owns the device's memory budget and
// forbids allocations behind its back.  xs_run_event with the batched kernel
// allocates its sort buffers on first use and when the batch grows; this entry
// point allocates nothing: its sort buffers, counters and queue live in
// g_static_scratch below.
//
// The array is a file-scope __device__ variable, so every GPU that loads the
// library holds it (6.5 MB) until the process exits.  Its name is only a
// host-side stand-in in host code; the device address comes from
// cudaGetSymbolAddress, looked up with the device current on the first call
// on each device, and again on the first call after that device's CUDA
// context was re-created (a cudaDeviceReset elsewhere in the process), when
// the array may sit at another address.
#include <cuda.h>

#include <cstring>
#include <mutex>

#include "xsgb_internal.h"

namespace xsgb {

constexpr long kStaticMaxLookups = 1L << 19;  // 524,288 lookups per call
constexpr int kStaticMaxBuckets = 4096;       // energy buckets per material
constexpr size_t kStaticCounters = 256;       // verification, error[4], queue
constexpr size_t kStaticOffs = (size_t)kMaterials * kStaticMaxBuckets * 4;
constexpr size_t kStaticSeg = 256;            // seg[13] and cnt[12]
constexpr size_t kStaticPadded = (size_t)kStaticMaxLookups + kMaterials * 32;
constexpr size_t kStaticBytes =
    kStaticCounters + kStaticOffs + kStaticSeg + kStaticPadded * 8 + kStaticPadded * 4;

static __device__ __align__(256) unsigned char g_static_scratch[kStaticBytes];

static std::mutex g_static_mu;
// per device ordinal: the array's device address and the id of the CUDA
// context it was looked up in
struct StaticAddr {
    unsigned long long ctx_id;
    void *addr;
};
static StaticAddr g_static_addr[64];

typedef CUresult (*PFN_ctx_current)(CUcontext *);
typedef CUresult (*PFN_ctx_id)(CUcontext, unsigned long long *);

// Unique id of the calling thread's current CUDA context (ids are never
// reused within a process, unlike context handles); 0 when unavailable.
static unsigned long long current_context_id()
{
    static PFN_ctx_current get_current = nullptr;
    static PFN_ctx_id get_id = nullptr;
    static std::once_flag once;
    std::call_once(once, [] {
        void *f = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f, 12000, cudaEnableDefault, &q) ==
                cudaSuccess && q == cudaDriverEntryPointSuccess)
            get_current = (PFN_ctx_current)f;
        f = nullptr;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &f, 12000, cudaEnableDefault, &q) ==
                cudaSuccess && q == cudaDriverEntryPointSuccess)
            get_id = (PFN_ctx_id)f;
        cudaGetLastError();
    });
    CUcontext c = nullptr;
    unsigned long long id = 0;
    if (!get_current || !get_id || get_current(&c) != CUDA_SUCCESS || !c || get_id(c, &id) != CUDA_SUCCESS)
        return 0;
    return id;
}

// Device address of g_static_scratch on `device`, which must be current.
static xs_status static_scratch_address(int device, unsigned char **out)
{
    if (device < 0 || device >= 64) return fail(XS_ERR_NO_DEVICE, "device ordinal %d", device);
    const unsigned long long id = current_context_id();
    std::lock_guard<std::mutex> lock(g_static_mu);
    StaticAddr &e = g_static_addr[device];
    if (!e.addr || id == 0 || e.ctx_id != id) {
        void *p = nullptr;
        cudaError_t err = cudaGetSymbolAddress(&p, g_static_scratch);
        if (err != cudaSuccess) return cuda_fail(err, "cudaGetSymbolAddress(g_static_scratch)");
        e.addr = p;
        e.ctx_id = id;
    }
    *out = (unsigned char *)e.addr;
    return XS_OK;
}

// NULL, or memory the kernels on `device` can write: device memory of that
// device, or managed memory.
static bool device_or_null(const void *p, int device)
{
    if (!p) return true;
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    if (a.type == cudaMemoryTypeManaged) return true;
    return a.type == cudaMemoryTypeDevice && a.device == device;
}

// Makes `device` current for the scope and puts the caller's device back.
struct DeviceScope {
    int saved = -1;
    cudaError_t set(int device)
    {
        cudaError_t e = cudaGetDevice(&saved);
        if (e != cudaSuccess) {
            saved = -1;
            return e;
        }
        return saved == device ? cudaSuccess : cudaSetDevice(device);
    }
    ~DeviceScope()
    {
        int now = -1;
        if (saved >= 0 && cudaGetDevice(&now) == cudaSuccess && now != saved) cudaSetDevice(saved);
    }
};

}  // namespace xsgb

using namespace xsgb;

extern "C" xs_status xs_run_event_batched_static(xs_ctx *ctx, long first, long count, int arith,
                                                 int energy_buckets, double *macro_xs_out,
                                                 unsigned char *max_idx_out, void *stream,
                                                 unsigned long long *verification)
{
    if (!ctx || !verification) return fail(XS_ERR_INVALID_ARGUMENT, "xs_run_event_batched_static: NULL context or verification");
    if (first < 0 || count <= 0)
        return fail(XS_ERR_INVALID_ARGUMENT, "xs_run_event_batched_static: need first >= 0 and count > 0");
    if (count > kStaticMaxLookups)
        return fail(XS_ERR_INVALID_ARGUMENT,
                    "xs_run_event_batched_static: %ld lookups exceed the static scratch (at most %ld per call)",
                    count, kStaticMaxLookups);
    // default: the context's batched bucket count (tuned), within the array's limit
    if (energy_buckets <= 0)
        energy_buckets = ctx->batched_buckets < kStaticMaxBuckets ? ctx->batched_buckets : kStaticMaxBuckets;
    if (energy_buckets > kStaticMaxBuckets || (energy_buckets & (energy_buckets - 1)))
        return fail(XS_ERR_INVALID_ARGUMENT,
                    "xs_run_event_batched_static: energy_buckets %d must be a power of two <= %d",
                    energy_buckets, kStaticMaxBuckets);
    if (arith != XS_ARITH_FAST && arith != XS_ARITH_EXACT)
        return fail(XS_ERR_INVALID_ARGUMENT, "xs_run_event_batched_static: unknown arithmetic %d", arith);
    DeviceScope scope;   // the caller's current device is restored on return
    XS_CUDA(scope.set(ctx->device));
    if (!device_or_null(macro_xs_out, ctx->device) || !device_or_null(max_idx_out, ctx->device))
        return fail(XS_ERR_INVALID_ARGUMENT,
                    "xs_run_event_batched_static: outputs must be NULL or device memory of the context's device %d",
                    ctx->device);
    unsigned char *base = nullptr;
    xs_status s = static_scratch_address(ctx->device, &base);
    if (s != XS_OK) return s;
    int nb_log2 = 0;
    while ((1 << nb_log2) < energy_buckets) nb_log2++;

    BatchedScratch b;
    b.verification = (unsigned long long *)base;
    b.error = (int *)(base + 64);
    b.queue = (unsigned int *)(base + 128);
    b.offs = (int *)(base + kStaticCounters);
    b.seg = (int *)(base + kStaticCounters + kStaticOffs);
    b.cnt = b.seg + 16;
    b.sE = (double *)(base + kStaticCounters + kStaticOffs + kStaticSeg);
    b.sid = (int *)(base + kStaticCounters + kStaticOffs + kStaticSeg + kStaticPadded * 8);
    Outputs out;
    out.macro = macro_xs_out;
    out.max_idx = max_idx_out;

    cudaStream_t st = stream ? (cudaStream_t)stream : ctx->stream;
    // the array keeps the previous call's contents: clear the counters and
    // the histogram (the sort buffers are fully rewritten by the scatter)
    XS_CUDA(cudaMemsetAsync(base, 0, kStaticCounters, st));
    XS_CUDA(cudaMemsetAsync(b.offs, 0, (size_t)kMaterials * energy_buckets * 4, st));
    s = enqueue_batched_in(ctx, st, arith, first, count, nb_log2, b, out);
    if (s != XS_OK) return s;
    unsigned long long v = 0;
    int err[4] = {0, 0, 0, 0};
    XS_CUDA(cudaMemcpyAsync(&v, b.verification, sizeof v, cudaMemcpyDeviceToHost, st));
    XS_CUDA(cudaMemcpyAsync(err, b.error, sizeof err, cudaMemcpyDeviceToHost, st));
    XS_CUDA(cudaStreamSynchronize(st));
    if (err[0]) return fail((xs_status)err[0], "device check failed: entry %d, value %d", err[1], err[2]);
    *verification = v;
    return XS_OK;
}
