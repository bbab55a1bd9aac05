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
// cudaGetSymbolAddress, looked up once per device on that device's first call.
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
static void *g_static_addr[64];  // device address per device ordinal

static xs_status static_scratch_address(int device, unsigned char **out)
{
    if (device < 0 || device >= 64) return fail(XS_ERR_NO_DEVICE, "device ordinal %d", device);
    std::lock_guard<std::mutex> lock(g_static_mu);
    if (!g_static_addr[device]) {
        void *p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_static_scratch);
        if (e != cudaSuccess) return cuda_fail(e, "cudaGetSymbolAddress(g_static_scratch)");
        g_static_addr[device] = p;
    }
    *out = (unsigned char *)g_static_addr[device];
    return XS_OK;
}

static bool device_or_null(const void *p)
{
    if (!p) return true;
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged;
}

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
    if (energy_buckets <= 0) energy_buckets = 1024;
    if (energy_buckets > kStaticMaxBuckets || (energy_buckets & (energy_buckets - 1)))
        return fail(XS_ERR_INVALID_ARGUMENT,
                    "xs_run_event_batched_static: energy_buckets %d must be a power of two <= %d",
                    energy_buckets, kStaticMaxBuckets);
    if (arith != XS_ARITH_FAST && arith != XS_ARITH_EXACT)
        return fail(XS_ERR_INVALID_ARGUMENT, "xs_run_event_batched_static: unknown arithmetic %d", arith);
    XS_CUDA(cudaSetDevice(ctx->device));
    if (!device_or_null(macro_xs_out) || !device_or_null(max_idx_out))
        return fail(XS_ERR_INVALID_ARGUMENT, "xs_run_event_batched_static: outputs must be device memory or NULL");
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
