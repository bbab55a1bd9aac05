// gather_ceiling.cu -- the DRAM rate a gather of whole 128-byte lines reaches
// on this GPU, for the roofline of the lookup kernels that read one interval
// record (or bin record) per nuclide.
//
// Each warp reads 32 random 128-byte-aligned lines, one per lane (four 32-byte
// loads each), all inside one window of 2^W bytes chosen at random per iteration:
// the pattern of a warp of energy-sorted lookups reading one nuclide's
// records, whose addresses spread over a window set by the warp's energy
// range.  Windows from 64 KB to the whole buffer, then a streaming read of the
// buffer for comparison.  Prints one JSON line.
//
//   xsbench_gb300/_lib/xsgb_gather_ceiling [buffer_log2 = 33]
#include <cstdio>
#include <cstdlib>

#include <cuda_runtime.h>

namespace {

__device__ __forceinline__ unsigned long long mix64(unsigned long long x)
{
    // MurmurHash3's 64-bit finaliser (public domain), as a cheap scrambler
    x ^= x >> 33;
    x *= 0xff51afd7ed558ccdULL;
    x ^= x >> 33;
    x *= 0xc4ceb9fe1a85ec53ULL;
    x ^= x >> 33;
    return x;
}

__device__ __forceinline__ unsigned long long ld32_xor(const char *p)
{
    unsigned long long a, b, c, d;
    asm volatile("ld.global.nc.L1::no_allocate.v4.u64 {%0,%1,%2,%3}, [%4];"
                 : "=l"(a), "=l"(b), "=l"(c), "=l"(d)
                 : "l"(p));
    return a ^ b ^ c ^ d;
}

// buffer of 2^buf_log2 bytes; every address stays below it: the window base
// is (w << win_log2) with w < 2^(buf_log2 - win_log2), the line offset
// (l << 7) + 96 + 32 with l < 2^(win_log2 - 7)
__global__ void k_window_gather(const char *buf, int buf_log2, int win_log2, int iters,
                                unsigned long long *out)
{
    const unsigned long long tid = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x;
    const unsigned long long warp = tid >> 5;
    const unsigned lane = threadIdx.x & 31;
    const unsigned long long win_mask = (1ULL << (buf_log2 - win_log2)) - 1;
    const unsigned long long line_mask = (1ULL << (win_log2 - 7)) - 1;
    unsigned long long acc = 0;
    for (int r = 0; r < iters; r++) {
        const unsigned long long w = mix64(warp * 0x9E3779B97F4A7C15ULL + (unsigned)r) & win_mask;
        const unsigned long long l =
            mix64((warp << 20) ^ ((unsigned long long)r << 5) ^ lane ^ 0x5555ULL) & line_mask;
        const char *p = buf + (w << win_log2) + (l << 7);
        acc ^= ld32_xor(p) ^ ld32_xor(p + 32) ^ ld32_xor(p + 64) ^ ld32_xor(p + 96);
    }
    out[tid] = acc;
}

__global__ void k_stream_read(const ulonglong2 *buf, size_t n, unsigned long long *out)
{
    unsigned long long acc = 0;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n;
         i += (size_t)gridDim.x * blockDim.x) {
        const ulonglong2 v = __ldg(buf + i);
        acc ^= v.x ^ v.y;
    }
    out[blockIdx.x * (size_t)blockDim.x + threadIdx.x] = acc;
}

int fail(const char *what, cudaError_t e)
{
    printf("{\"error\": \"%s: %s\"}\n", what, cudaGetErrorString(e));
    return 1;
}

}  // namespace

int main(int argc, char **argv)
{
    const int buf_log2 = argc > 1 ? atoi(argv[1]) : 33;
    if (buf_log2 < 28 || buf_log2 > 37) {
        printf("{\"error\": \"buffer_log2 must be in [28, 37]\"}\n");
        return 2;
    }
    const size_t bytes = (size_t)1 << buf_log2;
    char *buf = nullptr;
    unsigned long long *out = nullptr;
    cudaError_t e = cudaMalloc(&buf, bytes);
    if (e != cudaSuccess) return fail("buffer", e);
    e = cudaMemset(buf, 1, bytes);
    if (e != cudaSuccess) return fail("memset", e);
    int sms = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, 0);
    const int threads = 256, blocks = sms * 8, iters = 256, reps = 5;
    const size_t nthreads = (size_t)threads * blocks;
    e = cudaMalloc(&out, nthreads * 8);
    if (e != cudaSuccess) return fail("output", e);
    cudaEvent_t a, b;
    cudaEventCreate(&a);
    cudaEventCreate(&b);
    printf("{\"buffer_bytes\": %zu, \"line_bytes\": 128, \"windows\": [", bytes);
    const int wins[] = {16, 20, 24, 27, 30};
    bool first = true;
    for (int w : wins) {
        if (w > buf_log2) continue;
        k_window_gather<<<blocks, threads>>>(buf, buf_log2, w, iters, out);
        cudaEventRecord(a);
        for (int i = 0; i < reps; i++) k_window_gather<<<blocks, threads>>>(buf, buf_log2, w, iters, out);
        cudaEventRecord(b);
        cudaEventSynchronize(b);
        float ms = 0.f;
        cudaEventElapsedTime(&ms, a, b);
        printf("%s{\"window_bytes\": %llu, \"gbs\": %.1f}", first ? "" : ", ", 1ULL << w,
               (double)nthreads * iters * 128 * reps / (ms * 1e-3) / 1e9);
        first = false;
    }
    const size_t n = bytes / 16;
    k_stream_read<<<blocks, threads>>>((const ulonglong2 *)buf, n, out);
    cudaEventRecord(a);
    for (int i = 0; i < reps; i++) k_stream_read<<<blocks, threads>>>((const ulonglong2 *)buf, n, out);
    cudaEventRecord(b);
    cudaEventSynchronize(b);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, a, b);
    e = cudaGetLastError();
    printf("], \"stream_read_gbs\": %.1f, \"status\": \"%s\"}\n",
           (double)bytes * reps / (ms * 1e-3) / 1e9, cudaGetErrorString(e));
    cudaFree(out);
    cudaFree(buf);
    return e == cudaSuccess ? 0 : 1;
}
