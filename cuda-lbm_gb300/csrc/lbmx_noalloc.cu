// lbmx_noalloc.cu -- lbmx_moment_sums_noalloc: the FP64 mass / momentum
// reduction of the step kernel as a stand-alone entry point that allocates
// no device memory.
//
// Who needs it: callers that may not call cudaMalloc at the point where they
// want the sums -- a host loop that must not stall the device between
// steps (cudaMalloc and cudaFree synchronise), a framework whose device
// memory all belongs to its own pool, or a process under a hard memory cap
// that has already reserved what it may use.  They pass their own density and
// velocity fields and an output location; the per-block partial sums live in
// the fixed array below instead of a buffer this library would allocate.
//
// The scratch is one file-scope __device__ array, so every GPU that loads the
// library holds its 24,608 bytes until the process exits, and every call on a
// device shares it: calls whose kernels overlap on the GPU (different
// streams, no ordering between them) race on it and must not be issued.  A
// call leaves its partials and result in the array; the completion counter,
// the only part that must start at zero, is cleared by each call before its
// kernel runs.
#include <cuda_runtime.h>

#include <cstdio>
#include <mutex>

#include "lbmx.h"

namespace {

constexpr int kNaThreads = 256;
constexpr int kNaMaxBlocks = 1024;  // grid of the reduction = partials capacity

// [0, 3 * kNaMaxBlocks): per-block partial sums; then 3 result slots; then
// the completion counter (as the bit pattern of a double slot)
constexpr int kNaSlots = 3 * kNaMaxBlocks + 3 + 1;
static __device__ __align__(256) double g_noalloc_scratch[kNaSlots];

struct NaScratch {
    double* partials;
    double* result;
    unsigned int* counter;
};

__global__ void __launch_bounds__(kNaThreads) moment_sums_kernel(const float* __restrict__ rho,
                                                                 const float* __restrict__ u, long long n,
                                                                 NaScratch s) {
    double v0 = 0.0, v1 = 0.0, v2 = 0.0;
    for (long long i = (long long)blockIdx.x * kNaThreads + threadIdx.x; i < n; i += (long long)gridDim.x * kNaThreads) {
        const double r = rho[i];
        v0 += r;
        v1 += r * (double)u[i];
        v2 += r * (double)u[n + i];
    }
    __shared__ double sh[kNaThreads / 32][3];
    __shared__ bool last;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int o = 16; o > 0; o >>= 1) {
        v0 += __shfl_down_sync(0xffffffffu, v0, o);
        v1 += __shfl_down_sync(0xffffffffu, v1, o);
        v2 += __shfl_down_sync(0xffffffffu, v2, o);
    }
    if (lane == 0) {
        sh[warp][0] = v0;
        sh[warp][1] = v1;
        sh[warp][2] = v2;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double t0 = 0.0, t1 = 0.0, t2 = 0.0;
        for (int w = 0; w < kNaThreads / 32; w++) {
            t0 += sh[w][0];
            t1 += sh[w][1];
            t2 += sh[w][2];
        }
        s.partials[3 * blockIdx.x + 0] = t0;
        s.partials[3 * blockIdx.x + 1] = t1;
        s.partials[3 * blockIdx.x + 2] = t2;
        __threadfence();
        last = atomicAdd(s.counter, 1u) == gridDim.x - 1;
    }
    __syncthreads();
    if (!last || threadIdx.x != 0) return;
    // the last block adds the partials in block order: deterministic
    __threadfence();
    double t0 = 0.0, t1 = 0.0, t2 = 0.0;
    for (unsigned b = 0; b < gridDim.x; b++) {
        t0 += __ldcg(s.partials + 3 * b + 0);
        t1 += __ldcg(s.partials + 3 * b + 1);
        t2 += __ldcg(s.partials + 3 * b + 2);
    }
    s.result[0] = t0;
    s.result[1] = t1;
    s.result[2] = t2;
    *s.counter = 0u;
}

// Device address of the scratch array, looked up once per device.  A host
// pointer to g_noalloc_scratch is only a stand-in for the symbol; kernels must
// be given the address cudaGetSymbolAddress returns for the current device.
// The cached address belongs to the device's primary context (the one the
// runtime API uses) and stays valid until that context is destroyed: a
// process that calls cudaDeviceReset, or that makes another driver context
// current on the device, must not call this entry point afterwards.
constexpr int kNaMaxDevices = 64;
std::mutex g_na_mutex;
double* g_na_addr[kNaMaxDevices] = {};

cudaError_t scratch_for_device(int dev, double** out) {
    std::lock_guard<std::mutex> lock(g_na_mutex);
    if (!g_na_addr[dev]) {
        void* p = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess) return e;
        g_na_addr[dev] = static_cast<double*>(p);
    }
    *out = g_na_addr[dev];
    return cudaSuccess;
}

// No handle carries a message for this entry point: the status code says
// what failed; the text goes to stderr for the operator.
lbmx_status na_fail(lbmx_status code, const char* msg, cudaError_t e) {
    fprintf(stderr, "%s%s%s\n", msg, e != cudaSuccess ? ": " : "", e != cudaSuccess ? cudaGetErrorString(e) : "");
    return code;
}

}  // namespace

extern "C" {

lbmx_status lbmx_moment_sums_noalloc(const float* rho, const float* u, int64_t n, double* sums3, void* stream) {
    if (!rho || !u || !sums3) return na_fail(LBMX_ERR_INVALID_ARGUMENT, "lbmx_moment_sums_noalloc: NULL argument", cudaSuccess);
    if (n <= 0) return na_fail(LBMX_ERR_INVALID_ARGUMENT, "lbmx_moment_sums_noalloc: n must be positive", cudaSuccess);
    if (n > LBMX_NOALLOC_MAX_NODES)
        return na_fail(LBMX_ERR_TOO_LARGE,
                       "lbmx_moment_sums_noalloc: n exceeds LBMX_NOALLOC_MAX_NODES (2^31 - 1 nodes)", cudaSuccess);
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return na_fail(LBMX_ERR_CUDA, "lbmx_moment_sums_noalloc: cudaGetDevice", e);
    if (dev < 0 || dev >= kNaMaxDevices)
        return na_fail(LBMX_ERR_UNSUPPORTED, "lbmx_moment_sums_noalloc: device ordinal above 63", cudaSuccess);
    double* base = nullptr;
    e = scratch_for_device(dev, &base);
    if (e != cudaSuccess) return na_fail(LBMX_ERR_CUDA, "lbmx_moment_sums_noalloc: cudaGetSymbolAddress", e);
    NaScratch s;
    s.partials = base;
    s.result = base + 3 * kNaMaxBlocks;
    s.counter = reinterpret_cast<unsigned int*>(base + 3 * kNaMaxBlocks + 3);
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    e = cudaMemsetAsync(s.counter, 0, sizeof(unsigned int), st);
    if (e != cudaSuccess) return na_fail(LBMX_ERR_CUDA, "lbmx_moment_sums_noalloc: clearing the counter", e);
    long long blocks = (n + kNaThreads - 1) / kNaThreads;
    if (blocks > kNaMaxBlocks) blocks = kNaMaxBlocks;
    moment_sums_kernel<<<(unsigned)blocks, kNaThreads, 0, st>>>(rho, u, (long long)n, s);
    e = cudaGetLastError();
    if (e != cudaSuccess) return na_fail(LBMX_ERR_CUDA, "lbmx_moment_sums_noalloc: launch", e);
    e = cudaMemcpyAsync(sums3, s.result, 3 * sizeof(double), cudaMemcpyDefault, st);
    if (e != cudaSuccess) return na_fail(LBMX_ERR_CUDA, "lbmx_moment_sums_noalloc: copying the result", e);
    // Only pageable host memory makes the call wait: its caller reads the
    // sums as soon as the call returns.  Device, managed and page-locked
    // host memory receive them in stream order, so the host is not blocked.
    cudaPointerAttributes pa;
    e = cudaPointerGetAttributes(&pa, sums3);
    if (e != cudaSuccess) return na_fail(LBMX_ERR_CUDA, "lbmx_moment_sums_noalloc: classifying sums3", e);
    if (pa.type == cudaMemoryTypeUnregistered) {
        e = cudaStreamSynchronize(st);
        if (e != cudaSuccess) return na_fail(LBMX_ERR_CUDA, "lbmx_moment_sums_noalloc: synchronize", e);
    }
    return LBMX_OK;
}

}  // extern "C"
