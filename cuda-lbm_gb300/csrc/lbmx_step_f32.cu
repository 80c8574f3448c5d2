// FP32 population storage instantiation of the step kernels.
#include "lbmx_kernels.cuh"
namespace lbmx {
LBMX_INSTANTIATE(float)

// the publication of a kModeSums step's sums when no later launch does it
__global__ void publish_kernel(double* acc, double* sums, double* series) { publish_sums(acc, sums, series, (int)threadIdx.x); }

cudaError_t launch_publish(double* acc, double* sums, double* series, cudaStream_t s) {
    publish_kernel<<<1, 32, 0, s>>>(acc, sums, series);
    return cudaGetLastError();
}
}
