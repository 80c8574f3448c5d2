// lbmx_ibm.cu -- the engine's marker rounds: one CTA runs ibm_rounds<float>
// (lbmx_ibm.cuh) on the marker patch before each step.
#include "lbmx.h"
#include "lbmx_ibm.cuh"

namespace lbmx {

__global__ void __launch_bounds__(kIbmThreads) ibm_iterate_kernel(const IbmArgs a) {
    extern __shared__ float sm[];
    ibm_rounds<float>(a, sm);
}

size_t ibm_smem_bytes(int npatch, int nm) { return ibm_smem_bytes_of<float>(npatch, nm); }

cudaError_t launch_ibm_iterate(const IbmArgs& a, cudaStream_t s) {
    const size_t smem = ibm_smem_bytes(a.npatch, a.nm);
    cudaError_t e = cudaFuncSetAttribute(ibm_iterate_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    ibm_iterate_kernel<<<1, kIbmThreads, smem, s>>>(a);
    return cudaGetLastError();
}

}  // namespace lbmx
