// lbmx_ibm.cu -- multi-direct immersed-boundary forcing on the marker patch.
//
// The reference runs ITER_MAX = 3 rounds of {interpolate, Lagrangian force,
// spread, correct, accumulate}, each round a handful of full-grid kernels
// (IBMManager<2>::multi_direct, src/IBM/IBMManager.cuh:222-252).  Only the
// nodes inside some marker's stencil ever change, so this engine keeps those
// nodes (the "patch") in shared memory of one CTA and runs all rounds there:
// the grid-sized passes disappear, and the step kernel adds the resulting
// force through a dense field that is zero away from the markers.
#include "lbmx.h"
#include "lbmx_internal.h"

namespace lbmx {

constexpr int kIbmThreads = 1024;

__global__ void __launch_bounds__(kIbmThreads) ibm_iterate_kernel(const IbmArgs a) {
    extern __shared__ float sm[];
    const int np = a.npatch, nm = a.nm, S2 = a.stencil * a.stencil;
    float* upx = sm;            // working velocity (u_prev of the reference)
    float* upy = upx + np;
    float* rho = upy + np;
    float* fix = rho + np;      // this round's spread force
    float* fiy = fix + np;
    float* ftx = fiy + np;      // force summed over rounds
    float* fty = ftx + np;
    float* mfx = fty + np;      // marker force of this round
    float* mfy = mfx + nm;
    float* mtx = mfy + nm;      // marker force summed over rounds
    float* mty = mtx + nm;
    const int tid = threadIdx.x;
    for (int i = tid; i < np; i += blockDim.x) {
        upx[i] = a.patch_u[i];
        upy[i] = a.patch_u[np + i];
        rho[i] = a.patch_rho[i];
        ftx[i] = 0.f;
        fty[i] = 0.f;
    }
    for (int k = tid; k < nm; k += blockDim.x) mtx[k] = mty[k] = 0.f;
    __syncthreads();
    for (int it = 0; it < a.iters; it++) {
        for (int i = tid; i < np; i += blockDim.x) fix[i] = fiy[i] = 0.f;
        // interpolate_velocities_kernel<2> (IBM_impl.cu:5-51) then
        // compute_lagrangian_kernel (IBM_impl.cuh:7-26), target velocity 0
        for (int k = tid; k < nm; k += blockDim.x) {
            float r = 0.f, ux = 0.f, uy = 0.f;
            for (int s = 0; s < S2; s++) {
                const int idx = a.sten_idx[k * S2 + s];
                if (idx < 0) continue;
                const float w = a.sten_w[k * S2 + s];
                r += w * rho[idx];
                ux += w * upx[idx];
                uy += w * upy[idx];
            }
            float fx = 2.0f * r * (0.0f - ux);
            float fy = 2.0f * r * (0.0f - uy);
            if (a.clamp) {
                fx = fx > 1e-8f ? fx : 0.0f;
                fy = fy > 1e-8f ? fy : 0.0f;
            }
            mfx[k] = fx;
            mfy[k] = fy;
            mtx[k] += fx;
            mty[k] += fy;
            if (it == a.iters - 1) {
                a.marker_u[k] = ux;
                a.marker_u[nm + k] = uy;
                a.marker_rho[k] = r;
            }
        }
        __syncthreads();
        // spread_forces_kernel<2> (IBM_impl.cu:120-154)
        for (int j = tid; j < nm * S2; j += blockDim.x) {
            const int k = j / S2;
            const int idx = a.sten_idx[j];
            if (idx < 0) continue;
            const float w = a.sten_w[j] * a.ds;
            atomicAdd(&fix[idx], w * mfx[k]);
            atomicAdd(&fiy[idx], w * mfy[k]);
        }
        __syncthreads();
        // correct_velocities_kernel + accumulate_forces_kernel (IBM_impl.cuh:28-68)
        for (int i = tid; i < np; i += blockDim.x) {
            float cx = upx[i] + fix[i] / (2.0f * rho[i]);
            float cy = upy[i] + fiy[i] / (2.0f * rho[i]);
            if (a.clamp) {
                cx = cx > 1e-8f ? cx : 0.0f;
                cy = cy > 1e-8f ? cy : 0.0f;
            }
            upx[i] = cx;
            upy[i] = cy;
            ftx[i] += fix[i];
            fty[i] += fiy[i];
        }
        __syncthreads();
    }
    for (int i = tid; i < np; i += blockDim.x) {
        const long long off = a.patch_nodes[i];
        a.ibm_force[off] = ftx[i];
        a.ibm_force[a.plane + off] = fty[i];
    }
    for (int k = tid; k < nm; k += blockDim.x) {
        a.marker_force[k] = mtx[k];
        a.marker_force[nm + k] = mty[k];
    }
}

size_t ibm_smem_bytes(int npatch, int nm) { return (size_t)(7 * npatch + 4 * nm) * sizeof(float); }

cudaError_t launch_ibm_iterate(const IbmArgs& a, cudaStream_t s) {
    const size_t smem = ibm_smem_bytes(a.npatch, a.nm);
    cudaError_t e = cudaFuncSetAttribute(ibm_iterate_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    ibm_iterate_kernel<<<1, kIbmThreads, smem, s>>>(a);
    return cudaGetLastError();
}

}  // namespace lbmx
