// lbmx_ibm.cuh -- the multi-direct immersed-boundary rounds on the marker
// patch, as a template over the arithmetic type (float for the engine, a
// tangent number for the tangent-linear model).
//
// The reference runs ITER_MAX = 3 rounds of {interpolate, Lagrangian force,
// spread, correct, accumulate}, each round a handful of full-grid kernels
// (IBMManager<2>::multi_direct, src/IBM/IBMManager.cuh:222-252).  Only the
// nodes inside some marker's stencil ever change, so this engine keeps those
// nodes (the "patch") in shared memory of one CTA and runs all rounds there:
// the grid-sized passes disappear, and the step kernel adds the resulting
// force through a dense field that is zero away from the markers.
#pragma once
#include "lbmx_dual.cuh"

namespace lbmx {

constexpr int kIbmThreads = 1024;

__device__ __forceinline__ void ibm_atomic_add(float* p, float v) { atomicAdd(p, v); }
template <int K>
__device__ __forceinline__ void ibm_atomic_add(Dual<K>* p, const Dual<K>& v) {
    atomicAdd(&p->v, v.v);
#pragma unroll
    for (int k = 0; k < K; k++) atomicAdd(&p->d[k], v.d[k]);
}
// the reference's clamps (IBM_impl.cuh:22-24, 42-44)
__device__ __forceinline__ float ibm_clamp(float x) { return x > 1e-8f ? x : 0.0f; }
template <int K>
__device__ __forceinline__ Dual<K> ibm_clamp(const Dual<K>& x) { return x.v > 1e-8f ? x : dconst<K>(0.0f); }

template <typename R>
size_t ibm_smem_bytes_of(int npatch, int nm) { return (size_t)(7 * npatch + 4 * nm) * sizeof(R); }

// All rounds of one step in one CTA; sm holds ibm_smem_bytes_of<R> bytes.
template <typename R>
__device__ void ibm_rounds(const IbmData<R>& a, R* sm) {
    const int np = a.npatch, nm = a.nm, S2 = a.stencil * a.stencil;
    const R zero = splat(0.0f, R{});
    R* upx = sm;            // working velocity (u_prev of the reference)
    R* upy = upx + np;
    R* rho = upy + np;
    R* fix = rho + np;      // this round's spread force
    R* fiy = fix + np;
    R* ftx = fiy + np;      // force summed over rounds
    R* fty = ftx + np;
    R* mfx = fty + np;      // marker force of this round
    R* mfy = mfx + nm;
    R* mtx = mfy + nm;      // marker force summed over rounds
    R* mty = mtx + nm;
    const int tid = threadIdx.x;
    for (int i = tid; i < np; i += blockDim.x) {
        upx[i] = a.patch_u[i];
        upy[i] = a.patch_u[np + i];
        rho[i] = a.patch_rho[i];
        ftx[i] = zero;
        fty[i] = zero;
    }
    for (int k = tid; k < nm; k += blockDim.x) mtx[k] = mty[k] = zero;
    __syncthreads();
    for (int it = 0; it < a.iters; it++) {
        for (int i = tid; i < np; i += blockDim.x) fix[i] = fiy[i] = zero;
        // interpolate_velocities_kernel<2> (IBM_impl.cu:5-51) then
        // compute_lagrangian_kernel (IBM_impl.cuh:7-26), target velocity 0
        for (int k = tid; k < nm; k += blockDim.x) {
            R r = zero, ux = zero, uy = zero;
            for (int s = 0; s < S2; s++) {
                const int idx = a.sten_idx[k * S2 + s];
                if (idx < 0) continue;
                const float w = a.sten_w[k * S2 + s];
                r = r + w * rho[idx];
                ux = ux + w * upx[idx];
                uy = uy + w * upy[idx];
            }
            R fx = 2.0f * r * (0.0f - ux);
            R fy = 2.0f * r * (0.0f - uy);
            if (a.clamp) {
                fx = ibm_clamp(fx);
                fy = ibm_clamp(fy);
            }
            mfx[k] = fx;
            mfy[k] = fy;
            mtx[k] = mtx[k] + fx;
            mty[k] = mty[k] + fy;
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
            ibm_atomic_add(&fix[idx], w * mfx[k]);
            ibm_atomic_add(&fiy[idx], w * mfy[k]);
        }
        __syncthreads();
        // correct_velocities_kernel + accumulate_forces_kernel (IBM_impl.cuh:28-68)
        for (int i = tid; i < np; i += blockDim.x) {
            R cx = upx[i] + fix[i] / (2.0f * rho[i]);
            R cy = upy[i] + fiy[i] / (2.0f * rho[i]);
            if (a.clamp) {
                cx = ibm_clamp(cx);
                cy = ibm_clamp(cy);
            }
            upx[i] = cx;
            upy[i] = cy;
            ftx[i] = ftx[i] + fix[i];
            fty[i] = fty[i] + fiy[i];
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

}  // namespace lbmx
