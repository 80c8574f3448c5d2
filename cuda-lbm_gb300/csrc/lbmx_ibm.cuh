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

__device__ __forceinline__ float ibm_shfl_xor(float x, int o) { return __shfl_xor_sync(0xffffffffu, x, o); }
template <int K>
__device__ __forceinline__ Dual<K> ibm_shfl_xor(const Dual<K>& x, int o) {
    Dual<K> r;
    r.v = __shfl_xor_sync(0xffffffffu, x.v, o);
#pragma unroll
    for (int k = 0; k < K; k++) r.d[k] = __shfl_xor_sync(0xffffffffu, x.d[k], o);
    return r;
}

// patch and marker state, then the stencils (index and weight per point)
template <typename R>
size_t ibm_smem_bytes_of(int npatch, int nm, int stencil) {
    return (size_t)(8 * npatch + 4 * nm) * sizeof(R) + (size_t)nm * stencil * stencil * (sizeof(int) + sizeof(float));
}

// All rounds of one step in one CTA; sm holds ibm_smem_bytes_of<R> bytes.
// The stencils are staged in shared memory once; each interpolation gives
// every stencil point its own thread and sums a marker's points with a fixed
// shuffle tree (S2 = stencil^2 = 4 or 16 points, consecutive in one warp).
template <typename R, int S2>
__device__ void ibm_rounds_s(const IbmData<R>& a, R* sm) {
    const int np = a.npatch, nm = a.nm;
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
    R* half_inv = mty + nm;  // 1 / (2 rho) of each patch node (rho is fixed over the rounds)
    int* sidx = reinterpret_cast<int*>(half_inv + np);
    float* sw = reinterpret_cast<float*>(sidx + nm * S2);
    const int tid = threadIdx.x;
    const int nj = nm * S2;
    for (int j = tid; j < nj; j += blockDim.x) {
        sidx[j] = a.sten_idx[j];
        sw[j] = a.sten_w[j];
    }
    for (int i = tid; i < np; i += blockDim.x) {
        upx[i] = a.patch_u[i];
        upy[i] = a.patch_u[np + i];
        rho[i] = a.patch_rho[i];
        half_inv[i] = 1.0f / (2.0f * rho[i]);
        ftx[i] = zero;
        fty[i] = zero;
    }
    for (int k = tid; k < nm; k += blockDim.x) mtx[k] = mty[k] = zero;
    __syncthreads();
    for (int it = 0; it < a.iters; it++) {
        for (int i = tid; i < np; i += blockDim.x) fix[i] = fiy[i] = zero;
        // interpolate_velocities_kernel<2> (IBM_impl.cu:5-51) then
        // compute_lagrangian_kernel (IBM_impl.cuh:7-26), target velocity 0
        for (int j0 = 0; j0 < nj; j0 += blockDim.x) {
            const int j = j0 + tid;
            R r = zero, ux = zero, uy = zero;
            const int idx = j < nj ? sidx[j] : -1;
            if (idx >= 0) {
                const float w = sw[j];
                r = w * rho[idx];
                ux = w * upx[idx];
                uy = w * upy[idx];
            }
            for (int o = S2 >> 1; o > 0; o >>= 1) {
                r = r + ibm_shfl_xor(r, o);
                ux = ux + ibm_shfl_xor(ux, o);
                uy = uy + ibm_shfl_xor(uy, o);
            }
            if (j >= nj || (j & (S2 - 1)) != 0) continue;
            const int k = j / S2;
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
        for (int j = tid; j < nj; j += blockDim.x) {
            const int k = j / S2;
            const int idx = sidx[j];
            if (idx < 0) continue;
            const float w = sw[j] * a.ds;
            ibm_atomic_add(&fix[idx], w * mfx[k]);
            ibm_atomic_add(&fiy[idx], w * mfy[k]);
        }
        __syncthreads();
        // correct_velocities_kernel + accumulate_forces_kernel (IBM_impl.cuh:28-68)
        for (int i = tid; i < np; i += blockDim.x) {
            R cx = upx[i] + fix[i] * half_inv[i];
            R cy = upy[i] + fiy[i] * half_inv[i];
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

// the rounds for the stencil of a (2x2 or 4x4 nodes per marker)
template <typename R>
__device__ void ibm_rounds(const IbmData<R>& a, R* sm) {
    if (a.stencil == 4) ibm_rounds_s<R, 16>(a, sm);
    else ibm_rounds_s<R, 4>(a, sm);
}

}  // namespace lbmx
