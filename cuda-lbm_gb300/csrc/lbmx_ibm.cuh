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

// Shared-memory state of the rounds: patch and marker values, then the
// stencils (index and weight per point) and the spread lists (for each patch
// node, the stencil points that touch it, in ascending order).
template <typename R>
size_t ibm_smem_bytes_of(int npatch, int nm, int stencil) {
    const size_t s2 = (size_t)stencil * stencil;
    return (size_t)(6 * npatch + 4 * nm) * sizeof(R) + (size_t)nm * s2 * (sizeof(int) + sizeof(float)) +
           ((size_t)npatch + 1 + (size_t)nm * s2) * sizeof(int);
}

template <typename R>
struct IbmSmem {
    R *upx, *upy, *rho, *half_inv;  // working velocity (u_prev of the reference), density, 1 / (2 rho)
    R *ftx, *fty;                   // Eulerian force summed over rounds
    R *mfx, *mfy, *mtx, *mty;       // marker force of this round and summed over rounds
    int* sidx;                      // [nm * S2] patch index or -1
    float* sw;                      // [nm * S2] kernel weight
    int* sp;                        // [npatch + 1] offsets into spj
    int* spj;                       // stencil points of each patch node
};

template <typename R>
__device__ __forceinline__ IbmSmem<R> ibm_layout(const IbmData<R>& a, R* sm) {
    const int np = a.npatch, nm = a.nm, nj = nm * a.stencil * a.stencil;
    IbmSmem<R> s;
    s.upx = sm;
    s.upy = s.upx + np;
    s.rho = s.upy + np;
    s.half_inv = s.rho + np;
    s.ftx = s.half_inv + np;
    s.fty = s.ftx + np;
    s.mfx = s.fty + np;
    s.mfy = s.mfx + nm;
    s.mtx = s.mfy + nm;
    s.mty = s.mtx + nm;
    s.sidx = reinterpret_cast<int*>(s.mty + nm);
    s.sw = reinterpret_cast<float*>(s.sidx + nj);
    s.sp = reinterpret_cast<int*>(s.sw + nj);
    s.spj = s.sp + np + 1;
    return s;
}

// Stage what does not depend on the flow (stencils, spread lists) and clear
// the accumulators; no barrier (the caller syncs before the rounds).
template <typename R>
__device__ void ibm_stage(const IbmData<R>& a, const IbmSmem<R>& s) {
    const int np = a.npatch, nm = a.nm, nj = nm * a.stencil * a.stencil;
    const R zero = splat(0.0f, R{});
    for (int j = threadIdx.x; j < nj; j += blockDim.x) {
        s.sidx[j] = a.sten_idx[j];
        s.sw[j] = a.sten_w[j];
    }
    const int nsp = a.spread[np];
    for (int j = threadIdx.x; j < np + 1 + nsp; j += blockDim.x) s.sp[j] = a.spread[j];
    for (int i = threadIdx.x; i < np; i += blockDim.x) s.ftx[i] = s.fty[i] = zero;
    for (int k = threadIdx.x; k < nm; k += blockDim.x) s.mtx[k] = s.mty[k] = zero;
}

// Patch density and uncorrected velocity of patch node i.
template <typename R>
__device__ __forceinline__ void ibm_set_patch(const IbmSmem<R>& s, int i, R rho, R ux, R uy) {
    s.rho[i] = rho;
    s.half_inv[i] = 1.0f / (2.0f * rho);
    s.upx[i] = ux;
    s.upy[i] = uy;
}

// All rounds of one step on the staged patch (ibm_stage, ibm_set_patch and a
// barrier before).  Each interpolation gives every stencil point its own
// thread and sums a marker's points with a fixed shuffle tree (S2 = stencil^2
// = 4 or 16 points, consecutive in one warp).  The spread gives every patch
// node a thread that adds the forces of the stencil points touching it in
// ascending order, so the result is the same bit for bit on every run, and
// applies the velocity correction in the same pass.
template <typename R, int S2>
__device__ void ibm_iterate_s(const IbmData<R>& a, const IbmSmem<R>& s) {
    const int np = a.npatch, nm = a.nm;
    const R zero = splat(0.0f, R{});
    const int tid = threadIdx.x;
    const int nj = nm * S2;
    for (int it = 0; it < a.iters; it++) {
        const bool last = it == a.iters - 1;
        // interpolate_velocities_kernel<2> (IBM_impl.cu:5-51) then
        // compute_lagrangian_kernel (IBM_impl.cuh:7-26), target velocity 0
        for (int j0 = 0; j0 < nj; j0 += blockDim.x) {
            const int j = j0 + tid;
            R r = zero, ux = zero, uy = zero;
            const int idx = j < nj ? s.sidx[j] : -1;
            if (idx >= 0) {
                const float w = s.sw[j];
                r = w * s.rho[idx];
                ux = w * s.upx[idx];
                uy = w * s.upy[idx];
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
            s.mfx[k] = fx;
            s.mfy[k] = fy;
            const R tx = s.mtx[k] + fx, ty = s.mty[k] + fy;
            s.mtx[k] = tx;
            s.mty[k] = ty;
            if (last) {
                a.marker_u[k] = ux;
                a.marker_u[nm + k] = uy;
                a.marker_rho[k] = r;
                a.marker_force[k] = tx;
                a.marker_force[nm + k] = ty;
            }
        }
        __syncthreads();
        // spread_forces_kernel<2> (IBM_impl.cu:120-154), then
        // correct_velocities_kernel + accumulate_forces_kernel (IBM_impl.cuh:28-68)
        for (int i = tid; i < np; i += blockDim.x) {
            R fx = zero, fy = zero;
            const int e1 = s.sp[i + 1];
            for (int e = s.sp[i]; e < e1; e++) {
                const int j = s.spj[e];
                const float w = s.sw[j] * a.ds;
                fx = fx + w * s.mfx[j / S2];
                fy = fy + w * s.mfy[j / S2];
            }
            R cx = s.upx[i] + fx * s.half_inv[i];
            R cy = s.upy[i] + fy * s.half_inv[i];
            if (a.clamp) {
                cx = ibm_clamp(cx);
                cy = ibm_clamp(cy);
            }
            s.upx[i] = cx;
            s.upy[i] = cy;
            const R tx = s.ftx[i] + fx, ty = s.fty[i] + fy;
            s.ftx[i] = tx;
            s.fty[i] = ty;
            if (last) {
                const long long off = a.patch_nodes[i];
                a.ibm_force[off] = tx;
                a.ibm_force[a.plane + off] = ty;
            }
        }
        __syncthreads();
    }
}

template <typename R>
__device__ void ibm_iterate(const IbmData<R>& a, const IbmSmem<R>& s) {
    if (a.stencil == 4) ibm_iterate_s<R, 16>(a, s);
    else ibm_iterate_s<R, 4>(a, s);
}

// All rounds of one step with the patch read from a.patch_rho / a.patch_u;
// sm holds ibm_smem_bytes_of<R> bytes.
template <typename R>
__device__ void ibm_rounds(const IbmData<R>& a, R* sm) {
    const IbmSmem<R> s = ibm_layout(a, sm);
    ibm_stage(a, s);
    for (int i = threadIdx.x; i < a.npatch; i += blockDim.x)
        ibm_set_patch(s, i, a.patch_rho[i], a.patch_u[i], a.patch_u[a.npatch + i]);
    __syncthreads();
    ibm_iterate(a, s);
}

}  // namespace lbmx
