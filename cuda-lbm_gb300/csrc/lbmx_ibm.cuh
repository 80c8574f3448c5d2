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

// ---------------------------------------------------------------------------
// The engine's (float) form of the same rounds, laid out for few shared-
// memory transactions: a patch node's working velocity, density and
// 1 / (2 rho) in one float4, a stencil point's patch index and weight in one
// int2, a spread entry's marker and weight (times ds) in one int2, a
// marker's force in one float2.  Four threads take a marker's 16 stencil
// points (four consecutive points each, summed in order, then a two-level
// shuffle tree; one thread per marker with the 2x2 stencil).  The patch node
// offsets and flags, which never change, are staged with the stencils before
// the kernel waits for the previous step, so the gather after the wait is a
// single round of population loads.
struct IbmFast {
    float4* ps;          // [np] {ux, uy, rho, 1 / (2 rho)}
    float2* ft;          // [np] Eulerian force summed over rounds
    float2* mf;          // [nm] marker force of this round
    float2* mt;          // [nm] marker force summed over rounds
    int2* st;            // [nm * S2] {patch index or -1, weight bits}
    int2* se;            // [nm * S2] spread entries {marker, weight * ds bits}
    int* sp;             // [np + 1] offsets into se
    int* pn;             // [np] patch node offsets (y * pitch + x)
    unsigned char* pf;   // [np] patch node flags
};

inline __host__ __device__ size_t ibm_fast_smem_bytes(int np, int nm, int stencil) {
    const size_t nj = (size_t)nm * stencil * stencil;
    return (size_t)np * (16 + 8) + (size_t)nm * (8 + 8) + nj * (8 + 8) + ((size_t)np + 1) * 4 + (size_t)np * 4 +
           (size_t)np + 16;
}

__device__ __forceinline__ IbmFast ibm_fast_layout(const IbmData<float>& a, void* sm) {
    const int np = a.npatch, nm = a.nm, nj = nm * a.stencil * a.stencil;
    IbmFast s;
    s.ps = static_cast<float4*>(sm);
    s.ft = reinterpret_cast<float2*>(s.ps + np);
    s.mf = s.ft + np;
    s.mt = s.mf + nm;
    s.st = reinterpret_cast<int2*>(s.mt + nm);
    s.se = s.st + nj;
    s.sp = reinterpret_cast<int*>(s.se + nj);
    s.pn = s.sp + np + 1;
    s.pf = reinterpret_cast<unsigned char*>(s.pn + np);
    return s;
}

// Stage what does not depend on the flow; no barrier.
static __device__ void ibm_fast_stage(const IbmData<float>& a, const IbmFast& s, const uint8_t* flags) {
    const int np = a.npatch, nm = a.nm, S2 = a.stencil * a.stencil, nj = nm * S2;
    for (int j = threadIdx.x; j < nj; j += blockDim.x) s.st[j] = make_int2(a.sten_idx[j], __float_as_int(a.sten_w[j]));
    const int nsp = a.spread[np];
    for (int i = threadIdx.x; i <= np; i += blockDim.x) s.sp[i] = a.spread[i];
    for (int e = threadIdx.x; e < nsp; e += blockDim.x) {
        const int j = a.spread[np + 1 + e];
        s.se[e] = make_int2(j / S2, __float_as_int(a.sten_w[j] * a.ds));
    }
    for (int i = threadIdx.x; i < np; i += blockDim.x) {
        const int off = a.patch_nodes[i];
        s.pn[i] = off;
        s.pf[i] = flags ? flags[off] : (unsigned char)0;
        s.ft[i] = make_float2(0.f, 0.f);
    }
    for (int k = threadIdx.x; k < nm; k += blockDim.x) s.mt[k] = make_float2(0.f, 0.f);
}

// All rounds of one step (ps filled and a barrier before); G threads per
// marker, G = S2 / 4.
template <int G>
__device__ void ibm_fast_iterate_g(const IbmData<float>& a, const IbmFast& s) {
    const int np = a.npatch, nm = a.nm, nq = nm * G;
    const int tid = threadIdx.x;
    for (int it = 0; it < a.iters; it++) {
        const bool last = it == a.iters - 1;
        // interpolate_velocities_kernel<2> (IBM_impl.cu:5-51) then
        // compute_lagrangian_kernel (IBM_impl.cuh:7-26), target velocity 0
        for (int t0 = 0; t0 < nq; t0 += blockDim.x) {
            const int t = t0 + tid;
            float r = 0.f, ux = 0.f, uy = 0.f;
            if (t < nq) {
#pragma unroll
                for (int p = 0; p < 4; p++) {
                    const int2 e = s.st[4 * t + p];
                    if (e.x >= 0) {
                        const float w = __int_as_float(e.y);
                        const float4 q = s.ps[e.x];
                        r = fmaf(w, q.z, r);
                        ux = fmaf(w, q.x, ux);
                        uy = fmaf(w, q.y, uy);
                    }
                }
            }
#pragma unroll
            for (int o = G >> 1; o > 0; o >>= 1) {
                r += __shfl_xor_sync(0xffffffffu, r, o);
                ux += __shfl_xor_sync(0xffffffffu, ux, o);
                uy += __shfl_xor_sync(0xffffffffu, uy, o);
            }
            if (t >= nq || (t & (G - 1)) != 0) continue;
            const int k = t / G;
            float fx = 2.0f * r * (0.0f - ux);
            float fy = 2.0f * r * (0.0f - uy);
            if (a.clamp) {
                fx = ibm_clamp(fx);
                fy = ibm_clamp(fy);
            }
            s.mf[k] = make_float2(fx, fy);
            const float2 m = s.mt[k];
            const float2 tt = make_float2(m.x + fx, m.y + fy);
            s.mt[k] = tt;
            if (last) {
                a.marker_u[k] = ux;
                a.marker_u[nm + k] = uy;
                a.marker_rho[k] = r;
                a.marker_force[k] = tt.x;
                a.marker_force[nm + k] = tt.y;
            }
        }
        __syncthreads();
        // spread_forces_kernel<2> (IBM_impl.cu:120-154), then
        // correct_velocities_kernel + accumulate_forces_kernel (IBM_impl.cuh:28-68),
        // each node's entries in ascending stencil-point order
        for (int i = tid; i < np; i += blockDim.x) {
            float fx = 0.f, fy = 0.f;
            const int e1 = s.sp[i + 1];
            for (int e = s.sp[i]; e < e1; e++) {
                const int2 ee = s.se[e];
                const float w = __int_as_float(ee.y);
                const float2 m = s.mf[ee.x];
                fx = fx + w * m.x;
                fy = fy + w * m.y;
            }
            const float4 q = s.ps[i];
            float cx = q.x + fx * q.w;
            float cy = q.y + fy * q.w;
            if (a.clamp) {
                cx = ibm_clamp(cx);
                cy = ibm_clamp(cy);
            }
            s.ps[i] = make_float4(cx, cy, q.z, q.w);
            const float2 f0 = s.ft[i];
            const float2 tf = make_float2(f0.x + fx, f0.y + fy);
            s.ft[i] = tf;
            if (last) {
                const long long off = s.pn[i];
                a.ibm_force[off] = tf.x;
                a.ibm_force[a.plane + off] = tf.y;
            }
        }
        __syncthreads();
    }
}

static __device__ void ibm_fast_iterate(const IbmData<float>& a, const IbmFast& s) {
    if (a.stencil == 4) ibm_fast_iterate_g<4>(a, s);
    else ibm_fast_iterate_g<1>(a, s);
}

}  // namespace lbmx
