// lbmx_dual.cuh -- forward-mode tangent numbers for the adjoint kernels.
//
// Dual<K> carries a value and K directional derivatives.  It supplies the
// arithmetic the templated per-node code of lbmx_device.cuh uses (splat, fma,
// vdiv, vsqrt, vmin, vpos_or and the operators), so the boundary, Brinkman
// and collision code differentiates itself: seeding one input's tangent with
// 1 yields that column of the node's Jacobian, exactly (to rounding).
#pragma once
#include "lbmx_device.cuh"

namespace lbmx {

template <int K>
struct Dual {
    float v;
    float d[K];
};

template <int K>
__device__ __forceinline__ Dual<K> dconst(float v) {
    Dual<K> r;
    r.v = v;
#pragma unroll
    for (int k = 0; k < K; k++) r.d[k] = 0.0f;
    return r;
}

template <int K> __device__ __forceinline__ Dual<K> splat(float s, Dual<K>) { return dconst<K>(s); }
template <int K> __device__ __forceinline__ Dual<K> splat(Dual<K> s, Dual<K>) { return s; }

template <int K>
__device__ __forceinline__ Dual<K> operator+(Dual<K> a, Dual<K> b) {
    Dual<K> r;
    r.v = a.v + b.v;
#pragma unroll
    for (int k = 0; k < K; k++) r.d[k] = a.d[k] + b.d[k];
    return r;
}
template <int K>
__device__ __forceinline__ Dual<K> operator-(Dual<K> a, Dual<K> b) {
    Dual<K> r;
    r.v = a.v - b.v;
#pragma unroll
    for (int k = 0; k < K; k++) r.d[k] = a.d[k] - b.d[k];
    return r;
}
template <int K>
__device__ __forceinline__ Dual<K> operator-(Dual<K> a) {
    Dual<K> r;
    r.v = -a.v;
#pragma unroll
    for (int k = 0; k < K; k++) r.d[k] = -a.d[k];
    return r;
}
template <int K>
__device__ __forceinline__ Dual<K> operator*(Dual<K> a, Dual<K> b) {
    Dual<K> r;
    r.v = a.v * b.v;
#pragma unroll
    for (int k = 0; k < K; k++) r.d[k] = fmaf(a.d[k], b.v, a.v * b.d[k]);
    return r;
}
template <int K>
__device__ __forceinline__ Dual<K> operator*(float s, Dual<K> b) {
    Dual<K> r;
    r.v = s * b.v;
#pragma unroll
    for (int k = 0; k < K; k++) r.d[k] = s * b.d[k];
    return r;
}
template <int K> __device__ __forceinline__ Dual<K> operator*(Dual<K> b, float s) { return s * b; }
template <int K> __device__ __forceinline__ Dual<K> operator+(float s, Dual<K> b) { return dconst<K>(s) + b; }
template <int K> __device__ __forceinline__ Dual<K> operator+(Dual<K> b, float s) { return b + dconst<K>(s); }
template <int K> __device__ __forceinline__ Dual<K> operator-(float s, Dual<K> b) { return dconst<K>(s) - b; }
template <int K> __device__ __forceinline__ Dual<K> operator-(Dual<K> b, float s) { return b - dconst<K>(s); }
template <int K>
__device__ __forceinline__ Dual<K> operator/(Dual<K> a, Dual<K> b) {
    Dual<K> r;
    r.v = a.v / b.v;
    const float ib = 1.0f / b.v;
#pragma unroll
    for (int k = 0; k < K; k++) r.d[k] = (a.d[k] - r.v * b.d[k]) * ib;
    return r;
}
template <int K> __device__ __forceinline__ Dual<K> operator/(float s, Dual<K> b) { return dconst<K>(s) / b; }
template <int K> __device__ __forceinline__ Dual<K> operator/(Dual<K> a, float s) { return a / dconst<K>(s); }

template <int K>
__device__ __forceinline__ Dual<K> fma(Dual<K> a, Dual<K> b, Dual<K> c) {
    Dual<K> r;
    r.v = fmaf(a.v, b.v, c.v);
#pragma unroll
    for (int k = 0; k < K; k++) r.d[k] = fmaf(a.d[k], b.v, fmaf(a.v, b.d[k], c.d[k]));
    return r;
}
template <int K> __device__ __forceinline__ Dual<K> fma(float a, Dual<K> b, Dual<K> c) { return fma(dconst<K>(a), b, c); }
template <int K> __device__ __forceinline__ Dual<K> vdiv(Dual<K> a, Dual<K> b) { return a / b; }
template <int K>
__device__ __forceinline__ Dual<K> vsqrt(Dual<K> a) {
    Dual<K> r;
    r.v = sqrtf(a.v);
    // the subgradient 0 at a = 0 (|u| of a node at rest)
    const float h = r.v > 0.0f ? 0.5f / r.v : 0.0f;
#pragma unroll
    for (int k = 0; k < K; k++) r.d[k] = a.d[k] * h;
    return r;
}
template <int K>
__device__ __forceinline__ Dual<K> vmin(Dual<K> a, float b) {
    return a.v <= b ? a : dconst<K>(b);
}
template <int K>
__device__ __forceinline__ Dual<K> vpos_or(Dual<K> a, float alt) {
    return a.v > 0.0f ? a : dconst<K>(alt);
}

}  // namespace lbmx
