// lbmx_device.cuh -- per-node device code of the D2Q9 engine: lattice,
// storage conversion, AA-pattern population access, boundary conditions and
// collision operators.  Every loop over populations is fully unrolled so the
// nine populations of a node live in registers.
//
// The collision operators are templates over the arithmetic type R: `float`
// for one node, `V2` for two neighbouring nodes carried in the two halves of
// a register pair and computed with Blackwell's packed FP32x2 instructions
// (FFMA2 / FADD2 / FMUL2), which halves the floating-point instruction count
// of the interior path.
#pragma once
#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <stdint.h>

#include "lbmx.h"
#include "lbmx_internal.h"

namespace lbmx {

// D2Q9 velocity set in the reference's order (src/core/lbm_constants.cuh:19-31):
// rest, E, N, W, S, NE, NW, SW, SE.
__host__ __device__ constexpr int CX(int q) {
    return (q == 1 || q == 5 || q == 8) ? 1 : ((q == 3 || q == 6 || q == 7) ? -1 : 0);
}
__host__ __device__ constexpr int CY(int q) {
    return (q == 2 || q == 5 || q == 6) ? 1 : ((q == 4 || q == 7 || q == 8) ? -1 : 0);
}
__host__ __device__ constexpr int OPP(int q) {
    return q == 0 ? 0 : (q <= 4 ? ((q + 1) % 4 + 1) : ((q - 3) % 4 + 5));
}
__host__ __device__ constexpr float WQ(int q) {
    return q == 0 ? 4.0f / 9.0f : (q <= 4 ? 1.0f / 9.0f : 1.0f / 36.0f);
}

// ---------------------------------------------------------------- arithmetic
// Two-node register pair with packed FP32x2 arithmetic (sm_100+).
struct V2 {
    float2 v;
};
__device__ __forceinline__ V2 splat(float s, V2) { return {make_float2(s, s)}; }
__device__ __forceinline__ float splat(float s, float) { return s; }
__device__ __forceinline__ V2 operator+(V2 a, V2 b) { return {__fadd2_rn(a.v, b.v)}; }
__device__ __forceinline__ V2 operator-(V2 a, V2 b) { return {__ffma2_rn(b.v, make_float2(-1.f, -1.f), a.v)}; }
__device__ __forceinline__ V2 operator*(V2 a, V2 b) { return {__fmul2_rn(a.v, b.v)}; }
__device__ __forceinline__ V2 operator*(float s, V2 b) { return {__fmul2_rn(make_float2(s, s), b.v)}; }
__device__ __forceinline__ V2 operator-(V2 a) { return {make_float2(-a.v.x, -a.v.y)}; }
__device__ __forceinline__ V2 fma(V2 a, V2 b, V2 c) { return {__ffma2_rn(a.v, b.v, c.v)}; }
__device__ __forceinline__ V2 fma(float a, V2 b, V2 c) { return {__ffma2_rn(make_float2(a, a), b.v, c.v)}; }
__device__ __forceinline__ float fma(float a, float b, float c) { return fmaf(a, b, c); }
__device__ __forceinline__ V2 vdiv(V2 a, V2 b) { return {make_float2(a.v.x / b.v.x, a.v.y / b.v.y)}; }
__device__ __forceinline__ float vdiv(float a, float b) { return a / b; }
__device__ __forceinline__ V2 vsqrt(V2 a) { return {make_float2(sqrtf(a.v.x), sqrtf(a.v.y))}; }
__device__ __forceinline__ float vsqrt(float a) { return sqrtf(a); }
__device__ __forceinline__ V2 vmin(V2 a, float b) { return {make_float2(fminf(a.v.x, b), fminf(a.v.y, b))}; }
__device__ __forceinline__ float vmin(float a, float b) { return fminf(a, b); }
__device__ __forceinline__ V2 vpos_or(V2 a, float alt) {
    return {make_float2(a.v.x > 0.f ? a.v.x : alt, a.v.y > 0.f ? a.v.y : alt)};
}
__device__ __forceinline__ float vpos_or(float a, float alt) { return a > 0.f ? a : alt; }

// ---------------------------------------------------------------- storage
// FP32 stores f itself; the 16-bit forms store the offset f - w_q, which is
// O(|u|) instead of O(1) and so keeps 10 (FP16) or 7 (BF16) significant bits
// for the part of f that carries the flow.  Offsets below FP16's normal
// range (2^-14) land on its subnormal grid of 2^-24; rounded stochastically
// that costs noise of at most 6e-8 per store, far below the 2^-11-relative
// noise of the offsets that carry the flow.
//
// Stores round stochastically by default: up with probability equal to the
// discarded fraction of the gap to the next representable value (Forsythe
// 1959; Connolly, Higham & Mary 2021), so each store is unbiased,
// E[stored] = exact.  Rounding to nearest gives a steady flow the same
// rounding error at every node every step -- a persistent source term whose
// effect the slow viscous modes amplify with the lattice size (about 1/(nu k^2)
// steps of it); stochastic errors are independent from step to step and
// average out instead.  The random bits come from a counter-based hash of
// (node offset, step), so a run is still bitwise reproducible.
template <typename T> struct Store;
//
// ld/st/ld2/st2 convert between f and the stored form; ldr/str/ld2r/st2r move
// the stored value itself (f for FP32, f - w for the 16-bit forms), for code
// that computes with offsets directly (kOffset<T>); the *_sr forms take
// random bits (sr_bits) and round stochastically.
template <typename T>
constexpr bool kOffset = sizeof(T) == 2;

// 32 well-mixed bits of a unit (two x-neighbouring nodes, even offset) and
// the step seed: the "lowbias32" integer finaliser (C. Wellons,
// hash-prospector) of a Weyl-scrambled key.  Each population's 32 random
// bits (sr_bits) serve both nodes of the unit: bits 15:0 the even node,
// bits 31:16 the odd one.
__device__ __forceinline__ uint32_t sr_hash(uint32_t unit, uint32_t seed) {
    uint32_t h = unit * 0x9E3779B1u ^ seed;
    h ^= h >> 16;
    h *= 0x7FEB352Du;
    h ^= h >> 15;
    h *= 0x846CA68Bu;
    h ^= h >> 16;
    return h;
}
// random bits of population q from a unit's hash: the product with an odd
// constant per q (a bijection, so uniform), its high half folded into its
// low half (again a bijection) -- otherwise the low half would depend on the
// hash's low bits only and repeat its pattern across the populations
__device__ __forceinline__ uint32_t sr_bits(uint32_t h, int q) {
    const uint32_t r = h * (0x2545F491u + 0x9E3779B8u * (uint32_t)q);
    return r ^ (r >> 16);
}

// The conversions themselves are the hardware's (PTX cvt.rs, sm_100 and
// later): two FP32 values to a packed pair, the upper element rounded with
// random bits rbits[31:16], the lower with rbits[15:0] (the random bits are
// added below the last kept bit, then the value is truncated).
__device__ __forceinline__ uint32_t cvt_rs_f16x2(float hi, float lo, uint32_t rbits) {
    uint32_t d;
    asm("cvt.rs.f16x2.f32 %0, %1, %2, %3;" : "=r"(d) : "f"(hi), "f"(lo), "r"(rbits));
    return d;
}
__device__ __forceinline__ uint32_t cvt_rs_bf16x2(float hi, float lo, uint32_t rbits) {
    uint32_t d;
    asm("cvt.rs.bf16x2.f32 %0, %1, %2, %3;" : "=r"(d) : "f"(hi), "f"(lo), "r"(rbits));
    return d;
}
// one value from the low half of a packed result; r16 in bits 15:0
__device__ __forceinline__ unsigned short sr_half_bits(float x, uint32_t r16) {
    return (unsigned short)(cvt_rs_f16x2(0.0f, x, r16) & 0xFFFFu);
}
__device__ __forceinline__ unsigned short sr_bf16_bits(float x, uint32_t r16) {
    return (unsigned short)(cvt_rs_bf16x2(0.0f, x, r16) & 0xFFFFu);
}
// the 16 random bits of node `lane` (0: x0, 1: x0 + 1) of a unit's 32
__device__ __forceinline__ uint32_t sr_lane16(uint32_t r, int lane) { return lane ? r >> 16 : r & 0xFFFFu; }

template <> struct Store<float> {
    static __device__ __forceinline__ float ldr(const float* p) { return *p; }
    static __device__ __forceinline__ float2 ld2r(const float* p) { return *reinterpret_cast<const float2*>(p); }
    static __device__ __forceinline__ void str(float* p, float v) { *p = v; }
    static __device__ __forceinline__ void st2r(float* p, float2 v) { *reinterpret_cast<float2*>(p) = v; }
    static __device__ __forceinline__ float ld(const float* p, float) { return *p; }
    static __device__ __forceinline__ void st(float* p, float v, float) { *p = v; }
    static __device__ __forceinline__ float2 ld2(const float* p, float) { return *reinterpret_cast<const float2*>(p); }
    static __device__ __forceinline__ void st2(float* p, float2 v, float) { *reinterpret_cast<float2*>(p) = v; }
    static __device__ __forceinline__ void str_sr(float* p, float v, uint32_t) { *p = v; }
    static __device__ __forceinline__ void st2r_sr(float* p, float2 v, uint32_t) {
        *reinterpret_cast<float2*>(p) = v;
    }
    static __device__ __forceinline__ void st_sr(float* p, float v, float, uint32_t) { *p = v; }
    // two consecutive values at any (element-aligned) address
    static __device__ __forceinline__ float2 ld2r_u(const float* p) { return make_float2(p[0], p[1]); }
    static __device__ __forceinline__ void st2r_u(float* p, float2 v) { p[0] = v.x; p[1] = v.y; }
    static __device__ __forceinline__ void st2r_sr_u(float* p, float2 v, uint32_t) { p[0] = v.x; p[1] = v.y; }
};
template <> struct Store<__half> {
    static __device__ __forceinline__ float ldr(const __half* p) { return __half2float(*p); }
    static __device__ __forceinline__ float2 ld2r(const __half* p) {
        return __half22float2(*reinterpret_cast<const __half2*>(p));
    }
    static __device__ __forceinline__ void str(__half* p, float v) { *p = __float2half_rn(v); }
    static __device__ __forceinline__ void st2r(__half* p, float2 v) {
        *reinterpret_cast<__half2*>(p) = __float22half2_rn(v);
    }
    static __device__ __forceinline__ float ld(const __half* p, float w) { return w + ldr(p); }
    static __device__ __forceinline__ void st(__half* p, float v, float w) { str(p, v - w); }
    static __device__ __forceinline__ float2 ld2(const __half* p, float w) {
        const float2 d = ld2r(p);
        return make_float2(d.x + w, d.y + w);
    }
    static __device__ __forceinline__ void st2(__half* p, float2 v, float w) { st2r(p, make_float2(v.x - w, v.y - w)); }
    // r16: 16 random bits (bits 15:0); r: a pair's 32
    static __device__ __forceinline__ void str_sr(__half* p, float v, uint32_t r16) {
        *reinterpret_cast<unsigned short*>(p) = sr_half_bits(v, r16);
    }
    static __device__ __forceinline__ void st2r_sr(__half* p, float2 v, uint32_t r) {
        *reinterpret_cast<uint32_t*>(p) = cvt_rs_f16x2(v.y, v.x, r);
    }
    static __device__ __forceinline__ void st_sr(__half* p, float v, float w, uint32_t r16) { str_sr(p, v - w, r16); }
    // two consecutive values at any (element-aligned) address: converted and
    // scaled as a pair, moved as two halves
    static __device__ __forceinline__ float2 ld2r_u(const __half* p) {
        return __half22float2(__halves2half2(p[0], p[1]));
    }
    static __device__ __forceinline__ void st2r_u(__half* p, float2 v) {
        const __half2 h = __float22half2_rn(v);
        p[0] = __low2half(h);
        p[1] = __high2half(h);
    }
    static __device__ __forceinline__ void st2r_sr_u(__half* p, float2 v, uint32_t r) {
        const uint32_t d = cvt_rs_f16x2(v.y, v.x, r);
        reinterpret_cast<unsigned short*>(p)[0] = (unsigned short)(d & 0xFFFFu);
        reinterpret_cast<unsigned short*>(p)[1] = (unsigned short)(d >> 16);
    }
};
template <> struct Store<__nv_bfloat16> {
    static __device__ __forceinline__ float ldr(const __nv_bfloat16* p) { return __bfloat162float(*p); }
    static __device__ __forceinline__ float2 ld2r(const __nv_bfloat16* p) {
        return __bfloat1622float2(*reinterpret_cast<const __nv_bfloat162*>(p));
    }
    static __device__ __forceinline__ void str(__nv_bfloat16* p, float v) { *p = __float2bfloat16_rn(v); }
    static __device__ __forceinline__ void st2r(__nv_bfloat16* p, float2 v) {
        *reinterpret_cast<__nv_bfloat162*>(p) = __float22bfloat162_rn(v);
    }
    static __device__ __forceinline__ float ld(const __nv_bfloat16* p, float w) { return w + __bfloat162float(*p); }
    static __device__ __forceinline__ void st(__nv_bfloat16* p, float v, float w) { *p = __float2bfloat16_rn(v - w); }
    static __device__ __forceinline__ float2 ld2(const __nv_bfloat16* p, float w) {
        const float2 d = __bfloat1622float2(*reinterpret_cast<const __nv_bfloat162*>(p));
        return make_float2(d.x + w, d.y + w);
    }
    static __device__ __forceinline__ void st2(__nv_bfloat16* p, float2 v, float w) {
        *reinterpret_cast<__nv_bfloat162*>(p) = __float22bfloat162_rn(make_float2(v.x - w, v.y - w));
    }
    static __device__ __forceinline__ void str_sr(__nv_bfloat16* p, float v, uint32_t r16) {
        *reinterpret_cast<unsigned short*>(p) = sr_bf16_bits(v, r16);
    }
    static __device__ __forceinline__ void st2r_sr(__nv_bfloat16* p, float2 v, uint32_t r) {
        *reinterpret_cast<uint32_t*>(p) = cvt_rs_bf16x2(v.y, v.x, r);
    }
    static __device__ __forceinline__ void st_sr(__nv_bfloat16* p, float v, float w, uint32_t r16) {
        str_sr(p, v - w, r16);
    }
    static __device__ __forceinline__ float2 ld2r_u(const __nv_bfloat16* p) {
        return __bfloat1622float2(__halves2bfloat162(p[0], p[1]));
    }
    static __device__ __forceinline__ void st2r_u(__nv_bfloat16* p, float2 v) {
        const __nv_bfloat162 h = __float22bfloat162_rn(v);
        p[0] = __low2bfloat16(h);
        p[1] = __high2bfloat16(h);
    }
    static __device__ __forceinline__ void st2r_sr_u(__nv_bfloat16* p, float2 v, uint32_t r) {
        const uint32_t d = cvt_rs_bf16x2(v.y, v.x, r);
        reinterpret_cast<unsigned short*>(p)[0] = (unsigned short)(d & 0xFFFFu);
        reinterpret_cast<unsigned short*>(p)[1] = (unsigned short)(d >> 16);
    }
};

__device__ __forceinline__ bool on_edge(const Geometry& g, int x, int y) {
    return x == 0 || y == 0 || x == g.nx - 1 || y == g.ny - 1;
}

__device__ __forceinline__ bool is_halfway(uint8_t fl) { return fl == LBMX_MOVING_WALL_BB || fl == LBMX_HALFWAY_BB; }

// Ladd's moving-wall term 2 w_q rho_w (c_q . u_w) / cs^2 with rho_w = 1
__device__ __forceinline__ float wall_term(const StepArgs& a, int q, uint8_t fl) {
    if (fl != LBMX_MOVING_WALL_BB) return 0.0f;
    return 6.0f * WQ(q) * ((float)CX(q) * a.wall_ux + (float)CY(q) * a.wall_uy);
}

// Post-stream populations of node (x, y) for the current step (general path).
// parity 1: f_q(x) sits in slot OPP(q) of the upstream node x - c_q;
// parity 0: it sits in slot q of x itself.  An upstream node outside a
// non-periodic domain sets bit q of *outmask; the value then comes from the
// edge store (what the reference's ping-pong buffers hold there, two steps
// old) or, on a half-way bounce-back node, from the node's own slot q, where
// the previous step left its reflected outgoing population.
template <typename T>
__device__ __forceinline__ void load_post_stream(const StepArgs& a, int x, int y, uint8_t fl, float f[9],
                                                 unsigned* outmask) {
    const Geometry& g = a.g;
    const T* F = static_cast<const T*>(a.f);
    const long long row = (long long)y * g.pitch;
    f[0] = Store<T>::ld(F + a.rest_plane * g.plane + row + x, WQ(0));
    const bool edge = on_edge(g, x, y);
    const bool hw = is_halfway(fl);
    const float* E = a.edge + ((long long)a.parity * g.perimeter + (edge ? edge_index(x, y, g.nx, g.ny) : 0)) * 9;
    // Every source address is chosen by selects, always in bounds, and all
    // loads are issued before any value is used: a node's nine loads are in
    // flight together instead of one after another behind branches.
    unsigned m = 0;
    const T* src[9];
#pragma unroll
    for (int q = 1; q < 9; q++) {
        int sx = x - CX(q), sy = y - CY(q);
        bool out = false;
        if (CX(q) != 0 && (sx < 0 || sx >= g.nx)) {
            if (g.periodic_x) sx = sx < 0 ? sx + g.nx : sx - g.nx;
            else out = true;
        }
        if (CY(q) != 0 && (sy < 0 || sy >= g.ny)) {
            if (g.periodic_y) sy = sy < 0 ? sy + g.ny : sy - g.ny;
            else out = true;
        }
        if (out) m |= 1u << q;
        // the node's own slot q (parity 0, or a half-way node's reflection),
        // else slot OPP(q) of the upstream node
        src[q] = (out || !a.parity) ? F + q * g.plane + row + x
                                    : F + OPP(q) * g.plane + (long long)sy * g.pitch + sx;
    }
    float vs[9], es[9];
#pragma unroll
    for (int q = 1; q < 9; q++) {
        vs[q] = Store<T>::ld(src[q], WQ(q));
        es[q] = ((m >> q) & 1u) && !hw ? E[q] : 0.0f;
    }
#pragma unroll
    for (int q = 1; q < 9; q++) {
        if ((m >> q) & 1u) f[q] = hw ? (a.parity ? vs[q] - wall_term(a, OPP(q), fl) : vs[q]) : es[q];
        else f[q] = vs[q];
    }
    *outmask = m;
}

// Write the post-collision populations of node (x, y) (general path).
// parity 1: f*_q goes to slot q of the downstream node x + c_q -- dropped
// when that node lies outside a non-periodic domain, as the reference's push
// skips it (streaming.cu:20-21), or, on a half-way node, reflected into the
// node's own free slot OPP(q); parity 0: to slot OPP(q) of x.
template <typename T>
__device__ __forceinline__ void store_post_collision(const StepArgs& a, int x, int y, const float f[9],
                                                     unsigned outmask, uint8_t fl, uint32_t seed) {
    const Geometry& g = a.g;
    T* F = static_cast<T*>(a.f);
    const long long row = (long long)y * g.pitch;
    const bool hw = is_halfway(fl);
    const bool sr = kOffset<T> && a.sr;
    const uint32_t h = sr ? sr_hash(((uint32_t)(row + x) >> 1) + a.sr_unit_origin, seed) : 0u;
    const int lane = (int)((row + x) & 1);
    // the value f of population q goes to p, rounded as configured (the
    // node's half of its unit's random bits)
    auto put = [&](T* p, float v, int q) {
        if (sr) Store<T>::st_sr(p, v, WQ(q), sr_lane16(sr_bits(h, q), lane));
        else Store<T>::st(p, v, WQ(q));
    };
    put(F + a.rest_plane * g.plane + row + x, f[0], 0);
#pragma unroll
    for (int q = 1; q < 9; q++) {
        if (a.parity) {
            int dx = x + CX(q), dy = y + CY(q);
            bool out = false;
            if (CX(q) != 0 && (dx < 0 || dx >= g.nx)) {
                if (g.periodic_x) dx = dx < 0 ? dx + g.nx : dx - g.nx;
                else out = true;
            }
            if (CY(q) != 0 && (dy < 0 || dy >= g.ny)) {
                if (g.periodic_y) dy = dy < 0 ? dy + g.ny : dy - g.ny;
                else out = true;
            }
            if (!out) put(F + q * g.plane + (long long)dy * g.pitch + dx, f[q], q);
            else if (hw) put(F + OPP(q) * g.plane + row + x, f[q] - wall_term(a, q, fl), q);
        } else {
            put(F + OPP(q) * g.plane + row + x, f[q], q);
        }
    }
    if (outmask && !hw) {
        float* E = a.edge + ((long long)a.parity * g.perimeter + edge_index(x, y, g.nx, g.ny)) * 9;
#pragma unroll
        for (int q = 1; q < 9; q++)
            if (outmask & (1u << q)) E[q] = f[q];
    }
}

// ---------------------------------------------------------------- boundaries
// All functors act on the post-stream populations of one node, in place,
// in the order the reference functors do.

__device__ __forceinline__ float feq_bc(int q, float rho, float ux, float uy) {
    // w*rho*(1 + cu/cs2 + cu^2/(2 cs2^2) - u^2/(2 cs2)), the all-float form of
    // pressureOutlet.cuh:30-40 / regularizedInlet.cuh:26-31
    const float cs2 = 1.0f / 3.0f;
    float cu = (float)CX(q) * ux + (float)CY(q) * uy;
    float uu = ux * ux + uy * uy;
    return WQ(q) * rho * (1.0f + cu / cs2 + cu * cu / (2.0f * cs2 * cs2) - uu / (2.0f * cs2));
}

// The Zou-He and bounce-back functors are templates over the arithmetic type
// R (float, or a tangent number when the tangent-linear model differentiates
// the step); with R = float they are the plain functors.

// BounceBack<2>::apply(true,true) -- bbDomainBoundary.cuh:26-49
template <typename R>
__device__ __forceinline__ void bc_bounce_back(const Geometry& g, R f[9], int x, int y) {
#pragma unroll
    for (int i = 1; i < 9; i++) {
        int xn = x + CX(i), yn = y + CY(i);
        if (xn < 0 || xn >= g.nx || yn < 0 || yn >= g.ny) f[OPP(i)] = f[i];
    }
}

// ZouHe::apply_top -- zouHeInflow.cuh:42-56
template <typename R>
__device__ __forceinline__ void bc_zouhe_top(R f[9], R ux) {
    const float uy = 0.0f;
    R rho = (f[0] + f[1] + f[3] + 2.0f * (f[2] + f[5] + f[6])) / (1.0f + uy);
    f[4] = f[2] - (2.0f / 3.0f) * rho * uy;
    R d = f[1] - f[3];
    f[7] = f[5] + 0.5f * d - 0.5f * rho * ux - (1.0f / 6.0f) * rho * uy;
    f[8] = f[6] - 0.5f * d + 0.5f * rho * ux - (1.0f / 6.0f) * rho * uy;
}

// ZouHe::apply_left -- zouHeInflow.cuh:9-22 (typo: f2 in the doubled term)
template <typename R>
__device__ __forceinline__ void bc_zouhe_left(R f[9], R ux, bool typo) {
    R fin = typo ? f[2] : f[3];
    R rho = (f[0] + f[2] + f[4] + 2.0f * (fin + f[6] + f[7])) / (1.0f - ux);
    f[1] = f[3] + (2.0f / 3.0f) * rho * ux;
    f[5] = f[7] - 0.5f * (f[2] - f[4]) + (1.0f / 6.0f) * rho * ux;
    f[8] = f[6] + 0.5f * (f[2] - f[4]) + (1.0f / 6.0f) * rho * ux;
}

// Zou-He pressure outlet at the right edge (no reference counterpart)
template <typename R>
__device__ __forceinline__ void bc_zouhe_pressure_right(R f[9], float rho) {
    R ux = -1.0f + (f[0] + f[2] + f[4] + 2.0f * (f[1] + f[5] + f[8])) / rho;
    f[3] = f[1] - (2.0f / 3.0f) * rho * ux;
    f[7] = f[5] + 0.5f * (f[2] - f[4]) - (1.0f / 6.0f) * rho * ux;
    f[6] = f[8] - 0.5f * (f[2] - f[4]) - (1.0f / 6.0f) * rho * ux;
}

// CylinderBoundary::apply -- cylinderBoundary.cuh:22-33 (full reversal)
template <typename R>
__device__ __forceinline__ void bc_cylinder(R f[9]) {
    R s[9];
#pragma unroll
    for (int i = 0; i < 9; i++) s[i] = f[i];
#pragma unroll
    for (int i = 0; i < 9; i++) f[OPP(i)] = s[i];
}

// Pi(1) of all populations, then f = f_eq + w/(2cs^4) Q:Pi
// (regularizedInlet.cuh:41-67, regularizedBounceBack.cuh:67-95)
__device__ __forceinline__ void regularize_tail(float f[9], const float fe[9], float rho, float ux, float uy) {
    const float cs2 = 1.0f / 3.0f;
    float pxx = 0.f, pyy = 0.f, pxy = 0.f;
#pragma unroll
    for (int q = 0; q < 9; q++) {
        pxx += (float)(CX(q) * CX(q)) * f[q];
        pyy += (float)(CY(q) * CY(q)) * f[q];
        pxy += (float)(CX(q) * CY(q)) * f[q];
    }
    pxx -= cs2 * rho + rho * ux * ux;
    pyy -= cs2 * rho + rho * uy * uy;
    pxy -= rho * ux * uy;
#pragma unroll
    for (int q = 0; q < 9; q++) {
        float qxx = (float)(CX(q) * CX(q)) - cs2, qyy = (float)(CY(q) * CY(q)) - cs2, qxy = (float)(CX(q) * CY(q));
        f[q] = fe[q] + (WQ(q) / (2.0f * cs2 * cs2)) * (qxx * pxx + qyy * pyy + 2.0f * qxy * pxy);
    }
}

// RegularizedInlet::apply_top -- regularizedInlet.cuh:14-69
__device__ __forceinline__ void bc_reg_inlet_top(float f[9], float ux) {
    const float uy = 0.0f;
    float rho = (f[0] + f[1] + f[3] + 2.0f * (f[2] + f[5] + f[6])) / (1.0f + uy);
    float fe[9];
#pragma unroll
    for (int q = 0; q < 9; q++) fe[q] = feq_bc(q, rho, ux, uy);
#pragma unroll
    for (int q = 0; q < 9; q++)
        if (CY(q) < 0) f[q] = fe[q] + (f[OPP(q)] - fe[OPP(q)]);
    regularize_tail(f, fe, rho, ux, uy);
}

// RegularizedBounceBack::apply -- regularizedBounceBack.cuh:13-99
__device__ __forceinline__ void bc_reg_bounce_back(const Geometry& g, float f[9], int x, int y) {
    bool unk[9];
    unk[0] = false;
#pragma unroll
    for (int i = 1; i < 9; i++) {
        if (x == 0) unk[i] = CX(i) > 0;
        else if (x == g.nx - 1) unk[i] = CX(i) < 0;
        else if (y == 0) unk[i] = CY(i) > 0;
        else if (y == g.ny - 1) unk[i] = CY(i) < 0;
        else unk[i] = false;
    }
    float rho = 0.f;
#pragma unroll
    for (int i = 0; i < 9; i++)
        if (!unk[i]) rho += (unk[OPP(i)] ? 2.0f : 1.0f) * f[i];
    float fe[9];
#pragma unroll
    for (int q = 0; q < 9; q++) fe[q] = feq_bc(q, rho, 0.f, 0.f);
#pragma unroll
    for (int q = 0; q < 9; q++)
        if (unk[q]) f[q] = fe[q] + (f[OPP(q)] - fe[OPP(q)]);
    regularize_tail(f, fe, rho, 0.f, 0.f);
}

// RegularizedCornerBounceBack::apply -- regularizedBounceBack.cuh:108-221;
// rho is the diagonal interior node's post-stream density.
__device__ __forceinline__ void bc_reg_corner(const Geometry& g, float f[9], int x, int y, float rho) {
    bool L = x == 0, R = x == g.nx - 1, B = y == 0, T = y == g.ny - 1;
    if (!((L || R) && (B || T))) return;
    bool unk[9];
    unk[0] = false;
#pragma unroll
    for (int i = 1; i < 9; i++)
        unk[i] = (L && CX(i) > 0) || (R && CX(i) < 0) || (B && CY(i) > 0) || (T && CY(i) < 0);
#pragma unroll
    for (int i = 0; i < 9; i++)
        if (unk[i]) f[i] = feq_bc(i, rho, 0.f, 0.f) - (f[OPP(i)] - feq_bc(OPP(i), rho, 0.f, 0.f));
    const float cs2 = 1.0f / 3.0f;
    float pxx = 0.f, pyy = 0.f, pxy = 0.f;
#pragma unroll
    for (int q = 0; q < 9; q++) {
        float fneq = f[q] - feq_bc(q, rho, 0.f, 0.f);
        pxx += (float)(CX(q) * CX(q)) * fneq;
        pyy += (float)(CY(q) * CY(q)) * fneq;
        pxy += (float)(CX(q) * CY(q)) * fneq;
    }
#pragma unroll
    for (int q = 0; q < 9; q++) {
        float qxx = (float)(CX(q) * CX(q)) - cs2, qyy = (float)(CY(q) * CY(q)) - cs2, qxy = (float)(CX(q) * CY(q));
        f[q] = feq_bc(q, rho, 0.f, 0.f) + (WQ(q) / (2.0f * cs2 * cs2)) * (qxx * pxx + qyy * pyy + 2.0f * qxy * pxy);
    }
}

// Parabolic inlet profile with peak u_bc over rows 0..ny-1 (no reference
// counterpart: the reference's inlets are uniform)
template <typename R>
__device__ __forceinline__ R parabolic_ux(R u_bc, int y, int ny) {
    const float h = (float)(ny - 1);
    return 4.0f * u_bc * (float)y * (h - (float)y) / (h * h);
}

// CornerBoundary (cornerBoundaries.cuh:38-82): Zou-He-style corners of a
// left inlet whose velocity the reference fixes at ux = 0.03, uy = 0.  The
// top-left one sets f2 from f4 and the bottom-left one f4 from f2, as the
// reference does.  The reference's 2-D boundary kernel never dispatches them
// (no BC_flag selects them); here they have flags of their own.
template <typename R>
__device__ __forceinline__ void bc_corner_top_left(R f[9]) {
    const float ux = 0.03f, uy = 0.0f;
    const R rho = (f[0] + f[3] + f[4] + f[6] + f[7]) / (1.0f - ux - uy);
    f[1] = f[3] + (2.0f / 3.0f) * rho * ux;
    f[2] = f[4];
    f[5] = f[7] + (1.0f / 6.0f) * rho * (ux + uy);
    f[8] = f[6] + (1.0f / 6.0f) * rho * (ux - uy);
}
template <typename R>
__device__ __forceinline__ void bc_corner_bottom_left(R f[9]) {
    const float ux = 0.03f, uy = 0.0f;
    const R rho = (f[0] + f[2] + f[3] + f[5] + f[6]) / (1.0f - ux + uy);
    f[1] = f[3] + (2.0f / 3.0f) * rho * ux;
    f[4] = f[2];
    f[5] = f[7] + (1.0f / 6.0f) * rho * (ux + uy);
    f[8] = f[6] + (1.0f / 6.0f) * rho * (ux - uy);
}

// Dispatch on the node's flag (boundaries_kernel_2D, boundaries.cuh:10-85).
__device__ __forceinline__ void apply_bc(const StepArgs& a, float f[9], int x, int y, uint8_t fl) {
    const Geometry& g = a.g;
    switch (fl) {
    case LBMX_BOUNCE_BACK: bc_bounce_back(g, f, x, y); break;
    case LBMX_ZOU_HE_TOP: bc_zouhe_top(f, a.u_bc); break;
    case LBMX_ZOU_HE_LEFT: bc_zouhe_left(f, a.u_bc, (a.quirks & LBMX_QUIRK_ZOUHE_LEFT) != 0); break;
    case LBMX_CYLINDER: bc_cylinder(f); break;
    case LBMX_ZG_OUTFLOW: {
        // zeroGradientOutflow.cuh:13-57: copy unknowns (c.n > 0) from the interior node
        int nxv = 0, nyv = 0;
        if (x == 0) nxv = 1;
        else if (x == g.nx - 1) nxv = -1;
        else if (y == 0) nyv = 1;
        else if (y == g.ny - 1) nyv = -1;
        else break;
        const float* A = a.aux + (long long)edge_index(x, y, g.nx, g.ny) * 9;
#pragma unroll
        for (int i = 0; i < 9; i++)
            if (CX(i) * nxv + CY(i) * nyv > 0) f[i] = A[i];
        break;
    }
    case LBMX_PRESSURE_OUTLET: {
        // pressureOutlet.cuh:10-41: equilibrium at rho = 1 with the interior velocity
        const float* A = a.aux + (long long)edge_index(x, y, g.nx, g.ny) * 9;
        float ux = A[1], uy = A[2];
#pragma unroll
        for (int i = 0; i < 9; i++) f[i] = feq_bc(i, 1.0f, ux, uy);
        break;
    }
    case LBMX_REGULARIZED_INLET_TOP: bc_reg_inlet_top(f, a.u_bc); break;
    case LBMX_REGULARIZED_BOUNCE_BACK: bc_reg_bounce_back(g, f, x, y); break;
    case LBMX_REGULARIZED_BOUNCE_BACK_CORNER:
        // only corner nodes act (and only they have neighbour data)
        if ((x == 0 || x == g.nx - 1) && (y == 0 || y == g.ny - 1))
            bc_reg_corner(g, f, x, y, a.aux[(long long)edge_index(x, y, g.nx, g.ny) * 9]);
        break;
    case LBMX_ZOU_HE_PRESSURE_RIGHT: bc_zouhe_pressure_right(f, a.rho_out_bc); break;
    case LBMX_ZOU_HE_PARABOLIC_LEFT: bc_zouhe_left(f, parabolic_ux(a.u_bc, y, g.ny), false); break;
    case LBMX_CORNER_TOP_LEFT: bc_corner_top_left(f); break;
    case LBMX_CORNER_BOTTOM_LEFT: bc_corner_bottom_left(f); break;
    default: break;  // half-way walls act in load/store; unknown flags are left alone as the reference does
    }
}

// ---------------------------------------------------------------- collision
// All operators take the post-stream (post-boundary) populations f, the
// density, the force-corrected velocity and the force, and overwrite f with
// the post-collision populations.  The rates (omega, S) and the CM_OPT grid
// averages have type P: float, or the adjoint's tangent type when gradients
// with respect to them are wanted.  With OFS, f holds offsets f - w_q on entry
// and on exit, and drho = rho - 1 = sum of the offsets comes exactly: every
// moment is then taken relative to its value at rest (the weights' moments
// folded in analytically), so the arithmetic keeps FP32 precision in the
// deviation from rest -- the flow -- and 16-bit storage needs no
// per-population add on load or store.  Without OFS, drho is unused.

// BGK<2>::apply with Guo forcing -- BGK.cuh:15-39
template <typename R, bool OFS = false, typename P = float>
__device__ __forceinline__ void collide_bgk(R f[9], R rho, R drho, R ux, R uy, R Fx, R Fy, P omega, bool forced) {
    const R uu = fma(ux, ux, uy * uy);
    const R one = splat(1.0f, ux);
    const R base = fma(splat(-1.5f, ux), uu, one);
    const P pref = 1.0f - 0.5f * omega;
#pragma unroll
    for (int q = 0; q < 9; q++) {
        const float cx = (float)CX(q), cy = (float)CY(q);
        R cu;
        if (CX(q) == 0) cu = cy * uy;
        else if (CY(q) == 0) cu = cx * ux;
        else cu = fma(cx, ux, cy * uy);
        // feq = w rho (1 + 3cu + 4.5cu^2 - 1.5uu); offset form:
        // feq - w = w (brm1 + drho (1 + brm1)) with brm1 = br - 1
        R feq;
        if (OFS) {
            const R brm1 = fma(cu, fma(splat(4.5f, ux), cu, splat(3.0f, ux)), splat(-1.5f, ux) * uu);
            feq = WQ(q) * fma(drho, brm1, brm1 + drho);
        } else {
            const R br = fma(cu, fma(splat(4.5f, ux), cu, splat(3.0f, ux)), base);
            feq = (WQ(q) * rho) * br;
        }
        R fn = fma(splat(omega, ux), feq - f[q], f[q]);
        if (forced) {
            // w (1 - omega/2) [ (3(c - u) + 9 (c.u) c) . F ]
            const R gx = fma(splat(9.0f * cx, ux), cu, 3.0f * (splat(cx, ux) - ux));
            const R gy = fma(splat(9.0f * cy, ux), cu, 3.0f * (splat(cy, ux) - uy));
            fn = fma(splat(WQ(q) * pref, ux), fma(gx, Fx, gy * Fy), fn);
        }
        f[q] = fn;
    }
}

// MRT<2>::apply -- MRT.cu:26-76.  m = M f with the Lallemand-Luo rows
// [rho, e, eps, jx, qx, jy, qy, pxx, pxy]; the equilibrium moments are
// M f_eq of the second-order equilibrium in closed form; the back transform
// uses M^-1 = M^T diag(1/|row|^2) (the rows are orthogonal).
template <typename R, bool OFS = false, typename P = float>
__device__ __forceinline__ void collide_mrt(R f[9], R rho, R drho, R ux, R uy, R Fx, R Fy, const P S[9],
                                            bool force_quirk, bool forced) {
    const R axis = (f[1] + f[2]) + (f[3] + f[4]);
    const R diag = (f[5] + f[6]) + (f[7] + f[8]);
    const R d13 = f[1] - f[3], d24 = f[2] - f[4];
    const R d58 = f[5] + f[8], d67 = f[6] + f[7];
    const R d56 = f[5] + f[6], d78 = f[7] + f[8];
    R m[9];
    m[1] = fma(splat(2.0f, rho), diag, fma(splat(-4.0f, rho), f[0], -axis));
    m[2] = fma(splat(4.0f, rho), f[0], fma(splat(-2.0f, rho), axis, diag));
    m[3] = d13 + (d58 - d67);
    m[4] = fma(splat(-2.0f, rho), d13, d58 - d67);
    m[5] = d24 + (d56 - d78);
    m[6] = fma(splat(-2.0f, rho), d24, d56 - d78);
    m[7] = (f[1] + f[3]) - (f[2] + f[4]);
    m[8] = (f[5] + f[7]) - (f[6] + f[8]);
    const R uu = fma(ux, ux, uy * uy);
    const R rux = rho * ux, ruy = rho * uy;
    R meq[9];
    // offset form: m and a are taken relative to the moments of w, (1, -2, 1,
    // 0, ...): meq[1] - (-2) = 3 rho uu - 2 drho, meq[2] - 1 = drho - 3 rho uu,
    // a[0] = drho / 9; m[1..8] need no shift
    meq[1] = OFS ? fma(3.0f * rho, uu, -2.0f * drho) : rho * fma(splat(3.0f, rho), uu, splat(-2.0f, rho));
    meq[2] = OFS ? fma(-3.0f * rho, uu, drho) : rho * fma(splat(-3.0f, rho), uu, splat(1.0f, rho));
    meq[3] = rux;
    meq[4] = -rux;
    meq[5] = ruy;
    meq[6] = -ruy;
    meq[7] = rho * fma(ux, ux, -(uy * uy));
    meq[8] = rux * uy;
    // post-collision moments m - S (m - m_eq), scaled by 1/|row|^2; the density
    // moment is conserved exactly (m_eq = m)
    const float inv_norm[9] = {1.0f / 9.0f, 1.0f / 36.0f, 1.0f / 36.0f, 1.0f / 6.0f, 1.0f / 12.0f,
                               1.0f / 6.0f, 1.0f / 12.0f, 0.25f, 0.25f};
    R a[9];
    a[0] = (1.0f / 9.0f) * (OFS ? drho : rho);
#pragma unroll
    for (int k = 1; k < 9; k++) a[k] = inv_norm[k] * fma(splat(-S[k], rho), m[k] - meq[k], m[k]);
    if (forced) {
        // (1 - S/2) F in moment space (MRT.cu:4-24, Silva & Semiao 2012)
        const R fu = fma(Fx, ux, Fy * uy);
        R Fm[9];
        Fm[1] = 6.0f * fu;
        Fm[2] = -6.0f * fu;
        Fm[3] = Fx;
        Fm[4] = force_quirk ? Fy : -Fx;
        Fm[5] = force_quirk ? -Fx : Fy;
        Fm[6] = -Fy;
        Fm[7] = 2.0f * fma(Fx, ux, -(Fy * uy));
        Fm[8] = fma(Fx, uy, Fy * ux);
#pragma unroll
        for (int k = 1; k < 9; k++) a[k] = fma(splat(inv_norm[k] * (1.0f - 0.5f * S[k]), rho), Fm[k], a[k]);
    }
    const R base_axis = a[0] - fma(splat(2.0f, rho), a[2], a[1]);
    const R base_diag = a[0] + fma(splat(2.0f, rho), a[1], a[2]);
    f[0] = fma(splat(4.0f, rho), a[2] - a[1], a[0]);
    const R ax = fma(splat(-2.0f, rho), a[4], a[3]);
    const R ay = fma(splat(-2.0f, rho), a[6], a[5]);
    f[1] = base_axis + (ax + a[7]);
    f[3] = base_axis - (ax - a[7]);
    f[2] = base_axis + (ay - a[7]);
    f[4] = base_axis - (ay + a[7]);
    const R px = a[3] + a[4], py = a[5] + a[6];
    f[5] = base_diag + ((px + py) + a[8]);
    f[6] = base_diag + ((py - px) - a[8]);
    f[7] = base_diag - ((px + py) - a[8]);
    f[8] = base_diag + ((px - py) - a[8]);
}

// CM<2,Adapter>::apply -- CM.cuh:27-138.  Central moments about the
// force-corrected velocity, De Rosis (2019) forcing, relaxation with S[i]
// or the adapter rate `hor` for i > 5 (NoAdapter: use_hor = false), back
// transform through raw moments (binomial shift) and the raw-moment basis
// of D2Q9, the same linear map as the reference's closed-form T^-1(u).
template <typename R, bool OFS = false, typename P = float>
__device__ __forceinline__ void collide_cm(R f[9], R rho, R drho, R ux, R uy, R Fx, R Fy, const P S[9], R hor,
                                           bool use_hor) {
    // raw moments; in offset form m20, m02 and m22 are taken relative to their
    // rest values 1/3, 1/3, 1/9 (the other raw moments vanish at rest)
    const R m10 = (f[1] - f[3]) + ((f[5] + f[8]) - (f[6] + f[7]));
    const R m01 = (f[2] - f[4]) + ((f[5] + f[6]) - (f[7] + f[8]));
    const R m22 = (f[5] + f[6]) + (f[7] + f[8]);
    const R m20 = (f[1] + f[3]) + m22;
    const R m02 = (f[2] + f[4]) + m22;
    const R m11 = (f[5] + f[7]) - (f[6] + f[8]);
    const R m21 = (f[5] + f[6]) - (f[7] + f[8]);
    const R m12 = (f[5] + f[8]) - (f[6] + f[7]);
    const R ux2 = ux * ux, uy2 = uy * uy, uxy = ux * uy;
    const R two = splat(2.0f, rho);
    const float third = 1.0f / 3.0f;
    // central moments kappa_ab = sum f (cx-ux)^a (cy-uy)^b (offset form: k20,
    // k02 less 1/3 and k22 less 1/9; the rest parts of m20, m02, m22 enter
    // k21, k12 and k22 as the explicit u/3 terms)
    const R k10 = fma(-ux, rho, m10);
    const R k01 = fma(-uy, rho, m01);
    const R k20 = fma(ux2, rho, fma(-two * ux, m10, m20));
    const R k02 = fma(uy2, rho, fma(-two * uy, m01, m02));
    const R k11 = fma(uxy, rho, fma(-ux, m01, fma(-uy, m10, m11)));
    R k21 = fma(-(ux2 * uy), rho, fma(two * uxy, m10, fma(ux2, m01, fma(-uy, m20, fma(-two * ux, m11, m21)))));
    R k12 = fma(-(ux * uy2), rho, fma(two * uxy, m01, fma(uy2, m10, fma(-ux, m02, fma(-two * uy, m11, m12)))));
    R k22 = fma(ux2 * uy2, rho,
                fma(-two * (ux2 * uy), m01,
                    fma(-two * (ux * uy2), m10,
                        fma(splat(4.0f, rho) * uxy, m11,
                            fma(uy2, m20, fma(ux2, m02, fma(-two * uy, m21, fma(-two * ux, m12, m22))))))));
    if (OFS) {
        k21 = fma(-uy, splat(third, rho), k21);
        k12 = fma(-ux, splat(third, rho), k12);
        k22 = fma(ux2 + uy2, splat(third, rho), k22);
    }
    const float cs2 = 1.0f / 3.0f;
    // relaxation k - s (k - k_eq) + (1 - s/2) F with k_eq = [rho, 0, 0,
    // 2 rho cs2, 0, 0, 0, 0, rho cs2^2] and F = [0, Fx, Fy, 0, 0, 0, Fy cs2, Fx cs2, 0]
    // (offset form: k_eq of ksum and k22 less their rest values, in drho)
    const R s3 = splat(S[3], rho), s4 = splat(S[4], rho), s5 = splat(S[5], rho);
    const R s6 = use_hor ? hor : splat(S[6], rho);
    const R s7 = use_hor ? hor : splat(S[7], rho);
    const R s8 = use_hor ? hor : splat(S[8], rho);
    const R one = splat(1.0f, rho), half = splat(0.5f, rho);
    const R rr = OFS ? drho : rho;
    const R c10 = fma(splat(-S[1], rho), k10, k10) + (1.0f - 0.5f * S[1]) * Fx;
    const R c01 = fma(splat(-S[2], rho), k01, k01) + (1.0f - 0.5f * S[2]) * Fy;
    const R ksum = k20 + k02, kdiff = k20 - k02;
    const R t3 = fma(-s3, ksum - (2.0f * cs2) * rr, ksum);
    const R t4 = fma(-s4, kdiff, kdiff);
    const R c11 = fma(-s5, k11, k11);
    const R c21 = fma(fma(-half, s6, one), cs2 * Fy, fma(-s6, k21, k21));
    const R c12 = fma(fma(-half, s7, one), cs2 * Fx, fma(-s7, k12, k12));
    const R c22 = fma(-s8, k22 - (cs2 * cs2) * rr, k22);
    const R c20 = 0.5f * (t3 + t4), c02 = 0.5f * (t3 - t4);
    const R c00 = rho;
    // back to raw moments (binomial shift by +u), then to populations
    // (offset form: r20, r02, r22 less their rest values; c20, c02 carry the
    // 1/3 into r21 and r12 explicitly)
    const R r10 = fma(ux, c00, c10);
    const R r01 = fma(uy, c00, c01);
    const R r20 = fma(ux2, c00, fma(two * ux, c10, c20));
    const R r02 = fma(uy2, c00, fma(two * uy, c01, c02));
    const R r11 = fma(uxy, c00, fma(ux, c01, fma(uy, c10, c11)));
    R r21 = fma(ux2 * uy, c00, fma(two * uxy, c10, fma(ux2, c01, fma(uy, c20, fma(two * ux, c11, c21)))));
    R r12 = fma(ux * uy2, c00, fma(two * uxy, c01, fma(uy2, c10, fma(ux, c02, fma(two * uy, c11, c12)))));
    R r22 = fma(ux2 * uy2, c00,
                fma(two * (ux2 * uy), c01,
                    fma(two * (ux * uy2), c10,
                        fma(splat(4.0f, rho) * uxy, c11,
                            fma(uy2, c20, fma(ux2, c02, fma(two * uy, c21, fma(two * ux, c12, c22))))))));
    if (OFS) {
        r21 = fma(uy, splat(third, rho), r21);
        r12 = fma(ux, splat(third, rho), r12);
        r22 = fma(ux2 + uy2, splat(third, rho), r22);
    }
    const R o00 = OFS ? drho : c00;
    f[0] = (o00 - (r20 + r02)) + r22;
    f[1] = 0.5f * ((r10 + r20) - (r12 + r22));
    f[3] = 0.5f * ((r20 + r12) - (r10 + r22));
    f[2] = 0.5f * ((r01 + r02) - (r21 + r22));
    f[4] = 0.5f * ((r02 + r21) - (r01 + r22));
    f[5] = 0.25f * ((r11 + r21) + (r12 + r22));
    f[6] = 0.25f * ((r21 + r22) - (r11 + r12));
    f[7] = 0.25f * ((r11 + r22) - (r21 + r12));
    f[8] = 0.25f * ((r12 + r22) - (r11 + r21));
}

// Initial populations f_eq(rho, u) (init_node, src/core/init/init.cuh:12-27):
// second-order equilibrium, bracket in double as equilibrium.cu:13-38
// evaluates it (cs^2 and cs^4 rounded to float first, as there); the
// divisions become products with the reciprocals, computed once.  OFS: the
// offsets f_eq - w_q, formed in double before the rounding.
template <bool OFS = false>
__device__ __forceinline__ void init_equilibrium(float rho, float ux, float uy, float fe[9]) {
    const float cs = 1.0f / sqrtf(3.0f);
    const float cs2 = cs * cs, cs4 = cs2 * cs2;
    const double inv_cs2 = 1.0 / (double)cs2, half_inv_cs4 = 0.5 / (double)cs4;
    const float uu = ux * ux + uy * uy;
    const double base = 1.0 - 0.5 * (double)uu * inv_cs2;
#pragma unroll
    for (int q = 0; q < 9; q++) {
        const double cu = (double)((float)CX(q) * ux + (float)CY(q) * uy);
        const double br = base + cu * cu * half_inv_cs4 + cu * inv_cs2;
        fe[q] = OFS ? (float)((double)(WQ(q) * rho) * br - (double)WQ(q)) : (float)((double)(WQ(q) * rho) * br);
    }
}

// Brinkman drag of a partially solid node (Guo & Zhao 2002, Darcy term):
// F_B = -gamma rho u with u itself force-corrected, so
// u = (j + F/2) / (rho (1 + gamma/2)) and the collision sees F + F_B.
// gamma = 0 leaves u and F bit for bit unchanged.
template <typename R>
__device__ __forceinline__ void brinkman(R gm, R rho, R& ux, R& uy, R& Fx, R& Fy) {
    const R sc = vdiv(splat(1.0f, rho), fma(splat(0.5f, rho), gm, splat(1.0f, rho)));
    ux = ux * sc;
    uy = uy * sc;
    const R grho = gm * rho;
    Fx = fma(-grho, ux, Fx);
    Fy = fma(-grho, uy, Fy);
}

// OptimalAdapter::compute_higher_order_relaxation -- adapters.cuh:48-111
// (Li et al. 2020 regression, theta* = (0.0003, -0.00775, 0.00016, 0.0087)).
template <typename R, typename P = float>
__device__ __forceinline__ R optimal_rate(R rho, R jmag, R pimag, const P* avg) {
    R ts = (0.0003f / avg[0]) * rho;
    ts = fma(splat(-0.00775f / avg[1], rho), jmag, ts);
    ts = fma(splat(0.00016f / avg[2], rho), pimag, ts);
    ts = ts + splat(0.0087f, rho);
    ts = vpos_or(ts, 0.005f);
    ts = vmin(ts, 1.5f);
    return vdiv(splat(1.0f, rho), fma(splat(3.0f, rho), ts, splat(0.5f, rho)));
}

}  // namespace lbmx
