// lbmx_device.cuh -- per-node device code of the D2Q9 engine: lattice,
// storage conversion, AA-pattern population access, boundary conditions and
// collision operators.  Every loop over populations is fully unrolled so the
// nine populations of a node live in registers.
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

// ---------------------------------------------------------------- storage
// FP32 stores f itself; the 16-bit forms store the offset f - w_q, which is
// O(|u|) instead of O(1) and so keeps 10 (FP16) or 7 (BF16) significant bits
// for the part of f that carries the flow.
template <typename T> struct Store;
template <> struct Store<float> {
    static __device__ __forceinline__ float ld(const float* p, float) { return *p; }
    static __device__ __forceinline__ void st(float* p, float v, float) { *p = v; }
};
template <> struct Store<__half> {
    static __device__ __forceinline__ float ld(const __half* p, float w) { return w + __half2float(*p); }
    static __device__ __forceinline__ void st(__half* p, float v, float w) { *p = __float2half_rn(v - w); }
};
template <> struct Store<__nv_bfloat16> {
    static __device__ __forceinline__ float ld(const __nv_bfloat16* p, float w) { return w + __bfloat162float(*p); }
    static __device__ __forceinline__ void st(__nv_bfloat16* p, float v, float w) { *p = __float2bfloat16_rn(v - w); }
};

__device__ __forceinline__ bool on_edge(const Geometry& g, int x, int y) {
    return x == 0 || y == 0 || x == g.nx - 1 || y == g.ny - 1;
}

// Post-stream populations of node (x, y) for the current step.
// parity 1: f_q(x) sits in slot OPP(q) of the upstream node x - c_q;
// parity 0: it sits in slot q of x itself.  Upstream nodes outside a
// non-periodic domain read the edge store (bit q of *outmask set).
template <typename T>
__device__ __forceinline__ void load_post_stream(const StepArgs& a, int x, int y, float f[9],
                                                 unsigned* outmask) {
    const Geometry& g = a.g;
    const T* F = static_cast<const T*>(a.f);
    const long long row = (long long)y * g.pitch;
    f[0] = Store<T>::ld(F + a.rest_plane * g.plane + row + x, WQ(0));
    const bool edge = on_edge(g, x, y);
    const float* E = a.edge + ((long long)a.parity * g.perimeter + (edge ? edge_index(x, y, g.nx, g.ny) : 0)) * 9;
    unsigned m = 0;
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
        if (out) {
            f[q] = E[q];
            m |= 1u << q;
        } else if (a.parity) {
            f[q] = Store<T>::ld(F + OPP(q) * g.plane + (long long)sy * g.pitch + sx, WQ(q));
        } else {
            f[q] = Store<T>::ld(F + q * g.plane + row + x, WQ(q));
        }
    }
    *outmask = m;
}

// Write the post-collision populations of node (x, y).
// parity 1: f*_q goes to slot q of the downstream node x + c_q (dropped when
// that node lies outside a non-periodic domain, as the reference's push
// skips it, streaming.cu:20-21); parity 0: to slot OPP(q) of x.
template <typename T>
__device__ __forceinline__ void store_post_collision(const StepArgs& a, int x, int y, const float f[9],
                                                     unsigned outmask, uint8_t fl) {
    const Geometry& g = a.g;
    T* F = static_cast<T*>(a.f);
    const long long row = (long long)y * g.pitch;
    Store<T>::st(F + a.rest_plane * g.plane + row + x, f[0], WQ(0));
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
            if (!out) Store<T>::st(F + q * g.plane + (long long)dy * g.pitch + dx, f[q], WQ(q));
        } else {
            Store<T>::st(F + OPP(q) * g.plane + row + x, f[q], WQ(q));
        }
    }
    if (outmask) {
        const int e = edge_index(x, y, g.nx, g.ny);
        float* E = a.edge + ((long long)a.parity * g.perimeter + e) * 9;
        if (fl == LBMX_MOVING_WALL_BB || fl == LBMX_HALFWAY_BB) {
            // half-way bounce-back: a population leaving through the wall
            // (its reverse has an outside upstream node) comes back reversed
            // next step, with Ladd's term -2 w rho_w c.u_w / cs^2, rho_w = 1
            float* En = a.edge + ((long long)(a.parity ^ 1) * g.perimeter + e) * 9;
            const bool moving = fl == LBMX_MOVING_WALL_BB;
#pragma unroll
            for (int q = 1; q < 9; q++)
                if (outmask & (1u << OPP(q))) {
                    const float cu = (float)CX(q) * a.wall_ux + (float)CY(q) * a.wall_uy;
                    En[OPP(q)] = f[q] - (moving ? 6.0f * WQ(q) * cu : 0.0f);
                }
        } else {
#pragma unroll
            for (int q = 1; q < 9; q++)
                if (outmask & (1u << q)) E[q] = f[q];
        }
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

// BounceBack<2>::apply(true,true) -- bbDomainBoundary.cuh:26-49
__device__ __forceinline__ void bc_bounce_back(const Geometry& g, float f[9], int x, int y) {
#pragma unroll
    for (int i = 1; i < 9; i++) {
        int xn = x + CX(i), yn = y + CY(i);
        if (xn < 0 || xn >= g.nx || yn < 0 || yn >= g.ny) f[OPP(i)] = f[i];
    }
}

// ZouHe::apply_top -- zouHeInflow.cuh:42-56
__device__ __forceinline__ void bc_zouhe_top(float f[9], float ux) {
    const float uy = 0.0f;
    float rho = (f[0] + f[1] + f[3] + 2.0f * (f[2] + f[5] + f[6])) / (1.0f + uy);
    f[4] = f[2] - (2.0f / 3.0f) * rho * uy;
    float d = f[1] - f[3];
    f[7] = f[5] + 0.5f * d - 0.5f * rho * ux - (1.0f / 6.0f) * rho * uy;
    f[8] = f[6] - 0.5f * d + 0.5f * rho * ux - (1.0f / 6.0f) * rho * uy;
}

// ZouHe::apply_left -- zouHeInflow.cuh:9-22 (typo: f2 in the doubled term)
__device__ __forceinline__ void bc_zouhe_left(float f[9], float ux, bool typo) {
    float fin = typo ? f[2] : f[3];
    float rho = (f[0] + f[2] + f[4] + 2.0f * (fin + f[6] + f[7])) / (1.0f - ux);
    f[1] = f[3] + (2.0f / 3.0f) * rho * ux;
    f[5] = f[7] - 0.5f * (f[2] - f[4]) + (1.0f / 6.0f) * rho * ux;
    f[8] = f[6] + 0.5f * (f[2] - f[4]) + (1.0f / 6.0f) * rho * ux;
}

// Zou-He pressure outlet at the right edge (no reference counterpart)
__device__ __forceinline__ void bc_zouhe_pressure_right(float f[9], float rho) {
    float ux = -1.0f + (f[0] + f[2] + f[4] + 2.0f * (f[1] + f[5] + f[8])) / rho;
    f[3] = f[1] - (2.0f / 3.0f) * rho * ux;
    f[7] = f[5] + 0.5f * (f[2] - f[4]) - (1.0f / 6.0f) * rho * ux;
    f[6] = f[8] - 0.5f * (f[2] - f[4]) - (1.0f / 6.0f) * rho * ux;
}

// CylinderBoundary::apply -- cylinderBoundary.cuh:22-33 (full reversal)
__device__ __forceinline__ void bc_cylinder(float f[9]) {
    float s[9];
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
    case LBMX_MOVING_WALL_BB:
    case LBMX_HALFWAY_BB: break;  // applied by store_post_collision
    case LBMX_ZOU_HE_PRESSURE_RIGHT: bc_zouhe_pressure_right(f, a.rho_out_bc); break;
    case LBMX_ZOU_HE_PARABOLIC_LEFT: {
        float h = (float)(g.ny - 1);
        float ux = 4.0f * a.u_bc * (float)y * (h - (float)y) / (h * h);
        bc_zouhe_left(f, ux, false);
        break;
    }
    default: break;  // the reference leaves unknown flags alone
    }
}

// ---------------------------------------------------------------- collision

// BGK<2>::apply with Guo forcing -- BGK.cuh:15-39
__device__ __forceinline__ void collide_bgk(float f[9], float rho, float ux, float uy, float Fx, float Fy,
                                            float omega) {
    const float uu = ux * ux + uy * uy;
    const float pref = 1.0f - 0.5f * omega;
#pragma unroll
    for (int q = 0; q < 9; q++) {
        const float cx = (float)CX(q), cy = (float)CY(q);
        const float cu = cx * ux + cy * uy;
        const float feq = WQ(q) * rho * (1.0f + 3.0f * cu + 4.5f * cu * cu - 1.5f * uu);
        const float ft = WQ(q) * pref * ((3.0f * (cx - ux) + 9.0f * cu * cx) * Fx + (3.0f * (cy - uy) + 9.0f * cu * cy) * Fy);
        f[q] = f[q] - omega * (f[q] - feq) + ft;
    }
}

// MRT<2>::apply -- MRT.cu:26-76.  m = M f with the Lallemand-Luo rows
// [rho, e, eps, jx, qx, jy, qy, pxx, pxy]; the equilibrium moments are
// M f_eq of the second-order equilibrium in closed form; the back transform
// uses M^-1 = M^T diag(1/|row|^2) (the rows are orthogonal).
__device__ __forceinline__ void collide_mrt(float f[9], float rho, float ux, float uy, float Fx, float Fy,
                                            const float S[9], bool force_quirk) {
    const float axis = f[1] + f[2] + f[3] + f[4];
    const float diag = f[5] + f[6] + f[7] + f[8];
    float m[9];
    m[0] = f[0] + axis + diag;
    m[1] = -4.0f * f[0] - axis + 2.0f * diag;
    m[2] = 4.0f * f[0] - 2.0f * axis + diag;
    m[3] = f[1] - f[3] + f[5] - f[6] - f[7] + f[8];
    m[4] = -2.0f * (f[1] - f[3]) + f[5] - f[6] - f[7] + f[8];
    m[5] = f[2] - f[4] + f[5] + f[6] - f[7] - f[8];
    m[6] = -2.0f * (f[2] - f[4]) + f[5] + f[6] - f[7] - f[8];
    m[7] = f[1] - f[2] + f[3] - f[4];
    m[8] = f[5] - f[6] + f[7] - f[8];
    const float uu = ux * ux + uy * uy;
    float meq[9];
    meq[0] = rho;
    meq[1] = rho * (-2.0f + 3.0f * uu);
    meq[2] = rho * (1.0f - 3.0f * uu);
    meq[3] = rho * ux;
    meq[4] = -rho * ux;
    meq[5] = rho * uy;
    meq[6] = -rho * uy;
    meq[7] = rho * (ux * ux - uy * uy);
    meq[8] = rho * ux * uy;
    const float fu = Fx * ux + Fy * uy;
    float Fm[9];
    Fm[0] = 0.0f;
    Fm[1] = 6.0f * fu;
    Fm[2] = -6.0f * fu;
    Fm[3] = Fx;
    Fm[4] = force_quirk ? Fy : -Fx;
    Fm[5] = force_quirk ? -Fx : Fy;
    Fm[6] = -Fy;
    Fm[7] = 2.0f * (Fx * ux - Fy * uy);
    Fm[8] = Fx * uy + Fy * ux;
    float a[9];
    const float inv_norm[9] = {1.0f / 9.0f, 1.0f / 36.0f, 1.0f / 36.0f, 1.0f / 6.0f, 1.0f / 12.0f,
                               1.0f / 6.0f, 1.0f / 12.0f, 0.25f, 0.25f};
#pragma unroll
    for (int k = 0; k < 9; k++) {
        const float mp = m[k] - S[k] * (m[k] - meq[k]) + (1.0f - 0.5f * S[k]) * Fm[k];
        a[k] = mp * inv_norm[k];
    }
    const float base_axis = a[0] - a[1] - 2.0f * a[2];
    const float base_diag = a[0] + 2.0f * a[1] + a[2];
    f[0] = a[0] - 4.0f * a[1] + 4.0f * a[2];
    f[1] = base_axis + a[3] - 2.0f * a[4] + a[7];
    f[2] = base_axis + a[5] - 2.0f * a[6] - a[7];
    f[3] = base_axis - a[3] + 2.0f * a[4] + a[7];
    f[4] = base_axis - a[5] + 2.0f * a[6] - a[7];
    const float px = a[3] + a[4], py = a[5] + a[6];
    f[5] = base_diag + px + py + a[8];
    f[6] = base_diag - px + py - a[8];
    f[7] = base_diag - px - py + a[8];
    f[8] = base_diag + px - py - a[8];
}

// CM<2,Adapter>::apply -- CM.cuh:27-138.  Central moments about the
// force-corrected velocity, De Rosis (2019) forcing, relaxation with S[i]
// or the adapter rate for i > 5, back transform through raw moments.
// `hor` is the higher-order rate (CM_OPT) or negative for NoAdapter.
__device__ __forceinline__ void collide_cm(float f[9], float rho, float ux, float uy, float Fx, float Fy,
                                           const float S[9], float hor) {
    // raw moments of f
    const float m10 = f[1] - f[3] + f[5] - f[6] - f[7] + f[8];
    const float m01 = f[2] - f[4] + f[5] + f[6] - f[7] - f[8];
    const float m20 = f[1] + f[3] + f[5] + f[6] + f[7] + f[8];
    const float m02 = f[2] + f[4] + f[5] + f[6] + f[7] + f[8];
    const float m11 = f[5] - f[6] + f[7] - f[8];
    const float m21 = f[5] + f[6] - f[7] - f[8];
    const float m12 = f[5] - f[6] - f[7] + f[8];
    const float m22 = f[5] + f[6] + f[7] + f[8];
    const float m00 = rho;
    // central moments kappa_ab = sum f (cx-ux)^a (cy-uy)^b
    const float ux2 = ux * ux, uy2 = uy * uy;
    const float k10 = m10 - ux * m00;
    const float k01 = m01 - uy * m00;
    const float k20 = m20 - 2.0f * ux * m10 + ux2 * m00;
    const float k02 = m02 - 2.0f * uy * m01 + uy2 * m00;
    const float k11 = m11 - ux * m01 - uy * m10 + ux * uy * m00;
    const float k21 = m21 - 2.0f * ux * m11 - uy * m20 + ux2 * m01 + 2.0f * ux * uy * m10 - ux2 * uy * m00;
    const float k12 = m12 - 2.0f * uy * m11 - ux * m02 + uy2 * m10 + 2.0f * ux * uy * m01 - ux * uy2 * m00;
    const float k22 = m22 - 2.0f * ux * m12 - 2.0f * uy * m21 + ux2 * m02 + uy2 * m20 + 4.0f * ux * uy * m11
                    - 2.0f * ux * uy2 * m10 - 2.0f * ux2 * uy * m01 + ux2 * uy2 * m00;
    const float cs2 = 1.0f / 3.0f;
    float k[9] = {rho, k10, k01, k20 + k02, k20 - k02, k11, k21, k12, k22};
    const float keq[9] = {rho, 0.f, 0.f, 2.0f * rho * cs2, 0.f, 0.f, 0.f, 0.f, rho * cs2 * cs2};
    const float Fc[9] = {0.f, Fx, Fy, 0.f, 0.f, 0.f, Fy * cs2, Fx * cs2, 0.f};
#pragma unroll
    for (int i = 0; i < 9; i++) {
        const float s = (hor >= 0.0f && i > 5) ? hor : S[i];
        k[i] = k[i] - s * (k[i] - keq[i]) + (1.0f - 0.5f * s) * Fc[i];
    }
    // back to raw moments (binomial shift by +u), then to populations
    const float c00 = k[0], c10 = k[1], c01 = k[2];
    const float c20 = 0.5f * (k[3] + k[4]), c02 = 0.5f * (k[3] - k[4]);
    const float c11 = k[5], c21 = k[6], c12 = k[7], c22 = k[8];
    const float r10 = c10 + ux * c00;
    const float r01 = c01 + uy * c00;
    const float r20 = c20 + 2.0f * ux * c10 + ux2 * c00;
    const float r02 = c02 + 2.0f * uy * c01 + uy2 * c00;
    const float r11 = c11 + ux * c01 + uy * c10 + ux * uy * c00;
    const float r21 = c21 + 2.0f * ux * c11 + uy * c20 + ux2 * c01 + 2.0f * ux * uy * c10 + ux2 * uy * c00;
    const float r12 = c12 + 2.0f * uy * c11 + ux * c02 + uy2 * c10 + 2.0f * ux * uy * c01 + ux * uy2 * c00;
    const float r22 = c22 + 2.0f * ux * c12 + 2.0f * uy * c21 + ux2 * c02 + uy2 * c20 + 4.0f * ux * uy * c11
                    + 2.0f * ux * uy2 * c10 + 2.0f * ux2 * uy * c01 + ux2 * uy2 * c00;
    f[0] = c00 - r20 - r02 + r22;
    f[1] = 0.5f * (r10 + r20 - r12 - r22);
    f[3] = 0.5f * (-r10 + r20 + r12 - r22);
    f[2] = 0.5f * (r01 + r02 - r21 - r22);
    f[4] = 0.5f * (-r01 + r02 + r21 - r22);
    f[5] = 0.25f * (r11 + r21 + r12 + r22);
    f[6] = 0.25f * (-r11 + r21 - r12 + r22);
    f[7] = 0.25f * (r11 - r21 - r12 + r22);
    f[8] = 0.25f * (-r11 - r21 + r12 + r22);
}

// OptimalAdapter::compute_higher_order_relaxation -- adapters.cuh:48-111
// (Li et al. 2020 regression, theta* = (0.0003, -0.00775, 0.00016, 0.0087)).
__device__ __forceinline__ float optimal_rate(float rho, float jmag, float pimag, const float* avg) {
    float ts = 0.0003f * (rho / avg[0]);
    ts += -0.00775f * (jmag / avg[1]);
    ts += 0.00016f * (pimag / avg[2]);
    ts += 0.0087f;
    ts = ts > 0.0f ? ts : 0.005f;
    ts = fminf(ts, 1.5f);
    return 1.0f / (3.0f * ts + 0.5f);
}

}  // namespace lbmx
