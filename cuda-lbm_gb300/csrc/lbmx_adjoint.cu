// lbmx_adjoint.cu -- discrete adjoint of the D2Q9 step (no reference
// counterpart): gradients of an objective built from the step's moments with
// respect to the per-node Brinkman field gamma, the relaxation rate omega and
// the body force, by checkpointed recomputation.
//
// Forward model (the engine's step, written densely with ping-pong buffers,
// populations held as offsets f - w_q in FP32):
//   ps_t[x][q] = pc_{t-1}[x - c_q][q]          streaming (periodic wrap);
//                pc_{t-1}[x][OPP q] - W(OPP q)  half-way wall node, link out
//   fb_t = B(ps_t)                             on-node bounce-back (flag 1)
//   (pc_t, rho_t, u_t) = N(fb_t; gamma, omega, F [, averages_t])
//   J = sum over t >= first, x of w_rho rho + w_x rho u_x + w_y rho u_y
// N is the engine's per-node code: macroscopics, Guo force correction,
// Brinkman drag, collision (BGK, MRT, CM, CM_OPT).
//
// Reverse step t, per node x:
//   mu[q]  = lambda_{t+1}[x + c_q][q]  (the half-way reflection for links
//            that leave a wall node; 0 for links that leave the domain)
//   lambda_t[x][i] = sum_q mu[q] dpc_q/dps_i + sum_m w_m dmoment_m/dps_i
// by reverse mode written out by hand through B and N (adj_node_vjp: one
// pass over the node's values, then their adjoints in reverse order), with
// the parameter gradients of gamma, omega and F.  CM_OPT's rate depends on
// grid averages of the step; their sensitivity is reduced over the grid and
// returned to every node in a second pass (forward-mode tangents,
// lbmx_dual.cuh, of the averages' terms).
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <type_traits>
#include <vector>

#include "lbmx_dual.cuh"

namespace lbmx {
namespace {

// Threads per block of every adjoint kernel; the reverse kernel (about 100
// registers) is bounded to five 128-thread blocks per SM.
constexpr int kAdjBlock = 128;
constexpr int kAdjReverseBlocksPerSm = 5;
constexpr int kTan = 2;  // tangents per pass

struct AdjGeom {
    int nx, ny, px, py;
    long long n;
};

struct AdjArgs {
    AdjGeom g;
    uint32_t quirks;
    float omega;
    float S[9];
    uint32_t omega_mask;  // S entries tied to omega (their common value is the omega of the gradient)
    float fx, fy;         // uniform body force
    float wall_ux, wall_uy;
    const uint8_t* flags;   // [n] or null
    const float* gamma;     // [n] or null
    const float* weights;   // [3][n] objective weights or null
    int drag;               // the objective's node terms are multiplied by the node's gamma
};

__device__ __forceinline__ bool adj_halfway(uint8_t fl) { return fl == LBMX_MOVING_WALL_BB || fl == LBMX_HALFWAY_BB; }

__device__ __forceinline__ float adj_wall_term(const AdjArgs& a, int q, uint8_t fl) {
    if (fl != LBMX_MOVING_WALL_BB) return 0.0f;
    return 6.0f * WQ(q) * ((float)CX(q) * a.wall_ux + (float)CY(q) * a.wall_uy);
}

// node x + s * c_q (wrapped on periodic axes), or -1 outside the domain
__device__ __forceinline__ long long adj_link(const AdjGeom& g, int x, int y, int q, int s) {
    int nx = x + s * CX(q), ny = y + s * CY(q);
    if (nx < 0 || nx >= g.nx) {
        if (!g.px) return -1;
        nx = nx < 0 ? nx + g.nx : nx - g.nx;
    }
    if (ny < 0 || ny >= g.ny) {
        if (!g.py) return -1;
        ny = ny < 0 ? ny + g.ny : ny - g.ny;
    }
    return (long long)ny * g.nx + nx;
}

// post-stream populations of node (x, y) from the previous post-collision state
__device__ __forceinline__ void adj_gather(const AdjArgs& a, const float* pc, int x, int y, long long node, uint8_t fl,
                                           float ps[9]) {
    const long long n = a.g.n;
#pragma unroll
    for (int q = 0; q < 9; q++) {
        const long long s = adj_link(a.g, x, y, q, -1);
        if (s >= 0) ps[q] = pc[q * n + s];
        else if (adj_halfway(fl)) ps[q] = pc[OPP(q) * n + node] - adj_wall_term(a, OPP(q), fl);
        else ps[q] = 0.0f;  // overwritten by the node's bounce-back (checked on the host)
    }
}

// BounceBack<2>::apply as the engine applies it (the domain edge, whatever
// the periodicity, bbDomainBoundary.cuh:26-49)
template <typename R>
__device__ __forceinline__ void adj_bc(const AdjGeom& g, R f[9], int x, int y, uint8_t fl) {
    if (fl != LBMX_BOUNCE_BACK) return;
#pragma unroll
    for (int i = 1; i < 9; i++) {
        const int xn = x + CX(i), yn = y + CY(i);
        if (xn < 0 || xn >= g.nx || yn < 0 || yn >= g.ny) f[OPP(i)] = f[i];
    }
}

// The adjoint carries populations as offsets f - w_q (the engine's 16-bit
// form, here in FP32): at the low Mach numbers of a drag-damped flow, FP32
// then resolves the deviation from rest instead of the weights.  Half-way
// reflection and on-node bounce-back copy between opposite directions, whose
// weights are equal, so they act on offsets unchanged.

// density and force-corrected, Brinkman-corrected velocity, as general_node
template <typename R>
__device__ __forceinline__ void adj_macro(const R f[9], R gm, R& Fx, R& Fy, R& rho, R& drho, R& ux, R& uy) {
    rho = f[0];
    R jx = splat(0.0f, f[0]), jy = splat(0.0f, f[0]);
#pragma unroll
    for (int q = 1; q < 9; q++) {
        rho = rho + f[q];
        if (CX(q) == 1) jx = jx + f[q];
        if (CX(q) == -1) jx = jx - f[q];
        if (CY(q) == 1) jy = jy + f[q];
        if (CY(q) == -1) jy = jy - f[q];
    }
    drho = rho;                    // rho - 1, exactly
    rho = rho + splat(1.0f, rho);  // the weights sum to 1
    const R inv = vdiv(splat(1.0f, rho), rho);
    ux = jx * inv + vdiv(0.5f * Fx, rho);
    uy = jy * inv + vdiv(0.5f * Fy, rho);
    brinkman<R>(gm, rho, ux, uy, Fx, Fy);
}

template <typename R>
__device__ __forceinline__ R adj_pimag(const R f[9]) {
    // sum c_x^2 w = sum c_y^2 w = 1/3
    const R d = (((f[5] + f[6]) + f[7]) + f[8]) + splat(1.0f / 3.0f, f[0]);
    const R pxx = (f[1] + f[3]) + d, pyy = (f[2] + f[4]) + d;
    const R pxy = ((f[5] - f[6]) + f[7]) - f[8];
    return vsqrt(fma(pxx, pxx, fma(2.0f * pxy, pxy, pyy * pyy)));
}

// N: f (post-boundary) -> post-collision; mom = (rho, ux, uy)
template <typename R, int OP>
__device__ __forceinline__ void adj_node(const AdjArgs& a, R f[9], R gm, R Fx, R Fy, R omega, const R S[9],
                                         const R avg[3], R mom[3]) {
    R rho, drho, ux, uy;
    adj_macro<R>(f, gm, Fx, Fy, rho, drho, ux, uy);
    mom[0] = rho;
    mom[1] = ux;
    mom[2] = uy;
    if (OP == LBMX_BGK) {
        collide_bgk<R, true, R>(f, rho, drho, ux, uy, Fx, Fy, omega, true);
    } else if (OP == LBMX_MRT) {
        collide_mrt<R, true, R>(f, rho, drho, ux, uy, Fx, Fy, S, (a.quirks & LBMX_QUIRK_MRT_FORCE) != 0, true);
    } else if (OP == LBMX_CM) {
        collide_cm<R, true, R>(f, rho, drho, ux, uy, Fx, Fy, S, rho, false);
    } else {
        const R pimag = adj_pimag<R>(f);
        const R jmag = vsqrt(fma(ux, ux, uy * uy)) * rho;
        collide_cm<R, true, R>(f, rho, drho, ux, uy, Fx, Fy, S, optimal_rate<R, R>(rho, jmag, pimag, avg), true);
    }
}

// the node's terms of the CM_OPT grid averages: rho, rho |u|, |Pi|
template <typename R>
__device__ __forceinline__ void adj_avg_terms(const R f[9], R gm, R Fx, R Fy, R out[3]) {
    R rho, drho, ux, uy;
    adj_macro<R>(f, gm, Fx, Fy, rho, drho, ux, uy);
    out[0] = rho;
    out[1] = rho * vsqrt(fma(ux, ux, uy * uy));
    out[2] = adj_pimag<R>(f);
}

// deterministic block sums of C values; part[block][C] = (or +=) the sum:
// a fixed shuffle tree within each warp in the values' type (the reverse
// kernel's per-node gradient terms in FP32: the 64-bit pipe is narrow), the
// warps' totals in FP64
template <int C, typename V>
__device__ __forceinline__ void adj_block_sum(const V v[C], double* part, bool add) {
    __shared__ double sh[kAdjBlock / 32][C];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int c = 0; c < C; c++) {
        V t = v[c];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) t += __shfl_down_sync(0xffffffffu, t, o);
        if (lane == 0) sh[warp][c] = (double)t;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int c = 0; c < C; c++) {
            double s = 0.0;
            for (int w = 0; w < kAdjBlock / 32; w++) s += sh[w][c];
            if (add) part[(long long)blockIdx.x * C + c] += s;
            else part[(long long)blockIdx.x * C + c] = s;
        }
    }
}

// ---------------------------------------------------------------- reverse
// The node's vector-Jacobian product in reverse mode, written out by hand
// for BGK, MRT, CM and CM_OPT: one pass over the node's values, then their
// adjoints in reverse order (forward-mode tangents pushed 13 or 16
// directions through the collision, two at a time, 2.5 to 3 times slower).  In: the node's
// post-stream populations ps, its gamma, mu (the adjoints of its
// post-collision populations, centred: their mean c goes through the
// conserved mass, below) and the objective weights w of its moments.  Out:
// lam = d/dps of (mu . pc + objective), and the node's gamma, omega and
// body-force derivatives.

// post-collision adjoints -> moment-space adjoints of CM's back transform
// (raw moments r from central moments c by the binomial shift by +u), the
// collision's adjoints of rho, drho, u, F and S; b_f gets the raw-moment
// part (the populations' own adjoints through m = M f)
__device__ __forceinline__ void vjp_cm(const float f[9], float rho, float drho, float ux, float uy, float Fx, float Fy,
                                       const float S[9], const float mu[9], float b_f[9], float& b_rho, float& b_drho,
                                       float& b_ux, float& b_uy, float& b_Fx, float& b_Fy, float b_S[9]) {
    const float third = 1.0f / 3.0f;
    // forward: raw moments, central moments, relaxed central moments
    const float m10 = (f[1] - f[3]) + ((f[5] + f[8]) - (f[6] + f[7]));
    const float m01 = (f[2] - f[4]) + ((f[5] + f[6]) - (f[7] + f[8]));
    const float m22 = (f[5] + f[6]) + (f[7] + f[8]);
    const float m20 = (f[1] + f[3]) + m22;
    const float m02 = (f[2] + f[4]) + m22;
    const float m11 = (f[5] + f[7]) - (f[6] + f[8]);
    const float m21 = (f[5] + f[6]) - (f[7] + f[8]);
    const float m12 = (f[5] + f[8]) - (f[6] + f[7]);
    const float ux2 = ux * ux, uy2 = uy * uy, uxy = ux * uy;
    const float k10 = m10 - ux * rho;
    const float k01 = m01 - uy * rho;
    const float k20 = m20 - 2.0f * ux * m10 + ux2 * rho;
    const float k02 = m02 - 2.0f * uy * m01 + uy2 * rho;
    const float k11 = m11 - uy * m10 - ux * m01 + uxy * rho;
    const float k21 = m21 - 2.0f * ux * m11 - uy * m20 + ux2 * m01 + 2.0f * uxy * m10 - ux2 * uy * rho - uy * third;
    const float k12 = m12 - 2.0f * uy * m11 - ux * m02 + uy2 * m10 + 2.0f * uxy * m01 - ux * uy2 * rho - ux * third;
    const float k22 = m22 - 2.0f * ux * m12 - 2.0f * uy * m21 + ux2 * m02 + uy2 * m20 + 4.0f * uxy * m11 -
                      2.0f * ux * uy2 * m10 - 2.0f * ux2 * uy * m01 + ux2 * uy2 * rho + (ux2 + uy2) * third;
    const float ksum = k20 + k02, kdiff = k20 - k02;
    const float c10 = (1.0f - S[1]) * k10 + (1.0f - 0.5f * S[1]) * Fx;
    const float c01 = (1.0f - S[2]) * k01 + (1.0f - 0.5f * S[2]) * Fy;
    const float t3 = ksum - S[3] * (ksum - (2.0f * third) * drho);
    const float t4 = (1.0f - S[4]) * kdiff;
    const float c11 = (1.0f - S[5]) * k11;
    const float c21 = (1.0f - S[6]) * k21 + (1.0f - 0.5f * S[6]) * third * Fy;
    const float c12 = (1.0f - S[7]) * k12 + (1.0f - 0.5f * S[7]) * third * Fx;
    const float c20 = 0.5f * (t3 + t4), c02 = 0.5f * (t3 - t4), c00 = rho;
    // reverse: populations <- raw moments (f0 = drho - r20 - r02 + r22, ...)
    const float b_r22 = mu[0] - 0.5f * (mu[1] + mu[3] + mu[2] + mu[4]) + 0.25f * (mu[5] + mu[6] + mu[7] + mu[8]);
    const float b_r20 = 0.5f * (mu[1] + mu[3]) - mu[0];
    const float b_r02 = 0.5f * (mu[2] + mu[4]) - mu[0];
    const float b_r10 = 0.5f * (mu[1] - mu[3]);
    const float b_r01 = 0.5f * (mu[2] - mu[4]);
    const float b_r12 = 0.5f * (mu[3] - mu[1]) + 0.25f * ((mu[5] + mu[8]) - (mu[6] + mu[7]));
    const float b_r21 = 0.5f * (mu[4] - mu[2]) + 0.25f * ((mu[5] + mu[6]) - (mu[7] + mu[8]));
    const float b_r11 = 0.25f * ((mu[5] + mu[7]) - (mu[6] + mu[8]));
    b_drho += mu[0];
    // raw moments <- central moments (shift by +u)
    const float b_c10 = b_r10 + 2.0f * ux * b_r20 + uy * b_r11 + 2.0f * uxy * b_r21 + uy2 * b_r12 + 2.0f * ux * uy2 * b_r22;
    const float b_c01 = b_r01 + 2.0f * uy * b_r02 + ux * b_r11 + ux2 * b_r21 + 2.0f * uxy * b_r12 + 2.0f * ux2 * uy * b_r22;
    const float b_c20 = b_r20 + uy * b_r21 + uy2 * b_r22;
    const float b_c02 = b_r02 + ux * b_r12 + ux2 * b_r22;
    const float b_c11 = b_r11 + 2.0f * ux * b_r21 + 2.0f * uy * b_r12 + 4.0f * uxy * b_r22;
    const float b_c21 = b_r21 + 2.0f * uy * b_r22;
    const float b_c12 = b_r12 + 2.0f * ux * b_r22;
    const float b_c22 = b_r22;
    b_rho += ux * b_r10 + uy * b_r01 + ux2 * b_r20 + uy2 * b_r02 + uxy * b_r11 + ux2 * uy * b_r21 + ux * uy2 * b_r12 +
             ux2 * uy2 * b_r22;
    b_ux += c00 * b_r10 + (2.0f * c10 + 2.0f * ux * c00) * b_r20 + (c01 + uy * c00) * b_r11 +
            (2.0f * c11 + 2.0f * ux * c01 + 2.0f * uy * c10 + 2.0f * uxy * c00) * b_r21 +
            (c02 + 2.0f * uy * c01 + uy2 * c00 + third) * b_r12 +
            (2.0f * c12 + 2.0f * ux * c02 + 4.0f * uy * c11 + 2.0f * uy2 * c10 + 4.0f * uxy * c01 +
             2.0f * ux * uy2 * c00 + 2.0f * ux * third) * b_r22;
    b_uy += c00 * b_r01 + (2.0f * c01 + 2.0f * uy * c00) * b_r02 + (c10 + ux * c00) * b_r11 +
            (c20 + 2.0f * ux * c10 + ux2 * c00 + third) * b_r21 +
            (2.0f * c11 + 2.0f * ux * c01 + 2.0f * uy * c10 + 2.0f * uxy * c00) * b_r12 +
            (2.0f * c21 + 2.0f * uy * c20 + 4.0f * ux * c11 + 4.0f * uxy * c10 + 2.0f * ux2 * c01 +
             2.0f * ux2 * uy * c00 + 2.0f * uy * third) * b_r22;
    // central moments <- relaxation
    const float b_t3 = 0.5f * (b_c20 + b_c02), b_t4 = 0.5f * (b_c20 - b_c02);
    const float b_k10 = (1.0f - S[1]) * b_c10;
    b_S[1] += -(k10 + 0.5f * Fx) * b_c10;
    b_Fx += (1.0f - 0.5f * S[1]) * b_c10;
    const float b_k01 = (1.0f - S[2]) * b_c01;
    b_S[2] += -(k01 + 0.5f * Fy) * b_c01;
    b_Fy += (1.0f - 0.5f * S[2]) * b_c01;
    const float b_ksum = (1.0f - S[3]) * b_t3;
    b_drho += (2.0f * third) * S[3] * b_t3;
    b_S[3] += -(ksum - (2.0f * third) * drho) * b_t3;
    const float b_kdiff = (1.0f - S[4]) * b_t4;
    b_S[4] += -kdiff * b_t4;
    const float b_k20 = b_ksum + b_kdiff, b_k02 = b_ksum - b_kdiff;
    const float b_k11 = (1.0f - S[5]) * b_c11;
    b_S[5] += -k11 * b_c11;
    const float b_k21 = (1.0f - S[6]) * b_c21;
    b_S[6] += -(k21 + (0.5f * third) * Fy) * b_c21;
    b_Fy += (1.0f - 0.5f * S[6]) * third * b_c21;
    const float b_k12 = (1.0f - S[7]) * b_c12;
    b_S[7] += -(k12 + (0.5f * third) * Fx) * b_c12;
    b_Fx += (1.0f - 0.5f * S[7]) * third * b_c12;
    const float b_k22 = (1.0f - S[8]) * b_c22;
    b_drho += (third * third) * S[8] * b_c22;
    b_S[8] += -(k22 - (third * third) * drho) * b_c22;
    // raw moments <- central moments (shift by -u)
    const float b_m10 = b_k10 - 2.0f * ux * b_k20 - uy * b_k11 + 2.0f * uxy * b_k21 + uy2 * b_k12 - 2.0f * ux * uy2 * b_k22;
    const float b_m01 = b_k01 - 2.0f * uy * b_k02 - ux * b_k11 + ux2 * b_k21 + 2.0f * uxy * b_k12 - 2.0f * ux2 * uy * b_k22;
    const float b_m20 = b_k20 - uy * b_k21 + uy2 * b_k22;
    const float b_m02 = b_k02 - ux * b_k12 + ux2 * b_k22;
    const float b_m11 = b_k11 - 2.0f * ux * b_k21 - 2.0f * uy * b_k12 + 4.0f * uxy * b_k22;
    const float b_m21 = b_k21 - 2.0f * uy * b_k22;
    const float b_m12 = b_k12 - 2.0f * ux * b_k22;
    const float b_m22 = b_k22 + b_m20 + b_m02;
    b_rho += -ux * b_k10 - uy * b_k01 + ux2 * b_k20 + uy2 * b_k02 + uxy * b_k11 - ux2 * uy * b_k21 -
             ux * uy2 * b_k12 + ux2 * uy2 * b_k22;
    b_ux += -rho * b_k10 + (2.0f * ux * rho - 2.0f * m10) * b_k20 + (uy * rho - m01) * b_k11 +
            (2.0f * ux * m01 + 2.0f * uy * m10 - 2.0f * m11 - 2.0f * uxy * rho) * b_k21 +
            (2.0f * uy * m01 - m02 - uy2 * rho - third) * b_k12 +
            (2.0f * ux * m02 + 4.0f * uy * m11 - 2.0f * m12 - 2.0f * uy2 * m10 - 4.0f * uxy * m01 +
             2.0f * ux * uy2 * rho + 2.0f * ux * third) * b_k22;
    b_uy += -rho * b_k01 + (2.0f * uy * rho - 2.0f * m01) * b_k02 + (ux * rho - m10) * b_k11 +
            (2.0f * ux * m10 - m20 - ux2 * rho - third) * b_k21 +
            (2.0f * uy * m10 + 2.0f * ux * m01 - 2.0f * m11 - 2.0f * uxy * rho) * b_k12 +
            (2.0f * uy * m20 + 4.0f * ux * m11 - 2.0f * m21 - 4.0f * uxy * m10 - 2.0f * ux2 * m01 +
             2.0f * ux2 * uy * rho + 2.0f * uy * third) * b_k22;
    // populations <- raw moments
    b_f[1] += b_m10 + b_m20;
    b_f[3] += b_m20 - b_m10;
    b_f[2] += b_m01 + b_m02;
    b_f[4] += b_m02 - b_m01;
    b_f[5] += b_m22 + b_m10 + b_m01 + b_m11 + b_m21 + b_m12;
    b_f[6] += b_m22 - b_m10 + b_m01 - b_m11 + b_m21 - b_m12;
    b_f[7] += b_m22 - b_m10 - b_m01 + b_m11 - b_m21 - b_m12;
    b_f[8] += b_m22 + b_m10 - b_m01 - b_m11 - b_m21 + b_m12;
}

// MRT (Lallemand-Luo basis, offset form, forced): as vjp_cm
__device__ __forceinline__ void vjp_mrt(const float f[9], float rho, float drho, float ux, float uy, float Fx, float Fy,
                                        const float S[9], bool quirk, const float mu[9], float b_f[9], float& b_rho,
                                        float& b_drho, float& b_ux, float& b_uy, float& b_Fx, float& b_Fy,
                                        float b_S[9]) {
    const float inv_norm[9] = {1.0f / 9.0f, 1.0f / 36.0f, 1.0f / 36.0f, 1.0f / 6.0f, 1.0f / 12.0f,
                               1.0f / 6.0f, 1.0f / 12.0f, 0.25f, 0.25f};
    // forward: moments, equilibrium moments, force moments
    const float axis = (f[1] + f[2]) + (f[3] + f[4]);
    const float diag = (f[5] + f[6]) + (f[7] + f[8]);
    const float d13 = f[1] - f[3], d24 = f[2] - f[4];
    const float d58 = f[5] + f[8], d67 = f[6] + f[7];
    const float d56 = f[5] + f[6], d78 = f[7] + f[8];
    float m[9], meq[9], Fm[9];
    m[1] = 2.0f * diag - 4.0f * f[0] - axis;
    m[2] = 4.0f * f[0] - 2.0f * axis + diag;
    m[3] = d13 + (d58 - d67);
    m[4] = -2.0f * d13 + (d58 - d67);
    m[5] = d24 + (d56 - d78);
    m[6] = -2.0f * d24 + (d56 - d78);
    m[7] = (f[1] + f[3]) - (f[2] + f[4]);
    m[8] = (f[5] + f[7]) - (f[6] + f[8]);
    const float uu = ux * ux + uy * uy;
    const float rux = rho * ux, ruy = rho * uy;
    meq[1] = 3.0f * rho * uu - 2.0f * drho;
    meq[2] = drho - 3.0f * rho * uu;
    meq[3] = rux;
    meq[4] = -rux;
    meq[5] = ruy;
    meq[6] = -ruy;
    meq[7] = rho * (ux * ux - uy * uy);
    meq[8] = rux * uy;
    const float fu = Fx * ux + Fy * uy;
    Fm[1] = 6.0f * fu;
    Fm[2] = -6.0f * fu;
    Fm[3] = Fx;
    Fm[4] = quirk ? Fy : -Fx;
    Fm[5] = quirk ? -Fx : Fy;
    Fm[6] = -Fy;
    Fm[7] = 2.0f * (Fx * ux - Fy * uy);
    Fm[8] = Fx * uy + Fy * ux;
    // reverse: populations <- scaled post-collision moments a
    float b_a[9];
    const float b_axis_out = (mu[1] + mu[3]) + (mu[2] + mu[4]);
    const float b_diag_out = (mu[5] + mu[6]) + (mu[7] + mu[8]);
    const float b_ax = mu[1] - mu[3], b_ay = mu[2] - mu[4];
    const float b_px = (mu[5] + mu[8]) - (mu[6] + mu[7]), b_py = (mu[5] + mu[6]) - (mu[7] + mu[8]);
    b_a[0] = mu[0] + b_axis_out + b_diag_out;
    b_a[1] = -4.0f * mu[0] - b_axis_out + 2.0f * b_diag_out;
    b_a[2] = 4.0f * mu[0] - 2.0f * b_axis_out + b_diag_out;
    b_a[3] = b_ax + b_px;
    b_a[4] = b_px - 2.0f * b_ax;
    b_a[5] = b_ay + b_py;
    b_a[6] = b_py - 2.0f * b_ay;
    b_a[7] = (mu[1] + mu[3]) - (mu[2] + mu[4]);
    b_a[8] = (mu[5] + mu[7]) - (mu[6] + mu[8]);
    b_drho += b_a[0] * (1.0f / 9.0f);
    // a_k = inv_k ((1 - S_k) m_k + S_k meq_k + (1 - S_k / 2) Fm_k)
    float b_m[9], b_meq[9], b_Fm[9];
#pragma unroll
    for (int k = 1; k < 9; k++) {
        const float b = inv_norm[k] * b_a[k];
        b_m[k] = (1.0f - S[k]) * b;
        b_meq[k] = S[k] * b;
        b_Fm[k] = (1.0f - 0.5f * S[k]) * b;
        b_S[k] += (meq[k] - m[k] - 0.5f * Fm[k]) * b;
    }
    // force moments
    const float b_fu = 6.0f * (b_Fm[1] - b_Fm[2]);
    b_Fx += ux * b_fu + b_Fm[3] + 2.0f * ux * b_Fm[7] + uy * b_Fm[8];
    b_Fy += uy * b_fu - b_Fm[6] - 2.0f * uy * b_Fm[7] + ux * b_Fm[8];
    if (quirk) {
        b_Fy += b_Fm[4];
        b_Fx -= b_Fm[5];
    } else {
        b_Fx -= b_Fm[4];
        b_Fy += b_Fm[5];
    }
    b_ux += Fx * b_fu + 2.0f * Fx * b_Fm[7] + Fy * b_Fm[8];
    b_uy += Fy * b_fu - 2.0f * Fy * b_Fm[7] + Fx * b_Fm[8];
    // equilibrium moments
    const float b_uu = 3.0f * rho * (b_meq[1] - b_meq[2]);
    b_rho += 3.0f * uu * (b_meq[1] - b_meq[2]) + (ux * ux - uy * uy) * b_meq[7];
    b_drho += b_meq[2] - 2.0f * b_meq[1];
    const float b_rux = b_meq[3] - b_meq[4] + uy * b_meq[8];
    const float b_ruy = b_meq[5] - b_meq[6];
    b_uy += rux * b_meq[8];
    b_ux += 2.0f * rho * ux * b_meq[7] + rho * b_rux + 2.0f * ux * b_uu;
    b_uy += -2.0f * rho * uy * b_meq[7] + rho * b_ruy + 2.0f * uy * b_uu;
    b_rho += ux * b_rux + uy * b_ruy;
    // populations <- moments
    const float b_axis = -b_m[1] - 2.0f * b_m[2], b_diag = 2.0f * b_m[1] + b_m[2];
    const float b_d13 = b_m[3] - 2.0f * b_m[4], b_d5867 = b_m[3] + b_m[4];
    const float b_d24 = b_m[5] - 2.0f * b_m[6], b_d5678 = b_m[5] + b_m[6];
    b_f[0] += 4.0f * (b_m[2] - b_m[1]);
    b_f[1] += b_axis + b_d13 + b_m[7];
    b_f[3] += b_axis - b_d13 + b_m[7];
    b_f[2] += b_axis + b_d24 - b_m[7];
    b_f[4] += b_axis - b_d24 - b_m[7];
    b_f[5] += b_diag + b_d5867 + b_d5678 + b_m[8];
    b_f[6] += b_diag - b_d5867 + b_d5678 - b_m[8];
    b_f[7] += b_diag - b_d5867 - b_d5678 + b_m[8];
    b_f[8] += b_diag + b_d5867 - b_d5678 - b_m[8];
}

// BGK (offset form, forced): as vjp_cm; b_om the omega adjoint
__device__ __forceinline__ void vjp_bgk(const float f[9], float rho, float drho, float ux, float uy, float Fx, float Fy,
                                        float omega, const float mu[9], float b_f[9], float& b_rho, float& b_drho,
                                        float& b_ux, float& b_uy, float& b_Fx, float& b_Fy, float& b_om) {
    const float uu = ux * ux + uy * uy;
    const float pref = 1.0f - 0.5f * omega;
    float b_uu = 0.0f, b_pref = 0.0f;
#pragma unroll
    for (int q = 0; q < 9; q++) {
        const float cx = (float)CX(q), cy = (float)CY(q);
        const float cu = cx * ux + cy * uy;
        const float brm1 = cu * (4.5f * cu + 3.0f) - 1.5f * uu;
        const float feq = WQ(q) * (rho * brm1 + drho);
        const float gx = 9.0f * cx * cu + 3.0f * (cx - ux);
        const float gy = 9.0f * cy * cu + 3.0f * (cy - uy);
        // fn = f + omega (feq - f) + w pref (gx Fx + gy Fy)
        const float m = mu[q];
        b_f[q] += (1.0f - omega) * m;
        b_om += (feq - f[q]) * m;
        b_pref += WQ(q) * (gx * Fx + gy * Fy) * m;
        const float b_gx = WQ(q) * pref * Fx * m, b_gy = WQ(q) * pref * Fy * m;
        b_Fx += WQ(q) * pref * gx * m;
        b_Fy += WQ(q) * pref * gy * m;
        const float b_feq = omega * m;
        b_rho += WQ(q) * brm1 * b_feq;
        b_drho += WQ(q) * b_feq;
        const float b_brm1 = WQ(q) * rho * b_feq;
        const float b_cu = (9.0f * cu + 3.0f) * b_brm1 + 9.0f * (cx * b_gx + cy * b_gy);
        b_uu += -1.5f * b_brm1;
        b_ux += cx * b_cu - 3.0f * b_gx;
        b_uy += cy * b_cu - 3.0f * b_gy;
    }
    b_om += -0.5f * b_pref;
    b_ux += 2.0f * ux * b_uu;
    b_uy += 2.0f * uy * b_uu;
}

// The whole node: bounce-back, macroscopics with the Guo and Brinkman
// corrections, collision, objective.  lam[q] = d/dps_q; the parameter
// derivatives are returned through d_gamma, d_omega, d_fx, d_fy, and for
// CM_OPT the derivatives of the node's term by the three grid averages
// through d_avg.
template <int OP>
__device__ __forceinline__ void adj_node_vjp(const AdjArgs& a, int x, int y, uint8_t fl, const float ps[9], float gm,
                                             const float mu[9], float c, const float w[3], const float* avg,
                                             float lam[9], float* d_gamma, float* d_omega, float* d_fx, float* d_fy,
                                             float d_avg[3]) {
    float f[9];
#pragma unroll
    for (int q = 0; q < 9; q++) f[q] = ps[q];
    adj_bc<float>(a.g, f, x, y, fl);
    // macroscopics (adj_macro)
    float drho = f[0], jx = 0.0f, jy = 0.0f;
#pragma unroll
    for (int q = 1; q < 9; q++) {
        drho += f[q];
        if (CX(q) == 1) jx += f[q];
        if (CX(q) == -1) jx -= f[q];
        if (CY(q) == 1) jy += f[q];
        if (CY(q) == -1) jy -= f[q];
    }
    const float rho = drho + 1.0f;
    const float ux0 = (jx + 0.5f * a.fx) / rho, uy0 = (jy + 0.5f * a.fy) / rho;
    const float sc = 1.0f / (0.5f * gm + 1.0f);
    const float ux = ux0 * sc, uy = uy0 * sc;
    const float Fx = a.fx - gm * rho * ux, Fy = a.fy - gm * rho * uy;
    // adjoints
    float b_f[9] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
    float b_S[9] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
    float b_rho = 0.f, b_drho = 0.f, b_ux = 0.f, b_uy = 0.f, b_Fx = 0.f, b_Fy = 0.f, b_om = 0.f, b_gm = 0.f;
    // objective: w0 rho + w1 rho ux + w2 rho uy (drag: times gamma)
    {
        const float gscale = a.drag ? gm : 1.0f;
        b_rho += gscale * (w[0] + w[1] * ux + w[2] * uy);
        b_ux += gscale * w[1] * rho;
        b_uy += gscale * w[2] * rho;
        if (a.drag) b_gm += w[0] * rho + w[1] * rho * ux + w[2] * rho * uy;
    }
    if (OP == LBMX_BGK) {
        vjp_bgk(f, rho, drho, ux, uy, Fx, Fy, a.omega, mu, b_f, b_rho, b_drho, b_ux, b_uy, b_Fx, b_Fy, b_om);
    } else if (OP == LBMX_MRT) {
        vjp_mrt(f, rho, drho, ux, uy, Fx, Fy, a.S, (a.quirks & LBMX_QUIRK_MRT_FORCE) != 0, mu, b_f, b_rho, b_drho,
                b_ux, b_uy, b_Fx, b_Fy, b_S);
    } else if (OP == LBMX_CM) {
        vjp_cm(f, rho, drho, ux, uy, Fx, Fy, a.S, mu, b_f, b_rho, b_drho, b_ux, b_uy, b_Fx, b_Fy, b_S);
    } else {
        // CM_OPT: the higher-order rate hor = 1 / (3 ts + 1/2), ts the
        // clamped regression in rho, |j| = rho |u| and |Pi| over the grid
        // averages (optimal_rate), in place of S[6..8]
        const float d = (((f[5] + f[6]) + f[7]) + f[8]) + 1.0f / 3.0f;
        const float pxx = (f[1] + f[3]) + d, pyy = (f[2] + f[4]) + d;
        const float pxy = ((f[5] - f[6]) + f[7]) - f[8];
        const float pimag = sqrtf(pxx * pxx + 2.0f * pxy * pxy + pyy * pyy);
        const float umag = sqrtf(ux * ux + uy * uy);
        const float jmag = umag * rho;
        const float k0 = 0.0003f / avg[0], k1 = -0.00775f / avg[1], k2 = 0.00016f / avg[2];
        const float ts0 = k0 * rho + k1 * jmag + k2 * pimag + 0.0087f;
        const bool free = ts0 > 0.0f && ts0 <= 1.5f;  // else a constant
        const float ts = ts0 > 0.0f ? fminf(ts0, 1.5f) : 0.005f;
        const float hor = 1.0f / (3.0f * ts + 0.5f);
        float Sh[9];
#pragma unroll
        for (int k = 0; k < 9; k++) Sh[k] = k >= 6 ? hor : a.S[k];
        vjp_cm(f, rho, drho, ux, uy, Fx, Fy, Sh, mu, b_f, b_rho, b_drho, b_ux, b_uy, b_Fx, b_Fy, b_S);
        const float b_hor = b_S[6] + b_S[7] + b_S[8];
        b_S[6] = b_S[7] = b_S[8] = 0.0f;
        const float b_ts = free ? -3.0f * hor * hor * b_hor : 0.0f;
        d_avg[0] = -k0 / avg[0] * rho * b_ts;
        d_avg[1] = -k1 / avg[1] * jmag * b_ts;
        d_avg[2] = -k2 / avg[2] * pimag * b_ts;
        b_rho += k0 * b_ts + umag * k1 * b_ts;
        const float b_umag = rho * k1 * b_ts;
        if (umag > 0.0f) {
            b_ux += ux / umag * b_umag;
            b_uy += uy / umag * b_umag;
        }
        const float b_pimag = k2 * b_ts;
        if (pimag > 0.0f) {
            const float bxx = pxx / pimag * b_pimag, byy = pyy / pimag * b_pimag;
            const float bxy = 2.0f * pxy / pimag * b_pimag;
            const float bd = bxx + byy;
            b_f[1] += bxx;
            b_f[3] += bxx;
            b_f[2] += byy;
            b_f[4] += byy;
            b_f[5] += bd + bxy;
            b_f[6] += bd - bxy;
            b_f[7] += bd + bxy;
            b_f[8] += bd - bxy;
        }
    }
#pragma unroll
    for (int k = 0; k < 9; k++)
        if ((a.omega_mask >> k) & 1u) b_om += b_S[k];
    // Brinkman: F = F0 - gamma rho u, u = sc u0
    float b_fx = b_Fx, b_fy = b_Fy;
    b_gm += -rho * (ux * b_Fx + uy * b_Fy);
    b_rho += -gm * (ux * b_Fx + uy * b_Fy);
    b_ux += -gm * rho * b_Fx;
    b_uy += -gm * rho * b_Fy;
    const float b_ux0 = sc * b_ux, b_uy0 = sc * b_uy;
    b_gm += -0.5f * sc * sc * (ux0 * b_ux + uy0 * b_uy);
    // Guo correction: u0 = (j + F0 / 2) / rho
    const float b_jx = b_ux0 / rho, b_jy = b_uy0 / rho;
    b_fx += 0.5f * b_jx;
    b_fy += 0.5f * b_jy;
    b_rho += -(ux0 * b_jx + uy0 * b_jy);
    b_drho += b_rho;
#pragma unroll
    for (int q = 0; q < 9; q++) b_f[q] += b_drho + (float)CX(q) * b_jx + (float)CY(q) * b_jy;
    // bounce-back: f[OPP i] = f[i] for the links leaving the domain, undone
    // in reverse order; the mean c of the post-collision adjoints goes
    // through the conserved mass, whose derivative is the number of copies
    // of each post-stream population
    float cnt[9] = {1.f, 1.f, 1.f, 1.f, 1.f, 1.f, 1.f, 1.f, 1.f};
    if (fl == LBMX_BOUNCE_BACK) {
#pragma unroll
        for (int i = 8; i >= 1; i--) {
            const int xn = x + CX(i), yn = y + CY(i);
            if (xn < 0 || xn >= a.g.nx || yn < 0 || yn >= a.g.ny) {
                b_f[i] += b_f[OPP(i)];
                b_f[OPP(i)] = 0.0f;
                cnt[i] += cnt[OPP(i)];
                cnt[OPP(i)] = 0.0f;
            }
        }
    }
#pragma unroll
    for (int q = 0; q < 9; q++) lam[q] = fmaf(c, cnt[q], b_f[q]);
    *d_gamma = b_gm;
    *d_omega = b_om;
    *d_fx = b_fx;
    *d_fy = b_fy;
}

__global__ void adj_init_kernel(AdjGeom g, const float* rho, const float* u, float* pc) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= g.n) return;
    float fe[9];
    init_equilibrium<true>(rho[i], u[i], u[g.n + i], fe);
#pragma unroll
    for (int q = 0; q < 9; q++) pc[q * g.n + i] = fe[q];
}

// grid averages of step t (CM_OPT), block sums
__global__ void adj_avg_kernel(const AdjArgs a, const float* pc_prev, double* part) {
    const long long node = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    double v[3] = {0.0, 0.0, 0.0};
    if (node < a.g.n) {
        const int y = (int)(node / a.g.nx), x = (int)(node - (long long)y * a.g.nx);
        const uint8_t fl = a.flags ? a.flags[node] : (uint8_t)0;
        float f[9];
        adj_gather(a, pc_prev, x, y, node, fl, f);
        adj_bc<float>(a.g, f, x, y, fl);
        float t[3];
        adj_avg_terms<float>(f, a.gamma ? a.gamma[node] : 0.0f, a.fx, a.fy, t);
        v[0] = t[0];
        v[1] = t[1];
        v[2] = t[2];
    }
    adj_block_sum<3, double>(v, part, false);
}

// one step forward; the objective terms accumulate per node when `objective`
template <int OP>
__global__ void adj_forward_kernel(const AdjArgs a, const float* pc_prev, float* pc_next, const float* avg,
                                   int objective, double* jnode, float* rho_out, float* u_out) {
    const long long node = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (node >= a.g.n) return;
    const long long n = a.g.n;
    const int y = (int)(node / a.g.nx), x = (int)(node - (long long)y * a.g.nx);
    const uint8_t fl = a.flags ? a.flags[node] : (uint8_t)0;
    float f[9];
    adj_gather(a, pc_prev, x, y, node, fl, f);
    adj_bc<float>(a.g, f, x, y, fl);
    float mom[3];
    const float av[3] = {avg ? avg[0] : 1.0f, avg ? avg[1] : 1.0f, avg ? avg[2] : 1.0f};
    adj_node<float, OP>(a, f, a.gamma ? a.gamma[node] : 0.0f, a.fx, a.fy, a.omega, a.S, av, mom);
#pragma unroll
    for (int q = 0; q < 9; q++) pc_next[q * n + node] = f[q];
    if (objective && a.weights) {
        const double term = (double)a.weights[node] * mom[0] + (double)a.weights[n + node] * (mom[0] * mom[1]) +
                            (double)a.weights[2 * n + node] * (mom[0] * mom[2]);
        jnode[node] += a.drag ? (double)(a.gamma ? a.gamma[node] : 0.0f) * term : term;
    }
    if (rho_out) {
        rho_out[node] = mom[0];
        u_out[node] = mom[1];
        u_out[n + node] = mom[2];
    }
}

// Reverse of step t.  lam_next = lambda_{t+1} (null at the last step);
// writes lambda_t; g_gamma[node] += dJ/dgamma; part[block] += (domega, dFx,
// dFy); CM_OPT: avg_part[block] = this step's sensitivity to the averages.
template <int OP>
__global__ void __launch_bounds__(kAdjBlock, kAdjReverseBlocksPerSm) adj_reverse_kernel(const AdjArgs a, const float* pc_prev,
                                                                const float* lam_next, float* lam_out,
                                                                const float* avg, int objective, double* g_gamma,
                                                                double* part, double* avg_part) {
    const long long node = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    float sums[3] = {0.f, 0.f, 0.f}, asums[3] = {0.f, 0.f, 0.f};
    if (node < a.g.n) {
        const long long n = a.g.n;
        const int y = (int)(node / a.g.nx), x = (int)(node - (long long)y * a.g.nx);
        const uint8_t fl = a.flags ? a.flags[node] : (uint8_t)0;
        float mu[9];
#pragma unroll
        for (int q = 0; q < 9; q++) {
            float m = 0.0f;
            if (lam_next) {
                const long long d = adj_link(a.g, x, y, q, 1);
                if (d >= 0) m = lam_next[q * n + d];
                else if (adj_halfway(fl)) m = lam_next[OPP(q) * n + node];
            }
            mu[q] = m;
        }
        // The collision conserves mass, so a Jacobian column sums to an
        // integer -- 0 for the parameters, 1 (or more where bounce-back copies
        // a population) for a population -- while mu is nearly constant over
        // q.  Propagating mu - mean(mu) and adding mean(mu) times that
        // integer keeps FP32 from cancelling mean(mu) against the rounding
        // of the Jacobian.
        float c = 0.0f;
#pragma unroll
        for (int q = 0; q < 9; q++) c += mu[q];
        c *= 1.0f / 9.0f;
#pragma unroll
        for (int q = 0; q < 9; q++) mu[q] -= c;
        float ps[9];
        adj_gather(a, pc_prev, x, y, node, fl, ps);
        float w[3] = {0.0f, 0.0f, 0.0f};
        if (objective && a.weights) {
            w[0] = a.weights[node];
            w[1] = a.weights[n + node];
            w[2] = a.weights[2 * n + node];
        }
        const float gm = a.gamma ? a.gamma[node] : 0.0f;
        const float av[3] = {avg ? avg[0] : 1.0f, avg ? avg[1] : 1.0f, avg ? avg[2] : 1.0f};
        float lam[9], d_gamma;
        adj_node_vjp<OP>(a, x, y, fl, ps, gm, mu, c, w, av, lam, &d_gamma, &sums[0], &sums[1], &sums[2], asums);
#pragma unroll
        for (int q = 0; q < 9; q++) lam_out[q * n + node] = lam[q];
        g_gamma[node] += d_gamma;
    }
    adj_block_sum<3, float>(sums, part, true);
    if (OP == LBMX_CM_OPT) {
        __syncthreads();
        adj_block_sum<3, float>(asums, avg_part, false);
    }
}

// CM_OPT: lambda_t += (1/N) G . d(terms)/dps with G the reduced sensitivity
__global__ void adj_avg_back_kernel(const AdjArgs a, const float* pc_prev, const double* G, float* lam_out) {
    const long long node = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (node >= a.g.n) return;
    const long long n = a.g.n;
    const int y = (int)(node / a.g.nx), x = (int)(node - (long long)y * a.g.nx);
    const uint8_t fl = a.flags ? a.flags[node] : (uint8_t)0;
    float ps[9];
    adj_gather(a, pc_prev, x, y, node, fl, ps);
    const float inv_n = (float)(1.0 / (double)n);
    const float g0 = (float)G[0] * inv_n, g1 = (float)G[1] * inv_n, g2 = (float)G[2] * inv_n;
    const float gm = a.gamma ? a.gamma[node] : 0.0f;
    using R = Dual<kTan>;
#pragma unroll 1
    for (int p0 = 0; p0 < 9; p0 += kTan) {
        R f[9], t[3];
#pragma unroll
        for (int q = 0; q < 9; q++) {
            f[q] = dconst<kTan>(ps[q]);
#pragma unroll
            for (int k = 0; k < kTan; k++) f[q].d[k] = (p0 + k == q) ? 1.0f : 0.0f;
        }
        adj_bc<R>(a.g, f, x, y, fl);
        adj_avg_terms<R>(f, dconst<kTan>(gm), dconst<kTan>(a.fx), dconst<kTan>(a.fy), t);
#pragma unroll
        for (int k = 0; k < kTan; k++) {
            const int q = p0 + k;
            if (q >= 9) break;
            lam_out[q * n + node] += g0 * t[0].d[k] + g1 * t[1].d[k] + g2 * t[2].d[k];
        }
    }
}

// out[c] = sum over `count` rows of part[row][c] (one block, fixed order)
__global__ void adj_sum_kernel(const double* part, long long count, int C, double* out, int add) {
    __shared__ double sh[kAdjBlock];
    for (int c = 0; c < C; c++) {
        double t = 0.0;
        for (long long r = threadIdx.x; r < count; r += kAdjBlock) t += part[r * C + c];
        sh[threadIdx.x] = t;
        __syncthreads();
        for (int s = kAdjBlock / 2; s > 0; s >>= 1) {
            if ((int)threadIdx.x < s) sh[threadIdx.x] += sh[threadIdx.x + s];
            __syncthreads();
        }
        if (threadIdx.x == 0) out[c] = add ? out[c] + sh[0] : sh[0];
        __syncthreads();
    }
}

__global__ void adj_mean_kernel(const double* s, float* out, double inv) {
    // float means, as the engine's pre-pass stores them
    out[0] = (float)(s[0] * inv);
    out[1] = (float)(s[1] * inv);
    out[2] = (float)(s[2] * inv);
}

__global__ void adj_to_float_kernel(const double* src, float* dst, long long n) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) dst[i] = (float)src[i];
}

}  // namespace
}  // namespace lbmx

using namespace lbmx;

struct lbmx_adjoint {
    lbmx_params p;
    AdjArgs args;
    cudaStream_t stream = nullptr;
    bool own_stream = false;
    long long n = 0;
    int every = 1;          // checkpoint interval
    int T = 0;              // steps of the last forward run
    int first = 1;          // objective sums steps first..T
    uint8_t* flags = nullptr;
    float* gamma = nullptr;
    float* weights = nullptr;
    float* pc0 = nullptr;   // initial post-collision state [9][n]
    float* ping[2] = {nullptr, nullptr};
    float* ckpt = nullptr;  // [ncheck][9][n]
    int ncheck_cap = 0;
    float* seg = nullptr;   // [every + 1][9][n]
    float* lam[2] = {nullptr, nullptr};
    float* avg_hist = nullptr;  // [T + 1][3]
    int avg_cap = 0;
    double* jnode = nullptr;
    double* g_gamma = nullptr;
    double* part = nullptr;     // [blocks][3]
    double* avg_part = nullptr; // [blocks][3]
    double* red = nullptr;      // [8] reductions
    float* rho_out = nullptr;
    float* u_out = nullptr;
    long long blocks = 0;
    bool have_state = false, have_forward = false;
    char err[512] = {0};
};

static char g_adj_err[512];

static lbmx_status afail(lbmx_adjoint* a, lbmx_status code, const char* fmt, ...) {
    char* dst = a ? a->err : g_adj_err;
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(dst, 512, fmt, ap);
    va_end(ap);
    return code;
}

#define ADJ_CUDA(a, call)                                                                            \
    do {                                                                                            \
        cudaError_t e_ = (call);                                                                    \
        if (e_ != cudaSuccess)                                                                      \
            return afail((a), e_ == cudaErrorMemoryAllocation ? LBMX_ERR_OUT_OF_MEMORY : LBMX_ERR_CUDA, \
                         "%s: %s (%s:%d)", #call, cudaGetErrorString(e_), __FILE__, __LINE__);        \
    } while (0)

static void tie_omega(lbmx_adjoint* a) {
    // the S entries equal to omega move with it
    a->args.omega_mask = 0;
    for (int k = 0; k < 9; k++)
        if (a->p.op != LBMX_BGK && a->args.S[k] == a->args.omega) a->args.omega_mask |= 1u << k;
}

// Flags the adjoint can differentiate, and every population a bounce-back
// node reads from outside the domain overwritten from inside it.
static lbmx_status check_flags(lbmx_adjoint* a, const std::vector<uint8_t>& fl) {
    const int nx = a->p.nx, ny = a->p.ny;
    const bool px = a->p.periodic_x, py = a->p.periodic_y;
    auto outside = [&](int x, int y, bool periodic_aware) {
        const bool ox = x < 0 || x >= nx, oy = y < 0 || y >= ny;
        return periodic_aware ? ((ox && !px) || (oy && !py)) : (ox || oy);
    };
    for (int y = 0; y < ny; y++)
        for (int x = 0; x < nx; x++) {
            const uint8_t f = fl[(size_t)y * nx + x];
            if (f != LBMX_FLUID && f != LBMX_BOUNCE_BACK && f != LBMX_HALFWAY_BB && f != LBMX_MOVING_WALL_BB)
                return afail(a, LBMX_ERR_UNSUPPORTED,
                             "lbmx_adjoint: flag %d at (%d,%d) is not differentiated (fluid, bounce-back and half-way "
                             "walls are)", f, x, y);
            bool known[9];
            bool any_out = false;
            for (int q = 0; q < 9; q++) {
                known[q] = !outside(x - CX(q), y - CY(q), true);
                any_out |= !known[q];
            }
            if (!any_out || f == LBMX_HALFWAY_BB || f == LBMX_MOVING_WALL_BB) continue;
            if (f == LBMX_FLUID)
                return afail(a, LBMX_ERR_UNSUPPORTED,
                             "lbmx_adjoint: fluid node (%d,%d) on a non-periodic edge reads undefined populations", x, y);
            for (int i = 1; i < 9; i++)
                if (outside(x + CX(i), y + CY(i), false)) known[OPP(i)] = known[i];
            for (int q = 0; q < 9; q++)
                if (!known[q])
                    return afail(a, LBMX_ERR_UNSUPPORTED,
                                 "lbmx_adjoint: bounce-back node (%d,%d) keeps a population from outside the domain "
                                 "(use half-way walls there)", x, y);
        }
    return LBMX_OK;
}

template <typename Fn>
static cudaError_t op_dispatch(int op, Fn fn) {
    switch (op) {
    case LBMX_BGK: return fn(std::integral_constant<int, LBMX_BGK>());
    case LBMX_MRT: return fn(std::integral_constant<int, LBMX_MRT>());
    case LBMX_CM: return fn(std::integral_constant<int, LBMX_CM>());
    default: return fn(std::integral_constant<int, LBMX_CM_OPT>());
    }
}

static unsigned grid_of(long long n) { return (unsigned)((n + kAdjBlock - 1) / kAdjBlock); }

// averages of step t (CM_OPT) into avg_hist[t]
static lbmx_status step_averages(lbmx_adjoint* a, const float* pc_prev, int t) {
    adj_avg_kernel<<<grid_of(a->n), kAdjBlock, 0, a->stream>>>(a->args, pc_prev, a->avg_part);
    ADJ_CUDA(a, cudaGetLastError());
    adj_sum_kernel<<<1, kAdjBlock, 0, a->stream>>>(a->avg_part, a->blocks, 3, a->red, 0);
    ADJ_CUDA(a, cudaGetLastError());
    adj_mean_kernel<<<1, 1, 0, a->stream>>>(a->red, a->avg_hist + (size_t)3 * t, 1.0 / (double)a->n);
    ADJ_CUDA(a, cudaGetLastError());
    return LBMX_OK;
}

static lbmx_status forward_step(lbmx_adjoint* a, const float* prev, float* next, int t, bool objective,
                                bool store) {
    const bool opt = a->p.op == LBMX_CM_OPT;
    if (opt) {
        lbmx_status st = step_averages(a, prev, t);
        if (st != LBMX_OK) return st;
    }
    const float* avg = opt ? a->avg_hist + (size_t)3 * t : nullptr;
    ADJ_CUDA(a, op_dispatch(a->p.op, [&](auto opc) {
                 adj_forward_kernel<decltype(opc)::value><<<grid_of(a->n), kAdjBlock, 0, a->stream>>>(
                     a->args, prev, next, avg, objective ? 1 : 0, a->jnode, store ? a->rho_out : nullptr,
                     store ? a->u_out : nullptr);
                 return cudaGetLastError();
             }));
    return LBMX_OK;
}

extern "C" {

void lbmx_adjoint_destroy(lbmx_adjoint* a) {
    if (!a) return;
    int cur = 0;
    cudaGetDevice(&cur);
    cudaSetDevice(a->p.device);
    if (a->stream) cudaStreamSynchronize(a->stream);
    cudaFree(a->flags); cudaFree(a->gamma); cudaFree(a->weights); cudaFree(a->pc0);
    cudaFree(a->ping[0]); cudaFree(a->ping[1]); cudaFree(a->ckpt); cudaFree(a->seg);
    cudaFree(a->lam[0]); cudaFree(a->lam[1]); cudaFree(a->avg_hist); cudaFree(a->jnode);
    cudaFree(a->g_gamma); cudaFree(a->part); cudaFree(a->avg_part); cudaFree(a->red);
    cudaFree(a->rho_out); cudaFree(a->u_out);
    if (a->own_stream && a->stream) cudaStreamDestroy(a->stream);
    cudaSetDevice(cur);
    delete a;
}

lbmx_status lbmx_adjoint_create(const lbmx_params* p, const uint8_t* flags, int32_t checkpoint_every,
                                lbmx_adjoint** out) {
    if (!out) return afail(nullptr, LBMX_ERR_INVALID_ARGUMENT, "lbmx_adjoint_create: out is NULL");
    *out = nullptr;
    if (!p) return afail(nullptr, LBMX_ERR_INVALID_ARGUMENT, "lbmx_adjoint_create: params is NULL");
    if (p->nx < 3 || p->ny < 3 || (long long)p->nx * p->ny > (1LL << 31) - 1)
        return afail(nullptr, LBMX_ERR_INVALID_ARGUMENT, "lbmx_adjoint_create: bad lattice %d x %d", p->nx, p->ny);
    if (p->op < LBMX_BGK || p->op > LBMX_CM_OPT)
        return afail(nullptr, LBMX_ERR_INVALID_ARGUMENT, "lbmx_adjoint_create: unknown operator %d", p->op);
    if (p->storage != LBMX_STORAGE_F32)
        return afail(nullptr, LBMX_ERR_UNSUPPORTED, "lbmx_adjoint_create: the adjoint runs FP32 populations");
    if (p->quirks & (LBMX_QUIRK_REST_LAG | LBMX_QUIRK_IBM_2X2 | LBMX_QUIRK_IBM_CLAMP))
        return afail(nullptr, LBMX_ERR_UNSUPPORTED,
                     "lbmx_adjoint_create: quirks other than MRT_FORCE / ZOUHE_LEFT are not differentiated");
    if (checkpoint_every < 1)
        return afail(nullptr, LBMX_ERR_INVALID_ARGUMENT, "lbmx_adjoint_create: checkpoint_every < 1");
    if (cudaSetDevice(p->device) != cudaSuccess)
        return afail(nullptr, LBMX_ERR_CUDA, "lbmx_adjoint_create: cannot select device %d", p->device);
    lbmx_adjoint* a = new lbmx_adjoint();
    a->p = *p;
    a->n = (long long)p->nx * p->ny;
    a->every = checkpoint_every;
    a->blocks = grid_of(a->n);
    memset(&a->args, 0, sizeof(a->args));
    a->args.g = AdjGeom{p->nx, p->ny, p->periodic_x ? 1 : 0, p->periodic_y ? 1 : 0, a->n};
    a->args.quirks = p->quirks;
    a->args.omega = p->omega;
    for (int k = 0; k < 9; k++) a->args.S[k] = p->S[k];
    a->args.fx = p->body_fx;
    a->args.fy = p->body_fy;
    a->args.wall_ux = p->wall_ux;
    a->args.wall_uy = p->wall_uy;
    tie_omega(a);
    std::vector<uint8_t> fl((size_t)a->n, 0);
    if (flags && cudaMemcpy(fl.data(), flags, fl.size(), cudaMemcpyDefault) != cudaSuccess) {
        delete a;
        return afail(nullptr, LBMX_ERR_CUDA, "lbmx_adjoint_create: cannot read the flags");
    }
    if (check_flags(a, fl) != LBMX_OK) {
        afail(nullptr, LBMX_ERR_UNSUPPORTED, "%s", a->err);
        delete a;
        return LBMX_ERR_UNSUPPORTED;
    }
    auto bail = [&](const char* what) {
        afail(nullptr, LBMX_ERR_OUT_OF_MEMORY, "lbmx_adjoint_create: %s", what);
        lbmx_adjoint_destroy(a);
        return LBMX_ERR_OUT_OF_MEMORY;
    };
    const size_t state = (size_t)9 * a->n * sizeof(float);
    if (cudaMalloc((void**)&a->flags, (size_t)a->n) != cudaSuccess ||
        cudaMalloc((void**)&a->pc0, state) != cudaSuccess || cudaMalloc((void**)&a->ping[0], state) != cudaSuccess ||
        cudaMalloc((void**)&a->ping[1], state) != cudaSuccess ||
        cudaMalloc((void**)&a->jnode, (size_t)a->n * sizeof(double)) != cudaSuccess ||
        cudaMalloc((void**)&a->part, (size_t)a->blocks * 3 * sizeof(double)) != cudaSuccess ||
        cudaMalloc((void**)&a->avg_part, (size_t)a->blocks * 3 * sizeof(double)) != cudaSuccess ||
        cudaMalloc((void**)&a->red, 8 * sizeof(double)) != cudaSuccess ||
        cudaMalloc((void**)&a->rho_out, (size_t)a->n * sizeof(float)) != cudaSuccess ||
        cudaMalloc((void**)&a->u_out, (size_t)2 * a->n * sizeof(float)) != cudaSuccess)
        return bail("cudaMalloc failed");
    if (p->stream) {
        a->stream = (cudaStream_t)p->stream;
    } else {
        if (cudaStreamCreateWithFlags(&a->stream, cudaStreamNonBlocking) != cudaSuccess) return bail("no stream");
        a->own_stream = true;
    }
    cudaMemcpy(a->flags, fl.data(), fl.size(), cudaMemcpyHostToDevice);
    a->args.flags = a->flags;
    *out = a;
    return LBMX_OK;
}

lbmx_status lbmx_adjoint_set_state(lbmx_adjoint* a, const float* rho, const float* u) {
    if (!a || !rho || !u) return afail(a, LBMX_ERR_INVALID_ARGUMENT, "lbmx_adjoint_set_state: NULL argument");
    cudaSetDevice(a->p.device);
    float* tmp = nullptr;
    ADJ_CUDA(a, cudaMalloc((void**)&tmp, (size_t)3 * a->n * sizeof(float)));
    cudaMemcpyAsync(tmp, rho, (size_t)a->n * sizeof(float), cudaMemcpyDefault, a->stream);
    cudaMemcpyAsync(tmp + a->n, u, (size_t)2 * a->n * sizeof(float), cudaMemcpyDefault, a->stream);
    adj_init_kernel<<<grid_of(a->n), kAdjBlock, 0, a->stream>>>(a->args.g, tmp, tmp + a->n, a->pc0);
    const cudaError_t e = cudaStreamSynchronize(a->stream);
    cudaFree(tmp);
    ADJ_CUDA(a, e);
    a->have_state = true;
    a->have_forward = false;
    return LBMX_OK;
}

lbmx_status lbmx_adjoint_set_gamma(lbmx_adjoint* a, const float* gamma) {
    if (!a) return afail(a, LBMX_ERR_INVALID_ARGUMENT, "lbmx_adjoint_set_gamma: NULL handle");
    cudaSetDevice(a->p.device);
    if (!gamma) {
        cudaFree(a->gamma);
        a->gamma = nullptr;
    } else {
        if (!a->gamma) ADJ_CUDA(a, cudaMalloc((void**)&a->gamma, (size_t)a->n * sizeof(float)));
        ADJ_CUDA(a, cudaMemcpyAsync(a->gamma, gamma, (size_t)a->n * sizeof(float), cudaMemcpyDefault, a->stream));
        ADJ_CUDA(a, cudaStreamSynchronize(a->stream));
    }
    a->args.gamma = a->gamma;
    a->have_forward = false;
    return LBMX_OK;
}

lbmx_status lbmx_adjoint_set_scalars(lbmx_adjoint* a, float omega, float fx, float fy) {
    if (!a) return afail(a, LBMX_ERR_INVALID_ARGUMENT, "lbmx_adjoint_set_scalars: NULL handle");
    for (int k = 0; k < 9; k++)
        if ((a->args.omega_mask >> k) & 1u) a->args.S[k] = omega;
    a->args.omega = omega;
    a->args.fx = fx;
    a->args.fy = fy;
    a->have_forward = false;
    return LBMX_OK;
}

lbmx_status lbmx_adjoint_set_objective(lbmx_adjoint* a, const float* weights, int32_t first_step) {
    if (!a || !weights) return afail(a, LBMX_ERR_INVALID_ARGUMENT, "lbmx_adjoint_set_objective: NULL argument");
    if (first_step < 1) return afail(a, LBMX_ERR_INVALID_ARGUMENT, "lbmx_adjoint_set_objective: first_step < 1");
    cudaSetDevice(a->p.device);
    if (!a->weights) ADJ_CUDA(a, cudaMalloc((void**)&a->weights, (size_t)3 * a->n * sizeof(float)));
    ADJ_CUDA(a, cudaMemcpyAsync(a->weights, weights, (size_t)3 * a->n * sizeof(float), cudaMemcpyDefault, a->stream));
    ADJ_CUDA(a, cudaStreamSynchronize(a->stream));
    a->args.weights = a->weights;
    a->args.drag = 0;
    a->first = first_step;
    a->have_forward = false;
    return LBMX_OK;
}

lbmx_status lbmx_adjoint_set_objective_ex(lbmx_adjoint* a, const float* weights, int32_t first_step, int32_t kind) {
    if (!a) return afail(a, LBMX_ERR_INVALID_ARGUMENT, "lbmx_adjoint_set_objective_ex: NULL handle");
    if (kind != LBMX_OBJECTIVE_MOMENTS && kind != LBMX_OBJECTIVE_BRINKMAN_DRAG)
        return afail(a, LBMX_ERR_INVALID_ARGUMENT, "lbmx_adjoint_set_objective_ex: kind %d", kind);
    const lbmx_status st = lbmx_adjoint_set_objective(a, weights, first_step);
    if (st != LBMX_OK) return st;
    a->args.drag = kind == LBMX_OBJECTIVE_BRINKMAN_DRAG ? 1 : 0;
    return LBMX_OK;
}

lbmx_status lbmx_adjoint_forward(lbmx_adjoint* a, int32_t nsteps, double* objective) {
    if (!a) return afail(a, LBMX_ERR_INVALID_ARGUMENT, "lbmx_adjoint_forward: NULL handle");
    if (!a->have_state) return afail(a, LBMX_ERR_NOT_INITIALIZED, "lbmx_adjoint_forward: call lbmx_adjoint_set_state first");
    if (nsteps < 1) return afail(a, LBMX_ERR_INVALID_ARGUMENT, "lbmx_adjoint_forward: nsteps < 1");
    cudaSetDevice(a->p.device);
    const size_t state = (size_t)9 * a->n;
    const int ncheck = (nsteps + a->every - 1) / a->every;  // states at t = 0, every, 2 every, ...
    if (ncheck > a->ncheck_cap) {
        cudaFree(a->ckpt);
        a->ckpt = nullptr;
        ADJ_CUDA(a, cudaMalloc((void**)&a->ckpt, (size_t)ncheck * state * sizeof(float)));
        a->ncheck_cap = ncheck;
    }
    if (nsteps + 1 > a->avg_cap) {
        cudaFree(a->avg_hist);
        a->avg_hist = nullptr;
        ADJ_CUDA(a, cudaMalloc((void**)&a->avg_hist, (size_t)3 * (nsteps + 1) * sizeof(float)));
        a->avg_cap = nsteps + 1;
    }
    ADJ_CUDA(a, cudaMemsetAsync(a->jnode, 0, (size_t)a->n * sizeof(double), a->stream));
    ADJ_CUDA(a, cudaMemcpyAsync(a->ping[0], a->pc0, state * sizeof(float), cudaMemcpyDeviceToDevice, a->stream));
    int cur = 0;
    for (int t = 1; t <= nsteps; t++) {
        if ((t - 1) % a->every == 0)
            ADJ_CUDA(a, cudaMemcpyAsync(a->ckpt + (size_t)((t - 1) / a->every) * state, a->ping[cur],
                                        state * sizeof(float), cudaMemcpyDeviceToDevice, a->stream));
        lbmx_status st = forward_step(a, a->ping[cur], a->ping[cur ^ 1], t, t >= a->first, t == nsteps);
        if (st != LBMX_OK) return st;
        cur ^= 1;
    }
    adj_sum_kernel<<<1, kAdjBlock, 0, a->stream>>>(a->jnode, a->n, 1, a->red, 0);
    ADJ_CUDA(a, cudaGetLastError());
    double J = 0.0;
    ADJ_CUDA(a, cudaMemcpyAsync(&J, a->red, sizeof(double), cudaMemcpyDeviceToHost, a->stream));
    ADJ_CUDA(a, cudaStreamSynchronize(a->stream));
    if (objective) *objective = J;
    a->T = nsteps;
    a->have_forward = true;
    return LBMX_OK;
}

lbmx_status lbmx_adjoint_backward(lbmx_adjoint* a, float* grad_gamma, double* grad_scalars) {
    if (!a) return afail(a, LBMX_ERR_INVALID_ARGUMENT, "lbmx_adjoint_backward: NULL handle");
    if (!a->have_forward)
        return afail(a, LBMX_ERR_NOT_INITIALIZED, "lbmx_adjoint_backward: run lbmx_adjoint_forward with these inputs first");
    cudaSetDevice(a->p.device);
    const size_t state = (size_t)9 * a->n;
    if (!a->seg) ADJ_CUDA(a, cudaMalloc((void**)&a->seg, (size_t)(a->every + 1) * state * sizeof(float)));
    if (!a->lam[0]) {
        ADJ_CUDA(a, cudaMalloc((void**)&a->lam[0], state * sizeof(float)));
        ADJ_CUDA(a, cudaMalloc((void**)&a->lam[1], state * sizeof(float)));
    }
    if (!a->g_gamma) ADJ_CUDA(a, cudaMalloc((void**)&a->g_gamma, (size_t)a->n * sizeof(double)));
    ADJ_CUDA(a, cudaMemsetAsync(a->g_gamma, 0, (size_t)a->n * sizeof(double), a->stream));
    ADJ_CUDA(a, cudaMemsetAsync(a->part, 0, (size_t)a->blocks * 3 * sizeof(double), a->stream));
    const bool opt = a->p.op == LBMX_CM_OPT;
    const int T = a->T;
    const int ncheck = (T + a->every - 1) / a->every;
    int li = 0;
    bool first_rev = true;
    for (int c = ncheck - 1; c >= 0; c--) {
        const int t0 = c * a->every, t1 = std::min(T, t0 + a->every);
        // recompute the segment's states pc_t0 .. pc_t1
        ADJ_CUDA(a, cudaMemcpyAsync(a->seg, a->ckpt + (size_t)c * state, state * sizeof(float),
                                    cudaMemcpyDeviceToDevice, a->stream));
        for (int t = t0 + 1; t <= t1; t++) {
            const float* avg = opt ? a->avg_hist + (size_t)3 * t : nullptr;
            const float* prev = a->seg + (size_t)(t - 1 - t0) * state;
            float* next = a->seg + (size_t)(t - t0) * state;
            ADJ_CUDA(a, op_dispatch(a->p.op, [&](auto opc) {
                         adj_forward_kernel<decltype(opc)::value><<<grid_of(a->n), kAdjBlock, 0, a->stream>>>(
                             a->args, prev, next, avg, 0, nullptr, nullptr, nullptr);
                         return cudaGetLastError();
                     }));
        }
        for (int t = t1; t > t0; t--) {
            const float* prev = a->seg + (size_t)(t - 1 - t0) * state;
            const float* avg = opt ? a->avg_hist + (size_t)3 * t : nullptr;
            const float* lam_next = first_rev ? nullptr : a->lam[li];
            float* lam_out = a->lam[li ^ 1];
            const int objective = t >= a->first ? 1 : 0;
            ADJ_CUDA(a, op_dispatch(a->p.op, [&](auto opc) {
                         adj_reverse_kernel<decltype(opc)::value><<<grid_of(a->n), kAdjBlock, 0, a->stream>>>(
                             a->args, prev, lam_next, lam_out, avg, objective, a->g_gamma, a->part, a->avg_part);
                         return cudaGetLastError();
                     }));
            if (opt) {
                adj_sum_kernel<<<1, kAdjBlock, 0, a->stream>>>(a->avg_part, a->blocks, 3, a->red + 4, 0);
                ADJ_CUDA(a, cudaGetLastError());
                adj_avg_back_kernel<<<grid_of(a->n), kAdjBlock, 0, a->stream>>>(a->args, prev, a->red + 4, lam_out);
                ADJ_CUDA(a, cudaGetLastError());
            }
            li ^= 1;
            first_rev = false;
        }
    }
    adj_sum_kernel<<<1, kAdjBlock, 0, a->stream>>>(a->part, a->blocks, 3, a->red, 0);
    ADJ_CUDA(a, cudaGetLastError());
    double g3[3];
    ADJ_CUDA(a, cudaMemcpyAsync(g3, a->red, sizeof(g3), cudaMemcpyDeviceToHost, a->stream));
    if (grad_gamma) {
        float* tmp = a->lam[li ^ 1];  // free scratch
        adj_to_float_kernel<<<grid_of(a->n), kAdjBlock, 0, a->stream>>>(a->g_gamma, tmp, a->n);
        ADJ_CUDA(a, cudaGetLastError());
        ADJ_CUDA(a, cudaMemcpyAsync(grad_gamma, tmp, (size_t)a->n * sizeof(float), cudaMemcpyDefault, a->stream));
    }
    ADJ_CUDA(a, cudaStreamSynchronize(a->stream));
    if (grad_scalars) {
        grad_scalars[0] = g3[0];
        grad_scalars[1] = g3[1];
        grad_scalars[2] = g3[2];
    }
    return LBMX_OK;
}

lbmx_status lbmx_adjoint_moments(lbmx_adjoint* a, float* rho, float* u) {
    if (!a) return afail(a, LBMX_ERR_INVALID_ARGUMENT, "lbmx_adjoint_moments: NULL handle");
    if (!a->have_forward) return afail(a, LBMX_ERR_NOT_INITIALIZED, "lbmx_adjoint_moments: no forward run");
    cudaSetDevice(a->p.device);
    if (rho) ADJ_CUDA(a, cudaMemcpyAsync(rho, a->rho_out, (size_t)a->n * sizeof(float), cudaMemcpyDefault, a->stream));
    if (u) ADJ_CUDA(a, cudaMemcpyAsync(u, a->u_out, (size_t)2 * a->n * sizeof(float), cudaMemcpyDefault, a->stream));
    ADJ_CUDA(a, cudaStreamSynchronize(a->stream));
    return LBMX_OK;
}

const char* lbmx_adjoint_last_error(lbmx_adjoint* a) { return a ? a->err : g_adj_err; }

}  // extern "C"
