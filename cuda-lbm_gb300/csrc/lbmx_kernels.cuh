// lbmx_kernels.cuh -- kernels of the fused D2Q9 step, instantiated once per
// storage type by lbmx_step_{f32,f16,bf16}.cu.
//
// One step of the reference loop (src/main.cu:96-114) becomes:
//   [edge pre-pass]   neighbour data for ZG / pressure / corner boundaries
//   [IBM gather + iterate]  only with markers (lbmx_ibm.cu)
//   [average pre-pass]      only for CM_OPT without lagged averages
//   step kernel: pull post-stream populations (AA pattern), boundary,
//                moments, force correction, collision, store in place.
#pragma once
#include "lbmx_device.cuh"

namespace lbmx {

constexpr int kThreads = kBlockX * kBlockY;

// Six FP64 sums of a block -> partials[block]; the last block to finish
// reduces all partials in a fixed order (deterministic, unlike the
// reference's float atomicAdd in update_avg_mag, macroscopics.cuh:116-118).
__device__ __forceinline__ void block_sums(const StepArgs& a, double v[6], long long n_nodes) {
    __shared__ double sh[kThreads / 32][6];
    __shared__ bool is_last;
    const int tid = threadIdx.y * blockDim.x + threadIdx.x;
    const int lane = tid & 31, warp = tid >> 5;
#pragma unroll
    for (int k = 0; k < 6; k++) {
        double t = v[k];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) t += __shfl_down_sync(0xffffffffu, t, o);
        if (lane == 0) sh[warp][k] = t;
    }
    __syncthreads();
    const unsigned nblocks = gridDim.x * gridDim.y;
    const unsigned bid = blockIdx.y * gridDim.x + blockIdx.x;
    if (tid == 0) {
        double t[6] = {0, 0, 0, 0, 0, 0};
        for (int w = 0; w < kThreads / 32; w++)
            for (int k = 0; k < 6; k++) t[k] += sh[w][k];
        for (int k = 0; k < 6; k++) a.partials[(long long)bid * 6 + k] = t[k];
        __threadfence();
        unsigned done = atomicAdd(a.counter, 1u);
        is_last = (done == nblocks - 1);
    }
    __syncthreads();
    if (!is_last) return;
    __threadfence();
    double t[6] = {0, 0, 0, 0, 0, 0};
    for (unsigned b = tid; b < nblocks; b += kThreads)
        for (int k = 0; k < 6; k++) t[k] += __ldcg(a.partials + (long long)b * 6 + k);
#pragma unroll
    for (int k = 0; k < 6; k++) {
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) t[k] += __shfl_down_sync(0xffffffffu, t[k], o);
    }
    __syncthreads();
    if (lane == 0)
        for (int k = 0; k < 6; k++) sh[warp][k] = t[k];
    __syncthreads();
    if (tid == 0) {
        double s[6] = {0, 0, 0, 0, 0, 0};
        for (int w = 0; w < kThreads / 32; w++)
            for (int k = 0; k < 6; k++) s[k] += sh[w][k];
        if (a.sums)
            for (int k = 0; k < 6; k++) a.sums[k] = s[k];
        if (a.avg_out) {
            a.avg_out[0] = (float)(s[3] / (double)n_nodes);
            a.avg_out[1] = (float)(s[4] / (double)n_nodes);
            a.avg_out[2] = (float)(s[5] / (double)n_nodes);
        }
        *a.counter = 0u;
    }
}

// Post-stream, post-boundary populations of (x, y).
template <typename T>
__device__ __forceinline__ uint8_t gather_node(const StepArgs& a, int x, int y, float f[9], unsigned* outmask) {
    load_post_stream<T>(a, x, y, f, outmask);
    uint8_t fl = 0;
    if (a.flags) {
        fl = a.flags[(long long)y * a.g.pitch + x];
        if (fl) apply_bc(a, f, x, y, fl);
    }
    return fl;
}

__device__ __forceinline__ void node_force(const StepArgs& a, long long off, float* Fx, float* Fy) {
    float fx = a.body_fx, fy = a.body_fy;
    if (a.force) {
        fx = a.force[off];
        fy = a.force[a.g.plane + off];
    }
    if (a.ibm_force) {
        fx += a.ibm_force[off];
        fy += a.ibm_force[a.g.plane + off];
    }
    *Fx = fx;
    *Fy = fy;
}

template <typename T, int OP>
__global__ void __launch_bounds__(kThreads) step_kernel(const StepArgs a) {
    const int x = blockIdx.x * kBlockX + threadIdx.x;
    const int y = blockIdx.y * kBlockY + threadIdx.y;
    double v[6] = {0, 0, 0, 0, 0, 0};
    if (x < a.g.nx && y < a.g.ny) {
        const long long off = (long long)y * a.g.pitch + x;
        float f[9];
        unsigned outmask;
        const uint8_t fl = gather_node<T>(a, x, y, f, &outmask);
        // macroscopics (macroscopics.cu:17-33): rho, j, raw Pi
        float rho = 0.f, jx = 0.f, jy = 0.f;
#pragma unroll
        for (int q = 0; q < 9; q++) {
            rho += f[q];
            jx += (float)CX(q) * f[q];
            jy += (float)CY(q) * f[q];
        }
        float Fx, Fy;
        node_force(a, off, &Fx, &Fy);
        // u = j/rho (macroscopics.cu:30-31), then u += F/(2 rho) (:106-107)
        const float inv = 1.0f / rho;
        const float ux = jx * inv + 0.5f * Fx / rho;
        const float uy = jy * inv + 0.5f * Fy / rho;
        float pimag = 0.f;
        if (OP == LBMX_CM_OPT || a.partials) {
            const float pxx = f[1] + f[3] + f[5] + f[6] + f[7] + f[8];
            const float pyy = f[2] + f[4] + f[5] + f[6] + f[7] + f[8];
            const float pxy = f[5] - f[6] + f[7] - f[8];
            pimag = sqrtf(pxx * pxx + 2.0f * pxy * pxy + pyy * pyy);
        }
        if (a.rho_out) {
            a.rho_out[off] = rho;
            a.u_out[off] = ux;
            a.u_out[a.g.plane + off] = uy;
        }
        if (a.partials) {
            v[0] = rho;
            v[1] = (double)rho * ux;
            v[2] = (double)rho * uy;
            v[3] = rho;
            v[4] = rho * sqrtf(ux * ux + uy * uy);
            v[5] = pimag;
        }
        if (a.error_word && !isfinite(rho)) atomicOr(a.error_word, 1u);
        if (OP == LBMX_BGK) {
            collide_bgk(f, rho, ux, uy, Fx, Fy, a.omega);
        } else if (OP == LBMX_MRT) {
            collide_mrt(f, rho, ux, uy, Fx, Fy, a.S, (a.quirks & LBMX_QUIRK_MRT_FORCE) != 0);
        } else if (OP == LBMX_CM) {
            collide_cm(f, rho, ux, uy, Fx, Fy, a.S, -1.0f);
        } else {
            const float jmag = sqrtf(ux * ux + uy * uy) * rho;
            collide_cm(f, rho, ux, uy, Fx, Fy, a.S, optimal_rate(rho, jmag, pimag, a.avg));
        }
        store_post_collision<T>(a, x, y, f, outmask, fl);
    }
    if (a.partials) block_sums(a, v, (long long)a.g.nx * a.g.ny);
}

// Grid averages <rho>, <rho |u|>, <|Pi|> of the current step before any
// collision (update_avg_mag, macroscopics.cuh:50-120), for CM_OPT.
template <typename T>
__global__ void __launch_bounds__(kThreads) opt_prepass_kernel(const StepArgs a) {
    const int x = blockIdx.x * kBlockX + threadIdx.x;
    const int y = blockIdx.y * kBlockY + threadIdx.y;
    double v[6] = {0, 0, 0, 0, 0, 0};
    if (x < a.g.nx && y < a.g.ny) {
        const long long off = (long long)y * a.g.pitch + x;
        float f[9];
        unsigned outmask;
        gather_node<T>(a, x, y, f, &outmask);
        float rho = 0.f, jx = 0.f, jy = 0.f;
#pragma unroll
        for (int q = 0; q < 9; q++) {
            rho += f[q];
            jx += (float)CX(q) * f[q];
            jy += (float)CY(q) * f[q];
        }
        float Fx, Fy;
        node_force(a, off, &Fx, &Fy);
        const float inv = 1.0f / rho;
        const float ux = jx * inv + 0.5f * Fx / rho;
        const float uy = jy * inv + 0.5f * Fy / rho;
        const float pxx = f[1] + f[3] + f[5] + f[6] + f[7] + f[8];
        const float pyy = f[2] + f[4] + f[5] + f[6] + f[7] + f[8];
        const float pxy = f[5] - f[6] + f[7] - f[8];
        v[3] = rho;
        v[4] = rho * sqrtf(ux * ux + uy * uy);
        v[5] = sqrtf(pxx * pxx + 2.0f * pxy * pxy + pyy * pyy);
    }
    block_sums(a, v, (long long)a.g.nx * a.g.ny);
}

__device__ __forceinline__ void edge_coords(int e, int nx, int ny, int* x, int* y) {
    if (e < nx) { *x = e; *y = 0; }
    else if (e < 2 * nx) { *x = e - nx; *y = ny - 1; }
    else if (e < 2 * nx + ny - 2) { *x = 0; *y = e - 2 * nx + 1; }
    else { *x = nx - 1; *y = e - 2 * nx - (ny - 2) + 1; }
}

// Neighbour data of the boundaries that read another node, taken from the
// post-stream state before any boundary is applied.
template <typename T>
__global__ void edge_prepass_kernel(const StepArgs a, float* aux) {
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= a.g.perimeter) return;
    int x, y;
    edge_coords(e, a.g.nx, a.g.ny, &x, &y);
    const uint8_t fl = a.flags[(long long)y * a.g.pitch + x];
    float* A = aux + (long long)e * 9;
    float f[9];
    unsigned m;
    if (fl == LBMX_ZG_OUTFLOW) {
        int ix = x, iy = y;
        if (x == 0) ix = 1;
        else if (x == a.g.nx - 1) ix = a.g.nx - 2;
        else if (y == 0) iy = 1;
        else iy = a.g.ny - 2;
        load_post_stream<T>(a, ix, iy, f, &m);
#pragma unroll
        for (int q = 0; q < 9; q++) A[q] = f[q];
    } else if (fl == LBMX_PRESSURE_OUTLET) {
        // interior node = node - 1 (pressureOutlet.cuh:12-14); x >= 1 is enforced at set_flags
        load_post_stream<T>(a, x - 1, y, f, &m);
        float r = 0.f, jx = 0.f, jy = 0.f;
#pragma unroll
        for (int q = 0; q < 9; q++) r += f[q];
#pragma unroll
        for (int q = 0; q < 9; q++) {
            jx += f[q] * (float)CX(q);
            jy += f[q] * (float)CY(q);
        }
        A[0] = r;
        A[1] = jx / r;
        A[2] = jy / r;
    } else if (fl == LBMX_REGULARIZED_BOUNCE_BACK_CORNER) {
        int dx = x == 0 ? x + 1 : x - 1;
        int dy = y == 0 ? y + 1 : y - 1;
        dx = max(1, min(dx, a.g.nx - 2));
        dy = max(1, min(dy, a.g.ny - 2));
        load_post_stream<T>(a, dx, dy, f, &m);
        float r = 0.f;
#pragma unroll
        for (int q = 0; q < 9; q++) r += f[q];
        A[0] = r;
    }
}

// f = f_eq(rho, u) in the layout a parity-1 step reads (slot OPP(q) of each
// node), both rest planes and both edge-store parities
// (init_node, src/core/init/init.cuh:12-27).
template <typename T>
__global__ void init_kernel(const StepArgs a, const float* rho_in, const float* u_in, int has_rest_lag) {
    const int x = blockIdx.x * kBlockX + threadIdx.x;
    const int y = blockIdx.y * kBlockY + threadIdx.y;
    if (x >= a.g.nx || y >= a.g.ny) return;
    const long long n = (long long)a.g.nx * a.g.ny;
    const long long dn = (long long)y * a.g.nx + x;
    const long long off = (long long)y * a.g.pitch + x;
    const float rho = rho_in[dn], ux = u_in[dn], uy = u_in[n + dn];
    // second-order equilibrium, bracket in double as equilibrium.cu:13-38 evaluates it
    const float cs = 1.0f / sqrtf(3.0f);
    const float cs2 = cs * cs, cs4 = cs2 * cs2;
    float fe[9];
#pragma unroll
    for (int q = 0; q < 9; q++) {
        const float cu = (float)CX(q) * ux + (float)CY(q) * uy;
        const float uu = ux * ux + uy * uy;
        const double br = 1.0 + 0.5 * (double)cu * (double)cu / (double)cs4 - 0.5 * (double)uu / (double)cs2
                        + (double)cu / (double)cs2;
        fe[q] = (float)((double)(WQ(q) * rho) * br);
    }
    T* F = static_cast<T*>(a.f);
#pragma unroll
    for (int q = 0; q < 9; q++) Store<T>::st(F + OPP(q) * a.g.plane + off, fe[q], WQ(q));
    if (has_rest_lag) Store<T>::st(F + 9 * a.g.plane + off, fe[0], WQ(0));
    if (on_edge(a.g, x, y)) {
        const int e = edge_index(x, y, a.g.nx, a.g.ny);
        for (int p = 0; p < 2; p++)
#pragma unroll
            for (int q = 0; q < 9; q++) a.edge[((long long)p * a.g.perimeter + e) * 9 + q] = fe[q];
    }
    a.rho_out[off] = rho;
    a.u_out[off] = ux;
    a.u_out[a.g.plane + off] = uy;
}

// Canonical post-collision populations of the last step (see lbmx.h).
template <typename T>
__global__ void get_populations_kernel(const StepArgs a, float* out, int last_parity) {
    const int x = blockIdx.x * kBlockX + threadIdx.x;
    const int y = blockIdx.y * kBlockY + threadIdx.y;
    if (x >= a.g.nx || y >= a.g.ny) return;
    const Geometry& g = a.g;
    const long long n = (long long)g.nx * g.ny;
    const long long dn = (long long)y * g.nx + x;
    const T* F = static_cast<const T*>(a.f);
    out[dn] = Store<T>::ld(F + a.rest_plane * g.plane + (long long)y * g.pitch + x, WQ(0));
    const float nan = __int_as_float(0x7fc00000);
#pragma unroll
    for (int q = 1; q < 9; q++) {
        float v;
        if (!last_parity) {
            v = Store<T>::ld(F + OPP(q) * g.plane + (long long)y * g.pitch + x, WQ(q));
        } else {
            int dx = x + CX(q), dy = y + CY(q);
            bool out_d = false;
            if (dx < 0 || dx >= g.nx) { if (g.periodic_x) dx = dx < 0 ? dx + g.nx : dx - g.nx; else out_d = true; }
            if (dy < 0 || dy >= g.ny) { if (g.periodic_y) dy = dy < 0 ? dy + g.ny : dy - g.ny; else out_d = true; }
            if (!out_d) {
                v = Store<T>::ld(F + q * g.plane + (long long)dy * g.pitch + dx, WQ(q));
            } else {
                int sx = x - CX(q), sy = y - CY(q);
                bool out_s = (!g.periodic_x && (sx < 0 || sx >= g.nx)) || (!g.periodic_y && (sy < 0 || sy >= g.ny));
                v = out_s ? a.edge[((long long)1 * g.perimeter + edge_index(x, y, g.nx, g.ny)) * 9 + q] : nan;
            }
        }
        out[q * n + dn] = v;
    }
}

// Density and uncorrected velocity of the IBM patch nodes (the reference
// interpolates from d_rho and the copy of d_u taken before the force
// correction, IBMManager.cuh:227-228).
template <typename T>
__global__ void ibm_gather_kernel(const StepArgs a, const int* patch_nodes, int npatch, float* prho, float* pu) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= npatch) return;
    const int off = patch_nodes[i];
    const int y = off / a.g.pitch, x = off - y * a.g.pitch;
    float f[9];
    unsigned m;
    gather_node<T>(a, x, y, f, &m);
    float rho = 0.f, jx = 0.f, jy = 0.f;
#pragma unroll
    for (int q = 0; q < 9; q++) {
        rho += f[q];
        jx += (float)CX(q) * f[q];
        jy += (float)CY(q) * f[q];
    }
    const float inv = 1.0f / rho;
    prho[i] = rho;
    pu[i] = jx * inv;
    pu[npatch + i] = jy * inv;
}

inline dim3 grid_of(const Geometry& g) {
    return dim3((g.nx + kBlockX - 1) / kBlockX, (g.ny + kBlockY - 1) / kBlockY);
}

template <typename T>
cudaError_t launch_step(const StepArgs& a, int op, cudaStream_t s) {
    const dim3 grid = grid_of(a.g), block(kBlockX, kBlockY);
    switch (op) {
    case LBMX_BGK: step_kernel<T, LBMX_BGK><<<grid, block, 0, s>>>(a); break;
    case LBMX_MRT: step_kernel<T, LBMX_MRT><<<grid, block, 0, s>>>(a); break;
    case LBMX_CM: step_kernel<T, LBMX_CM><<<grid, block, 0, s>>>(a); break;
    default: step_kernel<T, LBMX_CM_OPT><<<grid, block, 0, s>>>(a); break;
    }
    return cudaGetLastError();
}

template <typename T>
cudaError_t launch_opt_prepass(const StepArgs& a, cudaStream_t s) {
    opt_prepass_kernel<T><<<grid_of(a.g), dim3(kBlockX, kBlockY), 0, s>>>(a);
    return cudaGetLastError();
}

template <typename T>
cudaError_t launch_edge_prepass(const StepArgs& a, float* aux, cudaStream_t s) {
    edge_prepass_kernel<T><<<(a.g.perimeter + 127) / 128, 128, 0, s>>>(a, aux);
    return cudaGetLastError();
}

template <typename T>
cudaError_t launch_init(const StepArgs& a, const float* rho, const float* u, cudaStream_t s) {
    init_kernel<T><<<grid_of(a.g), dim3(kBlockX, kBlockY), 0, s>>>(a, rho, u, a.rest_plane == 9 ? 1 : 0);
    return cudaGetLastError();
}

template <typename T>
cudaError_t launch_get_populations(const StepArgs& a, float* out, cudaStream_t s) {
    get_populations_kernel<T><<<grid_of(a.g), dim3(kBlockX, kBlockY), 0, s>>>(a, out, a.parity);
    return cudaGetLastError();
}

template <typename T>
cudaError_t launch_ibm_gather(const StepArgs& a, const int* patch_nodes, int npatch, float* prho, float* pu,
                              cudaStream_t s) {
    if (npatch <= 0) return cudaSuccess;
    ibm_gather_kernel<T><<<(npatch + 127) / 128, 128, 0, s>>>(a, patch_nodes, npatch, prho, pu);
    return cudaGetLastError();
}

#define LBMX_INSTANTIATE(T)                                                                              \
    template cudaError_t launch_step<T>(const StepArgs&, int, cudaStream_t);                             \
    template cudaError_t launch_opt_prepass<T>(const StepArgs&, cudaStream_t);                           \
    template cudaError_t launch_edge_prepass<T>(const StepArgs&, float*, cudaStream_t);                  \
    template cudaError_t launch_init<T>(const StepArgs&, const float*, const float*, cudaStream_t);      \
    template cudaError_t launch_get_populations<T>(const StepArgs&, float*, cudaStream_t);               \
    template cudaError_t launch_ibm_gather<T>(const StepArgs&, const int*, int, float*, float*, cudaStream_t);

}  // namespace lbmx
