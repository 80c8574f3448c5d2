// lbmx_tangent.cu -- tangent-linear (forward-mode) derivative of a run with
// respect to one scalar parameter: the inlet velocity u_bc, omega, the body
// force's x component or the moving wall's x velocity (no reference
// counterpart).
//
// Every value of the step carries one directional derivative (Dual<1>,
// lbmx_dual.cuh) through the engine's own templated per-node code: the
// Zou-He and bounce-back functors, the Guo-forced collision operators and the
// multi-direct IBM rounds (lbmx_ibm.cuh).  For one scalar input this gives
// the same exact derivative of the discrete model that an adjoint gives, for
// any number of outputs -- here the drag and lift of every step -- at the cost
// of one forward run with twice the state, and without checkpoints.
//
// The step is written densely with ping-pong buffers holding each node's
// post-collision populations (value planes [9][n], then tangent planes
// [9][n]).  Step t reads step t-1's buffer and overwrites step t-2's:
//   f_t[x][q] = pc_{t-1}[x - c_q][q]           upstream node in the domain
//             = pc_{t-1}[x][OPP q] - W(OPP q)  half-way wall node
//             = pc_{t-2}[x][q]                 upstream outside the domain:
// the population the reference's ping-pong buffer still holds there
// (streaming.cu:20-21 skips it), as the engine's edge store reproduces it.
// With LBMX_QUIRK_REST_LAG the rest population also comes from pc_{t-2}.
#include <cuda_runtime.h>

#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <type_traits>
#include <vector>

#include "lbmx_handle.h"
#include "lbmx_ibm.cuh"

namespace lbmx {
namespace {

using D = Dual<1>;
constexpr int kTanBX = 32, kTanBY = 4;

struct TanArgs {
    Geometry g;          // nx, ny, periodic_x, periodic_y (dense: pitch = nx)
    long long n;
    uint32_t quirks;
    int param;           // LBMX_TANGENT_*
    float omega;
    float S[9];
    uint32_t omega_mask; // S entries tied to omega
    float u_bc, rho_out_bc, wall_ux, wall_uy, fx, fy;
    int forced;
    const uint8_t* flags;  // [n]
    const D* ibm_force;    // [2][n] or null
};

__device__ __forceinline__ D dual(float v, bool seeded) { return D{v, {seeded ? 1.0f : 0.0f}}; }
__device__ __forceinline__ D load(const float* buf, long long n, int q, long long node) {
    return D{buf[q * n + node], {buf[(9 + q) * n + node]}};
}
__device__ __forceinline__ void put(float* buf, long long n, int q, long long node, const D& v) {
    buf[q * n + node] = v.v;
    buf[(9 + q) * n + node] = v.d[0];
}

// node x + s * c_q (wrapped on periodic axes), or -1 outside the domain
__device__ __forceinline__ long long tan_link(const TanArgs& a, int x, int y, int q, int s) {
    int nx = x + s * CX(q), ny = y + s * CY(q);
    if (nx < 0 || nx >= a.g.nx) {
        if (!a.g.periodic_x) return -1;
        nx = nx < 0 ? nx + a.g.nx : nx - a.g.nx;
    }
    if (ny < 0 || ny >= a.g.ny) {
        if (!a.g.periodic_y) return -1;
        ny = ny < 0 ? ny + a.g.ny : ny - a.g.ny;
    }
    return (long long)ny * a.g.nx + nx;
}

// post-stream, post-boundary populations of (x, y)
__device__ __forceinline__ void tan_gather(const TanArgs& a, const float* pin, const float* pout, int x, int y,
                                           long long node, uint8_t fl, D f[9]) {
    const long long n = a.n;
    f[0] = load((a.quirks & LBMX_QUIRK_REST_LAG) ? pout : pin, n, 0, node);
    const bool hw = fl == LBMX_MOVING_WALL_BB || fl == LBMX_HALFWAY_BB;
#pragma unroll
    for (int q = 1; q < 9; q++) {
        const long long s = tan_link(a, x, y, q, -1);
        if (s >= 0) {
            f[q] = load(pin, n, q, s);
        } else if (hw) {
            f[q] = load(pin, n, OPP(q), node);
            if (fl == LBMX_MOVING_WALL_BB) {
                // Ladd's term 6 w (c . u_w) of the outgoing direction OPP(q)
                const D wx = dual(a.wall_ux, a.param == LBMX_TANGENT_WALL_UX);
                const int o = OPP(q);
                f[q] = f[q] - 6.0f * WQ(o) * ((float)CX(o) * wx + dconst<1>((float)CY(o) * a.wall_uy));
            }
        } else {
            f[q] = load(pout, n, q, node);
        }
    }
    const D ubc = dual(a.u_bc, a.param == LBMX_TANGENT_U_BC);
    switch (fl) {
    case LBMX_BOUNCE_BACK: bc_bounce_back<D>(a.g, f, x, y); break;
    case LBMX_ZOU_HE_TOP: bc_zouhe_top<D>(f, ubc); break;
    case LBMX_ZOU_HE_LEFT: bc_zouhe_left<D>(f, ubc, (a.quirks & LBMX_QUIRK_ZOUHE_LEFT) != 0); break;
    case LBMX_CYLINDER: bc_cylinder<D>(f); break;
    case LBMX_ZOU_HE_PRESSURE_RIGHT: bc_zouhe_pressure_right<D>(f, a.rho_out_bc); break;
    case LBMX_ZOU_HE_PARABOLIC_LEFT: bc_zouhe_left<D>(f, parabolic_ux<D>(ubc, y, a.g.ny), false); break;
    default: break;
    }
}

__global__ void tan_init_kernel(const TanArgs a, const float* rho, const float* u, float* b0, float* b1) {
    const int x = blockIdx.x * kTanBX + threadIdx.x, y = blockIdx.y * kTanBY + threadIdx.y;
    if (x >= a.g.nx || y >= a.g.ny) return;
    const long long node = (long long)y * a.g.nx + x, n = a.n;
    float fe[9];
    init_equilibrium(rho[node], u[node], u[n + node], fe);
#pragma unroll
    for (int q = 0; q < 9; q++) {
        b0[q * n + node] = b1[q * n + node] = fe[q];
        b0[(9 + q) * n + node] = b1[(9 + q) * n + node] = 0.0f;
    }
}

// the IBM's input: density and uncorrected velocity at the patch nodes
__global__ void tan_ibm_gather_kernel(const TanArgs a, const float* pin, const float* pout, const int* patch_nodes,
                                      int np, D* prho, D* pu) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= np) return;
    const long long node = patch_nodes[i];
    const int y = (int)(node / a.g.nx), x = (int)(node - (long long)y * a.g.nx);
    D f[9];
    tan_gather(a, pin, pout, x, y, node, a.flags[node], f);
    D rho = dconst<1>(0.f), jx = dconst<1>(0.f), jy = dconst<1>(0.f);
#pragma unroll
    for (int q = 0; q < 9; q++) {
        rho = rho + f[q];
        jx = jx + (float)CX(q) * f[q];
        jy = jy + (float)CY(q) * f[q];
    }
    const D inv = 1.0f / rho;
    prho[i] = rho;
    pu[i] = jx * inv;
    pu[np + i] = jy * inv;
}

__global__ void __launch_bounds__(kIbmThreads) tan_ibm_kernel(const IbmData<D> a) {
    extern __shared__ float sm[];
    ibm_rounds<D>(a, reinterpret_cast<D*>(sm));
}

// drag, lift (minus the summed marker forces, as lbmx_ibm_forces) and their
// tangents of one step, summed in FP64 in a fixed order
__global__ void tan_series_kernel(const D* marker_force, int nm, double* out4) {
    __shared__ double s[4][256];
    const int tid = threadIdx.x;
    double v[4] = {0, 0, 0, 0};
    for (int k = tid; k < nm; k += 256) {
        v[0] += marker_force[k].v;
        v[1] += marker_force[nm + k].v;
        v[2] += marker_force[k].d[0];
        v[3] += marker_force[nm + k].d[0];
    }
    for (int c = 0; c < 4; c++) s[c][tid] = v[c];
    __syncthreads();
    for (int w = 128; w > 0; w >>= 1) {
        if (tid < w)
            for (int c = 0; c < 4; c++) s[c][tid] += s[c][tid + w];
        __syncthreads();
    }
    if (tid == 0) {
        out4[0] = -s[0][0];
        out4[1] = -s[1][0];
        out4[2] = -s[2][0];
        out4[3] = -s[3][0];
    }
}

template <int OP>
__global__ void __launch_bounds__(kTanBX * kTanBY) tan_step_kernel(const TanArgs a, const float* pin, float* pout,
                                                                    float* mom) {
    const int x = blockIdx.x * kTanBX + threadIdx.x, y = blockIdx.y * kTanBY + threadIdx.y;
    if (x >= a.g.nx || y >= a.g.ny) return;
    const long long node = (long long)y * a.g.nx + x, n = a.n;
    D f[9];
    tan_gather(a, pin, pout, x, y, node, a.flags[node], f);
    // macroscopics and the Guo half-force velocity, as the engine's general path
    D rho = dconst<1>(0.f), jx = dconst<1>(0.f), jy = dconst<1>(0.f);
#pragma unroll
    for (int q = 0; q < 9; q++) {
        rho = rho + f[q];
        jx = jx + (float)CX(q) * f[q];
        jy = jy + (float)CY(q) * f[q];
    }
    D Fx = dual(a.fx, a.param == LBMX_TANGENT_BODY_FX), Fy = dconst<1>(a.fy);
    if (a.ibm_force) {
        Fx = Fx + a.ibm_force[node];
        Fy = Fy + a.ibm_force[n + node];
    }
    const D inv = 1.0f / rho;
    const D ux = jx * inv + 0.5f * Fx / rho;
    const D uy = jy * inv + 0.5f * Fy / rho;
    if (mom) {
        mom[node] = rho.v;
        mom[n + node] = ux.v;
        mom[2 * n + node] = uy.v;
        mom[3 * n + node] = rho.d[0];
        mom[4 * n + node] = ux.d[0];
        mom[5 * n + node] = uy.d[0];
    }
    const bool om = a.param == LBMX_TANGENT_OMEGA;
    if (OP == LBMX_BGK) {
        collide_bgk<D, false, D>(f, rho, rho, ux, uy, Fx, Fy, dual(a.omega, om), a.forced != 0);
    } else {
        D S[9];
#pragma unroll
        for (int k = 0; k < 9; k++) S[k] = dual(a.S[k], om && ((a.omega_mask >> k) & 1u));
        if (OP == LBMX_MRT)
            collide_mrt<D, false, D>(f, rho, rho, ux, uy, Fx, Fy, S, (a.quirks & LBMX_QUIRK_MRT_FORCE) != 0,
                                     a.forced != 0);
        else
            collide_cm<D, false, D>(f, rho, rho, ux, uy, Fx, Fy, S, dconst<1>(0.f), false);
    }
#pragma unroll
    for (int q = 0; q < 9; q++) put(pout, n, q, node, f[q]);
}

}  // namespace
}  // namespace lbmx

using namespace lbmx;

struct lbmx_tangent {
    lbmx_params p;
    TanArgs args;
    cudaStream_t stream = nullptr;
    bool own_stream = false;
    long long n = 0;
    uint8_t* flags = nullptr;
    float* buf[2] = {nullptr, nullptr};  // [18][n] each
    float* mom = nullptr;                // [6][n]
    double* series = nullptr;            // [cap][4]
    int series_cap = 0;
    int cur = 0;                         // buffer with the latest post-collision state
    long long t = 0;
    bool have_state = false, have_mom = false;
    // markers
    int nm = 0, npatch = 0, stencil = 0;
    int* patch_nodes = nullptr;
    int* sten_idx = nullptr;
    int* spread = nullptr;
    float* sten_w = nullptr;
    D* patch_rho = nullptr;
    D* patch_u = nullptr;
    D* marker_u = nullptr;
    D* marker_rho = nullptr;
    D* marker_force = nullptr;
    D* ibm_force = nullptr;  // [2][n]
    char err[512] = {0};
};

namespace {

char g_tan_err[512];

lbmx_status tfail(lbmx_tangent* t, lbmx_status code, const char* fmt, ...) {
    char* dst = t ? t->err : g_tan_err;
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(dst, 512, fmt, ap);
    va_end(ap);
    return code;
}

#define TAN_CUDA(t, call)                                                                           \
    do {                                                                                            \
        cudaError_t e_ = (call);                                                                    \
        if (e_ != cudaSuccess)                                                                      \
            return tfail((t), e_ == cudaErrorMemoryAllocation ? LBMX_ERR_OUT_OF_MEMORY : LBMX_ERR_CUDA, \
                         "%s: %s (%s:%d)", #call, cudaGetErrorString(e_), __FILE__, __LINE__);        \
    } while (0)

dim3 node_grid(const lbmx_tangent* t) {
    return dim3((unsigned)((t->p.nx + kTanBX - 1) / kTanBX), (unsigned)((t->p.ny + kTanBY - 1) / kTanBY));
}

void free_markers(lbmx_tangent* t) {
    cudaFree(t->patch_nodes); cudaFree(t->sten_idx); cudaFree(t->sten_w); cudaFree(t->spread); cudaFree(t->patch_rho);
    cudaFree(t->patch_u); cudaFree(t->marker_u); cudaFree(t->marker_rho); cudaFree(t->marker_force);
    cudaFree(t->ibm_force);
    t->patch_nodes = t->sten_idx = t->spread = nullptr;
    t->sten_w = nullptr;
    t->patch_rho = t->patch_u = t->marker_u = t->marker_rho = t->marker_force = t->ibm_force = nullptr;
    t->nm = t->npatch = t->stencil = 0;
    t->args.ibm_force = nullptr;
}

bool supported_flag(uint8_t f) {
    switch (f) {
    case LBMX_FLUID: case LBMX_BOUNCE_BACK: case LBMX_ZOU_HE_TOP: case LBMX_ZOU_HE_LEFT: case LBMX_CYLINDER:
    case LBMX_MOVING_WALL_BB: case LBMX_ZOU_HE_PRESSURE_RIGHT: case LBMX_ZOU_HE_PARABOLIC_LEFT:
    case LBMX_HALFWAY_BB:
        return true;
    default:
        return false;
    }
}

}  // namespace

extern "C" {

void lbmx_tangent_destroy(lbmx_tangent* t) {
    if (!t) return;
    int dev = 0;
    cudaGetDevice(&dev);
    cudaSetDevice(t->p.device);
    if (t->stream) cudaStreamSynchronize(t->stream);
    free_markers(t);
    cudaFree(t->flags); cudaFree(t->buf[0]); cudaFree(t->buf[1]); cudaFree(t->mom); cudaFree(t->series);
    if (t->own_stream && t->stream) cudaStreamDestroy(t->stream);
    cudaSetDevice(dev);
    delete t;
}

lbmx_status lbmx_tangent_create(const lbmx_params* p, const uint8_t* flags, int32_t parameter, lbmx_tangent** out) {
    if (!out) return tfail(nullptr, LBMX_ERR_INVALID_ARGUMENT, "lbmx_tangent_create: out is NULL");
    *out = nullptr;
    if (!p) return tfail(nullptr, LBMX_ERR_INVALID_ARGUMENT, "lbmx_tangent_create: params is NULL");
    if (p->nx < 3 || p->ny < 3 || (long long)p->nx * p->ny > (1LL << 31) - 1)
        return tfail(nullptr, LBMX_ERR_INVALID_ARGUMENT, "lbmx_tangent_create: bad lattice %d x %d", p->nx, p->ny);
    if (p->op < LBMX_BGK || p->op > LBMX_CM)
        return tfail(nullptr, p->op == LBMX_CM_OPT ? LBMX_ERR_UNSUPPORTED : LBMX_ERR_INVALID_ARGUMENT,
                     "lbmx_tangent_create: operator %d is not differentiated (BGK, MRT and CM are)", p->op);
    if (parameter < LBMX_TANGENT_U_BC || parameter > LBMX_TANGENT_WALL_UX)
        return tfail(nullptr, LBMX_ERR_INVALID_ARGUMENT, "lbmx_tangent_create: unknown parameter %d", parameter);
    if (p->storage != LBMX_STORAGE_F32)
        return tfail(nullptr, LBMX_ERR_UNSUPPORTED, "lbmx_tangent_create: the tangent model runs FP32 populations");
    if (cudaSetDevice(p->device) != cudaSuccess)
        return tfail(nullptr, LBMX_ERR_CUDA, "lbmx_tangent_create: cannot select device %d", p->device);
    const long long n = (long long)p->nx * p->ny;
    std::vector<uint8_t> fl((size_t)n, 0);
    if (flags && cudaMemcpy(fl.data(), flags, fl.size(), cudaMemcpyDefault) != cudaSuccess)
        return tfail(nullptr, LBMX_ERR_CUDA, "lbmx_tangent_create: cannot read the flags");
    for (long long i = 0; i < n; i++)
        if (!supported_flag(fl[(size_t)i]))
            return tfail(nullptr, LBMX_ERR_UNSUPPORTED,
                         "lbmx_tangent_create: flag %d at (%lld,%lld) is not differentiated (fluid, bounce-back, "
                         "cylinder, Zou-He and half-way walls are)",
                         fl[(size_t)i], i % p->nx, i / p->nx);
    lbmx_tangent* t = new lbmx_tangent();
    t->p = *p;
    t->n = n;
    TanArgs& a = t->args;
    memset(&a, 0, sizeof(a));
    a.g.nx = p->nx;
    a.g.ny = p->ny;
    a.g.pitch = p->nx;
    a.g.periodic_x = p->periodic_x ? 1 : 0;
    a.g.periodic_y = p->periodic_y ? 1 : 0;
    a.g.plane = n;
    a.n = n;
    a.quirks = p->quirks;
    a.param = parameter;
    a.omega = p->omega;
    for (int k = 0; k < 9; k++) {
        a.S[k] = p->S[k];
        if (p->op != LBMX_BGK && p->S[k] == p->omega) a.omega_mask |= 1u << k;
    }
    a.u_bc = p->u_bc;
    a.rho_out_bc = p->rho_out;
    a.wall_ux = p->wall_ux;
    a.wall_uy = p->wall_uy;
    a.fx = p->body_fx;
    a.fy = p->body_fy;
    a.forced = (p->body_fx != 0.0f || p->body_fy != 0.0f || parameter == LBMX_TANGENT_BODY_FX) ? 1 : 0;
    auto bail = [&](const char* what) {
        tfail(nullptr, LBMX_ERR_OUT_OF_MEMORY, "lbmx_tangent_create: %s", what);
        lbmx_tangent_destroy(t);
        return LBMX_ERR_OUT_OF_MEMORY;
    };
    const size_t state = (size_t)18 * n * sizeof(float);
    if (cudaMalloc((void**)&t->flags, (size_t)n) != cudaSuccess || cudaMalloc((void**)&t->buf[0], state) != cudaSuccess ||
        cudaMalloc((void**)&t->buf[1], state) != cudaSuccess ||
        cudaMalloc((void**)&t->mom, (size_t)6 * n * sizeof(float)) != cudaSuccess)
        return bail("cudaMalloc failed");
    if (p->stream) {
        t->stream = (cudaStream_t)p->stream;
    } else {
        if (cudaStreamCreateWithFlags(&t->stream, cudaStreamNonBlocking) != cudaSuccess) return bail("no stream");
        t->own_stream = true;
    }
    if (cudaMemcpy(t->flags, fl.data(), fl.size(), cudaMemcpyHostToDevice) != cudaSuccess) return bail("flag upload");
    a.flags = t->flags;
    *out = t;
    return LBMX_OK;
}

lbmx_status lbmx_tangent_set_state(lbmx_tangent* t, const float* rho, const float* u) {
    if (!t || !rho || !u) return tfail(t, LBMX_ERR_INVALID_ARGUMENT, "lbmx_tangent_set_state: NULL argument");
    cudaSetDevice(t->p.device);
    float* tmp = nullptr;
    TAN_CUDA(t, cudaMalloc((void**)&tmp, (size_t)3 * t->n * sizeof(float)));
    cudaMemcpyAsync(tmp, rho, (size_t)t->n * sizeof(float), cudaMemcpyDefault, t->stream);
    cudaMemcpyAsync(tmp + t->n, u, (size_t)2 * t->n * sizeof(float), cudaMemcpyDefault, t->stream);
    tan_init_kernel<<<node_grid(t), dim3(kTanBX, kTanBY), 0, t->stream>>>(t->args, tmp, tmp + t->n, t->buf[0],
                                                                         t->buf[1]);
    const cudaError_t e0 = cudaGetLastError();
    const cudaError_t e = cudaStreamSynchronize(t->stream);
    cudaFree(tmp);
    TAN_CUDA(t, e0);
    TAN_CUDA(t, e);
    t->cur = 0;
    t->t = 0;
    t->have_state = true;
    t->have_mom = false;
    return LBMX_OK;
}

lbmx_status lbmx_tangent_set_markers(lbmx_tangent* t, const float* xy, int32_t n) {
    if (!t) return tfail(t, LBMX_ERR_INVALID_ARGUMENT, "lbmx_tangent_set_markers: NULL handle");
    if (n < 0 || (n > 0 && !xy)) return tfail(t, LBMX_ERR_INVALID_ARGUMENT, "lbmx_tangent_set_markers: bad marker array");
    cudaSetDevice(t->p.device);
    TAN_CUDA(t, cudaStreamSynchronize(t->stream));
    free_markers(t);
    if (n == 0) return LBMX_OK;
    std::vector<float> hxy(2 * (size_t)n);
    TAN_CUDA(t, cudaMemcpy(hxy.data(), xy, hxy.size() * sizeof(float), cudaMemcpyDefault));
    const bool two = (t->p.quirks & LBMX_QUIRK_IBM_2X2) != 0;
    std::vector<int> sidx, nodes;
    std::vector<float> sw;
    const int bad = ibm_build_stencil(t->p.nx, t->p.ny, t->p.nx, two, hxy.data(), n, sidx, sw, nodes);
    if (bad >= 0) return tfail(t, LBMX_ERR_INVALID_ARGUMENT, "lbmx_tangent_set_markers: marker %d is not finite", bad);
    const int np = (int)nodes.size();
    if (ibm_smem_bytes_of<D>(np, n, two ? 2 : 4) > 200 * 1024)
        return tfail(t, LBMX_ERR_TOO_LARGE,
                     "lbmx_tangent_set_markers: %d markers touch %d nodes; limit is 200 KB of patch state", n, np);
    t->nm = n;
    t->npatch = np;
    t->stencil = two ? 2 : 4;
    TAN_CUDA(t, cudaMalloc((void**)&t->patch_nodes, np * sizeof(int)));
    TAN_CUDA(t, cudaMalloc((void**)&t->sten_idx, sidx.size() * sizeof(int)));
    TAN_CUDA(t, cudaMalloc((void**)&t->sten_w, sw.size() * sizeof(float)));
    TAN_CUDA(t, cudaMalloc((void**)&t->patch_rho, np * sizeof(D)));
    TAN_CUDA(t, cudaMalloc((void**)&t->patch_u, 2 * (size_t)np * sizeof(D)));
    TAN_CUDA(t, cudaMalloc((void**)&t->marker_u, 2 * (size_t)n * sizeof(D)));
    TAN_CUDA(t, cudaMalloc((void**)&t->marker_rho, (size_t)n * sizeof(D)));
    TAN_CUDA(t, cudaMalloc((void**)&t->marker_force, 2 * (size_t)n * sizeof(D)));
    TAN_CUDA(t, cudaMalloc((void**)&t->ibm_force, 2 * (size_t)t->n * sizeof(D)));
    TAN_CUDA(t, cudaMemcpy(t->patch_nodes, nodes.data(), np * sizeof(int), cudaMemcpyHostToDevice));
    TAN_CUDA(t, cudaMemcpy(t->sten_idx, sidx.data(), sidx.size() * sizeof(int), cudaMemcpyHostToDevice));
    TAN_CUDA(t, cudaMemcpy(t->sten_w, sw.data(), sw.size() * sizeof(float), cudaMemcpyHostToDevice));
    const std::vector<int> spread = ibm_build_spread(np, sidx);
    TAN_CUDA(t, cudaMalloc((void**)&t->spread, spread.size() * sizeof(int)));
    TAN_CUDA(t, cudaMemcpy(t->spread, spread.data(), spread.size() * sizeof(int), cudaMemcpyHostToDevice));
    TAN_CUDA(t, cudaMemset(t->ibm_force, 0, 2 * (size_t)t->n * sizeof(D)));
    TAN_CUDA(t, cudaMemset(t->marker_force, 0, 2 * (size_t)n * sizeof(D)));
    TAN_CUDA(t, cudaFuncSetAttribute(tan_ibm_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     (int)ibm_smem_bytes_of<D>(np, n, t->stencil)));
    t->args.ibm_force = t->ibm_force;
    t->args.forced = 1;
    return LBMX_OK;
}

lbmx_status lbmx_tangent_run(lbmx_tangent* t, int32_t nsteps, double* series) {
    if (!t) return tfail(t, LBMX_ERR_INVALID_ARGUMENT, "lbmx_tangent_run: NULL handle");
    if (!t->have_state) return tfail(t, LBMX_ERR_NOT_INITIALIZED, "lbmx_tangent_run: call lbmx_tangent_set_state first");
    if (nsteps < 1) return tfail(t, LBMX_ERR_INVALID_ARGUMENT, "lbmx_tangent_run: nsteps < 1");
    cudaSetDevice(t->p.device);
    if (series && nsteps > t->series_cap) {
        cudaFree(t->series);
        t->series = nullptr;
        TAN_CUDA(t, cudaMalloc((void**)&t->series, (size_t)4 * nsteps * sizeof(double)));
        t->series_cap = nsteps;
    }
    if (series) TAN_CUDA(t, cudaMemsetAsync(t->series, 0, (size_t)4 * nsteps * sizeof(double), t->stream));
    IbmData<D> ia;
    memset(&ia, 0, sizeof(ia));
    ia.nm = t->nm;
    ia.npatch = t->npatch;
    ia.iters = t->p.ibm_iters > 0 ? t->p.ibm_iters : 3;
    ia.stencil = t->stencil;
    ia.sten_idx = t->sten_idx;
    ia.sten_w = t->sten_w;
    ia.spread = t->spread;
    ia.patch_nodes = t->patch_nodes;
    ia.patch_rho = t->patch_rho;
    ia.patch_u = t->patch_u;
    ia.marker_u = t->marker_u;
    ia.marker_rho = t->marker_rho;
    ia.marker_force = t->marker_force;
    ia.ibm_force = t->ibm_force;
    ia.plane = t->n;
    ia.clamp = (t->p.quirks & LBMX_QUIRK_IBM_CLAMP) ? 1 : 0;
    ia.ds = t->p.ibm_ds != 0.0f ? t->p.ibm_ds : 1.0f;
    const size_t ibm_smem = ibm_smem_bytes_of<D>(t->npatch, t->nm, t->stencil);
    for (int s = 0; s < nsteps; s++) {
        const float* pin = t->buf[t->cur];
        float* pout = t->buf[t->cur ^ 1];
        if (t->nm > 0) {
            tan_ibm_gather_kernel<<<(t->npatch + 127) / 128, 128, 0, t->stream>>>(
                t->args, pin, pout, t->patch_nodes, t->npatch, t->patch_rho, t->patch_u);
            TAN_CUDA(t, cudaGetLastError());
            tan_ibm_kernel<<<1, kIbmThreads, ibm_smem, t->stream>>>(ia);
            TAN_CUDA(t, cudaGetLastError());
            if (series) {
                tan_series_kernel<<<1, 256, 0, t->stream>>>(t->marker_force, t->nm, t->series + (size_t)4 * s);
                TAN_CUDA(t, cudaGetLastError());
            }
        }
        float* mom = s == nsteps - 1 ? t->mom : nullptr;
        switch (t->p.op) {
        case LBMX_BGK:
            tan_step_kernel<LBMX_BGK><<<node_grid(t), dim3(kTanBX, kTanBY), 0, t->stream>>>(t->args, pin, pout, mom);
            break;
        case LBMX_MRT:
            tan_step_kernel<LBMX_MRT><<<node_grid(t), dim3(kTanBX, kTanBY), 0, t->stream>>>(t->args, pin, pout, mom);
            break;
        default:
            tan_step_kernel<LBMX_CM><<<node_grid(t), dim3(kTanBX, kTanBY), 0, t->stream>>>(t->args, pin, pout, mom);
            break;
        }
        TAN_CUDA(t, cudaGetLastError());
        t->cur ^= 1;
        t->t++;
    }
    if (series)
        TAN_CUDA(t, cudaMemcpyAsync(series, t->series, (size_t)4 * nsteps * sizeof(double), cudaMemcpyDefault,
                                    t->stream));
    TAN_CUDA(t, cudaStreamSynchronize(t->stream));
    t->have_mom = true;
    return LBMX_OK;
}

lbmx_status lbmx_tangent_moments(lbmx_tangent* t, float* rho, float* u, float* drho, float* du) {
    if (!t) return tfail(t, LBMX_ERR_INVALID_ARGUMENT, "lbmx_tangent_moments: NULL handle");
    if (!t->have_mom) return tfail(t, LBMX_ERR_NOT_INITIALIZED, "lbmx_tangent_moments: no step run yet");
    cudaSetDevice(t->p.device);
    const size_t nb = (size_t)t->n * sizeof(float);
    if (rho) TAN_CUDA(t, cudaMemcpyAsync(rho, t->mom, nb, cudaMemcpyDefault, t->stream));
    if (u) TAN_CUDA(t, cudaMemcpyAsync(u, t->mom + t->n, 2 * nb, cudaMemcpyDefault, t->stream));
    if (drho) TAN_CUDA(t, cudaMemcpyAsync(drho, t->mom + 3 * t->n, nb, cudaMemcpyDefault, t->stream));
    if (du) TAN_CUDA(t, cudaMemcpyAsync(du, t->mom + 4 * t->n, 2 * nb, cudaMemcpyDefault, t->stream));
    TAN_CUDA(t, cudaStreamSynchronize(t->stream));
    return LBMX_OK;
}

int64_t lbmx_tangent_time(lbmx_tangent* t) { return t ? t->t : -1; }

const char* lbmx_tangent_last_error(lbmx_tangent* t) { return t ? t->err : g_tan_err; }

}  // extern "C"
