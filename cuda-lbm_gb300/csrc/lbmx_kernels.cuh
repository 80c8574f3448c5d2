// lbmx_kernels.cuh -- kernels of the fused D2Q9 step, instantiated once per
// storage type by lbmx_step_{f32,f16,bf16}.cu.
//
// One step of the reference loop (src/main.cu:96-114) becomes:
//   [edge pre-pass]   neighbour data for ZG / pressure / corner boundaries
//   [IBM gather + iterate]  only with markers (lbmx_ibm.cu)
//   [average pre-pass]      only for CM_OPT without lagged averages
//   step kernel: pull post-stream populations (AA pattern), boundary,
//                moments, force correction, collision, store in place.
//
// The step kernel works on "units" of two x-neighbouring nodes (x0 even).
// Units listed as special -- the domain perimeter and every unit holding a
// flagged or IBM-forced node -- go through the general per-node path, one
// node per thread, in chunks of 256 nodes that lead the work list.  Interior
// tiles of 128 x 4 nodes (rows 1..ny-2) follow, staged into shared memory by
// bulk asynchronous copies, one unit per thread, skipping the special units.
// Every CTA is persistent and claims items from one counter.  An interior unit needs no boundary,
// wrap or flag logic, reads its two nodes as one 64-bit (FP32) or 32-bit
// (16-bit) shared-memory access wherever the pair stays aligned, collides
// both nodes at once in packed FP32x2 arithmetic and stores in place.  The
// AA pattern makes every population slot the property of one node, so the
// two sets of CTAs never write the same memory.
#pragma once
#include <cstring>

#include "lbmx_device.cuh"
#include "lbmx_ibm.cuh"

namespace lbmx {

constexpr int kThreads = kStepThreads;

// The step's grid sums (mass, momentum, the CM_OPT average terms and the
// kinetic energy; kNumSums of them) are accumulated in exact 64-bit fixed
// point: each node's FP32 term, scaled by 2^30 and rounded, is added as an
// integer -- per thread, by warp shuffles, then across warps with integer
// atomics into the accumulators of a slot.  Integer addition is
// associative, so the sums are the same bit for bit whichever CTA claims
// which tile; a term's rounding is at most 2^-31 (5e-10), and the range
// (|sum| < 2^33) covers any lattice of up to 2^31 nodes at unit density.
// The reference adds float atomics (update_avg_mag,
// macroscopics.cuh:116-118; compute_kinetic_energy_kernel,
// scenarios/taylorGreen3D/postprocessing/kineticEnergy.cuh:7-40); FP64
// arithmetic, a small fraction of FP32's rate on GB300, appears only in the
// final conversion.
using Acc = long long;
constexpr float kFixScale = 1073741824.0f;  // 2^30
// round-to-nearest-even of t * 2^30 as a 64-bit integer.  The FP32 -> S64
// conversion instruction runs on the FP64 pipe, a small fraction of FP32's
// rate on GB300, so terms below 2048 in magnitude take the FP32 adder
// instead: adding 1.5 * 2^23 to v (|v| < 2^22) leaves rint(v) in the low
// mantissa bits.  With x = t * 2^30 (exact), h = rint(x / 2^20) and the
// remainder r = x - h * 2^20 (exact: |r| <= 2^19, a multiple of x's ulp),
// rint(x) = h * 2^20 + rint(r) bit for bit, ties to even included, since
// h * 2^20 is an even integer.  Larger terms and NaN keep the conversion.
__device__ __forceinline__ Acc fix(float t) {
    const float x = __fmul_rn(t, kFixScale);
    if (!(fabsf(t) < 2048.0f)) return __float2ll_rn(x);
    constexpr float kMagic = 12582912.0f;  // 1.5 * 2^23
    const float hb = __fadd_rn(__fmul_rn(x, 9.5367431640625e-07f), kMagic);  // x * 2^-20, rounded to an integer
    const float hf = __fadd_rn(hb, -kMagic);
    const float r = __fmaf_rn(-hf, 1048576.0f, x);
    const int h = __float_as_int(hb) - 0x4B400000;
    const int lo = __float_as_int(__fadd_rn(r, kMagic)) - 0x4B400000;
    return ((Acc)h << 20) + (Acc)lo;
}

// which accumulators a set of sums uses: mass and momentum always, the
// kinetic energy and the CM_OPT average terms on request
__host__ __device__ __forceinline__ unsigned sums_mask(bool ke, bool averages) {
    return 0x7u | (ke ? 1u << kSumKE : 0u) | (averages ? 0x30u : 0u);
}

// A warp's totals of the accumulators in `mask` into its slot.
__device__ __forceinline__ void warp_sums(double* partials, const Acc v[kNumSums], unsigned mask) {
    const int tid = threadIdx.y * blockDim.x + threadIdx.x;
    const int lane = tid & 31, warp = tid >> 5;
    const int nwarps = (blockDim.x * blockDim.y + 31) >> 5;
    unsigned long long* acc =
        reinterpret_cast<unsigned long long*>(partials) + ((blockIdx.x * nwarps + warp) % kSumSlots) * kNumSums;
#pragma unroll
    for (int k = 0; k < kNumSums; k++) {
        if (!((mask >> k) & 1u)) continue;
        Acc t = v[k];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) t += __shfl_down_sync(0xffffffffu, t, o);
        if (lane == 0 && t != 0) atomicAdd(acc + k, (unsigned long long)t);
    }
}

// kModeSums: mass and momentum of the whole CTA (warp shuffles, the warps'
// totals added in shared memory), one atomic per sum into the CTA's slot --
// at the end of a step every CTA reduces at once, and one atomic per warp
// queued on the 32 slots' addresses.  Every thread of the CTA calls it.
__device__ __forceinline__ void cta_sums(double* partials, const Acc v[kNumSums]) {
    __shared__ Acc sh[kStepThreads / 32][3];
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
#pragma unroll
    for (int k = 0; k < 3; k++) {
        Acc t = v[k];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) t += __shfl_down_sync(0xffffffffu, t, o);
        if (lane == 0) sh[warp][k] = t;
    }
    __syncthreads();
    if (tid < 3) {
        Acc t = 0;
#pragma unroll
        for (int w = 0; w < kStepThreads / 32; w++) t += sh[w][tid];
        unsigned long long* acc = reinterpret_cast<unsigned long long*>(partials) + (blockIdx.x % kSumSlots) * kNumSums;
        if (t != 0) atomicAdd(acc + tid, (unsigned long long)t);
    }
}

// The sums in `mask` of an accumulator set, by one warp: lane j takes slot j
// (integer totals, the same bits in any order), in one round of loads; the
// slots are zeroed for their next use.  Every lane gets s (the other sums 0);
// lane 0 writes raw when given.
static_assert(kSumSlots == 32, "collect_sums: one slot per lane");
__device__ __forceinline__ void collect_sums(double* partials, unsigned mask, double s[kNumSums], long long* raw,
                                             int lane) {
    unsigned long long* acc = reinterpret_cast<unsigned long long*>(partials) + lane * kNumSums;
    unsigned long long t[kNumSums];
#pragma unroll
    for (int k = 0; k < kNumSums; k++) {
        t[k] = 0ull;
        if ((mask >> k) & 1u) {
            t[k] = __ldcg(acc + k);
            acc[k] = 0ull;
        }
    }
#pragma unroll
    for (int k = 0; k < kNumSums; k++) {
        if ((mask >> k) & 1u)
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) t[k] += __shfl_xor_sync(0xffffffffu, t[k], o);
        s[k] = (double)(long long)t[k] * (1.0 / (double)kFixScale);
        if (raw && lane == 0) raw[k] = (long long)t[k];
    }
}

// The sums array and a step's series entry: {rho, rho ux, rho uy}, then the
// kinetic energy when it was reduced.
__device__ __forceinline__ void write_sums(const double s[kNumSums], double* sums, double* series, bool ke) {
    if (sums)
        for (int k = 0; k < kNumSums; k++) sums[k] = s[k];
    if (series) {
        for (int k = 0; k < 3; k++) series[k] = s[k];
        if (ke) series[3] = s[kSumKE];
    }
}

// Publish a kModeSums step's sums (mass and momentum only), by one warp.
__device__ __forceinline__ void publish_sums(double* partials, double* sums, double* series, int lane) {
    double sv[kNumSums];
    collect_sums(partials, sums_mask(false, false), sv, nullptr, lane);
    if (lane == 0) write_sums(sv, sums, series, false);
}

// Grid reduction of the accumulators; the last CTA to finish publishes the
// sums (sums, series, averages) and zeroes the accumulators for the next launch.
__device__ __forceinline__ void block_sums(const StepArgs& a, const Acc v[kNumSums], long long n_nodes) {
    __shared__ bool is_last;
    const int tid = threadIdx.y * blockDim.x + threadIdx.x;
    const unsigned mask = sums_mask(a.ke != 0, a.avg_out != nullptr);
    warp_sums(a.partials, v, mask);
    __syncthreads();
    if (tid == 0) {
        __threadfence();
        const unsigned done = atomicAdd(a.counter, 1u);
        is_last = (done == gridDim.x - 1);
    }
    __syncthreads();
    if (!is_last || tid >= 32) return;
    __threadfence();
    double s[kNumSums];
    collect_sums(a.partials, mask, s, a.raw_sums, tid);
    if (tid != 0) return;
    write_sums(s, a.sums, a.series, a.ke != 0);
    if (a.avg_out) {
        a.avg_out[0] = (float)(s[0] / (double)n_nodes);
        a.avg_out[1] = (float)(s[4] / (double)n_nodes);
        a.avg_out[2] = (float)(s[5] / (double)n_nodes);
    }
    *a.counter = 0u;
    __threadfence();
}

// Post-stream, post-boundary populations of (x, y); returns the node's flag.
template <typename T>
__device__ __forceinline__ uint8_t gather_node(const StepArgs& a, int x, int y, float f[9], unsigned* outmask) {
    const uint8_t fl = a.flags ? a.flags[(long long)y * a.g.pitch + x] : (uint8_t)0;
    load_post_stream<T>(a, x, y, fl, f, outmask);
    if (fl) apply_bc(a, f, x, y, fl);
    return fl;
}

__device__ __forceinline__ void node_force(const StepArgs& a, long long off, float* Fx, float* Fy) {
    float fx = a.body_fx, fy = a.body_fy;
    if (a.force) {
        fx = a.force[off];
        fy = a.force[a.g.plane + off];
    }
    if (a.ibm_force) {
        // written by the IBM kernel this grid may have overlapped: read
        // through L2
        fx += __ldcg(a.ibm_force + off);
        fy += __ldcg(a.ibm_force + a.g.plane + off);
    }
    *Fx = fx;
    *Fy = fy;
}

// One node through the general path (special units).  The lean and sums
// step variants inline it (one node per thread is a long dependent chain;
// the arguments then come straight from the parameter bank); the full
// variants, whose tiles need every register, call it out of line
// (general_node).  Both step kernels, single-lattice and batched, make the
// same choice for the same variant, so a lattice steps bit for bit alike
// in either.
template <typename T, int OP>
__device__ __forceinline__ void general_node_body(const StepArgs& a, int x, int y, Acc v[kNumSums], uint32_t seed) {
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
    float ux = jx * inv + 0.5f * Fx / rho;
    float uy = jy * inv + 0.5f * Fy / rho;
    if (a.gamma) brinkman<float>(a.gamma[off], rho, ux, uy, Fx, Fy);
    float pimag = 0.f;
    if (OP == LBMX_CM_OPT || (a.partials && a.avg_out)) {
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
        // a node's terms in fixed point; the averages' terms only when
        // averages are produced
        v[0] += fix(rho);
        v[1] += fix(rho * ux);
        v[2] += fix(rho * uy);
        if (a.ke) v[kSumKE] += fix(0.5f * rho * (ux * ux + uy * uy));
        if (a.avg_out) {
            v[4] += fix(rho * sqrtf(ux * ux + uy * uy));
            v[5] += fix(pimag);
        }
    }
    if (a.check_finite && !isfinite(rho)) atomicOr(a.error_word, 1u);
    if (OP == LBMX_BGK) {
        collide_bgk<float>(f, rho, rho, ux, uy, Fx, Fy, a.omega, a.forced);
    } else if (OP == LBMX_MRT) {
        collide_mrt<float>(f, rho, rho, ux, uy, Fx, Fy, a.S, (a.quirks & LBMX_QUIRK_MRT_FORCE) != 0, a.forced);
    } else if (OP == LBMX_CM) {
        collide_cm<float>(f, rho, rho, ux, uy, Fx, Fy, a.S, 0.f, false);
    } else {
        const float jmag = sqrtf(ux * ux + uy * uy) * rho;
        collide_cm<float>(f, rho, rho, ux, uy, Fx, Fy, a.S, optimal_rate<float>(rho, jmag, pimag, a.avg), true);
    }
    store_post_collision<T>(a, x, y, f, outmask, fl, seed);
}

template <typename T, int OP>
__device__ __noinline__ void general_node(const StepArgs& a, int x, int y, Acc v[kNumSums], uint32_t seed) {
    general_node_body<T, OP>(a, x, y, v, seed);
}

// ---------------------------------------------------------------- staging
// Interior tiles of kStageW x kStageH nodes are staged through a ring of
// shared-memory buffers filled by the tensor memory accelerator: one 3-D
// tiled TMA load (cp.async.bulk.tensor, completion counted on an mbarrier)
// per population plane brings a (kStageW + halo) x kStageH box, so the bytes
// in flight per SM do not depend on how many registers the collision needs.
// The box starts one 16-byte chunk left of the tile and ends one chunk right
// of it, which covers the one-node x shift of the neighbour-access step and
// keeps the box's x coordinate on a 16-byte boundary; boxes that stick out of
// the lattice are zero-filled by the TMA unit (those nodes are never used).

__device__ __forceinline__ uint32_t smem_addr(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint64_t* bar, unsigned count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, unsigned bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes) : "memory");
}
__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_addr(bar)) : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, unsigned parity) {
    uint32_t ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(ok)
        : "r"(smem_addr(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}
// bounded wait: gives up after `limit` polls (the caller reports the failure)
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, unsigned parity, unsigned limit) {
    for (unsigned i = 0; i < limit; i++)
        if (mbar_try_wait(bar, parity)) return true;
    return false;
}
// orders this thread's earlier shared-memory accesses before later async-proxy writes
__device__ __forceinline__ void fence_proxy_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }
// 3-D tiled TMA load of one box at element coordinates (x, y, z)
__device__ __forceinline__ void tma_load_3d(void* dst, const CUtensorMap* tmap, int x, int y, int z, uint64_t* bar) {
    asm volatile(
        "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], "
        "[%5];" ::"r"(smem_addr(dst)),
        "l"(reinterpret_cast<uint64_t>(tmap)), "r"(x), "r"(y), "r"(z), "r"(smem_addr(bar))
        : "memory");
}

template <typename T, int TW_ = kStageW, int TH_ = kStageH>
struct Staging {
    static constexpr int A = 16 / (int)sizeof(T);   // elements per 16-byte chunk
    static constexpr int TW = TW_, TH = TH_;
    static constexpr int ROWS = 2 * kConsumerWarps * 32 / TW;  // tile rows one pass of the consumers covers
    static constexpr int TWP = TW + 2 * A;           // box width: the tile plus one chunk each side
    static constexpr int NST = sizeof(T) == 4 ? 3 : (TW_ * TH_ > kStageW * kStageH ? LBMX_NST16 : 4);
    // one population's box, its slot padded to 128 bytes: every box lands on
    // a 128-byte boundary of shared memory
    static constexpr int BOX_ELEMS = TH * TWP;
    static constexpr int SLAB = (int)(((BOX_ELEMS * sizeof(T) + 127) / 128) * 128 / sizeof(T));
    static constexpr int STAGE_ELEMS = 9 * SLAB;
    static constexpr unsigned STAGE_BYTES = (unsigned)(9 * BOX_ELEMS * sizeof(T));  // bytes the nine boxes bring
    static constexpr size_t BUF_BYTES = (size_t)NST * STAGE_ELEMS * sizeof(T);
    // after the buffers: full[NST], empty[NST] mbarriers, one work slot per stage
    static constexpr size_t SMEM = BUF_BYTES + 2 * NST * sizeof(uint64_t) + NST * sizeof(int4);
};

constexpr unsigned kWaitLimit = 1u << 20;  // polls before a wait gives up

// Work slot of a stage, written by the producer before it arms the stage's
// full barrier and read by the consumers after the barrier completes:
// code >= 0 an interior tile whose first node is (x0, y0); code <= -2 special
// chunk -code - 2; code == -1 no more work.  w: the lattice (batched kernel).
__device__ __forceinline__ void put_slot(int4* slot, int code, int x0, int y0, int w) {
    volatile int* p = reinterpret_cast<volatile int*>(slot);
    p[0] = code;
    p[1] = x0;
    p[2] = y0;
    p[3] = w;
}
__device__ __forceinline__ int4 get_slot(const int4* slot) {
    const volatile int* p = reinterpret_cast<const volatile int*>(slot);
    return make_int4(p[0], p[1], p[2], p[3]);
}

// Issue the nine box loads of one tile into stage buffer `buf` (producer warp;
// lane 0 has already armed `bar` with Staging<T>::STAGE_BYTES).  Population q
// lands in slab q (TH rows of TWP elements); node x of tile row r then sits at
// column x - x0 + A - (parity-1 x shift of q).
template <typename T, int P, int TW = kStageW, int TH = kStageH>
__device__ __forceinline__ void stage_issue(const StepArgs& a, const CUtensorMap* tmap, int x0, int y0, T* buf,
                                            uint64_t* bar) {
    using St = Staging<T, TW, TH>;
    const int lane = threadIdx.x & 31;
    if (lane >= 9) return;
    const int q = lane;
    // parity 1 reads slot OPP(q) of the upstream nodes, rows shifted by -c_y(q)
    int plane, dy;
    switch (q) {
#define LBMX_Q(QV)                                                     \
    case QV:                                                           \
        plane = QV == 0 ? a.rest_plane : (P ? OPP(QV) : QV);          \
        dy = P ? -CY(QV) : 0;                                          \
        break;
        LBMX_Q(0) LBMX_Q(1) LBMX_Q(2) LBMX_Q(3) LBMX_Q(4) LBMX_Q(5) LBMX_Q(6) LBMX_Q(7) LBMX_Q(8)
#undef LBMX_Q
    default: plane = 0; dy = 0;
    }
    tma_load_3d(buf + (size_t)q * St::SLAB, tmap, x0 - St::A, y0 + dy, plane, bar);
}

// accumulators an interior-path variant (step_mode) touches
__host__ __device__ constexpr int mode_sums(int mode) { return mode == kModeLean ? 0 : (mode == kModeSums ? 3 : 6); }

// Collide two staged interior nodes (x0, x0+1) of row y and store them in place.
template <typename T, int OP, int P, int TW = kStageW, int TH = kStageH, int MODE = kModeFull>
__device__ __forceinline__ void interior_unit(const StepArgs& a, const T* sbuf, int r, int lx, int x0, int y,
                                              Acc v[kNumSums], uint32_t seed, const float* ibf = nullptr) {
    using St = Staging<T, TW, TH>;
    const Geometry& g = a.g;
    T* F = static_cast<T*>(a.f);
    const long long off = (long long)y * g.pitch + x0;
    const long long plane = g.plane;
    // 16-bit storage: f holds the stored offsets f - w throughout (the
    // collision works in offset form); FP32: f itself
    constexpr bool OFS = kOffset<T>;
    V2 f[9];
#pragma unroll
    for (int q = 0; q < 9; q++) {
        const bool shifted = P && CX(q) != 0;
        const T* s = sbuf + q * St::SLAB + r * St::TWP + 2 * lx + (shifted ? St::A - CX(q) : St::A);
        f[q].v = shifted ? Store<T>::ld2r_u(s) : Store<T>::ld2r(s);
    }
    V2 rho = ((f[0] + f[1]) + (f[2] + f[3])) + ((f[4] + f[5]) + (f[6] + f[7])) + f[8];
    const V2 drho = rho;                     // offset form: rho - 1, exactly
    if (OFS) rho = rho + splat(1.0f, rho);  // the weights sum to 1
    const V2 jx = (f[1] - f[3]) + ((f[5] + f[8]) - (f[6] + f[7]));
    const V2 jy = (f[2] - f[4]) + ((f[5] + f[6]) - (f[7] + f[8]));
    V2 Fx = {make_float2(a.body_fx, a.body_fx)}, Fy = {make_float2(a.body_fy, a.body_fy)};
    if (MODE == kModeFull && a.force) {
        Fx.v = *reinterpret_cast<const float2*>(a.force + off);
        Fy.v = *reinterpret_cast<const float2*>(a.force + plane + off);
    }
    if (ibf) {
        // a tile with IBM patch nodes: the forces this step's IBM kernel
        // wrote (zero off the patch), through L2 as in node_force
        Fx = Fx + V2{__ldcg(reinterpret_cast<const float2*>(ibf + off))};
        Fy = Fy + V2{__ldcg(reinterpret_cast<const float2*>(ibf + plane + off))};
    }
    const V2 inv = vdiv(splat(1.0f, rho), rho);
    V2 ux = fma(0.5f * Fx, inv, jx * inv);
    V2 uy = fma(0.5f * Fy, inv, jy * inv);
    if (MODE == kModeFull && a.gamma) brinkman<V2>(V2{*reinterpret_cast<const float2*>(a.gamma + off)}, rho, ux, uy, Fx, Fy);
    V2 pimag = splat(0.f, rho);
    if (OP == LBMX_CM_OPT || (MODE == kModeFull && a.partials && a.avg_out)) {
        // offset form: sum c_x^2 w = sum c_y^2 w = 1/3
        const V2 d = OFS ? (f[5] + f[6]) + ((f[7] + f[8]) + splat(1.0f / 3.0f, rho)) : (f[5] + f[6]) + (f[7] + f[8]);
        const V2 pxx = (f[1] + f[3]) + d, pyy = (f[2] + f[4]) + d;
        const V2 pxy = (f[5] + f[7]) - (f[6] + f[8]);
        pimag = vsqrt(fma(pxx, pxx, fma(2.0f * pxy, pxy, pyy * pyy)));
    }
    if (MODE == kModeFull && a.rho_out) {
        *reinterpret_cast<float2*>(a.rho_out + off) = rho.v;
        *reinterpret_cast<float2*>(a.u_out + off) = ux.v;
        *reinterpret_cast<float2*>(a.u_out + plane + off) = uy.v;
    }
    if (MODE == kModeSums || (MODE == kModeFull && a.partials)) {
        // the unit's terms in fixed point, the two nodes' summed in FP32
        // first (a fixed pairing, so the sums stay the same bit for bit):
        // half the 64-bit conversions, which run on the narrow FP64 pipe;
        // the averages' terms only when averages are produced
        const V2 jx2 = rho * ux, jy2 = rho * uy;
        v[0] += fix(rho.v.x + rho.v.y);
        v[1] += fix(jx2.v.x + jx2.v.y);
        v[2] += fix(jy2.v.x + jy2.v.y);
        if (MODE == kModeFull && a.ke) {
            const V2 e2 = rho * fma(ux, ux, uy * uy);
            v[kSumKE] += fix(0.5f * (e2.v.x + e2.v.y));
        }
        if (MODE == kModeFull && a.avg_out) {
            v[4] += fix(rho.v.x * sqrtf(ux.v.x * ux.v.x + uy.v.x * uy.v.x)) +
                    fix(rho.v.y * sqrtf(ux.v.y * ux.v.y + uy.v.y * uy.v.y));
            v[5] += fix(pimag.v.x) + fix(pimag.v.y);
        }
    }
    if (MODE == kModeFull && a.check_finite && !(isfinite(rho.v.x) && isfinite(rho.v.y))) atomicOr(a.error_word, 1u);
    if (OP == LBMX_BGK) {
        collide_bgk<V2, OFS>(f, rho, drho, ux, uy, Fx, Fy, a.omega, a.forced);
    } else if (OP == LBMX_MRT) {
        collide_mrt<V2, OFS>(f, rho, drho, ux, uy, Fx, Fy, a.S, (a.quirks & LBMX_QUIRK_MRT_FORCE) != 0, a.forced);
    } else if (OP == LBMX_CM) {
        collide_cm<V2, OFS>(f, rho, drho, ux, uy, Fx, Fy, a.S, rho, false);
    } else {
        const V2 jmag = rho * vsqrt(fma(ux, ux, uy * uy));
        collide_cm<V2, OFS>(f, rho, drho, ux, uy, Fx, Fy, a.S, optimal_rate<V2>(rho, jmag, pimag, a.avg), true);
    }
    // slot q of the downstream nodes x + c_q (parity 1) or the nodes' own
    // slot OPP(q) (parity 0): byte offsets of this launch, from the host
    char* base = reinterpret_cast<char*>(F + off);
    if (OFS && a.sr) {
        // stochastic rounding, random bits from each node's hash
        const uint32_t h = sr_hash(((uint32_t)off >> 1) + a.sr_unit_origin, seed);
#pragma unroll
        for (int q = 0; q < 9; q++) {
            T* p = reinterpret_cast<T*>(base + a.st_off[q]);
            const uint32_t r = sr_bits(h, q);
            if (P == 0 || CX(q) == 0) Store<T>::st2r_sr(p, f[q].v, r);
            else Store<T>::st2r_sr_u(p, f[q].v, r);
        }
    } else {
#pragma unroll
        for (int q = 0; q < 9; q++) {
            T* p = reinterpret_cast<T*>(base + a.st_off[q]);
            if (P == 0 || CX(q) == 0) Store<T>::st2r(p, f[q].v);
            else Store<T>::st2r_u(p, f[q].v);
        }
    }
}

// One chunk of special nodes: consumer thread t takes node `first + t` of
// the special-unit list (two nodes per unit).
template <typename T, int OP, int MODE = kModeFull>
__device__ __forceinline__ void special_chunk(const StepArgs& a, int chunk, int tid, Acc v[kNumSums], uint32_t seed) {
    const int k = chunk * kSpecialChunk + tid;
    if (k >= 2 * a.nspecial) return;
    const int off = a.special_units[k >> 1];
    const int y = off / a.g.pitch, x = off - y * a.g.pitch + (k & 1);
    if (x >= a.g.nx) return;
    // the out-of-line call gets its own accumulators, so the caller's stay
    // in registers
    Acc t[kNumSums] = {0, 0, 0, 0, 0, 0};
    if (MODE == kModeFull) general_node<T, OP>(a, x, y, t, seed);
    else general_node_body<T, OP>(a, x, y, t, seed);
    if (mode_sums(MODE) > 0 && a.partials)
#pragma unroll
        for (int k = 0; k < mode_sums(MODE); k++) v[k] += t[k];
}

template <typename T, int OP, int P, int MODE>
__global__ void __launch_bounds__(kThreads, kCtasPerSm) step_kernel(const StepArgs a, const __grid_constant__ CUtensorMap tmap) {
    constexpr int TW = step_tile_w((int)sizeof(T)), TH = step_tile_h((int)sizeof(T));
    // Persistent CTAs, warp-specialised: warp 8 produces (claims the next
    // work items, its CTA's own block first and then from a global counter;
    // for an interior tile it bulk-copies the tile into the ring), warps 0-7
    // consume.  Items 0..dep_chunk-1 are chunks of special nodes (general
    // path, one node per consumer thread, nothing staged) so the boundary
    // work spreads over every SM; the interior tiles away from an IBM patch
    // follow, then the chunks and the tiles next to one.  full[s] completes
    // when a stage's bytes have landed (or at once for a special chunk);
    // empty[s] when all eight consumer warps are done with it.
    using St = Staging<T, TW, TH>;
    Acc v[kNumSums] = {0, 0, 0, 0, 0, 0};
    const int tid = threadIdx.x;
    extern __shared__ __align__(128) unsigned char smem_raw[];
    T* bufs = reinterpret_cast<T*>(smem_raw);
    uint64_t* full = reinterpret_cast<uint64_t*>(smem_raw + St::BUF_BYTES);
    uint64_t* empty = full + St::NST;
    int4* slot = reinterpret_cast<int4*>(empty + St::NST);
    const int nchunks = a.special_chunks;
    const int ntiles = a.tiles_x * a.tiles_y;
    const int nitems = nchunks + ntiles;
    // item order: chunks [0, dep), the tiles that do not wait, chunks
    // [dep, nchunks), then the tiles that do (tile_order lists the tiles in
    // that order; without it every tile is early and in place)
    const int dep = min(a.dep_chunk, nchunks);
    const int early_tiles = a.tile_order ? a.dep_tile : ntiles;
    const int warp = tid >> 5, lane = tid & 31;
    if (tid == 0) {
        for (int s = 0; s < St::NST; s++) {
            mbar_init(&full[s], 1);
            mbar_init(&empty[s], kConsumerWarps);
        }
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    // The out-of-line general path (full variants) reads the arguments
    // through a pointer: into this shared copy, not into the kernel's
    // parameter space, which a pointer reaches only through slow generic
    // loads (a 256-node chunk took 1.3 times as long from there).
    __shared__ StepArgs sa;
    if (MODE == kModeFull && tid == 32 && nchunks > 0) sa = a;
    // Programmatic dependent launch: this grid may have started while the
    // previous step's grid was still draining.  Wait for that grid to finish
    // (its writes are then visible) before touching anything it wrote, then
    // let the next step's grid start its own prologue: every CTA of this grid
    // is resident by now, so the waiting grid cannot hold SM slots this one
    // still needs.  Without the launch attribute both are no-ops.
    // `early` (the IBM kernel of this step precedes): that kernel started
    // only after the previous step had finished, and it reads and writes
    // only the patch nodes' slots and forces, so every item before the
    // dependent chunks runs at once; the producer marks the dependent chunks
    // and each thread waits before its first one, and before it exits.
    if (!a.early) asm volatile("griddepcontrol.wait;" ::: "memory");
    asm volatile("griddepcontrol.launch_dependents;" :::);
    // the next step's work counter (the previous launch used it and has
    // finished)
    if (tid == 0 && blockIdx.x == 0) *a.tile_counter_next = 0ull;
    __syncthreads();
    if (warp == kConsumerWarps) {
        // the previous step's sums, if it left them, by CTA 0's producer
        // before its first claim while the consumers start (published by
        // one thread before the CTA's barrier they cost a 1024^2 step 2.9 us)
        if (blockIdx.x == 0 && a.pub_acc) publish_sums(a.pub_acc, a.pub_sums, a.pub_series, lane);
        // producer: claims `tile_chunk` consecutive items per atomic
        int k = 0;
        bool failed = false;
        int next = 0, left = 0;
        for (;; k++) {
            const int s = k % St::NST;
            if (k >= St::NST && !mbar_wait(&empty[s], (unsigned)(((k / St::NST) - 1) & 1), kWaitLimit)) {
                if (lane == 0) atomicOr(a.error_word, 2u);
                failed = true;
                break;
            }
            if (left == 0) {
                // the first claim of every CTA is its own block of items (no
                // atomic: all CTAs claim at once at the start); the counter
                // hands out the items after those
                int base = (int)blockIdx.x * a.tile_chunk;
                if (k > 0) {
                    if (lane == 0)
                        base = (int)gridDim.x * a.tile_chunk +
                               (int)atomicAdd(a.tile_counter, (unsigned long long)a.tile_chunk);
                    base = __shfl_sync(0xffffffffu, base, 0);
                }
                next = base;
                left = a.tile_chunk;
            }
            const int item = next++;
            left--;
            if (item >= nitems) {
                if (lane == 0) {
                    put_slot(&slot[s], -1, 0, 0, 0);
                    mbar_arrive(&full[s]);
                }
                break;
            }
            int chunk = -1, tile;
            const bool later = item >= dep + early_tiles;
            if (item < dep) chunk = item;
            else if (item < dep + early_tiles) tile = item - dep;
            else if (item < nchunks + early_tiles) chunk = item - early_tiles;
            else tile = item - nchunks;
            if (chunk >= 0) {
                if (lane == 0) {
                    put_slot(&slot[s], -2 - chunk, 0, 0, later ? 1 : 0);
                    mbar_arrive(&full[s]);
                }
                __syncwarp();
                continue;
            }
            // a tile that waits is staged at once all the same: the IBM
            // kernel only reads populations
            if (a.tile_order) tile = __ldg(a.tile_order + tile);
            const int ty = tile / a.tiles_x, tx = tile - ty * a.tiles_x;
            const int x0 = tx * St::TW, y0 = ty * St::TH;
            if (lane == 0) {
                put_slot(&slot[s], tile, x0, y0, later ? 1 : 0);
                fence_proxy_async_smem();
                mbar_expect_tx(&full[s], St::STAGE_BYTES);
            }
            __syncwarp();
            stage_issue<T, P, TW, TH>(a, &tmap, x0, y0, bufs + (size_t)s * St::STAGE_ELEMS, &full[s]);
        }
        // On the normal path the consumers have waited for every fill.  If
        // they stopped releasing stages, let the fills still unconsumed
        // (at most one per stage) land before the CTA exits (bounded).
        if (failed && lane == 0)
            for (int j = max(0, k - St::NST); j < k; j++)
                mbar_wait(&full[j % St::NST], (unsigned)((j / St::NST) & 1), kWaitLimit);
    } else {
        // consumers
        const int lx = tid % (St::TW / 2), r0 = tid / (St::TW / 2);
        bool waited = !a.early;
        for (int i = 0;; i++) {
            const int s = i % St::NST;
            if (!mbar_wait(&full[s], (unsigned)((i / St::NST) & 1), kWaitLimit)) {
                if (lane == 0) atomicOr(a.error_word, 2u);
                break;
            }
            const int4 sl = get_slot(&slot[s]);
            if (sl.x == -1) break;
            if (sl.w && !waited) {
                asm volatile("griddepcontrol.wait;" ::: "memory");
                waited = true;
            }
            if (sl.x < 0) {
                if (MODE == kModeFull) special_chunk<T, OP, MODE>(sa, -2 - sl.x, tid, v, a.sr_seed);
                else special_chunk<T, OP, MODE>(a, -2 - sl.x, tid, v, a.sr_seed);
            } else {
                const float* ibf = sl.w ? a.ibm_force : nullptr;
                const int x0 = sl.y + 2 * lx;
#pragma unroll 1
                for (int r = r0; r < TH; r += St::ROWS) {
                    const int y = sl.z + r;
                    // parity 1: not on the perimeter; parity 0: both nodes in the
                    // lattice; either way, not marked for the general path
                    bool live = P ? (y > 0 && y < a.g.ny - 1 && x0 > 0 && x0 + 1 < a.g.nx - 1)
                                  : (y < a.g.ny && x0 + 1 < a.g.nx);
                    if (live && a.special_bits) {
                        const long long unit = ((long long)y * a.g.pitch + x0) >> 1;
                        live = ((a.special_bits[unit >> 5] >> (unit & 31)) & 1u) == 0;
                    }
                    if (live)
                        interior_unit<T, OP, P, TW, TH, MODE>(a, bufs + (size_t)s * St::STAGE_ELEMS, r, lx, x0, y,
                                                              v, a.sr_seed, ibf);
                }
            }
            __syncwarp();
            if (lane == 0) mbar_arrive(&empty[s]);
        }
    }
    // an early-started grid finishes only after the grid it overlapped
    if (a.early) asm volatile("griddepcontrol.wait;" ::: "memory");
    // kModeSums: each CTA adds its totals and is done (the next launch
    // publishes them); kModeFull: the last CTA publishes
    if (MODE == kModeSums) cta_sums(a.partials, v);
    else if (MODE == kModeFull && a.partials) block_sums(a, v, (long long)a.g.nx * a.g.ny);
}


// The CM_OPT average terms of one node from its post-stream, post-boundary
// populations f: rho, rho |u| (force-corrected u, Brinkman included) and the
// raw |Pi| (update_avg_mag, macroscopics.cuh:50-120).  One division: u is
// (j + F/2) times 1 / rho.
__device__ __forceinline__ void opt_terms(const StepArgs& a, long long off, const float f[9], Acc v[kNumSums]) {
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
    float ux = fmaf(0.5f, Fx, jx) * inv;
    float uy = fmaf(0.5f, Fy, jy) * inv;
    if (a.gamma) brinkman<float>(a.gamma[off], rho, ux, uy, Fx, Fy);
    const float pxx = f[1] + f[3] + f[5] + f[6] + f[7] + f[8];
    const float pyy = f[2] + f[4] + f[5] + f[6] + f[7] + f[8];
    const float pxy = f[5] - f[6] + f[7] - f[8];
    v[0] += fix(rho);
    v[4] += fix(rho * sqrtf(ux * ux + uy * uy));
    v[5] += fix(sqrtf(pxx * pxx + 2.0f * pxy * pxy + pyy * pyy));
}

// Grid averages <rho>, <rho |u|>, <|Pi|> of the current step before any
// collision (update_avg_mag, macroscopics.cuh:50-120), for CM_OPT.  The nodes
// split as in the step kernel.  Units the tiles take (special bit clear; in a
// neighbour-access step also off the perimeter) load their 18 populations
// directly, one unit of two x-neighbours per thread over row segments of
// 2 * kThreads nodes; the pairs that do not shift in x are single aligned
// loads.  The parity's general-path units are spread over every thread of
// the grid, one node each, through the general path.  The terms are summed
// in exact fixed point, so the averages do not depend on the order.
template <typename T>
__global__ void __launch_bounds__(kThreads, kCtasPerSm) opt_prepass_kernel(const StepArgs a) {
    asm volatile("griddepcontrol.wait;" ::: "memory");
    asm volatile("griddepcontrol.launch_dependents;" :::);
    Acc v[kNumSums] = {0, 0, 0, 0, 0, 0};
    const Geometry& g = a.g;
    const T* F = static_cast<const T*>(a.f);
    const int seg_w = 2 * kThreads;
    const int segs = (g.nx + seg_w - 1) / seg_w;
    const int items = segs * g.ny;
    for (int it = blockIdx.x; it < items; it += gridDim.x) {
        const int y = it / segs;
        const int x0 = (it - y * segs) * seg_w + 2 * (int)threadIdx.x;
        if (x0 + 1 >= g.nx) continue;  // a lone last node is a general-path unit
        if (a.parity && !(y > 0 && y < g.ny - 1 && x0 > 0 && x0 + 1 < g.nx - 1)) continue;
        const long long n0 = (long long)y * g.pitch + x0;
        if (a.special_bits) {
            const long long unit = n0 >> 1;
            if ((a.special_bits[unit >> 5] >> (unit & 31)) & 1u) continue;
        }
        float f0[9], f1[9];
        const float2 r = Store<T>::ld2(F + a.rest_plane * g.plane + n0, WQ(0));
        f0[0] = r.x;
        f1[0] = r.y;
#pragma unroll
        for (int q = 1; q < 9; q++) {
            if (!a.parity) {
                const float2 p = Store<T>::ld2(F + q * g.plane + n0, WQ(q));
                f0[q] = p.x;
                f1[q] = p.y;
            } else if (CX(q) == 0) {
                const float2 p = Store<T>::ld2(F + OPP(q) * g.plane + n0 - CY(q) * g.pitch, WQ(q));
                f0[q] = p.x;
                f1[q] = p.y;
            } else {
                const T* src = F + OPP(q) * g.plane + n0 - CY(q) * g.pitch - CX(q);
                f0[q] = Store<T>::ld(src, WQ(q));
                f1[q] = Store<T>::ld(src + 1, WQ(q));
            }
        }
        opt_terms(a, n0, f0, v);
        opt_terms(a, n0 + 1, f1, v);
    }
    const int nthreads = gridDim.x * kThreads;
    for (int k = blockIdx.x * kThreads + threadIdx.x; k < 2 * a.nspecial; k += nthreads) {
        const int off = a.special_units[k >> 1] + (k & 1);
        const int y = off / g.pitch, x = off - y * g.pitch;
        if (x >= g.nx) continue;
        float f[9];
        unsigned outmask;
        gather_node<T>(a, x, y, f, &outmask);
        opt_terms(a, off, f, v);
    }
    block_sums(a, v, (long long)g.nx * g.ny);
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
    asm volatile("griddepcontrol.wait;" ::: "memory");
    asm volatile("griddepcontrol.launch_dependents;" :::);
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
        load_post_stream<T>(a, ix, iy, a.flags[(long long)iy * a.g.pitch + ix], f, &m);
#pragma unroll
        for (int q = 0; q < 9; q++) A[q] = f[q];
    } else if (fl == LBMX_PRESSURE_OUTLET) {
        // interior node = node - 1 (pressureOutlet.cuh:12-14); x >= 1 is enforced at set_flags
        load_post_stream<T>(a, x - 1, y, a.flags[(long long)y * a.g.pitch + x - 1], f, &m);
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
        load_post_stream<T>(a, dx, dy, a.flags[(long long)dy * a.g.pitch + dx], f, &m);
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
    const int x = blockIdx.x * 32 + threadIdx.x;
    const int y = blockIdx.y * 4 + threadIdx.y;
    if (x >= a.g.nx || y >= a.g.ny) return;
    const long long n = (long long)a.g.nx * a.g.ny;
    const long long dn = (long long)y * a.g.nx + x;
    const long long off = (long long)y * a.g.pitch + x;
    const float rho = rho_in[dn], ux = u_in[dn], uy = u_in[n + dn];
    float fe[9];
    init_equilibrium(rho, ux, uy, fe);
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
    const int x = blockIdx.x * 32 + threadIdx.x;
    const int y = blockIdx.y * 4 + threadIdx.y;
    if (x >= a.g.nx || y >= a.g.ny) return;
    const Geometry& g = a.g;
    const long long n = (long long)g.nx * g.ny;
    const long long dn = (long long)y * g.nx + x;
    const long long row = (long long)y * g.pitch;
    const T* F = static_cast<const T*>(a.f);
    const uint8_t fl = a.flags ? a.flags[row + x] : (uint8_t)0;
    out[dn] = Store<T>::ld(F + a.rest_plane * g.plane + row + x, WQ(0));
    const float nan = __int_as_float(0x7fc00000);
#pragma unroll
    for (int q = 1; q < 9; q++) {
        float v;
        if (!last_parity) {
            v = Store<T>::ld(F + OPP(q) * g.plane + row + x, WQ(q));
        } else {
            int dx = x + CX(q), dy = y + CY(q);
            bool out_d = false;
            if (dx < 0 || dx >= g.nx) { if (g.periodic_x) dx = dx < 0 ? dx + g.nx : dx - g.nx; else out_d = true; }
            if (dy < 0 || dy >= g.ny) { if (g.periodic_y) dy = dy < 0 ? dy + g.ny : dy - g.ny; else out_d = true; }
            if (!out_d) {
                v = Store<T>::ld(F + q * g.plane + (long long)dy * g.pitch + dx, WQ(q));
            } else if (is_halfway(fl)) {
                // reflected into the node's own slot OPP(q), minus the wall term
                v = Store<T>::ld(F + OPP(q) * g.plane + row + x, WQ(q)) + wall_term(a, q, fl);
            } else {
                int sx = x - CX(q), sy = y - CY(q);
                bool out_s = (!g.periodic_x && (sx < 0 || sx >= g.nx)) || (!g.periodic_y && (sy < 0 || sy >= g.ny));
                v = out_s ? a.edge[((long long)1 * g.perimeter + edge_index(x, y, g.nx, g.ny)) * 9 + q] : nan;
            }
        }
        out[q * n + dn] = v;
    }
}

// The IBM of one step in one CTA: density and uncorrected velocity of the
// patch nodes (the reference interpolates from d_rho and the copy of d_u
// taken before the force correction, IBMManager.cuh:227-228), gathered
// straight into shared memory, then the multi-direct rounds
// (ibm_fast_iterate, lbmx_ibm.cuh).  The stencils, spread lists, patch node
// offsets and flags do not depend on the flow, so they are staged before the
// wait for the previous step.  Launched with programmatic stream
// serialization like the step kernel: it waits for the previous step before
// reading the populations and lets the next step kernel launch and wait
// behind it.
template <typename T>
__global__ void __launch_bounds__(kIbmThreads) ibm_step_kernel(const StepArgs a, const IbmArgs ib) {
    extern __shared__ float4 sm4[];
    const IbmFast s = ibm_fast_layout(ib, sm4);
    ibm_fast_stage(ib, s, a.flags);
    __syncthreads();
    asm volatile("griddepcontrol.wait;" ::: "memory");
    asm volatile("griddepcontrol.launch_dependents;" :::);
    for (int i = threadIdx.x; i < ib.npatch; i += blockDim.x) {
        const int off = s.pn[i];
        const uint8_t fl = s.pf[i];
        const int y = off / a.g.pitch, x = off - y * a.g.pitch;
        float f[9];
        unsigned m;
        load_post_stream<T>(a, x, y, fl, f, &m);  // gather_node with the staged flag
        if (fl) apply_bc(a, f, x, y, fl);
        float rho = 0.f, jx = 0.f, jy = 0.f;
#pragma unroll
        for (int q = 0; q < 9; q++) {
            rho += f[q];
            jx += (float)CX(q) * f[q];
            jy += (float)CY(q) * f[q];
        }
        const float inv = 1.0f / rho;
        s.ps[i] = make_float4(jx * inv, jy * inv, rho, 1.0f / (2.0f * rho));
    }
    __syncthreads();
    ibm_fast_iterate(ib, s);
    // drag and lift of the step: minus the summed marker forces, in FP64,
    // each lane taking every 32nd marker, then a fixed shuffle tree
    if (ib.force_series && threadIdx.x < 32) {
        double dx = 0.0, dy = 0.0;
        for (int k = threadIdx.x; k < ib.nm; k += 32) {
            const float2 m = s.mt[k];
            dx += (double)m.x;
            dy += (double)m.y;
        }
        for (int o = 16; o > 0; o >>= 1) {
            dx += __shfl_xor_sync(0xffffffffu, dx, o);
            dy += __shfl_xor_sync(0xffffffffu, dy, o);
        }
        if (threadIdx.x == 0) {
            ib.force_series[0] = -dx;
            ib.force_series[1] = -dy;
        }
    }
}

template <typename T, int OP, int P, int MODE>
static cudaError_t launch_step_variant(const StepArgs& a, const CUtensorMap& tmap, unsigned grid, cudaStream_t s) {
    // the staged ring needs more than the default 48 KB; set once per device
    static unsigned long long configured = 0;
    int dev = 0;
    cudaGetDevice(&dev);
    if (!(configured >> (dev & 63) & 1ull)) {
        cudaError_t e = cudaFuncSetAttribute(
            step_kernel<T, OP, P, MODE>, cudaFuncAttributeMaxDynamicSharedMemorySize,
            (int)Staging<T, step_tile_w((int)sizeof(T)), step_tile_h((int)sizeof(T))>::SMEM);
        if (e != cudaSuccess) return e;
        configured |= 1ull << (dev & 63);
    }
    // launched with programmatic stream serialization: a step that directly
    // follows another overlaps its launch and prologue with that one's tail
    // (the kernel waits on griddepcontrol.wait before its first dependent access)
    cudaLaunchConfig_t cfg;
    memset(&cfg, 0, sizeof(cfg));
    cfg.gridDim = dim3(grid);
    cfg.blockDim = dim3(kThreads);
    cfg.dynamicSmemBytes = Staging<T, step_tile_w((int)sizeof(T)), step_tile_h((int)sizeof(T))>::SMEM;
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, step_kernel<T, OP, P, MODE>, a, tmap);
}

template <typename T, int OP, int P>
static cudaError_t launch_step_lean(const StepArgs& a, const CUtensorMap& tmap, unsigned grid, cudaStream_t s) {
    switch (step_mode(a)) {
    case kModeLean: return launch_step_variant<T, OP, P, kModeLean>(a, tmap, grid, s);
    case kModeSums: return launch_step_variant<T, OP, P, kModeSums>(a, tmap, grid, s);
    default: return launch_step_variant<T, OP, P, kModeFull>(a, tmap, grid, s);
    }
}

template <typename T>
cudaError_t launch_step(const StepArgs& a, const CUtensorMap& tmap, int op, cudaStream_t s) {
    const unsigned grid = (unsigned)a.num_ctas;
#define LBMX_STEP_CASE(OPV)                                                    \
    return a.parity ? launch_step_lean<T, OPV, 1>(a, tmap, grid, s)            \
                    : launch_step_lean<T, OPV, 0>(a, tmap, grid, s);
    switch (op) {
    case LBMX_BGK: LBMX_STEP_CASE(LBMX_BGK)
    case LBMX_MRT: LBMX_STEP_CASE(LBMX_MRT)
    case LBMX_CM: LBMX_STEP_CASE(LBMX_CM)
    default: LBMX_STEP_CASE(LBMX_CM_OPT)
    }
#undef LBMX_STEP_CASE
}

// A launch with programmatic stream serialization: the kernel may start
// during the previous grid's tail and waits in griddepcontrol.wait before
// its first dependent access (the pre-passes and the IBM kernel sit between
// two step kernels, which are launched the same way).
template <typename... KArgs, typename... Args>
static cudaError_t launch_pdl(void (*kernel)(KArgs...), unsigned grid, unsigned block, cudaStream_t s,
                              Args... args) {
    cudaLaunchConfig_t cfg;
    memset(&cfg, 0, sizeof(cfg));
    cfg.gridDim = dim3(grid);
    cfg.blockDim = dim3(block);
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, kernel, args...);
}

template <typename T>
cudaError_t launch_opt_prepass(const StepArgs& a, cudaStream_t s) {
    return launch_pdl(opt_prepass_kernel<T>, (unsigned)a.num_ctas, kThreads, s, a);
}

template <typename T>
cudaError_t launch_edge_prepass(const StepArgs& a, float* aux, cudaStream_t s) {
    return launch_pdl(edge_prepass_kernel<T>, (unsigned)((a.g.perimeter + 127) / 128), 128u, s, a, aux);
}

template <typename T>
cudaError_t launch_init(const StepArgs& a, const float* rho, const float* u, cudaStream_t s) {
    const dim3 grid((a.g.nx + 31) / 32, (a.g.ny + 3) / 4);
    init_kernel<T><<<grid, dim3(32, 4), 0, s>>>(a, rho, u, a.rest_plane == 9 ? 1 : 0);
    return cudaGetLastError();
}

template <typename T>
cudaError_t launch_get_populations(const StepArgs& a, float* out, cudaStream_t s) {
    const dim3 grid((a.g.nx + 31) / 32, (a.g.ny + 3) / 4);
    get_populations_kernel<T><<<grid, dim3(32, 4), 0, s>>>(a, out, a.parity);
    return cudaGetLastError();
}

template <typename T>
cudaError_t launch_ibm_step(const StepArgs& a, const IbmArgs& ib, cudaStream_t s) {
    if (ib.npatch <= 0) return cudaSuccess;
    const size_t smem = ibm_fast_smem_bytes(ib.npatch, ib.nm, ib.stencil);
    // the attribute grows with the patch: raise it when a larger one comes
    static int configured[64] = {0};
    int dev = 0;
    cudaGetDevice(&dev);
    if ((int)smem > configured[dev & 63]) {
        cudaError_t e = cudaFuncSetAttribute(ibm_step_kernel<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return e;
        configured[dev & 63] = (int)smem;
    }
    cudaLaunchConfig_t cfg;
    memset(&cfg, 0, sizeof(cfg));
    cfg.gridDim = dim3(1);
    cfg.blockDim = dim3(kIbmThreads);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, ibm_step_kernel<T>, a, ib);
}

#define LBMX_INSTANTIATE(T)                                                                              \
    template cudaError_t launch_step<T>(const StepArgs&, const CUtensorMap&, int, cudaStream_t);         \
    template cudaError_t launch_opt_prepass<T>(const StepArgs&, cudaStream_t);                           \
    template cudaError_t launch_edge_prepass<T>(const StepArgs&, float*, cudaStream_t);                  \
    template cudaError_t launch_init<T>(const StepArgs&, const float*, const float*, cudaStream_t);      \
    template cudaError_t launch_get_populations<T>(const StepArgs&, float*, cudaStream_t);               \
    template cudaError_t launch_ibm_step<T>(const StepArgs&, const IbmArgs&, cudaStream_t);

}  // namespace lbmx
