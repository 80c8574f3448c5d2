// lbmx_batch_kernels.cuh -- many independent lattices advanced by one
// persistent launch, instantiated once per storage type by
// lbmx_batch_{f32,f16,bf16}.cu.
//
// The reference steps one lattice per process (src/main.cu:96-114).  Here a
// work list holds, for every lattice of a batch, its interior tiles
// (TMA-staged, packed FP32x2 collision) followed by its chunks of special
// units (perimeter and flagged nodes, general path): the same two paths as the
// single-lattice step kernel, with the lattice read from the work item.  All
// CTAs are persistent and warp-specialised; the producer warp claims items
// from one counter, fills the stage ring with the item's tile (nothing for a
// special chunk) and hands the item index to the consumers.  The tile shape
// TW x TH is a template parameter (64 x 8, 128 x 4 or 128 x 8 nodes; each
// consumer thread takes TW * TH / 512 units of it) chosen by the batch
// autotuner.
#pragma once
#include "lbmx_kernels.cuh"

namespace lbmx {

template <typename T, int OP, int P, int TW, int TH, bool LEAN>
__global__ void __launch_bounds__(kThreads, (sizeof(T) == 4 && TW * TH > kStageW * kStageH) ? 2 : kCtasPerSm)
    batch_step_kernel(const BatchArgs b) {
    using St = Staging<T, TW, TH>;
    extern __shared__ __align__(128) unsigned char smem_raw[];
    T* bufs = reinterpret_cast<T*>(smem_raw);
    uint64_t* full = reinterpret_cast<uint64_t*>(smem_raw + St::BUF_BYTES);
    uint64_t* empty = full + St::NST;
    int4* slot = reinterpret_cast<int4*>(empty + St::NST);
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    // every lattice of the batch stands at this step index (the last CTA of
    // the previous launch advanced it)
    const uint32_t seed = sr_seed_of((long long)*b.step);
    if (tid == 0) {
        for (int s = 0; s < St::NST; s++) {
            mbar_init(&full[s], 1);
            mbar_init(&empty[s], kConsumerWarps);
        }
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();
    if (warp == kConsumerWarps) {
        int k = 0, next = 0, left = 0;
        bool failed = false;
        for (;; k++) {
            const int s = k % St::NST;
            if (k >= St::NST && !mbar_wait(&empty[s], (unsigned)(((k / St::NST) - 1) & 1), kWaitLimit)) {
                if (lane == 0) atomicOr(b.error_word, 2u);
                failed = true;
                break;
            }
            if (left == 0) {
                // the first claim of every CTA is its own block of items (no
                // atomic at the start); the counter hands out the rest
                int base = (int)blockIdx.x * b.chunk;
                if (k > 0) {
                    if (lane == 0)
                        base = (int)gridDim.x * b.chunk + (int)atomicAdd(b.counter, (unsigned long long)b.chunk);
                    base = __shfl_sync(0xffffffffu, base, 0);
                }
                next = base;
                left = b.chunk;
            }
            const int item = next++;
            left--;
            if (item >= b.nitems) {
                if (lane == 0) {
                    put_slot(&slot[s], -1, 0, 0, 0);
                    mbar_arrive(&full[s]);
                }
                break;
            }
            const int2 it = b.items[item];
            if (it.y < 0) {
                // a chunk of special nodes: nothing to stage
                if (lane == 0) {
                    put_slot(&slot[s], -2 - (-it.y - 1), 0, 0, it.x);
                    mbar_arrive(&full[s]);
                }
                __syncwarp();
                continue;
            }
            const StepArgs& a = b.lat[it.x];
            const int ty = it.y / a.tiles_x, tx = it.y - ty * a.tiles_x;
            const int x0 = tx * TW, y0 = ty * TH;
            if (lane == 0) {
                put_slot(&slot[s], it.y, x0, y0, it.x);
                fence_proxy_async_smem();
                mbar_expect_tx(&full[s], St::STAGE_BYTES);
            }
            __syncwarp();
            stage_issue<T, P, TW, TH>(a, b.tmaps + it.x, x0, y0, bufs + (size_t)s * St::STAGE_ELEMS, &full[s]);
        }
        if (failed && lane == 0)
            for (int j = max(0, k - St::NST); j < k; j++)
                mbar_wait(&full[j % St::NST], (unsigned)((j / St::NST) & 1), kWaitLimit);
    } else {
        Acc v[kNumSums] = {0, 0, 0, 0, 0, 0};  // unused: batched steps keep no grid sums
        const int lx = tid % (TW / 2), r0 = tid / (TW / 2);
        for (int i = 0;; i++) {
            const int s = i % St::NST;
            if (!mbar_wait(&full[s], (unsigned)((i / St::NST) & 1), kWaitLimit)) {
                if (lane == 0) atomicOr(b.error_word, 2u);
                break;
            }
            const int4 sl = get_slot(&slot[s]);
            if (sl.x == -1) break;
            const StepArgs& a = b.lat[sl.w];
            if (sl.x >= 0) {
                const int x0 = sl.y + 2 * lx;
#pragma unroll
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
                        interior_unit<T, OP, P, TW, TH, LEAN ? kModeLean : kModeFull>(a, bufs + (size_t)s * St::STAGE_ELEMS, r, lx, x0, y, v,
                                                              seed);
                }
            } else {
                special_chunk<T, OP, LEAN ? kModeLean : kModeFull>(a, -2 - sl.x, tid, v, seed);
            }
            __syncwarp();
            if (lane == 0) mbar_arrive(&empty[s]);
        }
    }
    // the last CTA to finish re-arms the item counter for the next launch
    if (tid == 0) {
        __threadfence();
        if (atomicAdd(b.done, 1u) == gridDim.x - 1) {
            *b.counter = 0ull;
            *b.done = 0u;
            *b.step += 1u;
            __threadfence();
        }
    }
}

// grid == 0: only set the kernel's shared-memory attribute (before a capture)
template <typename T, int OP, int P, int TW, int TH, bool LEAN>
static cudaError_t launch_batch_variant(const BatchArgs& b, unsigned grid, cudaStream_t s) {
    static unsigned long long configured = 0;
    int dev = 0;
    cudaGetDevice(&dev);
    if (!(configured >> (dev & 63) & 1ull)) {
        cudaError_t e = cudaFuncSetAttribute(batch_step_kernel<T, OP, P, TW, TH, LEAN>,
                                             cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             (int)Staging<T, TW, TH>::SMEM);
        if (e != cudaSuccess) return e;
        configured |= 1ull << (dev & 63);
    }
    if (grid == 0) return cudaSuccess;
    batch_step_kernel<T, OP, P, TW, TH, LEAN><<<grid, kThreads, Staging<T, TW, TH>::SMEM, s>>>(b);
    return cudaGetLastError();
}

template <typename T, int OP, int TW, int TH>
static cudaError_t launch_batch_shape(const BatchArgs& b, int parity, bool lean, unsigned grid, cudaStream_t s) {
    if (lean)
        return parity ? launch_batch_variant<T, OP, 1, TW, TH, true>(b, grid, s)
                      : launch_batch_variant<T, OP, 0, TW, TH, true>(b, grid, s);
    return parity ? launch_batch_variant<T, OP, 1, TW, TH, false>(b, grid, s)
                  : launch_batch_variant<T, OP, 0, TW, TH, false>(b, grid, s);
}

template <typename T, int OP>
static cudaError_t launch_batch_op(const BatchArgs& b, int parity, int tile_w, int tile_h, bool lean, unsigned grid,
                                   cudaStream_t s) {
    if (tile_w == 64 && tile_h == 8) return launch_batch_shape<T, OP, 64, 8>(b, parity, lean, grid, s);
    if (tile_w == 128 && tile_h == 4) return launch_batch_shape<T, OP, 128, 4>(b, parity, lean, grid, s);
    if (tile_w == 128 && tile_h == 8) return launch_batch_shape<T, OP, 128, 8>(b, parity, lean, grid, s);
    return cudaErrorInvalidValue;
}

template <typename T>
cudaError_t launch_batch_step(const BatchArgs& b, int op, int parity, int tile_w, int tile_h, bool lean,
                              unsigned grid, cudaStream_t s) {
    switch (op) {
    case LBMX_BGK: return launch_batch_op<T, LBMX_BGK>(b, parity, tile_w, tile_h, lean, grid, s);
    case LBMX_MRT: return launch_batch_op<T, LBMX_MRT>(b, parity, tile_w, tile_h, lean, grid, s);
    case LBMX_CM: return launch_batch_op<T, LBMX_CM>(b, parity, tile_w, tile_h, lean, grid, s);
    default: return cudaErrorInvalidValue;
    }
}

#define LBMX_INSTANTIATE_BATCH(T) \
    template cudaError_t launch_batch_step<T>(const BatchArgs&, int, int, int, int, bool, unsigned, cudaStream_t);

}  // namespace lbmx
