// lbmx_internal.h -- structures shared by the host launcher and the kernels.
#pragma once
#include <stdint.h>
#include <cuda.h>  // CUtensorMap (the descriptor type only; no driver calls are linked)
#include <cuda_runtime.h>

namespace lbmx {

// Geometry and storage of one lattice in HBM.
//
// Populations: plane-major SoA, plane q at f + q*plane, row pitch `pitch`
// elements (a multiple of 32 so every row starts on a 128-byte line).  The
// in-place AA streaming pattern keeps one buffer: after a step of parity 0
// (and after init) slot OPP(q) of node x holds f*_q(x); after a step of
// parity 1 slot q of node x+c_q holds f*_q(x).  Plane 9 exists only with
// the rest-population quirk (f0 from two steps back, one plane per parity).
//
// Edge store: nodes on the domain perimeter keep, per parity, the
// post-collision value of every population whose upstream node lies outside
// a non-periodic domain; that value is what the reference's ping-pong
// buffers hand back two steps later (src/core/streaming/streaming.cu:20-21).
struct Geometry {
    int nx, ny, pitch;
    int periodic_x, periodic_y;
    long long plane;   // elements per population plane (ny * pitch)
    int perimeter;     // 2*nx + 2*(ny-2)
};

struct StepArgs {
    Geometry g;
    void* f;                 // population storage (float / __half / __nv_bfloat16)
    const uint8_t* flags;    // [ny][pitch] boundary flags, nullptr if all fluid
    float* edge;             // [2][perimeter][9]
    const float* aux;        // [perimeter][9] neighbour data for ZG / pressure / corner
    const float* force;      // [2][plane] per-node body force or nullptr
    const float* ibm_force;  // [2][plane] IBM force (zero away from markers) or nullptr
    const float* gamma;      // [plane] Brinkman solid fraction or nullptr
    const float* avg;        // CM_OPT grid averages {rho, |j|, |Pi|} (device)
    float* rho_out;          // [plane] moments written when non-null
    float* u_out;            // [2][plane]
    double* partials;        // one accumulator set of the grid sums (kAccPerSet) when non-null
    unsigned int* counter;   // last-block-done counter for the sums
    double* sums;            // [kNumSums] final sums
    double* series;          // or null: the sums' series entry (sums 0..2, then the kinetic
                             // energy when `ke`) is also written here (device-accessible)
    int ke;                  // the sums include the kinetic energy 1/2 rho |u|^2 (accumulator kSumKE)
    float* avg_out;          // averages produced by the last block (lagged CM_OPT / pre-pass)
    unsigned int* error_word;// bit 0: non-finite density seen, bit 1: a staging wait gave up
    int check_finite;        // look for non-finite densities this step
    uint32_t quirks;
    int parity;              // step index & 1; 1 = neighbour-access phase
    int rest_plane;          // plane that holds f0 this step (0 or 9)
    int sr;                  // 16-bit stores round stochastically (else to nearest)
    uint32_t sr_seed;        // sr_seed_of(step index) for the rounding hash
    uint32_t sr_unit_origin; // added to a node's unit offset in the rounding hash (a y-slab's rows in the whole lattice)
    long long st_off[9];     // byte offset, from a node's plane-0 element, of the slot its q-th
                             // post-collision population goes to this step (interior nodes)
    float omega;
    float S[9];
    float u_bc, wall_ux, wall_uy, rho_out_bc;
    float body_fx, body_fy;
    int forced;              // any non-zero force (body, field or IBM)
    // work split of the step kernel (lbmx_kernels.cuh)
    // The general path's units of this step (set_step picks the parity's):
    // a neighbour-access step (parity 1) takes every perimeter unit (the
    // tiles find them by position) and the units with a flagged node
    // (special_bits marks those off the perimeter); an own-node step
    // (parity 0) only units with a boundary functor, a fluid node reading
    // the edge store or a missing second node
    // (special_bits marks them all) -- there a half-way or moving wall node
    // reads and writes only its own slots, exactly as an interior node does.
    const int* special_units;      // unit offsets y*pitch + x0 handled by the general path
    int nspecial;
    int special_chunks;            // work items of kSpecialChunk special nodes that lead the work list
    // chunks from dep_chunk on hold units within one node of an IBM patch
    // node (the list puts those units last); they go after the early tiles.
    // With the tiles below, they are the only items that read what the IBM
    // kernel of this step writes or write what it reads.
    // dep_chunk = special_chunks: none.
    int dep_chunk;
    // tiles in tile_order from dep_tile on hold a node within one node of an
    // IBM patch node: they follow the dependent chunks and add the IBM force
    // (tile_order null: no IBM, tiles in place)
    const int* tile_order;
    int dep_tile;
    int early;                     // run the items before the dependent ones before waiting on the preceding grid
    const uint32_t* special_bits;  // 1 bit per unit (see above), or nullptr
    int tiles_x, tiles_y;          // tiles of kStageW x kStageH nodes covering the lattice
    int num_ctas;                  // persistent CTAs that walk the interior tiles
    unsigned long long* tile_counter;       // next work item to claim (this step's of two counters)
    unsigned long long* tile_counter_next;  // the other counter: zeroed at the start for the next step
    int tile_chunk;                    // consecutive tiles taken per claim
    // sums of the previous step left for this launch to publish (kModeSums
    // steps publish one launch late; see step_mode): accumulators, the
    // sums array, the series entry or null
    double* pub_acc;
    double* pub_sums;
    double* pub_series;
    long long* raw_sums;     // or null: the last CTA also writes the integer fixed-point sums [kNumSums]
};

// Seed of the stochastic-rounding hash for step index s (a Weyl sequence:
// every step of a run gets a different seed).
__host__ __device__ __forceinline__ uint32_t sr_seed_of(long long s) {
    return (uint32_t)s * 0x9E3779B9u + 0x7F4A7C15u;
}

// perimeter index of a node on the domain edge
__host__ __device__ inline int edge_index(int x, int y, int nx, int ny) {
    if (y == 0) return x;
    if (y == ny - 1) return nx + x;
    if (x == 0) return 2 * nx + (y - 1);
    return 2 * nx + (ny - 2) + (y - 1);
}

// host launchers (one translation unit per storage type)
// tmap: 3-D tiled TMA descriptor over the population planes,
// dims {pitch, ny, planes}, box {kStageW + 2 * 16 B of halo, kStageH, 1}
template <typename T>
cudaError_t launch_step(const StepArgs& a, const CUtensorMap& tmap, int op, cudaStream_t s);
template <typename T>
cudaError_t launch_edge_prepass(const StepArgs& a, float* aux, cudaStream_t s);
template <typename T>
cudaError_t launch_opt_prepass(const StepArgs& a, cudaStream_t s);
template <typename T>
cudaError_t launch_init(const StepArgs& a, const float* rho, const float* u, cudaStream_t s);
template <typename T>
cudaError_t launch_get_populations(const StepArgs& a, float* out, cudaStream_t s);
// IBM multi-direct forcing on the marker patch (lbmx_ibm.cu)
// The marker rounds' data; R is float for the engine and a tangent number
// for the tangent-linear model.
template <typename R>
struct IbmData {
    int nm, npatch, iters, stencil;     // stencil: 2 or 4 nodes per axis
    const int* sten_idx;                // [nm][stencil^2] patch index or -1
    const float* sten_w;                // [nm][stencil^2] kernel weight
    const int* spread;                  // [npatch + 1] offsets, then the stencil points of each patch node (ascending)
    const int* patch_nodes;             // [npatch] node offset (y*pitch + x)
    const R* patch_rho;                 // [npatch]
    const R* patch_u;                   // [2][npatch] uncorrected velocity
    R* marker_u;                        // [2][nm] last interpolated velocity
    R* marker_rho;                      // [nm]
    R* marker_force;                    // [2][nm] summed over iterations
    R* ibm_force;                       // [2][plane] dense Eulerian force
    double* force_series;               // this step's {drag, lift} entry or null (engine only)
    long long plane;
    int clamp;
    float ds;
};
using IbmArgs = IbmData<float>;
// the IBM of one step: patch gather and marker rounds (lbmx_kernels.cuh)
template <typename T>
cudaError_t launch_ibm_step(const StepArgs& a, const IbmArgs& ib, cudaStream_t s);

// Many lattices in one persistent launch (lbmx_batch.cu).  Work items are
// interior tiles and chunks of special units of every lattice; the
// persistent CTAs claim them from one counter in list order.
struct BatchArgs {
    const StepArgs* lat;          // [count] per-lattice arguments of this launch
    const CUtensorMap* tmaps;     // [count] TMA descriptors for the launch's tile width (64-byte aligned)
    const int2* items;            // {lattice, tile >= 0 | -(special chunk + 1)}
    int nitems;
    int chunk;                    // items claimed per atomic
    unsigned long long* counter;  // next item (reset by the last CTA)
    unsigned int* done;           // CTAs finished in this launch
    unsigned int* error_word;     // bit 1: a staging wait gave up
    unsigned int* step;           // step index of this launch (for the rounding hash; the last CTA advances it)
};
// tile shape tile_w x tile_h: 64 x 8, 128 x 4 or 128 x 8; op: BGK, MRT or CM;
// grid 0 only prepares the kernel (attributes) for a later graph capture
template <typename T>
cudaError_t launch_batch_step(const BatchArgs& b, int op, int parity, int tile_w, int tile_h, bool lean,
                              unsigned grid, cudaStream_t s);

// step-kernel geometry: an interior tile is 128 x 4 nodes; each of the 256
// consumer threads takes two x-neighbouring nodes of one row.  The batched
// kernel also runs 64 x 8 and 128 x 8 tiles.
constexpr int kStepThreads = 288;  // 8 consumer warps + 1 producer warp
constexpr int kConsumerWarps = 8;
// The grid sums of a step: 0-2 mass and momentum {rho, rho ux, rho uy},
// 3 the kinetic energy 1/2 rho |u|^2, 4-5 the CM_OPT average terms
// {rho |u|, |Pi|} (their third, <rho>, is sum 0 over the node count).  They
// go into kSumSlots copies of the kNumSums fixed-point accumulators (warp w
// of CTA b adds to slot (9 b + w) % kSumSlots), so few warps contend for one
// address; a handle holds two such sets, one per step parity.
constexpr int kNumSums = 6;
constexpr int kSumKE = 3;
constexpr int kSumSlots = 32;
constexpr int kAccPerSet = kSumSlots * kNumSums;
// the handle's sums buffer holds two more doubles after the sums: the
// drag / lift slot lbmx_step_forces copies pageable series from
constexpr int kSumForces = kNumSums;
constexpr int kSumsBufferLen = kNumSums + 2;

// Interior-path variant of a step launch:
//   kModeLean  no per-node force or Brinkman field, no moment store, no sums,
//              no finite check -- straight-line code;
//   kModeSums  the lean path plus the mass / momentum sums, published by the
//              next launch on the stream (or lbmx's publish kernel), so the
//              step itself ends with no fence or counter;
//   kModeFull  everything, decided per launch from the arguments (the
//              kinetic energy among them: one more live accumulator would
//              cost the kModeSums variants registers); the last CTA
//              publishes its own sums.
constexpr int kModeLean = 0, kModeSums = 1, kModeFull = 2;
inline int step_mode(const StepArgs& a) {
    const bool plain = !a.force && !a.gamma && !a.rho_out && !a.check_finite;
    if (plain && !a.partials) return kModeLean;
    if (plain && !a.avg_out && !a.ke) return kModeSums;
    return kModeFull;
}
// publishes the mass and momentum sums in acc (one accumulator set) into
// sums / series
cudaError_t launch_publish(double* acc, double* sums, double* series, cudaStream_t s);
constexpr int kCtasPerSm = 3;      // resident persistent CTAs per SM (72 registers per thread)
constexpr int kStageW = 128;
constexpr int kStageH = 4;
// The single-lattice kernel's tile shape for 16-bit storage, and the ring
// depth of 16-bit tiles larger than 512 nodes.  128 x 8 tiles, two units per
// consumer thread in a 3-stage ring, measured fastest on GB300 for 16-bit
// storage (issue-bound there: the per-tile work is spread over two units).
#ifndef LBMX_TW16
#define LBMX_TW16 128
#endif
#ifndef LBMX_TH16
#define LBMX_TH16 8
#endif
#ifndef LBMX_NST16
#define LBMX_NST16 3
#endif
constexpr int kStageW16 = LBMX_TW16;
constexpr int kStageH16 = LBMX_TH16;
// interior tile shape of the single-lattice step kernel, by element size
// (a tile of more than 512 nodes gives each consumer thread several units)
__host__ __device__ constexpr int step_tile_w(int elem_bytes) { return elem_bytes == 2 ? kStageW16 : kStageW; }
__host__ __device__ constexpr int step_tile_h(int elem_bytes) { return elem_bytes == 2 ? kStageH16 : kStageH; }
constexpr int kSpecialChunk = kConsumerWarps * 32;  // special nodes per work item (one per consumer thread)
// guard elements before and after the population planes: staged row copies
// reach one 16-byte chunk beyond a row segment on each side
constexpr int kGuardElems = 64;

}  // namespace lbmx
