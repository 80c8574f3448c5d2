// lbmx_handle.h -- the state behind an lbmx_handle, shared by the C-ABI
// translation units (lbmx_api.cu, lbmx_batch.cu).
#pragma once
#include <cuda_bf16.h>
#include <cuda_fp16.h>

#include <vector>

#include "lbmx.h"
#include "lbmx_internal.h"

struct lbmx_handle {
    lbmx_params p;
    lbmx::Geometry g;
    cudaStream_t stream = nullptr;
    bool own_stream = false;
    void* f = nullptr;
    int nplanes = 9;
    uint8_t* flags = nullptr;      // device, pitched; null while every node is fluid
    bool has_aux_bc = false;
    float* edge = nullptr;         // [2][perimeter][9]
    float* aux = nullptr;          // [perimeter][9]
    float* force = nullptr;        // [2][plane] optional per-node body force
    float* ibm_force = nullptr;    // [2][plane]
    float* gamma = nullptr;        // [plane] Brinkman solid fraction, null: none
    float* rho_out = nullptr;      // [plane]
    float* u_out = nullptr;        // [2][plane]
    float* staging = nullptr;      // dense [3][n] upload / readback staging
    float* pop_out = nullptr;      // dense [9][n] readback staging
    double* partials = nullptr;    // [2][kAccPerSet] fixed-point grid accumulators of the step's sums
    unsigned int* counter = nullptr;
    double* sums = nullptr;        // [6]
    float* avg = nullptr;          // [3]
    unsigned int* error_word = nullptr;
    long long blocks = 0;
    long long t = 0;
    bool initialized = false;
    bool have_avg = false;
    bool ext_avg = false;          // the next step uses averages set by lbmx_set_averages
    uint32_t ghost_mask = 0;       // bit 0: row 0, bit 1: row ny-1 is a ghost row (never stepped)
    long long row_origin = 0;      // row of the whole lattice that handle row 0 stands for (y-slabs)
    int whole_ny = 0;              // rows of a y-periodic whole lattice (y-slabs), else 0
    long long* raw_sums = nullptr; // [kNumSums] integer sums of lbmx_opt_partials
    // immersed boundary
    int nm = 0, npatch = 0, stencil = 0;
    int* patch_nodes = nullptr;
    int* sten_idx = nullptr;
    float* sten_w = nullptr;
    int* spread = nullptr;         // spread lists of the patch nodes (IbmData::spread)
    float* marker_u = nullptr;
    float* marker_rho = nullptr;
    float* marker_force = nullptr;
    std::vector<int> patch_host;   // IBM patch node offsets
    // work split of the step kernel
    std::vector<uint8_t> flags_host;  // pitched copy of the flags (empty: all fluid)
    std::vector<uint8_t> flags_in;    // lbmx_set_flags' dense copy of the caller's flags
    // general-path units of a neighbour-access step (parity 1) and of an
    // own-node step (parity 0)
    int* special_units = nullptr;
    uint32_t* special_bits = nullptr;
    int* special_units0 = nullptr;
    uint32_t* special_bits0 = nullptr;
    uint32_t* bits_buf = nullptr;     // the storage behind special_bits / special_bits0 (which may be null)
    uint32_t* bits0_buf = nullptr;
    size_t cap_units = 0, cap_units0 = 0, cap_bits = 0, cap_bits0 = 0;  // bytes of the four buffers
    int nspecial0 = 0, special_chunks0 = 0;
    int dep_chunk = 0, dep_chunk0 = 0;  // first chunk of each list with units next to the IBM patch
    int* tile_order = nullptr;          // tiles away from the IBM patch, then the others (null without markers)
    int dep_tile = 0;                   // tiles away from the patch
    int nspecial = 0, special_chunks = 0, tiles_x = 0, tiles_y = 0, num_ctas = 0, num_sms = 1;
    void* f_alloc = nullptr;  // population allocation including the guard elements
    unsigned long long* tile_counter = nullptr;  // [2] work counters, alternating by step
    long long last_step = -2;      // step index of the last single-lattice launch
    double* pend_acc = nullptr;    // accumulators of a step whose sums are not yet published
    double* pend_series = nullptr; // and that step's series entry or null
    int tile_chunk = 1;            // neighbour-access steps (num_ctas, tile_chunk) and own-node
    int num_ctas0 = 0, tile_chunk0 = 1;  // steps (num_ctas0, tile_chunk0)
    CUtensorMap tmap;  // the type carries the 64-byte alignment TMA needs  // TMA descriptor of the population planes
    long long partial_cap = 0;
    char err[512] = {0};
};

namespace lbmx {

size_t elem_size(int storage);
// kernel arguments of the handle's current configuration (no step yet)
StepArgs base_args(const lbmx_handle* h);
// parity and rest-population plane of step index s (1-based)
void set_step(const lbmx_handle* h, StepArgs& a, long long s);
// 3-D tiled TMA descriptor over the population planes for tile_w x tile_h tiles
bool encode_population_map(const lbmx_handle* h, CUtensorMap* out, int tile_w, int tile_h);
// Peskin stencils of n markers (host array xy[2k], xy[2k+1]) on an nx x ny
// lattice with row pitch `pitch`: sidx / sw [n][S*S] (S = 2 or 4) patch index
// (-1 outside the lattice) and weight, nodes the patch's node offsets.
// Returns -1, or the index of the first non-finite marker.
int ibm_build_stencil(int nx, int ny, long long pitch, bool two_by_two, const float* xy, int n,
                      std::vector<int>& sidx, std::vector<float>& sw, std::vector<int>& nodes);
// Spread lists of a stencil over np patch nodes: [np + 1] offsets, then for
// each patch node the stencil points (indices into sidx) that touch it, in
// ascending order.
std::vector<int> ibm_build_spread(int np, const std::vector<int>& sidx);

template <typename Fn>
cudaError_t dispatch(int storage, Fn fn) {
    switch (storage) {
    case LBMX_STORAGE_F16_OFFSET: return fn(__half());
    case LBMX_STORAGE_BF16_OFFSET: return fn(__nv_bfloat16());
    default: return fn(float());
    }
}

}  // namespace lbmx
