// lbmx_api.cu -- the C-ABI of liblbmx.so: handle lifetime, uploads, the
// per-step launch sequence, readback and error reporting.
#include <cuda_bf16.h>
#include <cuda_fp16.h>

#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <string>
#include <unordered_map>
#include <algorithm>
#include <vector>

#include "lbmx_handle.h"

namespace lbmx {
size_t ibm_smem_bytes(int npatch, int nm, int stencil);
}

using namespace lbmx;

static char g_create_err[512];

static lbmx_status fail(lbmx_handle* h, lbmx_status code, const char* fmt, ...) {
    char* dst = h ? h->err : g_create_err;
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(dst, 512, fmt, ap);
    va_end(ap);
    return code;
}

#define LBMX_CUDA(h, call)                                                                          \
    do {                                                                                           \
        cudaError_t e_ = (call);                                                                   \
        if (e_ != cudaSuccess)                                                                     \
            return fail((h), e_ == cudaErrorMemoryAllocation ? LBMX_ERR_OUT_OF_MEMORY : LBMX_ERR_CUDA, \
                        "%s: %s (%s:%d)", #call, cudaGetErrorString(e_), __FILE__, __LINE__);        \
    } while (0)

size_t lbmx::elem_size(int storage) { return storage == LBMX_STORAGE_F32 ? 4 : 2; }

// 3-D tiled TMA descriptor over the population planes: dims {nx, ny,
// planes}, row stride pitch; box {tile_w + 2 chunks of 16 bytes, tile_h, 1};
// out-of-range elements read as zero.  cuTensorMapEncodeTiled comes from the driver
// through the runtime's entry-point query (no link against libcuda).
typedef CUresult (*EncodeTiledFn)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                  const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                  CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

bool lbmx::encode_population_map(const lbmx_handle* h, CUtensorMap* out, int tile_w, int tile_h) {
    static EncodeTiledFn encode = nullptr;
    if (!encode) {
        void* fn = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q) !=
                cudaSuccess ||
            q != cudaDriverEntryPointSuccess || !fn)
            return false;
        encode = reinterpret_cast<EncodeTiledFn>(fn);
    }
    const int es = (int)elem_size(h->p.storage);
    const CUtensorMapDataType dt = h->p.storage == LBMX_STORAGE_F32 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT32
                                   : h->p.storage == LBMX_STORAGE_F16_OFFSET ? CU_TENSOR_MAP_DATA_TYPE_FLOAT16
                                                                             : CU_TENSOR_MAP_DATA_TYPE_BFLOAT16;
    // the row extent is nx, not the padded pitch: box columns past the
    // lattice are zero-filled by the TMA unit without reading memory
    const cuuint64_t dims[3] = {(cuuint64_t)h->g.nx, (cuuint64_t)h->g.ny, (cuuint64_t)h->nplanes};
    const cuuint64_t strides[2] = {(cuuint64_t)h->g.pitch * es, (cuuint64_t)h->g.plane * es};
    const cuuint32_t box[3] = {(cuuint32_t)(tile_w + 2 * 16 / es), (cuuint32_t)tile_h, 1u};
    const cuuint32_t estr[3] = {1u, 1u, 1u};
    return encode(out, dt, 3, h->f, dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
                  CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                  CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

StepArgs lbmx::base_args(const lbmx_handle* h) {
    StepArgs a;
    memset(&a, 0, sizeof(a));
    a.g = h->g;
    a.f = h->f;
    a.flags = h->flags;
    a.edge = h->edge;
    a.aux = h->aux;
    a.force = h->force;
    a.ibm_force = h->nm > 0 ? h->ibm_force : nullptr;
    a.gamma = h->gamma;
    a.avg = h->avg;
    a.quirks = h->p.quirks;
    a.omega = h->p.omega;
    for (int i = 0; i < 9; i++) a.S[i] = h->p.S[i];
    a.u_bc = h->p.u_bc;
    a.wall_ux = h->p.wall_ux;
    a.wall_uy = h->p.wall_uy;
    a.rho_out_bc = h->p.rho_out;
    a.body_fx = h->p.body_fx;
    a.body_fy = h->p.body_fy;
    a.forced = (h->p.body_fx != 0.0f || h->p.body_fy != 0.0f || h->force != nullptr || h->nm > 0 ||
                h->gamma != nullptr) ? 1 : 0;
    a.special_units = h->special_units;
    a.nspecial = h->nspecial;
    a.special_chunks = h->special_chunks;
    a.dep_chunk = h->dep_chunk;
    a.tile_order = h->tile_order;
    a.dep_tile = h->dep_tile;
    a.special_bits = h->special_bits;
    a.tiles_x = h->tiles_x;
    a.tiles_y = h->tiles_y;
    a.num_ctas = h->num_ctas;
    a.error_word = h->error_word;
    a.tile_chunk = h->tile_chunk;
    a.sr = (h->p.storage != LBMX_STORAGE_F32 && !(h->p.options & LBMX_OPTION_ROUND_NEAREST)) ? 1 : 0;
    a.sr_unit_origin = (uint32_t)((unsigned long long)(h->row_origin * h->g.pitch) >> 1);
    return a;
}

// Split the lattice between the two kinds of step-kernel work items: units
// (two x-neighbouring nodes, x0 even) on the perimeter or holding a flagged
// node take the general path; the kernel finds perimeter units by position
// and the others through a bit per unit.  IBM patch nodes stay in the tiles,
// which add the IBM force when they hold one.
static lbmx_status rebuild_special(lbmx_handle* h) {
    const Geometry& g = h->g;
    const int units_per_row = g.pitch / 2;
    const uint8_t* F = h->flags_host.empty() ? nullptr : h->flags_host.data();  // pitched, zero past nx
    bool any_interior = false;
    std::vector<int> units, units0;
    std::vector<uint32_t> bits(((size_t)g.ny * units_per_row + 31) / 32, 0u), bits0(bits.size(), 0u);
    const auto set_bit = [](std::vector<uint32_t>& b, size_t u) { b[u >> 5] |= 1u << (u & 31); };
    // an own-node step (parity 0) runs a node through the tiles unless it has
    // a boundary functor or (fluid on a non-periodic edge) reads the edge store
    const auto plain0 = [](uint8_t f, bool edge) {
        return f == LBMX_HALFWAY_BB || f == LBMX_MOVING_WALL_BB || (f == LBMX_FLUID && !edge);
    };
    for (int y = 0; y < g.ny; y++) {
        const uint8_t* row = F ? F + (size_t)y * g.pitch : nullptr;
        const size_t u_row = (size_t)y * units_per_row;
        // ghost rows (a y-slab's copies of its neighbours' boundary rows) are
        // in no unit list; parity 0 marks them so the tiles skip them too,
        // parity 1 tiles skip them as perimeter rows
        if (((h->ghost_mask & 1u) && y == 0) || ((h->ghost_mask & 2u) && y == g.ny - 1)) {
            for (int x0 = 0; x0 < g.nx; x0 += 2) set_bit(bits0, u_row + x0 / 2);
            continue;
        }
        const bool yedge = y == 0 || y == g.ny - 1;
        const bool open_y = !g.periodic_y && yedge;
        // a y-slab of a y-periodic lattice: the lattice's first and last
        // rows take the general path of a neighbour-access step, as there
        const long long wy = h->whole_ny > 0 ? ((h->row_origin + y) % h->whole_ny + h->whole_ny) % h->whole_ny : -1;
        const bool wrap_row = h->whole_ny > 0 && (wy == 0 || wy == h->whole_ny - 1);
        const auto unit = [&](int x0) {
            const bool pair = x0 + 1 < g.nx;
            const uint8_t f0 = row ? row[x0] : (uint8_t)LBMX_FLUID;
            const uint8_t f1 = row && pair ? row[x0 + 1] : (uint8_t)LBMX_FLUID;
            const bool perim = yedge || x0 == 0 || x0 + 1 >= g.nx - 1;
            const bool flagged = (f0 | f1) != 0;
            const size_t u = u_row + x0 / 2;
            if (perim || flagged || wrap_row) units.push_back(y * g.pitch + x0);
            if (!perim && (flagged || wrap_row)) {
                set_bit(bits, u);
                any_interior = true;
            }
            const bool e0 = open_y || (!g.periodic_x && (x0 == 0 || x0 == g.nx - 1));
            const bool e1 = open_y || (!g.periodic_x && x0 + 1 == g.nx - 1);
            if (!pair || !plain0(f0, e0) || !plain0(f1, e1)) {
                units0.push_back(y * g.pitch + x0);
                set_bit(bits0, u);
            }
        };
        // the units from last_start on are on the perimeter (x0 + 1 >= nx - 1)
        const int last_start = std::max(0, (g.nx - 1) & ~1);
        if (yedge || wrap_row) {
            for (int x0 = 0; x0 < g.nx; x0 += 2) unit(x0);
            continue;
        }
        // elsewhere in the row only a flagged unit can be in a list: skip
        // fluid nodes eight at a time
        unit(0);
        for (int x0 = 2; x0 < last_start;) {
            if (!row) break;
            if ((x0 & 7) == 0 && x0 + 8 <= last_start) {
                uint64_t w;
                memcpy(&w, row + x0, 8);
                if (w == 0) {
                    x0 += 8;
                    continue;
                }
            }
            if (row[x0] | row[x0 + 1]) unit(x0);
            x0 += 2;
        }
        for (int x0 = std::max(2, last_start); x0 < g.nx; x0 += 2) unit(x0);
    }
    // Work that touches the IBM patch goes last: with the IBM kernel still
    // running, the step kernel takes every other item first.  A node's update
    // reads and writes only its own AA slots and reads its own force entry,
    // and the IBM kernel reads the patch nodes' slots and writes their
    // forces; the margin of one node covers boundary functors that read a
    // neighbour.  In each list the units near the patch go last, and the
    // tiles near it follow all others.
    std::vector<char> near;
    if (!h->patch_host.empty()) {
        near.assign((size_t)g.plane, 0);
        for (int off : h->patch_host) {
            const int py = off / g.pitch, px = off % g.pitch;
            for (int dy = -1; dy <= 1; dy++)
                for (int dx = -1; dx <= 1; dx++) {
                    int x = px + dx, y = py + dy;
                    if (g.periodic_x) x = (x + g.nx) % g.nx;
                    if (g.periodic_y) y = (y + g.ny) % g.ny;
                    if (x >= 0 && x < g.nx && y >= 0 && y < g.ny) near[(size_t)y * g.pitch + x] = 1;
                }
        }
    }
    const auto by_patch = [&](std::vector<int>& list) {
        if (near.empty()) return (int)list.size();
        const auto it = std::stable_partition(list.begin(), list.end(), [&](int u) {
            return !near[(size_t)u] && !(u % g.pitch + 1 < g.nx && near[(size_t)u + 1]);
        });
        return (int)(it - list.begin());
    };
    const int indep = by_patch(units), indep0 = by_patch(units0);
    // device copies, in buffers that only grow (a cudaFree / cudaMalloc pair
    // per list cost about as much as building the lists); null unit bits:
    // none marked
    LBMX_CUDA(h, cudaStreamSynchronize(h->stream));
    const auto upload = [&](const void* src, size_t bytes, void** buf, size_t* cap) -> cudaError_t {
        if (!*buf || *cap < bytes) {
            cudaFree(*buf);
            *buf = nullptr;
            *cap = 0;
            const cudaError_t e = cudaMalloc(buf, std::max<size_t>(bytes, 4));
            if (e != cudaSuccess) return e;
            *cap = std::max<size_t>(bytes, 4);
        }
        return bytes ? cudaMemcpy(*buf, src, bytes, cudaMemcpyHostToDevice) : cudaSuccess;
    };
    LBMX_CUDA(h, upload(units.data(), units.size() * sizeof(int), (void**)&h->special_units, &h->cap_units));
    LBMX_CUDA(h, upload(units0.data(), units0.size() * sizeof(int), (void**)&h->special_units0, &h->cap_units0));
    h->special_bits = h->special_bits0 = nullptr;
    if (any_interior) {
        LBMX_CUDA(h, upload(bits.data(), bits.size() * sizeof(uint32_t), (void**)&h->bits_buf, &h->cap_bits));
        h->special_bits = h->bits_buf;
    }
    if (!units0.empty() || h->ghost_mask) {
        LBMX_CUDA(h, upload(bits0.data(), bits0.size() * sizeof(uint32_t), (void**)&h->bits0_buf, &h->cap_bits0));
        h->special_bits0 = h->bits0_buf;
    }
    h->nspecial = (int)units.size();
    h->special_chunks = (2 * h->nspecial + kSpecialChunk - 1) / kSpecialChunk;
    h->nspecial0 = (int)units0.size();
    h->special_chunks0 = (2 * h->nspecial0 + kSpecialChunk - 1) / kSpecialChunk;
    // a chunk is dependent from the one holding the first patch-adjacent unit
    h->dep_chunk = indep == h->nspecial ? h->special_chunks : 2 * indep / kSpecialChunk;
    h->dep_chunk0 = indep0 == h->nspecial0 ? h->special_chunks0 : 2 * indep0 / kSpecialChunk;
    const int es = (int)elem_size(h->p.storage);
    const int tw = step_tile_w(es), th = step_tile_h(es);
    h->tiles_x = (g.nx + tw - 1) / tw;
    h->tiles_y = (g.ny + th - 1) / th;
    cudaFree(h->tile_order);
    h->tile_order = nullptr;
    h->dep_tile = h->tiles_x * h->tiles_y;
    if (!near.empty()) {
        std::vector<int> first, last;
        for (int t = 0; t < h->tiles_x * h->tiles_y; t++) {
            const int ty = t / h->tiles_x, tx = t % h->tiles_x;
            bool touches = false;
            for (int y = ty * th; y < std::min(g.ny, ty * th + th) && !touches; y++)
                for (int x = tx * tw; x < std::min(g.nx, tx * tw + tw); x++)
                    if (near[(size_t)y * g.pitch + x]) {
                        touches = true;
                        break;
                    }
            (touches ? last : first).push_back(t);
        }
        h->dep_tile = (int)first.size();
        first.insert(first.end(), last.begin(), last.end());
        LBMX_CUDA(h, cudaMalloc((void**)&h->tile_order, first.size() * sizeof(int)));
        LBMX_CUDA(h, cudaMemcpy(h->tile_order, first.data(), first.size() * sizeof(int), cudaMemcpyHostToDevice));
    }
    // Persistent CTAs walk the work list, kCtasPerSm per SM, except in the
    // steps with general-path chunks of a lattice so small that three CTAs
    // per SM would get fewer than four items each: there two per SM.  A
    // chunk is one node per thread, a long chain of dependent loads and
    // arithmetic that a third CTA on the SM stretches (9 -> 14 us on a 1024^2
    // cavity); with only two or three tiles to follow it, its CTA then ends
    // last (the 1024^2 FP16 step with 128 x 8 tiles: 16.4 us flushed with
    // two CTAs per SM in its neighbour-access steps, 18.4 with three; the
    // FP32 step with 128 x 4 tiles: 16.4 with three, 18.4 with two).  With
    // IBM markers, two per SM below 16 items per CTA: the step's grid then
    // fits beside the IBM kernel's CTA it overlaps (the 2048 x 512 cylinder
    // 16.8 us a step with two, 17.3 with three).  Claims take about 1/16 of
    // a CTA's share: few atomics on large lattices, one item at a time on
    // small ones.
    const long long tiles = (long long)h->tiles_x * h->tiles_y;
    const long long few = (h->patch_host.empty() ? 4LL : 16LL) * kCtasPerSm * h->num_sms;
    const auto split = [&](int chunks, int* num_ctas, int* tile_chunk) {
        const long long items = tiles + chunks;
        const int per_sm = (items >= few || chunks == 0) ? kCtasPerSm : 2;
        *num_ctas = (int)std::max<long long>(1, std::min<long long>(items, (long long)per_sm * h->num_sms));
        *tile_chunk = (int)std::max<long long>(1, items / (16LL * *num_ctas));
    };
    split(h->special_chunks, &h->num_ctas, &h->tile_chunk);
    split(h->special_chunks0, &h->num_ctas0, &h->tile_chunk0);
    if (!h->partials) {
        // two sets (one per step parity) of kSumSlots copies of the six
        // fixed-point grid accumulators (zero between uses)
        LBMX_CUDA(h, cudaMalloc((void**)&h->partials, (size_t)2 * kAccPerSet * sizeof(double)));
        LBMX_CUDA(h, cudaMemset(h->partials, 0, (size_t)2 * kAccPerSet * sizeof(double)));
    }
    return LBMX_OK;
}

// A staged tile whose copies never completed (bit 1 of the error word) is a
// hard failure of the steps since the last check; the word is cleared.
static lbmx_status check_pipeline(lbmx_handle* h) {
    unsigned int w = 0;
    LBMX_CUDA(h, cudaMemcpyAsync(&w, h->error_word, sizeof(w), cudaMemcpyDeviceToHost, h->stream));
    LBMX_CUDA(h, cudaStreamSynchronize(h->stream));
    if (w & 2u) {
        LBMX_CUDA(h, cudaMemsetAsync(h->error_word, 0, sizeof(w), h->stream));
        return fail(h, LBMX_ERR_CUDA, "step kernel: a shared-memory staging wait gave up; results are invalid");
    }
    return LBMX_OK;
}

// parity and rest-population plane of step index s (1-based)
void lbmx::set_step(const lbmx_handle* h, StepArgs& a, long long s) {
    a.parity = (int)(s & 1);
    a.rest_plane = (h->p.quirks & LBMX_QUIRK_REST_LAG) ? (a.parity ? 9 : 0) : 0;
    a.sr_seed = sr_seed_of(s);
    // the general path's units of this parity
    a.special_units = a.parity ? h->special_units : h->special_units0;
    a.nspecial = a.parity ? h->nspecial : h->nspecial0;
    a.special_chunks = a.parity ? h->special_chunks : h->special_chunks0;
    a.dep_chunk = a.parity ? h->dep_chunk : h->dep_chunk0;
    a.num_ctas = a.parity ? h->num_ctas : h->num_ctas0;
    a.tile_chunk = a.parity ? h->tile_chunk : h->tile_chunk0;
    a.special_bits = a.parity ? h->special_bits : h->special_bits0;
    // two work counters, alternating by step: each launch zeroes the other
    a.tile_counter = h->tile_counter + (s & 1);
    a.tile_counter_next = h->tile_counter + ((s + 1) & 1);
    // interior store targets: parity 1 -> slot q of the node x + c_q,
    // parity 0 -> the node's own slot OPP(q) (D2Q9 order: rest, E, N, W, S, NE, NW, SW, SE)
    static const int cx[9] = {0, 1, 0, -1, 0, 1, -1, -1, 1};
    static const int cy[9] = {0, 0, 1, 0, -1, 1, 1, -1, -1};
    static const int opp[9] = {0, 3, 4, 1, 2, 7, 8, 5, 6};
    const long long es = (long long)elem_size(h->p.storage);
    const Geometry& g = h->g;
    a.st_off[0] = (long long)a.rest_plane * g.plane * es;
    for (int q = 1; q < 9; q++)
        a.st_off[q] = (a.parity ? (long long)q * g.plane + (long long)cy[q] * g.pitch + cx[q]
                                : (long long)opp[q] * g.plane) * es;
}

static void free_ibm(lbmx_handle* h) {
    cudaFree(h->patch_nodes); cudaFree(h->sten_idx); cudaFree(h->sten_w); cudaFree(h->spread);
    cudaFree(h->marker_u);
    cudaFree(h->marker_rho); cudaFree(h->marker_force); cudaFree(h->ibm_force);
    h->patch_nodes = nullptr; h->sten_idx = nullptr; h->sten_w = nullptr; h->spread = nullptr;
    h->marker_u = h->marker_rho = h->marker_force = h->ibm_force = nullptr;
    h->nm = h->npatch = 0;
    h->patch_host.clear();
}

extern "C" {

int32_t lbmx_version(void) { return LBMX_VERSION; }

void lbmx_params_default(lbmx_params* p) {
    if (!p) return;
    memset(p, 0, sizeof(*p));
    p->op = LBMX_BGK;
    p->storage = LBMX_STORAGE_F32;
    p->ibm_iters = 3;
    p->omega = 1.0f;
    for (int i = 0; i < 9; i++) p->S[i] = 1.0f;
    p->rho_out = 1.0f;
    p->ibm_ds = 1.0f;
}

void lbmx_destroy(lbmx_handle* h) {
    if (!h) return;
    int cur = 0;
    cudaGetDevice(&cur);
    cudaSetDevice(h->p.device);
    if (h->stream) cudaStreamSynchronize(h->stream);
    free_ibm(h);
    cudaFree(h->f_alloc); cudaFree(h->flags); cudaFree(h->edge); cudaFree(h->aux);
    cudaFree(h->force); cudaFree(h->gamma); cudaFree(h->rho_out); cudaFree(h->u_out); cudaFree(h->staging);
    cudaFree(h->pop_out); cudaFree(h->partials); cudaFree(h->counter); cudaFree(h->sums); cudaFree(h->raw_sums);
    cudaFree(h->avg); cudaFree(h->error_word); cudaFree(h->special_units); cudaFree(h->bits_buf);
    cudaFree(h->special_units0); cudaFree(h->bits0_buf); cudaFree(h->tile_order);
    cudaFree(h->tile_counter);
    if (h->own_stream && h->stream) cudaStreamDestroy(h->stream);
    cudaSetDevice(cur);
    delete h;
}

lbmx_status lbmx_create(const lbmx_params* p, lbmx_handle** out) {
    if (!out) return fail(nullptr, LBMX_ERR_INVALID_ARGUMENT, "lbmx_create: out is NULL");
    *out = nullptr;
    if (!p) return fail(nullptr, LBMX_ERR_INVALID_ARGUMENT, "lbmx_create: params is NULL");
    if (p->nx < 3 || p->ny < 3)
        return fail(nullptr, LBMX_ERR_INVALID_ARGUMENT, "lbmx_create: nx, ny must be >= 3 (got %d x %d)", p->nx, p->ny);
    // node offsets y * pitch + x are 32-bit in the work lists and tiles, so
    // the plane with its rows padded to whole tiles must fit
    const long long padded_plane = (long long)p->ny * (((long long)p->nx + kStageW - 1) / kStageW * kStageW);
    if (padded_plane > (1LL << 31) - 1)
        return fail(nullptr, LBMX_ERR_TOO_LARGE,
                    "lbmx_create: %d x %d nodes (%lld with rows padded to whole %d-node tiles) exceeds 2^31-1",
                    p->nx, p->ny, padded_plane, kStageW);
    if (p->op < LBMX_BGK || p->op > LBMX_CM_OPT)
        return fail(nullptr, LBMX_ERR_INVALID_ARGUMENT, "lbmx_create: unknown operator %d", p->op);
    if (p->storage < LBMX_STORAGE_F32 || p->storage > LBMX_STORAGE_BF16_OFFSET)
        return fail(nullptr, LBMX_ERR_INVALID_ARGUMENT, "lbmx_create: unknown storage %d", p->storage);
    if (cudaSetDevice(p->device) != cudaSuccess)
        return fail(nullptr, LBMX_ERR_CUDA, "lbmx_create: cannot select device %d", p->device);
    lbmx_handle* h = new lbmx_handle();
    h->p = *p;
    if (h->p.ibm_iters <= 0) h->p.ibm_iters = 3;
    if (h->p.ibm_ds == 0.0f) h->p.ibm_ds = 1.0f;
    Geometry& g = h->g;
    g.nx = p->nx;
    g.ny = p->ny;
    g.pitch = (p->nx + kStageW - 1) / kStageW * kStageW;  // whole staged tiles per row
    g.periodic_x = p->periodic_x ? 1 : 0;
    g.periodic_y = p->periodic_y ? 1 : 0;
    g.plane = (long long)g.ny * g.pitch;
    g.perimeter = 2 * g.nx + 2 * (g.ny - 2);
    h->nplanes = (p->quirks & LBMX_QUIRK_REST_LAG) ? 10 : 9;
    const long long n = (long long)g.nx * g.ny;
#define ALLOC(ptr, bytes)                                                                  \
    do {                                                                                    \
        cudaError_t e_ = cudaMalloc((void**)&(ptr), (bytes));                               \
        if (e_ != cudaSuccess) {                                                            \
            fail(nullptr, LBMX_ERR_OUT_OF_MEMORY, "lbmx_create: cudaMalloc(%zu): %s",       \
                 (size_t)(bytes), cudaGetErrorString(e_));                                  \
            lbmx_destroy(h);                                                                \
            return LBMX_ERR_OUT_OF_MEMORY;                                                  \
        }                                                                                   \
    } while (0)
    ALLOC(h->f_alloc, ((size_t)h->nplanes * g.plane + 2 * kGuardElems) * elem_size(p->storage));
    h->f = static_cast<char*>(h->f_alloc) + (size_t)kGuardElems * elem_size(p->storage);
    cudaDeviceGetAttribute(&h->num_sms, cudaDevAttrMultiProcessorCount, p->device);
    if (h->num_sms < 1) h->num_sms = 1;
    if (!encode_population_map(h, &h->tmap, step_tile_w((int)elem_size(p->storage)),
                               step_tile_h((int)elem_size(p->storage)))) {
        fail(nullptr, LBMX_ERR_CUDA, "lbmx_create: cannot build the TMA descriptor (cuTensorMapEncodeTiled)");
        lbmx_destroy(h);
        return LBMX_ERR_CUDA;
    }
    ALLOC(h->edge, (size_t)2 * g.perimeter * 9 * sizeof(float));
    ALLOC(h->aux, (size_t)g.perimeter * 9 * sizeof(float));
    ALLOC(h->rho_out, (size_t)g.plane * sizeof(float));
    ALLOC(h->u_out, (size_t)2 * g.plane * sizeof(float));
    ALLOC(h->staging, (size_t)3 * n * sizeof(float));
    ALLOC(h->counter, sizeof(unsigned int));
    ALLOC(h->sums, kSumsBufferLen * sizeof(double));
    ALLOC(h->avg, 3 * sizeof(float));
    ALLOC(h->error_word, sizeof(unsigned int));
    ALLOC(h->tile_counter, 2 * sizeof(unsigned long long));
#undef ALLOC
    if (p->stream) {
        h->stream = (cudaStream_t)p->stream;
    } else {
        if (cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking) != cudaSuccess) {
            fail(nullptr, LBMX_ERR_CUDA, "lbmx_create: cudaStreamCreate failed");
            lbmx_destroy(h);
            return LBMX_ERR_CUDA;
        }
        h->own_stream = true;
    }
    cudaMemsetAsync(h->counter, 0, sizeof(unsigned int), h->stream);
    cudaMemsetAsync(h->sums, 0, kSumsBufferLen * sizeof(double), h->stream);
    cudaMemsetAsync(h->avg, 0, 3 * sizeof(float), h->stream);
    cudaMemsetAsync(h->error_word, 0, sizeof(unsigned int), h->stream);
    cudaMemsetAsync(h->tile_counter, 0, 2 * sizeof(unsigned long long), h->stream);
    cudaMemsetAsync(h->aux, 0, (size_t)g.perimeter * 9 * sizeof(float), h->stream);
    if (cudaStreamSynchronize(h->stream) != cudaSuccess) {
        fail(nullptr, LBMX_ERR_CUDA, "lbmx_create: initial clears failed");
        lbmx_destroy(h);
        return LBMX_ERR_CUDA;
    }
    if (rebuild_special(h) != LBMX_OK) {
        fail(nullptr, LBMX_ERR_OUT_OF_MEMORY, "lbmx_create: %s", h->err);
        lbmx_destroy(h);
        return LBMX_ERR_OUT_OF_MEMORY;
    }
    *out = h;
    return LBMX_OK;
}

lbmx_status lbmx_set_flags(lbmx_handle* h, const uint8_t* flags) {
    if (!h || !flags) return fail(h, LBMX_ERR_INVALID_ARGUMENT, "lbmx_set_flags: NULL argument");
    cudaSetDevice(h->p.device);
    const Geometry& g = h->g;
    const long long n = (long long)g.nx * g.ny;
    // a staging buffer kept with the handle: a fresh megabyte each call came
    // from new pages, faulted in on first touch
    std::vector<uint8_t>& hf = h->flags_in;
    hf.resize((size_t)n);
    // host memory (pinned or not) is read directly, device memory copied
    cudaPointerAttributes pa;
    if (cudaPointerGetAttributes(&pa, flags) == cudaSuccess &&
        (pa.type == cudaMemoryTypeHost || pa.type == cudaMemoryTypeUnregistered)) {
        memcpy(hf.data(), flags, (size_t)n);
    } else {
        cudaGetLastError();
        LBMX_CUDA(h, cudaMemcpy(hf.data(), flags, n, cudaMemcpyDefault));
    }
    bool any = false, aux = false;
    for (int y = 0; y < g.ny; y++)
        for (int x = 0; x < g.nx; x++) {
            const uint8_t* r = &hf[(long long)y * g.nx];
            // eight fluid nodes at a time
            if ((x & 7) == 0 && x + 8 <= g.nx) {
                uint64_t w;
                memcpy(&w, r + x, 8);
                if (w == 0) {
                    x += 7;
                    continue;
                }
            }
            const uint8_t fl = r[x];
            if (fl == 0) continue;
            any = true;
            const bool edge = x == 0 || y == 0 || x == g.nx - 1 || y == g.ny - 1;
            if (fl == LBMX_ZOU_HE_TOP_LEFT_TOP_INFLOW || fl == LBMX_ZOU_HE_TOP_RIGHT_TOP_INFLOW)
                return fail(h, LBMX_ERR_INVALID_FLAGS,
                            "lbmx_set_flags: flag %d at (%d,%d) is not implemented by the reference (it asserts)", fl, x, y);
            if (fl > LBMX_CORNER_BOTTOM_LEFT)
                return fail(h, LBMX_ERR_INVALID_FLAGS, "lbmx_set_flags: unknown flag %d at (%d,%d)", fl, x, y);
            if (fl == LBMX_PRESSURE_OUTLET && (!edge || x == 0))
                return fail(h, LBMX_ERR_INVALID_FLAGS,
                            "lbmx_set_flags: PRESSURE_OUTLET at (%d,%d) must sit on the domain edge with x >= 1", x, y);
            if ((fl == LBMX_ZG_OUTFLOW || fl == LBMX_REGULARIZED_BOUNCE_BACK_CORNER) && edge) aux = true;
            if (fl == LBMX_PRESSURE_OUTLET) aux = true;
        }
    LBMX_CUDA(h, cudaStreamSynchronize(h->stream));
    if (!any) {
        cudaFree(h->flags);
        h->flags = nullptr;
        h->has_aux_bc = false;
        h->flags_host.clear();
        return rebuild_special(h);
    }
    if (!h->flags) {
        cudaError_t e = cudaMalloc((void**)&h->flags, (size_t)g.plane);
        if (e != cudaSuccess) return fail(h, LBMX_ERR_OUT_OF_MEMORY, "lbmx_set_flags: cudaMalloc failed");
    }
    h->flags_host.assign((size_t)g.plane, 0);
    for (int y = 0; y < g.ny; y++)
        memcpy(&h->flags_host[(size_t)y * g.pitch], &hf[(size_t)y * g.nx], g.nx);
    LBMX_CUDA(h, cudaMemcpy(h->flags, h->flags_host.data(), (size_t)g.plane, cudaMemcpyHostToDevice));
    h->has_aux_bc = aux;
    return rebuild_special(h);
}

static lbmx_status upload_force(lbmx_handle* h, const float* force) {
    const Geometry& g = h->g;
    const long long n = (long long)g.nx * g.ny;
    if (!force) {
        cudaFree(h->force);
        h->force = nullptr;
        return LBMX_OK;
    }
    std::vector<float> hf(2 * n);
    LBMX_CUDA(h, cudaMemcpy(hf.data(), force, 2 * n * sizeof(float), cudaMemcpyDefault));
    bool uniform = true;
    for (long long i = 1; i < n && uniform; i++)
        uniform = hf[i] == hf[0] && hf[n + i] == hf[n];
    if (uniform) {
        // the common case (every reference scenario): no per-node force reads
        h->p.body_fx = hf[0];
        h->p.body_fy = hf[n];
        cudaFree(h->force);
        h->force = nullptr;
        return LBMX_OK;
    }
    if (!h->force) {
        cudaError_t e = cudaMalloc((void**)&h->force, (size_t)2 * g.plane * sizeof(float));
        if (e != cudaSuccess) return fail(h, LBMX_ERR_OUT_OF_MEMORY, "force field: cudaMalloc failed");
    }
    LBMX_CUDA(h, cudaMemsetAsync(h->force, 0, (size_t)2 * g.plane * sizeof(float), h->stream));
    for (int c = 0; c < 2; c++)
        LBMX_CUDA(h, cudaMemcpy2DAsync(h->force + c * g.plane, g.pitch * sizeof(float), hf.data() + c * n,
                                       g.nx * sizeof(float), g.nx * sizeof(float), g.ny, cudaMemcpyHostToDevice,
                                       h->stream));
    LBMX_CUDA(h, cudaStreamSynchronize(h->stream));
    return LBMX_OK;
}

lbmx_status lbmx_set_brinkman(lbmx_handle* h, const float* gamma) {
    if (!h) return fail(h, LBMX_ERR_INVALID_ARGUMENT, "lbmx_set_brinkman: NULL handle");
    cudaSetDevice(h->p.device);
    const Geometry& g = h->g;
    LBMX_CUDA(h, cudaStreamSynchronize(h->stream));
    if (!gamma) {
        cudaFree(h->gamma);
        h->gamma = nullptr;
        return LBMX_OK;
    }
    if (!h->gamma) {
        cudaError_t e = cudaMalloc((void**)&h->gamma, (size_t)g.plane * sizeof(float));
        if (e != cudaSuccess) return fail(h, LBMX_ERR_OUT_OF_MEMORY, "lbmx_set_brinkman: cudaMalloc failed");
        LBMX_CUDA(h, cudaMemsetAsync(h->gamma, 0, (size_t)g.plane * sizeof(float), h->stream));
    }
    LBMX_CUDA(h, cudaMemcpy2DAsync(h->gamma, g.pitch * sizeof(float), gamma, g.nx * sizeof(float),
                                   g.nx * sizeof(float), g.ny, cudaMemcpyDefault, h->stream));
    LBMX_CUDA(h, cudaStreamSynchronize(h->stream));
    return LBMX_OK;
}

lbmx_status lbmx_set_force_field(lbmx_handle* h, const float* force) {
    if (!h) return fail(h, LBMX_ERR_INVALID_ARGUMENT, "lbmx_set_force_field: NULL handle");
    cudaSetDevice(h->p.device);
    return upload_force(h, force);
}

lbmx_status lbmx_init_from_fields(lbmx_handle* h, const float* rho, const float* u, const float* force) {
    if (!h || !rho || !u) return fail(h, LBMX_ERR_INVALID_ARGUMENT, "lbmx_init_from_fields: NULL argument");
    cudaSetDevice(h->p.device);
    const Geometry& g = h->g;
    const long long n = (long long)g.nx * g.ny;
    LBMX_CUDA(h, cudaMemcpyAsync(h->staging, rho, n * sizeof(float), cudaMemcpyDefault, h->stream));
    LBMX_CUDA(h, cudaMemcpyAsync(h->staging + n, u, 2 * n * sizeof(float), cudaMemcpyDefault, h->stream));
    if (force) {
        lbmx_status st = upload_force(h, force);
        if (st != LBMX_OK) return st;
    }
    StepArgs a = base_args(h);
    a.rho_out = h->rho_out;
    a.u_out = h->u_out;
    a.rest_plane = (h->p.quirks & LBMX_QUIRK_REST_LAG) ? 9 : 0;
    LBMX_CUDA(h, cudaMemsetAsync(h->rho_out, 0, (size_t)g.plane * sizeof(float), h->stream));
    LBMX_CUDA(h, cudaMemsetAsync(h->u_out, 0, (size_t)2 * g.plane * sizeof(float), h->stream));
    LBMX_CUDA(h, dispatch(h->p.storage, [&](auto tag) {
                  return launch_init<decltype(tag)>(a, h->staging, h->staging + n, h->stream);
              }));
    LBMX_CUDA(h, cudaStreamSynchronize(h->stream));
    h->t = 0;
    h->last_step = -2;
    h->pend_acc = h->pend_series = nullptr;
    h->initialized = true;
    h->have_avg = false;
    return LBMX_OK;
}

// One step (index s = t+1); store: write moments and FP64 sums; sums: the
// FP64 sums only; ke: the sums include the kinetic energy; series: where the
// step's series entry (sums 0..2, then the kinetic energy) also goes.
static lbmx_status run_step(lbmx_handle* h, bool store, bool check, bool sums, bool ke,
                            double* series = nullptr, double* force_series = nullptr) {
    const long long s = h->t + 1;
    StepArgs a = base_args(h);
    set_step(h, a, s);
    cudaStream_t st = h->stream;
    const int storage = h->p.storage;
    // this step's work counter was zeroed by the previous launch, unless that
    // was not this handle's previous step (a fresh state, batched steps)
    if (h->last_step != s - 1)
        LBMX_CUDA(h, cudaMemsetAsync(h->tile_counter, 0, 2 * sizeof(unsigned long long), st));
    double* acc = h->partials + (size_t)(s & 1) * kAccPerSet;
    if (h->has_aux_bc)
        LBMX_CUDA(h, dispatch(storage, [&](auto tag) { return launch_edge_prepass<decltype(tag)>(a, h->aux, st); }));
    if (h->nm > 0) {
        IbmArgs ia{};
        ia.nm = h->nm;
        ia.npatch = h->npatch;
        ia.iters = h->p.ibm_iters;
        ia.stencil = h->stencil;
        ia.sten_idx = h->sten_idx;
        ia.sten_w = h->sten_w;
        ia.spread = h->spread;
        ia.patch_nodes = h->patch_nodes;
        ia.marker_u = h->marker_u;
        ia.marker_rho = h->marker_rho;
        ia.marker_force = h->marker_force;
        ia.ibm_force = h->ibm_force;
        ia.plane = h->g.plane;
        ia.clamp = (h->p.quirks & LBMX_QUIRK_IBM_CLAMP) ? 1 : 0;
        ia.ds = h->p.ibm_ds;
        ia.force_series = force_series;
        LBMX_CUDA(h, dispatch(storage, [&](auto tag) {
                      return launch_ibm_step<decltype(tag)>(a, ia, st);
                  }));
    }
    const bool opt = h->p.op == LBMX_CM_OPT;
    const bool ext = opt && h->ext_avg;
    h->ext_avg = false;
    const bool lagged = opt && !ext && (h->p.options & LBMX_OPTION_LAGGED_AVERAGES) && h->have_avg;
    if (opt && !lagged && !ext) {
        StepArgs b = a;
        b.partials = acc;
        b.counter = h->counter;
        b.sums = nullptr;
        b.avg_out = h->avg;
        LBMX_CUDA(h, dispatch(storage, [&](auto tag) { return launch_opt_prepass<decltype(tag)>(b, st); }));
        h->have_avg = true;
    }
    if (store) {
        a.rho_out = h->rho_out;
        a.u_out = h->u_out;
    }
    if (store || lagged || sums) {
        a.partials = acc;
        a.counter = h->counter;
        a.sums = (store || sums) ? h->sums : nullptr;
        a.ke = (store || sums) && ke ? 1 : 0;
        // lagged CM_OPT: the averages of this step feed the next one
        a.avg_out = lagged ? h->avg : nullptr;
    }
    a.check_finite = check ? 1 : 0;
    a.series = series;
    // with the IBM kernel just launched, the step starts on the items away
    // from the patch while the marker rounds run
    a.early = h->nm > 0 ? 1 : 0;
    // the previous step's sums, if it left them to this launch
    if (h->pend_acc) {
        a.pub_acc = h->pend_acc;
        a.pub_sums = h->sums;
        a.pub_series = h->pend_series;
        h->pend_acc = h->pend_series = nullptr;
    }
    LBMX_CUDA(h, dispatch(storage, [&](auto tag) { return launch_step<decltype(tag)>(a, h->tmap, h->p.op, st); }));
    if (step_mode(a) == kModeSums) {
        h->pend_acc = acc;
        h->pend_series = series;
    }
    h->last_step = s;
    h->t = s;
    return LBMX_OK;
}

// Publish sums a step left to the next launch when no step follows.
static lbmx_status flush_sums(lbmx_handle* h) {
    if (!h->pend_acc) return LBMX_OK;
    LBMX_CUDA(h, launch_publish(h->pend_acc, h->sums, h->pend_series, h->stream));
    h->pend_acc = h->pend_series = nullptr;
    return LBMX_OK;
}

lbmx_status lbmx_step_ex(lbmx_handle* h, int32_t nsteps, uint32_t flags) {
    if (!h) return fail(h, LBMX_ERR_INVALID_ARGUMENT, "lbmx_step: NULL handle");
    if (!h->initialized) return fail(h, LBMX_ERR_NOT_INITIALIZED, "lbmx_step: call lbmx_init_from_fields first");
    if (nsteps < 0) return fail(h, LBMX_ERR_INVALID_ARGUMENT, "lbmx_step: nsteps < 0");
    cudaSetDevice(h->p.device);
    const bool check = (flags & LBMX_STEP_CHECK_FINITE) != 0;
    if (check) LBMX_CUDA(h, cudaMemsetAsync(h->error_word, 0, sizeof(unsigned int), h->stream));
    const bool ke = (flags & LBMX_STEP_KINETIC_ENERGY) != 0;
    for (int i = 0; i < nsteps; i++) {
        const bool last = i == nsteps - 1;
        lbmx_status st = run_step(h, last && (flags & LBMX_STEP_STORE_MOMENTS), last && check,
                                  (flags & LBMX_STEP_SUMS) != 0, ke);
        if (st != LBMX_OK) return st;
    }
    lbmx_status fs = flush_sums(h);
    if (fs != LBMX_OK) return fs;
    if (check) {
        unsigned int w = 0;
        LBMX_CUDA(h, cudaMemcpyAsync(&w, h->error_word, sizeof(w), cudaMemcpyDeviceToHost, h->stream));
        LBMX_CUDA(h, cudaStreamSynchronize(h->stream));
        if (w) return fail(h, LBMX_ERR_NONFINITE, "lbmx_step: non-finite density at step %lld", h->t);
    }
    return LBMX_OK;
}

lbmx_status lbmx_step_sums(lbmx_handle* h, int32_t nsteps, uint32_t flags, double* series) {
    if (!h || !series) return fail(h, LBMX_ERR_INVALID_ARGUMENT, "lbmx_step_sums: NULL argument");
    if (!h->initialized) return fail(h, LBMX_ERR_NOT_INITIALIZED, "lbmx_step_sums: call lbmx_init_from_fields first");
    if (nsteps < 0) return fail(h, LBMX_ERR_INVALID_ARGUMENT, "lbmx_step_sums: nsteps < 0");
    cudaSetDevice(h->p.device);
    const bool check = (flags & LBMX_STEP_CHECK_FINITE) != 0;
    if (check) LBMX_CUDA(h, cudaMemsetAsync(h->error_word, 0, sizeof(unsigned int), h->stream));
    // device memory and pinned host memory: the step kernel writes each
    // step's sums there itself (no copy between the steps); pageable host
    // memory: a copy per step
    cudaPointerAttributes attr;
    bool direct = false;
    if (cudaPointerGetAttributes(&attr, series) == cudaSuccess)
        direct = attr.type == cudaMemoryTypeDevice || attr.type == cudaMemoryTypeManaged ||
                 (attr.type == cudaMemoryTypeHost && attr.devicePointer != nullptr);
    else
        cudaGetLastError();
    double* dev_series = direct ? static_cast<double*>(attr.devicePointer) : nullptr;
    // a step's entry: {rho, rho ux, rho uy}, then the kinetic energy
    const bool ke = (flags & LBMX_STEP_KINETIC_ENERGY) != 0;
    const size_t stride = ke ? 4 : 3;
    for (int i = 0; i < nsteps; i++) {
        const bool last = i == nsteps - 1;
        lbmx_status st = run_step(h, last && (flags & LBMX_STEP_STORE_MOMENTS), last && check, true, ke,
                                  direct ? dev_series + stride * (size_t)i : nullptr);
        if (st != LBMX_OK) return st;
        if (!direct) {
            if ((st = flush_sums(h)) != LBMX_OK) return st;
            LBMX_CUDA(h, cudaMemcpyAsync(series + stride * (size_t)i, h->sums, 3 * sizeof(double),
                                         cudaMemcpyDefault, h->stream));
            if (ke)
                LBMX_CUDA(h, cudaMemcpyAsync(series + stride * (size_t)i + 3, h->sums + kSumKE, sizeof(double),
                                             cudaMemcpyDefault, h->stream));
        }
    }
    lbmx_status fs = flush_sums(h);
    if (fs != LBMX_OK) return fs;
    if (check) {
        unsigned int w = 0;
        LBMX_CUDA(h, cudaMemcpyAsync(&w, h->error_word, sizeof(w), cudaMemcpyDeviceToHost, h->stream));
        LBMX_CUDA(h, cudaStreamSynchronize(h->stream));
        if (w) return fail(h, LBMX_ERR_NONFINITE, "lbmx_step_sums: non-finite density at step %lld", h->t);
    }
    return LBMX_OK;
}

lbmx_status lbmx_step_forces(lbmx_handle* h, int32_t nsteps, uint32_t flags, double* series) {
    if (!h || !series) return fail(h, LBMX_ERR_INVALID_ARGUMENT, "lbmx_step_forces: NULL argument");
    if (!h->initialized) return fail(h, LBMX_ERR_NOT_INITIALIZED, "lbmx_step_forces: call lbmx_init_from_fields first");
    if (nsteps < 0) return fail(h, LBMX_ERR_INVALID_ARGUMENT, "lbmx_step_forces: nsteps < 0");
    if (h->nm <= 0) return fail(h, LBMX_ERR_INVALID_ARGUMENT, "lbmx_step_forces: the lattice has no IBM markers");
    cudaSetDevice(h->p.device);
    const bool check = (flags & LBMX_STEP_CHECK_FINITE) != 0;
    if (check) LBMX_CUDA(h, cudaMemsetAsync(h->error_word, 0, sizeof(unsigned int), h->stream));
    // as lbmx_step_sums: written by the kernel where it can reach the series,
    // else through a device slot (the sums buffer's spare entries) per step
    cudaPointerAttributes attr;
    bool direct = false;
    if (cudaPointerGetAttributes(&attr, series) == cudaSuccess)
        direct = attr.type == cudaMemoryTypeDevice || attr.type == cudaMemoryTypeManaged ||
                 (attr.type == cudaMemoryTypeHost && attr.devicePointer != nullptr);
    else
        cudaGetLastError();
    double* dev_series = direct ? static_cast<double*>(attr.devicePointer) : nullptr;
    double* slot = h->sums + kSumForces;
    const bool ke = (flags & LBMX_STEP_KINETIC_ENERGY) != 0;
    for (int i = 0; i < nsteps; i++) {
        const bool last = i == nsteps - 1;
        lbmx_status st = run_step(h, last && (flags & LBMX_STEP_STORE_MOMENTS), last && check,
                                  (flags & LBMX_STEP_SUMS) != 0, ke, nullptr,
                                  direct ? dev_series + 2 * (size_t)i : slot);
        if (st != LBMX_OK) return st;
        if (!direct)
            LBMX_CUDA(h, cudaMemcpyAsync(series + 2 * (size_t)i, slot, 2 * sizeof(double), cudaMemcpyDefault,
                                         h->stream));
    }
    lbmx_status fs = flush_sums(h);
    if (fs != LBMX_OK) return fs;
    if (!direct || check) {
        unsigned int w = 0;
        if (check)
            LBMX_CUDA(h, cudaMemcpyAsync(&w, h->error_word, sizeof(w), cudaMemcpyDeviceToHost, h->stream));
        LBMX_CUDA(h, cudaStreamSynchronize(h->stream));
        if (w) return fail(h, LBMX_ERR_NONFINITE, "lbmx_step_forces: non-finite density at step %lld", h->t);
    }
    return LBMX_OK;
}

lbmx_status lbmx_step(lbmx_handle* h, int32_t nsteps) {
    return lbmx_step_ex(h, nsteps, LBMX_STEP_STORE_MOMENTS);
}

lbmx_status lbmx_moment_sums_async(lbmx_handle* h, double* sums3) {
    if (!h || !sums3) return fail(h, LBMX_ERR_INVALID_ARGUMENT, "lbmx_moment_sums_async: NULL argument");
    if (!h->initialized) return fail(h, LBMX_ERR_NOT_INITIALIZED, "lbmx_moment_sums_async: not initialized");
    cudaSetDevice(h->p.device);
    LBMX_CUDA(h, cudaMemcpyAsync(sums3, h->sums, 3 * sizeof(double), cudaMemcpyDefault, h->stream));
    return LBMX_OK;
}

lbmx_status lbmx_kinetic_energy(lbmx_handle* h, double* ke) {
    if (!h || !ke) return fail(h, LBMX_ERR_INVALID_ARGUMENT, "lbmx_kinetic_energy: NULL argument");
    if (!h->initialized) return fail(h, LBMX_ERR_NOT_INITIALIZED, "lbmx_kinetic_energy: not initialized");
    cudaSetDevice(h->p.device);
    double v = 0.0;
    LBMX_CUDA(h, cudaMemcpyAsync(&v, h->sums + kSumKE, sizeof(double), cudaMemcpyDeviceToHost, h->stream));
    LBMX_CUDA(h, cudaStreamSynchronize(h->stream));
    *ke = v;
    return LBMX_OK;
}

lbmx_status lbmx_moments(lbmx_handle* h, float* rho, float* u, double* sums3) {
    if (!h) return fail(h, LBMX_ERR_INVALID_ARGUMENT, "lbmx_moments: NULL handle");
    if (!h->initialized) return fail(h, LBMX_ERR_NOT_INITIALIZED, "lbmx_moments: not initialized");
    cudaSetDevice(h->p.device);
    const Geometry& g = h->g;
    const long long n = (long long)g.nx * g.ny;
    if (rho)
        LBMX_CUDA(h, cudaMemcpy2DAsync(rho, g.nx * sizeof(float), h->rho_out, g.pitch * sizeof(float),
                                       g.nx * sizeof(float), g.ny, cudaMemcpyDefault, h->stream));
    if (u)
        for (int c = 0; c < 2; c++)
            LBMX_CUDA(h, cudaMemcpy2DAsync(u + c * n, g.nx * sizeof(float), h->u_out + c * g.plane,
                                           g.pitch * sizeof(float), g.nx * sizeof(float), g.ny, cudaMemcpyDefault,
                                           h->stream));
    if (sums3) {
        double s[6];
        LBMX_CUDA(h, cudaMemcpyAsync(s, h->sums, sizeof(s), cudaMemcpyDeviceToHost, h->stream));
        LBMX_CUDA(h, cudaStreamSynchronize(h->stream));
        sums3[0] = s[0];
        sums3[1] = s[1];
        sums3[2] = s[2];
    }
    LBMX_CUDA(h, cudaStreamSynchronize(h->stream));
    return check_pipeline(h);
}

lbmx_status lbmx_get_populations(lbmx_handle* h, float* out) {
    if (!h || !out) return fail(h, LBMX_ERR_INVALID_ARGUMENT, "lbmx_get_populations: NULL argument");
    if (!h->initialized) return fail(h, LBMX_ERR_NOT_INITIALIZED, "lbmx_get_populations: not initialized");
    cudaSetDevice(h->p.device);
    const long long n = (long long)h->g.nx * h->g.ny;
    if (!h->pop_out) LBMX_CUDA(h, cudaMalloc((void**)&h->pop_out, (size_t)9 * n * sizeof(float)));
    StepArgs a = base_args(h);
    // parity and rest plane of the last step taken (init looks like a parity-0 step)
    set_step(h, a, h->t);
    if (h->t == 0) a.parity = 0;
    LBMX_CUDA(h, dispatch(h->p.storage, [&](auto tag) {
                  return launch_get_populations<decltype(tag)>(a, h->pop_out, h->stream);
              }));
    LBMX_CUDA(h, cudaMemcpyAsync(out, h->pop_out, (size_t)9 * n * sizeof(float), cudaMemcpyDefault, h->stream));
    LBMX_CUDA(h, cudaStreamSynchronize(h->stream));
    return LBMX_OK;
}

// ---------------------------------------------------------------- y-slabs
lbmx_status lbmx_set_slab(lbmx_handle* h, uint32_t ghost_mask, int64_t row_origin, int32_t whole_ny) {
    if (!h) return fail(h, LBMX_ERR_INVALID_ARGUMENT, "lbmx_set_slab: NULL handle");
    if (ghost_mask > 3u)
        return fail(h, LBMX_ERR_INVALID_ARGUMENT, "lbmx_set_slab: ghost mask %u (bits 0 and 1 only)", ghost_mask);
    if (ghost_mask && h->g.periodic_y)
        return fail(h, LBMX_ERR_INVALID_ARGUMENT, "lbmx_set_slab: a lattice with ghost rows is not periodic in y");
    if (h->g.ny < 3) return fail(h, LBMX_ERR_INVALID_ARGUMENT, "lbmx_set_slab: ny < 3");
    if (ghost_mask && h->nm > 0) return fail(h, LBMX_ERR_UNSUPPORTED, "lbmx_set_slab: IBM markers on a y-slab");
    cudaSetDevice(h->p.device);
    LBMX_CUDA(h, cudaStreamSynchronize(h->stream));
    if (whole_ny < 0 || (whole_ny > 0 && whole_ny < h->g.ny - 2))
        return fail(h, LBMX_ERR_INVALID_ARGUMENT, "lbmx_set_slab: whole_ny %d", whole_ny);
    h->ghost_mask = ghost_mask;
    h->row_origin = row_origin;
    h->whole_ny = whole_ny;
    return rebuild_special(h);
}

// Raw slot copies of one row: for each population q in plane_mask
// (ascending), nx stored elements of plane q, row `row`.
static lbmx_status halo_copy(lbmx_handle* h, int32_t row, uint32_t plane_mask, void* buf, bool get, const char* who) {
    if (!h || !buf) return fail(h, LBMX_ERR_INVALID_ARGUMENT, "%s: NULL argument", who);
    if (!h->initialized) return fail(h, LBMX_ERR_NOT_INITIALIZED, "%s: not initialized", who);
    if (row < 0 || row >= h->g.ny || plane_mask == 0 || plane_mask > 0x1FFu)
        return fail(h, LBMX_ERR_INVALID_ARGUMENT, "%s: row %d or plane mask 0x%x out of range", who, row, plane_mask);
    cudaSetDevice(h->p.device);
    const size_t es = elem_size(h->p.storage), bytes = (size_t)h->g.nx * es;
    char* f = static_cast<char*>(h->f);
    char* b = static_cast<char*>(buf);
    static const int cx[9] = {0, 1, 0, -1, 0, 1, -1, -1, 1};
    for (int q = 0; q < 9; q++) {
        if (!((plane_mask >> q) & 1u)) continue;
        char* slot = f + ((size_t)q * h->g.plane + (size_t)row * h->g.pitch) * es;
        // a put writes only the slots a node of the neighbouring row writes in
        // a neighbour-access step: on a lattice not periodic in x, slot q of
        // the column whose upstream column x - c_q is outside belongs to the
        // node itself (a half-way wall reflects into it)
        size_t skip_lo = 0, skip_hi = 0;
        if (!get && !h->g.periodic_x) {
            if (cx[q] > 0) skip_lo = 1;
            if (cx[q] < 0) skip_hi = 1;
        }
        const size_t n = bytes - (skip_lo + skip_hi) * es;
        if (get)
            LBMX_CUDA(h, cudaMemcpyAsync(b, slot, bytes, cudaMemcpyDefault, h->stream));
        else
            LBMX_CUDA(h, cudaMemcpyAsync(slot + skip_lo * es, b + skip_lo * es, n, cudaMemcpyDefault, h->stream));
        b += bytes;
    }
    return LBMX_OK;
}

lbmx_status lbmx_halo_get(lbmx_handle* h, int32_t row, uint32_t plane_mask, void* buf) {
    return halo_copy(h, row, plane_mask, buf, true, "lbmx_halo_get");
}

lbmx_status lbmx_halo_put(lbmx_handle* h, int32_t row, uint32_t plane_mask, const void* buf) {
    return halo_copy(h, row, plane_mask, const_cast<void*>(buf), false, "lbmx_halo_put");
}

lbmx_status lbmx_opt_partials(lbmx_handle* h, int64_t* sums3) {
    if (!h || !sums3) return fail(h, LBMX_ERR_INVALID_ARGUMENT, "lbmx_opt_partials: NULL argument");
    if (!h->initialized) return fail(h, LBMX_ERR_NOT_INITIALIZED, "lbmx_opt_partials: not initialized");
    if (h->p.op != LBMX_CM_OPT) return fail(h, LBMX_ERR_UNSUPPORTED, "lbmx_opt_partials: the operator is not CM_OPT");
    cudaSetDevice(h->p.device);
    if (!h->raw_sums) LBMX_CUDA(h, cudaMalloc((void**)&h->raw_sums, kNumSums * sizeof(long long)));
    const long long s = h->t + 1;
    StepArgs a = base_args(h);
    set_step(h, a, s);
    if (h->has_aux_bc)
        LBMX_CUDA(h, dispatch(h->p.storage, [&](auto tag) { return launch_edge_prepass<decltype(tag)>(a, h->aux, h->stream); }));
    StepArgs b = a;
    b.partials = h->partials + (size_t)(s & 1) * kAccPerSet;
    b.counter = h->counter;
    b.sums = nullptr;
    b.avg_out = h->avg;
    b.raw_sums = h->raw_sums;
    LBMX_CUDA(h, dispatch(h->p.storage, [&](auto tag) { return launch_opt_prepass<decltype(tag)>(b, h->stream); }));
    long long r[kNumSums];
    LBMX_CUDA(h, cudaMemcpyAsync(r, h->raw_sums, sizeof(r), cudaMemcpyDeviceToHost, h->stream));
    LBMX_CUDA(h, cudaStreamSynchronize(h->stream));
    sums3[0] = r[0];
    sums3[1] = r[4];
    sums3[2] = r[5];
    return LBMX_OK;
}

lbmx_status lbmx_set_averages(lbmx_handle* h, const float* avg3) {
    if (!h || !avg3) return fail(h, LBMX_ERR_INVALID_ARGUMENT, "lbmx_set_averages: NULL argument");
    if (h->p.op != LBMX_CM_OPT) return fail(h, LBMX_ERR_UNSUPPORTED, "lbmx_set_averages: the operator is not CM_OPT");
    cudaSetDevice(h->p.device);
    LBMX_CUDA(h, cudaMemcpyAsync(h->avg, avg3, 3 * sizeof(float), cudaMemcpyDefault, h->stream));
    LBMX_CUDA(h, cudaStreamSynchronize(h->stream));
    h->ext_avg = true;
    h->have_avg = true;
    return LBMX_OK;
}

lbmx_status lbmx_averages(lbmx_handle* h, float* avg3) {
    if (!h || !avg3) return fail(h, LBMX_ERR_INVALID_ARGUMENT, "lbmx_averages: NULL argument");
    cudaSetDevice(h->p.device);
    LBMX_CUDA(h, cudaMemcpyAsync(avg3, h->avg, 3 * sizeof(float), cudaMemcpyDeviceToHost, h->stream));
    LBMX_CUDA(h, cudaStreamSynchronize(h->stream));
    return LBMX_OK;
}

}  // extern "C"

// Peskin 4-point kernel (src/IBM/IBMUtils.cuh:24-33), evaluated in double on the host
static double delta4(double r) {
    const double a = std::fabs(r);
    if (a < 1.0) return 0.125 * (3.0 - 2.0 * a + std::sqrt(1.0 + 4.0 * a - 4.0 * r * r));
    if (a < 2.0) return 0.125 * (5.0 - 2.0 * a - std::sqrt(-7.0 + 12.0 * a - 4.0 * r * r));
    return 0.0;
}

namespace lbmx {
int ibm_build_stencil(int nx, int ny, long long pitch, bool two, const float* hxy, int n, std::vector<int>& sidx,
                      std::vector<float>& sw, std::vector<int>& nodes) {
    const int S = two ? 2 : 4, lo = two ? 0 : -1, S2 = S * S;
    sidx.assign((size_t)n * S2, -1);
    sw.assign((size_t)n * S2, 0.f);
    nodes.clear();
    std::unordered_map<long long, int> map;
    for (int k = 0; k < n; k++) {
        const float px = hxy[2 * k], py = hxy[2 * k + 1];
        if (!std::isfinite(px) || !std::isfinite(py)) return k;
        const float gx = std::floor(px), gy = std::floor(py);
        // x offset outer, y offset inner, as the reference's stencil loops (IBM_impl.cu:19-20)
        for (int i = 0; i < S; i++)
            for (int j = 0; j < S; j++) {
                const int xn = (int)(gx + (float)(lo + i)), yn = (int)(gy + (float)(lo + j));
                if (xn < 0 || xn >= nx || yn < 0 || yn >= ny) continue;
                const long long off = (long long)yn * pitch + xn;
                auto it = map.find(off);
                int idx;
                if (it == map.end()) {
                    idx = (int)nodes.size();
                    map.emplace(off, idx);
                    nodes.push_back((int)off);
                } else {
                    idx = it->second;
                }
                sidx[(size_t)k * S2 + i * S + j] = idx;
                sw[(size_t)k * S2 + i * S + j] = (float)(delta4((double)px - xn) * delta4((double)py - yn));
            }
    }
    return -1;
}

std::vector<int> ibm_build_spread(int np, const std::vector<int>& sidx) {
    std::vector<int> sp((size_t)np + 1, 0);
    for (int idx : sidx)
        if (idx >= 0) sp[(size_t)idx + 1]++;
    for (int i = 0; i < np; i++) sp[(size_t)i + 1] += sp[(size_t)i];
    sp.resize((size_t)np + 1 + (size_t)sp[(size_t)np]);
    std::vector<int> fill(sp.begin(), sp.begin() + np);
    for (size_t j = 0; j < sidx.size(); j++)
        if (sidx[j] >= 0) sp[(size_t)np + 1 + (size_t)fill[(size_t)sidx[j]]++] = (int)j;
    return sp;
}
}  // namespace lbmx

extern "C" {

lbmx_status lbmx_ibm_set_markers(lbmx_handle* h, const float* xy, int32_t n) {
    if (!h) return fail(h, LBMX_ERR_INVALID_ARGUMENT, "lbmx_ibm_set_markers: NULL handle");
    if (n < 0 || (n > 0 && !xy)) return fail(h, LBMX_ERR_INVALID_ARGUMENT, "lbmx_ibm_set_markers: bad marker array");
    if (n > 0 && h->ghost_mask) return fail(h, LBMX_ERR_UNSUPPORTED, "lbmx_ibm_set_markers: IBM markers on a y-slab");
    cudaSetDevice(h->p.device);
    LBMX_CUDA(h, cudaStreamSynchronize(h->stream));
    free_ibm(h);
    if (n == 0) return rebuild_special(h);
    const Geometry& g = h->g;
    std::vector<float> hxy(2 * (size_t)n);
    LBMX_CUDA(h, cudaMemcpy(hxy.data(), xy, 2 * (size_t)n * sizeof(float), cudaMemcpyDefault));
    const bool two = (h->p.quirks & LBMX_QUIRK_IBM_2X2) != 0;
    const int S = two ? 2 : 4, S2 = S * S;
    std::vector<int> sidx, nodes;
    std::vector<float> sw;
    const int bad = lbmx::ibm_build_stencil(g.nx, g.ny, g.pitch, two, hxy.data(), n, sidx, sw, nodes);
    if (bad >= 0) return fail(h, LBMX_ERR_INVALID_ARGUMENT, "lbmx_ibm_set_markers: marker %d is not finite", bad);
    const int np = (int)nodes.size();
    if (lbmx::ibm_smem_bytes(np, n, S) > 200 * 1024)
        return fail(h, LBMX_ERR_TOO_LARGE, "lbmx_ibm_set_markers: %d markers touch %d nodes; limit is 200 KB of patch state",
                    n, np);
    h->nm = n;
    h->npatch = np;
    h->stencil = S;
    LBMX_CUDA(h, cudaMalloc((void**)&h->patch_nodes, np * sizeof(int)));
    LBMX_CUDA(h, cudaMalloc((void**)&h->sten_idx, (size_t)n * S2 * sizeof(int)));
    LBMX_CUDA(h, cudaMalloc((void**)&h->sten_w, (size_t)n * S2 * sizeof(float)));
    LBMX_CUDA(h, cudaMalloc((void**)&h->marker_u, 2 * (size_t)n * sizeof(float)));
    LBMX_CUDA(h, cudaMalloc((void**)&h->marker_rho, (size_t)n * sizeof(float)));
    LBMX_CUDA(h, cudaMalloc((void**)&h->marker_force, 2 * (size_t)n * sizeof(float)));
    LBMX_CUDA(h, cudaMalloc((void**)&h->ibm_force, 2 * (size_t)g.plane * sizeof(float)));
    LBMX_CUDA(h, cudaMemcpy(h->patch_nodes, nodes.data(), np * sizeof(int), cudaMemcpyHostToDevice));
    LBMX_CUDA(h, cudaMemcpy(h->sten_idx, sidx.data(), sidx.size() * sizeof(int), cudaMemcpyHostToDevice));
    LBMX_CUDA(h, cudaMemcpy(h->sten_w, sw.data(), sw.size() * sizeof(float), cudaMemcpyHostToDevice));
    const std::vector<int> spread = lbmx::ibm_build_spread(np, sidx);
    LBMX_CUDA(h, cudaMalloc((void**)&h->spread, spread.size() * sizeof(int)));
    LBMX_CUDA(h, cudaMemcpy(h->spread, spread.data(), spread.size() * sizeof(int), cudaMemcpyHostToDevice));
    LBMX_CUDA(h, cudaMemset(h->ibm_force, 0, 2 * (size_t)g.plane * sizeof(float)));
    LBMX_CUDA(h, cudaMemset(h->marker_force, 0, 2 * (size_t)n * sizeof(float)));
    LBMX_CUDA(h, cudaMemset(h->marker_u, 0, 2 * (size_t)n * sizeof(float)));
    LBMX_CUDA(h, cudaMemset(h->marker_rho, 0, (size_t)n * sizeof(float)));
    h->patch_host = nodes;  // patch nodes read the IBM force: general path
    return rebuild_special(h);
}

lbmx_status lbmx_ibm_forces(lbmx_handle* h, float* force, double* drag_lift) {
    if (!h) return fail(h, LBMX_ERR_INVALID_ARGUMENT, "lbmx_ibm_forces: NULL handle");
    cudaSetDevice(h->p.device);
    std::vector<float> hf(2 * (size_t)h->nm);
    if (h->nm > 0)
        LBMX_CUDA(h, cudaMemcpyAsync(hf.data(), h->marker_force, hf.size() * sizeof(float), cudaMemcpyDeviceToHost,
                                     h->stream));
    LBMX_CUDA(h, cudaStreamSynchronize(h->stream));
    if (force && h->nm > 0) memcpy(force, hf.data(), hf.size() * sizeof(float));
    if (drag_lift) {
        double dx = 0, dy = 0;
        for (int k = 0; k < h->nm; k++) {
            dx += hf[k];
            dy += hf[h->nm + k];
        }
        drag_lift[0] = -dx;
        drag_lift[1] = -dy;
    }
    return LBMX_OK;
}

int64_t lbmx_time(lbmx_handle* h) { return h ? h->t : -1; }

// ---------------------------------------------------------------- checkpoints
// File: a fixed header, the population planes in the handle's storage type and
// in-place (AA) order, the edge store, the grid averages, then a CRC-32 of
// everything before it.  The configuration (flags, markers, forces) is the
// caller's and is set again before a load.

// CRC-32 (IEEE 802.3, reflected polynomial 0xEDB88320), table-driven
struct Crc32Table {
    uint32_t v[256];
    Crc32Table() {
        for (uint32_t i = 0; i < 256; i++) {
            uint32_t c = i;
            for (int k = 0; k < 8; k++) c = (c & 1u) ? 0xEDB88320u ^ (c >> 1) : c >> 1;
            v[i] = c;
        }
    }
};

static uint32_t crc32_update(uint32_t crc, const void* data, size_t n) {
    static const Crc32Table table;  // thread-safe one-time construction
    const unsigned char* p = static_cast<const unsigned char*>(data);
    crc = ~crc;
    for (size_t i = 0; i < n; i++) crc = table.v[(crc ^ p[i]) & 0xFFu] ^ (crc >> 8);
    return ~crc;
}

struct CheckpointHeader {
    char magic[8];  // "LBMXCKP2"
    int32_t nx, ny, pitch, nplanes, storage, op, periodic_x, periodic_y;
    uint32_t quirks, reserved;
    int64_t t;
    int64_t f_bytes, edge_bytes;
};

lbmx_status lbmx_checkpoint_save(lbmx_handle* h, const char* path) {
    if (!h || !path) return fail(h, LBMX_ERR_INVALID_ARGUMENT, "lbmx_checkpoint_save: NULL argument");
    if (!h->initialized) return fail(h, LBMX_ERR_NOT_INITIALIZED, "lbmx_checkpoint_save: not initialized");
    cudaSetDevice(h->p.device);
    CheckpointHeader hd;
    memset(&hd, 0, sizeof(hd));
    memcpy(hd.magic, "LBMXCKP2", 8);
    hd.nx = h->g.nx; hd.ny = h->g.ny; hd.pitch = h->g.pitch; hd.nplanes = h->nplanes;
    hd.storage = h->p.storage; hd.op = h->p.op; hd.periodic_x = h->g.periodic_x; hd.periodic_y = h->g.periodic_y;
    hd.quirks = h->p.quirks; hd.t = h->t;
    hd.f_bytes = (int64_t)h->nplanes * h->g.plane * (int64_t)elem_size(h->p.storage);
    hd.edge_bytes = (int64_t)2 * h->g.perimeter * 9 * (int64_t)sizeof(float);
    std::vector<char> f((size_t)hd.f_bytes), edge((size_t)hd.edge_bytes);
    float avg[3];
    LBMX_CUDA(h, cudaStreamSynchronize(h->stream));
    LBMX_CUDA(h, cudaMemcpy(f.data(), h->f, f.size(), cudaMemcpyDeviceToHost));
    LBMX_CUDA(h, cudaMemcpy(edge.data(), h->edge, edge.size(), cudaMemcpyDeviceToHost));
    LBMX_CUDA(h, cudaMemcpy(avg, h->avg, sizeof(avg), cudaMemcpyDeviceToHost));
    uint32_t crc = crc32_update(0, &hd, sizeof(hd));
    crc = crc32_update(crc, f.data(), f.size());
    crc = crc32_update(crc, edge.data(), edge.size());
    crc = crc32_update(crc, avg, sizeof(avg));
    FILE* fp = fopen(path, "wb");
    if (!fp) return fail(h, LBMX_ERR_INVALID_ARGUMENT, "lbmx_checkpoint_save: cannot open %s", path);
    bool ok = fwrite(&hd, sizeof(hd), 1, fp) == 1 && fwrite(f.data(), 1, f.size(), fp) == f.size() &&
              fwrite(edge.data(), 1, edge.size(), fp) == edge.size() && fwrite(avg, sizeof(avg), 1, fp) == 1 &&
              fwrite(&crc, sizeof(crc), 1, fp) == 1;
    ok = (fclose(fp) == 0) && ok;
    if (!ok) return fail(h, LBMX_ERR_INVALID_ARGUMENT, "lbmx_checkpoint_save: write to %s failed", path);
    return LBMX_OK;
}

lbmx_status lbmx_checkpoint_load(lbmx_handle* h, const char* path) {
    if (!h || !path) return fail(h, LBMX_ERR_INVALID_ARGUMENT, "lbmx_checkpoint_load: NULL argument");
    cudaSetDevice(h->p.device);
    FILE* fp = fopen(path, "rb");
    if (!fp) return fail(h, LBMX_ERR_INVALID_ARGUMENT, "lbmx_checkpoint_load: cannot open %s", path);
    CheckpointHeader hd;
    if (fread(&hd, sizeof(hd), 1, fp) != 1 || memcmp(hd.magic, "LBMXCKP2", 8) != 0) {
        fclose(fp);
        return fail(h, LBMX_ERR_INVALID_ARGUMENT, "lbmx_checkpoint_load: %s is not an lbmx checkpoint", path);
    }
    const int64_t f_bytes = (int64_t)h->nplanes * h->g.plane * (int64_t)elem_size(h->p.storage);
    const int64_t edge_bytes = (int64_t)2 * h->g.perimeter * 9 * (int64_t)sizeof(float);
    if (hd.nx != h->g.nx || hd.ny != h->g.ny || hd.pitch != h->g.pitch || hd.nplanes != h->nplanes ||
        hd.storage != h->p.storage || hd.op != h->p.op || hd.periodic_x != h->g.periodic_x ||
        hd.periodic_y != h->g.periodic_y || hd.quirks != h->p.quirks || hd.f_bytes != f_bytes ||
        hd.edge_bytes != edge_bytes) {
        fclose(fp);
        return fail(h, LBMX_ERR_INVALID_ARGUMENT,
                    "lbmx_checkpoint_load: %s was written for a different lattice or configuration", path);
    }
    std::vector<char> f((size_t)f_bytes), edge((size_t)edge_bytes);
    float avg[3];
    uint32_t crc_file = 0;
    const bool ok = fread(f.data(), 1, f.size(), fp) == f.size() && fread(edge.data(), 1, edge.size(), fp) == edge.size() &&
                    fread(avg, sizeof(avg), 1, fp) == 1 && fread(&crc_file, sizeof(crc_file), 1, fp) == 1;
    fclose(fp);
    if (!ok) return fail(h, LBMX_ERR_INVALID_ARGUMENT, "lbmx_checkpoint_load: %s is truncated", path);
    uint32_t crc = crc32_update(0, &hd, sizeof(hd));
    crc = crc32_update(crc, f.data(), f.size());
    crc = crc32_update(crc, edge.data(), edge.size());
    crc = crc32_update(crc, avg, sizeof(avg));
    if (crc != crc_file) return fail(h, LBMX_ERR_INVALID_ARGUMENT, "lbmx_checkpoint_load: %s fails its CRC-32", path);
    LBMX_CUDA(h, cudaStreamSynchronize(h->stream));
    LBMX_CUDA(h, cudaMemcpy(h->f, f.data(), f.size(), cudaMemcpyHostToDevice));
    LBMX_CUDA(h, cudaMemcpy(h->edge, edge.data(), edge.size(), cudaMemcpyHostToDevice));
    LBMX_CUDA(h, cudaMemcpy(h->avg, avg, sizeof(avg), cudaMemcpyHostToDevice));
    h->t = hd.t;
    h->last_step = -2;
    h->pend_acc = h->pend_series = nullptr;
    h->initialized = true;
    h->have_avg = h->p.op == LBMX_CM_OPT && hd.t > 0;
    return LBMX_OK;
}

// ImageData (.vti) with appended raw Float32 density and 3-component velocity
// (z = 0), the layout of the reference's save_vtk (src/core/lbm.cuh:269-343).
lbmx_status lbmx_write_vti(lbmx_handle* h, const char* path) {
    if (!h || !path) return fail(h, LBMX_ERR_INVALID_ARGUMENT, "lbmx_write_vti: NULL argument");
    const Geometry& g = h->g;
    const size_t n = (size_t)g.nx * g.ny;
    std::vector<float> rho(n), u(2 * n);
    lbmx_status st = lbmx_moments(h, rho.data(), u.data(), nullptr);
    if (st != LBMX_OK) return st;
    std::vector<float> u3(3 * n);
    for (size_t i = 0; i < n; i++) {
        u3[3 * i] = u[i];
        u3[3 * i + 1] = u[n + i];
        u3[3 * i + 2] = 0.0f;
    }
    FILE* fp = fopen(path, "wb");
    if (!fp) return fail(h, LBMX_ERR_INVALID_ARGUMENT, "lbmx_write_vti: cannot open %s", path);
    const uint64_t rho_bytes = n * sizeof(float), u_bytes = 3 * n * sizeof(float);
    fprintf(fp, "<?xml version=\"1.0\"?>\n");
    fprintf(fp, "<VTKFile type=\"ImageData\" version=\"1.0\" byte_order=\"LittleEndian\" header_type=\"UInt64\">\n");
    fprintf(fp, "  <ImageData WholeExtent=\"0 %d 0 %d 0 0\" Origin=\"0 0 0\" Spacing=\"1 1 1\">\n", g.nx - 1, g.ny - 1);
    fprintf(fp, "    <Piece Extent=\"0 %d 0 %d 0 0\">\n", g.nx - 1, g.ny - 1);
    fprintf(fp, "      <PointData Scalars=\"Density\" Vectors=\"Velocity\">\n");
    fprintf(fp, "        <DataArray type=\"Float32\" Name=\"Density\" format=\"appended\" offset=\"0\"/>\n");
    fprintf(fp,
            "        <DataArray type=\"Float32\" Name=\"Velocity\" NumberOfComponents=\"3\" format=\"appended\" "
            "offset=\"%llu\"/>\n",
            (unsigned long long)(rho_bytes + sizeof(uint64_t)));
    fprintf(fp, "      </PointData>\n      <CellData>\n      </CellData>\n    </Piece>\n  </ImageData>\n");
    fprintf(fp, "  <AppendedData encoding=\"raw\">\n   _");
    bool ok = fwrite(&rho_bytes, sizeof(rho_bytes), 1, fp) == 1 && fwrite(rho.data(), 1, rho_bytes, fp) == rho_bytes &&
              fwrite(&u_bytes, sizeof(u_bytes), 1, fp) == 1 && fwrite(u3.data(), 1, u_bytes, fp) == u_bytes;
    fprintf(fp, "\n  </AppendedData>\n</VTKFile>\n");
    ok = (fclose(fp) == 0) && ok;
    if (!ok) return fail(h, LBMX_ERR_INVALID_ARGUMENT, "lbmx_write_vti: write to %s failed", path);
    return LBMX_OK;
}

lbmx_status lbmx_synchronize(lbmx_handle* h) {
    if (!h) return fail(h, LBMX_ERR_INVALID_ARGUMENT, "lbmx_synchronize: NULL handle");
    cudaSetDevice(h->p.device);
    LBMX_CUDA(h, cudaStreamSynchronize(h->stream));
    return check_pipeline(h);
}

const char* lbmx_last_error(lbmx_handle* h) { return h ? h->err : g_create_err; }

}  // extern "C"
