// lbmx_batch.cu -- the batch C-ABI: many lattices advanced by one persistent
// launch per step (lbmx_batch_kernels.cuh), CUDA-graph replay of the step
// sequence and an autotuner over tile shape, CTAs per SM and claim size.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <vector>

#include "lbmx_handle.h"

using namespace lbmx;

namespace {

// argument variants of one lattice: plain step, moments stored, moments
// stored + finite check (the last step of a call)
constexpr int kVariants = 3;

}  // namespace

struct lbmx_batch {
    std::vector<lbmx_handle*> lat;
    int device = 0, storage = 0, op = 0, num_sms = 1;
    cudaStream_t stream = nullptr;
    bool own_stream = false;  // false: every lattice runs on this one stream
    lbmx_batch_config cfg{128, 4, kCtasPerSm, 1, 16};
    // device state of the current configuration
    StepArgs* d_args = nullptr;        // [kVariants][2 parities][count]
    CUtensorMap* d_tmaps = nullptr;    // [count]
    int2* d_items[2] = {nullptr, nullptr};  // work list of an own-node (0) and a neighbour-access (1) step
    int nitems[2] = {0, 0}, items_cap[2] = {0, 0};
    unsigned long long* counter = nullptr;
    unsigned int* done = nullptr;
    unsigned int* error_word = nullptr;
    unsigned int* step = nullptr;      // step index of the next launch (rounding hash seed)
    std::vector<StepArgs> host_args;   // what d_args holds
    int args_tile_w = 0, args_tile_h = 0;  // tile shape d_tmaps / d_items were built for
    bool lean = false;                     // no lattice has a per-node force or Brinkman field
    // streams of the lattices (distinct), one event each, and the batch's end event
    std::vector<cudaStream_t> streams;
    std::vector<cudaEvent_t> stream_events;
    cudaEvent_t end_event = nullptr;
    cudaGraphExec_t graph[2] = {nullptr, nullptr};  // by parity of the first step
    int graph_len = 0;
    char err[512] = {0};
};

static char g_batch_err[512];

static lbmx_status bfail(lbmx_batch* b, lbmx_status code, const char* fmt, ...) {
    char* dst = b ? b->err : g_batch_err;
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(dst, 512, fmt, ap);
    va_end(ap);
    return code;
}

#define BATCH_CUDA(b, call)                                                                          \
    do {                                                                                            \
        cudaError_t e_ = (call);                                                                    \
        if (e_ != cudaSuccess)                                                                      \
            return bfail((b), e_ == cudaErrorMemoryAllocation ? LBMX_ERR_OUT_OF_MEMORY : LBMX_ERR_CUDA, \
                         "%s: %s (%s:%d)", #call, cudaGetErrorString(e_), __FILE__, __LINE__);        \
    } while (0)

static void drop_graphs(lbmx_batch* b) {
    for (auto& g : b->graph) {
        if (g) cudaGraphExecDestroy(g);
        g = nullptr;
    }
    b->graph_len = 0;
}

static bool valid_config(const lbmx_batch_config& c) {
    const bool shape = (c.tile_w == 64 && c.tile_h == 8) || (c.tile_w == 128 && (c.tile_h == 4 || c.tile_h == 8));
    return shape && (c.ctas_per_sm >= 1 && c.ctas_per_sm <= kCtasPerSm) &&
           c.chunk >= 1 && c.chunk <= 64 && c.graph_steps >= 0 && c.graph_steps <= 64 && c.graph_steps % 2 == 0;
}

// Per-lattice kernel arguments of every variant for the configured tile
// shape; re-uploaded (and the graphs dropped) when a lattice changed since
// the last call (new flags, force field or special-unit list).
static lbmx_status refresh(lbmx_batch* b) {
    const int n = (int)b->lat.size();
    const int tw = b->cfg.tile_w, th = b->cfg.tile_h;
    std::vector<StepArgs> args((size_t)kVariants * 2 * n);
    for (int l = 0; l < n; l++) {
        const lbmx_handle* h = b->lat[l];
        StepArgs a = base_args(h);
        a.tiles_x = (h->g.nx + tw - 1) / tw;
        a.tiles_y = (h->g.ny + th - 1) / th;
        a.special_chunks = 0;
        a.num_ctas = 0;
        a.tile_counter = a.tile_counter_next = nullptr;
        // whole-struct memcpy keeps the (zeroed) padding, so the memcmp below
        // sees only real changes
        for (int v = 0; v < kVariants; v++)
            for (int p = 0; p < 2; p++) {
                StepArgs c;
                memcpy(&c, &a, sizeof(c));
                set_step(h, c, p);  // parity of step index p
                if (v >= 1) {
                    c.rho_out = h->rho_out;
                    c.u_out = h->u_out;
                }
                if (v == 2) {
                    c.check_finite = 1;
                    c.error_word = b->error_word;
                }
                memcpy(&args[((size_t)v * 2 + p) * n + l], &c, sizeof(c));
            }
    }
    const bool same_args =
        b->host_args.size() == args.size() && memcmp(b->host_args.data(), args.data(), args.size() * sizeof(StepArgs)) == 0;
    if (same_args && b->args_tile_w == tw && b->args_tile_h == th) return LBMX_OK;
    drop_graphs(b);
    if (!b->d_args) BATCH_CUDA(b, cudaMalloc((void**)&b->d_args, args.size() * sizeof(StepArgs)));
    BATCH_CUDA(b, cudaMemcpyAsync(b->d_args, args.data(), args.size() * sizeof(StepArgs), cudaMemcpyHostToDevice,
                                  b->stream));
    // TMA descriptors and, per parity, the work list
    std::vector<CUtensorMap> maps(n);
    for (int l = 0; l < n; l++)
        if (!encode_population_map(b->lat[l], &maps[l], tw, th))
            return bfail(b, LBMX_ERR_CUDA, "lbmx_batch: cannot build the TMA descriptor of lattice %d", l);
    if (!b->d_tmaps) BATCH_CUDA(b, cudaMalloc((void**)&b->d_tmaps, (size_t)n * sizeof(CUtensorMap)));
    BATCH_CUDA(b, cudaMemcpyAsync(b->d_tmaps, maps.data(), (size_t)n * sizeof(CUtensorMap), cudaMemcpyHostToDevice,
                                  b->stream));
    // Per parity, each lattice's tiles, then its special chunks: a chunk is
    // one node per thread, a chain of scattered loads that its lattice's
    // tiles have just brought into L2, and the chunks spread over the whole
    // launch instead of all waiting on DRAM together at its start.
    std::vector<int2> items[2];
    for (int p = 0; p < 2; p++) {
        for (int l = 0; l < n; l++) {
            const StepArgs& a = args[l];
            const long long tiles = (long long)a.tiles_x * a.tiles_y;
            for (long long t = 0; t < tiles; t++) items[p].push_back(make_int2(l, (int)t));
            const int ns = p ? b->lat[l]->nspecial : b->lat[l]->nspecial0;
            const int chunks = (2 * ns + kSpecialChunk - 1) / kSpecialChunk;
            for (int c = 0; c < chunks; c++) items[p].push_back(make_int2(l, -(c + 1)));
        }
        if (items[p].size() > (size_t)0x7fffffff)
            return bfail(b, LBMX_ERR_TOO_LARGE, "lbmx_batch: too many work items");
        if ((int)items[p].size() > b->items_cap[p]) {
            cudaFree(b->d_items[p]);
            b->d_items[p] = nullptr;
            BATCH_CUDA(b, cudaMalloc((void**)&b->d_items[p], items[p].size() * sizeof(int2)));
            b->items_cap[p] = (int)items[p].size();
        }
        BATCH_CUDA(b, cudaMemcpyAsync(b->d_items[p], items[p].data(), items[p].size() * sizeof(int2),
                                      cudaMemcpyHostToDevice, b->stream));
        b->nitems[p] = (int)items[p].size();
    }
    BATCH_CUDA(b, cudaStreamSynchronize(b->stream));
    b->host_args.swap(args);
    b->args_tile_w = tw;
    b->args_tile_h = th;
    b->lean = true;
    for (const lbmx_handle* h : b->lat) b->lean = b->lean && !h->force && !h->gamma;
    return LBMX_OK;
}

// Launches of step index s (edge pre-passes of the lattices that need one,
// then the batched step kernel).
static lbmx_status launch_one(lbmx_batch* b, long long s, int variant) {
    const int n = (int)b->lat.size();
    const int parity = (int)(s & 1);
    for (int l = 0; l < n; l++) {
        lbmx_handle* h = b->lat[l];
        if (!h->has_aux_bc) continue;
        StepArgs a = base_args(h);
        set_step(h, a, s);
        BATCH_CUDA(b, dispatch(b->storage, [&](auto tag) {
                       return launch_edge_prepass<decltype(tag)>(a, h->aux, b->stream);
                   }));
    }
    BatchArgs ba;
    ba.lat = b->d_args + ((size_t)variant * 2 + parity) * n;
    ba.tmaps = b->d_tmaps;
    ba.items = b->d_items[parity];
    ba.nitems = b->nitems[parity];
    ba.chunk = b->cfg.chunk;
    ba.counter = b->counter;
    ba.done = b->done;
    ba.error_word = b->error_word;
    ba.step = b->step;
    const unsigned grid = (unsigned)std::max(1, std::min(b->nitems[parity], b->cfg.ctas_per_sm * b->num_sms));
    // plain steps of lattices without per-node force or Brinkman fields run
    // the kernel without those branches
    const bool lean = variant == 0 && b->lean;
    BATCH_CUDA(b, dispatch(b->storage, [&](auto tag) {
                   return launch_batch_step<decltype(tag)>(ba, b->op, parity, b->cfg.tile_w, b->cfg.tile_h, lean,
                                                           grid, b->stream);
               }));
    return LBMX_OK;
}

// CUDA graphs of graph_steps plain steps, one per parity of the first step.
static lbmx_status build_graphs(lbmx_batch* b) {
    const int len = b->cfg.graph_steps;
    // the kernels' shared-memory attributes are set outside the capture
    BatchArgs none;
    memset(&none, 0, sizeof(none));
    for (int p = 0; p < 2; p++)
        BATCH_CUDA(b, dispatch(b->storage, [&](auto tag) {
                       return launch_batch_step<decltype(tag)>(none, b->op, p, b->cfg.tile_w, b->cfg.tile_h, b->lean, 0,
                                                               b->stream);
                   }));
    for (int p = 0; p < 2; p++) {
        cudaGraph_t g = nullptr;
        BATCH_CUDA(b, cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal));
        lbmx_status st = LBMX_OK;
        for (int i = 0; i < len && st == LBMX_OK; i++) st = launch_one(b, p + i, 0);
        const cudaError_t e = cudaStreamEndCapture(b->stream, &g);
        if (st != LBMX_OK) {
            if (g) cudaGraphDestroy(g);
            return st;
        }
        BATCH_CUDA(b, e);
        const cudaError_t ei = cudaGraphInstantiate(&b->graph[p], g, 0);
        cudaGraphDestroy(g);
        BATCH_CUDA(b, ei);
    }
    b->graph_len = len;
    return LBMX_OK;
}

__global__ void set_step_word(unsigned int* w, unsigned int v) { *w = v; }

// nsteps steps from step count t; last_variant for the final step.
static lbmx_status run_steps(lbmx_batch* b, long long t, int nsteps, int last_variant) {
    // the kernels take the step index for the stochastic-rounding hash from
    // the device (graph replays cannot carry it as an argument); each launch
    // advances it
    set_step_word<<<1, 1, 0, b->stream>>>(b->step, (unsigned int)(t + 1));
    BATCH_CUDA(b, cudaGetLastError());
    int i = 0;
    while (i < nsteps) {
        const int left = nsteps - i;
        const bool graphable = b->cfg.graph_steps > 0 && left - 1 >= b->cfg.graph_steps;
        if (graphable) {
            if (b->graph_len != b->cfg.graph_steps) {
                drop_graphs(b);
                lbmx_status st = build_graphs(b);
                if (st != LBMX_OK) return st;
            }
            BATCH_CUDA(b, cudaGraphLaunch(b->graph[(t + i + 1) & 1], b->stream));
            i += b->cfg.graph_steps;
            continue;
        }
        lbmx_status st = launch_one(b, t + i + 1, i == nsteps - 1 ? last_variant : 0);
        if (st != LBMX_OK) return st;
        i++;
    }
    return LBMX_OK;
}

static lbmx_status check_lattices(lbmx_batch* b) {
    const long long t = b->lat[0]->t;
    for (size_t l = 0; l < b->lat.size(); l++) {
        const lbmx_handle* h = b->lat[l];
        if (!h->initialized) return bfail(b, LBMX_ERR_NOT_INITIALIZED, "lbmx_batch: lattice %zu is not initialised", l);
        if (h->t != t)
            return bfail(b, LBMX_ERR_INVALID_ARGUMENT, "lbmx_batch: lattice %zu is at step %lld, lattice 0 at %lld", l,
                         h->t, t);
        if (h->nm > 0) return bfail(b, LBMX_ERR_UNSUPPORTED, "lbmx_batch: lattice %zu carries IBM markers", l);
    }
    return LBMX_OK;
}

static lbmx_status wait_lattices(lbmx_batch* b) {
    if (!b->own_stream) return LBMX_OK;
    for (size_t i = 0; i < b->streams.size(); i++) {
        BATCH_CUDA(b, cudaEventRecord(b->stream_events[i], b->streams[i]));
        BATCH_CUDA(b, cudaStreamWaitEvent(b->stream, b->stream_events[i], 0));
    }
    return LBMX_OK;
}

static lbmx_status release_lattices(lbmx_batch* b) {
    if (!b->own_stream) return LBMX_OK;
    BATCH_CUDA(b, cudaEventRecord(b->end_event, b->stream));
    for (cudaStream_t s : b->streams) BATCH_CUDA(b, cudaStreamWaitEvent(s, b->end_event, 0));
    return LBMX_OK;
}

extern "C" {

void lbmx_batch_destroy(lbmx_batch* b) {
    if (!b) return;
    int cur = 0;
    cudaGetDevice(&cur);
    cudaSetDevice(b->device);
    // a borrowed stream belongs to the lattices and may already be gone:
    // wait for the device instead of touching it
    if (b->own_stream && b->stream) cudaStreamSynchronize(b->stream);
    else cudaDeviceSynchronize();
    drop_graphs(b);
    cudaFree(b->d_args); cudaFree(b->d_tmaps); cudaFree(b->d_items[0]); cudaFree(b->d_items[1]);
    cudaFree(b->counter); cudaFree(b->done); cudaFree(b->error_word); cudaFree(b->step);
    for (cudaEvent_t e : b->stream_events) cudaEventDestroy(e);
    if (b->end_event) cudaEventDestroy(b->end_event);
    if (b->own_stream && b->stream) cudaStreamDestroy(b->stream);
    cudaSetDevice(cur);
    delete b;
}

lbmx_status lbmx_batch_create(lbmx_handle* const* lattices, int32_t count, lbmx_batch** out) {
    if (!out) return bfail(nullptr, LBMX_ERR_INVALID_ARGUMENT, "lbmx_batch_create: out is NULL");
    *out = nullptr;
    if (!lattices || count < 1) return bfail(nullptr, LBMX_ERR_INVALID_ARGUMENT, "lbmx_batch_create: no lattices");
    const lbmx_handle* h0 = lattices[0];
    for (int l = 0; l < count; l++) {
        const lbmx_handle* h = lattices[l];
        if (!h) return bfail(nullptr, LBMX_ERR_INVALID_ARGUMENT, "lbmx_batch_create: lattice %d is NULL", l);
        if (h->p.device != h0->p.device || h->p.storage != h0->p.storage || h->p.op != h0->p.op)
            return bfail(nullptr, LBMX_ERR_INVALID_ARGUMENT,
                         "lbmx_batch_create: lattice %d differs from lattice 0 in device, storage or operator", l);
        for (int k = 0; k < l; k++)
            if (lattices[k] == h)
                return bfail(nullptr, LBMX_ERR_INVALID_ARGUMENT, "lbmx_batch_create: lattice %d appears twice", l);
    }
    if (h0->p.op == LBMX_CM_OPT)
        return bfail(nullptr, LBMX_ERR_UNSUPPORTED,
                     "lbmx_batch_create: CM_OPT needs a grid-wide average before each step; step it alone");
    if (cudaSetDevice(h0->p.device) != cudaSuccess)
        return bfail(nullptr, LBMX_ERR_CUDA, "lbmx_batch_create: cannot select device %d", h0->p.device);
    lbmx_batch* b = new lbmx_batch();
    b->lat.assign(lattices, lattices + count);
    b->device = h0->p.device;
    b->storage = h0->p.storage;
    b->op = h0->p.op;
    b->num_sms = std::max(1, h0->num_sms);
    lbmx_status st = check_lattices(b);
    if (st != LBMX_OK) {
        bfail(nullptr, st, "%s", b->err);
        delete b;
        return st;
    }
    auto cleanup = [&](lbmx_status code, const char* what) {
        bfail(nullptr, code, "lbmx_batch_create: %s", what);
        lbmx_batch_destroy(b);
        return code;
    };
    for (lbmx_handle* h : b->lat)
        if (std::find(b->streams.begin(), b->streams.end(), h->stream) == b->streams.end())
            b->streams.push_back(h->stream);
    if (b->streams.size() == 1) {
        // one stream for every lattice: the batch runs on it, no cross-stream waits
        b->stream = b->streams[0];
    } else {
        b->own_stream = true;
        if (cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking) != cudaSuccess ||
            cudaEventCreateWithFlags(&b->end_event, cudaEventDisableTiming) != cudaSuccess)
            return cleanup(LBMX_ERR_CUDA, "cannot create the batch stream");
        for (size_t i = 0; i < b->streams.size(); i++) {
            cudaEvent_t e = nullptr;
            if (cudaEventCreateWithFlags(&e, cudaEventDisableTiming) != cudaSuccess)
                return cleanup(LBMX_ERR_CUDA, "cannot create an event");
            b->stream_events.push_back(e);
        }
    }
    if (cudaMalloc((void**)&b->counter, sizeof(unsigned long long)) != cudaSuccess ||
        cudaMalloc((void**)&b->done, sizeof(unsigned int)) != cudaSuccess ||
        cudaMalloc((void**)&b->error_word, sizeof(unsigned int)) != cudaSuccess ||
        cudaMalloc((void**)&b->step, sizeof(unsigned int)) != cudaSuccess)
        return cleanup(LBMX_ERR_OUT_OF_MEMORY, "cudaMalloc failed");
    cudaMemsetAsync(b->step, 0, sizeof(unsigned int), b->stream);
    cudaMemsetAsync(b->counter, 0, sizeof(unsigned long long), b->stream);
    cudaMemsetAsync(b->done, 0, sizeof(unsigned int), b->stream);
    cudaMemsetAsync(b->error_word, 0, sizeof(unsigned int), b->stream);
    if (refresh(b) != LBMX_OK) return cleanup(LBMX_ERR_CUDA, b->err);
    *out = b;
    return LBMX_OK;
}

lbmx_status lbmx_batch_set_config(lbmx_batch* b, const lbmx_batch_config* cfg) {
    if (!b || !cfg) return bfail(b, LBMX_ERR_INVALID_ARGUMENT, "lbmx_batch_set_config: NULL argument");
    if (!valid_config(*cfg))
        return bfail(b, LBMX_ERR_INVALID_ARGUMENT,
                     "lbmx_batch_set_config: tile_w %d, ctas_per_sm %d, chunk %d, graph_steps %d out of range",
                     cfg->tile_w, cfg->ctas_per_sm, cfg->chunk, cfg->graph_steps);
    cudaSetDevice(b->device);
    const bool relaunch = cfg->tile_w != b->cfg.tile_w || cfg->ctas_per_sm != b->cfg.ctas_per_sm ||
                          cfg->chunk != b->cfg.chunk || cfg->graph_steps != b->cfg.graph_steps;
    b->cfg = *cfg;
    if (relaunch) drop_graphs(b);
    return refresh(b);
}

lbmx_status lbmx_batch_get_config(lbmx_batch* b, lbmx_batch_config* cfg) {
    if (!b || !cfg) return bfail(b, LBMX_ERR_INVALID_ARGUMENT, "lbmx_batch_get_config: NULL argument");
    *cfg = b->cfg;
    return LBMX_OK;
}

lbmx_status lbmx_batch_step(lbmx_batch* b, int32_t nsteps, uint32_t flags) {
    if (!b) return bfail(b, LBMX_ERR_INVALID_ARGUMENT, "lbmx_batch_step: NULL batch");
    if (nsteps < 0) return bfail(b, LBMX_ERR_INVALID_ARGUMENT, "lbmx_batch_step: nsteps < 0");
    if (nsteps == 0) return LBMX_OK;
    cudaSetDevice(b->device);
    lbmx_status st = check_lattices(b);
    if (st != LBMX_OK) return st;
    if ((st = refresh(b)) != LBMX_OK) return st;
    const bool check = (flags & LBMX_STEP_CHECK_FINITE) != 0;
    const int last = check ? 2 : (flags & LBMX_STEP_STORE_MOMENTS) ? 1 : 0;
    const long long t = b->lat[0]->t;
    if ((st = wait_lattices(b)) != LBMX_OK) return st;
    if (check) BATCH_CUDA(b, cudaMemsetAsync(b->error_word, 0, sizeof(unsigned int), b->stream));
    st = run_steps(b, t, nsteps, last);
    if (st != LBMX_OK) return st;
    for (lbmx_handle* h : b->lat) h->t = t + nsteps;
    if ((st = release_lattices(b)) != LBMX_OK) return st;
    if (check) {
        unsigned int w = 0;
        BATCH_CUDA(b, cudaMemcpyAsync(&w, b->error_word, sizeof(w), cudaMemcpyDeviceToHost, b->stream));
        BATCH_CUDA(b, cudaStreamSynchronize(b->stream));
        if (w & 2u) return bfail(b, LBMX_ERR_CUDA, "lbmx_batch_step: a shared-memory staging wait gave up");
        if (w & 1u) return bfail(b, LBMX_ERR_NONFINITE, "lbmx_batch_step: non-finite density at step %lld", t + nsteps);
    }
    return LBMX_OK;
}

lbmx_status lbmx_batch_synchronize(lbmx_batch* b) {
    if (!b) return bfail(b, LBMX_ERR_INVALID_ARGUMENT, "lbmx_batch_synchronize: NULL batch");
    cudaSetDevice(b->device);
    unsigned int w = 0;
    BATCH_CUDA(b, cudaMemcpyAsync(&w, b->error_word, sizeof(w), cudaMemcpyDeviceToHost, b->stream));
    BATCH_CUDA(b, cudaStreamSynchronize(b->stream));
    if (w & 2u) {
        BATCH_CUDA(b, cudaMemsetAsync(b->error_word, 0, sizeof(w), b->stream));
        return bfail(b, LBMX_ERR_CUDA, "batched step: a shared-memory staging wait gave up; results are invalid");
    }
    return LBMX_OK;
}

lbmx_status lbmx_batch_autotune(lbmx_batch* b, int32_t trial_steps, lbmx_batch_config* chosen) {
    if (!b) return bfail(b, LBMX_ERR_INVALID_ARGUMENT, "lbmx_batch_autotune: NULL batch");
    if (trial_steps < 1) return bfail(b, LBMX_ERR_INVALID_ARGUMENT, "lbmx_batch_autotune: trial_steps < 1");
    cudaSetDevice(b->device);
    lbmx_status st = check_lattices(b);
    if (st != LBMX_OK) return st;
    // snapshot of every lattice's dynamic state (populations, edge store)
    size_t total = 0;
    std::vector<size_t> fb(b->lat.size()), eb(b->lat.size());
    for (size_t l = 0; l < b->lat.size(); l++) {
        const lbmx_handle* h = b->lat[l];
        fb[l] = (size_t)h->nplanes * h->g.plane * elem_size(h->p.storage);
        eb[l] = (size_t)2 * h->g.perimeter * 9 * sizeof(float);
        total += (fb[l] + eb[l] + 255) / 256 * 256;
    }
    char* snap = nullptr;
    BATCH_CUDA(b, cudaMalloc((void**)&snap, total));
    if ((st = wait_lattices(b)) != LBMX_OK) {
        cudaFree(snap);
        return st;
    }
    auto copy_state = [&](bool save) -> cudaError_t {
        size_t o = 0;
        for (size_t l = 0; l < b->lat.size(); l++) {
            lbmx_handle* h = b->lat[l];
            char* s = snap + o;
            cudaError_t e = save ? cudaMemcpyAsync(s, h->f, fb[l], cudaMemcpyDeviceToDevice, b->stream)
                                 : cudaMemcpyAsync(h->f, s, fb[l], cudaMemcpyDeviceToDevice, b->stream);
            if (e == cudaSuccess)
                e = save ? cudaMemcpyAsync(s + fb[l], h->edge, eb[l], cudaMemcpyDeviceToDevice, b->stream)
                         : cudaMemcpyAsync(h->edge, s + fb[l], eb[l], cudaMemcpyDeviceToDevice, b->stream);
            if (e != cudaSuccess) return e;
            o += (fb[l] + eb[l] + 255) / 256 * 256;
        }
        return cudaSuccess;
    };
    cudaError_t ce = copy_state(true);
    if (ce != cudaSuccess) {
        cudaFree(snap);
        BATCH_CUDA(b, ce);
    }
    const lbmx_batch_config keep = b->cfg;
    lbmx_batch_config best = keep;
    float best_ms = -1.0f;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    const long long t0 = b->lat[0]->t;
    long long t = t0;
    st = LBMX_OK;
    static const int shapes[3][2] = {{64, 8}, {128, 4}, {128, 8}};
    static const int chunks[5] = {1, 2, 4, 8, 16};
    for (int ti = 0; ti < 3 && st == LBMX_OK; ti++)
        for (int c = 1; c <= kCtasPerSm && st == LBMX_OK; c++)
            for (int ki = 0; ki < 5 && st == LBMX_OK; ki++) {
                // trials launch directly: one launch per step for every
                // candidate, so graphs would not change the ranking
                lbmx_batch_config cand{shapes[ti][0], shapes[ti][1], c, chunks[ki], 0};
                b->cfg = cand;
                drop_graphs(b);
                if ((st = refresh(b)) != LBMX_OK) break;
                if ((st = run_steps(b, t, 2, 0)) != LBMX_OK) break;
                t += 2;
                if (cudaEventRecord(e0, b->stream) != cudaSuccess) { st = LBMX_ERR_CUDA; break; }
                if ((st = run_steps(b, t, trial_steps, 0)) != LBMX_OK) break;
                t += trial_steps;
                if (cudaEventRecord(e1, b->stream) != cudaSuccess || cudaEventSynchronize(e1) != cudaSuccess) {
                    st = bfail(b, LBMX_ERR_CUDA, "lbmx_batch_autotune: trial failed");
                    break;
                }
                float ms = 0.0f;
                cudaEventElapsedTime(&ms, e0, e1);
                if (best_ms < 0.0f || ms < best_ms) {
                    best_ms = ms;
                    best = cand;
                    best.graph_steps = keep.graph_steps;
                }
            }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    // put the lattices back as they were; trial steps count for nothing
    ce = copy_state(false);
    const cudaError_t ws = cudaStreamSynchronize(b->stream);
    cudaFree(snap);
    for (lbmx_handle* h : b->lat) h->t = t0;
    drop_graphs(b);
    b->cfg = (st == LBMX_OK) ? best : keep;
    if (st != LBMX_OK) {
        refresh(b);
        return st;
    }
    BATCH_CUDA(b, ce);
    BATCH_CUDA(b, ws);
    if ((st = refresh(b)) != LBMX_OK) return st;
    if ((st = release_lattices(b)) != LBMX_OK) return st;
    if (chosen) *chosen = b->cfg;
    return lbmx_batch_synchronize(b);
}

const char* lbmx_batch_last_error(lbmx_batch* b) { return b ? b->err : g_batch_err; }

}  // extern "C"
