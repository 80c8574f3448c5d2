// lbmx_scenario.cuh -- run an unchanged cuda-lbm scenario on the engine.
//
// A reference scenario is a ScenarioTrait struct plus an Init functor
// (operator()(rho, u, force, node), evaluated on the device), a Boundary
// functor ((x, y) -> BC_flag, evaluated on the host), S/omega/u_max
// constants and optional IBM bodies (src/scenarios/scenario.cuh:22-78).
// lbmx_compat::create<Scenario>() does what the reference's
// LBM<2>::allocate/init do with them (src/core/lbm.cuh:92-125,
// src/core/init/init.cuh:45-86) and hands the results to the C-ABI:
//
//   #define NX 256
//   #define NY 256
//   #define PERIODIC_X                    // the reference's streaming macros
//   #define PERIODIC_Y
//   #include "lbmx_scenario.cuh"          // -I cuda-lbm_gb300/compat -I include
//   #include "scenarios/taylorGreen/taylorGreenScenario.cuh"
//   lbmx_compat::Solver<TaylorGreenScenario> sim;
//   lbmx_compat::create<TaylorGreenScenario>(&sim.h);
//   sim.step(1000);
//   float err = TaylorGreenScenario::compute_error(sim);
//
// One scenario per translation unit (the functors' device constants are
// per translation unit).  Init::apply_forces is evaluated once, at init: the
// engine keeps that force field (the reference re-applies it every step,
// macroscopics.cuh:13-48, which is the same for a state-independent force).
#pragma once
#include <cuda_runtime.h>

#include <cstdint>
#include <cstring>
#include <vector>

#include "lbmx.h"
#include "scenarios/scenario.cuh"

namespace lbmx_compat {

template <class Init>
__global__ void run_init_functor(Init init, float* rho, float* u, float* force, int n) {
    const int node = blockIdx.x * blockDim.x + threadIdx.x;
    if (node < n) init(rho, u, force, node);
}

// the device constants the scenario's functors may read (vis, tau, omega,
// C, OPP, WEIGHTS, S -- the reference's send_consts, src/core/lbm.cuh:63-82)
template <class Scenario>
inline cudaError_t upload_constants() {
    const float v = Scenario::viscosity, t = Scenario::tau, o = Scenario::omega;
    cudaError_t e = cudaMemcpyToSymbol(vis, &v, sizeof(float));
    if (e == cudaSuccess) e = cudaMemcpyToSymbol(tau, &t, sizeof(float));
    if (e == cudaSuccess) e = cudaMemcpyToSymbol(omega, &o, sizeof(float));
    if (e == cudaSuccess) e = cudaMemcpyToSymbol(C, h_C, sizeof(h_C));
    if (e == cudaSuccess) e = cudaMemcpyToSymbol(OPP, h_OPP, sizeof(h_OPP));
    if (e == cudaSuccess) e = cudaMemcpyToSymbol(WEIGHTS, h_weights, sizeof(h_weights));
    if (e == cudaSuccess) e = cudaMemcpyToSymbol(S, Scenario::S, sizeof(float) * 9);
    return e;
}

// The members of LBM<2> a scenario's compute_error reads: h_rho, h_u (AoS,
// u[2*node + c]), timestep, update_ts and update_macroscopics().
template <class Scenario>
struct Solver {
    lbmx_handle* h = nullptr;
    std::vector<float> h_rho, h_u;
    int timestep = 0, update_ts = 0;

    ~Solver() { lbmx_destroy(h); }

    // n reference time steps; Scenario::update_ts sees every step index
    lbmx_status step(int n) {
        for (int i = 0; i < n; i++) Scenario::update_ts((float)(++timestep));
        return lbmx_step(h, n);
    }

    void update_macroscopics() {
        const int n = NX * NY;
        std::vector<float> planes(2 * (size_t)n);
        h_rho.resize(n);
        h_u.resize(2 * (size_t)n);
        if (lbmx_moments(h, h_rho.data(), planes.data(), nullptr) != LBMX_OK) return;
        for (int i = 0; i < n; i++) {
            h_u[2 * i] = planes[i];
            h_u[2 * i + 1] = planes[n + i];
        }
        update_ts = timestep;
    }
};

// Build an engine handle for Scenario: lattice NX x NY, periodicity from
// PERIODIC_X / PERIODIC_Y, the scenario's operator, S, omega and u_max.
template <class Scenario>
inline lbmx_status create(lbmx_handle** out, uint32_t quirks = LBMX_QUIRKS_REFERENCE,
                          int storage = LBMX_STORAGE_F32, int device = 0) {
    constexpr int n = NX * NY;
    *out = nullptr;
    lbmx_params p;
    lbmx_params_default(&p);
    p.nx = NX;
    p.ny = NY;
#ifdef PERIODIC_X
    p.periodic_x = 1;
#endif
#ifdef PERIODIC_Y
    p.periodic_y = 1;
#endif
    p.op = Scenario::CollisionOp::lbmx_op;
    if (p.op < 0) return LBMX_ERR_UNSUPPORTED;
    p.storage = storage;
    p.quirks = quirks;
    p.device = device;
    p.omega = Scenario::omega;
    for (int i = 0; i < 9; i++) p.S[i] = Scenario::S[i];
    p.u_bc = Scenario::u_max;
    lbmx_handle* h = nullptr;
    lbmx_status st = lbmx_create(&p, &h);
    if (st != LBMX_OK) return st;

    // Init functor on the device, into AoS staging (init.cuh:29-43)
    if (cudaSetDevice(device) != cudaSuccess || upload_constants<Scenario>() != cudaSuccess) {
        lbmx_destroy(h);
        return LBMX_ERR_CUDA;
    }
    float* d = nullptr;
    if (cudaMalloc(&d, 5 * sizeof(float) * (size_t)n) != cudaSuccess) {
        lbmx_destroy(h);
        return LBMX_ERR_OUT_OF_MEMORY;
    }
    cudaMemset(d, 0, 5 * sizeof(float) * (size_t)n);
    run_init_functor<<<(n + 255) / 256, 256>>>(Scenario::init(), d, d + n, d + 3 * n, n);
    std::vector<float> host(5 * (size_t)n);
    const cudaError_t e = cudaMemcpy(host.data(), d, host.size() * sizeof(float), cudaMemcpyDeviceToHost);
    cudaFree(d);
    if (e != cudaSuccess) {
        lbmx_destroy(h);
        return LBMX_ERR_CUDA;
    }
    std::vector<float> rho(host.begin(), host.begin() + n), u(2 * (size_t)n), force(2 * (size_t)n);
    for (int i = 0; i < n; i++) {
        u[i] = host[n + 2 * i];
        u[n + i] = host[n + 2 * i + 1];
        force[i] = host[3 * n + 2 * i];
        force[n + i] = host[3 * n + 2 * i + 1];
    }

    // Boundary functor on the host, y outer / x inner (boundaries.cuh:170-197)
    std::vector<uint8_t> flags(n);
    auto bc = Scenario::boundary();
    for (int y = 0; y < NY; y++)
        for (int x = 0; x < NX; x++) flags[y * NX + x] = (uint8_t)bc(x, y);

    // IBM bodies (IBMManager::init_and_dispatch, IBMManager.cuh:54-109)
    Scenario::IBM_bodies.clear();
    Scenario::add_bodies();
    std::vector<float> xy;
    for (const IBMBody& b : Scenario::IBM_bodies) xy.insert(xy.end(), b.points, b.points + 2 * b.num_points);

    if ((st = lbmx_set_flags(h, flags.data())) != LBMX_OK ||
        (st = lbmx_init_from_fields(h, rho.data(), u.data(), force.data())) != LBMX_OK ||
        (xy.size() && (st = lbmx_ibm_set_markers(h, xy.data(), (int32_t)(xy.size() / 2))) != LBMX_OK)) {
        lbmx_destroy(h);
        return st;
    }
    *out = h;
    return LBMX_OK;
}

}  // namespace lbmx_compat
