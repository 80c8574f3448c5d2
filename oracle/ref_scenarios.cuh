// ref_scenarios.cuh -- golden-vector scenarios written against the
// reference's scenario contract (ScenarioTrait<Init, Boundary, Validation,
// CollisionOp>, src/scenarios/scenario.cuh:22-78).  Test infrastructure:
// compiled only into oracle/ref_harness.cu against the patched reference.
//
// Selected by -D flags:
//   LBX_CASE  1 Taylor-Green (periodic), 2 lid-driven cavity with the
//             reference's regularized walls (lidDrivenCavityFunctors.cuh:41-56),
//             3 body-force channel with bounce-back walls and an IBM cylinder,
//             4 Zou-He inlet / zero-gradient outlet channel with an IBM
//             cylinder, 5 Zou-He inlet / pressure outlet channel
//   LBX_OPID  0 BGK<2>, 1 MRT<2>, 2 CM<2,NoAdapter>, 3 CM<2,OptimalAdapter>
//   LBX_NU    kinematic viscosity;  LBX_NO_MARKERS drops the IBM body
#pragma once
#include "scenarios/scenario.cuh"
#include "IBM/IBM_generators.cuh"

#if LBX_OPID == 0
using LbxOp = BGK<2>;
#elif LBX_OPID == 1
using LbxOp = MRT<2>;
#elif LBX_OPID == 2
using LbxOp = CM<2, NoAdapter>;
#else
using LbxOp = CM<2, OptimalAdapter>;
#endif

#if LBX_CASE == 1
#define LBX_UMAX 0.04f
#elif LBX_CASE == 2
#define LBX_UMAX 0.1f
#else
#define LBX_UMAX 0.05f
#endif

#if LBX_CASE == 3
// force for u_max = 0.05 between the walls (poiseuilleFunctors.cuh:37)
#define LBX_FX (8.0f * LBX_NU * LBX_UMAX / (float)(NY * NY))
#else
#define LBX_FX 0.0f
#endif

struct GoldenInit {
    float u0;
    __host__ __device__ GoldenInit(float u0_) : u0(u0_) {}

    __host__ __device__ void apply_forces(float* rho, float* u, float* force, int node) {
        force[get_vec_index(node, 0)] = LBX_FX;
        force[get_vec_index(node, 1)] = 0.0f;
    }

    __device__ void operator()(float* rho, float* u, float* force, int node) {
        float r = 1.0f, ux = 0.0f, uy = 0.0f;
#if LBX_CASE == 1
        const int x = node % NX, y = node / NX;
        const float k = 2.0f * 3.14159265358979f / (float)NX;
        ux = u0 * sinf(k * x) * cosf(k * y);
        uy = -u0 * cosf(k * x) * sinf(k * y);
        r = 1.0f - 3.0f * (u0 * u0 / 4.0f) * (cosf(2.0f * k * x) + cosf(2.0f * k * y));
#endif
        rho[node] = r;
        u[get_vec_index(node, 0)] = ux;
        u[get_vec_index(node, 1)] = uy;
        apply_forces(rho, u, force, node);
    }
};

struct GoldenBoundary {
    __host__ __device__ int operator()(int x, int y) const {
#if LBX_CASE == 2
        if ((x == 0 || x == NX - 1) && (y == 0 || y == NY - 1)) return BC_flag::REGULARIZED_BOUNCE_BACK_CORNER;
        if (y == NY - 1) return BC_flag::REGULARIZED_INLET_TOP;
        if (x == 0 || x == NX - 1 || y == 0) return BC_flag::REGULARIZED_BOUNCE_BACK;
        return BC_flag::FLUID;
#elif LBX_CASE == 3
        return (y == 0 || y == NY - 1) ? BC_flag::BOUNCE_BACK : BC_flag::FLUID;
#elif LBX_CASE == 4 || LBX_CASE == 5
        if (y == 0 || y == NY - 1) return BC_flag::BOUNCE_BACK;
        if (x == 0) return BC_flag::ZOU_HE_LEFT;
        if (x == NX - 1) return LBX_CASE == 4 ? BC_flag::ZG_OUTFLOW : BC_flag::PRESSURE_OUTLET;
        return BC_flag::FLUID;
#else
        return BC_flag::FLUID;
#endif
    }
};

struct GoldenScenario : public ScenarioTrait<GoldenInit, GoldenBoundary, void, LbxOp> {
    static constexpr float u_max = LBX_UMAX;
    static constexpr float viscosity = LBX_NU;
    static constexpr float tau = viscosity_to_tau(viscosity);
    static constexpr float omega = 1.0f / tau;
#if LBX_OPID == 1
    static constexpr float S[quadratures] = {0.0f, 1.0f, 1.4f, 0.0f, 1.2f, 0.0f, 1.9f, omega, omega};
#else
    static constexpr float S[quadratures] = {0.0f, 0.0f, 0.0f, 1.0f, omega, omega, 1.0f, 1.0f, 1.0f};
#endif

    static const char* name() { return "Golden"; }
    static InitType init() { return InitType(u_max); }
    static BoundaryType boundary() { return BoundaryType(); }

    static void add_bodies() {
#if (LBX_CASE == 3 || LBX_CASE == 4) && !defined(LBX_NO_MARKERS)
        IBM_bodies.push_back(create_cylinder(NX / 4.0f + 0.3f, NY / 2.0f + 0.1f, NY / 8.0f, 16));
#endif
    }
};
