// lbmx compat: the scenario contract of cuda-lbm
// (ScenarioTrait<Init, Boundary, Validation, CollisionOp, Adapter>,
// src/scenarios/scenario.cuh:22-78), member for member, so a scenario header
// written for the reference compiles unchanged.  lbmx_compat::create()
// (lbmx_scenario.cuh) turns a scenario into an engine handle.
#ifndef FLOW_SCENARIO_H
#define FLOW_SCENARIO_H

#include <array>
#include <string>
#include <type_traits>
#include <vector>

#include "IBM/IBMBody.cuh"
#include "IBM/IBM_generators.cuh"
#include "core/collision/collision.cuh"

// S matrix with every non-conserved MRT moment relaxed at omega_val
#define DEFAULT_MRT_S_MATRIX(omega_val) \
    {0.0f, omega_val, omega_val, 0.0f, omega_val, 0.0f, omega_val, omega_val, omega_val}

template <typename InitFunctor, typename BoundaryFunctor, typename ValidationFunctor = void,
          typename CollisionType = BGK<2>, typename AdapterType = NoAdapter>
struct ScenarioTrait {
    using InitType = InitFunctor;
    using BoundaryType = BoundaryFunctor;
    using ValidationType = ValidationFunctor;
    using CollisionOp = CollisionType;
    using AdapterOp = AdapterType;

    static constexpr float viscosity = 1.0f / 6.0f;
    static constexpr float tau = viscosity_to_tau(viscosity);
    static constexpr float omega = 1.0f / tau;
    static inline float t = 0.0f;
    static inline std::vector<IBMBody> IBM_bodies;

    // a scenario that uses MRT or CM defines its own S; this default relaxes
    // every non-conserved moment at omega (BGK-equivalent MRT)
    static constexpr float S[quadratures] = {0.0f, omega, omega, 0.0f, omega, 0.0f, omega, omega, omega};

    static constexpr float u_max = 0.1f;

    static const char* name() { return "BaseScenario"; }
    static InitType initCondition() { return InitType(); }
    static BoundaryType boundaryCondition() { return BoundaryType(); }

    static constexpr bool has_analytical_solution = !std::is_same<ValidationFunctor, void>::value;

    template <typename LBMSolver>
    static float compute_error(LBMSolver& solver);

    static void add_bodies() {}
    static void update_ts(float new_ts) { t = new_ts; }
};

#endif
