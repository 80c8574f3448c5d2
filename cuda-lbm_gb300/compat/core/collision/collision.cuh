// lbmx compat: the collision-operator tags a scenario names as its
// CollisionOp (BGK<2>, MRT<2>, CM<2, NoAdapter>, CM<2, OptimalAdapter>;
// src/core/collision/{BGK,MRT,CM}, adapters.cuh).  Here they only select the
// engine's operator: lbmx_op is the LBMX_* value lbmx_create receives.
#ifndef COLLISION_OPS_H
#define COLLISION_OPS_H
#include "core/lbm_constants.cuh"
#include "lbmx.h"

struct MomentInfo {
    float rho_avg_norm;
    float j_avg_norm;
    float pi_avg_norm;
};

struct AdapterBase {
    static constexpr int i_star = 5;
};
struct NoAdapter : AdapterBase {
    static constexpr int lbmx_op = LBMX_CM;
};
struct OptimalAdapter : AdapterBase {
    static constexpr int lbmx_op = LBMX_CM_OPT;
};
// the reference's EmpiricalAdapter exists only for D3Q27
struct EmpiricalAdapter : AdapterBase {
    static constexpr int lbmx_op = -1;
};

template <int dim>
struct BGK {
    static_assert(dim == 2, "lbmx runs the D2Q9 lattice");
    static constexpr int lbmx_op = LBMX_BGK;
};
template <int dim>
struct MRT {
    static_assert(dim == 2, "lbmx runs the D2Q9 lattice");
    static constexpr int lbmx_op = LBMX_MRT;
};
template <int dim, typename AdapterType = NoAdapter>
struct CM {
    static_assert(dim == 2, "lbmx runs the D2Q9 lattice");
    static constexpr int lbmx_op = AdapterType::lbmx_op;
};

#endif
