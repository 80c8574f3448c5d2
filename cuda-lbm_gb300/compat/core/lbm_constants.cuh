// lbmx compat: the lattice names a cuda-lbm scenario uses
// (src/core/lbm_constants.cuh).  Values that are a data format -- the D2Q9
// velocity order, OPP, the weights and the BC_flag numbers -- are the
// reference's; field indexing is AoS, the layout the reference's 2-D
// functors write (u[2*node]) and that the compat driver converts.
#ifndef LBM_CONSTANTS_H
#define LBM_CONSTANTS_H
#include <math.h>
#include <stdint.h>

#include "defines.hpp"

constexpr uint8_t dimensions = 2;
constexpr uint8_t quadratures = 9;
const float cs = 0.577350269189625764f;
const float cs2 = 1.0f / 3.0f;

// rest, E, N, W, S, NE, NW, SW, SE
const int h_C[18] = {0, 0, 1, 0, 0, 1, -1, 0, 0, -1, 1, 1, -1, 1, -1, -1, 1, -1};
const int h_OPP[9] = {0, 3, 4, 1, 2, 7, 8, 5, 6};
const float h_weights[9] = {4.0f / 9.0f, 1.0f / 9.0f, 1.0f / 9.0f, 1.0f / 9.0f, 1.0f / 9.0f,
                            1.0f / 36.0f, 1.0f / 36.0f, 1.0f / 36.0f, 1.0f / 36.0f};

#ifndef M_PI
#define M_PI 3.14159265358979323846
#endif

// device constants a functor may read; the compat driver fills them for the
// scenario it builds (one scenario per translation unit)
static __constant__ float WEIGHTS[9];
static __constant__ int C[18];
static __constant__ int OPP[9];
static __constant__ float vis;
static __constant__ float tau;
static __constant__ float omega;
static __constant__ float S[9];

constexpr int num_nodes = NX * NY * NZ;

__host__ __device__ __forceinline__ int get_node_index(int node, int quadrature = 0) {
    return node * quadratures + quadrature;
}
__host__ __device__ __forceinline__ int get_vec_index(int node, int component) { return node * dimensions + component; }
__host__ __device__ __forceinline__ int get_node_from_coords(int x, int y, int z = 0) { return y * NX + x; }
__host__ __device__ __forceinline__ void get_coords_from_node(int node, int& x, int& y, int& z) {
    x = node % NX;
    y = node / NX;
    z = 0;
}

constexpr inline float viscosity_to_tau(float v) { return 3 * v + 0.5f; }
constexpr inline float tau_to_viscosity(float t) { return (t - 0.5f) / 3.0f; }
constexpr float compute_reynolds(float u_max, float domain_size, float viscosity) { return (u_max * domain_size) / viscosity; }

// boundary flags: the reference's numbering (lbm_constants.cuh:376-396)
enum BC_flag {
    FLUID,
    BOUNCE_BACK,
    ZOU_HE_TOP,
    ZOU_HE_LEFT,
    ZOU_HE_TOP_LEFT_TOP_INFLOW,
    ZOU_HE_TOP_RIGHT_TOP_INFLOW,
    CYLINDER,
    ZG_OUTFLOW,
    PRESSURE_OUTLET,
    REGULARIZED_INLET_TOP,
    REGULARIZED_INLET_LEFT,
    REGULARIZED_BOUNCE_BACK,
    REGULARIZED_BOUNCE_BACK_CORNER,
    EXTRAPOLATED_CORNER_EDGE,
    CORNER_EDGE_BOUNCE_BACK,
    PRESSURE_INLET_LEFT,
    GUO_VELOCITY_INLET,
    GUO_PRESSURE_OUTLET,
    REGULARIZED_OUTLET,
};

#endif
