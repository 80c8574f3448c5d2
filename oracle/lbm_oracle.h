/*
 * lbm_oracle.h -- CPU restatement of the reference D2Q9 time step.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the checker for the CUDA
 * engine (tests/, __graft_entry__.smoke() and the CPU-baseline leg of
 * bench.py); the product never links or calls it.
 *
 * It follows the reference's host loop (src/main.cu:96-114) step by step,
 * with the same ping-pong push-streaming buffers the reference uses, so it is
 * an independent formulation of the in-place streaming done by the engine:
 *   stream (push, q = 1..8)  src/core/streaming/streaming.cu:3-33
 *   swap                     src/core/lbm.cuh:345-350
 *   boundaries               src/core/boundaries/boundaries.cuh:10-85
 *   macroscopics             src/core/macroscopics/macroscopics.cu:4-38
 *   reset forces             src/core/macroscopics/macroscopics.cuh:13-48
 *   IBM multi-direct         src/IBM/IBMManager.cuh:222-252
 *   correct macroscopics     src/core/macroscopics/macroscopics.cu:98-110
 *   moment averages          src/core/macroscopics/macroscopics.cuh:50-120
 *   equilibrium              src/core/equilibrium/equilibrium.cu:5-39
 *   collide                  src/core/collision/{BGK,MRT,CM}
 *
 * Built twice: liboracle64 (double) and liboracle32 (float arithmetic, closer
 * to the reference's FP32 operation order).  Every array crossing this API is
 * double precision; layouts are y-major nodes (node = y*nx + x) and
 * component planes (ux plane then uy plane; population q plane q).
 *
 * Parity status: pinned against dumps of the patched reference build where
 * tests/golden/ holds them (see tests/golden/make_golden.sh); otherwise pinned
 * only by the reference's analytic validators (Taylor-Green decay,
 * Poiseuille profile).
 */
#ifndef LBM_ORACLE_H
#define LBM_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* collision operators (reference: BGK<2>, MRT<2>, CM<2,NoAdapter>, CM<2,OptimalAdapter>) */
enum { LBO_BGK = 0, LBO_MRT = 1, LBO_CM = 2, LBO_CM_OPT = 3 };

/* reproduce-the-reference switches (bit mask) */
enum {
    LBO_QUIRK_REST_LAG    = 1 << 0, /* q=0 never streamed: f0 from two steps back (streaming.cu:9) */
    LBO_QUIRK_ZOUHE_LEFT  = 1 << 1, /* rho uses f2 where f3 belongs (zouHeInflow.cuh:15-16)      */
    LBO_QUIRK_MRT_FORCE   = 1 << 2, /* forcing moments in [jx,jy,qx,qy] order (MRT.cu:18-19)      */
    LBO_QUIRK_IBM_2X2     = 1 << 3, /* 2x2 stencil of the 4-point kernel (IBM_impl.cu:19-20)      */
    LBO_QUIRK_IBM_CLAMP   = 1 << 4, /* drop negative forces / velocities (IBM_impl.cuh:22-24,42-44) */
    LBO_QUIRKS_REFERENCE  = 0x1f
};

/* boundary flags: values 0..12 are the reference's BC_flag (lbm_constants.cuh:376-396);
 * 32..35 are boundaries the reference does not have; 36..37 are reference
 * functors its 2-D boundary kernel never dispatches (CornerBoundary). */
enum {
    LBO_FLUID = 0, LBO_BOUNCE_BACK = 1, LBO_ZOU_HE_TOP = 2, LBO_ZOU_HE_LEFT = 3,
    LBO_ZOU_HE_TOP_LEFT_TOP_INFLOW = 4, LBO_ZOU_HE_TOP_RIGHT_TOP_INFLOW = 5,
    LBO_CYLINDER = 6, LBO_ZG_OUTFLOW = 7, LBO_PRESSURE_OUTLET = 8,
    LBO_REGULARIZED_INLET_TOP = 9, LBO_REGULARIZED_INLET_LEFT = 10,
    LBO_REGULARIZED_BOUNCE_BACK = 11, LBO_REGULARIZED_BOUNCE_BACK_CORNER = 12,
    LBO_MOVING_WALL_BB = 32, LBO_ZOU_HE_PRESSURE_RIGHT = 33, LBO_ZOU_HE_PARABOLIC_LEFT = 34,
    LBO_HALFWAY_BB = 35, LBO_CORNER_TOP_LEFT = 36, LBO_CORNER_BOTTOM_LEFT = 37
};

typedef struct lbo_params {
    int nx, ny;
    int periodic_x, periodic_y;
    int op;            /* LBO_* operator */
    int quirks;        /* LBO_QUIRK_* mask */
    int ibm_iters;     /* multi-direct iterations (reference ITER_MAX = 3) */
    int threads;       /* OpenMP threads (0 = runtime default) */
    double omega;      /* BGK relaxation rate */
    double S[9];       /* MRT rates (M row order) or CM rates (central-moment order) */
    double u_bc;       /* Scenario::u_max used by Zou-He / regularized inlets */
    double wall_ux, wall_uy; /* moving-wall velocity */
    double rho_out;    /* Zou-He pressure outlet density */
    double ibm_ds;     /* marker arc-length weight on spread forces (reference: 1) */
} lbo_params;

typedef struct lbo lbo;

lbo*  lbo_create(const lbo_params* p);
void  lbo_destroy(lbo* o);
int   lbo_set_flags(lbo* o, const uint8_t* flags);
/* rho[n], u[2n], force[2n] (force = Init::apply_forces result, re-applied each step) */
int   lbo_init(lbo* o, const double* rho, const double* u, const double* force);
int   lbo_set_markers(lbo* o, const double* xy, int n);   /* xy AoS [2n] */
/* per-node Brinkman solid fraction gamma[n] (NULL: none); no reference counterpart */
int   lbo_set_gamma(lbo* o, const double* gamma);
int   lbo_step(lbo* o, int nsteps);
long  lbo_time(const lbo* o);
/* post-collision populations of the last step, [9][n] */
void  lbo_get_f(const lbo* o, double* f);
/* the reference's d_rho / d_u / d_force after the last step: pre-collision
 * density, force-corrected velocity and total force */
void  lbo_get_moments(const lbo* o, double* rho, double* u, double* force);
void  lbo_get_avg(const lbo* o, double* avg3);
void  lbo_get_marker(const lbo* o, double* u2n, double* rho_n, double* force2n);
/* FP64 sums of rho, rho*ux, rho*uy over the last step's moment fields */
void  lbo_get_sums(const lbo* o, double* sums3);

#ifdef __cplusplus
}
#endif
#endif
