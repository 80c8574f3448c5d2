/*
 * lbmx.h -- C-ABI of the GB300 D2Q9 lattice Boltzmann engine (liblbmx.so).
 *
 * Plain C types only: a caller-owned opaque handle, plain pointers and sizes,
 * integer status codes.  No call exits the process or resets the device
 * (the reference's checkCudaErrors does both, src/util/utility.cu:4-12).
 *
 * Every pointer argument that carries a field may point to host memory
 * (pageable or pinned) or to device memory of the handle's GPU; the engine
 * copies with cudaMemcpyDefault.  Field layouts match the reference's
 * shipped SoA form (src/core/lbm_constants.cuh:317-327): node = y*nx + x,
 * vector fields as component planes (all x components, then all y).
 *
 * Each entry point names the reference interface it replaces.
 */
#ifndef LBMX_H
#define LBMX_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define LBMX_VERSION 1

typedef int32_t lbmx_status;
enum {
    LBMX_OK = 0,
    LBMX_ERR_INVALID_ARGUMENT = 1,
    LBMX_ERR_OUT_OF_MEMORY = 2,
    LBMX_ERR_CUDA = 3,
    LBMX_ERR_INVALID_FLAGS = 4,   /* a flag the engine cannot apply (see lbmx_set_flags) */
    LBMX_ERR_NOT_INITIALIZED = 5, /* lbmx_step before lbmx_init_from_fields */
    LBMX_ERR_UNSUPPORTED = 6,
    LBMX_ERR_NONFINITE = 7,       /* LBMX_STEP_CHECK_FINITE found NaN/Inf density */
    LBMX_ERR_TOO_LARGE = 8
};

/* Collision operators: BGK<2>, MRT<2>, CM<2,NoAdapter>, CM<2,OptimalAdapter>
 * (src/core/collision/BGK/BGK.cuh:13-51, MRT/MRT.cu:26-76, CM/CM.cuh:27-138,
 *  adapters.cuh:16-22 and :48-111). */
enum { LBMX_BGK = 0, LBMX_MRT = 1, LBMX_CM = 2, LBMX_CM_OPT = 3 };

/* Population storage in HBM.  Offset forms store f_q - w_q in 16 bits; all
 * arithmetic is FP32 in every form. */
enum { LBMX_STORAGE_F32 = 0, LBMX_STORAGE_F16_OFFSET = 1, LBMX_STORAGE_BF16_OFFSET = 2 };

/* Boundary flags.  0..12 keep the values of the reference's BC_flag
 * (src/core/lbm_constants.cuh:376-396); 32..35 are boundaries the reference
 * does not have; 36..37 are reference functors that its 2-D boundary kernel
 * never dispatches (no BC_flag selects them). */
enum {
    LBMX_FLUID = 0,
    LBMX_BOUNCE_BACK = 1,            /* BounceBack<2>, bbDomainBoundary.cuh:14-50 */
    LBMX_ZOU_HE_TOP = 2,             /* ZouHe::apply_top, zouHeInflow.cuh:42-56 */
    LBMX_ZOU_HE_LEFT = 3,            /* ZouHe::apply_left, zouHeInflow.cuh:9-22 */
    LBMX_ZOU_HE_TOP_LEFT_TOP_INFLOW = 4,  /* not implemented by the reference (asserts): rejected */
    LBMX_ZOU_HE_TOP_RIGHT_TOP_INFLOW = 5, /* not implemented by the reference (asserts): rejected */
    LBMX_CYLINDER = 6,               /* CylinderBoundary, cylinderBoundary.cuh:21-34 */
    LBMX_ZG_OUTFLOW = 7,             /* ZG_OutflowBoundary<2>, zeroGradientOutflow.cuh:6-60 */
    LBMX_PRESSURE_OUTLET = 8,        /* PressureOutlet, pressureOutlet.cuh:6-43 */
    LBMX_REGULARIZED_INLET_TOP = 9,  /* RegularizedInlet::apply_top, regularizedInlet.cuh:13-70 */
    LBMX_REGULARIZED_INLET_LEFT = 10,/* no 2-D dispatch in the reference: left untouched */
    LBMX_REGULARIZED_BOUNCE_BACK = 11,        /* regularizedBounceBack.cuh:6-100 */
    LBMX_REGULARIZED_BOUNCE_BACK_CORNER = 12, /* regularizedBounceBack.cuh:102-222 */
    LBMX_MOVING_WALL_BB = 32,        /* half-way bounce-back with wall velocity (wall_ux, wall_uy) */
    LBMX_ZOU_HE_PRESSURE_RIGHT = 33, /* Zou-He pressure outlet at x = nx-1, density rho_out */
    LBMX_ZOU_HE_PARABOLIC_LEFT = 34, /* Zou-He velocity inlet at x = 0, parabolic profile of peak u_bc */
    LBMX_HALFWAY_BB = 35,            /* stationary half-way bounce-back */
    LBMX_CORNER_TOP_LEFT = 36,       /* CornerBoundary::apply_top_left, cornerBoundaries.cuh:39-59 (ux = 0.03) */
    LBMX_CORNER_BOTTOM_LEFT = 37     /* CornerBoundary::apply_bottom_left, cornerBoundaries.cuh:61-81 (ux = 0.03) */
};

/* Switches that reproduce the reference's as-shipped behaviour. */
enum {
    LBMX_QUIRK_REST_LAG = 1u << 0,   /* q=0 is never streamed (streaming.cu:9): f0 two steps back */
    LBMX_QUIRK_ZOUHE_LEFT = 1u << 1, /* rho of the left Zou-He inlet uses f2 for f3 (zouHeInflow.cuh:15-16) */
    LBMX_QUIRK_MRT_FORCE = 1u << 2,  /* MRT forcing moments in [jx,jy,qx,qy] order (MRT.cu:18-19) */
    LBMX_QUIRK_IBM_2X2 = 1u << 3,    /* 2x2 stencil for the 4-point kernel (IBM_impl.cu:19-20) */
    LBMX_QUIRK_IBM_CLAMP = 1u << 4,  /* drop negative IBM forces/velocities (IBM_impl.cuh:22-24, 42-44) */
    LBMX_QUIRKS_REFERENCE = 0x1fu
};

/* lbmx_params.options */
enum {
    LBMX_OPTION_LAGGED_AVERAGES = 1u << 0, /* CM_OPT: use the previous step's grid averages (one pass) */
    LBMX_OPTION_ROUND_NEAREST = 1u << 1    /* 16-bit storage rounds to nearest instead of stochastically */
};

/* lbmx_step_ex flags */
enum {
    LBMX_STEP_STORE_MOMENTS = 1u << 0, /* last step stores rho, u and the FP64 sums */
    LBMX_STEP_CHECK_FINITE = 1u << 1,  /* last step flags non-finite densities */
    LBMX_STEP_SUMS = 1u << 2,          /* every step reduces the FP64 sums (no fields stored) */
    LBMX_STEP_KINETIC_ENERGY = 1u << 3 /* the steps that reduce the sums also reduce the kinetic energy */
};

/* Replaces the compile-time NX/NY/PERIODIC_* macros and the Scenario
 * constexprs (viscosity/tau/omega, S[], u_max) the reference bakes in
 * (src/defines.hpp:4-70, src/scenarios/scenario.cuh:36-59). */
typedef struct lbmx_params {
    int32_t nx, ny;
    int32_t periodic_x, periodic_y;
    int32_t op;          /* LBMX_BGK ... LBMX_CM_OPT */
    int32_t storage;     /* LBMX_STORAGE_* */
    uint32_t quirks;     /* LBMX_QUIRK_* */
    uint32_t options;    /* LBMX_OPTION_* */
    int32_t ibm_iters;   /* multi-direct iterations (reference ITER_MAX = 3) */
    int32_t device;      /* CUDA device ordinal */
    float omega;         /* BGK rate (Scenario::omega) */
    float S[9];          /* MRT (M-row order) or CM (central-moment order) rates (Scenario::S) */
    float u_bc;          /* Scenario::u_max for Zou-He / regularized / parabolic inlets */
    float wall_ux, wall_uy; /* LBMX_MOVING_WALL_BB velocity */
    float rho_out;       /* LBMX_ZOU_HE_PRESSURE_RIGHT density */
    float ibm_ds;        /* marker weight on spread forces (reference: 1) */
    float body_fx, body_fy; /* uniform body force when no force field is given */
    void* stream;        /* cudaStream_t to run on; NULL: the handle creates one */
} lbmx_params;

typedef struct lbmx_handle lbmx_handle;

/* Library version (LBMX_VERSION). */
int32_t lbmx_version(void);

/* Defaults: BGK, omega 1, FP32, no quirks, 3 IBM iterations, rho_out 1. */
void lbmx_params_default(lbmx_params* p);

/* Replaces LBM<2>::allocate<S>() + send_consts<S>() (src/core/lbm.cuh:92-125, :63-82). */
lbmx_status lbmx_create(const lbmx_params* p, lbmx_handle** out);

/* Replaces ~LBM() / LBM::free() (src/core/lbm.cuh:127-140, :379-381). */
void lbmx_destroy(lbmx_handle* h);

/* Replaces LBM::setup_boundary_flags (src/core/boundaries/boundaries.cuh:170-197):
 * nx*ny bytes of BC_flag values evaluated by the scenario's Boundary functor.
 * Rejected (LBMX_ERR_INVALID_FLAGS): flags 4 and 5 (the reference asserts),
 * values above 35, ZG / pressure / corner flags off the domain edge, and a
 * pressure outlet at x = 0 (it reads node x-1). */
lbmx_status lbmx_set_flags(lbmx_handle* h, const uint8_t* flags);

/* Replaces init_kernel / LBM::init<S> (src/core/init/init.cuh:10-86): rho[n],
 * u[2n] and the Init functor's force[2n] (NULL: the uniform body force of
 * the params).  Populations start at the second-order equilibrium. */
lbmx_status lbmx_init_from_fields(lbmx_handle* h, const float* rho, const float* u, const float* force);

/* Replaces reset_forces_kernel / Init::apply_forces (macroscopics.cuh:13-48):
 * the per-node force re-applied every step; NULL returns to the uniform
 * body force of the params. */
lbmx_status lbmx_set_force_field(lbmx_handle* h, const float* force);

/* Replaces one pass of the reference loop body (src/main.cu:96-114):
 * stream, boundaries, macroscopics, IBM, force correction, averages,
 * equilibrium and collision, fused.  Stores moments on the last step. */
lbmx_status lbmx_step(lbmx_handle* h, int32_t nsteps);
lbmx_status lbmx_step_ex(lbmx_handle* h, int32_t nsteps, uint32_t flags);

/* No counterpart in the reference.  Per-node Brinkman solid fraction
 * gamma[n] (NULL: none): a Darcy drag F_B = -gamma rho u acts with the body
 * force (Guo & Zhao 2002), u = (j + F/2) / (rho (1 + gamma/2)); gamma = 0 is
 * open fluid, gamma = 1 damps the velocity by a third each step. */
lbmx_status lbmx_set_brinkman(lbmx_handle* h, const float* gamma);

/* Replaces LBM::update_macroscopics (src/core/lbm.cuh:148-154): the last
 * stored step's density rho[n] and force-corrected velocity u[2n] (the
 * reference's d_rho / d_u), and FP64 sums {rho, rho*ux, rho*uy}.  Any output
 * pointer may be NULL. */
lbmx_status lbmx_moments(lbmx_handle* h, float* rho, float* u, double* sums3);

/* The FP64 sums {rho, rho*ux, rho*uy} of the last stored step, copied into
 * sums3 (pinned host or device memory) on the handle's stream without
 * waiting: they are valid once the stream has reached that point
 * (lbmx_synchronize, or an event).  The reference reads its sums back with a
 * blocking copy every step (macroscopics.cuh:177); a loop that reads the
 * sums of every step this way keeps the GPU busy instead. */
lbmx_status lbmx_moment_sums_async(lbmx_handle* h, double* sums3);

/* nsteps steps (flags as lbmx_step_ex) that also reduce the FP64 sums of
 * every step into series[3 * k .. 3 * k + 2] for step k (pinned host or
 * device memory), copied without waiting; the series is complete once the
 * stream has reached the end (lbmx_synchronize).  With
 * LBMX_STEP_KINETIC_ENERGY a step's entry is four wide,
 * series[4 * k .. 4 * k + 3] = {rho, rho*ux, rho*uy, kinetic energy}. */
lbmx_status lbmx_step_sums(lbmx_handle* h, int32_t nsteps, uint32_t flags, double* series);

/* nsteps steps (flags as lbmx_step_ex) of a lattice with IBM markers that
 * also record every step's drag and lift -- minus the marker forces summed
 * over the markers in FP64, in marker order, as lbmx_ibm_forces returns them
 * -- into series[2 * k], series[2 * k + 1] for step k.  The IBM kernel writes
 * them itself when series is device, managed or pinned host memory (the
 * series is complete once the stream has reached the end); pageable host
 * memory gets a copy per step.  The reference has no drag or lift; its
 * marker forces stay on the device (IBMManager.cuh:222-252). */
lbmx_status lbmx_step_forces(lbmx_handle* h, int32_t nsteps, uint32_t flags, double* series);

/* The kinetic energy 1/2 sum rho |u|^2 (force-corrected u, the velocity
 * lbmx_moments returns) of the last step that reduced the FP64 sums with
 * LBMX_STEP_KINETIC_ENERGY set; 0 when that step's flags did not include it.
 * Blocks until the stream has reached that step.  Replaces the reference's
 * separate reduction pass over the stored fields, calculate_kinetic_energy /
 * compute_kinetic_energy_kernel
 * (src/scenarios/taylorGreen3D/postprocessing/kineticEnergy.cuh:7-40, there
 * in 3-D with FP32 atomics); here it is fused into the step kernel in exact
 * 64-bit fixed point, so it is the same bit for bit on every run. */
lbmx_status lbmx_kinetic_energy(lbmx_handle* h, double* ke);

/* Post-collision populations of the last step, out[9*n], population planes
 * in the reference's velocity order.  Slots whose value streamed out of a
 * non-periodic domain in the last step hold NaN. */
lbmx_status lbmx_get_populations(lbmx_handle* h, float* out);

/* The grid averages {<rho>, <rho|u|>, <|Pi|>} of the last step (the
 * reference's d_moment_avg, src/core/lbm.cu:19); computed for CM_OPT only. */
lbmx_status lbmx_averages(lbmx_handle* h, float* avg3);

/* --- y-slab decomposition.  No counterpart in the reference, which runs one
 * lattice on one device (src/main.cu:39-41).  A lattice of NY rows is split
 * into slabs of whole rows, one handle each, whose lattice adds a ghost row
 * on each side that has a neighbouring slab: a copy of that neighbour's
 * boundary row.  Ghost rows are never stepped.  In a neighbour-access step
 * (odd step index) a boundary row reads three populations from its ghost row
 * and writes three into it, so each slab, around that step:
 *   before: fills its lower ghost row's planes 4, 7, 8 and its upper ghost
 *           row's planes 2, 5, 6 from the neighbours' boundary rows;
 *   after:  returns its lower ghost row's planes 4, 7, 8 and its upper ghost
 *           row's planes 2, 5, 6 into the neighbours' boundary rows.
 * An own-node step (even index) exchanges nothing.  With CM_OPT the slabs'
 * integer average sums (lbmx_opt_partials) are added over all slabs and the
 * averages set on each (lbmx_set_averages) before every step, so a split
 * lattice steps bit for bit as the whole one, 16-bit storage included.
 * cuda-lbm_gb300/lbmx_slabs.py drives this protocol. */

/* Makes the handle a y-slab: row 0 (ghost_mask bit 0) and row ny-1 (bit 1)
 * are ghost rows, and handle row 0 stands for row row_origin of the whole
 * lattice (the stochastic-rounding hash uses whole-lattice node offsets, so
 * 16-bit storage rounds as in the whole lattice).  whole_ny: the whole
 * lattice's row count when it is periodic in y, else 0 -- its first and last
 * rows then take the general path in neighbour-access steps, as they do in
 * the whole lattice.  The slab's own lattice must not be periodic in y (the
 * ghost rows carry the wrap) and carries no IBM markers. */
lbmx_status lbmx_set_slab(lbmx_handle* h, uint32_t ghost_mask, int64_t row_origin, int32_t whole_ny);

/* Copy the stored slots of row `row`, population planes in plane_mask
 * (ascending q), nx stored elements each (4 bytes for FP32 storage, 2 for
 * the 16-bit offset forms), out to buf / in from buf, on the handle's stream:
 * device, managed or pinned buf is stream-ordered; pageable host memory is
 * copied before the call returns.  A put writes only the slots that a node of
 * the neighbouring row writes in a neighbour-access step: on a lattice not
 * periodic in x it leaves slot q of the column whose upstream column x - c_q
 * lies outside the lattice (a half-way wall node reflects into that slot
 * itself). */
lbmx_status lbmx_halo_get(lbmx_handle* h, int32_t row, uint32_t plane_mask, void* buf);
lbmx_status lbmx_halo_put(lbmx_handle* h, int32_t row, uint32_t plane_mask, const void* buf);

/* CM_OPT: the integer fixed-point sums (units of 2^-30) of rho, rho|u| and
 * |Pi| over the stepped nodes for the next step, the terms of its grid
 * averages (update_avg_mag, macroscopics.cuh:50-120).  Adding the sums of
 * all slabs gives exactly the whole lattice's. */
lbmx_status lbmx_opt_partials(lbmx_handle* h, int64_t* sums3);

/* CM_OPT: the next step uses these averages {<rho>, <rho|u|>, <|Pi|>}
 * instead of computing its own.  The whole lattice's are
 * (float)((double)sum * 2^-30 / (double)nodes) of the summed partials. */
lbmx_status lbmx_set_averages(lbmx_handle* h, const float* avg3);

/* Replaces IBMManager<2>::init_and_dispatch (src/IBM/IBMManager.cuh:54-109):
 * n static markers, xy[2n] interleaved (the reference's IBMBody.points). */
lbmx_status lbmx_ibm_set_markers(lbmx_handle* h, const float* xy, int32_t n);

/* Marker forces of the last step, summed over the multi-direct iterations,
 * force[2n] as planes, and drag/lift = -sum of marker forces (FP64). */
lbmx_status lbmx_ibm_forces(lbmx_handle* h, float* force, double* drag_lift);

/* Steps taken since lbmx_init_from_fields. */
int64_t lbmx_time(lbmx_handle* h);

/* No counterpart in the reference (it writes output only, never state).
 * Save the dynamic state -- populations in storage form, the edge store, the
 * step count and the CM_OPT averages -- with a CRC-32; loading it into a
 * handle created with the same params (and given the same flags, force and
 * markers) continues bit for bit.  A file for another lattice, storage,
 * operator or quirk set, or one that fails its CRC, is rejected with
 * LBMX_ERR_INVALID_ARGUMENT. */
lbmx_status lbmx_checkpoint_save(lbmx_handle* h, const char* path);
lbmx_status lbmx_checkpoint_load(lbmx_handle* h, const char* path);

/* Replaces LBM::save_vtk (src/core/lbm.cuh:269-343): ImageData .vti with
 * appended raw Float32 density and 3-component velocity (z = 0) of the last
 * stored step.  The velocity array's offset counts the 8-byte length header
 * of the density array, as the VTK appended format defines it (the
 * reference's offset omits it). */
lbmx_status lbmx_write_vti(lbmx_handle* h, const char* path);

/* Waits for the handle's stream. */
lbmx_status lbmx_synchronize(lbmx_handle* h);

/* Message of the last failed call on this handle ("" if none); with a NULL
 * handle, the message of the last failed lbmx_create. */
const char* lbmx_last_error(lbmx_handle* h);

/* No counterpart in the reference.  FP64 sums {rho, rho*ux, rho*uy} over n
 * nodes of caller-owned device fields rho[n] and u[2n] (x plane, then y
 * plane) into sums3 (host or device memory), on `stream` (a cudaStream_t;
 * NULL = legacy default stream).  When sums3 is pageable host memory the call
 * returns after the sums have arrived.  Otherwise (device, managed or
 * page-locked host memory) the host is not blocked: the sums are there once
 * `stream` has reached this call's work.
 *
 * For callers that may not allocate device memory where they need the sums:
 * between steps of a loop that must not stall the GPU (cudaMalloc and
 * cudaFree synchronise the device), inside a framework whose device memory
 * all belongs to its own pool, or under a hard memory cap.  It calls no
 * cudaMalloc, cudaFree or other allocating routine: its scratch is a fixed
 * 24,608-byte array in the library's device image, which every GPU that
 * loads the library keeps until the process exits.
 *
 * n above LBMX_NOALLOC_MAX_NODES returns LBMX_ERR_TOO_LARGE.  The first call
 * on a device looks up the array's device address (cudaGetSymbolAddress), so
 * make that first call before any stream capture.  That address is kept for
 * the device's primary context: do not call this after cudaDeviceReset or
 * with another driver context current on the device.  All calls on a device
 * share the array: calls whose work can overlap on the GPU (different
 * streams with no ordering between them) race and must not be made. */
#define LBMX_NOALLOC_MAX_NODES 2147483647LL
lbmx_status lbmx_moment_sums_noalloc(const float* rho, const float* u, int64_t n, double* sums3, void* stream);

/* ------------------------------------------------------------------ adjoint
 * No counterpart in the reference.  Gradients of an objective of the step's
 * moments,
 *     J = sum over steps t >= first_step and nodes x of
 *         w_rho(x) rho_t(x) + w_x(x) rho_t u_x,t(x) + w_y(x) rho_t u_y,t(x),
 * with respect to the per-node Brinkman field gamma, the relaxation rate
 * omega (with every S entry equal to omega at creation) and the uniform body
 * force, by a discrete adjoint of the step: forward-mode tangents through the
 * per-node boundary / Brinkman / collision code give each node's Jacobian
 * exactly, and the populations are recomputed from checkpoints taken every
 * `checkpoint_every` steps, so memory is (steps / every + every) states.
 * FP32 populations; any operator; fluid, bounce-back (where it reads no
 * population from outside the domain) and half-way / moving walls; no IBM. */
typedef struct lbmx_adjoint lbmx_adjoint;

lbmx_status lbmx_adjoint_create(const lbmx_params* p, const uint8_t* flags, int32_t checkpoint_every,
                                lbmx_adjoint** out);
void lbmx_adjoint_destroy(lbmx_adjoint* a);
/* initial rho[n], u[2n] (populations start at equilibrium, as lbmx_init_from_fields) */
lbmx_status lbmx_adjoint_set_state(lbmx_adjoint* a, const float* rho, const float* u);
lbmx_status lbmx_adjoint_set_gamma(lbmx_adjoint* a, const float* gamma);
lbmx_status lbmx_adjoint_set_scalars(lbmx_adjoint* a, float omega, float body_fx, float body_fy);
/* weights[3n]: w_rho, w_x, w_y planes */
lbmx_status lbmx_adjoint_set_objective(lbmx_adjoint* a, const float* weights, int32_t first_step);
/* Objective kinds of lbmx_adjoint_set_objective_ex. */
enum { LBMX_OBJECTIVE_MOMENTS = 0, LBMX_OBJECTIVE_BRINKMAN_DRAG = 1 };
/* As lbmx_adjoint_set_objective; with LBMX_OBJECTIVE_BRINKMAN_DRAG each
 * node's term is multiplied by its Brinkman fraction:
 * J = sum over t >= first, x of gamma (w_rho rho + w_x rho u_x + w_y rho u_y),
 * so w_x = 1 gives the x drag the fluid exerts on the porous solid,
 * sum gamma rho u_x (the Darcy force is -gamma rho u on the fluid).  Its
 * gamma gradient includes the explicit term. */
lbmx_status lbmx_adjoint_set_objective_ex(lbmx_adjoint* a, const float* weights, int32_t first_step, int32_t kind);
/* nsteps steps from the initial state; J into *objective */
lbmx_status lbmx_adjoint_forward(lbmx_adjoint* a, int32_t nsteps, double* objective);
/* dJ/dgamma[n] (may be NULL) and {dJ/domega, dJ/dFx, dJ/dFy} of the last forward run */
lbmx_status lbmx_adjoint_backward(lbmx_adjoint* a, float* grad_gamma, double* grad_scalars);
/* rho[n], u[2n] of the last forward step */
lbmx_status lbmx_adjoint_moments(lbmx_adjoint* a, float* rho, float* u);
const char* lbmx_adjoint_last_error(lbmx_adjoint* a);

/* ------------------------------------------------------------------ tangent
 * No counterpart in the reference.  The tangent-linear (forward-mode)
 * derivative of a run with respect to one scalar parameter: every value of
 * the step carries its derivative through the same per-node boundary,
 * collision and IBM code as the engine.  For one input this is the exact
 * derivative of the discrete model that an adjoint would give, for every
 * output at once -- the drag and lift of every step, the final moments --
 * at the cost of one forward run and with no checkpoints.
 * FP32 populations; BGK, MRT or CM; fluid, bounce-back, cylinder, Zou-He
 * (top, left, parabolic left, pressure right) and half-way / moving walls;
 * IBM markers; every quirk. */
typedef struct lbmx_tangent lbmx_tangent;

enum {
    LBMX_TANGENT_U_BC = 0,    /* params.u_bc: Zou-He inlet velocity / parabolic peak */
    LBMX_TANGENT_OMEGA = 1,   /* params.omega, with the S entries equal to it */
    LBMX_TANGENT_BODY_FX = 2, /* params.body_fx */
    LBMX_TANGENT_WALL_UX = 3  /* params.wall_ux of LBMX_MOVING_WALL_BB */
};

lbmx_status lbmx_tangent_create(const lbmx_params* p, const uint8_t* flags, int32_t parameter, lbmx_tangent** out);
void lbmx_tangent_destroy(lbmx_tangent* t);
/* initial rho[n], u[2n] (equilibrium populations, as lbmx_init_from_fields;
 * the initial state does not depend on the parameter) */
lbmx_status lbmx_tangent_set_state(lbmx_tangent* t, const float* rho, const float* u);
/* IBM markers, as lbmx_ibm_set_markers */
lbmx_status lbmx_tangent_set_markers(lbmx_tangent* t, const float* xy, int32_t n);
/* nsteps further steps; series (may be NULL) receives per step
 * {drag, lift, d drag / d parameter, d lift / d parameter}, drag and lift as
 * lbmx_ibm_forces gives them */
lbmx_status lbmx_tangent_run(lbmx_tangent* t, int32_t nsteps, double* series);
/* rho[n], u[2n] of the last step and their derivatives drho[n], du[2n]
 * (any may be NULL) */
lbmx_status lbmx_tangent_moments(lbmx_tangent* t, float* rho, float* u, float* drho, float* du);
int64_t lbmx_tangent_time(lbmx_tangent* t);
const char* lbmx_tangent_last_error(lbmx_tangent* t);

/* ------------------------------------------------------------------ batches
 * No counterpart in the reference, which runs one lattice per process
 * (src/main.cu:96-114).  A batch advances many independent lattices -- any
 * sizes, relaxation rates, flags and forces -- in one persistent kernel
 * launch per step, replayed from CUDA graphs.  Every step gives each lattice
 * bit for bit what lbmx_step gives it alone.
 *
 * The lattices are ordinary handles, created, flagged and initialised as
 * usual and still read with lbmx_moments / lbmx_get_populations /
 * lbmx_checkpoint_save.  They must share device, storage and operator (BGK,
 * MRT or CM; not CM_OPT), carry no IBM markers and stand at the same step
 * count; each lattice's stream waits for the batch's steps.  Batched steps
 * leave the FP64 sums of lbmx_moments untouched.  Destroy the batch before
 * its lattices. */
typedef struct lbmx_batch lbmx_batch;

typedef struct lbmx_batch_config {
    int32_t tile_w;       /* interior tile shape tile_w x tile_h: 64 x 8, 128 x 4 or 128 x 8 */
    int32_t tile_h;
    int32_t ctas_per_sm;  /* persistent CTAs per SM: 1, 2 or 3 */
    int32_t chunk;        /* work items claimed per atomic: 1..64 */
    int32_t graph_steps;  /* steps per CUDA graph replay: 0 (no graph) or even, <= 64 */
} lbmx_batch_config;

lbmx_status lbmx_batch_create(lbmx_handle* const* lattices, int32_t count, lbmx_batch** out);
void lbmx_batch_destroy(lbmx_batch* b);
lbmx_status lbmx_batch_set_config(lbmx_batch* b, const lbmx_batch_config* cfg);
lbmx_status lbmx_batch_get_config(lbmx_batch* b, lbmx_batch_config* cfg);
/* Time every configuration for trial_steps steps (after two warm-up steps)
 * and keep the fastest; the lattices are put back as they were. */
lbmx_status lbmx_batch_autotune(lbmx_batch* b, int32_t trial_steps, lbmx_batch_config* chosen);
/* nsteps steps of every lattice; flags as lbmx_step_ex (a non-finite
 * density in any lattice gives LBMX_ERR_NONFINITE). */
lbmx_status lbmx_batch_step(lbmx_batch* b, int32_t nsteps, uint32_t flags);
lbmx_status lbmx_batch_synchronize(lbmx_batch* b);
/* Message of the last failed call on this batch; with NULL, of the last
 * failed lbmx_batch_create. */
const char* lbmx_batch_last_error(lbmx_batch* b);

#ifdef __cplusplus
}
#endif
#endif /* LBMX_H */
