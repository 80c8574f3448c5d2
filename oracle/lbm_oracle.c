/*
 * lbm_oracle.c -- CPU restatement of the reference D2Q9 step (test infrastructure).
 *
 * TEST INFRASTRUCTURE ONLY: the checker for the CUDA engine, never part of
 * the product path.  See lbm_oracle.h for the map onto the reference files.
 *
 * Compile with -DORACLE_REAL=float for the FP32 variant.  In the float
 * variant the second-order equilibrium is still evaluated in double, as the
 * reference's equilibrium_node does through pow() and double literals
 * (src/core/equilibrium/equilibrium.cu:13-38).
 */
#include "lbm_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#ifndef ORACLE_REAL
#define ORACLE_REAL double
#endif
typedef ORACLE_REAL real;

/* D2Q9 velocity set in the reference's order: rest, E, N, W, S, NE, NW, SW, SE
 * (src/core/lbm_constants.cuh:19-31). */
static const int CX[9] = {0, 1, 0, -1, 0, 1, -1, -1, 1};
static const int CY[9] = {0, 0, 1, 0, -1, 1, 1, -1, -1};
static const int OPP[9] = {0, 3, 4, 1, 2, 7, 8, 5, 6};
static real W[9];

/* Lallemand-Luo moment basis rows [rho, e, eps, jx, qx, jy, qy, pxx, pxy]
 * (src/core/lbm_constants.cuh:33-43).  The rows are mutually orthogonal, so the
 * inverse is M^T diag(1/|row|^2); it is formed that way in init_tables(). */
static const int MM[9][9] = {
    { 1,  1,  1,  1,  1,  1,  1,  1,  1},
    {-4, -1, -1, -1, -1,  2,  2,  2,  2},
    { 4, -2, -2, -2, -2,  1,  1,  1,  1},
    { 0,  1,  0, -1,  0,  1, -1, -1,  1},
    { 0, -2,  0,  2,  0,  1, -1, -1,  1},
    { 0,  0,  1,  0, -1,  1,  1, -1, -1},
    { 0,  0, -2,  0,  2,  1,  1, -1, -1},
    { 0,  1, -1,  1, -1,  0,  0,  0,  0},
    { 0,  0,  0,  0,  0,  1, -1,  1, -1}};
static real MINV[9][9];

static void init_tables(void) {
    static int done = 0;
    if (done) return;
    W[0] = (real)(4.0 / 9.0);
    for (int q = 1; q <= 4; q++) W[q] = (real)(1.0 / 9.0);
    for (int q = 5; q <= 8; q++) W[q] = (real)(1.0 / 36.0);
    for (int k = 0; k < 9; k++) {
        int nrm = 0;
        for (int i = 0; i < 9; i++) nrm += MM[k][i] * MM[k][i];
        for (int i = 0; i < 9; i++) MINV[i][k] = (real)((double)MM[k][i] / (double)nrm);
    }
    done = 1;
}

struct lbo {
    lbo_params p;
    int nx, ny;
    long n;
    real *f, *fb;        /* [9][n] current / back buffer (ping-pong, src/core/lbm.cuh:36-37) */
    real *feq;           /* [9][n] */
    real *rho, *ux, *uy, *pimag;
    real *fx, *fy;       /* LBM force */
    real *bfx, *bfy;     /* body force from Init::apply_forces */
    real *gamma;         /* Brinkman solid fraction, NULL: none (no reference counterpart) */
    real *aux;           /* [9][n] neighbour data for ZG / pressure / corner boundaries */
    uint8_t *flags;
    int has_aux_bc;
    /* immersed boundary */
    int nm;
    real *mx, *my, *mux, *muy, *mrho, *mfx, *mfy, *mftx, *mfty;
    real *upx, *upy, *fix, *fiy;
    real avg[3];
    double sums[3];
    long t;
};

static void* xcalloc(size_t n, size_t s) { return calloc(n ? n : 1, s); }

lbo* lbo_create(const lbo_params* p) {
    init_tables();
    if (!p || p->nx < 3 || p->ny < 3) return NULL;
    lbo* o = (lbo*)xcalloc(1, sizeof(lbo));
    o->p = *p;
    if (o->p.ibm_iters <= 0) o->p.ibm_iters = 3;
    if (o->p.ibm_ds == 0.0) o->p.ibm_ds = 1.0;
    o->nx = p->nx; o->ny = p->ny; o->n = (long)p->nx * p->ny;
    long n = o->n;
    o->f = (real*)xcalloc(9 * n, sizeof(real));
    o->fb = (real*)xcalloc(9 * n, sizeof(real));
    o->feq = (real*)xcalloc(9 * n, sizeof(real));
    o->aux = (real*)xcalloc(9 * n, sizeof(real));
    o->rho = (real*)xcalloc(n, sizeof(real));
    o->ux = (real*)xcalloc(n, sizeof(real));
    o->uy = (real*)xcalloc(n, sizeof(real));
    o->pimag = (real*)xcalloc(n, sizeof(real));
    o->fx = (real*)xcalloc(n, sizeof(real));
    o->fy = (real*)xcalloc(n, sizeof(real));
    o->bfx = (real*)xcalloc(n, sizeof(real));
    o->bfy = (real*)xcalloc(n, sizeof(real));
    o->flags = (uint8_t*)xcalloc(n, 1);
    return o;
}

static void free_markers(lbo* o) {
    free(o->mx); free(o->my); free(o->mux); free(o->muy); free(o->mrho);
    free(o->mfx); free(o->mfy); free(o->mftx); free(o->mfty);
    free(o->upx); free(o->upy); free(o->fix); free(o->fiy);
    o->mx = o->my = o->mux = o->muy = o->mrho = o->mfx = o->mfy = o->mftx = o->mfty = NULL;
    o->upx = o->upy = o->fix = o->fiy = NULL;
    o->nm = 0;
}

void lbo_destroy(lbo* o) {
    if (!o) return;
    free(o->f); free(o->fb); free(o->feq); free(o->aux);
    free(o->rho); free(o->ux); free(o->uy); free(o->pimag);
    free(o->fx); free(o->fy); free(o->bfx); free(o->bfy); free(o->flags); free(o->gamma);
    free_markers(o);
    free(o);
}

int lbo_set_flags(lbo* o, const uint8_t* flags) {
    memcpy(o->flags, flags, (size_t)o->n);
    o->has_aux_bc = 0;
    for (long i = 0; i < o->n; i++) {
        uint8_t fl = flags[i];
        if (fl == LBO_ZG_OUTFLOW || fl == LBO_PRESSURE_OUTLET || fl == LBO_REGULARIZED_BOUNCE_BACK_CORNER)
            o->has_aux_bc = 1;
    }
    return 0;
}

/* Second-order equilibrium as the reference evaluates it: a float weight times
 * a float density, times a bracket computed in double (equilibrium.cu:13-38). */
static inline real feq_ref(int q, real rho, real ux, real uy) {
    const float cs = 1.0f / sqrtf(3.0f);
    const float cs2 = cs * cs;
    const float cs4 = cs2 * cs2;
    real cu = (real)CX[q] * ux + (real)CY[q] * uy;
    real uu = ux * ux + uy * uy;
    real wr = W[q] * rho;
    double br = 1.0 + 0.5 * (double)cu * (double)cu / (double)cs4 - 0.5 * (double)uu / (double)cs2
              + 1.0 * (double)cu / (double)cs2;
    if (sizeof(real) == sizeof(double)) /* exact-arithmetic form for the FP64 oracle */
        br = 1.0 + 4.5 * (double)cu * (double)cu - 1.5 * (double)uu + 3.0 * (double)cu;
    return (real)((double)wr * br);
}

/* equilibrium used inside the boundary functors: all-float form
 * w*rho*(1 + cu/cs2 + cu^2/(2cs2^2) - u^2/(2cs2)) (pressureOutlet.cuh:30-40,
 * regularizedInlet.cuh:26-31, regularizedBounceBack.cuh:52-57) */
static inline real feq_bc(int q, real rho, real ux, real uy) {
    const real cs2 = (real)1 / (real)3;
    real cu = (real)CX[q] * ux + (real)CY[q] * uy;
    real uu = ux * ux + uy * uy;
    return W[q] * rho * ((real)1 + cu / cs2 + cu * cu / ((real)2 * cs2 * cs2) - uu / ((real)2 * cs2));
}

/* ---------------------------------------------------------------- boundaries */

/* BounceBack<2>::apply with (true,true): outward-neighbour test on geometry,
 * sequential over i (bbDomainBoundary.cuh:26-49). */
static void bc_bounce_back(const lbo* o, real* f, int x, int y) {
    for (int i = 1; i < 9; i++) {
        int xn = x + CX[i], yn = y + CY[i];
        if (xn < 0 || xn >= o->nx || yn < 0 || yn >= o->ny) f[OPP[i]] = f[i];
    }
}

/* Half-way bounce-back, moving (LBO_MOVING_WALL_BB, wall velocity) or
 * stationary (LBO_HALFWAY_BB); no reference counterpart.  Applied during the
 * push: a population whose downstream node lies outside a non-periodic
 * domain returns to its own node reversed, with Ladd's momentum term
 * -2 w_i rho_w (c_i . u_w) / cs^2 (rho_w = 1).  The wall sits half a link
 * outside the flagged node; mass is conserved exactly. */
static inline real halfway_term(const lbo* o, int i, uint8_t fl) {
    if (fl != LBO_MOVING_WALL_BB) return 0;
    real cu = (real)CX[i] * (real)o->p.wall_ux + (real)CY[i] * (real)o->p.wall_uy;
    return (real)6 * W[i] * cu;
}

/* ZouHe::apply_top (zouHeInflow.cuh:42-56) */
static void bc_zouhe_top(const lbo* o, real* f) {
    const real ux = (real)o->p.u_bc, uy = 0;
    real rho = (f[0] + f[1] + f[3] + (real)2 * (f[2] + f[5] + f[6])) / ((real)1 + uy);
    f[4] = f[2] - ((real)2 / (real)3) * rho * uy;
    real d = f[1] - f[3];
    f[7] = f[5] + (real)0.5 * d - ((real)1 / (real)2) * rho * ux - ((real)1 / (real)6) * rho * uy;
    f[8] = f[6] - (real)0.5 * d + ((real)1 / (real)2) * rho * ux - ((real)1 / (real)6) * rho * uy;
}

/* ZouHe::apply_left (zouHeInflow.cuh:9-22); `typo` keeps f2 in the doubled term. */
static void bc_zouhe_left(real* f, real ux, int typo) {
    real f_in = typo ? f[2] : f[3];
    real rho = (f[0] + f[2] + f[4] + 2 * (f_in + f[6] + f[7])) / ((real)1 - ux);
    f[1] = f[3] + ((real)2 / (real)3) * rho * ux;
    f[5] = f[7] - (real)0.5 * (f[2] - f[4]) + ((real)1 / (real)6) * rho * ux;
    f[8] = f[6] + (real)0.5 * (f[2] - f[4]) + ((real)1 / (real)6) * rho * ux;
}

/* Zou-He pressure outlet on the right edge (no reference counterpart). */
static void bc_zouhe_pressure_right(const lbo* o, real* f) {
    const real rho = (real)o->p.rho_out;
    real ux = (real)-1 + (f[0] + f[2] + f[4] + (real)2 * (f[1] + f[5] + f[8])) / rho;
    f[3] = f[1] - ((real)2 / (real)3) * rho * ux;
    f[7] = f[5] + (real)0.5 * (f[2] - f[4]) - ((real)1 / (real)6) * rho * ux;
    f[6] = f[8] - (real)0.5 * (f[2] - f[4]) - ((real)1 / (real)6) * rho * ux;
}

/* CylinderBoundary::apply: full reversal (cylinderBoundary.cuh:22-33) */
static void bc_cylinder(real* f) {
    real s[9];
    for (int j = 0; j < 9; j++) s[j] = f[j];
    for (int i = 0; i < 9; i++) f[OPP[i]] = s[i];
}

/* shared tail of the regularized boundaries: Pi(1) from all populations,
 * then f = f_eq + w/(2cs^4) Q:Pi (regularizedInlet.cuh:41-67) */
static void regularize_tail(real* f, const real* fe, real rho, real ux, real uy) {
    const real cs2 = (real)1 / (real)3;
    real pxx = 0, pyy = 0, pxy = 0;
    for (int q = 0; q < 9; q++) {
        real cx = (real)CX[q], cy = (real)CY[q];
        pxx += cx * cx * f[q];
        pyy += cy * cy * f[q];
        pxy += cx * cy * f[q];
    }
    pxx -= cs2 * rho + rho * ux * ux;
    pyy -= cs2 * rho + rho * uy * uy;
    pxy -= rho * ux * uy;
    for (int q = 0; q < 9; q++) {
        real cx = (real)CX[q], cy = (real)CY[q];
        real qxx = cx * cx - cs2, qyy = cy * cy - cs2, qxy = cx * cy;
        real fneq = (W[q] / ((real)2 * cs2 * cs2)) * (qxx * pxx + qyy * pyy + (real)2 * qxy * pxy);
        f[q] = fe[q] + fneq;
    }
}

/* RegularizedInlet::apply_top (regularizedInlet.cuh:14-69) */
static void bc_reg_inlet_top(const lbo* o, real* f) {
    const real ux = (real)o->p.u_bc, uy = 0;
    real rho = (f[0] + f[1] + f[3] + (real)2 * (f[2] + f[5] + f[6])) / ((real)1 + uy);
    real fe[9];
    for (int q = 0; q < 9; q++) fe[q] = feq_bc(q, rho, ux, uy);
    for (int q = 0; q < 9; q++)
        if (CY[q] < 0) f[q] = fe[q] + (f[OPP[q]] - fe[OPP[q]]);
    regularize_tail(f, fe, rho, ux, uy);
}

/* RegularizedBounceBack::apply (regularizedBounceBack.cuh:13-99) */
static void bc_reg_bounce_back(const lbo* o, real* f, int x, int y) {
    int unk[9] = {0};
    for (int i = 1; i < 9; i++) {
        if (x == 0) unk[i] = CX[i] > 0;
        else if (x == o->nx - 1) unk[i] = CX[i] < 0;
        else if (y == 0) unk[i] = CY[i] > 0;
        else if (y == o->ny - 1) unk[i] = CY[i] < 0;
    }
    real rho = 0;
    for (int i = 0; i < 9; i++)
        if (!unk[i]) rho += (real)(unk[OPP[i]] ? 2 : 1) * f[i];
    real fe[9];
    for (int q = 0; q < 9; q++) fe[q] = feq_bc(q, rho, 0, 0);
    for (int q = 0; q < 9; q++)
        if (unk[q]) f[q] = fe[q] + (f[OPP[q]] - fe[OPP[q]]);
    regularize_tail(f, fe, rho, 0, 0);
}

/* RegularizedCornerBounceBack::apply (regularizedBounceBack.cuh:108-221);
 * rho_diag is the diagonal interior node's post-stream density. */
static void bc_reg_corner(const lbo* o, real* f, int x, int y, real rho) {
    int L = x == 0, R = x == o->nx - 1, B = y == 0, T = y == o->ny - 1;
    if (!((L || R) && (B || T))) return;
    int unk[9] = {0};
    for (int i = 1; i < 9; i++)
        unk[i] = (L && CX[i] > 0) || (R && CX[i] < 0) || (B && CY[i] > 0) || (T && CY[i] < 0);
    for (int i = 0; i < 9; i++)
        if (unk[i]) f[i] = feq_bc(i, rho, 0, 0) - (f[OPP[i]] - feq_bc(OPP[i], rho, 0, 0));
    const real cs2 = (real)1 / (real)3;
    real pxx = 0, pyy = 0, pxy = 0;
    for (int q = 0; q < 9; q++) {
        real fneq = f[q] - feq_bc(q, rho, 0, 0);
        real cx = (real)CX[q], cy = (real)CY[q];
        pxx += cx * cx * fneq;
        pyy += cy * cy * fneq;
        pxy += cx * cy * fneq;
    }
    for (int q = 0; q < 9; q++) {
        real cx = (real)CX[q], cy = (real)CY[q];
        real qxx = cx * cx - cs2, qyy = cy * cy - cs2, qxy = cx * cy;
        real fneq = (W[q] / ((real)2 * cs2 * cs2)) * (qxx * pxx + qyy * pyy + (real)2 * qxy * pxy);
        f[q] = feq_bc(q, rho, 0, 0) + fneq;
    }
}

/* neighbour data read by ZG outflow, pressure outlet and regularized corner,
 * taken from the post-stream state before any boundary writes. */
static void bc_aux(lbo* o, int x, int y, real* aux) {
    const int nx = o->nx, ny = o->ny;
    long node = (long)y * nx + x;
    uint8_t fl = o->flags[node];
    const long n = o->n;
    if (fl == LBO_ZG_OUTFLOW) {
        /* zeroGradientOutflow.cuh:13-44: interior node along the first matching edge */
        int ix = x, iy = y;
        if (x == 0) ix = 1;
        else if (x == nx - 1) ix = nx - 2;
        else if (y == 0) iy = 1;
        else if (y == ny - 1) iy = ny - 2;
        else return;
        long in = (long)iy * nx + ix;
        for (int q = 0; q < 9; q++) aux[q] = o->f[q * n + in];
    } else if (fl == LBO_PRESSURE_OUTLET) {
        /* pressureOutlet.cuh:10-27: interior node = node - 1 */
        long in = node - 1;
        real r = 0, ux = 0, uy = 0;
        for (int q = 0; q < 9; q++) r += o->f[q * n + in];
        for (int q = 0; q < 9; q++) {
            ux += o->f[q * n + in] * (real)CX[q];
            uy += o->f[q * n + in] * (real)CY[q];
        }
        aux[0] = r; aux[1] = ux / r; aux[2] = uy / r;
    } else if (fl == LBO_REGULARIZED_BOUNCE_BACK_CORNER) {
        int dx = x == 0 ? x + 1 : x - 1;
        int dy = y == 0 ? y + 1 : y - 1;
        dx = dx < 1 ? 1 : (dx > nx - 2 ? nx - 2 : dx);
        dy = dy < 1 ? 1 : (dy > ny - 2 ? ny - 2 : dy);
        long dn = (long)dy * nx + dx;
        real r = 0;
        for (int q = 0; q < 9; q++) r += o->f[q * n + dn];
        aux[0] = r;
    }
}

/* CornerBoundary::apply_top_left / apply_bottom_left
 * (src/functors/boundaryConditions/cornerBoundaries.cuh:39-59, 61-81): the
 * corners of a left inlet whose velocity is fixed at ux = 0.03, uy = 0; the
 * top-left one sets f2 from f4, the bottom-left one f4 from f2, as there. */
static void bc_corner_top_left(real* f) {
    const real ux = (real)0.03f, uy = 0;
    real rho = (f[0] + f[3] + f[4] + f[6] + f[7]) / ((real)1 - ux - uy);
    f[1] = f[3] + ((real)2 / 3) * rho * ux;
    f[2] = f[4];
    f[5] = f[7] + ((real)1 / 6) * rho * (ux + uy);
    f[8] = f[6] + ((real)1 / 6) * rho * (ux - uy);
}

static void bc_corner_bottom_left(real* f) {
    const real ux = (real)0.03f, uy = 0;
    real rho = (f[0] + f[2] + f[3] + f[5] + f[6]) / ((real)1 - ux + uy);
    f[1] = f[3] + ((real)2 / 3) * rho * ux;
    f[4] = f[2];
    f[5] = f[7] + ((real)1 / 6) * rho * (ux + uy);
    f[8] = f[6] + ((real)1 / 6) * rho * (ux - uy);
}

static void apply_bc(const lbo* o, real* f, int x, int y, uint8_t fl, const real* aux) {
    switch (fl) {
    case LBO_FLUID: break;
    case LBO_BOUNCE_BACK: bc_bounce_back(o, f, x, y); break;
    case LBO_ZOU_HE_TOP: bc_zouhe_top(o, f); break;
    case LBO_ZOU_HE_LEFT:
        bc_zouhe_left(f, (real)o->p.u_bc, (o->p.quirks & LBO_QUIRK_ZOUHE_LEFT) != 0);
        break;
    case LBO_CYLINDER: bc_cylinder(f); break;
    case LBO_ZG_OUTFLOW: {
        int nxv = 0, nyv = 0;
        if (x == 0) nxv = 1;
        else if (x == o->nx - 1) nxv = -1;
        else if (y == 0) nyv = 1;
        else if (y == o->ny - 1) nyv = -1;
        else break;
        for (int i = 0; i < 9; i++)
            if (CX[i] * nxv + CY[i] * nyv > 0) f[i] = aux[i];
        break;
    }
    case LBO_PRESSURE_OUTLET:
        for (int i = 0; i < 9; i++) f[i] = feq_bc(i, (real)1, aux[1], aux[2]);
        break;
    case LBO_REGULARIZED_INLET_TOP: bc_reg_inlet_top(o, f); break;
    case LBO_REGULARIZED_BOUNCE_BACK: bc_reg_bounce_back(o, f, x, y); break;
    case LBO_REGULARIZED_BOUNCE_BACK_CORNER: bc_reg_corner(o, f, x, y, aux[0]); break;
    case LBO_MOVING_WALL_BB: case LBO_HALFWAY_BB: break; /* applied while streaming */
    case LBO_ZOU_HE_PRESSURE_RIGHT: bc_zouhe_pressure_right(o, f); break;
    case LBO_ZOU_HE_PARABOLIC_LEFT: {
        real h = (real)(o->ny - 1);
        real ux = (real)4 * (real)o->p.u_bc * (real)y * (h - (real)y) / (h * h);
        bc_zouhe_left(f, ux, 0);
        break;
    }
    case LBO_CORNER_TOP_LEFT: bc_corner_top_left(f); break;
    case LBO_CORNER_BOTTOM_LEFT: bc_corner_bottom_left(f); break;
    default: break; /* the reference prints "Unknown Flag" and leaves the node alone */
    }
}

/* ---------------------------------------------------------------- IBM */

/* Peskin 4-point kernel, delta4 (src/IBM/IBMUtils.cuh:24-33) */
static inline real delta4(real r) {
    real a = (real)fabs((double)r);
    if (a < (real)1) return (real)0.125 * ((real)3 - (real)2 * a + (real)sqrt((double)((real)1 + (real)4 * a - (real)4 * r * r)));
    if (a < (real)2) return (real)0.125 * ((real)5 - (real)2 * a - (real)sqrt((double)((real)-7 + (real)12 * a - (real)4 * r * r)));
    return 0;
}

static void ibm_multi_direct(lbo* o) {
    const int nx = o->nx, ny = o->ny, nm = o->nm;
    const long n = o->n;
    const int q2 = (o->p.quirks & LBO_QUIRK_IBM_2X2) != 0;
    const int clamp = (o->p.quirks & LBO_QUIRK_IBM_CLAMP) != 0;
    const int lo = q2 ? 0 : -1, hi = q2 ? 1 : 2;
    memcpy(o->upx, o->ux, n * sizeof(real));
    memcpy(o->upy, o->uy, n * sizeof(real));
    for (int k = 0; k < nm; k++) o->mftx[k] = o->mfty[k] = 0;
    for (int it = 0; it < o->p.ibm_iters; it++) {
        memset(o->fix, 0, n * sizeof(real));
        memset(o->fiy, 0, n * sizeof(real));
        /* interpolate_velocities_kernel<2> (IBM_impl.cu:5-51) */
        for (int k = 0; k < nm; k++) {
            real px = o->mx[k], py = o->my[k];
            real gx = (real)floor((double)px), gy = (real)floor((double)py);
            real ux = 0, uy = 0, r = 0;
            for (int i = lo; i <= hi; i++)
                for (int j = lo; j <= hi; j++) {
                    int xn = (int)(gx + (real)i), yn = (int)(gy + (real)j);
                    if (xn >= nx || xn < 0 || yn >= ny || yn < 0) continue;
                    real w = delta4(px - (real)xn) * delta4(py - (real)yn);
                    long nd = (long)yn * nx + xn;
                    r += w * o->rho[nd];
                    ux += w * o->upx[nd];
                    uy += w * o->upy[nd];
                }
            o->mux[k] = ux; o->muy[k] = uy; o->mrho[k] = r;
        }
        /* compute_lagrangian_kernel (IBM_impl.cuh:7-26), target velocity 0 */
        for (int k = 0; k < nm; k++) {
            real fxk = (real)2 * o->mrho[k] * ((real)0 - o->mux[k]);
            real fyk = (real)2 * o->mrho[k] * ((real)0 - o->muy[k]);
            if (clamp) {
                fxk = fxk > (real)1e-8f ? fxk : 0;
                fyk = fyk > (real)1e-8f ? fyk : 0;
            }
            o->mfx[k] = fxk; o->mfy[k] = fyk;
            o->mftx[k] += fxk; o->mfty[k] += fyk;
        }
        /* spread_forces_kernel<2> (IBM_impl.cu:120-154) */
        for (int k = 0; k < nm; k++) {
            real px = o->mx[k], py = o->my[k];
            real gx = (real)floor((double)px), gy = (real)floor((double)py);
            for (int i = lo; i <= hi; i++)
                for (int j = lo; j <= hi; j++) {
                    int xn = (int)(gx + (real)i), yn = (int)(gy + (real)j);
                    if (xn >= nx || xn < 0 || yn >= ny || yn < 0) continue;
                    real w = delta4(px - (gx + (real)i)) * delta4(py - (gy + (real)j)) * (real)o->p.ibm_ds;
                    long nd = (long)yn * nx + xn;
                    o->fix[nd] += w * o->mfx[k];
                    o->fiy[nd] += w * o->mfy[k];
                }
        }
        /* correct_velocities_kernel + accumulate_forces_kernel (IBM_impl.cuh:28-68) */
        for (long nd = 0; nd < n; nd++) {
            real cx = o->upx[nd] + o->fix[nd] / ((real)2 * o->rho[nd]);
            real cy = o->upy[nd] + o->fiy[nd] / ((real)2 * o->rho[nd]);
            if (clamp) {
                cx = (double)cx > 1e-8 ? cx : 0;
                cy = (double)cy > 1e-8 ? cy : 0;
            }
            o->upx[nd] = cx; o->upy[nd] = cy;
            o->fx[nd] += o->fix[nd];
            o->fy[nd] += o->fiy[nd];
        }
    }
}

int lbo_set_markers(lbo* o, const double* xy, int nm) {
    free_markers(o);
    if (nm <= 0) return 0;
    long n = o->n;
    o->nm = nm;
    o->mx = (real*)xcalloc(nm, sizeof(real)); o->my = (real*)xcalloc(nm, sizeof(real));
    o->mux = (real*)xcalloc(nm, sizeof(real)); o->muy = (real*)xcalloc(nm, sizeof(real));
    o->mrho = (real*)xcalloc(nm, sizeof(real));
    o->mfx = (real*)xcalloc(nm, sizeof(real)); o->mfy = (real*)xcalloc(nm, sizeof(real));
    o->mftx = (real*)xcalloc(nm, sizeof(real)); o->mfty = (real*)xcalloc(nm, sizeof(real));
    o->upx = (real*)xcalloc(n, sizeof(real)); o->upy = (real*)xcalloc(n, sizeof(real));
    o->fix = (real*)xcalloc(n, sizeof(real)); o->fiy = (real*)xcalloc(n, sizeof(real));
    for (int k = 0; k < nm; k++) { o->mx[k] = (real)xy[2 * k]; o->my[k] = (real)xy[2 * k + 1]; }
    return 0;
}

/* ---------------------------------------------------------------- collision */

static void collide_bgk(const lbo* o, long nd) {
    const long n = o->n;
    const real om = (real)o->p.omega, cs2 = (real)1 / (real)3;
    real fx = o->fx[nd], fy = o->fy[nd], ux = o->ux[nd], uy = o->uy[nd];
    for (int q = 0; q < 9; q++) {
        real cx = (real)CX[q], cy = (real)CY[q];
        real ft = W[q] * (((real)1 - (real)0.5 * om) * ((cx - ux) / cs2 + (cx * ux + cy * uy) * cx / (cs2 * cs2)) * fx
                        + ((real)1 - (real)0.5 * om) * ((cy - uy) / cs2 + (cx * ux + cy * uy) * cy / (cs2 * cs2)) * fy);
        real* fp = &o->f[q * n + nd];
        *fp = *fp - om * (*fp - o->feq[q * n + nd]) + ft;
    }
}

/* MRT<2>::apply + compute_forcing_term (MRT.cu:4-76) */
static void collide_mrt(const lbo* o, long nd) {
    const long n = o->n;
    real fx = o->fx[nd], fy = o->fy[nd], ux = o->ux[nd], uy = o->uy[nd];
    real F[9];
    F[0] = 0;
    F[1] = (real)6 * (fx * ux + fy * uy);
    F[2] = (real)-6 * (fx * ux + fy * uy);
    F[3] = fx;
    if (o->p.quirks & LBO_QUIRK_MRT_FORCE) { F[4] = fy; F[5] = -fx; }
    else { F[4] = -fx; F[5] = fy; }
    F[6] = -fy;
    F[7] = (real)2 * (fx * ux - fy * uy);
    F[8] = fx * uy + fy * ux;
    real m[9], mp[9];
    for (int k = 0; k < 9; k++) {
        real a = 0, b = 0;
        for (int i = 0; i < 9; i++) {
            a += (real)MM[k][i] * o->f[i * n + nd];
            b += (real)MM[k][i] * o->feq[i * n + nd];
        }
        m[k] = a;
        real s = (real)o->p.S[k];
        mp[k] = a - s * (a - b) + ((real)1 - s / (real)2) * F[k];
    }
    (void)m;
    for (int k = 0; k < 9; k++) {
        real v = 0;
        for (int i = 0; i < 9; i++) v += MINV[k][i] * mp[i];
        o->f[k * n + nd] = v;
    }
}

/* Central-moment collision CM<2,Adapter>::apply (CM.cuh:27-138).  The back
 * transform f = T^-1(u) k* is done by shifting central moments to raw moments
 * (binomial expansion about u) and inverting the raw-moment basis of D2Q9,
 * which is the same linear map as the reference's closed-form T^-1(u). */
static void collide_cm(const lbo* o, long nd) {
    const long n = o->n;
    real ux = o->ux[nd], uy = o->uy[nd], Fx = o->fx[nd], Fy = o->fy[nd];
    real f[9];
    real rho = 0;
    for (int i = 0; i < 9; i++) { f[i] = o->f[i * n + nd]; rho += f[i]; }
    real k[9] = {0}, pi[3] = {0};
    k[0] = rho;
    for (int i = 0; i < 9; i++) {
        real ccx = (real)CX[i] - ux, ccy = (real)CY[i] - uy;
        real ccx2 = ccx * ccx, ccy2 = ccy * ccy;
        real fi = f[i];
        k[1] += fi * ccx;
        k[2] += fi * ccy;
        k[3] += fi * (ccx2 + ccy2);
        k[4] += fi * (ccx2 - ccy2);
        k[5] += fi * ccx * ccy;
        k[6] += fi * ccx2 * ccy;
        k[7] += fi * ccx * ccy2;
        k[8] += fi * ccx2 * ccy2;
        pi[0] += fi * (real)(CX[i] * CX[i]);
        pi[1] += fi * (real)(CX[i] * CY[i]);
        pi[2] += fi * (real)(CY[i] * CY[i]);
    }
    real pimag = (real)sqrt((double)(pi[0] * pi[0] + (real)2 * pi[1] * pi[1] + pi[2] * pi[2]));
    const real cs2 = (real)1 / (real)3;
    real keq[9] = {rho, 0, 0, (real)2 * rho * cs2, 0, 0, 0, 0, rho * cs2 * cs2};
    real F[9] = {0, Fx, Fy, 0, 0, 0, Fy * cs2, Fx * cs2, 0};
    real hor = 1;
    if (o->p.op == LBO_CM_OPT) {
        /* OptimalAdapter::compute_higher_order_relaxation (adapters.cuh:48-111) */
        real jmag = (real)sqrt((double)(ux * ux + uy * uy)) * rho;
        real sp[4] = {rho / o->avg[0], jmag / o->avg[1], pimag / o->avg[2], (real)1};
        const real th[4] = {(real)0.0003f, (real)-0.00775f, (real)0.00016f, (real)0.0087f};
        real ts = 0;
        for (int i = 0; i < 4; i++) ts += th[i] * sp[i];
        ts = ts > (real)0 ? ts : (real)0.005f;
        ts = ts < (real)1.5f ? ts : (real)1.5f;
        hor = (real)1 / ((real)3 * ts + (real)0.5);
    }
    real kp[9];
    for (int i = 0; i < 9; i++) {
        real s = (o->p.op == LBO_CM_OPT && i > 5) ? hor : (real)o->p.S[i];
        kp[i] = k[i] - s * (k[i] - keq[i]) + ((real)1 - (real)0.5 * s) * F[i];
    }
    /* central moments kappa_ab about u from the k basis */
    real c00 = kp[0], c10 = kp[1], c01 = kp[2];
    real c20 = (kp[3] + kp[4]) * (real)0.5, c02 = (kp[3] - kp[4]) * (real)0.5;
    real c11 = kp[5], c21 = kp[6], c12 = kp[7], c22 = kp[8];
    /* raw moments m_ab = sum_{i<=a, j<=b} C(a,i) C(b,j) ux^(a-i) uy^(b-j) kappa_ij */
    real m00 = c00;
    real m10 = c10 + ux * c00;
    real m01 = c01 + uy * c00;
    real m20 = c20 + (real)2 * ux * c10 + ux * ux * c00;
    real m02 = c02 + (real)2 * uy * c01 + uy * uy * c00;
    real m11 = c11 + ux * c01 + uy * c10 + ux * uy * c00;
    real m21 = c21 + (real)2 * ux * c11 + uy * c20 + ux * ux * c01 + (real)2 * ux * uy * c10 + ux * ux * uy * c00;
    real m12 = c12 + (real)2 * uy * c11 + ux * c02 + uy * uy * c10 + (real)2 * ux * uy * c01 + ux * uy * uy * c00;
    real m22 = c22 + (real)2 * ux * c12 + (real)2 * uy * c21 + ux * ux * c02 + uy * uy * c20
             + (real)4 * ux * uy * c11 + (real)2 * ux * uy * uy * c10 + (real)2 * ux * ux * uy * c01
             + ux * ux * uy * uy * c00;
    /* D2Q9 populations from raw moments (velocities in {-1,0,1}) */
    real out[9];
    out[0] = m00 - m20 - m02 + m22;
    out[1] = (real)0.5 * (m10 + m20 - m12 - m22);
    out[3] = (real)0.5 * (-m10 + m20 + m12 - m22);
    out[2] = (real)0.5 * (m01 + m02 - m21 - m22);
    out[4] = (real)0.5 * (-m01 + m02 + m21 - m22);
    out[5] = (real)0.25 * (m11 + m21 + m12 + m22);
    out[6] = (real)0.25 * (-m11 + m21 - m12 + m22);
    out[7] = (real)0.25 * (m11 - m21 - m12 + m22);
    out[8] = (real)0.25 * (-m11 - m21 + m12 + m22);
    for (int i = 0; i < 9; i++) o->f[i * n + nd] = out[i];
}

/* ---------------------------------------------------------------- driver */

/* Brinkman drag F_B = -gamma rho u of a partially solid node (Guo & Zhao
 * 2002), no reference counterpart: u = (j + F/2) / (rho (1 + gamma/2)) and
 * the collision sees F + F_B.  NULL removes the field. */
int lbo_set_gamma(lbo* o, const double* gamma) {
    if (!gamma) {
        free(o->gamma);
        o->gamma = NULL;
        return 0;
    }
    if (!o->gamma) o->gamma = (real*)xcalloc(o->n, sizeof(real));
    for (long i = 0; i < o->n; i++) o->gamma[i] = (real)gamma[i];
    return 0;
}

int lbo_init(lbo* o, const double* rho, const double* u, const double* force) {
    const long n = o->n;
    for (long i = 0; i < n; i++) {
        o->rho[i] = (real)rho[i];
        o->ux[i] = (real)u[i];
        o->uy[i] = (real)u[n + i];
        o->bfx[i] = force ? (real)force[i] : 0;
        o->bfy[i] = force ? (real)force[n + i] : 0;
        o->fx[i] = o->bfx[i];
        o->fy[i] = o->bfy[i];
        /* init_node: f = f_back = f_eq (init.cuh:12-27) */
        for (int q = 0; q < 9; q++) {
            real v = feq_ref(q, o->rho[i], o->ux[i], o->uy[i]);
            o->feq[q * n + i] = v;
            o->f[q * n + i] = v;
            o->fb[q * n + i] = v;
        }
    }
    o->t = 0;
    return 0;
}

long lbo_time(const lbo* o) { return o->t; }

static void one_step(lbo* o) {
    const int nx = o->nx, ny = o->ny;
    const long n = o->n;
    const int px = o->p.periodic_x, py = o->p.periodic_y;
    o->t++;
    /* stream: push q = 1..8 (q = 0 too unless the reference quirk is on) */
    const int q0 = (o->p.quirks & LBO_QUIRK_REST_LAG) ? 1 : 0;
#pragma omp parallel for schedule(static)
    for (int y = 0; y < ny; y++)
        for (int x = 0; x < nx; x++) {
            long nd = (long)y * nx + x;
            uint8_t fl = o->flags[nd];
            int halfway = fl == LBO_MOVING_WALL_BB || fl == LBO_HALFWAY_BB;
            for (int q = q0; q < 9; q++) {
                int xn = x + CX[q], yn = y + CY[q];
                if (px) xn = (xn + nx) % nx;
                if (py) yn = (yn + ny) % ny;
                if (xn < 0 || xn >= nx || yn < 0 || yn >= ny) {
                    if (halfway) o->fb[OPP[q] * n + nd] = o->f[q * n + nd] - halfway_term(o, q, fl);
                    continue;
                }
                o->fb[q * n + (long)yn * nx + xn] = o->f[q * n + nd];
            }
        }
    real* tmp = o->f; o->f = o->fb; o->fb = tmp;
    /* boundaries */
    if (o->has_aux_bc) {
#pragma omp parallel for schedule(static)
        for (int y = 0; y < ny; y++)
            for (int x = 0; x < nx; x++) {
                long nd = (long)y * nx + x;
                uint8_t fl = o->flags[nd];
                if (fl == LBO_ZG_OUTFLOW || fl == LBO_PRESSURE_OUTLET || fl == LBO_REGULARIZED_BOUNCE_BACK_CORNER) {
                    real a[9] = {0};
                    bc_aux(o, x, y, a);
                    for (int q = 0; q < 9; q++) o->aux[q * n + nd] = a[q];
                }
            }
    }
#pragma omp parallel for schedule(static)
    for (int y = 0; y < ny; y++)
        for (int x = 0; x < nx; x++) {
            long nd = (long)y * nx + x;
            uint8_t fl = o->flags[nd];
            if (fl == LBO_FLUID) continue;
            real fl9[9], a[9];
            for (int q = 0; q < 9; q++) { fl9[q] = o->f[q * n + nd]; a[q] = o->aux[q * n + nd]; }
            apply_bc(o, fl9, x, y, fl, a);
            for (int q = 0; q < 9; q++) o->f[q * n + nd] = fl9[q];
        }
    /* uncorrected macroscopics + force reset */
#pragma omp parallel for schedule(static)
    for (long nd = 0; nd < n; nd++) {
        real r = 0, jx = 0, jy = 0, pxx = 0, pxy = 0, pyy = 0;
        for (int q = 0; q < 9; q++) {
            real fq = o->f[q * n + nd];
            r += fq;
            jx += fq * (real)CX[q];
            jy += fq * (real)CY[q];
            pxx += fq * (real)(CX[q] * CX[q]);
            pxy += fq * (real)(CX[q] * CY[q]);
            pyy += fq * (real)(CY[q] * CY[q]);
        }
        o->rho[nd] = r;
        real inv = (real)1 / r;
        o->ux[nd] = jx * inv;
        o->uy[nd] = jy * inv;
        o->pimag[nd] = (real)sqrt((double)(pxx * pxx + (real)2 * pxy * pxy + pyy * pyy));
        o->fx[nd] = o->bfx[nd];
        o->fy[nd] = o->bfy[nd];
    }
    if (o->nm > 0) ibm_multi_direct(o);
    /* correct macroscopics, sums, averages */
    double s0 = 0, s1 = 0, s2 = 0, a0 = 0, a1 = 0, a2 = 0;
#pragma omp parallel for schedule(static) reduction(+ : s0, s1, s2, a0, a1, a2)
    for (long nd = 0; nd < n; nd++) {
        real r = o->rho[nd];
        o->ux[nd] += (real)0.5 * o->fx[nd] / r;
        o->uy[nd] += (real)0.5 * o->fy[nd] / r;
        if (o->gamma) {
            const real g = o->gamma[nd];
            const real sc = (real)1 / ((real)0.5 * g + (real)1);
            o->ux[nd] *= sc;
            o->uy[nd] *= sc;
            o->fx[nd] -= g * r * o->ux[nd];
            o->fy[nd] -= g * r * o->uy[nd];
        }
        s0 += (double)r;
        s1 += (double)r * (double)o->ux[nd];
        s2 += (double)r * (double)o->uy[nd];
        a0 += (double)r;
        a1 += (double)(r * (real)sqrt((double)(o->ux[nd] * o->ux[nd] + o->uy[nd] * o->uy[nd])));
        a2 += (double)o->pimag[nd];
    }
    o->sums[0] = s0; o->sums[1] = s1; o->sums[2] = s2;
    o->avg[0] = (real)(a0 / (double)n);
    o->avg[1] = (real)(a1 / (double)n);
    o->avg[2] = (real)(a2 / (double)n);
    /* equilibrium + collide */
    const int op = o->p.op;
#pragma omp parallel for schedule(static)
    for (long nd = 0; nd < n; nd++) {
        if (op == LBO_BGK || op == LBO_MRT)
            for (int q = 0; q < 9; q++) o->feq[q * n + nd] = feq_ref(q, o->rho[nd], o->ux[nd], o->uy[nd]);
        if (op == LBO_BGK) collide_bgk(o, nd);
        else if (op == LBO_MRT) collide_mrt(o, nd);
        else collide_cm(o, nd);
    }
}

int lbo_step(lbo* o, int nsteps) {
#ifdef _OPENMP
    if (o->p.threads > 0) omp_set_num_threads(o->p.threads);
#endif
    for (int s = 0; s < nsteps; s++) one_step(o);
    return 0;
}

void lbo_get_f(const lbo* o, double* f) {
    for (long i = 0; i < 9 * o->n; i++) f[i] = (double)o->f[i];
}

void lbo_get_moments(const lbo* o, double* rho, double* u, double* force) {
    const long n = o->n;
    for (long i = 0; i < n; i++) {
        if (rho) rho[i] = (double)o->rho[i];
        if (u) { u[i] = (double)o->ux[i]; u[n + i] = (double)o->uy[i]; }
        if (force) { force[i] = (double)o->fx[i]; force[n + i] = (double)o->fy[i]; }
    }
}

void lbo_get_avg(const lbo* o, double* avg3) {
    for (int i = 0; i < 3; i++) avg3[i] = (double)o->avg[i];
}

void lbo_get_marker(const lbo* o, double* u2n, double* rho_n, double* force2n) {
    for (int k = 0; k < o->nm; k++) {
        if (u2n) { u2n[k] = (double)o->mux[k]; u2n[o->nm + k] = (double)o->muy[k]; }
        if (rho_n) rho_n[k] = (double)o->mrho[k];
        if (force2n) { force2n[k] = (double)o->mftx[k]; force2n[o->nm + k] = (double)o->mfty[k]; }
    }
}

void lbo_get_sums(const lbo* o, double* sums3) {
    for (int i = 0; i < 3; i++) sums3[i] = o->sums[i];
}
