/*
 * TEST INFRASTRUCTURE ONLY -- see fvm_oracle.h.  CPU restatement of the
 * reference's explicit FVM step, written to reproduce its FP64 results bit for
 * bit: every expression keeps the reference's operation order, including
 * products with the zero components of axis normals.  Build with
 * -ffp-contract=off (no FMA contraction) and without fast-math.
 */
#include "fvm_oracle.h"

#include <float.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define NV 5

typedef struct { double x, y, z; } vec3;

static inline double dot3(vec3 a, vec3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }

/* ------------------------------------------------------------------------ */
/* Grid: cell centres by accumulation, grid.h:124-344.                      */
/* ------------------------------------------------------------------------ */

static void axis_grid(const orc_config* c, int a, int n, int g, double length, double* X, double* H) {
    /* CompressionX starts as one default BlockNode (pos 0, q 1, N -1) and
       InitLocal appends a closing BlockNode(L) (grid.h:165). */
    double pos[ORC_MAX_BLOCKS + 1], q[ORC_MAX_BLOCKS + 1];
    int nc[ORC_MAX_BLOCKS + 1];
    int nb = c->n_blocks[a];
    if (nb <= 0) {
        nb = 1;
        pos[0] = 0.0; q[0] = 1.0; nc[0] = -1;
    } else {
        for (int b = 0; b < nb; ++b) { pos[b] = c->block_pos[a][b]; q[b] = c->block_q[a][b]; nc[b] = c->block_cells[a][b]; }
    }
    pos[nb] = length; q[nb] = 1.0; nc[nb] = -1;
    int nnodes = nb + 1;

    double stp = 1.0;
    if (nc[0] < 1) {
        stp = length / n;
        nc[0] = n;
    } else {
        double bl_len = pos[1] - pos[0];
        int ncells = nc[0];
        if (q[0] == 1.0) stp = bl_len / ncells;
        else stp = bl_len * (1.0 - q[0]) / (1.0 - pow(q[0], ncells));
    }
    double xc = -(g * stp) + 0.5 * stp;
    int ci = 0;
    for (; ci < g; ++ci) { X[ci] = xc; H[ci] = stp; xc += stp; }
    for (int b = 1; b < nnodes; ++b) {
        double qb = q[b - 1];
        for (int i = 0; i < nc[b - 1]; ++i) {
            X[ci + i] = xc;
            H[ci + i] = stp;
            xc += 0.5 * stp * (1.0 + qb);
            stp *= qb;
        }
        ci += nc[b - 1];
        if (nc[b] > 0) {
            double new_len = pos[b + 1] - pos[b];
            int new_nc = nc[b];
            double new_q = q[b];
            if (new_q == 1.0) stp = new_len / new_nc;
            else stp = new_len * (1.0 - new_q) / (1.0 - pow(new_q, new_nc));
            xc = pos[b] + 0.5 * stp;
        }
    }
    for (int i = 0; i < g; ++i) { X[ci + i] = xc; H[ci + i] = stp; xc += stp; }
}

void orc_dims(const orc_config* c, int* nxa, int* nya, int* nza) {
    *nxa = c->nx + 2;
    *nya = c->ndims > 1 ? c->ny + 2 : 1;
    *nza = c->ndims > 2 ? c->nz + 2 : 1;
}

int orc_grid(const orc_config* c, double* x, double* hx, double* y, double* hy, double* z, double* hz) {
    int nxa, nya, nza;
    orc_dims(c, &nxa, &nya, &nza);
    axis_grid(c, 0, c->nx, 1, c->length[0], x, hx);
    if (c->ndims > 1) axis_grid(c, 1, c->ny, 1, c->length[1], y, hy);
    else { y[0] = 0.0; hy[0] = 1.0; }
    if (c->ndims > 2) axis_grid(c, 2, c->nz, 1, c->length[2], z, hz);
    else { z[0] = 0.0; hz[0] = 1.0; }
    (void)nxa; (void)nya; (void)nza;
    return 0;
}

/* ------------------------------------------------------------------------ */
/* Working context                                                          */
/* ------------------------------------------------------------------------ */

typedef struct {
    const orc_config* c;
    int nxa, nya, nza, ncells;
    int gx, gy, gz;            /* ghost offsets per axis (1 if active) */
    int imin, imax, jmin, jmax, kmin, kmax;
    double *x, *hx, *y, *hy, *z, *hz;
    double* vol;               /* grid.h:347-360 */
    double* spectral;          /* per cell, ExplicitRungeKuttaFVM.h:31 */
    double* resid;             /* AoS like values */
    /* reconstruction objects, one per cell of the values array
       (ExplicitRungeKuttaFVM.h:36,61-72): vals, grads[3][5], lim[5] */
    double* rvals;
    double* rgrad;
    double* rlim;
    double* eps2;              /* Venkatakrishnan eps^2 per cell (Limiters.h:93-96) */
    const double* U;           /* the step's values (cell values for the viscous fluxes) */
    /* velocity gradients per cell (gradientVelocityX/Y/Z, ExplicitRungeKuttaFVM.h:
       81-134): vgrad[(cell * 3 + d) * 3 + e] = d(velocity d)/d(axis e) */
    double* vgrad;
} orc_ctx;

static inline int cidx(const orc_ctx* w, int i, int j, int k) {
    return (k * w->nya + j) * w->nxa + i;
}

/* ------------------------------------------------------------------------ */
/* EOS helpers                                                              */
/* ------------------------------------------------------------------------ */

/* Pressure from conserved variables: ideal gas as RoeSolverPerfectGasEOS.h:49;
   stiffened gas p = (g-1)(rhoE - rho|u|^2/2) - g p_inf (not in the reference). */
static inline double eos_pressure(const orc_config* c, double ro, double vx, double vy, double vz, double roE) {
    double p = (c->gamma - 1.0) * (roE - ro * (vx * vx + vy * vy + vz * vz) / 2.0);
    if (c->eos == ORC_EOS_STIFFENED) p = p - c->gamma * c->p_inf;
    return p;
}

/* ------------------------------------------------------------------------ */
/* Boundary conditions, BCGeneral.h:100-268                                 */
/* ------------------------------------------------------------------------ */

static void bc_dummy_values(const orc_config* c, int side, const double* in, vec3 n, double* out) {
    int t = c->bc_type[side];
    switch (t) {
    case ORC_BC_SYMMETRY: { /* BCGeneral.h:214-226 */
        vec3 rv = {in[1], in[2], in[3]};
        double s = dot3(n, rv);
        vec3 rn = {s * n.x, s * n.y, s * n.z};
        for (int v = 0; v < NV; ++v) out[v] = in[v];
        out[1] -= 2.0 * rn.x;
        out[2] -= 2.0 * rn.y;
        out[3] -= 2.0 * rn.z;
        break;
    }
    case ORC_BC_WALL: /* BCGeneral.h:229-238 */
        for (int v = 0; v < NV; ++v) out[v] = in[v];
        out[1] *= (-1);
        out[2] *= (-1);
        out[3] *= (-1);
        break;
    case ORC_BC_MOVING_WALL: { /* BCGeneral.h:241-268 */
        double rho = in[0];
        vec3 vin = {in[1] / rho, in[2] / rho, in[3] / rho};
        double rhoe = in[4] - 0.5 * rho * dot3(vin, vin);
        vec3 vb = {c->bc_velocity[side][0], c->bc_velocity[side][1], c->bc_velocity[side][2]};
        vec3 vd = {2.0 * vb.x - vin.x, 2.0 * vb.y - vin.y, 2.0 * vb.z - vin.z};
        out[0] = rho;
        out[1] = rho * vd.x;
        out[2] = rho * vd.y;
        out[3] = rho * vd.z;
        out[4] = rhoe + 0.5 * rho * dot3(vd, vd);
        break;
    }
    case ORC_BC_SUBSONIC_INLET: { /* BCGeneral.h:186-196 */
        double r = c->bc_density[side];
        vec3 vv = {c->bc_velocity[side][0], c->bc_velocity[side][1], c->bc_velocity[side][2]};
        out[0] = r;
        out[1] = r * vv.x;
        out[2] = r * vv.y;
        out[3] = r * vv.z;
        double eint = c->bc_pstatic[side] / (c->gamma - 1);
        if (c->eos == ORC_EOS_STIFFENED) eint = eint + c->gamma * c->p_inf / (c->gamma - 1);
        out[4] = eint + 0.5 * r * dot3(vv, vv);
        break;
    }
    default: /* Natural (BCGeneral.h:207-211), SubsonicOutlet (:200-204) */
        for (int v = 0; v < NV; ++v) out[v] = in[v];
        break;
    }
}

/* BC table entry of the boundary face of `side` in the row of cell (i, j, k)
   (values-array indices; the tangential ones identify the face): the side's
   own BC, or for a position-dependent side the kind its marker function gave
   at the face's centre (Kernel::InitBoundaryConditions kernel.h:284-316,
   BCinfo::getMarker BCGeneral.h:52-56). */
static int bc_entry(const orc_ctx* w, int side, int i, int j, int k) {
    const unsigned char* m = w->c->bc_marker[side];
    if (!m) return side;
    const int a = side / 2;
    const int ii = i - w->imin, jj = j - w->jmin, kk = k - w->kmin;
    const int nx = w->c->nx, ny = w->c->ndims > 1 ? w->c->ny : 1;
    const int f = a == 0 ? jj + ny * kk : (a == 1 ? ii + nx * kk : ii + nx * jj);
    return 6 + m[f];
}

/* ExchangeValues (kernel.h:334-690) on one rank, then ComputeDummyCellValues
   (kernel.h:693-915): periodic axes copy the opposite interior layer, other
   axes apply the side's BC to the mirror cell with faceNormalL on both sides
   (kernel.h:760,829,899). */
static void fill_ghosts(orc_ctx* w, double* U) {
    const orc_config* c = w->c;
    double out[NV];
    /* x */
    for (int k = w->kmin; k <= w->kmax; ++k)
        for (int j = w->jmin; j <= w->jmax; ++j) {
            double* lo = U + (size_t)cidx(w, w->imin - 1, j, k) * NV;
            double* hi = U + (size_t)cidx(w, w->imax + 1, j, k) * NV;
            const double* first = U + (size_t)cidx(w, w->imin, j, k) * NV;
            const double* last = U + (size_t)cidx(w, w->imax, j, k) * NV;
            if (c->periodic[0]) {
                memcpy(hi, first, sizeof(double) * NV);
                memcpy(lo, last, sizeof(double) * NV);
            } else {
                vec3 nl = {-1.0, 0.0, 0.0};
                bc_dummy_values(c, bc_entry(w, 0, w->imin, j, k), first, nl, out); memcpy(lo, out, sizeof out);
                bc_dummy_values(c, bc_entry(w, 1, w->imax, j, k), last, nl, out); memcpy(hi, out, sizeof out);
            }
        }
    if (c->ndims < 2) return;
    for (int i = w->imin; i <= w->imax; ++i)
        for (int k = w->kmin; k <= w->kmax; ++k) {
            double* lo = U + (size_t)cidx(w, i, w->jmin - 1, k) * NV;
            double* hi = U + (size_t)cidx(w, i, w->jmax + 1, k) * NV;
            const double* first = U + (size_t)cidx(w, i, w->jmin, k) * NV;
            const double* last = U + (size_t)cidx(w, i, w->jmax, k) * NV;
            if (c->periodic[1]) {
                memcpy(hi, first, sizeof(double) * NV);
                memcpy(lo, last, sizeof(double) * NV);
            } else {
                vec3 nl = {0.0, -1.0, 0.0};
                bc_dummy_values(c, bc_entry(w, 2, i, w->jmin, k), first, nl, out); memcpy(lo, out, sizeof out);
                bc_dummy_values(c, bc_entry(w, 3, i, w->jmax, k), last, nl, out); memcpy(hi, out, sizeof out);
            }
        }
    if (c->ndims < 3) return;
    for (int i = w->imin; i <= w->imax; ++i)
        for (int j = w->jmin; j <= w->jmax; ++j) {
            double* lo = U + (size_t)cidx(w, i, j, w->kmin - 1) * NV;
            double* hi = U + (size_t)cidx(w, i, j, w->kmax + 1) * NV;
            const double* first = U + (size_t)cidx(w, i, j, w->kmin) * NV;
            const double* last = U + (size_t)cidx(w, i, j, w->kmax) * NV;
            if (c->periodic[2]) {
                memcpy(hi, first, sizeof(double) * NV);
                memcpy(lo, last, sizeof(double) * NV);
            } else {
                vec3 nl = {0.0, 0.0, -1.0};
                bc_dummy_values(c, bc_entry(w, 4, i, j, w->kmin), first, nl, out); memcpy(lo, out, sizeof out);
                bc_dummy_values(c, bc_entry(w, 5, i, j, w->kmax), last, nl, out); memcpy(hi, out, sizeof out);
            }
        }
}

/* ------------------------------------------------------------------------ */
/* Reconstruction, ExplicitRungeKuttaFVM.h:879-925 and src/Reconstruction   */
/* ------------------------------------------------------------------------ */

/* BarsJespersen l-function, Limiters.h:80-82: std::min(1.0, r). */
static inline double lim_bj(double um, double ui, double d2) {
    double r = (um - ui) / d2;
    return (r < 1.0) ? r : 1.0;
}

/* Venkatakrishnan l-function, Limiters.h:102-115. */
static inline double lim_venkat(double um, double ui, double d2, double umax, double umin, double eps2) {
    double un = 0.5 * (umax - umin);
    um /= un;
    ui /= un;
    d2 /= un;
    double dm = um - ui;
    return ((dm * dm + eps2) + 2 * d2 * dm) / (dm * dm + 2 * d2 * d2 + dm * d2 + eps2);
}

static void reconstruct_cell(orc_ctx* w, const double* U, int i, int j, int k) {
    const orc_config* c = w->c;
    int nd = c->ndims;
    int ci = cidx(w, i, j, k);
    const double* val = U + (size_t)ci * NV;
    double* rv = w->rvals + (size_t)ci * NV;
    double* rg = w->rgrad + (size_t)ci * 3 * NV; /* [axis][var] */
    double* rl = w->rlim + (size_t)ci * NV;
    for (int v = 0; v < NV; ++v) { rv[v] = val[v]; rl[v] = 1.0; }
    for (int a = 0; a < 3 * NV; ++a) rg[a] = 0.0;
    if (c->recon == ORC_RECON_PWC) return;

    /* stencil x-, x+, y-, y+, z-, z+ (ExplicitRungeKuttaFVM.h:898-916) */
    const double* st[6];
    double sc[6]; /* neighbour centre coordinate along its axis */
    st[0] = U + (size_t)cidx(w, i - 1, j, k) * NV; sc[0] = w->x[i - 1];
    st[1] = U + (size_t)cidx(w, i + 1, j, k) * NV; sc[1] = w->x[i + 1];
    if (nd > 1) {
        st[2] = U + (size_t)cidx(w, i, j - 1, k) * NV; sc[2] = w->y[j - 1];
        st[3] = U + (size_t)cidx(w, i, j + 1, k) * NV; sc[3] = w->y[j + 1];
    }
    if (nd > 2) {
        st[4] = U + (size_t)cidx(w, i, j, k - 1) * NV; sc[4] = w->z[k - 1];
        st[5] = U + (size_t)cidx(w, i, j, k + 1) * NV; sc[5] = w->z[k + 1];
    }
    double cc[3] = {w->x[i], w->y[j], w->z[k]};

    if (c->recon == ORC_RECON_ENO2) {
        /* ENO2PointsStencil.h:202-239 */
        for (int a = 0; a < nd; ++a) {
            for (int v = 0; v < NV; ++v) {
                double gl = (val[v] - st[2 * a][v]) / (cc[a] - sc[2 * a]);
                double gr = (st[2 * a + 1][v] - val[v]) / (sc[2 * a + 1] - cc[a]);
                rg[a * NV + v] = (fabs(gl) < fabs(gr)) ? gl : gr;
            }
        }
        return;
    }

    /* Linear2PointsStencil.h:147-178: central slopes on conserved variables */
    for (int a = 0; a < nd; ++a) {
        double d = sc[2 * a + 1] - sc[2 * a];
        for (int v = 0; v < NV; ++v) rg[a * NV + v] = (st[2 * a + 1][v] - st[2 * a][v]) / d;
    }
    if (c->recon == ORC_RECON_LINEAR2) return;

    /* Linear2psLim.h:305-374: projections to the 2*nDim face centres,
       SampleSolution(point) - vals with the full 3-component dot product. */
    double h[3] = {w->hx[i], w->hy[j], w->hz[k]};
    double proj[6][NV];
    for (int f = 0; f < 2 * nd; ++f) {
        int a = f / 2;
        double s = (f & 1) ? 0.5 * h[a] : -0.5 * h[a];
        vec3 p = {a == 0 ? s : 0.0, a == 1 ? s : 0.0, a == 2 ? s : 0.0};
        for (int v = 0; v < NV; ++v) {
            vec3 g = {rg[0 * NV + v], rg[1 * NV + v], rg[2 * NV + v]};
            proj[f][v] = (val[v] + dot3(g, p)) - val[v];
        }
    }
    /* Limiter::ComputeLimiterValues, Limiters.h:28-67 */
    double eps2 = w->eps2 ? w->eps2[ci] : 0.0;
    for (int v = 0; v < NV; ++v) {
        double umax = val[v], umin = val[v];
        for (int nb = 0; nb < 2 * nd; ++nb) {
            double vn = st[nb][v];
            if (umax < vn) umax = vn;
            if (umin > vn) umin = vn;
        }
        if (umax - umin < 3.0 * DBL_MIN) continue;
        double lmin = 1.0;
        for (int f = 0; f < 2 * nd; ++f) {
            double lv = 1.0;
            double d2 = proj[f][v];
            if (c->limiter == ORC_LIM_VENKAT) {
                if (d2 > 0) lv = lim_venkat(umax, val[v], d2, umax, umin, eps2);
                if (d2 < 0) lv = lim_venkat(umin, val[v], d2, umax, umin, eps2);
            } else {
                if (d2 > 0) lv = lim_bj(umax, val[v], d2);
                if (d2 < 0) lv = lim_bj(umin, val[v], d2);
            }
            if (lmin > lv) lmin = lv;
        }
        rl[v] = lmin;
    }
}

/* SampleSolution at a face offset along axis a (PiecewiseConstant.h:15,
   Linear2PointsStencil.h:26-30, Linear2psLim.h:17-21), with the ghost-cell
   copy semantics of ExchangeReconstructions (:928-1147) handled by the
   caller passing the source cell. */
static void sample(const orc_ctx* w, int ci, int a, double s, double* out) {
    const orc_config* c = w->c;
    const double* rv = w->rvals + (size_t)ci * NV;
    if (c->recon == ORC_RECON_PWC) { for (int v = 0; v < NV; ++v) out[v] = rv[v]; return; }
    const double* rg = w->rgrad + (size_t)ci * 3 * NV;
    const double* rl = w->rlim + (size_t)ci * NV;
    vec3 p = {a == 0 ? s : 0.0, a == 1 ? s : 0.0, a == 2 ? s : 0.0};
    for (int v = 0; v < NV; ++v) {
        vec3 g = {rg[0 * NV + v], rg[1 * NV + v], rg[2 * NV + v]};
        if (c->recon == ORC_RECON_LINEAR2_LIM) out[v] = rv[v] + rl[v] * dot3(g, p);
        else out[v] = rv[v] + dot3(g, p);
    }
}

/* Ghost reconstruction objects on periodic axes are deserialised copies of
   the opposite interior cell's object (ExchangeReconstructions on one rank);
   only vals, the active-axis gradients and the limiter travel
   (Linear2PointsStencil.h:117-143, Linear2psLim.h:279-301). */
static void exchange_recon(orc_ctx* w) {
    const orc_config* c = w->c;
    int nd = c->ndims;
    size_t g3 = 3 * NV;
#define COPY_RECON(dst, src)                                                              \
    do {                                                                                  \
        memcpy(w->rvals + (size_t)(dst) * NV, w->rvals + (size_t)(src) * NV, sizeof(double) * NV); \
        for (int a_ = 0; a_ < nd; ++a_)                                                   \
            memcpy(w->rgrad + (size_t)(dst) * g3 + a_ * NV, w->rgrad + (size_t)(src) * g3 + a_ * NV, \
                   sizeof(double) * NV);                                                  \
        memcpy(w->rlim + (size_t)(dst) * NV, w->rlim + (size_t)(src) * NV, sizeof(double) * NV); \
    } while (0)
    if (c->periodic[0])
        for (int j = w->jmin; j <= w->jmax; ++j)
            for (int k = w->kmin; k <= w->kmax; ++k) {
                COPY_RECON(cidx(w, w->imax + 1, j, k), cidx(w, w->imin, j, k));
                COPY_RECON(cidx(w, w->imin - 1, j, k), cidx(w, w->imax, j, k));
            }
    if (nd > 1 && c->periodic[1])
        for (int i = w->imin; i <= w->imax; ++i)
            for (int k = w->kmin; k <= w->kmax; ++k) {
                COPY_RECON(cidx(w, i, w->jmax + 1, k), cidx(w, i, w->jmin, k));
                COPY_RECON(cidx(w, i, w->jmin - 1, k), cidx(w, i, w->jmax, k));
            }
    if (nd > 2 && c->periodic[2])
        for (int i = w->imin; i <= w->imax; ++i)
            for (int j = w->jmin; j <= w->jmax; ++j) {
                COPY_RECON(cidx(w, i, j, w->kmax + 1), cidx(w, i, j, w->kmin));
                COPY_RECON(cidx(w, i, j, w->kmin - 1), cidx(w, i, j, w->kmax));
            }
#undef COPY_RECON
}

/* ------------------------------------------------------------------------ */
/* Riemann solvers                                                          */
/* ------------------------------------------------------------------------ */

/* Physical flux F(U).n, RoeSolverPerfectGasEOS.h:41-58 (+ stiffened p). */
static void phys_flux(const orc_config* c, const double* U, vec3 n, double* res) {
    double ro = U[0];
    double vx = U[1] / ro;
    double vy = U[2] / ro;
    double vz = U[3] / ro;
    double roE = U[4];
    double p = eos_pressure(c, ro, vx, vy, vz, roE);
    double vn = vx * n.x + vy * n.y + vz * n.z;
    res[0] = ro * vn;
    res[1] = ro * vn * vx + n.x * p;
    res[2] = ro * vn * vy + n.y * p;
    res[3] = ro * vn * vz + n.z * p;
    res[4] = vn * (roE + p);
}

static inline double harten(double z, double eps) {
    z = fabs(z);
    if (z < eps) z = ((z * z) / eps + eps) * 0.5;
    return z;
}

/* RoeSolverPerfectGasEOS::ComputeFlux, RoeSolverPerfectGasEOS.h:74-160.
   The stiffened-gas variant (not in the reference) only changes the
   enthalpy, h = (E + p)/rho, through the -g p_inf/rho term. */
static double roe_flux(const orc_config* c, const double* UL, const double* UR, vec3 fn, double* flux) {
    const double g = c->gamma;
    double FL[NV], FR[NV];
    phys_flux(c, UL, fn, FL);
    phys_flux(c, UR, fn, FR);
    for (int i = 0; i < NV; ++i) flux[i] = FL[i] + FR[i];
    double ro_l = UL[0];
    double ro_r = UR[0];
    vec3 vl = {UL[1] / ro_l, UL[2] / ro_l, UL[3] / ro_l};
    vec3 vr = {UR[1] / ro_r, UR[2] / ro_r, UR[3] / ro_r};
    double e_l = UL[4] / ro_l;
    double e_r = UR[4] / ro_r;
    double k = 0.5 * dot3(vl, vl);
    double h_l = (e_l - k) * g + k;
    k = 0.5 * dot3(vr, vr);
    double h_r = (e_r - k) * g + k;
    if (c->eos == ORC_EOS_STIFFENED) {
        h_l = h_l - g * c->p_inf / ro_l;
        h_r = h_r - g * c->p_inf / ro_r;
    }
    double ql = sqrt(ro_l) / (sqrt(ro_l) + sqrt(ro_r));
    double qr = sqrt(ro_r) / (sqrt(ro_l) + sqrt(ro_r));
    vec3 vel = {ql * vl.x + qr * vr.x, ql * vl.y + qr * vr.y, ql * vl.z + qr * vr.z};
    double h = ql * h_l + qr * h_r;
    double phi2 = 0.5 * (g - 1) * dot3(vel, vel);
    double dn = 1.0;
    double cs = sqrt((g - 1) * h - phi2);
    double uw = dot3(vel, fn);
    double eig_max = fabs(uw) + cs * dn;
    double AA1 = harten(uw, c->eps * eig_max);
    double AA3 = harten(uw + cs * dn, c->eps * eig_max);
    double AA4 = harten(uw - cs * dn, c->eps * eig_max);
    double Eig1 = AA1;
    double Eiga = (AA3 - AA4) * 0.5 / (dn * cs);
    double Eigb = (AA3 + AA4) * 0.5 - AA1;
    double Qa[NV] = {0, fn.x, fn.y, fn.z, uw};
    double Qb[NV] = {1, vel.x, vel.y, vel.z, h};
    vec3 dvr = {vr.x - vel.x, vr.y - vel.y, vr.z - vel.z};
    vec3 dvl = {vl.x - vel.x, vl.y - vel.y, vl.z - vel.z};
    vec3 rfr = {ro_r * fn.x, ro_r * fn.y, ro_r * fn.z};
    vec3 rfl = {ro_l * fn.x, ro_l * fn.y, ro_l * fn.z};
    double R1 = phi2 * ro_r - (g - 1) * ro_r * (dot3(vel, vr) - e_r);
    double D1 = dot3(rfr, dvr);
    double R2 = phi2 * ro_l - (g - 1) * ro_l * (dot3(vel, vl) - e_l);
    double D2 = dot3(rfl, dvl);
    double C2 = 1.0 / (cs * cs);
    double DN2 = 1.0 / (dn * dn);
    for (int i = 0; i < NV; ++i) {
        flux[i] += (Eig1 * UL[i] + Eiga * (R2 * Qa[i] + D2 * Qb[i]) + Eigb * (R2 * Qb[i] * C2 + D2 * Qa[i] * DN2)
                    - Eig1 * UR[i] - Eiga * (R1 * Qa[i] + D1 * Qb[i]) - Eigb * (R1 * Qb[i] * C2 + D1 * Qa[i] * DN2));
        flux[i] *= 0.5;
    }
    return eig_max;
}

/* HLLC flux (Toro, ch. 10.4, eqs. 10.37-10.39) with Einfeldt-type wave
   speeds from Roe averages (Toro eq. 10.52).  Not in the reference: this
   restatement is its oracle.  MaxEigenvalue = max(|S_L|, |S_R|). */
static double hllc_flux(const orc_config* c, const double* UL, const double* UR, int a, double* flux) {
    const double g = c->gamma;
    const double pinf = (c->eos == ORC_EOS_STIFFENED) ? c->p_inf : 0.0;
    int m = 1 + a;
    double rl = UL[0], rr = UR[0];
    double ul = UL[m] / rl, ur = UR[m] / rr;
    double vlx = UL[1] / rl, vly = UL[2] / rl, vlz = UL[3] / rl;
    double vrx = UR[1] / rr, vry = UR[2] / rr, vrz = UR[3] / rr;
    double pl = eos_pressure(c, rl, vlx, vly, vlz, UL[4]);
    double pr = eos_pressure(c, rr, vrx, vry, vrz, UR[4]);
    double cl = sqrt(g * (pl + pinf) / rl);
    double cr = sqrt(g * (pr + pinf) / rr);
    double hl = (UL[4] + pl) / rl;
    double hr = (UR[4] + pr) / rr;
    double sl = sqrt(rl), sr = sqrt(rr);
    double wl = sl / (sl + sr), wr = sr / (sl + sr);
    double ut = wl * ul + wr * ur;
    double vtx = wl * vlx + wr * vrx, vty = wl * vly + wr * vry, vtz = wl * vlz + wr * vrz;
    double ht = wl * hl + wr * hr;
    double ct = sqrt((g - 1) * (ht - 0.5 * (vtx * vtx + vty * vty + vtz * vtz)));
    double SL = fmin(ul - cl, ut - ct);
    double SR = fmax(ur + cr, ut + ct);
    double lam = fmax(fabs(SL), fabs(SR));
    double ml = rl * (SL - ul), mr = rr * (SR - ur);
    double sstar = (pr - pl + ul * ml - ur * mr) / (ml - mr);
    double FL[NV], FR[NV];
    vec3 n = {a == 0 ? 1.0 : 0.0, a == 1 ? 1.0 : 0.0, a == 2 ? 1.0 : 0.0};
    if (SL >= 0.0) {
        phys_flux(c, UL, n, flux);
    } else if (SR <= 0.0) {
        phys_flux(c, UR, n, flux);
    } else if (sstar >= 0.0) {
        phys_flux(c, UL, n, FL);
        double coef = ml / (SL - sstar);
        double us[NV];
        us[0] = coef;
        us[1] = coef * vlx; us[2] = coef * vly; us[3] = coef * vlz;
        us[m] = coef * sstar;
        us[4] = coef * (UL[4] / rl + (sstar - ul) * (sstar + pl / ml));
        for (int v = 0; v < NV; ++v) flux[v] = FL[v] + SL * (us[v] - UL[v]);
    } else {
        phys_flux(c, UR, n, FR);
        double coef = mr / (SR - sstar);
        double us[NV];
        us[0] = coef;
        us[1] = coef * vrx; us[2] = coef * vry; us[3] = coef * vrz;
        us[m] = coef * sstar;
        us[4] = coef * (UR[4] / rr + (sstar - ur) * (sstar + pr / mr));
        for (int v = 0; v < NV; ++v) flux[v] = FR[v] + SR * (us[v] - UR[v]);
    }
    return lam;
}

/* Exact (Godunov) flux of GodunovSolverPerfectGasEOS::ComputeFlux
   (GodunovSolverPerfectGasEOS.h:266-430), ideal gas.  The star pressure is the
   root of fL(p) + fR(p) + (uR - uL) (f1/f2, :56-96).  The reference minimises
   its square with alglib 3.8.0's minlm (Levenberg-Marquardt with numerical
   derivatives, diffstep 1e-6, stopping at a gradient below epsg = 1e-10,
   starting from (pL + pR)/2, :143-187); this restatement uses Newton-Raphson on
   the root with the analytic derivative (Toro, Riemann Solvers and Numerical
   Methods for Fluid Dynamics, 3rd ed., sec. 4.3.1), started from the
   primitive-variable guess (Toro eq. 4.47) and stopped at a relative change
   below 1e-14, so p* agrees with the reference to the reference's own solver
   tolerance.  Everything after p* follows the reference's steps and
   operation order. */
static double god_f(double g, double rk, double pk, double p) {
    double res;
    if (p > pk) {
        double A = 2 / ((g + 1.0) * rk);
        double B = pk * (g - 1.0) / (g + 1.0);
        res = (p - pk) * sqrt(A / (p + B));
    } else {
        double a = sqrt(g * pk / rk);
        res = pow(p / pk, (g - 1.0) / (2 * g)) - 1.0;
        res *= 2 * a / (g - 1.0);
    }
    return res;
}

static double god_df(double g, double rk, double pk, double p) {
    if (p > pk) {
        double A = 2 / ((g + 1.0) * rk);
        double B = pk * (g - 1.0) / (g + 1.0);
        return sqrt(A / (B + p)) * (1.0 - (p - pk) / (2.0 * (B + p)));
    }
    return pow(p / pk, -(g + 1.0) / (2.0 * g)) / (rk * sqrt(g * pk / rk));
}

int orc_godunov_pstar(double g, double rl, double ul, double pl, double rr, double ur, double pr, double* ps) {
    double al = sqrt(g * pl / rl), ar = sqrt(g * pr / rr);
    double du = ur - ul;
    /* Both pressure functions are finite for p above lo: a side with a
       negative (unphysical, reconstructed) pressure is on its shock branch,
       which needs p + B > 0. */
    double lo = 0.0;
    if (pl < 0) lo = fmax(lo, -pl * (g - 1.0) / (g + 1.0));
    if (pr < 0) lo = fmax(lo, -pr * (g - 1.0) / (g + 1.0));
    double floor_p = lo + 1e-12 * (fabs(pl) + fabs(pr));
    double p = 0.5 * (pl + pr) - 0.125 * du * (rl + rr) * (al + ar);
    if (!(p > floor_p)) p = 0.5 * (pl + pr);
    if (!(p > floor_p)) p = 2.0 * floor_p;
    for (int it = 0; it < 60; ++it) {
        double f = god_f(g, rl, pl, p) + god_f(g, rr, pr, p) + du;
        double d = god_df(g, rl, pl, p) + god_df(g, rr, pr, p);
        double pn = p - f / d;
        if (!(pn > floor_p)) pn = floor_p;
        double ch = 2.0 * fabs(pn - p) / (pn + p);
        p = pn;
        if (ch < 1e-14) { *ps = p; return 1; }
    }
    *ps = p;
    return 0;
}

static double godunov_flux(const orc_config* c, const double* UL, const double* UR, int a, double* flux) {
    const double g = c->gamma;
    vec3 fn = {a == 0 ? 1.0 : 0.0, a == 1 ? 1.0 : 0.0, a == 2 ? 1.0 : 0.0};
    double roL = UL[0], roR = UR[0];
    vec3 velL = {UL[1] / UL[0], UL[2] / UL[0], UL[3] / UL[0]};
    vec3 velR = {UR[1] / UR[0], UR[2] / UR[0], UR[3] / UR[0]};
    /* GetPressure (:17-25) */
    double pL = (g - 1.0) * roL * (UL[4] / roL - (velL.x * velL.x + velL.y * velL.y + velL.z * velL.z) / 2.0);
    double pR = (g - 1.0) * roR * (UR[4] / roR - (velR.x * velR.x + velR.y * velR.y + velR.z * velR.z) / 2.0);
    double uL = dot3(velL, fn), uR = dot3(velR, fn);
    /* ComputeStarVariables (:143-264) */
    double pStar;
    orc_godunov_pstar(g, roL, uL, pL, roR, uR, pR, &pStar);
    double uStar = 0.5 * (uL + uR) + 0.5 * (god_f(g, roR, pR, pStar) - god_f(g, roL, pL, pStar));
    double C = (g - 1.0) / (g + 1.0);
    double maxs = 0, roStarL, roStarR, SL = 0, SHL = 0, STL = 0, SR = 0, SHR = 0, STR = 0;
    int shockL, shockR;
    double pRatioL = pStar / pL, aL = sqrt(g * pL / roL);
    if (pStar > pL) {
        shockL = 1;
        roStarL = pRatioL + C;
        roStarL /= C * pRatioL + 1.0;
        roStarL *= roL;
        SL = sqrt((g + 1) * pRatioL / (2 * g) + (g - 1) / (2 * g));
        SL = uL - aL * SL;
        maxs = fmax(maxs, fabs(SL));
    } else {
        shockL = 0;
        roStarL = roL * pow(pRatioL, 1.0 / g);
        SHL = uL - aL;
        double aStarL = aL * pow(pRatioL, (g - 1) / (2 * g));
        STL = uStar - aStarL;
        maxs = fmax(maxs, fabs(SHL));
    }
    double pRatioR = pStar / pR, aR = sqrt(g * pR / roR);
    if (pStar > pR) {
        shockR = 1;
        roStarR = pRatioR + C;
        roStarR /= C * pRatioR + 1.0;
        roStarR *= roR;
        SR = sqrt((g + 1) * pRatioR / (2 * g) + (g - 1) / (2 * g));
        SR = uR + aR * SR;
        maxs = fmax(maxs, fabs(SR));
    } else {
        shockR = 0;
        roStarR = roR * pow(pRatioR, 1.0 / g);
        SHR = uR + aR;
        double aStarR = aR * pow(pRatioR, (g - 1) / (2 * g));
        STR = uStar + aStarR;
        maxs = fmax(maxs, fabs(SHR));
    }
    /* sampling at S = x/t = 0 (:299-393) */
    const double S = 0;
    double ro, u, p;
    vec3 vel;
    if (uStar >= S) {
        vel = velL;
        if (shockL) {
            if (SL >= S) { ro = roL; u = uL; p = pL; }
            else { ro = roStarL; u = uStar; p = pStar; }
        } else {
            if (SHL > S) { ro = roL; u = uL; p = pL; }
            else if (S > STL) { ro = roStarL; u = uStar; p = pStar; }
            else {
                double aL2 = sqrt(g * pL / roL);
                double CL = 2.0 / (g + 1) + (g - 1) * (uL - S) / ((g + 1) * aL2);
                double CLRo = pow(CL, 2.0 / (g - 1));
                double CLP = pow(CL, 2.0 * g / (g - 1));
                ro = CLRo * roL;
                u = aL2 + 0.5 * (g - 1) * uL + S;
                u *= 2 / (g + 1);
                p = CLP * pL;
            }
        }
    } else {
        vel = velR;
        if (shockR) {
            if (SR <= S) { ro = roR; u = uR; p = pR; }
            else { ro = roStarR; u = uStar; p = pStar; }
        } else {
            if (SHR < S) { ro = roR; u = uR; p = pR; }
            else if (S < STR) { ro = roStarR; u = uStar; p = pStar; }
            else {
                double aR2 = sqrt(g * pR / roR);
                double CR = 2.0 / (g + 1) - (g - 1) * (uR - S) / ((g + 1) * aR2);
                double CRRo = pow(CR, 2.0 / (g - 1));
                double CRP = pow(CR, 2.0 * g / (g - 1));
                ro = CRRo * roR;
                u = -aR2 + 0.5 * (g - 1) * uR + S;
                u *= 2 / (g + 1);
                p = CRP * pR;
            }
        }
    }
    /* face state and F(Uface) (:396-427, :28-46) */
    double vn0 = dot3(vel, fn);
    vec3 Vf = {vel.x + (u - vn0) * fn.x, vel.y + (u - vn0) * fn.y, vel.z + (u - vn0) * fn.z};
    double Uf[NV];
    Uf[0] = ro;
    Uf[1] = ro * Vf.x;
    Uf[2] = ro * Vf.y;
    Uf[3] = ro * Vf.z;
    Uf[4] = ro * (p / (ro * (g - 1.0)) + 0.5 * dot3(Vf, Vf));
    {
        double r = Uf[0];
        double vx = Uf[1] / r, vy = Uf[2] / r, vz = Uf[3] / r;
        double roE = Uf[4];
        double pp = (g - 1.0) * (roE - r * (vx * vx + vy * vy + vz * vz) / 2.0);
        double vn = vx * fn.x + vy * fn.y + vz * fn.z;
        flux[0] = r * vn;
        flux[1] = r * vn * vx + fn.x * pp;
        flux[2] = r * vn * vy + fn.y * pp;
        flux[3] = r * vn * vz + fn.z * pp;
        flux[4] = vn * (roE + pp);
    }
    return maxs;
}

static double riemann(const orc_config* c, const double* UL, const double* UR, int a, double* flux) {
    vec3 fn = {a == 0 ? 1.0 : 0.0, a == 1 ? 1.0 : 0.0, a == 2 ? 1.0 : 0.0};
    if (c->solver == ORC_RS_HLLC) return hllc_flux(c, UL, UR, a, flux);
    if (c->solver == ORC_RS_GODUNOV) return godunov_flux(c, UL, UR, a, flux);
    return roe_flux(c, UL, UR, fn, flux);
}


/* ------------------------------------------------------------------------ */
/* Viscous part, ExplicitRungeKuttaFVM.h:81-874                             */
/* ------------------------------------------------------------------------ */

/* Velocity component d of a cell's conserved values (VariablesTransition.h:18-36). */
static inline double vel(const double* V, int d) { return V[1 + d] / V[0]; }

static inline double* vgrad_of(orc_ctx* w, int cell, int d) { return w->vgrad + ((size_t)cell * 3 + d) * 3; }

static inline double det3(double a00, double a01, double a02, double a10, double a11, double a12, double a20,
                          double a21, double a22) {
    return a00 * (a11 * a22 - a12 * a21) - a01 * (a10 * a22 - a12 * a20) + a02 * (a10 * a21 - a11 * a20);
}

/* Least-squares gradient (GradientComputer::ExecuteByLeastSquares,
   GradientComputer.h:20-52): the g minimising |A g - rhs| with rows
   A_r = point - points_r (first nd components) and rhs_r = value - values_r.
   The reference solves it with Eigen 3.2.5's JacobiSVD; this restatement
   solves the normal equations (A^T A) g = A^T rhs by Cramer's rule (1x1 to
   3x3, well conditioned for these stencils), so it agrees with the reference
   to rounding, not bit for bit. */
static void ls_gradient(int nd, int m, const double (*A)[3], const double* rhs, double* g) {
    double M[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}}, b[3] = {0, 0, 0};
    for (int r = 0; r < m; ++r)
        for (int a = 0; a < nd; ++a) {
            b[a] += A[r][a] * rhs[r];
            for (int e = 0; e < nd; ++e) M[a][e] += A[r][a] * A[r][e];
        }
    g[0] = g[1] = g[2] = 0.0;
    if (nd == 1) {
        g[0] = b[0] / M[0][0];
    } else if (nd == 2) {
        const double det = M[0][0] * M[1][1] - M[0][1] * M[1][0];
        g[0] = (b[0] * M[1][1] - M[0][1] * b[1]) / det;
        g[1] = (M[0][0] * b[1] - b[0] * M[1][0]) / det;
    } else {
        const double det = det3(M[0][0], M[0][1], M[0][2], M[1][0], M[1][1], M[1][2], M[2][0], M[2][1], M[2][2]);
        g[0] = det3(b[0], M[0][1], M[0][2], b[1], M[1][1], M[1][2], b[2], M[2][1], M[2][2]) / det;
        g[1] = det3(M[0][0], b[0], M[0][2], M[1][0], b[1], M[1][2], M[2][0], b[2], M[2][2]) / det;
        g[2] = det3(M[0][0], M[0][1], b[0], M[1][0], M[1][1], b[1], M[2][0], M[2][1], b[2]) / det;
    }
}

/* Ghost-cell gradients beyond one boundary cell (ComputeDummyCellGradients,
   ExplicitRungeKuttaFVM.h:318-680): the least-squares gradient at the face
   centre from the face value (BCGeneral::getFaceValues, BCGeneral.h:90-94:
   the mean of the cell and its BC image) and the stencil of
   Stencil::InternalBorderStencil (Stencil.h:28-63) plus the ghost cell,
   extrapolated as 2 g_face - g_cell. */
static void dummy_gradient(orc_ctx* w, const double* U, int a, int side, int i, int j, int k) {
    const orc_config* c = w->c;
    const int nd = c->ndims;
    const double* X[3] = {w->x, w->y, w->z};
    const double* H[3] = {w->hx, w->hy, w->hz};
    int ix[3] = {i, j, k};
    const int inner = cidx(w, i, j, k);
    int gi[3] = {i, j, k};
    gi[a] += side ? 1 : -1;
    const int ghost = cidx(w, gi[0], gi[1], gi[2]);
    double fc[3] = {w->x[i], w->y[j], w->z[k]};
    fc[a] = side ? X[a][ix[a]] + 0.5 * H[a][ix[a]] : X[a][ix[a]] - 0.5 * H[a][ix[a]];
    const double* Vin = U + (size_t)inner * NV;
    vec3 n = {a == 0 ? (side ? 1.0 : -1.0) : 0.0, a == 1 ? (side ? 1.0 : -1.0) : 0.0,
              a == 2 ? (side ? 1.0 : -1.0) : 0.0};
    double du[NV], Vf[NV];
    bc_dummy_values(c, bc_entry(w, 2 * a + side, i, j, k), Vin, n, du);
    for (int v = 0; v < NV; ++v) Vf[v] = 0.5 * (Vin[v] + du[v]);
    /* stencil: the cell, its neighbours along the other active axes, the ghost */
    int st[7][3], m = 0;
    st[m][0] = i; st[m][1] = j; st[m][2] = k; ++m;
    for (int b = 0; b < nd; ++b) {
        if (b == a) continue;
        for (int sg = 1; sg >= -1; sg -= 2) {
            st[m][0] = i; st[m][1] = j; st[m][2] = k;
            st[m][b] += sg;
            ++m;
        }
    }
    st[m][0] = gi[0]; st[m][1] = gi[1]; st[m][2] = gi[2]; ++m;
    double A[7][3], rhs[7], g[3];
    for (int r = 0; r < m; ++r) {
        A[r][0] = fc[0] - w->x[st[r][0]];
        A[r][1] = fc[1] - w->y[st[r][1]];
        A[r][2] = fc[2] - w->z[st[r][2]];
    }
    for (int d = 0; d < 3; ++d) {
        const double value = Vf[1 + d] / Vf[0];
        for (int r = 0; r < m; ++r) rhs[r] = value - vel(U + (size_t)cidx(w, st[r][0], st[r][1], st[r][2]) * NV, d);
        ls_gradient(nd, m, (const double (*)[3])A, rhs, g);
        double* gg = vgrad_of(w, ghost, d);
        const double* gc = vgrad_of(w, inner, d);
        for (int e = 0; e < 3; ++e) gg[e] = 2.0 * g[e] - gc[e];
    }
}

/* ComputeVelocityGradients (ExplicitRungeKuttaFVM.h:81-134): central
   differences inside (Kernel::ComputeGradientNonUniformStructured,
   kernel.h:918-938), the periodic exchange of ExchangeGradients (:136-316) on
   one rank, then the ghost gradients of non-periodic sides. */
static void velocity_gradients(orc_ctx* w, const double* U) {
    const orc_config* c = w->c;
    const int nd = c->ndims;
    for (int k = w->kmin; k <= w->kmax; ++k)
        for (int j = w->jmin; j <= w->jmax; ++j)
            for (int i = w->imin; i <= w->imax; ++i) {
                const int id = cidx(w, i, j, k);
                for (int d = 0; d < 3; ++d) {
                    double* g = vgrad_of(w, id, d);
                    const double dux = vel(U + (size_t)cidx(w, i + 1, j, k) * NV, d) -
                                       vel(U + (size_t)cidx(w, i - 1, j, k) * NV, d);
                    g[0] = dux / (w->x[i + 1] - w->x[i - 1]);
                    g[1] = 0.0;
                    g[2] = 0.0;
                    if (nd > 1) {
                        const double duy = vel(U + (size_t)cidx(w, i, j + 1, k) * NV, d) -
                                           vel(U + (size_t)cidx(w, i, j - 1, k) * NV, d);
                        g[1] = duy / (w->y[j + 1] - w->y[j - 1]);
                    }
                    if (nd > 2) {
                        const double duz = vel(U + (size_t)cidx(w, i, j, k + 1) * NV, d) -
                                           vel(U + (size_t)cidx(w, i, j, k - 1) * NV, d);
                        g[2] = duz / (w->z[k + 1] - w->z[k - 1]);
                    }
                }
            }
    const int lo[3] = {w->imin, w->jmin, w->kmin}, hi[3] = {w->imax, w->jmax, w->kmax};
    for (int a = 0; a < nd; ++a) {
        /* transverse cells of the two boundary layers along a (interior range) */
        const int b1 = a == 0 ? 1 : 0, b2 = a == 2 ? 1 : 2;
        for (int p = lo[b1]; p <= hi[b1]; ++p)
            for (int q = lo[b2]; q <= hi[b2]; ++q) {
                int cl[3], ch[3];
                cl[a] = lo[a]; ch[a] = hi[a];
                cl[b1] = ch[b1] = p;
                cl[b2] = ch[b2] = q;
                if (c->periodic[a]) {
                    int gl[3] = {cl[0], cl[1], cl[2]}, gh[3] = {ch[0], ch[1], ch[2]};
                    gl[a] -= 1;
                    gh[a] += 1;
                    const int il = cidx(w, cl[0], cl[1], cl[2]), ih = cidx(w, ch[0], ch[1], ch[2]);
                    const int jl = cidx(w, gl[0], gl[1], gl[2]), jh = cidx(w, gh[0], gh[1], gh[2]);
                    memcpy(vgrad_of(w, jh, 0), vgrad_of(w, il, 0), sizeof(double) * 9);
                    memcpy(vgrad_of(w, jl, 0), vgrad_of(w, ih, 0), sizeof(double) * 9);
                }
            }
    }
    for (int a = 0; a < nd; ++a) {
        if (c->periodic[a]) continue;
        const int b1 = a == 0 ? 1 : 0, b2 = a == 2 ? 1 : 2;
        for (int p = lo[b1]; p <= hi[b1]; ++p)
            for (int q = lo[b2]; q <= hi[b2]; ++q) {
                int cl[3], ch[3];
                cl[a] = lo[a]; ch[a] = hi[a];
                cl[b1] = ch[b1] = p;
                cl[b2] = ch[b2] = q;
                dummy_gradient(w, U, a, 0, cl[0], cl[1], cl[2]);
                dummy_gradient(w, U, a, 1, ch[0], ch[1], ch[2]);
            }
    }
}

/* Viscous flux of the face between cells cm and cp along axis a, s the index
   of cp along a (ComputeViscousFluxes, ExplicitRungeKuttaFVM.h:683-874): face
   velocity gradients from the two cells' gradients weighted by the cell
   sizes, the normal derivatives by the two-point difference, the stress
   tensor with second viscosity -2/3 mu, and the work of the stresses. */
static void viscous_flux(orc_ctx* w, int a, int cm, int cp, int s, double* fv) {
    const orc_config* c = w->c;
    const double* X = a == 0 ? w->x : (a == 1 ? w->y : w->z);
    const double* H = a == 0 ? w->hx : (a == 1 ? w->hy : w->hz);
    const double* UL = w->U + (size_t)cm * NV;
    const double* UR = w->U + (size_t)cp * NV;
    const double dx = X[s] - X[s - 1];
    const double l = H[s - 1] / dx;
    const double r = H[s] / dx;
    double D[3][3], uu[3];
    for (int d = 0; d < 3; ++d) {
        const double* gL = vgrad_of(w, cm, d);
        const double* gR = vgrad_of(w, cp, d);
        for (int e = 0; e < 3; ++e) D[d][e] = 0.5 * (r * gL[e] + l * gR[e]);
        D[d][a] = (vel(UR, d) - vel(UL, d)) / dx;
    }
    for (int d = 0; d < 3; ++d) uu[d] = 0.5 * (l * vel(UR, d) + r * vel(UL, d));
    const double mu = c->viscosity;
    const double sv = (-2.0 / 3.0) * mu;
    const double td = sv * (D[0][0] + D[1][1] + D[2][2]);
    fv[0] = 0.0;
    if (a == 0) {
        const double txx = td + 2 * mu * D[0][0];
        const double txy = mu * (D[0][1] + D[1][0]);
        const double txz = mu * (D[0][2] + D[2][0]);
        fv[1] = txx; fv[2] = txy; fv[3] = txz;
        fv[4] = uu[0] * txx + uu[1] * txy + uu[2] * txz;
    } else if (a == 1) {
        const double tyy = td + 2 * mu * D[1][1];
        const double txy = mu * (D[0][1] + D[1][0]);
        const double tyz = mu * (D[1][2] + D[2][1]);
        fv[1] = txy; fv[2] = tyy; fv[3] = tyz;
        fv[4] = uu[0] * txy + uu[1] * tyy + uu[2] * tyz;
    } else {
        const double tzz = td + 2 * mu * D[2][2];
        const double txz = mu * (D[0][2] + D[2][0]);
        const double tyz = mu * (D[1][2] + D[2][1]);
        fv[1] = txz; fv[2] = tyz; fv[3] = tzz;
        fv[4] = uu[0] * txz + uu[1] * tyz + uu[2] * tzz;
    }
}

/* ------------------------------------------------------------------------ */
/* Residual, ExplicitRungeKuttaFVM.h:1150-1424                              */
/* ------------------------------------------------------------------------ */

/* One line of faces along axis a through the transverse cell (t1,t2). */
static void residual_line(orc_ctx* w, int a, int p, int q) {
    const orc_config* c = w->c;
    int lo = a == 0 ? w->imin : (a == 1 ? w->jmin : w->kmin);
    int hi = a == 0 ? w->imax : (a == 1 ? w->jmax : w->kmax);
    const double* hh = a == 0 ? w->hx : (a == 1 ? w->hy : w->hz);
    double fS;
    int i, j, k;
    /* (p,q) are (j,k) for x faces, (i,k) for y faces, (i,j) for z faces. */
    if (a == 0) {
        j = p; k = q;
        fS = 0;
        if (c->ndims == 1) fS = 1.0;
        if (c->ndims == 2) fS = w->hy[j];
        if (c->ndims == 3) fS = w->hy[j] * w->hz[k];
    } else if (a == 1) {
        i = p; k = q;
        fS = w->hx[i];
        if (c->ndims == 3) fS = w->hx[i] * w->hz[k];
    } else {
        i = p; j = q;
        fS = w->hx[i] * w->hy[j];
    }
    double fl[NV] = {0, 0, 0, 0, 0}, fr[NV], UL[NV], UR[NV];
    vec3 fn = {a == 0 ? 1.0 : 0.0, a == 1 ? 1.0 : 0.0, a == 2 ? 1.0 : 0.0};
    for (int s = lo; s <= hi + 1; ++s) {
        if (a == 0) i = s; else if (a == 1) j = s; else k = s;
        int cm = a == 0 ? cidx(w, s - 1, j, k) : (a == 1 ? cidx(w, i, s - 1, k) : cidx(w, i, j, s - 1));
        int cp = cidx(w, i, j, k);
        double hl = 0.5 * hh[s - 1];
        double hr = -0.5 * hh[s];
        if (s == lo && !c->periodic[a]) {
            sample(w, cp, a, hr, UR);
            bc_dummy_values(c, bc_entry(w, 2 * a, i, j, k), UR, fn, UL);
        } else if (s == hi + 1 && !c->periodic[a]) {
            sample(w, cm, a, hl, UL);
            bc_dummy_values(c, bc_entry(w, 2 * a + 1, i, j, k), UL, fn, UR);
        } else {
            sample(w, cm, a, hl, UL);
            sample(w, cp, a, hr, UR);
        }
        double lam = riemann(c, UL, UR, a, fr);
        double fvisc[NV] = {0, 0, 0, 0, 0};
        if (c->viscous) viscous_flux(w, a, cm, cp, s, fvisc);
        for (int v = 0; v < NV; ++v) fr[v] -= fvisc[v];
        w->spectral[cp] += fS * lam;
        if (s > lo) {
            for (int v = 0; v < NV; ++v) w->resid[(size_t)cm * NV + v] -= (fr[v] - fl[v]) * fS;
            w->spectral[cm] += fS * lam;
            /* viscous spectral-radius term, added whatever IsViscousFlow is
               (:1239-1248); Prandtl number 1 */
            double roFace = sqrt(UL[0] * UR[0]);
            double t1 = 4.0 / (3.0 * roFace), t2 = c->gamma / roFace;
            double vsr = (t1 < t2) ? t2 : t1;
            vsr *= c->viscosity / 1.0;
            vsr *= fS * fS;
            vsr /= w->vol[cm];
            w->spectral[cm] += vsr;
        }
        for (int v = 0; v < NV; ++v) fl[v] = fr[v];
    }
}

static void compute_residual(orc_ctx* w) {
    const orc_config* c = w->c;
    memset(w->spectral, 0, sizeof(double) * w->ncells);
    memset(w->resid, 0, sizeof(double) * (size_t)w->ncells * NV);
    int nj = w->jmax - w->jmin + 1, nk = w->kmax - w->kmin + 1, ni = w->imax - w->imin + 1;
    /* I step (k outer, j inner); lines are independent */
#pragma omp parallel for schedule(static)
    for (int t = 0; t < nj * nk; ++t) residual_line(w, 0, w->jmin + t % nj, w->kmin + t / nj);
    if (c->ndims > 1) {
#pragma omp parallel for schedule(static)
        for (int t = 0; t < ni * nk; ++t) residual_line(w, 1, w->imin + t % ni, w->kmin + t / ni);
    }
    if (c->ndims > 2) {
#pragma omp parallel for schedule(static)
        for (int t = 0; t < ni * nj; ++t) residual_line(w, 2, w->imin + t % ni, w->jmin + t / ni);
    }
}

/* Source terms after the face fluxes (ExplicitRungeKuttaFVM.h:1421-1423):
   Kernel::ProcessExternalForces (kernel.h:941-965) and
   ProcessExternalAcceleration (:966-989), on the state the step started from. */
static void add_sources(orc_ctx* w, const double* U) {
    const orc_config* c = w->c;
    if (!c->external_force && !c->uniform_acceleration) return;
    for (int i = w->imin; i <= w->imax; ++i)
        for (int j = w->jmin; j <= w->jmax; ++j)
            for (int k = w->kmin; k <= w->kmax; ++k) {
                int idx = cidx(w, i, j, k);
                double volume = w->hx[i] * w->hy[j] * w->hz[k];
                const double* V = U + (size_t)idx * NV;
                vec3 vel = {V[1] / V[0], V[2] / V[0], V[3] / V[0]};
                double* R = w->resid + (size_t)idx * NV;
                if (c->external_force) {
                    vec3 sg = {c->sigma[0], c->sigma[1], c->sigma[2]};
                    R[1] += volume * sg.x;
                    R[2] += volume * sg.y;
                    R[3] += volume * sg.z;
                    R[4] += dot3(sg, vel) * volume;
                }
            }
    if (!c->uniform_acceleration) return;
    for (int i = w->imin; i <= w->imax; ++i)
        for (int j = w->jmin; j <= w->jmax; ++j)
            for (int k = w->kmin; k <= w->kmax; ++k) {
                int idx = cidx(w, i, j, k);
                double volume = w->hx[i] * w->hy[j] * w->hz[k];
                const double* V = U + (size_t)idx * NV;
                vec3 vel = {V[1] / V[0], V[2] / V[0], V[3] / V[0]};
                double ro = V[0];
                vec3 g = {c->acceleration[0], c->acceleration[1], c->acceleration[2]};
                vec3 rg = {ro * g.x, ro * g.y, ro * g.z};
                double* R = w->resid + (size_t)idx * NV;
                R[1] += ro * volume * g.x;
                R[2] += ro * volume * g.y;
                R[3] += ro * volume * g.z;
                R[4] += dot3(rg, vel) * volume;
            }
}

/* ------------------------------------------------------------------------ */
/* Step: ExplicitRungeKuttaFVM::IterationStep, :1440-1491                   */
/* ------------------------------------------------------------------------ */

static void iteration_step(orc_ctx* w, double* U, orc_step_info* info) {
    const orc_config* c = w->c;
    fill_ghosts(w, U);
    if (c->recon != ORC_RECON_PWC) {
        int ni = w->imax - w->imin + 1, nj = w->jmax - w->jmin + 1, nk = w->kmax - w->kmin + 1;
#pragma omp parallel for schedule(static)
        for (int t = 0; t < ni * nj * nk; ++t) {
            int i = w->imin + t % ni, j = w->jmin + (t / ni) % nj, k = w->kmin + t / (ni * nj);
            reconstruct_cell(w, U, i, j, k);
        }
    } else {
        for (int k = w->kmin; k <= w->kmax; ++k)
            for (int j = w->jmin; j <= w->jmax; ++j)
                for (int i = w->imin; i <= w->imax; ++i) reconstruct_cell(w, U, i, j, k);
    }
    exchange_recon(w);
    w->U = U;
    if (c->viscous) velocity_gradients(w, U);
    compute_residual(w);
    add_sources(w, U);

    /* ComputeTimeStep, :1427-1437: (volumes / spectralRadius).min() * CFL,
       min in libstdc++'s __valarray_min order. */
    double m = w->vol[0] / w->spectral[0];
    for (int t = 1; t < w->ncells; ++t) {
        double r = w->vol[t] / w->spectral[t];
        if (r < m) m = r;
    }
    double dt = m * c->cfl;
    if ((c->save_solution_time > 0) && (info->next_solution_time < info->time + dt)) dt = info->next_solution_time - info->time;
    if ((c->save_slice_time > 0) && (info->next_slice_time < info->time + dt)) dt = info->next_slice_time - info->time;
    info->dt = dt;

    /* UpdateSolution, kernel.h:319-331 */
#pragma omp parallel for schedule(static)
    for (int t = 0; t < w->ncells; ++t)
        for (int v = 0; v < NV; ++v) U[(size_t)t * NV + v] += dt * (w->resid[(size_t)t * NV + v] / w->vol[t]);
    /* residual norms: (volumes * abs(R)).sum() on a valarray expression,
       which libstdc++ accumulates from the last element down */
    for (int v = 0; v < NV; ++v) {
        int t = w->ncells - 1;
        double s = w->vol[t] * fabs(w->resid[(size_t)t * NV + v]);
        while (t != 0) { --t; s += w->vol[t] * fabs(w->resid[(size_t)t * NV + v]); }
        info->residual[v] = s;
    }
    info->time += dt;
    info->iteration++;
}

int orc_advance(const orc_config* c, double* values, int n_steps, orc_step_info* info) {
#ifdef _OPENMP
    if (c->threads > 0) omp_set_num_threads(c->threads);
#endif
    orc_ctx w;
    memset(&w, 0, sizeof w);
    w.c = c;
    orc_dims(c, &w.nxa, &w.nya, &w.nza);
    w.ncells = w.nxa * w.nya * w.nza;
    w.gx = 1; w.gy = c->ndims > 1; w.gz = c->ndims > 2;
    w.imin = 1; w.imax = c->nx;
    w.jmin = w.gy; w.jmax = c->ndims > 1 ? c->ny : 0;
    w.kmin = w.gz; w.kmax = c->ndims > 2 ? c->nz : 0;
    w.x = malloc(sizeof(double) * w.nxa); w.hx = malloc(sizeof(double) * w.nxa);
    w.y = malloc(sizeof(double) * w.nya); w.hy = malloc(sizeof(double) * w.nya);
    w.z = malloc(sizeof(double) * w.nza); w.hz = malloc(sizeof(double) * w.nza);
    orc_grid(c, w.x, w.hx, w.y, w.hy, w.z, w.hz);
    w.vol = malloc(sizeof(double) * w.ncells);
    w.spectral = malloc(sizeof(double) * w.ncells);
    w.resid = malloc(sizeof(double) * (size_t)w.ncells * NV);
    w.rvals = calloc((size_t)w.ncells * NV, sizeof(double));
    w.rgrad = calloc((size_t)w.ncells * 3 * NV, sizeof(double));
    w.rlim = calloc((size_t)w.ncells * NV, sizeof(double));
    if (c->viscous) w.vgrad = calloc((size_t)w.ncells * 9, sizeof(double));
    if (!w.vol || !w.spectral || !w.resid || !w.rvals || !w.rgrad || !w.rlim || (c->viscous && !w.vgrad)) return 1;
    for (int k = 0; k < w.nza; ++k)
        for (int j = 0; j < w.nya; ++j)
            for (int i = 0; i < w.nxa; ++i) w.vol[cidx(&w, i, j, k)] = w.hx[i] * w.hy[j] * w.hz[k];
    if (c->recon == ORC_RECON_LINEAR2_LIM && c->limiter == ORC_LIM_VENKAT) {
        /* limVenkatar::SendCellInfo, Limiters.h:93-96, K = 5 (Constants.h:11) */
        w.eps2 = malloc(sizeof(double) * w.ncells);
        for (int k = 0; k < w.nza; ++k)
            for (int j = 0; j < w.nya; ++j)
                for (int i = 0; i < w.nxa; ++i) {
                    double dx = pow(w.hx[i] * w.hy[j] * w.hz[k], 1.0 / c->ndims);
                    w.eps2[cidx(&w, i, j, k)] = pow(5.0 * dx, 3.0);
                }
    }
    if (n_steps >= 0) {
        for (int s = 0; s < n_steps; ++s) iteration_step(&w, values, info);
    } else {
        /* Kernel::Run, kernel.h:1701-1850 */
        for (;;) {
            iteration_step(&w, values, info);
            if ((c->save_solution_time > 0) && (info->next_solution_time == info->time))
                info->next_solution_time += c->save_solution_time;
            if ((c->save_slice_time > 0) && (info->next_slice_time == info->time))
                info->next_slice_time += c->save_slice_time;
            if (info->iteration == c->max_iteration) break;
            if (info->time >= c->max_time) break;
        }
    }
    free(w.x); free(w.hx); free(w.y); free(w.hy); free(w.z); free(w.hz);
    free(w.vol); free(w.spectral); free(w.resid); free(w.rvals); free(w.rgrad); free(w.rlim); free(w.eps2);
    free(w.vgrad);
    return 0;
}

/* ------------------------------------------------------------------------ */
/* Exact Riemann solver (Toro ch. 4) for a stiffened gas                    */
/* ------------------------------------------------------------------------ */

static void pressure_fn(double g, double pinf, double p, double rk, double pk, double ck, double* f, double* fd) {
    double pp = p + pinf, pkk = pk + pinf;
    if (p <= pk) { /* rarefaction */
        double pr = pp / pkk;
        *f = 2.0 * ck / (g - 1.0) * (pow(pr, (g - 1.0) / (2.0 * g)) - 1.0);
        *fd = (1.0 / (rk * ck)) * pow(pr, -(g + 1.0) / (2.0 * g));
    } else { /* shock */
        double A = 2.0 / ((g + 1.0) * rk);
        double B = (g - 1.0) / (g + 1.0) * pkk;
        double qrt = sqrt(A / (pp + B));
        *f = (p - pk) * qrt;
        *fd = (1.0 - 0.5 * (p - pk) / (B + pp)) * qrt;
    }
}

int orc_exact_riemann(double g, double pinf, double rl, double ul, double pl, double rr, double ur, double pr,
                      double s, double* rho, double* u, double* p) {
    double cl = sqrt(g * (pl + pinf) / rl), cr = sqrt(g * (pr + pinf) / rr);
    /* two-rarefaction initial guess in p + p_inf, Toro eq. 4.46 */
    double z = (g - 1.0) / (2.0 * g);
    double num = cl + cr - 0.5 * (g - 1.0) * (ur - ul);
    double den = cl / pow(pl + pinf, z) + cr / pow(pr + pinf, z);
    double ps = pow(num / den, 1.0 / z) - pinf;
    if (!(ps > -pinf)) ps = 0.5 * (pl + pr);
    int it = 0;
    for (; it < 200; ++it) {
        double fl, fdl, fr, fdr;
        pressure_fn(g, pinf, ps, rl, pl, cl, &fl, &fdl);
        pressure_fn(g, pinf, ps, rr, pr, cr, &fr, &fdr);
        double pn = ps - (fl + fr + ur - ul) / (fdl + fdr);
        if (pn + pinf <= 0.0) pn = 0.5 * (ps + pinf) - pinf; /* keep p + p_inf positive */
        double ch = 2.0 * fabs(pn - ps) / fabs(pn + ps + 2.0 * pinf);
        ps = pn;
        if (ch < 1e-15) break;
    }
    double fl, fdl, fr, fdr;
    pressure_fn(g, pinf, ps, rl, pl, cl, &fl, &fdl);
    pressure_fn(g, pinf, ps, rr, pr, cr, &fr, &fdr);
    double us = 0.5 * (ul + ur) + 0.5 * (fr - fl);
    double gm = (g - 1.0) / (g + 1.0);
    double PS = ps + pinf, PL = pl + pinf, PR = pr + pinf;
    if (s <= us) {
        if (ps > pl) { /* left shock */
            double sh = ul - cl * sqrt((g + 1.0) / (2.0 * g) * PS / PL + (g - 1.0) / (2.0 * g));
            if (s <= sh) { *rho = rl; *u = ul; *p = pl; }
            else { *rho = rl * (PS / PL + gm) / (gm * PS / PL + 1.0); *u = us; *p = ps; }
        } else { /* left rarefaction */
            double shl = ul - cl;
            double cs = cl * pow(PS / PL, z);
            double stl = us - cs;
            if (s <= shl) { *rho = rl; *u = ul; *p = pl; }
            else if (s >= stl) { *rho = rl * pow(PS / PL, 1.0 / g); *u = us; *p = ps; }
            else {
                double cc = 2.0 / (g + 1.0) + gm / cl * (ul - s);
                *rho = rl * pow(cc, 2.0 / (g - 1.0));
                *u = 2.0 / (g + 1.0) * (cl + 0.5 * (g - 1.0) * ul + s);
                *p = PL * pow(cc, 2.0 * g / (g - 1.0)) - pinf;
            }
        }
    } else {
        if (ps > pr) { /* right shock */
            double sh = ur + cr * sqrt((g + 1.0) / (2.0 * g) * PS / PR + (g - 1.0) / (2.0 * g));
            if (s >= sh) { *rho = rr; *u = ur; *p = pr; }
            else { *rho = rr * (PS / PR + gm) / (gm * PS / PR + 1.0); *u = us; *p = ps; }
        } else { /* right rarefaction */
            double shr = ur + cr;
            double cs = cr * pow(PS / PR, z);
            double str = us + cs;
            if (s >= shr) { *rho = rr; *u = ur; *p = pr; }
            else if (s <= str) { *rho = rr * pow(PS / PR, 1.0 / g); *u = us; *p = ps; }
            else {
                double cc = 2.0 / (g + 1.0) - gm / cr * (ur - s);
                *rho = rr * pow(cc, 2.0 / (g - 1.0));
                *u = 2.0 / (g + 1.0) * (-cr + 0.5 * (g - 1.0) * ur + s);
                *p = PR * pow(cc, 2.0 * g / (g - 1.0)) - pinf;
            }
        }
    }
    return it;
}

/* ------------------------------------------------------------------------ */
/* Synthetic initial states of the benchmark scenarios                      */
/* ------------------------------------------------------------------------ */
/* The benchmark inputs are this project's own seeded scenarios (the reference
   has no benchmark inputs).  Restated here so the CPU legs of the bench build
   their inputs without the product library; tests/test_capi_host.py checks
   this restatement bit for bit against ts_fill_scenario.  The scenarios are
   point-sampled at the cell centres, as Kernel::SetInitialConditions does
   (kernel.h:125-146), with a counter-based hash of (seed, i, j, k). */

double orc_hash_uniform(unsigned long long seed, long long i, long long j, long long k) {
    unsigned long long z = seed * 0x9E3779B97F4A7C15ULL + (unsigned long long)i * 0xBF58476D1CE4E5B9ULL +
                           (unsigned long long)j * 0x94D049BB133111EBULL + (unsigned long long)k * 0xD6E8FEB86659FD39ULL;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
    z ^= z >> 31;
    return (double)(z >> 11) * 0x1.0p-53;
}

int orc_fill_scenario(const orc_config* c, int scenario, unsigned long long seed, const double* prm, int n_params,
                      double* values) {
    static const int need[4] = {7, 5, 5, 16};
    if (scenario < 0 || scenario > 3 || n_params < need[scenario]) return 1;
    int nxa, nya, nza;
    orc_dims(c, &nxa, &nya, &nza);
    double* x = (double*)malloc(sizeof(double) * (size_t)nxa);
    double* hx = (double*)malloc(sizeof(double) * (size_t)nxa);
    double* y = (double*)malloc(sizeof(double) * (size_t)nya);
    double* hy = (double*)malloc(sizeof(double) * (size_t)nya);
    double* z = (double*)malloc(sizeof(double) * (size_t)nza);
    double* hz = (double*)malloc(sizeof(double) * (size_t)nza);
    if (!x || !hx || !y || !hy || !z || !hz) return 2;
    orc_grid(c, x, hx, y, hy, z, hz);
    const int nd = c->ndims;
    const int nx = c->nx, ny = nd > 1 ? c->ny : 1, nz = nd > 2 ? c->nz : 1;
    const double gm1 = c->gamma - 1.0;
    const double pshift = c->eos == ORC_EOS_STIFFENED ? c->gamma * c->p_inf : 0.0;
#pragma omp parallel for schedule(static) if (c->threads != 1)
    for (int k = 0; k < nz; ++k)
        for (int j = 0; j < ny; ++j)
            for (int i = 0; i < nx; ++i) {
                double* o = values + 5 * (((size_t)k * ny + j) * nx + i);
                const double xc = x[i + 1];
                const double yc = nd > 1 ? y[j + 1] : 0.0;
                const double zc = nd > 2 ? z[k + 1] : 0.0;
                double rho = 1.0, u = 0.0, v = 0.0, w = 0.0, p = 1.0;
                if (scenario == 0) {          /* shock tube: x0, rhoL, uL, pL, rhoR, uR, pR */
                    if (xc > prm[0]) { rho = prm[4]; u = prm[5]; p = prm[6]; }
                    else { rho = prm[1]; u = prm[2]; p = prm[3]; }
                } else if (scenario == 1) {   /* shear layer: rho_in, rho_out, u, p, noise */
                    const int inner = fabs(yc - 0.5 * c->length[1]) < 0.25 * c->length[1];
                    rho = inner ? prm[0] : prm[1];
                    u = inner ? prm[2] : -prm[2];
                    p = prm[3];
                    v = prm[4] * (2.0 * orc_hash_uniform(seed, i, j, k) - 1.0);
                } else if (scenario == 2) {   /* blast: rho, p_out, p_in, radius, noise */
                    const double dx = xc - 0.5 * c->length[0];
                    const double dy = nd > 1 ? yc - 0.5 * c->length[1] : 0.0;
                    const double dz = nd > 2 ? zc - 0.5 * c->length[2] : 0.0;
                    rho = prm[0] * (1.0 + prm[4] * (2.0 * orc_hash_uniform(seed, i, j, k) - 1.0));
                    p = (dx * dx + dy * dy + dz * dz < prm[3] * prm[3]) ? prm[2] : prm[1];
                } else {                      /* quadrants: 4 x (rho, u, v, p) for ++, -+, --, +- */
                    const int right = xc > 0.5 * c->length[0];
                    const int top = nd > 1 ? yc > 0.5 * c->length[1] : 1;
                    const int q = top ? (right ? 0 : 1) : (right ? 3 : 2);
                    rho = prm[4 * q + 0]; u = prm[4 * q + 1]; v = prm[4 * q + 2]; p = prm[4 * q + 3];
                }
                o[0] = rho;
                o[1] = rho * u;
                o[2] = rho * v;
                o[3] = rho * w;
                o[4] = (p + pshift) / gm1 + 0.5 * rho * (u * u + v * v + w * w);
            }
    free(x); free(hx); free(y); free(hy); free(z); free(hz);
    return 0;
}
