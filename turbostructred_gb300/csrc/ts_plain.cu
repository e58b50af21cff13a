// Plain FP64 path: the drop-in for ExplicitRungeKuttaFVM<R>::IterationStep
// (src/Methods/ExplicitRungeKuttaFVM.h:1440-1491) on one GB300.
//
// This translation unit is compiled with --fmad=false and IEEE division and
// square root, and every expression keeps the reference's operation order, so
// results match the reference's FP64 CPU path bit for bit (up to the sign of
// exact zeros: products with the zero components of axis normals, which the
// reference evaluates, are dropped here).
//
// One step is six launches on the handle's stream:
//   k_ghost<A>   ghost layers per axis: periodic copy or boundary condition
//                (Kernel::ExchangeValues + ComputeDummyCellValues, kernel.h:334-915)
//   k_recon      per-cell slopes and limiter (ComputeSolutionReconstruction, :879-925)
//   k_flux<A>    one kernel per face direction: face states, EOS, Riemann flux
//                and max eigenvalue (ComputeResidual face loops, :1182-1419)
//   k_dt         spectral radius per cell, V/SR, warp-shuffle min, last block
//                finalises dt (ComputeTimeStep, :1427-1437)
//   k_update     flux divergence fused with the stage update
//                (residual accumulation :1232 + Kernel::UpdateSolution, kernel.h:319-331)
//   k_finish     time/iteration and the Kernel::Run termination rules
// FP64 is scarce on GB300 (about 2 FMA/clk/SM), so this path is compute-bound;
// the layout and launches are chosen for coalescing, not for bandwidth.
#include <cuda_runtime.h>

#include "ts_plain.h"

namespace ts {

namespace {

__device__ __forceinline__ long long vidx(const Layout& L, int v) { return (long long)v * L.plane; }

// ---------------------------------------------------------------------------
// Boundary conditions (BCGeneral.h:186-268) for a normal sgn*e_A; `side` is
// the BC table entry (the domain side, or the kind a marker selected).
// ---------------------------------------------------------------------------
__device__ __forceinline__ void bc_values(const Phys& ph, int side, int A, double sgn, const double in[NV],
                                          double out[NV]) {
    const int t = ph.bc.type[side];
#pragma unroll
    for (int v = 0; v < NV; ++v) out[v] = in[v];
    if (t == TS_BC_SYMMETRY) {
        // rVinNormal = (n.rVin) n ; res -= 2 rVinNormal (BCGeneral.h:214-226)
        const double m = in[1 + A];
        const double s = sgn * m;
        const double rn = s * sgn;
        out[1 + A] = m - 2.0 * rn;
    } else if (t == TS_BC_WALL) {
        out[1] = in[1] * (-1.0);
        out[2] = in[2] * (-1.0);
        out[3] = in[3] * (-1.0);
    } else if (t == TS_BC_MOVING_WALL) {
        const double rho = in[0];
        const double ux = in[1] / rho, uy = in[2] / rho, uz = in[3] / rho;
        const double rhoe = in[4] - 0.5 * rho * (ux * ux + uy * uy + uz * uz);
        const double dx = 2.0 * ph.bc.vel[side][0] - ux;
        const double dy = 2.0 * ph.bc.vel[side][1] - uy;
        const double dz = 2.0 * ph.bc.vel[side][2] - uz;
        out[1] = rho * dx;
        out[2] = rho * dy;
        out[3] = rho * dz;
        out[4] = rhoe + 0.5 * rho * (dx * dx + dy * dy + dz * dz);
    } else if (t == TS_BC_SUBSONIC_INLET) {
        const double r = ph.bc.density[side];
        const double vx = ph.bc.vel[side][0], vy = ph.bc.vel[side][1], vz = ph.bc.vel[side][2];
        out[0] = r;
        out[1] = r * vx;
        out[2] = r * vy;
        out[3] = r * vz;
        double eint = ph.bc.pstatic[side] / (ph.gamma - 1);
        if (ph.eos == TS_EOS_STIFFENED_GAS) eint = eint + ph.gamma * ph.p_inf / (ph.gamma - 1);
        out[4] = eint + 0.5 * r * (vx * vx + vy * vy + vz * vz);
    }
    // Natural and SubsonicOutlet copy the inner state (BCGeneral.h:200-211).
}

// ---------------------------------------------------------------------------
// Riemann solvers
// ---------------------------------------------------------------------------
__device__ __forceinline__ double pressure(const Phys& ph, double ro, double vx, double vy, double vz, double roE) {
    double p = (ph.gamma - 1.0) * (roE - ro * (vx * vx + vy * vy + vz * vz) / 2.0);
    if (ph.eos == TS_EOS_STIFFENED_GAS) p = p - ph.gamma * ph.p_inf;
    return p;
}

// F(U).e_A (RoeSolverPerfectGasEOS.h:41-58).
template <int A>
__device__ __forceinline__ void phys_flux(const Phys& ph, const double U[NV], double res[NV]) {
    const double ro = U[0];
    const double vel[3] = {U[1] / ro, U[2] / ro, U[3] / ro};
    const double roE = U[4];
    const double p = pressure(ph, ro, vel[0], vel[1], vel[2], roE);
    const double vn = vel[A];
    const double rvn = ro * vn;
    res[0] = rvn;
#pragma unroll
    for (int b = 0; b < 3; ++b) res[1 + b] = (b == A) ? rvn * vel[b] + p : rvn * vel[b];
    res[4] = vn * (roE + p);
}

__device__ __forceinline__ double harten(double z, double eps) {
    z = fabs(z);
    if (z < eps) z = ((z * z) / eps + eps) * 0.5;
    return z;
}

// RoeSolverPerfectGasEOS::ComputeFlux (RoeSolverPerfectGasEOS.h:74-160) with
// fn = e_A; dn = 1 so dn*c = c and 1/(dn*dn) = 1 exactly.
template <int A>
__device__ double roe_flux(const Phys& ph, const double UL[NV], const double UR[NV], double flux[NV]) {
    const double g = ph.gamma;
    double FL[NV], FR[NV];
    phys_flux<A>(ph, UL, FL);
    phys_flux<A>(ph, UR, FR);
#pragma unroll
    for (int i = 0; i < NV; ++i) flux[i] = FL[i] + FR[i];
    const double ro_l = UL[0], ro_r = UR[0];
    const double vl[3] = {UL[1] / ro_l, UL[2] / ro_l, UL[3] / ro_l};
    const double vr[3] = {UR[1] / ro_r, UR[2] / ro_r, UR[3] / ro_r};
    const double e_l = UL[4] / ro_l, e_r = UR[4] / ro_r;
    double k = 0.5 * (vl[0] * vl[0] + vl[1] * vl[1] + vl[2] * vl[2]);
    double h_l = (e_l - k) * g + k;
    k = 0.5 * (vr[0] * vr[0] + vr[1] * vr[1] + vr[2] * vr[2]);
    double h_r = (e_r - k) * g + k;
    if (ph.eos == TS_EOS_STIFFENED_GAS) {
        h_l = h_l - g * ph.p_inf / ro_l;
        h_r = h_r - g * ph.p_inf / ro_r;
    }
    const double sl = sqrt(ro_l), sr = sqrt(ro_r);
    const double ql = sl / (sl + sr);
    const double qr = sr / (sl + sr);
    const double vel[3] = {ql * vl[0] + qr * vr[0], ql * vl[1] + qr * vr[1], ql * vl[2] + qr * vr[2]};
    const double h = ql * h_l + qr * h_r;
    const double phi2 = 0.5 * (g - 1) * (vel[0] * vel[0] + vel[1] * vel[1] + vel[2] * vel[2]);
    const double c = sqrt((g - 1) * h - phi2);
    const double uw = vel[A];
    const double eig_max = fabs(uw) + c;
    const double he = ph.eps * eig_max;
    const double AA1 = harten(uw, he);
    const double AA3 = harten(uw + c, he);
    const double AA4 = harten(uw - c, he);
    const double Eig1 = AA1;
    const double Eiga = (AA3 - AA4) * 0.5 / c;
    const double Eigb = (AA3 + AA4) * 0.5 - AA1;
    const double R1 = phi2 * ro_r - (g - 1) * ro_r * ((vel[0] * vr[0] + vel[1] * vr[1] + vel[2] * vr[2]) - e_r);
    const double D1 = ro_r * (vr[A] - vel[A]);
    const double R2 = phi2 * ro_l - (g - 1) * ro_l * ((vel[0] * vl[0] + vel[1] * vl[1] + vel[2] * vl[2]) - e_l);
    const double D2 = ro_l * (vl[A] - vel[A]);
    const double C2 = 1.0 / (c * c);
    // Qa = (0, e_A, uw), Qb = (1, vel, h); terms multiplying a zero Qa entry
    // are exact zeros and are left out.
    {
        const double t = Eig1 * UL[0] + Eiga * D2 + Eigb * (R2 * C2) - Eig1 * UR[0] - Eiga * D1 - Eigb * (R1 * C2);
        flux[0] = (flux[0] + t) * 0.5;
    }
#pragma unroll
    for (int b = 0; b < 3; ++b) {
        double t;
        if (b == A)
            t = Eig1 * UL[1 + b] + Eiga * (R2 + D2 * vel[b]) + Eigb * (R2 * vel[b] * C2 + D2) - Eig1 * UR[1 + b] -
                Eiga * (R1 + D1 * vel[b]) - Eigb * (R1 * vel[b] * C2 + D1);
        else
            t = Eig1 * UL[1 + b] + Eiga * (D2 * vel[b]) + Eigb * (R2 * vel[b] * C2) - Eig1 * UR[1 + b] -
                Eiga * (D1 * vel[b]) - Eigb * (R1 * vel[b] * C2);
        flux[1 + b] = (flux[1 + b] + t) * 0.5;
    }
    {
        const double t = Eig1 * UL[4] + Eiga * (R2 * uw + D2 * h) + Eigb * (R2 * h * C2 + D2 * uw) - Eig1 * UR[4] -
                         Eiga * (R1 * uw + D1 * h) - Eigb * (R1 * h * C2 + D1 * uw);
        flux[4] = (flux[4] + t) * 0.5;
    }
    return eig_max;
}

// HLLC (Toro ch. 10.4) with Einfeldt-type speeds from Roe averages; same
// operation order as the oracle's restatement.  Not in the reference.
template <int A>
__device__ double hllc_flux(const Phys& ph, const double UL[NV], const double UR[NV], double flux[NV]) {
    const double g = ph.gamma;
    const double pinf = ph.eos == TS_EOS_STIFFENED_GAS ? ph.p_inf : 0.0;
    const int m = 1 + A;
    const double rl = UL[0], rr = UR[0];
    const double ul = UL[m] / rl, ur = UR[m] / rr;
    const double vlx = UL[1] / rl, vly = UL[2] / rl, vlz = UL[3] / rl;
    const double vrx = UR[1] / rr, vry = UR[2] / rr, vrz = UR[3] / rr;
    const double pl = pressure(ph, rl, vlx, vly, vlz, UL[4]);
    const double pr = pressure(ph, rr, vrx, vry, vrz, UR[4]);
    const double cl = sqrt(g * (pl + pinf) / rl);
    const double cr = sqrt(g * (pr + pinf) / rr);
    const double hl = (UL[4] + pl) / rl;
    const double hr = (UR[4] + pr) / rr;
    const double sl = sqrt(rl), sr = sqrt(rr);
    const double wl = sl / (sl + sr), wr = sr / (sl + sr);
    const double ut = wl * ul + wr * ur;
    const double vtx = wl * vlx + wr * vrx, vty = wl * vly + wr * vry, vtz = wl * vlz + wr * vrz;
    const double ht = wl * hl + wr * hr;
    const double ct = sqrt((g - 1) * (ht - 0.5 * (vtx * vtx + vty * vty + vtz * vtz)));
    const double SL = fmin(ul - cl, ut - ct);
    const double SR = fmax(ur + cr, ut + ct);
    const double lam = fmax(fabs(SL), fabs(SR));
    const double ml = rl * (SL - ul), mr = rr * (SR - ur);
    const double sstar = (pr - pl + ul * ml - ur * mr) / (ml - mr);
    if (SL >= 0.0) {
        phys_flux<A>(ph, UL, flux);
    } else if (SR <= 0.0) {
        phys_flux<A>(ph, UR, flux);
    } else if (sstar >= 0.0) {
        double F[NV], us[NV];
        phys_flux<A>(ph, UL, F);
        const double coef = ml / (SL - sstar);
        us[0] = coef;
        us[1] = coef * vlx; us[2] = coef * vly; us[3] = coef * vlz;
        us[m] = coef * sstar;
        us[4] = coef * (UL[4] / rl + (sstar - ul) * (sstar + pl / ml));
#pragma unroll
        for (int v = 0; v < NV; ++v) flux[v] = F[v] + SL * (us[v] - UL[v]);
    } else {
        double F[NV], us[NV];
        phys_flux<A>(ph, UR, F);
        const double coef = mr / (SR - sstar);
        us[0] = coef;
        us[1] = coef * vrx; us[2] = coef * vry; us[3] = coef * vrz;
        us[m] = coef * sstar;
        us[4] = coef * (UR[4] / rr + (sstar - ur) * (sstar + pr / mr));
#pragma unroll
        for (int v = 0; v < NV; ++v) flux[v] = F[v] + SR * (us[v] - UR[v]);
    }
    return lam;
}

// Exact (Godunov) flux, GodunovSolverPerfectGasEOS::ComputeFlux
// (GodunovSolverPerfectGasEOS.h:266-430), ideal gas.  p* solves
// fL(p) + fR(p) + (uR - uL) = 0 (f1/f2, :56-96).  The reference minimises the
// square of that function with alglib's Levenberg-Marquardt (stopping at a
// gradient below 1e-10, :143-187); here a bounded Newton-Raphson iteration
// on the root with the analytic derivative (Toro, sec. 4.3.1) from the
// primitive-variable guess (Toro eq. 4.47), to a relative change below 1e-14.
// Everything after p* keeps the reference's steps and operation order.
__device__ __forceinline__ double god_f(double g, double rk, double pk, double p) {
    double res;
    if (p > pk) {
        const double A = 2 / ((g + 1.0) * rk);
        const double B = pk * (g - 1.0) / (g + 1.0);
        res = (p - pk) * sqrt(A / (p + B));
    } else {
        const double a = sqrt(g * pk / rk);
        res = pow(p / pk, (g - 1.0) / (2 * g)) - 1.0;
        res *= 2 * a / (g - 1.0);
    }
    return res;
}

__device__ __forceinline__ double god_df(double g, double rk, double pk, double p) {
    if (p > pk) {
        const double A = 2 / ((g + 1.0) * rk);
        const double B = pk * (g - 1.0) / (g + 1.0);
        return sqrt(A / (B + p)) * (1.0 - (p - pk) / (2.0 * (B + p)));
    }
    return pow(p / pk, -(g + 1.0) / (2.0 * g)) / (rk * sqrt(g * pk / rk));
}

// Returns false when 60 iterations do not converge (the caller flags it).
__device__ bool god_pstar(double g, double rl, double ul, double pl, double rr, double ur, double pr, double& ps) {
    const double al = sqrt(g * pl / rl), ar = sqrt(g * pr / rr);
    const double du = ur - ul;
    // both pressure functions are finite above lo (a side with a negative
    // reconstructed pressure is on its shock branch, which needs p + B > 0)
    double lo = 0.0;
    if (pl < 0) lo = fmax(lo, -pl * (g - 1.0) / (g + 1.0));
    if (pr < 0) lo = fmax(lo, -pr * (g - 1.0) / (g + 1.0));
    const double floor_p = lo + 1e-12 * (fabs(pl) + fabs(pr));
    double p = 0.5 * (pl + pr) - 0.125 * du * (rl + rr) * (al + ar);
    if (!(p > floor_p)) p = 0.5 * (pl + pr);
    if (!(p > floor_p)) p = 2.0 * floor_p;
    for (int it = 0; it < 60; ++it) {
        const double f = god_f(g, rl, pl, p) + god_f(g, rr, pr, p) + du;
        const double d = god_df(g, rl, pl, p) + god_df(g, rr, pr, p);
        double pn = p - f / d;
        if (!(pn > floor_p)) pn = floor_p;
        const double ch = 2.0 * fabs(pn - p) / (pn + p);
        p = pn;
        if (ch < 1e-14) { ps = p; return true; }
    }
    ps = p;
    return false;
}

template <int A>
__device__ double godunov_flux(const Phys& ph, const double UL[NV], const double UR[NV], double flux[NV],
                               bool& converged) {
    const double g = ph.gamma;
    const double roL = UL[0], roR = UR[0];
    const double velL[3] = {UL[1] / UL[0], UL[2] / UL[0], UL[3] / UL[0]};
    const double velR[3] = {UR[1] / UR[0], UR[2] / UR[0], UR[3] / UR[0]};
    // GetPressure (:17-25)
    const double pL =
        (g - 1.0) * roL * (UL[4] / roL - (velL[0] * velL[0] + velL[1] * velL[1] + velL[2] * velL[2]) / 2.0);
    const double pR =
        (g - 1.0) * roR * (UR[4] / roR - (velR[0] * velR[0] + velR[1] * velR[1] + velR[2] * velR[2]) / 2.0);
    const double uL = velL[A], uR = velR[A];
    // ComputeStarVariables (:143-264)
    double pStar;
    converged = god_pstar(g, roL, uL, pL, roR, uR, pR, pStar);
    const double uStar = 0.5 * (uL + uR) + 0.5 * (god_f(g, roR, pR, pStar) - god_f(g, roL, pL, pStar));
    const double C = (g - 1.0) / (g + 1.0);
    double maxs = 0, roStarL, roStarR, SL = 0, SHL = 0, STL = 0, SR = 0, SHR = 0, STR = 0;
    bool shockL, shockR;
    const double pRatioL = pStar / pL, aL = sqrt(g * pL / roL);
    if (pStar > pL) {
        shockL = true;
        roStarL = pRatioL + C;
        roStarL /= C * pRatioL + 1.0;
        roStarL *= roL;
        SL = sqrt((g + 1) * pRatioL / (2 * g) + (g - 1) / (2 * g));
        SL = uL - aL * SL;
        maxs = fmax(maxs, fabs(SL));
    } else {
        shockL = false;
        roStarL = roL * pow(pRatioL, 1.0 / g);
        SHL = uL - aL;
        const double aStarL = aL * pow(pRatioL, (g - 1) / (2 * g));
        STL = uStar - aStarL;
        maxs = fmax(maxs, fabs(SHL));
    }
    const double pRatioR = pStar / pR, aR = sqrt(g * pR / roR);
    if (pStar > pR) {
        shockR = true;
        roStarR = pRatioR + C;
        roStarR /= C * pRatioR + 1.0;
        roStarR *= roR;
        SR = sqrt((g + 1) * pRatioR / (2 * g) + (g - 1) / (2 * g));
        SR = uR + aR * SR;
        maxs = fmax(maxs, fabs(SR));
    } else {
        shockR = false;
        roStarR = roR * pow(pRatioR, 1.0 / g);
        SHR = uR + aR;
        const double aStarR = aR * pow(pRatioR, (g - 1) / (2 * g));
        STR = uStar + aStarR;
        maxs = fmax(maxs, fabs(SHR));
    }
    // sampling at S = x/t = 0 (:299-393)
    const double S = 0;
    double ro, u, p;
    const double* vel;
    if (uStar >= S) {
        vel = velL;
        if (shockL) {
            if (SL >= S) { ro = roL; u = uL; p = pL; }
            else { ro = roStarL; u = uStar; p = pStar; }
        } else if (SHL > S) {
            ro = roL; u = uL; p = pL;
        } else if (S > STL) {
            ro = roStarL; u = uStar; p = pStar;
        } else {
            const double aL2 = sqrt(g * pL / roL);
            const double CL = 2.0 / (g + 1) + (g - 1) * (uL - S) / ((g + 1) * aL2);
            const double CLRo = pow(CL, 2.0 / (g - 1));
            const double CLP = pow(CL, 2.0 * g / (g - 1));
            ro = CLRo * roL;
            u = aL2 + 0.5 * (g - 1) * uL + S;
            u *= 2 / (g + 1);
            p = CLP * pL;
        }
    } else {
        vel = velR;
        if (shockR) {
            if (SR <= S) { ro = roR; u = uR; p = pR; }
            else { ro = roStarR; u = uStar; p = pStar; }
        } else if (SHR < S) {
            ro = roR; u = uR; p = pR;
        } else if (S < STR) {
            ro = roStarR; u = uStar; p = pStar;
        } else {
            const double aR2 = sqrt(g * pR / roR);
            const double CR = 2.0 / (g + 1) - (g - 1) * (uR - S) / ((g + 1) * aR2);
            const double CRRo = pow(CR, 2.0 / (g - 1));
            const double CRP = pow(CR, 2.0 * g / (g - 1));
            ro = CRRo * roR;
            u = -aR2 + 0.5 * (g - 1) * uR + S;
            u *= 2 / (g + 1);
            p = CRP * pR;
        }
    }
    // face state (:396-404): normal velocity u, tangential from the upwind side
    double Vf[3];
#pragma unroll
    for (int b = 0; b < 3; ++b) Vf[b] = (b == A) ? vel[b] + (u - vel[A]) : vel[b];
    double Uf[NV];
    Uf[0] = ro;
    Uf[1] = ro * Vf[0];
    Uf[2] = ro * Vf[1];
    Uf[3] = ro * Vf[2];
    Uf[4] = ro * (p / (ro * (g - 1.0)) + 0.5 * (Vf[0] * Vf[0] + Vf[1] * Vf[1] + Vf[2] * Vf[2]));
    // F(Uface, n) (:28-46)
    {
        const double r = Uf[0];
        const double vx = Uf[1] / r, vy = Uf[2] / r, vz = Uf[3] / r;
        const double roE = Uf[4];
        const double pp = (g - 1.0) * (roE - r * (vx * vx + vy * vy + vz * vz) / 2.0);
        const double v3[3] = {vx, vy, vz};
        const double vn = v3[A];
        flux[0] = r * vn;
#pragma unroll
        for (int b = 0; b < 3; ++b) flux[1 + b] = (b == A) ? r * vn * v3[b] + pp : r * vn * v3[b];
        flux[4] = vn * (roE + pp);
    }
    return maxs;
}

// ---------------------------------------------------------------------------
// Kernels
// ---------------------------------------------------------------------------

// Transverse (p,q) -> (i,j,k) for a line along axis A.
template <int A>
__device__ __forceinline__ void line_cell(int p, int q, int s, int& i, int& j, int& k) {
    if (A == 0) { i = s; j = p; k = q; }
    else if (A == 1) { i = p; j = s; k = q; }
    else { i = p; j = q; k = s; }
}

template <int A>
__global__ void k_ghost(PlainBufs b, Phys ph) {
    if (b.ctl->stop_req) return;
    const Layout& L = b.L;
    const int n1 = (A == 0) ? L.ny : L.nx;
    const int n2 = (A == 2) ? L.ny : L.nz;
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n1 * n2) return;
    const int p = t % n1, q = t / n1;
    int i, j, k;
    line_cell<A>(p, q, 0, i, j, k);
    const long long c0 = L.at(i, j, k);
    const long long st = L.stride(A);
    const int n = L.n(A);
    double* U = b.U;
    if (ph.periodic[A]) {
#pragma unroll
        for (int v = 0; v < NV; ++v) {
            double* u = U + vidx(L, v) + c0;
            u[-1 * st] = u[(long long)(n - 1) * st];
            u[(long long)n * st] = u[0];
            u[-2 * st] = u[(long long)(n - 2) * st];
            u[(long long)(n + 1) * st] = u[st];
        }
        return;
    }
    double in[NV], out[NV];
    // the BC of this row's boundary face on each side (its marker, if the
    // side is position-dependent: the same one for both ghost layers)
    const int idl = bc_id(ph.bc.mark, 2 * A, face_index(2 * A, i, j, k, L.nx, L.ny));
    const int idr = bc_id(ph.bc.mark, 2 * A + 1, face_index(2 * A + 1, i, j, k, L.nx, L.ny));
    // left side ghosts mirror cells 0 and 1; right side mirror n-1 and n-2
    // (ComputeDummyCellValues, kernel.h:731-765); faceNormalL on both sides.
    for (int layer = 1; layer <= GHOST; ++layer) {
#pragma unroll
        for (int v = 0; v < NV; ++v) in[v] = U[vidx(L, v) + c0 + (long long)(layer - 1) * st];
        bc_values(ph, idl, A, -1.0, in, out);
#pragma unroll
        for (int v = 0; v < NV; ++v) U[vidx(L, v) + c0 - (long long)layer * st] = out[v];
#pragma unroll
        for (int v = 0; v < NV; ++v) in[v] = U[vidx(L, v) + c0 + (long long)(n - layer) * st];
        bc_values(ph, idr, A, -1.0, in, out);
#pragma unroll
        for (int v = 0; v < NV; ++v) U[vidx(L, v) + c0 + (long long)(n - 1 + layer) * st] = out[v];
    }
}


// ---------------------------------------------------------------------------
// Viscous part (ExplicitRungeKuttaFVM.h:81-874), FP64 like the rest of the path
// ---------------------------------------------------------------------------

// Velocity component d of cell c (VariablesTransition.h:18-36).
__device__ __forceinline__ double velc(const PlainBufs& b, long long c, int d) {
    return b.U[vidx(b.L, 1 + d) + c] / b.U[vidx(b.L, 0) + c];
}

__device__ __forceinline__ double vgrad(const PlainBufs& b, long long c, int d, int e) {
    return b.VG[vidx(b.L, 3 * d + e) + c];
}

// Central-difference gradients of the three velocity components in every
// interior cell (Kernel::ComputeGradientNonUniformStructured, kernel.h:918-938).
__global__ void k_vgrad(PlainBufs b, Phys ph) {
    if (b.ctl->stop_req) return;
    const Layout& L = b.L;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y, k = blockIdx.z;
    if (i >= L.nx) return;
    const long long c = L.at(i, j, k);
    const int nd = ph.nd;
    for (int d = 0; d < 3; ++d) {
        const double dux = velc(b, c + L.stride(0), d) - velc(b, c - L.stride(0), d);
        const double gx = dux / (b.cx[0][i + 1 + L.gx] - b.cx[0][i - 1 + L.gx]);
        double gy = 0.0, gz = 0.0;
        if (nd > 1) {
            const double duy = velc(b, c + L.stride(1), d) - velc(b, c - L.stride(1), d);
            gy = duy / (b.cx[1][j + 1 + L.gy] - b.cx[1][j - 1 + L.gy]);
        }
        if (nd > 2) {
            const double duz = velc(b, c + L.stride(2), d) - velc(b, c - L.stride(2), d);
            gz = duz / (b.cx[2][k + 1 + L.gz] - b.cx[2][k - 1 + L.gz]);
        }
        b.VG[vidx(L, 3 * d) + c] = gx;
        b.VG[vidx(L, 3 * d + 1) + c] = gy;
        b.VG[vidx(L, 3 * d + 2) + c] = gz;
    }
}

__device__ __forceinline__ double det3(double a00, double a01, double a02, double a10, double a11, double a12,
                                       double a20, double a21, double a22) {
    return a00 * (a11 * a22 - a12 * a21) - a01 * (a10 * a22 - a12 * a20) + a02 * (a10 * a21 - a11 * a20);
}

// Least-squares gradient of GradientComputer::ExecuteByLeastSquares
// (GradientComputer.h:20-52) by the normal equations (A^T A) g = A^T rhs and
// Cramer's rule; the reference uses Eigen's JacobiSVD, which agrees to
// rounding.
__device__ void ls_gradient(int nd, int m, const double (*A)[3], const double* rhs, double* g) {
    double M[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}}, bb[3] = {0, 0, 0};
    for (int r = 0; r < m; ++r)
        for (int a = 0; a < nd; ++a) {
            bb[a] += A[r][a] * rhs[r];
            for (int e = 0; e < nd; ++e) M[a][e] += A[r][a] * A[r][e];
        }
    g[0] = g[1] = g[2] = 0.0;
    if (nd == 1) {
        g[0] = bb[0] / M[0][0];
    } else if (nd == 2) {
        const double det = M[0][0] * M[1][1] - M[0][1] * M[1][0];
        g[0] = (bb[0] * M[1][1] - M[0][1] * bb[1]) / det;
        g[1] = (M[0][0] * bb[1] - bb[0] * M[1][0]) / det;
    } else {
        const double det = det3(M[0][0], M[0][1], M[0][2], M[1][0], M[1][1], M[1][2], M[2][0], M[2][1], M[2][2]);
        g[0] = det3(bb[0], M[0][1], M[0][2], bb[1], M[1][1], M[1][2], bb[2], M[2][1], M[2][2]) / det;
        g[1] = det3(M[0][0], bb[0], M[0][2], M[1][0], bb[1], M[1][2], M[2][0], bb[2], M[2][2]) / det;
        g[2] = det3(M[0][0], M[0][1], bb[0], M[1][0], M[1][1], bb[1], M[2][0], M[2][1], bb[2]) / det;
    }
}

// Ghost gradients beyond boundary cell (i, j, k) on side `side` of axis A
// (ComputeDummyCellGradients, ExplicitRungeKuttaFVM.h:318-680): least-squares
// gradient at the face centre from the face value (mean of the cell and its
// BC image, BCGeneral::getFaceValues) and the stencil of
// Stencil::InternalBorderStencil plus the ghost cell; ghost = 2 g_face - g_cell.
template <int A>
__device__ void dummy_gradient(const PlainBufs& b, const Phys& ph, int side, int i, int j, int k) {
    const Layout& L = b.L;
    const int nd = ph.nd;
    const int ix[3] = {i, j, k};
    const int go[3] = {L.gx, L.gy, L.gz};
    const long long inner = L.at(i, j, k);
    const long long ghost = inner + (side ? L.stride(A) : -L.stride(A));
    double fc[3] = {b.cx[0][i + L.gx], b.cx[1][j + L.gy], b.cx[2][k + L.gz]};
    const double xa = b.cx[A][ix[A] + go[A]], ha = b.ch[A][ix[A] + go[A]];
    fc[A] = side ? xa + 0.5 * ha : xa - 0.5 * ha;
    double Vin[NV], du[NV], Vf[NV];
#pragma unroll
    for (int v = 0; v < NV; ++v) Vin[v] = b.U[vidx(L, v) + inner];
    bc_values(ph, bc_id(ph.bc.mark, 2 * A + side, face_index(2 * A + side, i, j, k, L.nx, L.ny)), A,
              side ? 1.0 : -1.0, Vin, du);
#pragma unroll
    for (int v = 0; v < NV; ++v) Vf[v] = 0.5 * (Vin[v] + du[v]);
    // stencil: the cell, its neighbours along the other active axes (+ then -), the ghost
    int st[7][3];
    int m = 0;
    st[m][0] = i; st[m][1] = j; st[m][2] = k; ++m;
    for (int a = 0; a < nd; ++a) {
        if (a == A) continue;
        for (int sg = 1; sg >= -1; sg -= 2) {
            st[m][0] = i; st[m][1] = j; st[m][2] = k;
            st[m][a] += sg;
            ++m;
        }
    }
    st[m][0] = i; st[m][1] = j; st[m][2] = k;
    st[m][A] += side ? 1 : -1;
    ++m;
    double Am[7][3], rhs[7], g[3];
    for (int r = 0; r < m; ++r) {
        Am[r][0] = fc[0] - b.cx[0][st[r][0] + L.gx];
        Am[r][1] = fc[1] - b.cx[1][st[r][1] + L.gy];
        Am[r][2] = fc[2] - b.cx[2][st[r][2] + L.gz];
    }
    for (int d = 0; d < 3; ++d) {
        const double value = Vf[1 + d] / Vf[0];
        for (int r = 0; r < m; ++r) rhs[r] = value - velc(b, L.at(st[r][0], st[r][1], st[r][2]), d);
        ls_gradient(nd, m, Am, rhs, g);
        for (int e = 0; e < 3; ++e) b.VG[vidx(L, 3 * d + e) + ghost] = 2.0 * g[e] - vgrad(b, inner, d, e);
    }
}

// Gradients of the first ghost layer along axis A: the opposite interior
// cell's on a periodic axis (ExchangeGradients on one rank,
// ExplicitRungeKuttaFVM.h:136-316), least squares otherwise.
template <int A>
__global__ void k_vgrad_bc(PlainBufs b, Phys ph) {
    if (b.ctl->stop_req) return;
    const Layout& L = b.L;
    const int n1 = (A == 0) ? L.ny : L.nx;
    const int n2 = (A == 2) ? L.ny : L.nz;
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n1 * n2) return;
    const int p = t % n1, q = t / n1;
    int i, j, k;
    line_cell<A>(p, q, 0, i, j, k);
    const long long c0 = L.at(i, j, k);
    const long long st = L.stride(A);
    const int n = L.n(A);
    if (ph.periodic[A]) {
        for (int pl = 0; pl < 9; ++pl) {
            double* g = b.VG + vidx(L, pl) + c0;
            g[(long long)n * st] = g[0];
            g[-st] = g[(long long)(n - 1) * st];
        }
        return;
    }
    int ih = i, jh = j, kh = k;
    if (A == 0) ih = n - 1; else if (A == 1) jh = n - 1; else kh = n - 1;
    dummy_gradient<A>(b, ph, 0, i, j, k);
    dummy_gradient<A>(b, ph, 1, ih, jh, kh);
}

// Viscous flux of the face along axis A between cells cl and cr, s the
// index of cr along A (ComputeViscousFluxes, ExplicitRungeKuttaFVM.h:683-874).
template <int A>
__device__ void visc_flux(const PlainBufs& b, const Phys& ph, long long cl, long long cr, int s, double fv[NV]) {
    const Layout& L = b.L;
    const int g0 = (A == 0) ? L.gx : (A == 1 ? L.gy : L.gz);
    const double dx = b.cx[A][s + g0] - b.cx[A][s - 1 + g0];
    const double l = b.ch[A][s - 1 + g0] / dx;
    const double r = b.ch[A][s + g0] / dx;
    double D[3][3], uu[3];
    for (int d = 0; d < 3; ++d) {
        for (int e = 0; e < 3; ++e) D[d][e] = 0.5 * (r * vgrad(b, cl, d, e) + l * vgrad(b, cr, d, e));
        D[d][A] = (velc(b, cr, d) - velc(b, cl, d)) / dx;
    }
    for (int d = 0; d < 3; ++d) uu[d] = 0.5 * (l * velc(b, cr, d) + r * velc(b, cl, d));
    const double mu = ph.visc;
    const double sv = (-2.0 / 3.0) * mu;
    const double td = sv * (D[0][0] + D[1][1] + D[2][2]);
    fv[0] = 0.0;
    if (A == 0) {
        const double txx = td + 2 * mu * D[0][0];
        const double txy = mu * (D[0][1] + D[1][0]);
        const double txz = mu * (D[0][2] + D[2][0]);
        fv[1] = txx; fv[2] = txy; fv[3] = txz;
        fv[4] = uu[0] * txx + uu[1] * txy + uu[2] * txz;
    } else if (A == 1) {
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

// Venkatakrishnan l-function (Limiters.h:102-115).
// Comparisons of doubles on the integer pipe.  GB300 executes FP64 at about
// two operations per clock per SM, and half of k_recon's FP64-pipe
// instructions were comparisons (measured with ncu).  dkey is monotone in the
// value and gives -0 and +0 the same key, so dkey(a) < dkey(b) is exactly
// a < b, and the sign tests below are exactly x > 0 and x < 0, for every
// non-NaN a, b, x (a NaN only arises in a run whose health flags stop it).
__device__ __forceinline__ long long dkey(double x) {
    const long long b = __double_as_longlong(x);
    return b < 0 ? (b ^ 0x7FFFFFFFFFFFFFFFLL) + 1 : b;
}
__device__ __forceinline__ bool dlt(double a, double b) { return dkey(a) < dkey(b); }
__device__ __forceinline__ bool dpos(double x) { return __double_as_longlong(x) > 0; }
__device__ __forceinline__ bool dneg(double x) {
    const long long b = __double_as_longlong(x);
    return b < 0 && b != (long long)0x8000000000000000ULL;
}
// |a| < |b|: the magnitudes' bit patterns order like their values
__device__ __forceinline__ bool dabs_lt(double a, double b) {
    return (__double_as_longlong(a) & 0x7FFFFFFFFFFFFFFFLL) < (__double_as_longlong(b) & 0x7FFFFFFFFFFFFFFFLL);
}

__device__ __forceinline__ double venkat(double um, double ui, double d2, double umax, double umin, double eps2) {
    const double un = 0.5 * (umax - umin);
    um /= un;
    ui /= un;
    d2 /= un;
    const double dm = um - ui;
    return ((dm * dm + eps2) + 2 * d2 * dm) / (dm * dm + 2 * d2 * d2 + dm * d2 + eps2);
}

// Per interior cell: slopes (Linear2PointsStencil.h:147-178 or
// ENO2PointsStencil.h:202-239) and, for Linear2psLim, the limiter
// (Linear2psLim.h:305-374, Limiters.h:28-119).
__global__ void k_recon(PlainBufs b, Phys ph) {
    if (b.ctl->stop_req) return;
    const Layout& L = b.L;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y, k = blockIdx.z;
    if (i >= L.nx) return;
    const int nd = ph.nd;
    const long long c = L.at(i, j, k);
    const int ix[3] = {i, j, k};
    double val[NV], nb[6][NV], g[3][NV];
#pragma unroll
    for (int v = 0; v < NV; ++v) val[v] = b.U[vidx(L, v) + c];
    for (int a = 0; a < nd; ++a) {
        const long long st = L.stride(a);
#pragma unroll
        for (int v = 0; v < NV; ++v) {
            nb[2 * a][v] = b.U[vidx(L, v) + c - st];
            nb[2 * a + 1][v] = b.U[vidx(L, v) + c + st];
        }
    }
    for (int a = 0; a < nd; ++a) {
        const double* X = b.cx[a];
        const int g0 = (a == 0) ? L.gx : (a == 1 ? L.gy : L.gz);
        const double xm = X[ix[a] - 1 + g0], xc = X[ix[a] + g0], xp = X[ix[a] + 1 + g0];
        if (ph.recon == TS_RECON_ENO2_2POINTS) {
#pragma unroll
            for (int v = 0; v < NV; ++v) {
                const double gl = (val[v] - nb[2 * a][v]) / (xc - xm);
                const double gr = (nb[2 * a + 1][v] - val[v]) / (xp - xc);
                g[a][v] = dabs_lt(gl, gr) ? gl : gr;
            }
        } else {
            const double d = xp - xm;
#pragma unroll
            for (int v = 0; v < NV; ++v) g[a][v] = (nb[2 * a + 1][v] - nb[2 * a][v]) / d;
        }
#pragma unroll
        for (int v = 0; v < NV; ++v) b.G[vidx(L, a * NV + v) + c] = g[a][v];
    }
    if (ph.recon != TS_RECON_LINEAR_2POINTS_LIMITED) return;

    // Projections (SampleSolution(+-h/2) - vals) to the 2*nDim faces.
    double hcell[3];
    hcell[0] = b.ch[0][i + L.gx];
    hcell[1] = b.ch[1][j + L.gy];
    hcell[2] = b.ch[2][k + L.gz];
    const double eps2 = b.eps2 ? b.eps2[c] : 0.0;
#pragma unroll
    for (int v = 0; v < NV; ++v) {
        double umax = val[v], umin = val[v];
        long long kmax = dkey(umax), kmin = kmax;
        for (int f = 0; f < 2 * nd; ++f) {
            const double vn = nb[f][v];
            const long long kv = dkey(vn);
            if (kmax < kv) { umax = vn; kmax = kv; }
            if (kmin > kv) { umin = vn; kmin = kv; }
        }
        double lmin = 1.0;
        if (!dlt(umax - umin, 3.0 * 2.2250738585072014e-308)) {
            for (int f = 0; f < 2 * nd; ++f) {
                const int a = f >> 1;
                const double s = (f & 1) ? 0.5 * hcell[a] : -0.5 * hcell[a];
                const double d2 = (val[v] + g[a][v] * s) - val[v];
                double lv = 1.0;
                if (ph.limiter == TS_LIM_VENKATAKRISHNAN) {
                    if (dpos(d2)) lv = venkat(umax, val[v], d2, umax, umin, eps2);
                    if (dneg(d2)) lv = venkat(umin, val[v], d2, umax, umin, eps2);
                } else {
                    // r = (umax - u) / d2 (or umin) only matters below 1: where
                    // the exact quotient is >= 1, the rounded one is too (RN is
                    // monotone and 1 is representable), so lv = 1 without the
                    // division, bit for bit
                    if (dpos(d2)) {
                        const double a = umax - val[v];
                        if (dlt(a, d2)) { const double r = a / d2; lv = dlt(r, 1.0) ? r : 1.0; }
                    }
                    if (dneg(d2)) {
                        const double a = umin - val[v];
                        if (dlt(d2, a)) { const double r = a / d2; lv = dlt(r, 1.0) ? r : 1.0; }
                    }
                }
                if (dlt(lv, lmin)) lmin = lv;
            }
        }
        b.Lim[vidx(L, v) + c] = lmin;
    }
}

__device__ __forceinline__ double face_area(const PlainBufs& b, int nd, int a, int i, int j, int k) {
    const Layout& L = b.L;
    const double hx = b.ch[0][i + L.gx], hy = b.ch[1][j + L.gy], hz = b.ch[2][k + L.gz];
    if (a == 0) return nd == 1 ? 1.0 : (nd == 2 ? hy : hy * hz);
    if (a == 1) return nd == 2 ? hx : hx * hz;
    return hx * hy;
}

// Face-centred sample of a cell's reconstruction (SampleSolution).
__device__ __forceinline__ void sample(const PlainBufs& b, const Phys& ph, long long c, int a, double s,
                                       double out[NV]) {
    const Layout& L = b.L;
#pragma unroll
    for (int v = 0; v < NV; ++v) out[v] = b.U[vidx(L, v) + c];
    if (ph.recon == TS_RECON_PIECEWISE_CONSTANT) return;
    if (ph.recon == TS_RECON_LINEAR_2POINTS_LIMITED) {
#pragma unroll
        for (int v = 0; v < NV; ++v) out[v] = out[v] + b.Lim[vidx(L, v) + c] * (b.G[vidx(L, a * NV + v) + c] * s);
    } else {
#pragma unroll
        for (int v = 0; v < NV; ++v) out[v] = out[v] + b.G[vidx(L, a * NV + v) + c] * s;
    }
}

// One face per thread along axis A; faces are stored at their right cell.
template <int A>
__global__ void k_flux(PlainBufs b, Phys ph) {
    if (b.ctl->stop_req) return;
    const Layout& L = b.L;
    int i, j, k;
    if (A == 0) {
        // nx + 1 faces per row: one flat index over all rows, so that no
        // block holds a row's last face alone
        const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
        const long long row = L.nx + 1;
        if (t >= row * L.ny * L.nz) return;
        i = (int)(t % row);
        const long long r = t / row;
        j = (int)(r % L.ny);
        k = (int)(r / L.ny);
    } else {
        i = blockIdx.x * blockDim.x + threadIdx.x;
        j = blockIdx.y;
        k = blockIdx.z;
        if (i >= L.nx) return;
    }
    const int s = (A == 0) ? i : (A == 1 ? j : k);
    const int n = L.n(A);
    const long long st = L.stride(A);
    const long long cf = L.at(i, j, k);  // cell to the right of the face
    const double* H = b.ch[A];
    const int g0 = (A == 0) ? L.gx : (A == 1 ? L.gy : L.gz);
    double UL[NV], UR[NV];
    if (s == 0 && !ph.periodic[A]) {
        sample(b, ph, cf, A, -0.5 * H[s + g0], UR);
        bc_values(ph, bc_id(ph.bc.mark, 2 * A, face_index(2 * A, i, j, k, L.nx, L.ny)), A, 1.0, UR, UL);
    } else if (s == n && !ph.periodic[A]) {
        sample(b, ph, cf - st, A, 0.5 * H[s - 1 + g0], UL);
        bc_values(ph, bc_id(ph.bc.mark, 2 * A + 1, face_index(2 * A + 1, i, j, k, L.nx, L.ny)), A, 1.0, UL, UR);
    } else {
        // A ghost reconstruction on a periodic axis is the opposite interior
        // cell's object sampled with the ghost's own h (ExchangeReconstructions).
        const long long cl = (s == 0) ? cf + (long long)(n - 1) * st : cf - st;
        const long long cr = (s == n) ? cf - (long long)n * st : cf;
        sample(b, ph, cl, A, 0.5 * H[s - 1 + g0], UL);
        sample(b, ph, cr, A, -0.5 * H[s + g0], UR);
    }
    double F[NV];
    double lam;
    if (ph.solver == TS_RS_GODUNOV) {
        bool ok;
        lam = godunov_flux<A>(ph, UL, UR, F, ok);
        if (!ok) atomicOr(&b.ctl->health, (unsigned)TS_HEALTH_RIEMANN);
    } else {
        lam = (ph.solver == TS_RS_HLLC) ? hllc_flux<A>(ph, UL, UR, F) : roe_flux<A>(ph, UL, UR, F);
    }
    // viscous flux subtracted from the convective one (ExplicitRungeKuttaFVM.h:1220-1222);
    // the cell values and gradients of the ghost cells serve the domain faces
    if (ph.viscous) {
        double fv[NV];
        visc_flux<A>(b, ph, cf - st, cf, s, fv);
#pragma unroll
        for (int v = 0; v < NV; ++v) F[v] -= fv[v];
    }
#pragma unroll
    for (int v = 0; v < NV; ++v) b.F[A][vidx(L, v) + cf] = F[v];
    b.Lam[A][cf] = lam;
    // viscous spectral-radius term of the face for its left cell (:1239-1248),
    // Prandtl number 1, only for faces whose left cell is interior
    if (ph.visc != 0.0 && s > 0) {
        const double roFace = sqrt(UL[0] * UR[0]);
        const double t1 = 4.0 / (3.0 * roFace), t2 = ph.gamma / roFace;
        double vsr = (t1 < t2) ? t2 : t1;
        vsr *= ph.visc / 1.0;
        const double fS = face_area(b, ph.nd, A, i, j, k);
        vsr *= fS * fS;
        int il = i, jl = j, kl = k;
        if (A == 0) il -= 1; else if (A == 1) jl -= 1; else kl -= 1;
        const double Vl = b.ch[0][il + L.gx] * b.ch[1][jl + L.gy] * b.ch[2][kl + L.gz];
        vsr /= Vl;
        b.VSR[A][cf] = vsr;
    }
}

__device__ __forceinline__ double warp_min(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = fmin(v, __shfl_xor_sync(0xffffffffu, v, o));
    return v;
}


// Spectral radius per cell in the reference's accumulation order (x-left,
// x-right, y-left, ...), V/SR, block min by warp shuffles; the high-side
// ghost cells, whose SR is their single face term, join the min.  The last
// block to finish reduces the block minima and sets dt.
__global__ void k_dt(PlainBufs b, Phys ph) {
    if (b.ctl->stop_req) return;
    const Layout& L = b.L;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y, k = blockIdx.z;
    const int nd = ph.nd;
    double r = __longlong_as_double(0x7ff0000000000000LL);  // +inf
    if (i < L.nx) {
        const long long c = L.at(i, j, k);
        const double hx = b.ch[0][i + L.gx], hy = b.ch[1][j + L.gy], hz = b.ch[2][k + L.gz];
        const double V = hx * hy * hz;
        double sr = 0.0;
        const int ix[3] = {i, j, k};
        for (int a = 0; a < nd; ++a) {
            const double fS = face_area(b, nd, a, i, j, k);
            const long long st = L.stride(a);
            sr += fS * b.Lam[a][c];
            sr += fS * b.Lam[a][c + st];
            if (ph.visc != 0.0) sr += b.VSR[a][c + st];
            if (ix[a] == L.n(a) - 1) {
                double hg[3] = {hx, hy, hz};
                hg[a] = b.ch[a][L.n(a) + (a == 0 ? L.gx : (a == 1 ? L.gy : L.gz))];
                const double Vg = hg[0] * hg[1] * hg[2];
                r = fmin(r, Vg / (fS * b.Lam[a][c + st]));
            }
        }
        r = fmin(r, V / sr);
    }
    __shared__ double wmin[32];
    r = warp_min(r);
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    if (lane == 0) wmin[wid] = r;
    __syncthreads();
    const int nblk = gridDim.x * gridDim.y * gridDim.z;
    const int bid = blockIdx.x + gridDim.x * (blockIdx.y + gridDim.y * blockIdx.z);
    __shared__ bool last;
    if (threadIdx.x == 0) {
        double m = wmin[0];
        for (int w = 1; w < (int)(blockDim.x + 31) / 32; ++w) m = fmin(m, wmin[w]);
        b.partial[bid] = m;
        __threadfence();
        last = (atomicAdd(&b.ctl->blocks_done, 1u) == (unsigned)(nblk - 1));
    }
    __syncthreads();
    if (!last) return;
    __threadfence();
    double m = __longlong_as_double(0x7ff0000000000000LL);
    for (int t = threadIdx.x; t < nblk; t += blockDim.x) m = fmin(m, ((volatile double*)b.partial)[t]);
    m = warp_min(m);
    if (lane == 0) wmin[wid] = m;
    __syncthreads();
    if (threadIdx.x == 0) {
        m = wmin[0];
        for (int w = 1; w < (int)(blockDim.x + 31) / 32; ++w) m = fmin(m, wmin[w]);
        Ctl* ctl = b.ctl;
        double dt = m * ph.cfl;
        if ((ctl->save_sol > 0) && (ctl->next_sol < ctl->time + dt)) dt = ctl->next_sol - ctl->time;
        if ((ctl->save_slice > 0) && (ctl->next_slice < ctl->time + dt)) dt = ctl->next_slice - ctl->time;
        ctl->dt_min_raw = m;
        ctl->dt = dt;
        for (int v = 0; v < NV; ++v) ctl->res[v] = 0.0;
        ctl->blocks_done = 0;
    }
}

// Residual R = -sum_a (F_{a,+} - F_{a,-}) fS_a accumulated from zero in the
// reference's direction order, then U += dt*(R/V); residual norms and health.
__global__ void k_update(PlainBufs b, Phys ph) {
    if (b.ctl->stop_req) return;
    const Layout& L = b.L;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y, k = blockIdx.z;
    const int nd = ph.nd;
    double nrm[NV] = {0, 0, 0, 0, 0};
    unsigned int health = 0;
    if (i < L.nx) {
        const long long c = L.at(i, j, k);
        const double hx = b.ch[0][i + L.gx], hy = b.ch[1][j + L.gy], hz = b.ch[2][k + L.gz];
        const double V = hx * hy * hz;
        const double dt = b.ctl->dt;
        double R[NV] = {0.0, 0.0, 0.0, 0.0, 0.0};
        for (int a = 0; a < nd; ++a) {
            const double fS = face_area(b, nd, a, i, j, k);
            const long long st = L.stride(a);
#pragma unroll
            for (int v = 0; v < NV; ++v) {
                const double* F = b.F[a] + vidx(L, v);
                R[v] -= (F[c + st] - F[c]) * fS;
            }
        }
        double uo[NV], u[NV];
#pragma unroll
        for (int v = 0; v < NV; ++v) uo[v] = b.U[vidx(L, v) + c];
        // source terms after the face fluxes (ExplicitRungeKuttaFVM.h:1421-1423;
        // ProcessExternalForces and ProcessExternalAcceleration, kernel.h:941-989)
        if (ph.force || ph.accel) {
            const double vu = uo[1] / uo[0], vv = uo[2] / uo[0], vw = uo[3] / uo[0];
            if (ph.force) {
                R[1] += V * ph.sigma[0];
                R[2] += V * ph.sigma[1];
                R[3] += V * ph.sigma[2];
                R[4] += (ph.sigma[0] * vu + ph.sigma[1] * vv + ph.sigma[2] * vw) * V;
            }
            if (ph.accel) {
                const double ro = uo[0];
                R[1] += ro * V * ph.g[0];
                R[2] += ro * V * ph.g[1];
                R[3] += ro * V * ph.g[2];
                R[4] += ((ro * ph.g[0]) * vu + (ro * ph.g[1]) * vv + (ro * ph.g[2]) * vw) * V;
            }
        }
#pragma unroll
        for (int v = 0; v < NV; ++v) {
            u[v] = uo[v] + dt * (R[v] / V);
            b.U[vidx(L, v) + c] = u[v];
            nrm[v] = V * fabs(R[v]);
        }
        const double ke = 0.5 * (u[1] * u[1] + u[2] * u[2] + u[3] * u[3]) / u[0];
        const double p = pressure(ph, u[0], 0.0, 0.0, 0.0, u[4] - ke);
        if (!(u[0] == u[0]) || !(u[4] == u[4]) || !(p == p)) health |= TS_HEALTH_NAN;
        if (u[0] <= 0.0) health |= TS_HEALTH_NEG_DENSITY;
        if (p <= 0.0 && ph.eos == TS_EOS_IDEAL_GAS) health |= TS_HEALTH_NEG_PRESSURE;
        if (ph.eos == TS_EOS_STIFFENED_GAS && p + ph.p_inf <= 0.0) health |= TS_HEALTH_NEG_PRESSURE;
    }
    // block sums of the diagnostic norms (accumulation order differs from the
    // reference's serial sum; the norms are reported, never fed back)
    __shared__ double red[NV][32];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
    for (int v = 0; v < NV; ++v) {
        double s = nrm[v];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
        if (lane == 0) red[v][wid] = s;
    }
    health = __reduce_or_sync(0xffffffffu, health);
    if (lane == 0 && health) atomicOr(&b.ctl->health, health);
    __syncthreads();
    if (threadIdx.x < NV) {
        double s = 0.0;
        for (int w = 0; w < (int)(blockDim.x + 31) / 32; ++w) s += red[threadIdx.x][w];
        atomicAdd(&b.ctl->res[threadIdx.x], s);
    }
}

// time += dt, iteration++ (IterationStep :1486-1487); under Run also the
// snapshot-time bookkeeping and termination test (kernel.h:1763-1846).
__global__ void k_finish(Ctl* ctl) {
    if (ctl->stop_req) return;
    ctl->time += ctl->dt;
    ctl->iteration += 1;
    if (!ctl->run_mode) return;
    if ((ctl->save_sol > 0) && (ctl->next_sol == ctl->time)) ctl->next_sol += ctl->save_sol;
    if ((ctl->save_slice > 0) && (ctl->next_slice == ctl->time)) ctl->next_slice += ctl->save_slice;
    if (ctl->iteration == ctl->max_iteration || ctl->time >= ctl->max_time) ctl->stop_req = 1;
}

}  // namespace

int plain_partial_blocks(const Layout& L) {
    const int bx = (L.nx + kPlainBlock - 1) / kPlainBlock;
    return bx * L.ny * L.nz;
}

cudaError_t plain_step(const PlainBufs& b, const Phys& ph, cudaStream_t st, cudaEvent_t* ev, int* n_launch,
                       const char** names) {
    const Layout& L = b.L;
    const dim3 blk(kPlainBlock);
    const dim3 cells((L.nx + kPlainBlock - 1) / kPlainBlock, L.ny, L.nz);
    auto ghost_grid = [&](int a) {
        const int n1 = (a == 0) ? L.ny : L.nx;
        const int n2 = (a == 2) ? L.ny : L.nz;
        return dim3((n1 * n2 + kPlainBlock - 1) / kPlainBlock);
    };
    int nl = 0;
    if (ev) cudaEventRecord(ev[0], st);
    auto mark = [&](const char* name) {
        if (names) names[nl] = name;
        ++nl;
        if (ev) cudaEventRecord(ev[nl], st);
    };
    k_ghost<0><<<ghost_grid(0), blk, 0, st>>>(b, ph);
    mark("k_ghost_x");
    if (ph.nd > 1) { k_ghost<1><<<ghost_grid(1), blk, 0, st>>>(b, ph); mark("k_ghost_y"); }
    if (ph.nd > 2) { k_ghost<2><<<ghost_grid(2), blk, 0, st>>>(b, ph); mark("k_ghost_z"); }
    if (ph.viscous) {
        k_vgrad<<<cells, blk, 0, st>>>(b, ph);
        mark("k_vgrad");
        k_vgrad_bc<0><<<ghost_grid(0), blk, 0, st>>>(b, ph);
        mark("k_vgrad_bc_x");
        if (ph.nd > 1) { k_vgrad_bc<1><<<ghost_grid(1), blk, 0, st>>>(b, ph); mark("k_vgrad_bc_y"); }
        if (ph.nd > 2) { k_vgrad_bc<2><<<ghost_grid(2), blk, 0, st>>>(b, ph); mark("k_vgrad_bc_z"); }
    }
    if (ph.recon != TS_RECON_PIECEWISE_CONSTANT) { k_recon<<<cells, blk, 0, st>>>(b, ph); mark("k_recon"); }
    const long long xfaces = (long long)(L.nx + 1) * L.ny * L.nz;
    k_flux<0><<<dim3((unsigned)((xfaces + kPlainBlock - 1) / kPlainBlock)), blk, 0, st>>>(b, ph);
    mark("k_flux_x");
    if (ph.nd > 1) { k_flux<1><<<dim3(cells.x, L.ny + 1, L.nz), blk, 0, st>>>(b, ph); mark("k_flux_y"); }
    if (ph.nd > 2) { k_flux<2><<<dim3(cells.x, L.ny, L.nz + 1), blk, 0, st>>>(b, ph); mark("k_flux_z"); }
    k_dt<<<cells, blk, 0, st>>>(b, ph);
    mark("k_dt");
    k_update<<<cells, blk, 0, st>>>(b, ph);
    mark("k_update");
    k_finish<<<1, 1, 0, st>>>(b.ctl);
    mark("k_finish");
    if (n_launch) *n_launch = nl;
    return cudaGetLastError();
}

}  // namespace ts
