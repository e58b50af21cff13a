// Mixed-precision explicit FVM step on GB300: one fused, persistent kernel
// per RK stage.
//
// Precision split: reconstruction, EOS and Riemann flux in FP32; the
// conserved state, the stage accumulation U += dt R / V and the dt reduction
// in FP64 (the increment dt R / V itself carries FP32 accuracy, since R does).
//
// Deferred update.  dt^n depends on the whole field U^n, so a step cannot
// finish U^{n+1} in the sweep that computes R^n without a second pass.  The
// kernel of step n+1 therefore reads U^n (FP64) and R^n (FP32) with dt^n,
// forms U^{n+1} on the fly (FP64 for the cells it owns, written out; an FP32
// working copy for the stencil, identical in every CTA that loads the cell),
// computes R^{n+1} and the CFL maximum, and writes U^{n+1} and R^{n+1}.  One
// pass per step: 40 B FP64 read + 20 B FP32 read + 40 B + 20 B written per
// cell-update.  A final apply pass materialises the state for the host.
//
// Tiling.  Each CTA owns an x-y tile (TX x TY cells) and marches along z
// (2.5D blocking), keeping a 3-plane ring of the FP32 working state with a
// 2-cell halo, a 2-plane ring of limited half-slopes with a 1-cell halo and
// the face fluxes in shared memory; CTAs get contiguous ranges of
// (column, plane) work so the persistent grid is balanced to one plane.
//
// Ghost cells are virtual: a load outside the domain wraps on periodic axes
// and mirrors plus applies the boundary condition (BCGeneral.h:186-268)
// otherwise, and boundary faces take the flux against the BC image of the
// inner face state (ExplicitRungeKuttaFVM.h:1198-1209).
//
// FP64 is scarce on GB300 (about 2 FP64 operations per clock per SM,
// conversions included), so FP64<->FP32 conversions are done with integer
// bit operations and the only FP64 arithmetic per owned cell is the five
// state additions.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "ts_mixed.h"

namespace ts {
namespace {

constexpr int HB = 2;  // halo of the working-state box

struct MixArgs {
    Layout L;
    double* U[2];
    float* R[2];
    const AxisGeo* geo[3];
    int goff[3];  // index offset into geo per axis (ghost width or 0)
    Ctl* ctl;
    MixPhys mp;
    int tx, ty, ncx;
    long long total;  // columns x planes
    int per_cta;      // planes per CTA
};

// ---------------------------------------------------------------------------
// FP64 <-> FP32 on the integer pipe
// ---------------------------------------------------------------------------
// Truncating FP64 -> FP32 for finite values with |x| < 2^128; |x| < 2^-126
// gives a signed zero.  Four integer operations instead of a conversion on
// the FP64 pipe.
__device__ __forceinline__ float f64_to_f32(double d) {
    const unsigned int hi = (unsigned int)__double2hiint(d);
    const unsigned int lo = (unsigned int)__double2loint(d);
    const unsigned int sign = hi & 0x80000000u;
    const unsigned int t = __funnelshift_l(lo, hi - 0x38000000u, 3);
    const unsigned int e = (hi >> 20) & 0x7FFu;
    return __uint_as_float(e < 897u ? sign : ((t & 0x7FFFFFFFu) | sign));
}

// Exact FP32 -> FP64 for normal numbers and zeros (FP32 runs flush-to-zero).
__device__ __forceinline__ double f32_to_f64(float f) {
    const unsigned int b = __float_as_uint(f);
    const unsigned int a = b & 0x7FFFFFFFu;
    const unsigned int hi = (a ? (a >> 3) + 0x38000000u : 0u) | (b & 0x80000000u);
    return __hiloint2double((int)hi, (int)(b << 29));
}

__device__ __forceinline__ void resolve(int idx, int n, int periodic, int side_lo, int& src, int& side) {
    side = -1;
    src = idx;
    if (idx < 0) {
        if (periodic) src = idx + n;
        else { src = -1 - idx; side = side_lo; }
    } else if (idx >= n) {
        if (periodic) src = idx - n;
        else { src = 2 * n - 1 - idx; side = side_lo + 1; }
    }
}

// Boundary-condition image of a state (shifted energy) across `side`.
__device__ __forceinline__ void bc32(const MixPhys& p, int side, int A, float w[NV]) {
    const int t = p.bc_type[side];
    if (t == TS_BC_SYMMETRY) {
        w[1 + A] = -w[1 + A];
    } else if (t == TS_BC_WALL) {
        w[1] = -w[1]; w[2] = -w[2]; w[3] = -w[3];
    } else if (t == TS_BC_MOVING_WALL) {
        const float r = w[0], ir = 1.0f / r;
        const float vx = w[1] * ir, vy = w[2] * ir, vz = w[3] * ir;
        const float dx = 2.0f * p.bc_vel[side][0] - vx, dy = 2.0f * p.bc_vel[side][1] - vy,
                    dz = 2.0f * p.bc_vel[side][2] - vz;
        w[1] = r * dx; w[2] = r * dy; w[3] = r * dz;
        w[4] = w[4] + 0.5f * r * ((dx * dx + dy * dy + dz * dz) - (vx * vx + vy * vy + vz * vz));
    } else if (t == TS_BC_SUBSONIC_INLET) {
#pragma unroll
        for (int v = 0; v < NV; ++v) w[v] = p.bc_state[side][v];
    }
}

// ---------------------------------------------------------------------------
// FP32 Riemann solvers along axis A.  States carry the shifted energy
// E' = E - einf, so p = (g-1)(E' - rho |u|^2 / 2) for both equations of state
// without cancellation; E = E' + einf where the total energy enters.
// ---------------------------------------------------------------------------
__device__ __forceinline__ float harten32(float z, float e) {
    z = fabsf(z);
    return (z < e) ? ((z * z) / e + e) * 0.5f : z;
}

// Roe-Pike flux (RoeSolverPerfectGasEOS.h:74-160) in the equivalent form
// 1/2 [F(UL) + F(UR) + |A|(UL - UR)], |A| dU = a1 dU + Ac Qa + Bc Qb with
// Qa = (0, e_A, un), Qb = (1, u, H), Ac = Ea dR + Eb dD, Bc = Ea dD + Eb dR / c^2.
template <int A>
__device__ __forceinline__ float roe32(const MixPhys& p, const float UL[NV], const float UR[NV], float F[NV]) {
    const float gm1 = p.gm1;
    const float rl = 1.0f / UL[0], rr = 1.0f / UR[0];
    const float ulx = UL[1] * rl, uly = UL[2] * rl, ulz = UL[3] * rl;
    const float urx = UR[1] * rr, ury = UR[2] * rr, urz = UR[3] * rr;
    const float pl = gm1 * (UL[4] - 0.5f * UL[0] * (ulx * ulx + uly * uly + ulz * ulz));
    const float pr = gm1 * (UR[4] - 0.5f * UR[0] * (urx * urx + ury * ury + urz * urz));
    const float el = UL[4] + p.einf + pl, er = UR[4] + p.einf + pr;  // E + p
    const float sl = UL[0] * rsqrtf(UL[0]), sr = UR[0] * rsqrtf(UR[0]);
    const float inv = 1.0f / (sl + sr);
    const float ql = sl * inv, qr = sr * inv;
    const float ux = ql * ulx + qr * urx, uy = ql * uly + qr * ury, uz = ql * ulz + qr * urz;
    const float h = ql * (el * rl) + qr * (er * rr);
    const float q2 = ux * ux + uy * uy + uz * uz;
    const float c2 = gm1 * (h - 0.5f * q2);
    const float ic = rsqrtf(c2);
    const float c = c2 * ic;
    const float un = A == 0 ? ux : (A == 1 ? uy : uz);
    const float lam = fabsf(un) + c;
    float a1 = fabsf(un), a3 = fabsf(un + c), a4 = fabsf(un - c);
    if (p.eps > 0.0f) {
        const float he = p.eps * lam;
        a1 = harten32(un, he); a3 = harten32(un + c, he); a4 = harten32(un - c, he);
    }
    const float Ea = (a3 - a4) * 0.5f * ic;
    const float Eb = (a3 + a4) * 0.5f - a1;
    const float dr = UL[0] - UR[0], dmx = UL[1] - UR[1], dmy = UL[2] - UR[2], dmz = UL[3] - UR[3];
    const float de = UL[4] - UR[4];
    const float dm_n = A == 0 ? dmx : (A == 1 ? dmy : dmz);
    const float dR = 0.5f * gm1 * q2 * dr - gm1 * (ux * dmx + uy * dmy + uz * dmz - de);
    const float dD = dm_n - dr * un;
    const float Ac = Ea * dR + Eb * dD;
    const float Bc = Ea * dD + Eb * dR * (ic * ic);
    const float unl = A == 0 ? ulx : (A == 1 ? uly : ulz);
    const float unr = A == 0 ? urx : (A == 1 ? ury : urz);
    F[0] = 0.5f * (UL[0] * unl + UR[0] * unr + a1 * dr + Bc);
    F[1] = 0.5f * (UL[1] * unl + UR[1] * unr + (A == 0 ? pl + pr + Ac : 0.0f) + a1 * dmx + Bc * ux);
    F[2] = 0.5f * (UL[2] * unl + UR[2] * unr + (A == 1 ? pl + pr + Ac : 0.0f) + a1 * dmy + Bc * uy);
    F[3] = 0.5f * (UL[3] * unl + UR[3] * unr + (A == 2 ? pl + pr + Ac : 0.0f) + a1 * dmz + Bc * uz);
    F[4] = 0.5f * (el * unl + er * unr + a1 * de + Ac * un + Bc * h);
    return lam;
}

// HLLC (Toro ch. 10.4), Einfeldt-type speeds from Roe averages.
template <int A>
__device__ __forceinline__ float hllc32(const MixPhys& p, const float UL[NV], const float UR[NV], float F[NV]) {
    const float g = p.gamma, gm1 = p.gm1;
    const float rl = 1.0f / UL[0], rr = 1.0f / UR[0];
    const float vl[3] = {UL[1] * rl, UL[2] * rl, UL[3] * rl};
    const float vr[3] = {UR[1] * rr, UR[2] * rr, UR[3] * rr};
    const float pl = gm1 * (UL[4] - 0.5f * UL[0] * (vl[0] * vl[0] + vl[1] * vl[1] + vl[2] * vl[2]));
    const float pr = gm1 * (UR[4] - 0.5f * UR[0] * (vr[0] * vr[0] + vr[1] * vr[1] + vr[2] * vr[2]));
    const float El = UL[4] + p.einf, Er = UR[4] + p.einf;
    const float cl = sqrtf(g * (pl + p.pinf) * rl), cr = sqrtf(g * (pr + p.pinf) * rr);
    const float sl = UL[0] * rsqrtf(UL[0]), sr = UR[0] * rsqrtf(UR[0]);
    const float inv = 1.0f / (sl + sr);
    const float wl = sl * inv, wr = sr * inv;
    const float ul = vl[A], ur = vr[A];
    const float ut = wl * ul + wr * ur;
    const float vtx = wl * vl[0] + wr * vr[0], vty = wl * vl[1] + wr * vr[1], vtz = wl * vl[2] + wr * vr[2];
    const float ht = wl * ((El + pl) * rl) + wr * ((Er + pr) * rr);
    const float ct = sqrtf(gm1 * (ht - 0.5f * (vtx * vtx + vty * vty + vtz * vtz)));
    const float SL = fminf(ul - cl, ut - ct);
    const float SR = fmaxf(ur + cr, ut + ct);
    const float ml = UL[0] * (SL - ul), mr = UR[0] * (SR - ur);
    const float ss = (pr - pl + ul * ml - ur * mr) / (ml - mr);
    // F_L if 0 <= S_L, F_R if S_R <= 0, else the star state on the side of S*
    const bool supl = SL >= 0.0f, supr = SR <= 0.0f;
    const bool left = supl || (!supr && ss >= 0.0f);
    const float* U = left ? UL : UR;
    const float* v = left ? vl : vr;
    const float uk = left ? ul : ur, pk = left ? pl : pr, Ek = left ? El : Er, rk = left ? rl : rr;
    const float Sk = left ? SL : SR, mk = left ? ml : mr;
    // physical flux of the upwind side
    F[0] = U[0] * uk;
    F[1] = U[1] * uk + (A == 0 ? pk : 0.0f);
    F[2] = U[2] * uk + (A == 1 ? pk : 0.0f);
    F[3] = U[3] * uk + (A == 2 ? pk : 0.0f);
    F[4] = (Ek + pk) * uk;
    const bool star = !supl && !supr;
    if (star) {
        const float coef = mk / (Sk - ss);
        float us[NV];
        us[0] = coef;
        us[1] = coef * (A == 0 ? ss : v[0]);
        us[2] = coef * (A == 1 ? ss : v[1]);
        us[3] = coef * (A == 2 ? ss : v[2]);
        us[4] = coef * (Ek * rk + (ss - uk) * (ss + pk / mk));
        F[0] += Sk * (us[0] - U[0]);
        F[1] += Sk * (us[1] - U[1]);
        F[2] += Sk * (us[2] - U[2]);
        F[3] += Sk * (us[3] - U[3]);
        F[4] += Sk * (us[4] - Ek);
    }
    return fmaxf(fabsf(SL), fabsf(SR));
}

template <int SOLVER, int A>
__device__ __forceinline__ float flux32(const MixPhys& p, const float UL[NV], const float UR[NV], float F[NV]) {
    if (SOLVER == TS_RS_HLLC) return hllc32<A>(p, UL, UR, F);
    return roe32<A>(p, UL, UR, F);
}

// ---------------------------------------------------------------------------
// Shared-memory layout of one CTA
// ---------------------------------------------------------------------------
template <int ND>
struct Smem {
    float* W;   // [WS][NV][BY][BX]  FP32 working state, 2-cell halo
    float* D;   // [DS][3][NV][RY][RX] limited half-slopes, 1-cell halo
    float* Fx;  // [6][TY][TX+1]
    float* Fy;  // [6][TY+1][TX]
    float* Fz;  // [2][6][TY][TX]
    int TX, TY, BX, BY, RX, RY;
    static constexpr int WS = ND == 3 ? 3 : 1;
    static constexpr int DS = ND == 3 ? 2 : 1;

    __device__ void setup(float* base, int tx, int ty) {
        TX = tx; TY = ty;
        BX = tx + 2 * HB; BY = ND >= 2 ? ty + 2 * HB : 1;
        RX = tx + 2; RY = ND >= 2 ? ty + 2 : 1;
        W = base;
        D = W + WS * NV * BY * BX;
        Fx = D + DS * 3 * NV * RY * RX;
        Fy = Fx + 6 * ty * (tx + 1);
        Fz = Fy + (ND >= 2 ? 6 * (ty + 1) * tx : 0);
    }
    static size_t bytes(int tx, int ty) {
        const size_t bx = tx + 2 * HB, by = ND >= 2 ? ty + 2 * HB : 1, rx = tx + 2, ry = ND >= 2 ? ty + 2 : 1;
        size_t f = WS * NV * by * bx + DS * 3 * NV * ry * rx + 6 * ty * (tx + 1);
        if (ND >= 2) f += 6 * (ty + 1) * tx;
        if (ND == 3) f += 2 * 6 * ty * tx;
        return f * sizeof(float);
    }
    __device__ float& w(int s, int v, int y, int x) { return W[((s * NV + v) * BY + y) * BX + x]; }
    __device__ float& d(int s, int a, int v, int y, int x) { return D[(((s * 3 + a) * NV + v) * RY + y) * RX + x]; }
    __device__ float& fx(int v, int y, int x) { return Fx[(v * TY + y) * (TX + 1) + x]; }
    __device__ float& fy(int v, int y, int x) { return Fy[(v * (TY + 1) + y) * TX + x]; }
    __device__ float& fz(int s, int v, int y, int x) { return Fz[((s * 6 + v) * TY + y) * TX + x]; }
};

__device__ __forceinline__ int wslot(int p) { return (p + 3) % 3; }
__device__ __forceinline__ int dslot(int p) { return (p + 2) & 1; }

// ---------------------------------------------------------------------------
// Phase A: FP32 working state of plane p (and U^{n+1} of owned cells)
// ---------------------------------------------------------------------------
template <int ND>
__device__ void load_plane(const MixArgs& a, Smem<ND>& s, int i0, int j0, int p, int z0, int z1, float dtf,
                           unsigned int& health) {
    const Layout& L = a.L;
    const MixPhys& mp = a.mp;
    const int slot = ND == 3 ? wslot(p) : 0;
    int sk = 0, zs = -1;
    if (ND == 3) resolve(p, L.nz, mp.periodic[2], 4, sk, zs);
    const bool own_plane = p >= z0 && p < z1;
    const double* __restrict__ Uin = a.U[a.ctl->parity];
    double* __restrict__ Uout = a.U[a.ctl->parity ^ 1];
    const float* __restrict__ Rin = a.R[a.ctl->parity];
    const float hz_ih = a.geo[2][sk + a.goff[2]].ih;
    const int n = s.BX * s.BY;
    for (int t = threadIdx.x; t < n; t += blockDim.x) {
        const int lx = t % s.BX, ly = t / s.BX;
        const int dx = lx < HB ? HB - lx : (lx >= s.TX + HB ? lx - s.TX - HB + 1 : 0);
        const int dy = ND >= 2 ? (ly < HB ? HB - ly : (ly >= s.TY + HB ? ly - s.TY - HB + 1 : 0)) : 0;
        if (dx + dy > HB) continue;
        const int gi = i0 + lx - HB;
        const int gj = ND >= 2 ? j0 + ly - HB : 0;
        if (gi >= L.nx + HB) continue;
        if (ND >= 2 && gj >= L.ny + HB) continue;
        int si, xs, sj = 0, ys = -1;
        resolve(gi, L.nx, mp.periodic[0], 0, si, xs);
        if (ND >= 2) resolve(gj, L.ny, mp.periodic[1], 2, sj, ys);
        const long long c = L.at(si, sj, sk);
        const float cf = dtf * (a.geo[0][si + a.goff[0]].ih * a.geo[1][sj + a.goff[1]].ih * hz_ih);
        double u[NV];
        float inc[NV], w[NV];
#pragma unroll
        for (int v = 0; v < NV; ++v) u[v] = Uin[(long long)v * L.plane + c];
#pragma unroll
        for (int v = 0; v < NV; ++v) inc[v] = cf * Rin[(long long)v * L.plane + c];
#pragma unroll
        for (int v = 0; v < 4; ++v) w[v] = f64_to_f32(u[v]) + inc[v];
        w[4] = (mp.eos == TS_EOS_STIFFENED_GAS ? f64_to_f32(u[4] - mp.einf_d) : f64_to_f32(u[4])) + inc[4];
        if (xs >= 0) bc32(mp, xs, 0, w);
        if (ND >= 2 && ys >= 0) bc32(mp, ys, 1, w);
        if (ND == 3 && zs >= 0) bc32(mp, zs, 2, w);
#pragma unroll
        for (int v = 0; v < NV; ++v) s.w(slot, v, ly, lx) = w[v];
        if (own_plane && dx == 0 && dy == 0 && gi < L.nx && gj < L.ny) {
            double un[NV];
#pragma unroll
            for (int v = 0; v < NV; ++v) {
                un[v] = u[v] + f32_to_f64(inc[v]);
                Uout[(long long)v * L.plane + c] = un[v];
            }
            if (!(un[0] > 0.0)) health |= (un[0] == un[0]) ? TS_HEALTH_NEG_DENSITY : TS_HEALTH_NAN;
            if (!(w[4] == w[4])) health |= TS_HEALTH_NAN;
        }
    }
}

// ---------------------------------------------------------------------------
// Phase B: limited half-slopes of plane p on the tile plus a 1-cell ring
// ---------------------------------------------------------------------------
template <int ND>
__device__ void recon_plane(const MixArgs& a, Smem<ND>& s, int i0, int j0, int p) {
    const Layout& L = a.L;
    const MixPhys& mp = a.mp;
    const int ws = ND == 3 ? wslot(p) : 0;
    const int wd = ND == 3 ? wslot(p - 1) : 0, wu = ND == 3 ? wslot(p + 1) : 0;
    const int ds = ND == 3 ? dslot(p) : 0;
    int sk = 0, zs;
    if (ND == 3) {
        if ((p < 0 || p >= L.nz) && !mp.periodic[2]) return;
        resolve(p, L.nz, mp.periodic[2], 4, sk, zs);
    }
    const AxisGeo gz = a.geo[2][sk + a.goff[2]];
    const int n = s.RX * s.RY;
    for (int t = threadIdx.x; t < n; t += blockDim.x) {
        const int rx = t % s.RX, ry = t / s.RX;
        const int ox = (rx < 1 || rx > s.TX) ? 1 : 0;
        const int oy = ND >= 2 ? ((ry < 1 || ry > s.TY) ? 1 : 0) : 0;
        if (ox + oy > 1) continue;
        const int gi = i0 + rx - 1, gj = ND >= 2 ? j0 + ry - 1 : 0;
        if (gi > L.nx || (ND >= 2 && gj > L.ny)) continue;
        if ((gi < 0 || gi >= L.nx) && !mp.periodic[0]) continue;
        if (ND >= 2 && (gj < 0 || gj >= L.ny) && !mp.periodic[1]) continue;
        int si, xs, sj = 0, ys;
        resolve(gi, L.nx, 1, 0, si, xs);
        if (ND >= 2) resolve(gj, L.ny, 1, 2, sj, ys);
        const AxisGeo g[3] = {a.geo[0][si + a.goff[0]], a.geo[1][sj + a.goff[1]], gz};
        const int lx = rx + 1, ly = ND >= 2 ? ry + 1 : 0;
        float eps2 = 0.0f;
        if (mp.limiter == TS_LIM_VENKATAKRISHNAN && mp.recon == TS_RECON_LINEAR_2POINTS_LIMITED) {
            // eps^2 = (K (hx hy hz)^(1/nd))^3 with K = 5 (Limiters.h:93-96, Constants.h:11)
            const float vol = g[0].h * g[1].h * g[2].h;
            eps2 = 125.0f * (ND == 3 ? vol : (ND == 2 ? vol * sqrtf(vol) : vol * vol * vol));
        }
#pragma unroll
        for (int v = 0; v < NV; ++v) {
            const float w0 = s.w(ws, v, ly, lx);
            float nm[3], np[3];
            nm[0] = s.w(ws, v, ly, lx - 1);
            np[0] = s.w(ws, v, ly, lx + 1);
            if (ND >= 2) { nm[1] = s.w(ws, v, ly - 1, lx); np[1] = s.w(ws, v, ly + 1, lx); }
            if (ND == 3) { nm[2] = s.w(wd, v, ly, lx); np[2] = s.w(wu, v, ly, lx); }
            float dd[3];
            if (mp.recon == TS_RECON_ENO2_2POINTS) {
#pragma unroll
                for (int ax = 0; ax < ND; ++ax) {
                    const float gl = (w0 - nm[ax]) * g[ax].il, gr = (np[ax] - w0) * g[ax].ir;
                    dd[ax] = (fabsf(gl) < fabsf(gr) ? gl : gr) * g[ax].hh;
                }
            } else {
#pragma unroll
                for (int ax = 0; ax < ND; ++ax) dd[ax] = (np[ax] - nm[ax]) * g[ax].ks;
            }
            if (mp.recon == TS_RECON_LINEAR_2POINTS_LIMITED) {
                float umax = w0, umin = w0;
#pragma unroll
                for (int ax = 0; ax < ND; ++ax) {
                    umax = fmaxf(umax, fmaxf(nm[ax], np[ax]));
                    umin = fminf(umin, fminf(nm[ax], np[ax]));
                }
                float lim = 1.0f;
                if (umax - umin > 0.0f) {
                    if (mp.limiter == TS_LIM_VENKATAKRISHNAN) {
                        // Limiters.h:86-115, per face projection +-dd
                        const float iun = 2.0f / (umax - umin);
#pragma unroll
                        for (int ax = 0; ax < ND; ++ax) {
#pragma unroll
                            for (int sg = 0; sg < 2; ++sg) {
                                const float d2 = sg ? -dd[ax] : dd[ax];
                                if (d2 == 0.0f) continue;
                                const float dm = ((d2 > 0.0f ? umax : umin) - w0) * iun;
                                const float q = d2 * iun;
                                const float r = ((dm * dm + eps2) + 2.0f * q * dm) / (dm * dm + 2.0f * q * q + dm * q + eps2);
                                lim = fminf(lim, r);
                            }
                        }
                    } else {
                        // Barth-Jespersen (Limiters.h:74-83): the smallest admissible
                        // ratio over the 2*nd face projections +-dd.
                        float dmax = 0.0f;
#pragma unroll
                        for (int ax = 0; ax < ND; ++ax) dmax = fmaxf(dmax, fabsf(dd[ax]));
                        if (dmax > 0.0f) lim = fminf(1.0f, fminf(umax - w0, w0 - umin) / dmax);
                    }
                }
#pragma unroll
                for (int ax = 0; ax < ND; ++ax) dd[ax] *= lim;
            }
#pragma unroll
            for (int ax = 0; ax < ND; ++ax) s.d(ds, ax, v, ry, rx) = dd[ax];
        }
    }
}

// ---------------------------------------------------------------------------
// Phase C: fluxes of plane z (x and y faces) and of the z face above it
// ---------------------------------------------------------------------------
template <int ND, int SOLVER, int A>
__device__ __forceinline__ void face_flux(const MixPhys& mp, bool bc_lo, bool bc_hi, float UL[NV], float UR[NV],
                                          float F[NV], float& lam) {
    if (bc_lo) {
#pragma unroll
        for (int v = 0; v < NV; ++v) UL[v] = UR[v];
        bc32(mp, 2 * A, A, UL);
    } else if (bc_hi) {
#pragma unroll
        for (int v = 0; v < NV; ++v) UR[v] = UL[v];
        bc32(mp, 2 * A + 1, A, UR);
    }
    lam = flux32<SOLVER, A>(mp, UL, UR, F);
}

template <int ND, int SOLVER>
__device__ void flux_plane(const MixArgs& a, Smem<ND>& s, int i0, int j0, int z, bool do_xy, bool do_z) {
    const Layout& L = a.L;
    const MixPhys& mp = a.mp;
    const bool pwc = mp.recon == TS_RECON_PIECEWISE_CONSTANT;
    const int ws = ND == 3 ? wslot(z) : 0, ds = ND == 3 ? dslot(z) : 0;
    float UL[NV], UR[NV], F[NV], lam;
    if (do_xy) {
        const int nfx = (s.TX + 1) * s.TY;
        for (int t = threadIdx.x; t < nfx; t += blockDim.x) {
            const int fx = t % (s.TX + 1), fy = t / (s.TX + 1);
            const int gi = i0 + fx, gj = j0 + fy;
            if (gi > L.nx || gj >= L.ny) continue;
            const int ly = ND >= 2 ? fy + HB : 0, ry = ND >= 2 ? fy + 1 : 0;
#pragma unroll
            for (int v = 0; v < NV; ++v) {
                UL[v] = s.w(ws, v, ly, fx + 1) + (pwc ? 0.0f : s.d(ds, 0, v, ry, fx));
                UR[v] = s.w(ws, v, ly, fx + 2) - (pwc ? 0.0f : s.d(ds, 0, v, ry, fx + 1));
            }
            face_flux<ND, SOLVER, 0>(mp, gi == 0 && !mp.periodic[0], gi == L.nx && !mp.periodic[0], UL, UR, F, lam);
#pragma unroll
            for (int v = 0; v < NV; ++v) s.fx(v, fy, fx) = F[v];
            s.fx(5, fy, fx) = lam;
        }
        if (ND >= 2) {
            const int nfy = s.TX * (s.TY + 1);
            for (int t = threadIdx.x; t < nfy; t += blockDim.x) {
                const int fx = t % s.TX, fy = t / s.TX;
                const int gi = i0 + fx, gj = j0 + fy;
                if (gi >= L.nx || gj > L.ny) continue;
#pragma unroll
                for (int v = 0; v < NV; ++v) {
                    UL[v] = s.w(ws, v, fy + 1, fx + HB) + (pwc ? 0.0f : s.d(ds, 1, v, fy, fx + 1));
                    UR[v] = s.w(ws, v, fy + 2, fx + HB) - (pwc ? 0.0f : s.d(ds, 1, v, fy + 1, fx + 1));
                }
                face_flux<ND, SOLVER, 1>(mp, gj == 0 && !mp.periodic[1], gj == L.ny && !mp.periodic[1], UL, UR, F,
                                         lam);
#pragma unroll
                for (int v = 0; v < NV; ++v) s.fy(v, fy, fx) = F[v];
                s.fy(5, fy, fx) = lam;
            }
        }
    }
    if (ND == 3 && do_z) {
        // face between planes z and z+1, stored in slot dslot(z+1)
        const int wu = wslot(z + 1), du = dslot(z + 1), fs = dslot(z + 1);
        const int gk = z + 1;
        const int nf = s.TX * s.TY;
        for (int t = threadIdx.x; t < nf; t += blockDim.x) {
            const int fx = t % s.TX, fy = t / s.TX;
            if (i0 + fx >= L.nx || j0 + fy >= L.ny) continue;
#pragma unroll
            for (int v = 0; v < NV; ++v) {
                UL[v] = s.w(ws, v, fy + HB, fx + HB) + (pwc ? 0.0f : s.d(ds, 2, v, fy + 1, fx + 1));
                UR[v] = s.w(wu, v, fy + HB, fx + HB) - (pwc ? 0.0f : s.d(du, 2, v, fy + 1, fx + 1));
            }
            face_flux<ND, SOLVER, 2>(mp, gk == 0 && !mp.periodic[2], gk == L.nz && !mp.periodic[2], UL, UR, F, lam);
#pragma unroll
            for (int v = 0; v < NV; ++v) s.fz(fs, v, fy, fx) = F[v];
            s.fz(fs, 5, fy, fx) = lam;
        }
    }
}

// ---------------------------------------------------------------------------
// Phase D: residual and spectral radius of the owned cells of plane z
// ---------------------------------------------------------------------------
template <int ND>
__device__ void residual_plane(const MixArgs& a, Smem<ND>& s, int i0, int j0, int z, float& srmax) {
    const Layout& L = a.L;
    const int t = threadIdx.x;
    if (t >= s.TX * s.TY) return;
    const int tx = t % s.TX, ty = t / s.TX;
    const int gi = i0 + tx, gj = j0 + ty;
    if (gi >= L.nx || gj >= L.ny) return;
    const AxisGeo gx = a.geo[0][gi + a.goff[0]], gy = a.geo[1][gj + a.goff[1]], gz = a.geo[2][z + a.goff[2]];
    const float fsx = gy.h * gz.h, fsy = gx.h * gz.h, fsz = gx.h * gy.h;
    const float iv = gx.ih * gy.ih * gz.ih;
    float R[NV];
    const float lxl = s.fx(5, ty, tx), lxr = s.fx(5, ty, tx + 1);
#pragma unroll
    for (int v = 0; v < NV; ++v) R[v] = -(s.fx(v, ty, tx + 1) - s.fx(v, ty, tx)) * fsx;
    float sr = fsx * (lxl + lxr);
    if (gi == L.nx - 1) srmax = fmaxf(srmax, fsx * lxr * a.geo[0][L.nx + a.goff[0]].ih * gy.ih * gz.ih);
    if (ND >= 2) {
#pragma unroll
        for (int v = 0; v < NV; ++v) R[v] -= (s.fy(v, ty + 1, tx) - s.fy(v, ty, tx)) * fsy;
        const float lyr = s.fy(5, ty + 1, tx);
        sr += fsy * (s.fy(5, ty, tx) + lyr);
        if (gj == L.ny - 1) srmax = fmaxf(srmax, fsy * lyr * gx.ih * a.geo[1][L.ny + a.goff[1]].ih * gz.ih);
    }
    if (ND == 3) {
        const int dn = dslot(z), up = dslot(z + 1);
#pragma unroll
        for (int v = 0; v < NV; ++v) R[v] -= (s.fz(up, v, ty, tx) - s.fz(dn, v, ty, tx)) * fsz;
        const float lzr = s.fz(up, 5, ty, tx);
        sr += fsz * (s.fz(dn, 5, ty, tx) + lzr);
        if (z == L.nz - 1) srmax = fmaxf(srmax, fsz * lzr * gx.ih * gy.ih * a.geo[2][L.nz + a.goff[2]].ih);
    }
    srmax = fmaxf(srmax, sr * iv);
    float* __restrict__ Rout = a.R[a.ctl->parity ^ 1];
    const long long c = L.at(gi, gj, z);
#pragma unroll
    for (int v = 0; v < NV; ++v) Rout[(long long)v * L.plane + c] = R[v];
}

// ---------------------------------------------------------------------------
// The fused step kernel
// ---------------------------------------------------------------------------
template <int ND, int SOLVER>
__global__ void __launch_bounds__(256) k_mix_step(MixArgs a) {
    Ctl* ctl = a.ctl;
    if (ctl->stop_req) return;
    extern __shared__ float smem[];
    Smem<ND> s;
    s.setup(smem, a.tx, a.ty);
    const Layout& L = a.L;
    const float dtf = f64_to_f32(ctl->dt_apply);
    const int nz = ND == 3 ? L.nz : 1;
    float srmax = 0.0f;
    unsigned int health = 0;
    const long long beg = (long long)blockIdx.x * a.per_cta;
    const long long end = min(beg + a.per_cta, a.total);
    const bool pwc = a.mp.recon == TS_RECON_PIECEWISE_CONSTANT;
    for (long long gidx = beg; gidx < end;) {
        const int col = (int)(gidx / nz);
        const int z0 = (int)(gidx % nz);
        const int z1 = (int)min((long long)nz, z0 + (end - gidx));
        const int i0 = (col % a.ncx) * a.tx;
        const int j0 = (col / a.ncx) * a.ty;
        if (ND < 3) {
            load_plane<ND>(a, s, i0, j0, 0, 0, 1, dtf, health);
            __syncthreads();
            if (!pwc) { recon_plane<ND>(a, s, i0, j0, 0); __syncthreads(); }
            flux_plane<ND, SOLVER>(a, s, i0, j0, 0, true, false);
            __syncthreads();
            residual_plane<ND>(a, s, i0, j0, 0, srmax);
            __syncthreads();
        } else {
            // prologue: planes z0-2 .. z0+1, slopes of z0-1 and z0, z face z0-1/2
            load_plane<ND>(a, s, i0, j0, z0 - 2, z0, z1, dtf, health);
            load_plane<ND>(a, s, i0, j0, z0 - 1, z0, z1, dtf, health);
            load_plane<ND>(a, s, i0, j0, z0, z0, z1, dtf, health);
            __syncthreads();
            if (!pwc) { recon_plane<ND>(a, s, i0, j0, z0 - 1); }
            __syncthreads();
            load_plane<ND>(a, s, i0, j0, z0 + 1, z0, z1, dtf, health);
            __syncthreads();
            if (!pwc) { recon_plane<ND>(a, s, i0, j0, z0); __syncthreads(); }
            flux_plane<ND, SOLVER>(a, s, i0, j0, z0 - 1, false, true);
            __syncthreads();
            for (int z = z0; z < z1; ++z) {
                load_plane<ND>(a, s, i0, j0, z + 2, z0, z1, dtf, health);
                __syncthreads();
                if (!pwc) { recon_plane<ND>(a, s, i0, j0, z + 1); __syncthreads(); }
                flux_plane<ND, SOLVER>(a, s, i0, j0, z, true, true);
                __syncthreads();
                residual_plane<ND>(a, s, i0, j0, z, srmax);
            }
            __syncthreads();
        }
        gidx += z1 - z0;
    }
    // CFL: max over cells of SR/V, block max by warp shuffles, one atomic per
    // CTA; the last CTA to finish turns it into dt (FP64) and closes the step.
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) srmax = fmaxf(srmax, __shfl_xor_sync(0xffffffffu, srmax, o));
    health = __reduce_or_sync(0xffffffffu, health);
    __shared__ float wmax[32];
    __shared__ unsigned int whealth[32];
    __shared__ bool last;
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    if (lane == 0) { wmax[wid] = srmax; whealth[wid] = health; }
    __syncthreads();
    if (threadIdx.x == 0) {
        float m = 0.0f;
        unsigned int hh = 0;
        for (int k = 0; k < (int)(blockDim.x + 31) / 32; ++k) { m = fmaxf(m, wmax[k]); hh |= whealth[k]; }
        if (m > 0.0f) atomicMax(&ctl->srmax_bits, __float_as_uint(m));
        if (hh) atomicOr(&ctl->health, hh);
        __threadfence();
        last = atomicAdd(&ctl->blocks_done, 1u) == gridDim.x - 1;
    }
    __syncthreads();
    if (!last || threadIdx.x != 0) return;
    __threadfence();
    const float m = __uint_as_float(*(volatile unsigned int*)&ctl->srmax_bits);
    double dt = a.mp.cfl / (double)m;
    if ((ctl->save_sol > 0) && (ctl->next_sol < ctl->time + dt)) dt = ctl->next_sol - ctl->time;
    if ((ctl->save_slice > 0) && (ctl->next_slice < ctl->time + dt)) dt = ctl->next_slice - ctl->time;
    ctl->dt_min_raw = 1.0 / (double)m;
    ctl->dt = dt;
    ctl->dt_apply = dt;
    ctl->time += dt;
    ctl->iteration += 1;
    ctl->parity ^= 1;
    ctl->srmax_bits = 0u;
    ctl->blocks_done = 0u;
    if (ctl->run_mode) {
        if ((ctl->save_sol > 0) && (ctl->next_sol == ctl->time)) ctl->next_sol += ctl->save_sol;
        if ((ctl->save_slice > 0) && (ctl->next_slice == ctl->time)) ctl->next_slice += ctl->save_slice;
        if (ctl->iteration == ctl->max_iteration || ctl->time >= ctl->max_time) ctl->stop_req = 1;
    }
}

// U[parity] += dt R[parity] / V, R[parity] = 0 (materialise the pending update).
__global__ void k_mix_apply(MixArgs a) {
    const Layout& L = a.L;
    const long long n = L.cells();
    const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (t >= n) return;
    const int i = (int)(t % L.nx), j = (int)((t / L.nx) % L.ny), k = (int)(t / ((long long)L.nx * L.ny));
    const long long c = L.at(i, j, k);
    const int par = a.ctl->parity;
    const float dtf = f64_to_f32(a.ctl->dt_apply);
    const float cf = dtf * (a.geo[0][i + a.goff[0]].ih * a.geo[1][j + a.goff[1]].ih * a.geo[2][k + a.goff[2]].ih);
    double* U = a.U[par];
    float* R = a.R[par];
#pragma unroll
    for (int v = 0; v < NV; ++v) {
        U[(long long)v * L.plane + c] += f32_to_f64(cf * R[(long long)v * L.plane + c]);
        R[(long long)v * L.plane + c] = 0.0f;
    }
}

__global__ void k_mix_clear_pending(Ctl* ctl) { ctl->dt_apply = 0.0; }

template <int ND, int SOLVER>
void launch_step(const MixedBufs& mb, const MixArgs& a, cudaStream_t st) {
    k_mix_step<ND, SOLVER><<<mb.grid, mb.tx * mb.ty, mb.smem, st>>>(a);
}

template <int ND, int SOLVER>
cudaError_t set_smem_attr(size_t bytes) {
    return cudaFuncSetAttribute(k_mix_step<ND, SOLVER>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
}

template <int ND, int SOLVER>
int occupancy(int threads, size_t bytes) {
    int nb = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_mix_step<ND, SOLVER>, threads, bytes);
    return nb;
}

MixArgs make_args(const MixedBufs& mb) {
    MixArgs a;
    a.L = mb.L;
    a.U[0] = mb.U[0]; a.U[1] = mb.U[1];
    a.R[0] = mb.R[0]; a.R[1] = mb.R[1];
    for (int ax = 0; ax < 3; ++ax) a.geo[ax] = mb.geo[ax];
    a.goff[0] = mb.L.gx; a.goff[1] = mb.L.gy; a.goff[2] = mb.L.gz;
    a.ctl = mb.ctl;
    a.mp = mb.mp;
    a.tx = mb.tx; a.ty = mb.ty;
    a.ncx = (mb.L.nx + mb.tx - 1) / mb.tx;
    const int ncy = mb.L.nd >= 2 ? (mb.L.ny + mb.ty - 1) / mb.ty : 1;
    a.total = (long long)a.ncx * ncy * (mb.L.nd == 3 ? mb.L.nz : 1);
    a.per_cta = mb.planes_per_cta;
    return a;
}

size_t smem_bytes(int nd, int tx, int ty) {
    if (nd == 3) return Smem<3>::bytes(tx, ty);
    if (nd == 2) return Smem<2>::bytes(tx, ty);
    return Smem<1>::bytes(tx, ty);
}

template <class F>
auto dispatch(int nd, int solver, F&& f) {
    if (nd == 3) return solver == TS_RS_HLLC ? f.template operator()<3, TS_RS_HLLC>() : f.template operator()<3, TS_RS_ROE_PIKE>();
    if (nd == 2) return solver == TS_RS_HLLC ? f.template operator()<2, TS_RS_HLLC>() : f.template operator()<2, TS_RS_ROE_PIKE>();
    return solver == TS_RS_HLLC ? f.template operator()<1, TS_RS_HLLC>() : f.template operator()<1, TS_RS_ROE_PIKE>();
}

}  // namespace

ts_status mixed_set_tile(MixedBufs& mb, int tx, int ty, std::string& err) {
    const int nd = mb.L.nd;
    if (nd == 1) ty = 1;
    if (tx < 4 || ty < 1 || tx * ty > 256 || (tx * ty) % 32 != 0) {
        err = "tile must have 32..256 threads in whole warps";
        return TS_ERR_INVALID;
    }
    const size_t bytes = smem_bytes(nd, tx, ty);
    if (bytes > 227 * 1024) { err = "tile needs too much shared memory"; return TS_ERR_INVALID; }
    const int solver = mb.mp.solver;
    cudaError_t e = dispatch(nd, solver, [&]<int ND, int S>() { return set_smem_attr<ND, S>(bytes); });
    if (e != cudaSuccess) { err = std::string("cudaFuncSetAttribute: ") + cudaGetErrorString(e); return TS_ERR_CUDA; }
    const int per_sm = dispatch(nd, solver, [&]<int ND, int S>() { return occupancy<ND, S>(tx * ty, bytes); });
    if (per_sm < 1) { err = "mixed kernel does not fit on an SM with this tile"; return TS_ERR_UNSUPPORTED; }
    mb.tx = tx;
    mb.ty = ty;
    mb.smem = bytes;
    const int ncx = (mb.L.nx + tx - 1) / tx;
    const int ncy = nd >= 2 ? (mb.L.ny + ty - 1) / ty : 1;
    const long long total = (long long)ncx * ncy * (nd == 3 ? mb.L.nz : 1);
    const long long slots = (long long)mb.sms * per_sm;
    long long per = (total + slots - 1) / slots;
    if (per < 1) per = 1;
    mb.planes_per_cta = (int)per;
    mb.grid = (int)((total + per - 1) / per);
    return TS_OK;
}

ts_status mixed_init(const ts_config& c, const Layout& L, const Phys& ph, const HostGrid& g, Ctl* ctl,
                     const DeviceAlloc& alloc, MixedBufs& mb, std::string& err) {
    mb.L = L;
    mb.ctl = ctl;
    ts_status s;
    for (int b = 0; b < 2; ++b) {
        if ((s = alloc(sizeof(double) * NV * L.plane, (void**)&mb.U[b])) != TS_OK) return s;
        if ((s = alloc(sizeof(float) * NV * L.plane, (void**)&mb.R[b])) != TS_OK) return s;
        if (cudaMemset(mb.U[b], 0, sizeof(double) * NV * L.plane) != cudaSuccess ||
            cudaMemset(mb.R[b], 0, sizeof(float) * NV * L.plane) != cudaSuccess) {
            err = "cudaMemset failed";
            return TS_ERR_CUDA;
        }
    }
    // per-axis geometry with GHOST ghost entries on active axes
    bool uniform = true;
    for (int a = 0; a < 3; ++a) {
        const std::vector<double>& X = a == 0 ? g.x : (a == 1 ? g.y : g.z);
        const std::vector<double>& Hh = a == 0 ? g.hx : (a == 1 ? g.hy : g.hz);
        const int n = L.n(a);
        const int gw = a == 0 ? L.gx : (a == 1 ? L.gy : L.gz);
        std::vector<AxisGeo> geo(n + 2 * gw);
        auto xc = [&](int i) {  // centre of cell i (reference ghosts at -1 and n, beyond extrapolated)
            if (i >= -1 && i <= n) return X[i + 1];
            if (i < -1) return X[0] - (double)(-1 - i) * Hh[0];
            return X[n + 1] + (double)(i - n) * Hh[n + 1];
        };
        auto hc = [&](int i) { return Hh[std::min(std::max(i, -1), n) + 1]; };
        if (gw == 0) {
            geo[0] = AxisGeo{(float)Hh[0], (float)(0.5 * Hh[0]), 0.f, 0.f, 0.f, (float)(1.0 / Hh[0])};
        } else {
            for (int i = -gw; i < n + gw; ++i) {
                // periodic axes take the source cell's geometry for ghost entries
                int src = i;
                if (c.periodic[a] && (i < 0 || i >= n)) src = (i + n) % n;
                const double h = hc(src);
                const double xm = xc(src - 1), x0 = xc(src), xp = xc(src + 1);
                AxisGeo e;
                e.h = (float)h;
                e.hh = (float)(0.5 * h);
                e.ks = (float)(0.5 * h / (xp - xm));
                e.il = (float)(1.0 / (x0 - xm));
                e.ir = (float)(1.0 / (xp - x0));
                e.ih = (float)(1.0 / (i >= n || i < 0 ? hc(i) : h));
                geo[i + gw] = e;
                if (i >= 0 && i < n && Hh[i + 1] != Hh[1]) uniform = false;
            }
        }
        void* d;
        if ((s = alloc(sizeof(AxisGeo) * geo.size(), &d)) != TS_OK) return s;
        if (cudaMemcpy(d, geo.data(), sizeof(AxisGeo) * geo.size(), cudaMemcpyHostToDevice) != cudaSuccess) {
            err = "geometry upload failed";
            return TS_ERR_CUDA;
        }
        mb.geo[a] = (const AxisGeo*)d;
    }
    MixPhys& m = mb.mp;
    m.nd = L.nd;
    m.recon = c.reconstruction;
    m.limiter = c.limiter;
    m.solver = c.riemann_solver;
    m.eos = c.eos;
    for (int a = 0; a < 3; ++a) m.periodic[a] = ph.periodic[a];
    m.uniform = uniform;
    m.gamma = (float)ph.gamma;
    m.gm1 = (float)(ph.gamma - 1.0);
    m.pinf = (float)ph.p_inf;
    m.einf_d = c.eos == TS_EOS_STIFFENED_GAS ? ph.gamma * ph.p_inf / (ph.gamma - 1.0) : 0.0;
    m.einf = (float)m.einf_d;
    m.eps = (float)ph.eps;
    m.cfl = ph.cfl;
    for (int sd = 0; sd < 6; ++sd) {
        m.bc_type[sd] = ph.bc.type[sd];
        const double r = ph.bc.density[sd];
        const double vx = ph.bc.vel[sd][0], vy = ph.bc.vel[sd][1], vz = ph.bc.vel[sd][2];
        m.bc_state[sd][0] = (float)r;
        m.bc_state[sd][1] = (float)(r * vx);
        m.bc_state[sd][2] = (float)(r * vy);
        m.bc_state[sd][3] = (float)(r * vz);
        // inlet ghost energy, shifted: p/(g-1) + rho|v|^2/2 (the p_inf terms cancel)
        m.bc_state[sd][4] = (float)(ph.bc.pstatic[sd] / (ph.gamma - 1) + 0.5 * r * (vx * vx + vy * vy + vz * vz));
        for (int a = 0; a < 3; ++a) m.bc_vel[sd][a] = (float)ph.bc.vel[sd][a];
    }
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&mb.sms, cudaDevAttrMultiProcessorCount, dev);
    const int tx = L.nd == 1 ? 256 : 32;
    const int ty = L.nd == 1 ? 1 : 8;
    return mixed_set_tile(mb, tx, ty, err);
}

void mixed_step(MixedBufs& mb, const Phys&, cudaStream_t st, cudaEvent_t* ev, int* n_launch, const char** names) {
    const MixArgs a = make_args(mb);
    if (ev) cudaEventRecord(ev[0], st);
    dispatch(mb.L.nd, mb.mp.solver, [&]<int ND, int S>() { launch_step<ND, S>(mb, a, st); return 0; });
    if (ev) cudaEventRecord(ev[1], st);
    if (names) names[0] = "k_mix_step";
    if (n_launch) *n_launch = 1;
}

void mixed_reset(MixedBufs& mb, cudaStream_t st) {
    // caller has set parity 0 and dt_apply 0 in the control word
    cudaMemsetAsync(mb.R[0], 0, sizeof(float) * NV * mb.L.plane, st);
}

void mixed_materialize(MixedBufs& mb, const Phys&, cudaStream_t st) {
    const MixArgs a = make_args(mb);
    const long long n = mb.L.cells();
    k_mix_apply<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(a);
    k_mix_clear_pending<<<1, 1, 0, st>>>(mb.ctl);
}

double* mixed_state(MixedBufs& mb, int parity) { return mb.U[parity & 1]; }

}  // namespace ts

// ---------------------------------------------------------------------------
// ts_advance_noalloc: the fused mixed-precision step for callers that may not
// allocate device memory.  Everything the kernel needs beyond the caller's
// input and output -- both state buffers, both residual buffers, the grid
// geometry and the control word -- lives in one fixed array in device memory
// that is part of this library's module.
// ---------------------------------------------------------------------------
namespace ts {
namespace noalloc {

constexpr size_t kNaPlane = TS_NOALLOC_MAX_PLANE;
constexpr size_t kNaGeo = kNaPlane + 16;  // AxisGeo entries of all three axes together
constexpr size_t kNaBytes = 2 * NV * kNaPlane * sizeof(double) + 2 * NV * kNaPlane * sizeof(float) +
                            kNaGeo * sizeof(AxisGeo) + sizeof(Ctl) + 16 * 256;

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNaBytes];

constexpr int kNaMaxDevices = 64;
std::mutex g_noalloc_mutex;
void* g_noalloc_base[kNaMaxDevices] = {};

__global__ void k_na_scatter(const double* __restrict__ aos, Layout L, double* __restrict__ U) {
    const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (t >= L.cells()) return;
    const int i = (int)(t % L.nx), j = (int)((t / L.nx) % L.ny), k = (int)(t / ((long long)L.nx * L.ny));
    const long long c = L.at(i, j, k);
#pragma unroll
    for (int v = 0; v < NV; ++v) U[(long long)v * L.plane + c] = aos[t * NV + v];
}

__global__ void k_na_gather(double* __restrict__ aos, Layout L, const double* __restrict__ U0,
                            const double* __restrict__ U1, const Ctl* ctl) {
    const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (t >= L.cells()) return;
    const double* U = ctl->parity ? U1 : U0;
    const int i = (int)(t % L.nx), j = (int)((t / L.nx) % L.ny), k = (int)(t / ((long long)L.nx * L.ny));
    const long long c = L.at(i, j, k);
#pragma unroll
    for (int v = 0; v < NV; ++v) aos[t * NV + v] = U[(long long)v * L.plane + c];
}

}  // namespace noalloc
}  // namespace ts

using namespace ts;
using namespace ts::noalloc;

extern "C" ts_status ts_advance_noalloc(const ts_config* cfg, const double* state_in, double* state_out,
                                        int32_t n_steps, void* stream, ts_step_info* info) {
    if (!cfg || !state_in || !state_out) return fail(TS_ERR_INVALID, "NULL argument");
    if (n_steps < 0) return fail(TS_ERR_INVALID, "n_steps must be >= 0");
    if (cfg->precision != TS_PRECISION_MIXED)
        return fail(TS_ERR_UNSUPPORTED, "ts_advance_noalloc runs the mixed-precision step only");
    HostGrid grid;
    std::string err;
    ts_status s = build_grid(*cfg, grid, err);
    if (s != TS_OK) return fail(s, err);
    const Layout L = make_layout(*cfg);
    const size_t geo_entries = (size_t)(L.nx + 2 * L.gx) + (L.ny + 2 * L.gy) + (L.nz + 2 * L.gz);
    if ((size_t)L.plane > kNaPlane || geo_entries > kNaGeo)
        return fail(TS_ERR_INVALID, "grid too large for ts_advance_noalloc: a padded variable plane holds " +
                                        std::to_string(L.plane) + " elements, the limit is " +
                                        std::to_string(kNaPlane));
    int dev = cfg->device, ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || dev < 0 || dev >= ndev || dev >= kNaMaxDevices)
        return fail(TS_ERR_INVALID, "device ordinal out of range");
    int prev = -1;
    cudaGetDevice(&prev);
    if (prev != dev && cudaSetDevice(dev) != cudaSuccess) return fail(TS_ERR_CUDA, "cudaSetDevice failed");
    struct Restore {
        int prev, dev;
        ~Restore() { if (prev >= 0 && prev != dev) cudaSetDevice(prev); }
    } restore{prev, dev};

    // Once per device, with that device current: the scratch array's device
    // address (the host-side symbol is not a device pointer).
    unsigned char* base;
    {
        std::lock_guard<std::mutex> lock(g_noalloc_mutex);
        if (!g_noalloc_base[dev]) {
            void* p = nullptr;
            cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
            if (e != cudaSuccess || !p)
                return fail(TS_ERR_CUDA, std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e));
            g_noalloc_base[dev] = p;
        }
        base = static_cast<unsigned char*>(g_noalloc_base[dev]);
    }
    // bump allocation inside the scratch array
    size_t off = 0;
    auto carve = [&](size_t bytes, void** out) -> ts_status {
        off = (off + 255) & ~size_t(255);
        if (off + bytes > kNaBytes) return fail(TS_ERR_INVALID, "ts_advance_noalloc scratch exhausted");
        *out = base + off;
        off += bytes;
        return TS_OK;
    };
    Ctl* ctl = nullptr;
    if ((s = carve(sizeof(Ctl), (void**)&ctl)) != TS_OK) return s;
    MixedBufs mb;
    const Phys ph = make_phys(*cfg);
    if ((s = mixed_init(*cfg, L, ph, grid, ctl, carve, mb, err)) != TS_OK) return fail(s, err);

    cudaStream_t st = static_cast<cudaStream_t>(stream);
    Ctl c;
    std::memset(&c, 0, sizeof c);
    c.time = info ? info->time : 0.0;
    c.iteration = info ? info->iteration : 0;
    c.next_sol = info ? info->next_solution_time : cfg->save_solution_time;
    c.next_slice = info ? info->next_slice_time : cfg->save_slice_time;
    c.max_iteration = cfg->max_iteration;
    c.max_time = cfg->max_time;
    c.save_sol = cfg->save_solution_time;
    c.save_slice = cfg->save_slice_time;
#define NA_CUDA(call)                                                                                    \
    do {                                                                                                 \
        cudaError_t e_ = (call);                                                                         \
        if (e_ != cudaSuccess) return fail(TS_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
    } while (0)
    NA_CUDA(cudaMemcpyAsync(ctl, &c, sizeof c, cudaMemcpyHostToDevice, st));
    NA_CUDA(cudaMemsetAsync(mb.R[0], 0, sizeof(float) * NV * L.plane, st));
    const unsigned blocks = (unsigned)((L.cells() + 255) / 256);
    k_na_scatter<<<blocks, 256, 0, st>>>(state_in, L, mb.U[0]);
    for (int k = 0; k < n_steps; ++k) mixed_step(mb, ph, st);
    mixed_materialize(mb, ph, st);
    k_na_gather<<<blocks, 256, 0, st>>>(state_out, L, mb.U[0], mb.U[1], ctl);
    NA_CUDA(cudaGetLastError());
    NA_CUDA(cudaMemcpyAsync(&c, ctl, sizeof c, cudaMemcpyDeviceToHost, st));
    NA_CUDA(cudaStreamSynchronize(st));
#undef NA_CUDA
    if (info) {
        info->iteration = c.iteration;
        info->health = c.health;
        info->time = c.time;
        info->dt = c.dt;
        info->next_solution_time = c.next_sol;
        info->next_slice_time = c.next_slice;
        for (int v = 0; v < NV; ++v) info->residual[v] = 0.0;
    }
    return TS_OK;
}
