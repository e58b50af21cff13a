// FP32 building blocks of the mixed-precision step, shared by the fused
// kernels: FP64 <-> FP32 conversions on the integer pipe, ghost-index
// resolution, boundary-condition images and the FP32 Riemann solvers.
#pragma once

#include <cuda_runtime.h>

#include "ts_mixed.h"

namespace ts {
namespace mix32 {

// ---------------------------------------------------------------------------
// FP64 <-> FP32 on the integer pipe
// ---------------------------------------------------------------------------
// Round-to-nearest FP64 -> FP32 (ties away from zero) for finite values with
// |x| < 2^128; |x| < 2^-126 gives a signed zero (the FP32 path runs
// flush-to-zero).  Six integer operations instead of a conversion on the
// FP64 pipe: half an FP32 ulp (bit 28 of the low word) is added to the
// magnitude, the carry running into the exponent where the mantissa
// overflows, and the top 23 mantissa bits are kept.
__device__ __forceinline__ float f64_to_f32(double d) {
    const unsigned int hi = (unsigned int)__double2hiint(d);
    const unsigned int lo = (unsigned int)__double2loint(d);
    unsigned int rlo, rhi;
    asm("add.cc.u32 %0, %2, 0x10000000;\n\taddc.u32 %1, %3, 0;" : "=r"(rlo), "=r"(rhi) : "r"(lo), "r"(hi));
    const unsigned int sign = hi & 0x80000000u;
    const unsigned int t = __funnelshift_l(rlo, rhi - 0x38000000u, 3);
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

// BC table entry of boundary face f of `side` (ts_internal.h: face_index).
__device__ __forceinline__ int bc_id32(const MixPhys& p, int side, int f) { return bc_id(p.mark, side, f); }

// Boundary-condition image of a state (shifted energy) for BC table entry
// `side` (a domain side, or the kind its marker selected) on axis A.
__device__ __forceinline__ void bc32(const MixPhys& p, int side, int A, float w[NV]) {
    // entries 0-5 inline, 6.. from the extra-kinds table
    const bool extra = side >= 6;
    const int t = extra ? p.kinds->type[side - 6] : p.bc_type[side];
    if (t == TS_BC_SYMMETRY) {
        w[1 + A] = -w[1 + A];
    } else if (t == TS_BC_WALL) {
        w[1] = -w[1]; w[2] = -w[2]; w[3] = -w[3];
    } else if (t == TS_BC_MOVING_WALL) {
        const float* bv = extra ? p.kinds->vel[side - 6] : p.bc_vel[side];
        const float r = w[0], ir = 1.0f / r;
        const float vx = w[1] * ir, vy = w[2] * ir, vz = w[3] * ir;
        const float dx = 2.0f * bv[0] - vx, dy = 2.0f * bv[1] - vy, dz = 2.0f * bv[2] - vz;
        w[1] = r * dx; w[2] = r * dy; w[3] = r * dz;
        w[4] = w[4] + 0.5f * r * ((dx * dx + dy * dy + dz * dz) - (vx * vx + vy * vy + vz * vz));
    } else if (t == TS_BC_SUBSONIC_INLET) {
        const float* bs = extra ? p.kinds->state[side - 6] : p.bc_state[side];
#pragma unroll
        for (int v = 0; v < NV; ++v) w[v] = bs[v];
    }
}


__device__ __forceinline__ float harten32(float z, float e) {
    z = fabsf(z);
    return (z < e) ? ((z * z) / e + e) * 0.5f : z;
}

__device__ __forceinline__ float pick3(int a, float x, float y, float z) { return a == 0 ? x : (a == 1 ? y : z); }

// ---------------------------------------------------------------------------
// FP32 Riemann solvers along axis A (a compile-time argument: the normal
// components fold into register choices).  States carry the shifted energy
// E' = E - einf, so p = (g-1)(E' - rho |u|^2 / 2) for both equations of state
// without cancellation; E = E' + einf where the total energy enters.
// ---------------------------------------------------------------------------

// Roe-Pike flux (RoeSolverPerfectGasEOS.h:74-160) in the equivalent form
// 1/2 [F(UL) + F(UR) + |A|(UL - UR)], returned without the factor 1/2
// (flux_scale<SOLVER>), |A| dU = a1 dU + Ac Qa + Bc Qb with
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
    const float un = pick3(A, ux, uy, uz);
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
    const float dR = 0.5f * gm1 * q2 * dr - gm1 * (ux * dmx + uy * dmy + uz * dmz - de);
    const float dD = pick3(A, dmx, dmy, dmz) - dr * un;
    const float Ac = Ea * dR + Eb * dD;
    const float Bc = Ea * dD + Eb * dR * (ic * ic);
    const float unl = pick3(A, ulx, uly, ulz), unr = pick3(A, urx, ury, urz);
    const float pn = pl + pr + Ac;
    // twice the flux: the factor 1/2 is applied with the face areas
    F[0] = UL[0] * unl + UR[0] * unr + a1 * dr + Bc;
    F[1] = UL[1] * unl + UR[1] * unr + (A == 0 ? pn : 0.0f) + a1 * dmx + Bc * ux;
    F[2] = UL[2] * unl + UR[2] * unr + (A == 1 ? pn : 0.0f) + a1 * dmy + Bc * uy;
    F[3] = UL[3] * unl + UR[3] * unr + (A == 2 ? pn : 0.0f) + a1 * dmz + Bc * uz;
    F[4] = el * unl + er * unr + a1 * de + Ac * un + Bc * h;
    return lam;
}

// HLLC (Toro ch. 10.4), Einfeldt-type speeds from Roe averages.
template <int A>
__device__ __forceinline__ float hllc32(const MixPhys& p, const float UL[NV], const float UR[NV],
                                        float F[NV]) {
    const float g = p.gamma, gm1 = p.gm1;
    const float rl = 1.0f / UL[0], rr = 1.0f / UR[0];
    const float vlx = UL[1] * rl, vly = UL[2] * rl, vlz = UL[3] * rl;
    const float vrx = UR[1] * rr, vry = UR[2] * rr, vrz = UR[3] * rr;
    const float pl = gm1 * (UL[4] - 0.5f * UL[0] * (vlx * vlx + vly * vly + vlz * vlz));
    const float pr = gm1 * (UR[4] - 0.5f * UR[0] * (vrx * vrx + vry * vry + vrz * vrz));
    const float El = UL[4] + p.einf, Er = UR[4] + p.einf;
    const float cl = sqrtf(g * (pl + p.pinf) * rl), cr = sqrtf(g * (pr + p.pinf) * rr);
    const float sl = UL[0] * rsqrtf(UL[0]), sr = UR[0] * rsqrtf(UR[0]);
    const float inv = 1.0f / (sl + sr);
    const float wl = sl * inv, wr = sr * inv;
    const float ul = pick3(A, vlx, vly, vlz), ur = pick3(A, vrx, vry, vrz);
    const float ut = wl * ul + wr * ur;
    const float vtx = wl * vlx + wr * vrx, vty = wl * vly + wr * vry, vtz = wl * vlz + wr * vrz;
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
    const float vx = left ? vlx : vrx, vy = left ? vly : vry, vz = left ? vlz : vrz;
    const float uk = left ? ul : ur, pk = left ? pl : pr, Ek = left ? El : Er, rk = left ? rl : rr;
    const float Sk = left ? SL : SR, mk = left ? ml : mr;
    F[0] = U[0] * uk;
    F[1] = U[1] * uk + (A == 0 ? pk : 0.0f);
    F[2] = U[2] * uk + (A == 1 ? pk : 0.0f);
    F[3] = U[3] * uk + (A == 2 ? pk : 0.0f);
    F[4] = (Ek + pk) * uk;
    if (!supl && !supr) {
        const float coef = mk / (Sk - ss);
        F[0] += Sk * (coef - U[0]);
        F[1] += Sk * (coef * (A == 0 ? ss : vx) - U[1]);
        F[2] += Sk * (coef * (A == 1 ? ss : vy) - U[2]);
        F[3] += Sk * (coef * (A == 2 ? ss : vz) - U[3]);
        F[4] += Sk * (coef * (Ek * rk + (ss - uk) * (ss + pk / mk)) - Ek);
    }
    return fmaxf(fabsf(SL), fabsf(SR));
}

// Factor between the stored face flux and the flux.
template <int SOLVER>
__device__ __forceinline__ constexpr float flux_scale() { return SOLVER == TS_RS_HLLC ? 1.0f : 0.5f; }

template <int SOLVER, int A>
__device__ __forceinline__ float flux32(const MixPhys& p, const float UL[NV], const float UR[NV], float F[NV]) {
    if (SOLVER == TS_RS_HLLC) return hllc32<A>(p, UL, UR, F);
    return roe32<A>(p, UL, UR, F);
}

// ---------------------------------------------------------------------------
// Step bookkeeping shared by the fused kernels
// ---------------------------------------------------------------------------
// The residual norms of a warp's cells (FP32 per thread) added in FP64 to the
// stage's accumulator: one atomic per variable per warp.  `live` lanes of
// the warp take part (`mask`); values from lanes beyond them are discarded.
__device__ __forceinline__ void add_norms(Ctl* ctl, const float (&nrm)[NV], unsigned int mask, int lane, int live) {
#pragma unroll
    for (int v = 0; v < NV; ++v) {
        double x = (double)nrm[v];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            const double y = __shfl_down_sync(mask, x, o);
            if (lane + o < live) x += y;
        }
        if (lane == 0 && x != 0.0) atomicAdd(&ctl->res_acc[v], x);
    }
}

// dt of one problem from its CFL maximum, and the step's bookkeeping
// (ComputeTimeStep :1427-1437, time += dt and iteration++ :1486-1487, and the
// Kernel::Run snapshot/termination rules kernel.h:1763-1846).
__device__ __forceinline__ void finish_with(Ctl* ctl, float m, double cfl) {
    double dt = cfl / (double)m;
    if ((ctl->save_sol > 0) && (ctl->next_sol < ctl->time + dt)) dt = ctl->next_sol - ctl->time;
    if ((ctl->save_slice > 0) && (ctl->next_slice < ctl->time + dt)) dt = ctl->next_slice - ctl->time;
    ctl->dt_min_raw = 1.0 / (double)m;
    // the stage's residual norms (zeros when they are not formed)
#pragma unroll
    for (int v = 0; v < NV; ++v) {
        ctl->res[v] = ctl->res_acc[v];
        ctl->res_acc[v] = 0.0;
    }
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

__device__ __forceinline__ void finish_problem(Ctl* ctl, double cfl) {
    finish_with(ctl, __uint_as_float(*(volatile unsigned int*)&ctl->srmax_bits), cfl);
}

}  // namespace mix32
}  // namespace ts
