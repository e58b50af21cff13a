// Mixed-precision explicit FVM step on GB300: one fused, persistent kernel
// per RK stage, over a work list of one or many problems.
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
// This file holds the 1D and 2D kernels (3D problems run the TMA-staged
// k_mix3d of ts_mix3d.cu, on the same descriptors and control words).
//
// Work items.  A problem is cut into one-row tiles of TX cells along x (one
// thread per cell plus two halo threads at each end) and, in 2D, chunks of
// rows; one item is one (problem, tile, chunk).  A 2D item marches y through
// its chunk (2.5D blocking), keeping three rows of the FP32 working state, a
// 2-row ring of limited half-slopes and the face fluxes in shared memory.
// Every thread has fixed roles: one working-state position of the row (the
// next row's loads are issued into registers as soon as the current row is
// stored, so their latency hides behind the row's compute), at most one
// reconstruction position, the x face left of its cell (thread TX: the far
// face), the y face above its cell, and its cell's residual.  Items are
// indexed chunk-major and dealt round-robin to the persistent CTAs, so CTAs
// running at the same time sweep neighbouring tiles at the same y and share
// halo cells through L2.  Each problem has its own control word: the CTA that
// completes a problem's last item turns its CFL maximum into that problem's
// dt, so many problems of different sizes advance with their own time steps
// in one launch.  The last few long 1D problems of a batch run in the
// cluster tail kernel (k_mix_tail) instead: state on chip, many stages per
// launch.
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
#include <cooperative_groups.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "ts_flux32.cuh"
#include "ts_mixed.h"

namespace ts {
namespace {

constexpr int HB = 2;  // halo of the working-state box

using namespace mix32;

// ---------------------------------------------------------------------------
// Compile-time tile geometry and shared-memory layout (floats)
// ---------------------------------------------------------------------------
// Kernel axes: 0 = x, 1 = the tile's second axis (3D only), 2 = the marching
// axis (z in 3D, y in 2D).  ProbDesc maps each kernel axis to the problem's
// geometry, extent, strides and physical direction.
//
// One-row tiles (1D problems, and 2D problems marching along y): NT_
// threads own NT_ - 4 cells along x, so every thread has exactly one box
// position, at most one reconstruction position and at most one face per
// axis.  Kernel axis 1 of these problems is the inactive one (one cell).
template <int NT_, bool MARCH_>
struct Tile {
    static constexpr bool MARCH = MARCH_;
    static constexpr int NT = NT_;
    static constexpr int TX = NT - 2 * HB;                 // cells along x
    static constexpr int NAX = MARCH ? 2 : 1;              // active axes: x and the marching axis
    static constexpr int AZ = 1;                           // slope slot of the marching axis
    static constexpr int BX = TX + 2 * HB;                 // working-state box (one position per thread)
    static constexpr int RX = TX + 2;                      // reconstruction ring
    static constexpr int WS = MARCH ? 3 : 1;               // working-state planes kept
    static constexpr int DS = MARCH ? 2 : 1;               // slope planes kept
    static constexpr int W_OFF = 0;
    static constexpr int D_OFF = W_OFF + WS * NV * BX;
    static constexpr int FX_OFF = D_OFF + DS * NAX * NV * RX;
    static constexpr int FZ_OFF = FX_OFF + 6 * (TX + 1);
    static constexpr int TOTAL = FZ_OFF + (MARCH ? 2 * 6 * TX : 0);
    static constexpr size_t BYTES = (size_t)TOTAL * sizeof(float);
    static_assert(BX == NT && RX <= NT, "one box position and at most one ring position per thread");
    // resident CTAs per SM the register allocation is sized for: about 28
    // warps per SM for tiles that do not march (a 4096-tube batch took 2.00 s
    // at 77 registers, 6 CTAs of 128 threads per SM, and 1.81 s sized for 28
    // warps), 24 for marching tiles (which spill at 28; sized for 16 warps, a
    // single 1024^2 problem ran 1.5 % faster but batches of problems 17 %
    // slower)
    static constexpr int WARPS = (NT + 31) / 32;
    static constexpr int MINB = WARPS >= 16 ? 2 : ((MARCH ? 24 : 28) + WARPS - 1) / WARPS;

    static __device__ __forceinline__ int wslot(int p) { return (p + 3) % 3; }
    static __device__ __forceinline__ int w(int s, int v, int box) { return W_OFF + (s * NV + v) * BX + box; }
    static __device__ __forceinline__ int d(int s, int ax, int v, int ring) {
        return D_OFF + ((s * NAX + ax) * NV + v) * RX + ring;
    }
    static __device__ __forceinline__ int fx(int v, int x) { return FX_OFF + v * (TX + 1) + x; }
    static __device__ __forceinline__ int fz(int s, int v, int x) { return FZ_OFF + (s * 6 + v) * TX + x; }
    // the cell x of this thread in the tile; false if it owns none
    static __device__ __forceinline__ bool cell(int tid, int& x) {
        x = tid;
        return tid < TX;
    }
};

// Problem axis of kernel axis AX (0 or the marching axis 2): one-row
// marching tiles serve 2D problems (x, -, y), the others 1D problems (x).
template <class T, int AX>
__device__ __forceinline__ constexpr int phys_axis() {
    return AX == 0 ? 0 : 1;
}

__device__ __forceinline__ int dslot(int p) { return (p + 2) & 1; }

// The working-state position of a thread: where its source cell lives in a
// plane and how to turn it into the working copy.
struct BoxPos {
    int off;        // element offset of the source cell within a plane; -1: not used
    int box;        // box index in shared memory
    float cfxy;     // 1 / (h0 h1) of the source cell (kernel axes 0 and 1)
    int xs;         // boundary side applied after mirroring, or -1
    bool own;       // the cell belongs to this tile: write U^{n+1}
};

struct Prefetch {
    double u[NV];
    float r[NV];
};

template <class T>
__device__ __forceinline__ void setup_box(const ProbDesc& d, int i0, BoxPos& bp) {
    const int lx = threadIdx.x;
    bp.off = -1;
    const int dx = lx < HB ? HB - lx : (lx >= T::TX + HB ? lx - T::TX - HB + 1 : 0);
    const int gi = i0 + lx - HB;
    if (gi >= d.kn[0] + HB) return;
    int si;
    resolve(gi, d.kn[0], d.kper[0], 0, si, bp.xs);
    bp.off = si;
    bp.box = lx;
    bp.cfxy = __ldg(&d.kgeo[0][si + d.kgoff[0]].ih) * __ldg(&d.kgeo[1][d.kgoff[1]].ih);
    bp.own = dx == 0 && gi < d.kn[0];
}

// Source plane of marching index p (wrapped or mirrored), and the boundary
// side to apply (-1: none).
template <class T>
__device__ __forceinline__ int plane_of(const ProbDesc& d, int p, int& zs) {
    int sk = 0;
    zs = -1;
    if (T::MARCH) resolve(p, d.kn[2], d.kper[2], 2 * d.kphys[2], sk, zs);
    return sk;
}

// Issue the loads of plane p (FP64 state and FP32 pending residual) into registers.
template <class T>
__device__ __forceinline__ void issue(const ProbDesc& d, const double* __restrict__ Uin,
                                      const float* __restrict__ Rin, int p, const BoxPos& bp, Prefetch& pf) {
    const long long plane = d.L.plane;
    int zs;
    const int sk = plane_of<T>(d, p, zs);
    if (bp.off < 0) return;
    const long long c = d.kbase + sk * d.kstr[2] + bp.off;
#pragma unroll
    for (int v = 0; v < NV; ++v) pf.u[v] = __ldcg(Uin + v * plane + c);
#pragma unroll
    for (int v = 0; v < NV; ++v) pf.r[v] = __ldcg(Rin + v * plane + c);
}

// Turn the prefetched plane p into the FP32 working copy in shared memory and
// write U^{n+1} = U^n + dt R^n / V for the owned cells of planes [z0, z1).
template <class T>
__device__ __forceinline__ void store(const ProbDesc& d, float* sm, double* __restrict__ Uout, int p, int z0, int z1,
                                      float dtf, const BoxPos& bp, const Prefetch& pf, unsigned int& health) {
    const MixPhys& mp = d.mp;
    const long long plane = d.L.plane;
    int zs = -1;
    const int sk = plane_of<T>(d, p, zs);
    const long long zoff = d.kbase + sk * d.kstr[2];
    const float cfz = dtf * __ldg(&d.kgeo[2][sk + d.kgoff[2]].ih);
    const int slot = T::MARCH ? T::wslot(p) : 0;
    const bool own_plane = p >= z0 && p < z1;
    if (bp.off < 0) return;
    const float cf = bp.cfxy * cfz;
    float inc[NV], w[NV];
#pragma unroll
    // explicitly rounded products and FMAs (never split or re-fused by the
    // compiler): store() is inlined at several call sites, and a row's
    // working copy must be the same bits in the CTA that owns the row and in
    // the CTA that loads it as a halo row of its chunk
    for (int v = 0; v < NV; ++v) inc[v] = __fmul_rn(cf, pf.r[v]);
#pragma unroll
    for (int v = 0; v < 4; ++v) w[v] = __fmaf_rn(cf, pf.r[v], f64_to_f32(pf.u[v]));
    w[4] = __fmaf_rn(cf, pf.r[4],
                     mp.eos == TS_EOS_STIFFENED_GAS ? f64_to_f32(pf.u[4] - mp.einf_d) : f64_to_f32(pf.u[4]));
    // BC of the boundary face of this ghost's row (the x sides' faces are
    // numbered by the plane, the marching sides' by x)
    if (bp.xs >= 0) bc32(mp, bc_id32(mp, bp.xs, sk), 0, w);
    if (T::MARCH && zs >= 0) bc32(mp, bc_id32(mp, zs, bp.off), phys_axis<T, 2>(), w);
#pragma unroll
    for (int v = 0; v < NV; ++v) sm[T::w(slot, v, bp.box)] = w[v];
    if (own_plane && bp.own) {
        const long long c = zoff + bp.off;
        double un[NV];
#pragma unroll
        for (int v = 0; v < NV; ++v) {
            un[v] = pf.u[v] + f32_to_f64(inc[v]);
            __stcg(Uout + v * plane + c, un[v]);
        }
        // rho > 0 tested on the bit pattern (no FP64 comparison): positive
        // finite values and +inf are the integers 1 .. 0x7FF0000000000000
        const long long b = __double_as_longlong(un[0]);
        if (b <= 0 || b > 0x7FF0000000000000LL)
            health |= (b & 0x7FFFFFFFFFFFFFFFLL) > 0x7FF0000000000000LL ? TS_HEALTH_NAN : TS_HEALTH_NEG_DENSITY;
        if (!(w[4] == w[4])) health |= TS_HEALTH_NAN;
    }
}

// Ring slots of the marching planes around plane p (working state: p-1, p,
// p+1; slopes: p, p+1), computed once per plane.
struct Slots {
    int wm, w0, wp;  // working-state slots of planes p-1, p, p+1
    int d0, d1;      // slope slots of planes p, p+1
};

template <class T>
__device__ __forceinline__ Slots slots_of(int p) {
    Slots s;
    if (T::MARCH) {
        s.wm = T::wslot(p - 1); s.w0 = T::wslot(p); s.wp = T::wslot(p + 1);
        s.d0 = dslot(p); s.d1 = dslot(p + 1);
    } else {
        s.wm = s.w0 = s.wp = 0;
        s.d0 = s.d1 = 0;
    }
    return s;
}

// The reconstruction position of a thread for the current item (ring index
// = thread index): its box index and geometry entry (fixed while the item
// marches).
struct RingPos {
    int box;        // box index of the cell; -1: nothing to do
    int g0;         // geometry index along kernel axis 0
    float ks0;      // central-slope factor along kernel axis 0 (marching tiles)
};

template <class T>
__device__ __forceinline__ void setup_ring(const ProbDesc& d, int i0, RingPos& rp) {
    const int rx = threadIdx.x;
    rp.box = -1;
    if (rx >= T::RX) return;
    const int gi = i0 + rx - 1;
    if (gi > d.kn[0]) return;
    if ((gi < 0 || gi >= d.kn[0]) && !d.kper[0]) return;
    int si, xs;
    resolve(gi, d.kn[0], 1, 0, si, xs);
    rp.box = rx + 1;
    rp.g0 = si + d.kgoff[0];
    if (T::MARCH) rp.ks0 = d.kgeo[0][rp.g0].ks;
}

// Reconstruction kinds (the limiter choice folded in).
enum { RK_LINEAR = 1, RK_ENO2 = 2, RK_LIM_BJ = 3, RK_LIM_VK = 4 };

__host__ __device__ __forceinline__ int recon_kind(const MixPhys& mp) {
    if (mp.recon == TS_RECON_LINEAR_2POINTS) return RK_LINEAR;
    if (mp.recon == TS_RECON_ENO2_2POINTS) return RK_ENO2;
    if (mp.recon == TS_RECON_LINEAR_2POINTS_LIMITED)
        return mp.limiter == TS_LIM_VENKATAKRISHNAN ? RK_LIM_VK : RK_LIM_BJ;
    return 0;
}

// Limited half-slopes of plane p on the tile and its 1-cell ring; ring cells
// outside a non-periodic boundary are not needed.
template <class T, int KIND>
__device__ __forceinline__ void recon_k(const ProbDesc& d, float* sm, int p, const Slots& s, const RingPos& rp) {
    int sk = 0;
    if (T::MARCH) {
        if ((p < 0 || p >= d.kn[2]) && !d.kper[2]) return;
        int zs;
        resolve(p, d.kn[2], 1, 0, sk, zs);
    }
    AxisGeo gz;
    if (T::MARCH) gz = d.kgeo[2][sk + d.kgoff[2]];
    if (rp.box < 0) return;
    {
        const int t = threadIdx.x;
        const int box = rp.box;
        AxisGeo g[T::NAX];
        if (T::MARCH && (KIND == RK_LINEAR || KIND == RK_LIM_BJ)) {
            // central slopes need only ks, kept in registers while the item marches
            g[0].ks = rp.ks0;
        } else {
            g[0] = d.kgeo[0][rp.g0];
        }
        if (T::MARCH) g[T::AZ] = gz;
        float eps2 = 0.0f;
        if (KIND == RK_LIM_VK) {
            // eps^2 = (K (h1 ... hnd)^(1/nd))^3 with K = 5 (Limiters.h:93-96, Constants.h:11)
            float vol = g[0].h;
#pragma unroll
            for (int ax = 1; ax < T::NAX; ++ax) vol *= g[ax].h;
            eps2 = 125.0f * (T::NAX == 2 ? vol * sqrtf(vol) : vol * vol * vol);
        }
#pragma unroll
        for (int v = 0; v < NV; ++v) {
            const float w0 = sm[T::w(s.w0, v, box)];
            float nm[T::NAX], np[T::NAX];
            nm[0] = sm[T::w(s.w0, v, box - 1)];
            np[0] = sm[T::w(s.w0, v, box + 1)];
            if (T::MARCH) { nm[T::AZ] = sm[T::w(s.wm, v, box)]; np[T::AZ] = sm[T::w(s.wp, v, box)]; }
            float dd[T::NAX];
            if (KIND == RK_ENO2) {
#pragma unroll
                for (int ax = 0; ax < T::NAX; ++ax) {
                    const float gl = (w0 - nm[ax]) * g[ax].il, gr = (np[ax] - w0) * g[ax].ir;
                    dd[ax] = (fabsf(gl) < fabsf(gr) ? gl : gr) * g[ax].hh;
                }
            } else {
#pragma unroll
                for (int ax = 0; ax < T::NAX; ++ax) dd[ax] = (np[ax] - nm[ax]) * g[ax].ks;
            }
            if (KIND == RK_LIM_BJ) {
                // Barth-Jespersen (Limiters.h:74-83): the smallest admissible
                // ratio over the 2*nd face projections +-dd.  Branch-free: with
                // dmax = 0 every dd is 0 and the ratio (0/0 or x/0) is dropped
                // by fminf, so lim = 1 as in the reference.
                float umax = w0, umin = w0, dmax = 0.0f;
#pragma unroll
                for (int ax = 0; ax < T::NAX; ++ax) {
                    umax = fmaxf(umax, fmaxf(nm[ax], np[ax]));
                    umin = fminf(umin, fminf(nm[ax], np[ax]));
                    dmax = fmaxf(dmax, fabsf(dd[ax]));
                }
                const float lim = fminf(1.0f, fminf(umax - w0, w0 - umin) / dmax);
#pragma unroll
                for (int ax = 0; ax < T::NAX; ++ax) dd[ax] *= lim;
            }
            if (KIND == RK_LIM_VK) {
                float umax = w0, umin = w0;
#pragma unroll
                for (int ax = 0; ax < T::NAX; ++ax) {
                    umax = fmaxf(umax, fmaxf(nm[ax], np[ax]));
                    umin = fminf(umin, fminf(nm[ax], np[ax]));
                }
                float lim = 1.0f;
                if (umax - umin > 0.0f) {
                    // Limiters.h:86-115, per face projection +-dd
                    const float iun = 2.0f / (umax - umin);
#pragma unroll
                    for (int ax = 0; ax < T::NAX; ++ax) {
#pragma unroll
                        for (int sg = 0; sg < 2; ++sg) {
                            const float d2 = sg ? -dd[ax] : dd[ax];
                            if (d2 == 0.0f) continue;
                            const float dm = ((d2 > 0.0f ? umax : umin) - w0) * iun;
                            const float q = d2 * iun;
                            const float r =
                                ((dm * dm + eps2) + 2.0f * q * dm) / (dm * dm + 2.0f * q * q + dm * q + eps2);
                            lim = fminf(lim, r);
                        }
                    }
                }
#pragma unroll
                for (int ax = 0; ax < T::NAX; ++ax) dd[ax] *= lim;
            }
#pragma unroll
            for (int ax = 0; ax < T::NAX; ++ax) sm[T::d(s.d0, ax, v, t)] = dd[ax];
        }
    }
}

template <class T>
__device__ __forceinline__ void recon(const ProbDesc& d, float* sm, int p, int kind, const Slots& s,
                                      const RingPos& rp) {
    switch (kind) {
    case RK_LINEAR: recon_k<T, RK_LINEAR>(d, sm, p, s, rp); break;
    case RK_ENO2: recon_k<T, RK_ENO2>(d, sm, p, s, rp); break;
    case RK_LIM_VK: recon_k<T, RK_LIM_VK>(d, sm, p, s, rp); break;
    default: recon_k<T, RK_LIM_BJ>(d, sm, p, s, rp); break;
    }
}

// One face on kernel axis AX between the cells fx-1 and fx of the tile
// (AX = 0) or between cell fx of planes z and z+1 (AX = 2, the marching
// axis): face states, boundary image, Riemann flux and eigenvalue into the
// face array.  s holds the slots of plane z.
template <class T, int AX>
__device__ __forceinline__ bool face_in(const ProbDesc& d, const float* sm, int fx, int gi, int z, const Slots& s,
                                        bool pwc, float UL[NV], float UR[NV], int& out, int& vs) {
    static_assert(AX == 0 || (AX == 2 && T::MARCH), "faces on x or the marching axis");
    constexpr int A = phys_axis<T, AX>();
    constexpr int SA = AX == 0 ? 0 : T::AZ;
    int bl, br, rl, rr, g, n, per;
    int wl = s.w0, wr = s.w0, dl = s.d0, dr = s.d0;
    if (AX == 0) {
        if (gi > d.kn[0]) return false;
        bl = fx + 1; br = bl + 1;
        rl = fx; rr = rl + 1;
        g = gi; n = d.kn[0]; per = d.kper[0];
        out = T::fx(0, fx); vs = T::TX + 1;
    } else {
        if (gi >= d.kn[0]) return false;
        bl = br = fx + HB;
        rl = rr = fx + 1;
        wr = s.wp; dr = s.d1;
        g = z + 1; n = d.kn[2]; per = d.kper[2];
        out = T::fz(s.d1, 0, fx); vs = T::TX;
    }
#pragma unroll
    for (int v = 0; v < NV; ++v) {
        UL[v] = sm[T::w(wl, v, bl)] + (pwc ? 0.0f : sm[T::d(dl, SA, v, rl)]);
        UR[v] = sm[T::w(wr, v, br)] - (pwc ? 0.0f : sm[T::d(dr, SA, v, rr)]);
    }
    // boundary faces: the BC of this face (an x face is numbered by its
    // plane, a marching-axis face by its x index)
    const int f = AX == 0 ? z : gi;
    if (g == 0 && !per) {
#pragma unroll
        for (int v = 0; v < NV; ++v) UL[v] = UR[v];
        bc32(d.mp, bc_id32(d.mp, 2 * A, f), A, UL);
    } else if (g == n && !per) {
#pragma unroll
        for (int v = 0; v < NV; ++v) UR[v] = UL[v];
        bc32(d.mp, bc_id32(d.mp, 2 * A + 1, f), A, UR);
    }
    return true;
}

template <class T, int SOLVER, int AX>
__device__ __forceinline__ void face(const ProbDesc& d, float* sm, int fx, int gi, int z, const Slots& s, bool pwc) {
    float UL[NV], UR[NV], F[NV];
    int out, vs;
    if (!face_in<T, AX>(d, sm, fx, gi, z, s, pwc, UL, UR, out, vs)) return;
    const float lam = flux32<SOLVER, phys_axis<T, AX>()>(d.mp, UL, UR, F);
#pragma unroll
    for (int v = 0; v < NV; ++v) sm[out + v * vs] = F[v];
    sm[out + NV * vs] = lam;
}

// The faces of plane z this thread computes: the x face left of its cell
// (thread TX: the tile's far x face) and, marching, the face above its cell
// (between z and z+1).
template <class T, int SOLVER>
__device__ __forceinline__ void fluxes(const ProbDesc& d, float* sm, int i0, int z, bool pwc, bool do_x, bool do_z,
                                       const Slots& s) {
    const int tx = threadIdx.x;
    if (do_x && tx <= T::TX) face<T, SOLVER, 0>(d, sm, tx, i0 + tx, z, s, pwc);
    if constexpr (T::MARCH)
        if (do_z && tx < T::TX) face<T, SOLVER, 2>(d, sm, tx, i0 + tx, z, s, pwc);
}

// The working state (rho, momentum) of the thread's own cell in plane z, for
// the source terms; read before the barrier that precedes the residual (the
// next plane's store reuses the slot).
template <class T>
__device__ __forceinline__ float4 own_state(const float* sm, const Slots& s) {
    int tx;
    if (!T::cell(threadIdx.x, tx)) return make_float4(1.0f, 0.0f, 0.0f, 0.0f);
    const int box = tx + HB;
    return make_float4(sm[T::w(s.w0, 0, box)], sm[T::w(s.w0, 1, box)], sm[T::w(s.w0, 2, box)],
                       sm[T::w(s.w0, 3, box)]);
}

// Geometry of the thread's own cell along kernel axes 0 and 1 (fixed while
// an item marches): sizes, the face area normal to the marching axis, the
// inverse area, and the spectral-radius factor of the high x boundary face
// (0 where the cell is not the last one along x).
struct CellGeo {
    float hx, hy, fsz, ixy, farx;
};

template <class T>
__device__ __forceinline__ CellGeo cell_geo(const ProbDesc& d, int i0) {
    CellGeo c{1.0f, 1.0f, 1.0f, 1.0f, 0.0f};
    int tx;
    if (!T::cell(threadIdx.x, tx)) return c;
    const int gi = i0 + tx;
    if (gi >= d.kn[0]) return c;
    const AxisGeo gx = d.kgeo[0][gi + d.kgoff[0]], gy = d.kgeo[1][d.kgoff[1]];
    c.hx = gx.h;
    c.hy = gy.h;
    c.fsz = gx.h * gy.h;
    c.ixy = gx.ih * gy.ih;
    if (gi == d.kn[0] - 1) c.farx = d.kgeo[0][d.kn[0] + d.kgoff[0]].ih * gy.ih;
    return c;
}

// Residual R and spectral radius of the owned cell of this thread in plane z
// (hz, ihz: size and inverse size of plane z); false if the thread owns no
// cell.
template <class T, int SOLVER>
__device__ __forceinline__ bool residual_of(const ProbDesc& d, const float* sm, int i0, int z, const Slots& s,
                                            float4 own, const CellGeo& cg, float hz, float ihz, float& srmax,
                                            float R[NV]) {
    int tx;
    if (!T::cell(threadIdx.x, tx)) return false;
    const int gi = i0 + tx;
    if (gi >= d.kn[0]) return false;
    const float fsx = cg.hy * hz, fsz = cg.fsz;
    const float iv = cg.ixy * ihz;
    // face areas times the stored-flux factor
    const float kx = flux_scale<SOLVER>() * fsx, kz = flux_scale<SOLVER>() * fsz;
    const float lxl = sm[T::fx(5, tx)], lxr = sm[T::fx(5, tx + 1)];
#pragma unroll
    for (int v = 0; v < NV; ++v) R[v] = -(sm[T::fx(v, tx + 1)] - sm[T::fx(v, tx)]) * kx;
    float sr = fsx * (lxl + lxr);
    if (cg.farx != 0.0f) srmax = fmaxf(srmax, fsx * lxr * cg.farx * ihz);
    if (T::MARCH) {
        const int dn = s.d0, up = s.d1;
#pragma unroll
        for (int v = 0; v < NV; ++v) R[v] -= (sm[T::fz(up, v, tx)] - sm[T::fz(dn, v, tx)]) * kz;
        const float lzr = sm[T::fz(up, 5, tx)];
        sr += fsz * (sm[T::fz(dn, 5, tx)] + lzr);
        if (z == d.kn[2] - 1) srmax = fmaxf(srmax, fsz * lzr * cg.ixy * d.kgeo[2][d.kn[2] + d.kgoff[2]].ih);
    }
    srmax = fmaxf(srmax, sr * iv);
    // source terms after the face fluxes (kernel.h:941-989), on the working state
    const MixPhys& mp = d.mp;
    if (mp.force || mp.accel) {
        const float ro = own.x;
        const float iro = 1.0f / ro;
        const float vu = own.y * iro, vv = own.z * iro, vw = own.w * iro;
        const float vol = fsz * hz;
        if (mp.force) {
            R[1] += vol * mp.sigma[0];
            R[2] += vol * mp.sigma[1];
            R[3] += vol * mp.sigma[2];
            R[4] += (mp.sigma[0] * vu + mp.sigma[1] * vv + mp.sigma[2] * vw) * vol;
        }
        if (mp.accel) {
            R[1] += ro * vol * mp.g[0];
            R[2] += ro * vol * mp.g[1];
            R[3] += ro * vol * mp.g[2];
            R[4] += ((ro * mp.g[0]) * vu + (ro * mp.g[1]) * vv + (ro * mp.g[2]) * vw) * vol;
        }
    }
    return true;
}

// The same, written to the pending-residual planes Rout.
template <class T, int SOLVER>
__device__ __forceinline__ void residual(const ProbDesc& d, const float* sm, float* __restrict__ Rout, int i0, int z,
                                         const Slots& s, float4 own, const CellGeo& cg, float hz, float ihz,
                                         float& srmax, float (&nrm)[NV]) {
    float R[NV];
    if (!residual_of<T, SOLVER>(d, sm, i0, z, s, own, cg, hz, ihz, srmax, R)) return;
    if (d.mp.norms) {
        const float vol = cg.fsz * hz;
#pragma unroll
        for (int v = 0; v < NV; ++v) nrm[v] += vol * fabsf(R[v]);
    }
    int tx;
    T::cell(threadIdx.x, tx);
    const long long c = d.kbase + (i0 + tx) + z * d.kstr[2];
    const long long plane = d.L.plane;
#pragma unroll
    for (int v = 0; v < NV; ++v) __stcg(Rout + v * plane + c, R[v]);
}

// ---------------------------------------------------------------------------
// The fused step kernel
// ---------------------------------------------------------------------------

// One work item (tile column and chunk q of problem d).
template <class T, int SOLVER>
__device__ __forceinline__ void process_item(const ProbDesc& d, int q, int par, float dtf, float* sm, BoxPos& bp,
                                             Prefetch& pf, RingPos& rp, float& srmax, unsigned int& health,
                                             float (&nrm)[NV]) {
    const double* __restrict__ Uin = d.U[par];
    double* __restrict__ Uout = d.U[par ^ 1];
    const float* __restrict__ Rin = d.R[par];
    float* __restrict__ Rout = d.R[par ^ 1];
    const int kind = recon_kind(d.mp);
    const bool pwc = kind == 0;
    const bool src = d.mp.force || d.mp.accel;
    const int i0 = (q % d.ncol) * T::TX;
    setup_box<T>(d, i0, bp);
    if (!pwc) setup_ring<T>(d, i0, rp);
    if constexpr (!T::MARCH) {
        const Slots s = slots_of<T>(0);
        issue<T>(d, Uin, Rin, 0, bp, pf);
        store<T>(d, sm, Uout, 0, 0, 1, dtf, bp, pf, health);
        __syncthreads();
        if (!pwc) { recon<T>(d, sm, 0, kind, s, rp); __syncthreads(); }
        fluxes<T, SOLVER>(d, sm, i0, 0, pwc, true, false, s);
        const float4 own = src ? own_state<T>(sm, s) : make_float4(1.0f, 0.0f, 0.0f, 0.0f);
        __syncthreads();
        // a single plane: the geometry is loaded where it is used
        const CellGeo cg = cell_geo<T>(d, i0);
        const AxisGeo gz = d.kgeo[2][d.kgoff[2]];
        residual<T, SOLVER>(d, sm, Rout, i0, 0, s, own, cg, gz.h, gz.ih, srmax, nrm);
    } else {
        const CellGeo cg = cell_geo<T>(d, i0);
        const int z0 = (q / d.ncol) * d.ch, z1 = min(d.kn[2], z0 + d.ch);
        // Planes z0-2 .. z1+1 are loaded; the first two loop passes only
        // build the slopes of planes z0-1, z0 and the marching face z0-1/2.
        // Each pass: store plane z+2, slopes of plane z+1, faces of plane z,
        // residual of plane z (three barriers).
        issue<T>(d, Uin, Rin, z0 - 2, bp, pf);
        store<T>(d, sm, Uout, z0 - 2, z0, z1, dtf, bp, pf, health);
        issue<T>(d, Uin, Rin, z0 - 1, bp, pf);
        store<T>(d, sm, Uout, z0 - 1, z0, z1, dtf, bp, pf, health);
        issue<T>(d, Uin, Rin, z0, bp, pf);
#pragma unroll 1
        for (int z = z0 - 2; z < z1; ++z) {
            const Slots sf = slots_of<T>(z), sr = slots_of<T>(z + 1);
            // plane z+2 was prefetched during the previous pass
            store<T>(d, sm, Uout, z + 2, z0, z1, dtf, bp, pf, health);
            if (z + 3 <= z1 + 1) issue<T>(d, Uin, Rin, z + 3, bp, pf);
            __syncthreads();
            if (!pwc) { recon<T>(d, sm, z + 1, kind, sr, rp); __syncthreads(); }
            if (z >= z0 - 1) fluxes<T, SOLVER>(d, sm, i0, z, pwc, z >= z0, true, sf);
            const float4 own = src && z >= z0 ? own_state<T>(sm, sf) : make_float4(1.0f, 0.0f, 0.0f, 0.0f);
            __syncthreads();
            if (z >= z0) {
                const AxisGeo gz = d.kgeo[2][z + d.kgoff[2]];
                residual<T, SOLVER>(d, sm, Rout, i0, z, sf, own, cg, gz.h, gz.ih, srmax, nrm);
            }
        }
    }
}

// The item's CFL maximum and health into the problem's control word.  COUNT:
// the CTA that completes the problem's last item closes the problem's step;
// otherwise (batches) a separate kernel closes every listed problem's step
// after the stage, and items only post their maxima (no returned atomics).
template <class T, bool COUNT>
__device__ __forceinline__ void close_item(const ProbDesc& d, float srmax, unsigned int health, float (&nrm)[NV],
                                           float* wmax, unsigned int* whealth) {
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    // the last warp of a block whose size is not a multiple of 32 is partial
    const int live = min(32, T::NT - (threadIdx.x & ~31));
    const unsigned int mask = live == 32 ? 0xffffffffu : ((1u << live) - 1u);
    if (d.mp.norms) add_norms(d.ctl, nrm, mask, lane, live);
    // srmax >= 0: its bits order like unsigned integers
    const unsigned int mbits = __reduce_max_sync(mask, __float_as_uint(srmax));
    health = __reduce_or_sync(mask, health);
    if (lane == 0) { wmax[wid] = __uint_as_float(mbits); whealth[wid] = health; }
    __syncthreads();
    if (threadIdx.x == 0) {
        float m = 0.0f;
        unsigned int hh = 0;
        for (int k = 0; k < (T::NT + 31) / 32; ++k) { m = fmaxf(m, wmax[k]); hh |= whealth[k]; }
        Ctl* ctl = d.ctl;
        if (m > 0.0f) atomicMax(&ctl->srmax_bits, __float_as_uint(m));
        if (hh) atomicOr(&ctl->health, hh);
        if (COUNT) {
            __threadfence();
            if (atomicAdd(&ctl->blocks_done, 1u) == (unsigned)(d.nq - 1)) {
                __threadfence();
                finish_problem(ctl, d.mp.cfl);
            }
        }
    }
}

// BATCH = false: one problem whose descriptor is a kernel parameter (constant
// bank: every field is a free operand).  BATCH = true: a list of (problem,
// item) pairs; the descriptor is staged in shared memory when the problem
// changes from one item of the CTA to the next, and the problem's stop flag,
// parity and pending dt (constant during a batched stage: steps are closed
// by k_batch_finish) are read alongside it from the control-word array.
template <class T, int SOLVER, bool BATCH>
__global__ void __launch_bounds__(T::NT, T::MINB) k_mix_step(const __grid_constant__ ProbDesc one,
                                                    const ProbDesc* __restrict__ probs,
                                                    const Ctl* __restrict__ ctls,
                                                    const int2* __restrict__ items, int n_items,
                                                    int close_in_kernel) {
    extern __shared__ float sm[];
    __shared__ float wmax[32];
    __shared__ unsigned int whealth[32];
    BoxPos bp;
    Prefetch pf;
    RingPos rp;
    if constexpr (!BATCH) {
        if (one.ctl->stop_req) return;
        const int par = one.ctl->parity;
        const float dtf = __double2float_rn(one.ctl->dt_apply);  // once per launch
        for (int q = blockIdx.x; q < n_items; q += gridDim.x) {
            __syncthreads();  // the previous item is finished with shared memory
            float srmax = 0.0f, nrm[NV] = {0.0f, 0.0f, 0.0f, 0.0f, 0.0f};
            unsigned int health = 0;
            process_item<T, SOLVER>(one, q, par, dtf, sm, bp, pf, rp, srmax, health, nrm);
            close_item<T, true>(one, srmax, health, nrm, wmax, whealth);
        }
    } else {
        __shared__ ProbDesc sd;
        __shared__ int s_skip, s_par;
        __shared__ float s_dtf;  // the pending dt, rounded to FP32 once per problem
        const int nwords = (int)(sizeof(ProbDesc) / sizeof(int));
        int cur = -1;
        for (int it = blockIdx.x; it < n_items; it += gridDim.x) {
            const int2 pq = items[it];
            __syncthreads();  // the previous item is finished with shared memory
            if (pq.x != cur) {
                for (int k = threadIdx.x; k < nwords; k += T::NT) ((int*)&sd)[k] = ((const int*)(probs + pq.x))[k];
                if (threadIdx.x == 0) {
                    const Ctl& c = ctls[pq.x];
                    s_skip = c.stop_req;
                    s_par = c.parity;
                    s_dtf = __double2float_rn(c.dt_apply);
                }
                __syncthreads();
                cur = pq.x;
            }
            if (s_skip) continue;
            float srmax = 0.0f, nrm[NV] = {0.0f, 0.0f, 0.0f, 0.0f, 0.0f};
            unsigned int health = 0;
            process_item<T, SOLVER>(sd, pq.y, s_par, s_dtf, sm, bp, pf, rp, srmax, health, nrm);
            if (close_in_kernel) close_item<T, true>(sd, srmax, health, nrm, wmax, whealth);
            else close_item<T, false>(sd, srmax, health, nrm, wmax, whealth);
        }
    }
}


// ---------------------------------------------------------------------------
// Tail kernel: the last few long 1D problems of a batch, one thread-block
// cluster per problem, many stages per launch
// ---------------------------------------------------------------------------
// Each CTA of the cluster owns 508 consecutive cells and keeps their FP64
// state and FP32 pending residual in registers from stage to stage; halo
// cells come from the neighbouring CTAs' shared memory (distributed shared
// memory) and the CFL maximum is reduced into the first CTA's shared memory.
// Per stage: the pending update and working copy of the own cells, a cluster
// barrier, the halo pulls, slopes, faces and residual exactly as the batched
// kernel computes them for the same cells, the cluster-wide maximum, a second
// cluster barrier, and the step bookkeeping of finish_problem, which every
// CTA repeats on its own copy of the control word (the same maximum gives
// every CTA the same dt and the same stop decision, so all CTAs run the same
// number of stages and barriers).
using TailTile = Tile<512, false>;

template <int SOLVER>
__global__ void __launch_bounds__(512, 1) k_mix_tail(const ProbDesc* __restrict__ probs,
                                                     const int* __restrict__ list, int budget) {
    using T = TailTile;
    namespace cg = cooperative_groups;
    cg::cluster_group cluster = cg::this_cluster();
    extern __shared__ float sm[];
    float* rbuf = sm + T::TOTAL;            // residual of the own cells, NV planes of TX
    __shared__ float wmax[32];
    __shared__ unsigned int whealth[32];
    __shared__ unsigned int red[2][2];      // per stage parity: max bits, health (first CTA's are used)
    __shared__ Ctl sc;                      // this CTA's copy of the control word
    __shared__ int s_stop;
    __shared__ float s_dtf;                 // sc.dt_apply rounded to FP32 (once per stage)
    const int tid = threadIdx.x;
    const unsigned int rank = cluster.block_rank();
    const ProbDesc& d = probs[list[blockIdx.x / cluster.num_blocks()]];
    const MixPhys& mp = d.mp;
    const int i0 = (int)rank * T::TX;
    const long long plane = d.L.plane;
    if (tid < 4) red[tid >> 1][tid & 1] = 0u;
    if (tid == 0) {
        sc = *d.ctl;
        s_stop = sc.stop_req;
        s_dtf = __double2float_rn(sc.dt_apply);
    }
    const int kind = recon_kind(mp);
    const bool pwc = kind == 0;
    const bool src = mp.force || mp.accel;
    const bool stiff = mp.eos == TS_EOS_STIFFENED_GAS;
    BoxPos bp;
    RingPos rp;
    setup_box<T>(d, i0, bp);
    if (!pwc) setup_ring<T>(d, i0, rp);
    const CellGeo cg0 = cell_geo<T>(d, i0);
    const AxisGeo gz = d.kgeo[2][d.kgoff[2]];
    const Slots sl = slots_of<T>(0);
    const bool own = bp.off >= 0 && bp.own;
    __syncthreads();
    double u[NV];
    float r[NV];
    if (own) {
        const int par = sc.parity;
        const long long c = d.kbase + bp.off;
#pragma unroll
        for (int v = 0; v < NV; ++v) {
            u[v] = __ldcg(d.U[par] + v * plane + c);
            r[v] = __ldcg(d.R[par] + v * plane + c);
        }
    }
    cluster.sync();  // every CTA's reduction slots are zero before any remote update
    for (int st = 0; st < budget; ++st) {
        if (s_stop) break;
        unsigned int health = 0;
        // pending update of the own cell and its working copy (store())
        if (own) {
            const float cf = bp.cfxy * (s_dtf * gz.ih);
            float inc[NV], w[NV];
#pragma unroll
            for (int v = 0; v < NV; ++v) inc[v] = __fmul_rn(cf, r[v]);  // as store()
#pragma unroll
            for (int v = 0; v < 4; ++v) w[v] = __fmaf_rn(cf, r[v], f64_to_f32(u[v]));
            w[4] = __fmaf_rn(cf, r[4], stiff ? f64_to_f32(u[4] - mp.einf_d) : f64_to_f32(u[4]));
#pragma unroll
            for (int v = 0; v < NV; ++v) sm[T::w(0, v, bp.box)] = w[v];
#pragma unroll
            for (int v = 0; v < NV; ++v) u[v] = u[v] + f32_to_f64(inc[v]);
            const long long b = __double_as_longlong(u[0]);
            if (b <= 0 || b > 0x7FF0000000000000LL)
                health |= (b & 0x7FFFFFFFFFFFFFFFLL) > 0x7FF0000000000000LL ? TS_HEALTH_NAN : TS_HEALTH_NEG_DENSITY;
            if (!(w[4] == w[4])) health |= TS_HEALTH_NAN;
        }
        cluster.sync();
        // halo positions: the owner's working copy, then the boundary image
        if (bp.off >= 0 && !own) {
            const int si = bp.off;
            const int orank = si / T::TX;
            const float* owner = cluster.map_shared_rank(sm, orank);
            const int opos = si - orank * T::TX + HB;
            float w[NV];
#pragma unroll
            for (int v = 0; v < NV; ++v) w[v] = owner[T::w(0, v, opos)];
            if (bp.xs >= 0) bc32(mp, bc_id32(mp, bp.xs, 0), 0, w);
#pragma unroll
            for (int v = 0; v < NV; ++v) sm[T::w(0, v, bp.box)] = w[v];
        }
        __syncthreads();
        if (!pwc) { recon<T>(d, sm, 0, kind, sl, rp); __syncthreads(); }
        fluxes<T, SOLVER>(d, sm, i0, 0, pwc, true, false, sl);
        const float4 ow = src ? own_state<T>(sm, sl) : make_float4(1.0f, 0.0f, 0.0f, 0.0f);
        __syncthreads();
        float srmax = 0.0f, R[NV];
        if (residual_of<T, SOLVER>(d, sm, i0, 0, sl, ow, cg0, gz.h, gz.ih, srmax, R)) {
#pragma unroll
            for (int v = 0; v < NV; ++v) rbuf[v * T::TX + tid] = R[v];
        }
        // CTA maximum and health into the first CTA's slots
        const int lane = tid & 31, wid = tid >> 5;
        const unsigned int mbits = __reduce_max_sync(0xffffffffu, __float_as_uint(srmax));
        const unsigned int hw = __reduce_or_sync(0xffffffffu, health);
        if (lane == 0) { wmax[wid] = __uint_as_float(mbits); whealth[wid] = hw; }
        __syncthreads();
        if (tid == 0) {
            float m = 0.0f;
            unsigned int hh = 0;
            for (int k = 0; k < T::NT / 32; ++k) { m = fmaxf(m, wmax[k]); hh |= whealth[k]; }
            unsigned int* slot = cluster.map_shared_rank(&red[st & 1][0], 0);
            if (m > 0.0f) atomicMax(slot, __float_as_uint(m));
            if (hh) atomicOr(slot + 1, hh);
        }
        cluster.sync();
        if (tid == 0) {
            const unsigned int* slot = cluster.map_shared_rank(&red[st & 1][0], 0);
            const float m = __uint_as_float(slot[0]);
            const unsigned int hh = slot[1];
            sc.health |= hh;
            finish_with(&sc, m, mp.cfl);
            s_dtf = __double2float_rn(sc.dt_apply);
            // the first CTA clears the slots of the next stage (read by
            // nobody since the previous stage's second barrier)
            if (rank == 0) { red[(st + 1) & 1][0] = 0u; red[(st + 1) & 1][1] = 0u; }
            // a non-physical state stops the loop; the host stops the problem
            s_stop = sc.stop_req || hh != 0;
        }
        __syncthreads();
        if (own) {
            const int lx = bp.box - HB;
#pragma unroll
            for (int v = 0; v < NV; ++v) r[v] = rbuf[v * T::TX + lx];
        }
    }
    // the state and pending residual back where the batched kernel expects
    // them, and the control word
    __syncthreads();
    if (own) {
        const int par = sc.parity;
        const long long c = d.kbase + bp.off;
#pragma unroll
        for (int v = 0; v < NV; ++v) {
            d.U[par][v * plane + c] = u[v];
            d.R[par][v * plane + c] = r[v];
        }
    }
    if (rank == 0 && tid == 0) {
        Ctl* g = d.ctl;
        g->time = sc.time;
        g->dt = sc.dt;
        g->dt_min_raw = sc.dt_min_raw;
        g->dt_apply = sc.dt_apply;
        g->iteration = sc.iteration;
        g->parity = sc.parity;
        g->next_sol = sc.next_sol;
        g->next_slice = sc.next_slice;
        g->stop_req = sc.stop_req;
        g->health = sc.health;
        g->srmax_bits = 0u;
        g->blocks_done = 0u;
    }
    // no CTA leaves while another may still read its shared memory
    cluster.sync();
}

// U[parity] += dt R[parity] / V, R[parity] = 0 for problem p (materialise the
// pending update with the fused kernel's own rounding: (1/h0 h1) (dt / h2)
// over kernel axes).
__global__ void k_mix_apply(const ProbDesc* __restrict__ probs, int p) {
    const ProbDesc& d = probs[p];
    const Layout& L = d.L;
    const long long n = L.cells();
    const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (t >= n) return;
    const int i = (int)(t % L.nx), j = (int)((t / L.nx) % L.ny), k = (int)(t / ((long long)L.nx * L.ny));
    const long long c = L.at(i, j, k);
    const int a1 = L.nd == 3 ? j : 0, a2 = L.nd == 3 ? k : (L.nd == 2 ? j : 0);
    const int par = d.ctl->parity;
    const float dtf = __double2float_rn(d.ctl->dt_apply);
    const float cf = (d.kgeo[0][i + d.kgoff[0]].ih * d.kgeo[1][a1 + d.kgoff[1]].ih) *
                     (dtf * d.kgeo[2][a2 + d.kgoff[2]].ih);
    double* U = d.U[par];
    float* R = d.R[par];
#pragma unroll
    for (int v = 0; v < NV; ++v) {
        U[(long long)v * L.plane + c] += f32_to_f64(cf * R[(long long)v * L.plane + c]);
        R[(long long)v * L.plane + c] = 0.0f;
    }
}

__global__ void k_mix_clear_pending(const ProbDesc* __restrict__ probs, int p) { probs[p].ctl->dt_apply = 0.0; }

// Closes the stage of every listed problem that ran (batches): dt from its
// CFL maximum and the Run bookkeeping.
__global__ void k_batch_finish(const ProbDesc* __restrict__ probs, const int* __restrict__ slots, int n) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n) return;
    const ProbDesc& d = probs[slots[t]];
    if (d.ctl->stop_req) return;
    finish_problem(d.ctl, d.mp.cfl);
}

// Compiled tiles: (problem dimension, threads).  2D: one-row tiles marching
// y.  1D: one-row tiles, one plane.  (3D problems run k_mix3d.)
#define TS_MIXED_TILES_2D(X) X(2, 260) X(2, 132) X(2, 68)
#define TS_MIXED_TILES_1D(X) X(1, 512) X(1, 256) X(1, 128)

// Calls f.template operator()<Tile, SOLVER>() for the compiled tile matching
// (nd, tx) (ty is 1 for these problems); returns false when there is none.
template <class F>
bool with_tile(int nd, int tx, int ty, int solver, F&& f) {
    bool found = false;
    (void)ty;
#define TS_TRY(ND_, TX_)                                                                                \
    if (!found && nd == ND_ && tx == TX_) {                                                            \
        found = true;                                                                                  \
        if (solver == TS_RS_HLLC) f.template operator()<Tile<TX_, (ND_ >= 2)>, TS_RS_HLLC>();          \
        else f.template operator()<Tile<TX_, (ND_ >= 2)>, TS_RS_ROE_PIKE>();                           \
    }
    TS_MIXED_TILES_2D(TS_TRY)
    TS_MIXED_TILES_1D(TS_TRY)
#undef TS_TRY
    return found;
}

}  // namespace

bool mixed_tile_info(int nd, int tx, int ty, int solver, size_t* smem, int* per_sm, bool batch) {
    return with_tile(nd, tx, ty, solver, [&]<class T, int S>() {
        *smem = T::BYTES;
        *per_sm = 0;
        const int b = (int)T::BYTES;
        bool ok = cudaFuncSetAttribute(k_mix_step<T, S, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, b) ==
                  cudaSuccess;
        // all of the unified L1 / shared storage as shared memory: more resident CTAs
        cudaFuncSetAttribute(k_mix_step<T, S, false>, cudaFuncAttributePreferredSharedMemoryCarveout, 100);
        cudaFuncSetAttribute(k_mix_step<T, S, true>, cudaFuncAttributePreferredSharedMemoryCarveout, 100);
        ok = ok && cudaFuncSetAttribute(k_mix_step<T, S, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, b) ==
                       cudaSuccess;
        if (!ok) return;
        if (batch) {
            cudaOccupancyMaxActiveBlocksPerMultiprocessor(per_sm, k_mix_step<T, S, true>, T::NT, T::BYTES);
            return;
        }
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(per_sm, k_mix_step<T, S, false>, T::NT, T::BYTES);
    });
}

void mixed_launch_single(int nd, int tx, int ty, int solver, int grid, const ProbDesc& h_desc, cudaStream_t st) {
    if (grid <= 0 || h_desc.nq <= 0) return;
    with_tile(nd, tx, ty, solver, [&]<class T, int S>() {
        k_mix_step<T, S, false><<<grid, T::NT, T::BYTES, st>>>(h_desc, nullptr, nullptr, nullptr, h_desc.nq, 0);
    });
}

bool mixed_launch_batch(int nd, int tx, int ty, int solver, int grid, const ProbDesc* d_probs, const Ctl* d_ctls,
                        const int2* d_items, int n_items, cudaStream_t st, bool close_in_kernel) {
    if (nd == 3) return false;
    if (grid <= 0 || n_items <= 0) return true;
    ProbDesc none;
    std::memset(&none, 0, sizeof none);
    return with_tile(nd, tx, ty, solver, [&]<class T, int S>() {
        k_mix_step<T, S, true><<<grid, T::NT, T::BYTES, st>>>(none, d_probs, d_ctls, d_items, n_items,
                                                              close_in_kernel ? 1 : 0);
    });
}

int mixed_tail_cells() { return TailTile::TX; }

namespace {
template <int S>
bool tail_ready_for(int cluster) {
    const size_t bytes = TailTile::BYTES + sizeof(float) * NV * TailTile::TX;
    if (cudaFuncSetAttribute(k_mix_tail<S>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes) != cudaSuccess)
        return false;
    if (cluster > 8 &&
        cudaFuncSetAttribute(k_mix_tail<S>, cudaFuncAttributeNonPortableClusterSizeAllowed, 1) != cudaSuccess)
        return false;
    cudaLaunchConfig_t cfg = {};
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = cluster;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.gridDim = dim3(cluster);
    cfg.blockDim = dim3(TailTile::NT);
    cfg.dynamicSmemBytes = bytes;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    int n = 0;
    if (cudaOccupancyMaxActiveClusters(&n, k_mix_tail<S>, &cfg) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return n > 0;
}

template <int S>
cudaError_t tail_launch(int cluster, int n_problems, const ProbDesc* d_probs, const int* d_list, int budget,
                        cudaStream_t st) {
    cudaLaunchConfig_t cfg = {};
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = cluster;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.gridDim = dim3(cluster * n_problems);
    cfg.blockDim = dim3(TailTile::NT);
    cfg.dynamicSmemBytes = TailTile::BYTES + sizeof(float) * NV * TailTile::TX;
    cfg.stream = st;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, k_mix_tail<S>, d_probs, d_list, budget);
}
}  // namespace

bool mixed_tail_ready(int solver, int cluster) {
    if (cluster < 1 || cluster > kTailMaxCluster) return false;
    return solver == TS_RS_HLLC ? tail_ready_for<TS_RS_HLLC>(cluster) : tail_ready_for<TS_RS_ROE_PIKE>(cluster);
}

cudaError_t mixed_launch_tail(int solver, int cluster, int n_problems, const ProbDesc* d_probs, const int* d_list,
                              int budget, cudaStream_t st) {
    if (n_problems <= 0 || budget <= 0) return cudaSuccess;
    return solver == TS_RS_HLLC ? tail_launch<TS_RS_HLLC>(cluster, n_problems, d_probs, d_list, budget, st)
                                : tail_launch<TS_RS_ROE_PIKE>(cluster, n_problems, d_probs, d_list, budget, st);
}

void mixed_tile_cells(int nd, int tx, int ty, int* cx, int* cy) {
    *cx = nd == 3 ? tx : tx - 2 * HB;
    *cy = nd == 3 ? ty : 1;
}

void mixed_items(ProbDesc& d, int tx, int ty, int zchunks, long long slots) {
    const int nd = d.L.nd;
    int cx, cy;
    mixed_tile_cells(nd, tx, ty, &cx, &cy);
    d.ncx = (d.kn[0] + cx - 1) / cx;
    const int ncy = (d.kn[1] + cy - 1) / cy;
    d.ncol = d.ncx * ncy;
    const bool march = nd >= 2;
    const int nz = march ? d.kn[2] : 1;
    if (nd == 2 && zchunks <= 0) {
        // A stage of one 2D problem ends with its longest march: the chunk
        // count minimises the modelled stage time, over the waves of items,
        // (rows per item + 2.5 rows of start-up) x a per-row time that grows
        // with the wave's share of the CTA slots, 1 + fill (fitted on the
        // 1024^2 shear layer: 4.2 us per row at 67 % of the slots, 5.0 at
        // 99 %).  Measured on the shear layer, 132-thread rows: it picks the
        // fastest of the chunkings tried at 128^2 .. 2048^2 (1024^2: 94
        // chunks of 11 rows, 67 us per stage against 78 us for 64 chunks of
        // 16; 256^2: rows of one, 21 us against 51 us).
        const long long sl = std::max(1LL, slots);
        double best = 1e300;
        for (int c = 1; c <= nz; ++c) {
            const int ch = (nz + c - 1) / c;
            const long long q = (long long)d.ncol * ((nz + ch - 1) / ch);
            const long long full = q / sl, rest = q % sl;
            const double t = (ch + 2.5) * (2.0 * (double)full + (rest ? 1.0 + (double)rest / (double)sl : 0.0));
            if (t < best - 1e-9) { best = t; zchunks = c; }
        }
    }
    if (march && zchunks <= 0) {
        // Chunks of >= 16 planes; pick the count that best fills the
        // persistent grid, charging ~2 planes of start-up per chunk.
        double best = -1.0;
        for (int c = 1; c <= std::max(1, nz / 16); ++c) {
            const int ch = (nz + c - 1) / c;
            const int nch = (nz + ch - 1) / ch;
            const long long q = (long long)d.ncol * nch;
            const double waves = std::ceil((double)q / (double)std::max(1LL, slots));
            const double score = (double)q / (waves * (double)std::max(1LL, slots)) / (1.0 + 2.0 / ch);
            if (score > best + 1e-9) { best = score; zchunks = c; }
        }
    }
    zchunks = march ? std::max(1, std::min(zchunks, nz)) : 1;
    d.ch = march ? (nz + zchunks - 1) / zchunks : 1;
    d.nq = d.ncol * ((nz + d.ch - 1) / d.ch);
}

ts_status mixed_set_tile(MixedBufs& mb, int tx, int ty, int zchunks, std::string& err, cudaStream_t st) {
    const int nd = mb.desc.L.nd;
    if (nd < 3) ty = 1;
    size_t bytes = 0;
    int per_sm = 0;
    const bool found = nd == 3 ? mix3d_tile_info(tx, ty, mb.desc.mp.solver, mb.desc.mp.recon, mb.desc.mp.limiter,
                                                 &bytes, &per_sm)
                               : mixed_tile_info(nd, tx, ty, mb.desc.mp.solver, &bytes, &per_sm);
    if (!found) {
        err = "no compiled tile " + std::to_string(tx) + "x" + std::to_string(ty) + " for " + std::to_string(nd) + "D";
        return TS_ERR_UNSUPPORTED;
    }
    if (per_sm < 1) { err = "mixed kernel does not fit on an SM with this tile"; return TS_ERR_UNSUPPORTED; }
    mb.tx = tx;
    mb.ty = ty;
    mb.smem = bytes;
    const long long slots = (long long)mb.sms * per_sm;
    mixed_items(mb.desc, tx, ty, zchunks, slots);
    mb.zchunks = nd >= 2 ? (mb.desc.kn[2] + mb.desc.ch - 1) / mb.desc.ch : 1;
    mb.grid = (int)std::min<long long>(mb.desc.nq, slots);
    if (nd == 3) {
        // the 3D kernel closes the step once per CTA, after all its items
        mb.desc.nq = mb.grid;
        ts_status s = mix3d_make_maps(mb.desc, tx, ty, mb.maps, err);
        if (s != TS_OK) return s;
    }
    // ordered on the stream the steps run on (a pageable source is staged
    // before the call returns, so mb.desc may change afterwards)
    if (cudaMemcpyAsync(mb.d_desc, &mb.desc, sizeof(ProbDesc), cudaMemcpyHostToDevice, st) != cudaSuccess) {
        err = "descriptor upload failed";
        return TS_ERR_CUDA;
    }
    return TS_OK;
}

ts_status mixed_problem(const ts_config& c, const Layout& L, const Phys& ph, const HostGrid& g, Ctl* ctl,
                        const DeviceAlloc& alloc, ProbDesc& d, std::string& err, cudaStream_t st) {
    if (L.plane > (1LL << 31) - 1) { err = "grid too large for the mixed path"; return TS_ERR_INVALID; }
    d.L = L;
    d.ctl = ctl;
    const AxisGeo* axis_geo[3];
    const int goff[3] = {L.gx, L.gy, L.gz};
    ts_status s;
    // per-axis geometry with ghost entries on active axes
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
            }
        }
        void* p;
        if ((s = alloc(sizeof(AxisGeo) * geo.size(), &p)) != TS_OK) return s;
        // pageable source: staged before the call returns, so `geo` may go
        if (cudaMemcpyAsync(p, geo.data(), sizeof(AxisGeo) * geo.size(), cudaMemcpyHostToDevice, st) != cudaSuccess) {
            err = "geometry upload failed";
            return TS_ERR_CUDA;
        }
        axis_geo[a] = (const AxisGeo*)p;
    }
    // kernel axes: x, the tile's second axis, the marching axis
    // (3D: x, y, z; 2D: x, inactive z, y; 1D: x, inactive y, inactive z)
    const int map[3] = {0, L.nd == 2 ? 2 : 1, L.nd == 2 ? 1 : 2};
    for (int a = 0; a < 3; ++a) {
        d.kgeo[a] = axis_geo[map[a]];
        d.kgoff[a] = goff[map[a]];
        d.kn[a] = L.n(map[a]);
        d.kper[a] = ph.periodic[map[a]];
        d.kphys[a] = map[a];
        d.kstr[a] = L.stride(map[a]);
    }
    d.kbase = L.at(0, 0, 0);
    MixPhys& m = d.mp;
    std::memset(&m, 0, sizeof m);
    m.nd = L.nd;
    m.recon = c.reconstruction;
    m.limiter = c.limiter;
    m.solver = c.riemann_solver;
    m.eos = c.eos;
    for (int a = 0; a < 3; ++a) m.periodic[a] = ph.periodic[a];
    m.gamma = (float)ph.gamma;
    m.gm1 = (float)(ph.gamma - 1.0);
    m.pinf = (float)ph.p_inf;
    m.einf_d = c.eos == TS_EOS_STIFFENED_GAS ? ph.gamma * ph.p_inf / (ph.gamma - 1.0) : 0.0;
    m.einf = (float)m.einf_d;
    m.eps = (float)ph.eps;
    m.cfl = ph.cfl;
    // the six sides' BCs inline; a position-dependent side's extra kinds in
    // device memory
    MixBcKinds kinds;
    std::memset(&kinds, 0, sizeof kinds);
    for (int sd = 0; sd < kBcIds; ++sd) {
        const double r = ph.bc.density[sd];
        const double vx = ph.bc.vel[sd][0], vy = ph.bc.vel[sd][1], vz = ph.bc.vel[sd][2];
        // inlet ghost state, energy shifted: p/(g-1) + rho|v|^2/2 (the p_inf terms cancel)
        const float inl[5] = {(float)r, (float)(r * vx), (float)(r * vy), (float)(r * vz),
                             (float)(ph.bc.pstatic[sd] / (ph.gamma - 1) + 0.5 * r * (vx * vx + vy * vy + vz * vz))};
        int* type = sd < 6 ? &m.bc_type[sd] : &kinds.type[sd - 6];
        float* state = sd < 6 ? m.bc_state[sd] : kinds.state[sd - 6];
        float* vel = sd < 6 ? m.bc_vel[sd] : kinds.vel[sd - 6];
        *type = ph.bc.type[sd];
        for (int v = 0; v < 5; ++v) state[v] = inl[v];
        for (int a = 0; a < 3; ++a) vel[a] = (float)ph.bc.vel[sd][a];
    }
    bool marked = false;
    for (int sd = 0; sd < 6; ++sd) {
        m.mark[sd] = ph.bc.mark[sd];
        marked = marked || ph.bc.mark[sd];
    }
    m.kinds = nullptr;
    if (marked) {
        void* p;
        if ((s = alloc(sizeof(MixBcKinds), &p)) != TS_OK) return s;
        if (cudaMemcpyAsync(p, &kinds, sizeof kinds, cudaMemcpyHostToDevice, st) != cudaSuccess) {
            err = "boundary-condition table upload failed";
            return TS_ERR_CUDA;
        }
        m.kinds = static_cast<const MixBcKinds*>(p);
    }
    m.force = ph.force;
    m.accel = ph.accel;
    m.norms = c.residual_norms != 0;
    for (int a = 0; a < 3; ++a) {
        m.sigma[a] = (float)ph.sigma[a];
        m.g[a] = (float)ph.g[a];
    }
    return TS_OK;
}

ts_status mixed_init(const ts_config& c, const Layout& L, const Phys& ph, const HostGrid& g, Ctl* ctl,
                     const DeviceAlloc& alloc, MixedBufs& mb, std::string& err, cudaStream_t st, bool zero_buffers) {
    ts_status s;
    ProbDesc& d = mb.desc;
    std::memset(&d, 0, sizeof d);
    if ((s = mixed_problem(c, L, ph, g, ctl, alloc, d, err, st)) != TS_OK) return s;
    for (int b = 0; b < 2; ++b) {
        if ((s = alloc(sizeof(double) * NV * L.plane, (void**)&d.U[b])) != TS_OK) return s;
        if ((s = alloc(sizeof(float) * NV * L.plane, (void**)&d.R[b])) != TS_OK) return s;
        if (zero_buffers && (cudaMemsetAsync(d.U[b], 0, sizeof(double) * NV * L.plane, st) != cudaSuccess ||
                             cudaMemsetAsync(d.R[b], 0, sizeof(float) * NV * L.plane, st) != cudaSuccess)) {
            err = "cudaMemsetAsync failed";
            return TS_ERR_CUDA;
        }
    }
    if ((s = alloc(sizeof(ProbDesc), (void**)&mb.d_desc)) != TS_OK) return s;
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&mb.sms, cudaDevAttrMultiProcessorCount, dev);
    // 2D: 132-thread rows (measured on the 1024^2 shear layer: 13.3e9 against
    // 12.2e9 cell-updates/s for 260-thread rows)
    const int tx = L.nd == 3 ? 32 : (L.nd == 2 ? 132 : 256);
    const int ty = L.nd == 3 ? 8 : 1;
    return mixed_set_tile(mb, tx, ty, 0, err, st);
}

void mixed_step(MixedBufs& mb, const Phys&, cudaStream_t st, cudaEvent_t* ev, int* n_launch, const char** names) {
    const bool d3 = mb.desc.L.nd == 3;
    if (ev) cudaEventRecord(ev[0], st);
    if (d3) mix3d_launch(mb.tx, mb.ty, mb.grid, mb.desc, mb.maps, st);
    else mixed_launch_single(mb.desc.L.nd, mb.tx, mb.ty, mb.desc.mp.solver, mb.grid, mb.desc, st);
    if (ev) cudaEventRecord(ev[1], st);
    if (names) names[0] = d3 ? "k_mix3d" : "k_mix_step";
    if (n_launch) *n_launch = 1;
}

void mixed_reset(MixedBufs& mb, cudaStream_t st) {
    // caller has set parity 0 and dt_apply 0 in the control word
    cudaMemsetAsync(mb.desc.R[0], 0, sizeof(float) * NV * mb.desc.L.plane, st);
}

void mixed_apply(const ProbDesc* d_probs, int p, long long cells, cudaStream_t st) {
    k_mix_apply<<<(unsigned)((cells + 255) / 256), 256, 0, st>>>(d_probs, p);
    k_mix_clear_pending<<<1, 1, 0, st>>>(d_probs, p);
}

void mixed_batch_finish(const ProbDesc* d_probs, const int* d_slots, int n, cudaStream_t st) {
    if (n > 0) k_batch_finish<<<(n + 127) / 128, 128, 0, st>>>(d_probs, d_slots, n);
}

void mixed_materialize(MixedBufs& mb, const Phys&, cudaStream_t st) { mixed_apply(mb.d_desc, 0, mb.desc.L.cells(), st); }

double* mixed_state(MixedBufs& mb, int parity) { return mb.desc.U[parity & 1]; }

}  // namespace ts

// ---------------------------------------------------------------------------
// ts_advance_noalloc: the fused mixed-precision step for callers that may not
// allocate device memory.  Everything the kernel needs beyond the caller's
// input and output -- both state buffers, both residual buffers, the grid
// geometry, the problem descriptor and the control word -- lives in one fixed
// array in device memory that is part of this library's module.
// ---------------------------------------------------------------------------
namespace ts {
namespace noalloc {

constexpr size_t kNaPlane = TS_NOALLOC_MAX_PLANE;
constexpr size_t kNaGeo = kNaPlane + 16;  // AxisGeo entries of all three axes together
constexpr size_t kNaBytes = 2 * NV * kNaPlane * sizeof(double) + 2 * NV * kNaPlane * sizeof(float) +
                            kNaGeo * sizeof(AxisGeo) + sizeof(Ctl) + sizeof(ProbDesc) + 16 * 256;

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
    if (has_markers(*cfg))
        return fail(TS_ERR_UNSUPPORTED, "ts_advance_noalloc takes one boundary condition per side (no bc_marker)");
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
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    MixedBufs mb;
    const Phys ph = make_phys(*cfg);
    // every upload of the set-up is queued on the caller's stream, ahead of
    // the steps; the second state and residual buffers need no clearing (the
    // first stage writes every cell of them before anything reads them)
    if ((s = mixed_init(*cfg, L, ph, grid, ctl, carve, mb, err, st, false)) != TS_OK) return fail(s, err);

    Ctl c;
    std::memset(&c, 0, sizeof c);
    // A fresh run (no info, or iteration 0 at time 0) starts the snapshot
    // schedule at SaveSolutionTime / SaveSliceTime as Kernel::Init does
    // (kernel.h:259-263); a continued run keeps the caller's schedule.
    const bool fresh = !info || (info->iteration == 0 && info->time == 0.0);
    c.time = info ? info->time : 0.0;
    c.iteration = info ? info->iteration : 0;
    c.next_sol = fresh ? cfg->save_solution_time : info->next_solution_time;
    c.next_slice = fresh ? cfg->save_slice_time : info->next_slice_time;
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
    NA_CUDA(cudaMemsetAsync(mb.desc.R[0], 0, sizeof(float) * NV * L.plane, st));
    const unsigned blocks = (unsigned)((L.cells() + 255) / 256);
    k_na_scatter<<<blocks, 256, 0, st>>>(state_in, L, mb.desc.U[0]);
    for (int k = 0; k < n_steps; ++k) mixed_step(mb, ph, st);
    mixed_materialize(mb, ph, st);
    k_na_gather<<<blocks, 256, 0, st>>>(state_out, L, mb.desc.U[0], mb.desc.U[1], ctl);
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
        for (int v = 0; v < NV; ++v) info->residual[v] = c.res[v];  // zeros unless cfg->residual_norms
    }
    return TS_OK;
}

