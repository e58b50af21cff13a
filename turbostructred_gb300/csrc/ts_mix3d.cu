// Mixed-precision fused stage kernel for 3D problems on GB300: TMA-staged
// planes, shared working-state planes, per-column face fluxes in registers.
//
// The arithmetic is the mixed path's (FP32 reconstruction, EOS and Riemann
// flux; FP64 state, stage accumulation and dt; deferred update: the kernel of
// step n+1 reads U^n and the pending residual R^n, forms U^{n+1} on the fly,
// writes it and R^{n+1}).  What differs from the general fused kernel is how
// the data moves:
//
//  * Loads.  A work item is a TX x TY tile column marching z over a chunk of
//    planes.  For each plane one elected thread issues two TMA tensor loads
//    (cp.async.bulk.tensor, 4D maps over the SoA state: x, y, z, variable) of
//    the tile plus a 2-cell halo -- the FP64 U^n box and the FP32 R^n box --
//    into a two-stage shared-memory ring, completed on an mbarrier.  Loads run
//    two planes ahead of the conversion that consumes them.  No thread
//    computes a global address for the stencil; halo cells on a
//    non-periodic side are the mirrored cells of the same box (the boundary
//    image is applied in the conversion), halo cells on a periodic side
//    (edge tiles only) are read directly from global memory.
//  * Positions.  Every thread owns one cell of the tile; 80 threads also
//    own one cell of the 1-cell ring around it (the cells the tile's faces
//    need) and 84 one of the 2-cell frame (the ring cells' neighbours).  The
//    FP32 working copy of three planes (k, k+1, k+2) is kept in shared
//    memory, so the reconstruction reads its in-plane and z neighbours
//    there; the reconstruction writes the face states W + dx / W + dy of the
//    cells left of / below a face to shared memory and keeps the own cell's
//    other face states in registers.  The z face between planes k and k+1
//    is solved by the thread that owns the column, and its flux serves the
//    residuals of planes k and k+1 from registers.
//  * Per plane k, two phases separated by barriers: (A) convert plane k+2
//    (FP64 U + dt R / V -> FP32 working copy) and solve the x/y faces of
//    plane k; (B) the owned cell's FP64 update U^{n+1} of plane k+2 (its
//    FP64 adds overlap the FP32 work that follows), the limited slopes of
//    plane k+1, the z face between k and k+1, and the residual of plane k.
//
// Waits on an mbarrier are bounded: a wait that gives up sets
// TS_HEALTH_TIMEOUT in the problem's health word and the kernel runs on
// (every thread still reaches every barrier); the host reports it.
#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_runtime.h>

#include <cstdint>
#include <cstring>
#include <mutex>
#include <string>

#include "ts_flux32.cuh"
#include "ts_mixed.h"

namespace ts {
namespace {

using namespace mix32;

constexpr int HB3 = 2;  // halo of the staged box

// ---------------------------------------------------------------------------
// TMA and mbarrier (inline PTX, sm_90 and later)
// ---------------------------------------------------------------------------
__device__ __forceinline__ unsigned smem_u32(const void* p) { return (unsigned)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint64_t* bar, unsigned count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, unsigned bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
                 : "memory");
}

// Waits for the phase with the given parity to complete; gives up after
// about a second (2^31 SM clocks) and returns false.
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, unsigned parity) {
    const unsigned a = smem_u32(bar);
    const long long t0 = clock64();
    for (;;) {
        unsigned done;
        asm volatile(
            "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n\t}"
            : "=r"(done)
            : "r"(a), "r"(parity)
            : "memory");
        if (done) return true;
        if (clock64() - t0 > (1LL << 31)) return false;
    }
}

// 4D tiled tensor load (x, y, z, variable) into shared memory, completing
// on `bar`.  x must be a multiple of 16 bytes / element size.
__device__ __forceinline__ void tma_load4(void* dst, const CUtensorMap* map, int x, int y, int z, int v,
                                          uint64_t* bar) {
    asm volatile(
        "cp.async.bulk.tensor.4d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4, %5}], "
        "[%6];" ::"r"(smem_u32(dst)),
        "l"(map), "r"(x), "r"(y), "r"(z), "r"(v), "r"(smem_u32(bar))
        : "memory");
}

// ---------------------------------------------------------------------------
// Tile geometry and shared-memory layout
// ---------------------------------------------------------------------------
template <int TX_, int TY_>
struct Tile3 {
    static constexpr int TX = TX_, TY = TY_, NT = TX * TY;
    static constexpr int BX = TX + 2 * HB3, BY = TY + 2 * HB3, NBOX = BX * BY;
    static constexpr int N1 = 2 * (TX + TY);      // ring cells the faces need (no corners)
    static constexpr int N2 = 2 * (TX + TY) + 4;  // their other neighbours: the 2-cell frame and 4 corners
    static constexpr int F1 = NT - N1;            // ring cells go to threads [F1, NT)
    static_assert(N2 <= F1, "frame and ring cells on distinct threads");
    // far faces (x at TX, y at TY) on the threads between the two groups
    static constexpr int FFY = ((N2 + 31) / 32) * 32;  // y far faces: threads [FFY, FFY + TX)
    static constexpr int FFX = FFY + TX;               // x far faces: threads [FFX, FFX + TY)
    static_assert(FFX + TY <= F1 || TX * TY > 512, "far faces on threads without ring cells");
    // shared memory (bytes): two TMA stages (FP64 U box, FP32 R box), three
    // working-state planes (k, k+1, k+2), the x/y face states of one plane,
    // the x/y face fluxes of one plane
    static constexpr int SU = NBOX * NV * 8, SR = NBOX * NV * 4;
    static constexpr int TX_BYTES = SU + SR;                  // bytes the two boxes of a plane deliver
    static constexpr int STAGE = (TX_BYTES + 127) / 128 * 128;  // stage pitch (128-byte aligned)
    static constexpr int OFF_STAGE = 0;
    static constexpr int OFF_W = 2 * STAGE;
    static constexpr int NW = NV * NBOX;                   // floats per working-state plane
    static constexpr int NFVX = NV * TY * (TX + 2);         // x face states per slot
    static constexpr int NFVY = NV * (TY + 2) * TX;         // y face states per slot
    static constexpr int NWS = 3;                           // working-state planes kept
    static constexpr int OFF_FV = OFF_W + NWS * NW * 4;
    static constexpr int OFF_FX = OFF_FV + (NFVX + NFVY) * 4;
    static constexpr int NFX = 6 * TY * (TX + 1), NFY = 6 * (TY + 1) * TX;
    static constexpr int OFF_RED = OFF_FX + (NFX + NFY) * 4;  // per-warp maxima and health words
    static constexpr int OFF_FAIL = OFF_RED + 2 * 32 * 4;      // set once a wait gave up
    static constexpr int OFF_BAR = (OFF_FAIL + 4 + 15) / 16 * 16;
    static constexpr int BYTES = OFF_BAR + 2 * 8;
    static_assert(SU % 128 == 0 && STAGE % 128 == 0, "TMA destinations 128-byte aligned");
    static_assert((BX * 4) % 16 == 0, "TMA boxes: inner extent a multiple of 16 bytes");

    // shared-memory indices (floats unless noted)
    static __device__ __forceinline__ int w(int slot, int v, int box) { return slot * NW + v * NBOX + box; }
    // working-state slot of plane j (j >= -2)
    static __device__ __forceinline__ int wslot(int j) { return (j + 3) % 3; }
    static __device__ __forceinline__ int fvx(int v, int cy, int c) { return (v * TY + cy) * (TX + 2) + c; }
    static __device__ __forceinline__ int fvy(int v, int c, int cx) { return NFVX + (v * (TY + 2) + c) * TX + cx; }
    static __device__ __forceinline__ int fx(int v, int cy, int c) { return (v * TY + cy) * (TX + 1) + c; }
    static __device__ __forceinline__ int fy(int v, int c, int cx) { return NFX + (v * (TY + 1) + c) * TX + cx; }
};

// Cell (cx, cy) relative to the tile of the second position of thread t, and
// its role: 1 = ring cell left of the tile (cx = -1), 2 = right (cx = TX),
// 3 = below (cy = -1), 4 = above (cy = TY), 5 = frame/corner cell (no
// reconstruction), 0 = none.
template <class T>
__device__ __forceinline__ int second_cell(int t, int& cx, int& cy) {
    if (t >= T::F1) {
        const int f = t - T::F1;
        if (f < T::TY) { cx = -1; cy = f; return 1; }
        if (f < 2 * T::TY) { cx = T::TX; cy = f - T::TY; return 2; }
        if (f < 2 * T::TY + T::TX) { cx = f - 2 * T::TY; cy = -1; return 3; }
        cx = f - 2 * T::TY - T::TX; cy = T::TY;
        return 4;
    }
    if (t < T::N2) {
        const int g = t;
        if (g < T::TY) { cx = -2; cy = g; }
        else if (g < 2 * T::TY) { cx = T::TX + 1; cy = g - T::TY; }
        else if (g < 2 * T::TY + T::TX) { cx = g - 2 * T::TY; cy = -2; }
        else if (g < 2 * T::TY + 2 * T::TX) { cx = g - 2 * T::TY - T::TX; cy = T::TY + 1; }
        else {
            const int c = g - 2 * T::TY - 2 * T::TX;
            cx = (c & 1) ? T::TX : -1;
            cy = (c & 2) ? T::TY : -1;
        }
        return 5;
    }
    cx = cy = 0;
    return 0;
}

// One working-state position of a thread for the current item.
struct CPos {
    int wbox;    // box index (working state in shared memory); -1: unused
    int sbox;    // box index of the source in the staged box; -1: read from global memory
    int goff;    // plane offset of the source (periodic halo cells)
    int xs, ys;  // boundary side applied after mirroring, or -1
    float cfxy;  // 1 / (hx hy) of the source cell
};

// One reconstruction position: its box index and x/y geometry.
struct RPos {
    int box;          // -1: nothing to do
    float ks0, ks1;   // central-slope factors along x and y
    int g0, g1;       // geometry indices (x, y)
};

// Working copy of the state of one position (FP32, shifted energy).
struct W5 {
    float v[NV];
};

// The owned cell's FP64 update U^{n+1} = U^n + dt R^n / V of the plane just
// converted: formed after the barrier that ends the conversion phase, where
// the FP64 adds (a slow pipe on GB300) overlap FP32 work instead of
// holding every warp at the barrier.
struct PendingU {
    double u[NV];
    float inc[NV];
    unsigned int off;  // element offset of the cell
    bool on;
};

// Reconstruction kinds (the limiter choice folded in), as the general kernel.
enum { K_PWC = 0, K_LINEAR = 1, K_ENO2 = 2, K_LIM_BJ = 3, K_LIM_VK = 4 };

__host__ __device__ __forceinline__ int kind_of(const MixPhys& mp) {
    if (mp.recon == TS_RECON_LINEAR_2POINTS) return K_LINEAR;
    if (mp.recon == TS_RECON_ENO2_2POINTS) return K_ENO2;
    if (mp.recon == TS_RECON_LINEAR_2POINTS_LIMITED)
        return mp.limiter == TS_LIM_VENKATAKRISHNAN ? K_LIM_VK : K_LIM_BJ;
    return K_PWC;
}

// Limited half-slopes dd[3] (the projections to the high faces) of one
// variable from its value w0 and neighbours nm/np along x, y, z: the
// reconstruction of Linear2PointsStencil.h:66-97, ENO2PointsStencil.h:20-58
// and Linear2psLim.h:63-132 with the Barth-Jespersen and Venkatakrishnan
// limiters (Limiters.h:28-115), in FP32: dd[ax] the unlimited half-slope
// (explicitly rounded) and lim the limiter factor (1 without a limiter).  The
// caller forms the face states as fma(+-dd, lim, w0) on every code path, so a
// ring cell's states are the same bits in every CTA that computes them.
template <int KIND>
__device__ __forceinline__ void half_slopes(float w0, const float nm[3], const float np[3], const AxisGeo g[3],
                                            float eps2, float dd[3], float& lim) {
    lim = 1.0f;
    if (KIND == K_ENO2) {
#pragma unroll
        for (int ax = 0; ax < 3; ++ax) {
            const float gl = (w0 - nm[ax]) * g[ax].il, gr = (np[ax] - w0) * g[ax].ir;
            dd[ax] = __fmul_rn(fabsf(gl) < fabsf(gr) ? gl : gr, g[ax].hh);
        }
    } else {
#pragma unroll
        for (int ax = 0; ax < 3; ++ax) dd[ax] = __fmul_rn(np[ax] - nm[ax], g[ax].ks);
    }
    if (KIND == K_LIM_BJ) {
        // the smallest admissible ratio over the 6 face projections +-dd;
        // with dmax = 0 every dd is 0 and lim = 1 (the ratio is dropped by fminf)
        float umax = w0, umin = w0, dmax = 0.0f;
#pragma unroll
        for (int ax = 0; ax < 3; ++ax) {
            umax = fmaxf(umax, fmaxf(nm[ax], np[ax]));
            umin = fminf(umin, fminf(nm[ax], np[ax]));
            dmax = fmaxf(dmax, fabsf(dd[ax]));
        }
        lim = fminf(1.0f, fminf(umax - w0, w0 - umin) / dmax);
    }
    if (KIND == K_LIM_VK) {
        float umax = w0, umin = w0;
#pragma unroll
        for (int ax = 0; ax < 3; ++ax) {
            umax = fmaxf(umax, fmaxf(nm[ax], np[ax]));
            umin = fminf(umin, fminf(nm[ax], np[ax]));
        }
        if (umax - umin > 0.0f) {
            const float iun = 2.0f / (umax - umin);
#pragma unroll
            for (int ax = 0; ax < 3; ++ax) {
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
        }
    }
}

// Geometry of the own cell along x and y (fixed while an item marches):
// sizes, the face area normal to z, the inverse area, and the
// spectral-radius factors of the high boundary faces (0 where the cell is
// not the last one along the axis).
struct CellGeo3 {
    float hx, hy, fsz, ixy, farx, fary;
};

// Per-item state of a thread.
struct Item3 {
    int i0, j0, z0, z1;
    int cx, cy;   // own cell in the tile
    bool own;     // the own cell is inside the domain
    int own_off;  // plane offset of the own cell
    int role;     // role of the second position (second_cell)
    int cx2, cy2;
    CPos cp[2];
    RPos rp[2];
    CellGeo3 cg;
};

template <class T>
__device__ __forceinline__ void conv_pos(const ProbDesc& d, int i0, int j0, int cx, int cy, CPos& p) {
    const int gi = i0 + cx, gj = j0 + cy;
    p.wbox = -1;
    p.sbox = -1;
    p.goff = 0;
    p.xs = p.ys = -1;
    p.cfxy = 0.0f;
    // cells past the halo of the domain's far side are needed by nobody
    if (gi >= d.kn[0] + HB3 || gj >= d.kn[1] + HB3) return;
    int si, sj, xs, ys;
    resolve(gi, d.kn[0], d.kper[0], 0, si, xs);
    resolve(gj, d.kn[1], d.kper[1], 2, sj, ys);
    p.xs = xs;
    p.ys = ys;
    p.wbox = (cx + HB3) + (cy + HB3) * T::BX;
    const bool wrapped = (d.kper[0] && (gi < 0 || gi >= d.kn[0])) || (d.kper[1] && (gj < 0 || gj >= d.kn[1]));
    if (wrapped) p.goff = si + sj * (int)d.kstr[1];
    else p.sbox = (si - i0 + HB3) + (sj - j0 + HB3) * T::BX;  // itself, or its mirror image in the same box
    p.cfxy = __ldg(&d.kgeo[0][si + d.kgoff[0]].ih) * __ldg(&d.kgeo[1][sj + d.kgoff[1]].ih);
}

template <class T>
__device__ __forceinline__ void ring_pos(const ProbDesc& d, int i0, int j0, int cx, int cy, RPos& r) {
    const int gi = i0 + cx, gj = j0 + cy;
    r.box = -1;
    r.ks0 = r.ks1 = 0.0f;
    r.g0 = r.g1 = 0;
    if (gi > d.kn[0] || gj > d.kn[1]) return;
    // outside a non-periodic side: the boundary face takes the BC image of
    // the inner face state, no reconstruction there
    if ((gi < 0 || gi >= d.kn[0]) && !d.kper[0]) return;
    if ((gj < 0 || gj >= d.kn[1]) && !d.kper[1]) return;
    int si, sj, s_;
    resolve(gi, d.kn[0], 1, 0, si, s_);
    resolve(gj, d.kn[1], 1, 0, sj, s_);
    r.box = (cx + HB3) + (cy + HB3) * T::BX;
    r.g0 = si + d.kgoff[0];
    r.g1 = sj + d.kgoff[1];
    r.ks0 = __ldg(&d.kgeo[0][r.g0].ks);
    r.ks1 = __ldg(&d.kgeo[1][r.g1].ks);
}

template <class T>
__device__ __forceinline__ void setup_item(const ProbDesc& d, int q, Item3& it) {
    const int col = q % d.ncol;
    it.i0 = (col % d.ncx) * T::TX;
    it.j0 = (col / d.ncx) * T::TY;
    it.z0 = (q / d.ncol) * d.ch;
    it.z1 = min(d.kn[2], it.z0 + d.ch);
    const int tid = threadIdx.x;
    it.cx = tid % T::TX;
    it.cy = tid / T::TX;
    const int gi = it.i0 + it.cx, gj = it.j0 + it.cy;
    it.own = gi < d.kn[0] && gj < d.kn[1];
    it.own_off = (int)(d.kbase + gi + (long long)gj * d.kstr[1]);
    it.role = second_cell<T>(tid, it.cx2, it.cy2);
    conv_pos<T>(d, it.i0, it.j0, it.cx, it.cy, it.cp[0]);
    if (it.role) conv_pos<T>(d, it.i0, it.j0, it.cx2, it.cy2, it.cp[1]);
    else it.cp[1].wbox = -1;
    ring_pos<T>(d, it.i0, it.j0, it.cx, it.cy, it.rp[0]);
    if (it.role >= 1 && it.role <= 4) ring_pos<T>(d, it.i0, it.j0, it.cx2, it.cy2, it.rp[1]);
    else it.rp[1].box = -1;
    CellGeo3 c{1.0f, 1.0f, 1.0f, 1.0f, 0.0f, 0.0f};
    if (it.own) {
        const AxisGeo gx = d.kgeo[0][gi + d.kgoff[0]], gy = d.kgeo[1][gj + d.kgoff[1]];
        c.hx = gx.h;
        c.hy = gy.h;
        c.fsz = gx.h * gy.h;
        c.ixy = gx.ih * gy.ih;
        if (gi == d.kn[0] - 1) c.farx = d.kgeo[0][d.kn[0] + d.kgoff[0]].ih * gy.ih;
        if (gj == d.kn[1] - 1) c.fary = gx.ih * d.kgeo[1][d.kn[1] + d.kgoff[1]].ih;
    }
    it.cg = c;
}

// TMA loads of plane j (U^n FP64 box, R^n FP32 box) into stage `stage`.
template <class T>
__device__ __forceinline__ void issue_plane(const ProbDesc& d, const Mix3dMaps& maps, int par, unsigned char* smem,
                                            uint64_t* bar, int stage, int i0, int j0, int j) {
    int sk, zs;
    resolve(j, d.kn[2], d.kper[2], 4, sk, zs);
    unsigned char* dst = smem + T::OFF_STAGE + stage * T::STAGE;
    mbar_expect_tx(&bar[stage], (unsigned)T::TX_BYTES);
    const int x = i0 - HB3 + d.L.gx, y = j0 - HB3 + d.L.gy, z = sk + d.L.gz;
    tma_load4(dst, &maps.u[par], x, y, z, 0, &bar[stage]);
    tma_load4(dst + T::SU, &maps.r[par], x, y, z, 0, &bar[stage]);
}

// Conversion of plane j (staged): working copy W = U^n + dt R^n / V in FP32
// (boundary image applied on mirrored halo cells) into shared memory and the
// thread's registers; U^{n+1} of the owned cell written in FP64.
template <class T>
__device__ __forceinline__ void convert(const ProbDesc& d, const Item3& it, const unsigned char* stage,
                                        const double* __restrict__ Uin, const float* __restrict__ Rin,
                                        double* __restrict__ Uout, float* smw, int j, float dtf, PendingU& pu,
                                        unsigned int& health) {
    const MixPhys& mp = d.mp;
    const double* su = reinterpret_cast<const double*>(stage);
    const float* sr = reinterpret_cast<const float*>(stage + T::SU);
    int sk, zs;
    resolve(j, d.kn[2], d.kper[2], 4, sk, zs);
    const float cfz = dtf * __ldg(&d.kgeo[2][sk + d.kgoff[2]].ih);
    // offsets within a variable plane fit 32 bits (a plane holds < 2^31
    // elements, checked on the host); the stride between the five planes is
    // 64-bit (five planes of a 1024^3 grid exceed 2^32 elements)
    const size_t plane = (size_t)d.L.plane;
    const unsigned int zoff = (unsigned int)d.kbase + (unsigned int)sk * (unsigned int)d.kstr[2];
    const int slot = T::wslot(j);
    const bool own_plane = j >= it.z0 && j < it.z1;
    const bool stiff = mp.eos == TS_EOS_STIFFENED_GAS;
#pragma unroll
    for (int p = 0; p < 2; ++p) {
        const CPos& c = it.cp[p];
        if (c.wbox < 0) continue;
        double u[NV];
        float r[NV];
        if (c.sbox >= 0) {
#pragma unroll
            for (int v = 0; v < NV; ++v) {
                u[v] = su[v * T::NBOX + c.sbox];
                r[v] = sr[v * T::NBOX + c.sbox];
            }
        } else {
            // periodic halo cell of an edge tile: not in the staged box
#pragma unroll
            for (int v = 0; v < NV; ++v) {
                u[v] = __ldg(Uin + (zoff + (unsigned int)c.goff) + v * plane);
                r[v] = __ldg(Rin + (zoff + (unsigned int)c.goff) + v * plane);
            }
        }
        const float cf = c.cfxy * cfz;
        float w[NV];
        // the working copy as explicit FMAs (never split by the compiler): a
        // cell's copy must be the same bits in the CTA that owns it (position
        // 0) and in every CTA that converts it as a halo cell (position 1),
        // whose unrolled code could otherwise be contracted differently
        const double e4 = stiff ? u[4] - mp.einf_d : u[4];  // shifted energy (uniform choice)
#pragma unroll
        for (int v = 0; v < 4; ++v) w[v] = __fmaf_rn(cf, r[v], f64_to_f32(u[v]));
        w[4] = __fmaf_rn(cf, r[4], f64_to_f32(e4));
        if (c.xs >= 0 || c.ys >= 0 || zs >= 0) {
            // a halo cell beyond a non-periodic side: the BC of the boundary
            // face of its row (source cell indices recovered from the box or
            // the plane offset; halo cells only)
            int si, sj;
            if (c.sbox >= 0) {
                si = c.sbox % T::BX + it.i0 - HB3;
                sj = c.sbox / T::BX + it.j0 - HB3;
            } else {
                si = c.goff % (int)d.kstr[1];
                sj = c.goff / (int)d.kstr[1];
            }
            if (c.xs >= 0) bc32(mp, bc_id32(mp, c.xs, sj + d.kn[1] * sk), 0, w);
            if (c.ys >= 0) bc32(mp, bc_id32(mp, c.ys, si + d.kn[0] * sk), 1, w);
            if (zs >= 0) bc32(mp, bc_id32(mp, zs, si + d.kn[0] * sj), 2, w);
        }
#pragma unroll
        for (int v = 0; v < NV; ++v) smw[T::w(slot, v, c.wbox)] = w[v];
        if (p == 0) {
            pu.on = own_plane && it.own;
            pu.off = (unsigned int)it.own_off + (unsigned int)j * (unsigned int)d.kstr[2];
#pragma unroll
            for (int v = 0; v < NV; ++v) {
                pu.u[v] = u[v];
                pu.inc[v] = __fmul_rn(cf, r[v]);  // dt R / V in FP32, added to U^n in FP64
            }
            if (pu.on && !(w[4] == w[4])) health |= TS_HEALTH_NAN;
        }
    }
}

// U^{n+1} of the owned cell of the last converted plane, written in FP64.
__device__ __forceinline__ void apply_pending(const ProbDesc& d, double* __restrict__ Uout, const PendingU& pu,
                                              unsigned int& health) {
    if (!pu.on) return;
    const size_t plane = (size_t)d.L.plane;
    double un[NV];
#pragma unroll
    for (int v = 0; v < NV; ++v) {
        un[v] = pu.u[v] + f32_to_f64(pu.inc[v]);
        __stcs(Uout + pu.off + v * plane, un[v]);
    }
    // rho > 0 tested on the bit pattern (no FP64 comparison)
    const long long b = __double_as_longlong(un[0]);
    if (b <= 0 || b > 0x7FF0000000000000LL)
        health |= (b & 0x7FFFFFFFFFFFFFFFLL) > 0x7FF0000000000000LL ? TS_HEALTH_NAN : TS_HEALTH_NEG_DENSITY;
}

// Limited slopes of plane j at the thread's reconstruction positions (the
// working state of planes j-1, j, j+1 in shared memory); the face states go
// to shared memory (W + dx, W + dy of the cells left of / below a face;
// W - dx, W - dy of the far ring cells), the own cell's right-hand x/y
// states and both z states stay in registers.
template <class T, int KIND>
__device__ __forceinline__ void reconstruct(const ProbDesc& d, const Item3& it, float* sm, int j, W5& urx, W5& ury,
                                            W5& ulz, W5& urz) {
    if ((j < 0 || j >= d.kn[2]) && !d.kper[2]) return;
    int sk, s_;
    resolve(j, d.kn[2], 1, 0, sk, s_);
    const AxisGeo gz = d.kgeo[2][sk + d.kgoff[2]];
    const int s0 = T::wslot(j), sm1 = T::wslot(j - 1), sp1 = T::wslot(j + 1);
    const float* smw = sm + T::OFF_W / 4;
    float* fv = sm + T::OFF_FV / 4;
#pragma unroll
    for (int p = 0; p < 2; ++p) {
        const RPos& r = it.rp[p];
        if (r.box < 0) continue;
        AxisGeo g[3];
        if (KIND == K_ENO2 || KIND == K_LIM_VK) {
            g[0] = d.kgeo[0][r.g0];
            g[1] = d.kgeo[1][r.g1];
        } else {
            g[0].ks = r.ks0;
            g[1].ks = r.ks1;
        }
        g[2] = gz;
        float eps2 = 0.0f;
        if (KIND == K_LIM_VK) {
            // eps^2 = (K (h1 h2 h3)^(1/3))^3 with K = 5 (Limiters.h:93-96, Constants.h:11)
            eps2 = 125.0f * (g[0].h * g[1].h * g[2].h);
        }
        const int box = r.box;
        // second positions: one face state per variable, W + dd or W - dd
        // along x (ring cells left/right of the tile) or y (below/above)
        int fdst = 0, fstride = 0, fax = 0;
        float fsg = 1.0f;
        if (p == 1) {
            const int role = it.role;
            fax = role >= 3 ? 1 : 0;
            fsg = (role == 2 || role == 4) ? -1.0f : 1.0f;
            if (role == 1) fdst = T::fvx(0, it.cy2, 0);
            else if (role == 2) fdst = T::fvx(0, it.cy2, T::TX + 1);
            else if (role == 3) fdst = T::fvy(0, 0, it.cx2);
            else fdst = T::fvy(0, T::TY + 1, it.cx2);
            fstride = fax ? (T::TY + 2) * T::TX : T::TY * (T::TX + 2);
        }
#pragma unroll
        for (int v = 0; v < NV; ++v) {
            const float w0 = smw[T::w(s0, v, box)];
            float nm[3], np[3], dd[3] = {0.0f, 0.0f, 0.0f}, lim = 1.0f;
            nm[0] = smw[T::w(s0, v, box - 1)];
            np[0] = smw[T::w(s0, v, box + 1)];
            nm[1] = smw[T::w(s0, v, box - T::BX)];
            np[1] = smw[T::w(s0, v, box + T::BX)];
            nm[2] = smw[T::w(sm1, v, box)];
            np[2] = smw[T::w(sp1, v, box)];
            if (KIND != K_PWC) half_slopes<KIND>(w0, nm, np, g, eps2, dd, lim);
            // face states as explicit FMAs (never split or re-fused by the
            // compiler): a ring cell's state is computed by its own CTA and
            // by the neighbouring CTA along different code paths, and must
            // agree
            if (p == 0) {
                fv[T::fvx(v, it.cy, it.cx + 1)] = __fmaf_rn(dd[0], lim, w0);
                fv[T::fvy(v, it.cy + 1, it.cx)] = __fmaf_rn(dd[1], lim, w0);
                urx.v[v] = __fmaf_rn(-dd[0], lim, w0);
                ury.v[v] = __fmaf_rn(-dd[1], lim, w0);
                ulz.v[v] = __fmaf_rn(dd[2], lim, w0);
                urz.v[v] = __fmaf_rn(-dd[2], lim, w0);
            } else {
                const float dsel = fax ? dd[1] : dd[0];
                fv[fdst + v * fstride] = __fmaf_rn(fsg > 0.0f ? dsel : -dsel, lim, w0);
            }
        }
    }
}

// Flux through one face on axis A from its two states (boundary image on a
// non-periodic domain face: g == 0 or g == n), stored at `out` (stride vs).
template <int SOLVER, int A>
__device__ __forceinline__ float face_flux(const MixPhys& mp, float UL[NV], float UR[NV], int g, int n, int per,
                                           int f, float F[NV]) {
    // f: the face's index on its side (tangential cell indices), for a
    // position-dependent side's marker
    if (g == 0 && !per) {
#pragma unroll
        for (int v = 0; v < NV; ++v) UL[v] = UR[v];
        bc32(mp, bc_id32(mp, 2 * A, f), A, UL);
    } else if (g == n && !per) {
#pragma unroll
        for (int v = 0; v < NV; ++v) UR[v] = UL[v];
        bc32(mp, bc_id32(mp, 2 * A + 1, f), A, UR);
    }
    return flux32<SOLVER, A>(mp, UL, UR, F);
}

// The x face left of the own cell and the y face below it (side by side),
// and the tile's far faces on the threads that hold them.
template <class T, int SOLVER>
__device__ __forceinline__ void faces_xy(const ProbDesc& d, const Item3& it, float* sm, int k, const W5& urx,
                                         const W5& ury) {
    const MixPhys& mp = d.mp;
    const float* fv = sm + T::OFF_FV / 4;
    float* ff = sm + T::OFF_FX / 4;
    const int gi = it.i0 + it.cx, gj = it.j0 + it.cy;
    {
        float UL0[NV], UR0[NV], UL1[NV], UR1[NV], F0[NV], F1[NV];
#pragma unroll
        for (int v = 0; v < NV; ++v) {
            UL0[v] = fv[T::fvx(v, it.cy, it.cx)];
            UR0[v] = urx.v[v];
            UL1[v] = fv[T::fvy(v, it.cy, it.cx)];
            UR1[v] = ury.v[v];
        }
        // a face outside the domain is computed on whatever the registers
        // hold and not stored
        const bool ok0 = gi <= d.kn[0] && gj < d.kn[1];
        const bool ok1 = gi < d.kn[0] && gj <= d.kn[1];
        const float l0 = face_flux<SOLVER, 0>(mp, UL0, UR0, gi, d.kn[0], d.kper[0], gj + d.kn[1] * k, F0);
        const float l1 = face_flux<SOLVER, 1>(mp, UL1, UR1, gj, d.kn[1], d.kper[1], gi + d.kn[0] * k, F1);
        if (ok0) {
#pragma unroll
            for (int v = 0; v < NV; ++v) ff[T::fx(v, it.cy, it.cx)] = F0[v];
            ff[T::fx(NV, it.cy, it.cx)] = l0;
        }
        if (ok1) {
#pragma unroll
            for (int v = 0; v < NV; ++v) ff[T::fy(v, it.cy, it.cx)] = F1[v];
            ff[T::fy(NV, it.cy, it.cx)] = l1;
        }
    }
    const int tid = threadIdx.x;
    if (tid >= T::FFY && tid < T::FFY + T::TX) {
        // y face above the tile's top row, column c
        const int c = tid - T::FFY;
        const int fi = it.i0 + c, fj = it.j0 + T::TY;
        if (fi < d.kn[0] && fj <= d.kn[1]) {
            float UL[NV], UR[NV], F[NV];
#pragma unroll
            for (int v = 0; v < NV; ++v) {
                UL[v] = fv[T::fvy(v, T::TY, c)];
                UR[v] = fv[T::fvy(v, T::TY + 1, c)];
            }
            const float l = face_flux<SOLVER, 1>(mp, UL, UR, fj, d.kn[1], d.kper[1], fi + d.kn[0] * k, F);
#pragma unroll
            for (int v = 0; v < NV; ++v) ff[T::fy(v, T::TY, c)] = F[v];
            ff[T::fy(NV, T::TY, c)] = l;
        }
    } else if (tid >= T::FFX && tid < T::FFX + T::TY) {
        // x face right of the tile's last column, row r
        const int r = tid - T::FFX;
        const int fi = it.i0 + T::TX, fj = it.j0 + r;
        if (fi <= d.kn[0] && fj < d.kn[1]) {
            float UL[NV], UR[NV], F[NV];
#pragma unroll
            for (int v = 0; v < NV; ++v) {
                UL[v] = fv[T::fvx(v, r, T::TX)];
                UR[v] = fv[T::fvx(v, r, T::TX + 1)];
            }
            const float l = face_flux<SOLVER, 0>(mp, UL, UR, fi, d.kn[0], d.kper[0], fj + d.kn[1] * k, F);
#pragma unroll
            for (int v = 0; v < NV; ++v) ff[T::fx(v, r, T::TX)] = F[v];
            ff[T::fx(NV, r, T::TX)] = l;
        }
    }
}

// Residual R and spectral radius of the own cell in plane k from the x/y
// face fluxes in shared memory and the z-face fluxes below (fdn) and above
// (fup) in registers; R^{n+1} written in FP32.
template <class T, int SOLVER>
__device__ __forceinline__ void residual3(const ProbDesc& d, const Item3& it, const float* sm,
                                          float* __restrict__ Rout, int k, const float (&fdn)[NV + 1],
                                          const float (&fup)[NV + 1], float& srmax, float (&nrm)[NV]) {
    const float* ff = sm + T::OFF_FX / 4;
    const AxisGeo gz = d.kgeo[2][k + d.kgoff[2]];
    const float hz = gz.h, ihz = gz.ih;
    const CellGeo3& cg = it.cg;
    const int cx = it.cx, cy = it.cy;
    const float fsx = cg.hy * hz, fsy = cg.hx * hz, fsz = cg.fsz;
    const float iv = cg.ixy * ihz;
    const float kx = flux_scale<SOLVER>() * fsx, ky = flux_scale<SOLVER>() * fsy, kz = flux_scale<SOLVER>() * fsz;
    float R[NV];
    const float lxl = ff[T::fx(NV, cy, cx)], lxr = ff[T::fx(NV, cy, cx + 1)];
#pragma unroll
    for (int v = 0; v < NV; ++v) R[v] = -(ff[T::fx(v, cy, cx + 1)] - ff[T::fx(v, cy, cx)]) * kx;
    float sr = fsx * (lxl + lxr);
    if (cg.farx != 0.0f) srmax = fmaxf(srmax, fsx * lxr * cg.farx * ihz);
#pragma unroll
    for (int v = 0; v < NV; ++v) R[v] -= (ff[T::fy(v, cy + 1, cx)] - ff[T::fy(v, cy, cx)]) * ky;
    const float lyr = ff[T::fy(NV, cy + 1, cx)];
    sr += fsy * (ff[T::fy(NV, cy, cx)] + lyr);
    if (cg.fary != 0.0f) srmax = fmaxf(srmax, fsy * lyr * cg.fary * ihz);
#pragma unroll
    for (int v = 0; v < NV; ++v) R[v] -= (fup[v] - fdn[v]) * kz;
    sr += fsz * (fdn[NV] + fup[NV]);
    if (k == d.kn[2] - 1) srmax = fmaxf(srmax, fsz * fup[NV] * cg.ixy * d.kgeo[2][d.kn[2] + d.kgoff[2]].ih);
    srmax = fmaxf(srmax, sr * iv);
    // source terms after the face fluxes (kernel.h:941-989), on the working state
    const MixPhys& mp = d.mp;
    const float vol = fsz * hz;
    if (mp.force || mp.accel) {
        // the own cell's working state of plane k
        const float* smw = sm + T::OFF_W / 4;
        const int box = (cx + HB3) + (cy + HB3) * T::BX, s0 = T::wslot(k);
        const float ro = smw[T::w(s0, 0, box)];
        const float iro = 1.0f / ro;
        const float vu = smw[T::w(s0, 1, box)] * iro, vv = smw[T::w(s0, 2, box)] * iro,
                    vw = smw[T::w(s0, 3, box)] * iro;
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
    if (mp.norms) {
#pragma unroll
        for (int v = 0; v < NV; ++v) nrm[v] += vol * fabsf(R[v]);
    }
    const unsigned int o = (unsigned int)it.own_off + (unsigned int)k * (unsigned int)d.kstr[2];
    const size_t plane = (size_t)d.L.plane;
#pragma unroll
    for (int v = 0; v < NV; ++v) __stcs(Rout + o + v * plane, R[v]);
}

// One work item: the tile column (i0, j0) over planes [z0, z1).  Planes
// z0-2 .. z1+1 are loaded.  Pass k (two phases, one barrier each):
//   A: conversion of plane k+2; x/y faces of plane k;
//   B: slopes of plane k+1; z face k / k+1; residual of plane k.
template <class T, int SOLVER, int KIND>
__device__ __forceinline__ void march(const ProbDesc& d, const Mix3dMaps& maps, const Item3& it, int par, float dtf,
                                      unsigned char* smem, uint64_t* bar, unsigned int& phase, float& srmax,
                                      unsigned int& health, float (&nrm)[NV]) {
    const double* __restrict__ Uin = d.U[par];
    double* __restrict__ Uout = d.U[par ^ 1];
    const float* __restrict__ Rin = d.R[par];
    float* __restrict__ Rout = d.R[par ^ 1];
    float* sm = reinterpret_cast<float*>(smem);
    float* smw = sm + T::OFF_W / 4;
    const int z0 = it.z0, z1 = it.z1, last = z1 + 1;
    volatile unsigned int* fail = reinterpret_cast<volatile unsigned int*>(smem + T::OFF_FAIL);
    // after a wait gave up (seen by every thread at the next barrier), no
    // thread waits and no load is issued again: no arrival on a barrier
    // whose phase is still open
    const bool lead = threadIdx.x == 0;
    auto stage_of = [&](int j) { return (j - (z0 - 2)) & 1; };
    auto wait_stage = [&](int j) {
        const int s = stage_of(j);
        if (!*fail && !mbar_wait(&bar[s], (phase >> s) & 1u)) {
            health |= TS_HEALTH_TIMEOUT;
            *fail = 1u;
        }
        phase ^= 1u << s;
        return smem + T::OFF_STAGE + s * T::STAGE;
    };
    auto issue = [&](int j) {
        if (lead && !*fail) issue_plane<T>(d, maps, par, smem, bar, stage_of(j), it.i0, it.j0, j);
    };
    PendingU pu;
    pu.on = false;
    W5 urx, ury, ulz, urz;  // own cell: right-hand x/y states of the last reconstructed plane, z states
    float fdn[NV + 1], fup[NV + 1];  // z-face fluxes below and above the plane of the residual
#pragma unroll
    for (int v = 0; v <= NV; ++v) fdn[v] = fup[v] = 0.0f;

    issue(z0 - 2);
    issue(z0 - 1);
    // one loop for the start-up passes too (k = z0-4 .. z0-2 convert planes
    // z0-2 .. z0 and reconstruct plane z0-1): a single copy of each phase
    // keeps the kernel's code small
#pragma unroll 1
    for (int k = z0 - 4; k < z1; ++k) {
        // phase A
        convert<T>(d, it, wait_stage(k + 2), Uin, Rin, Uout, smw, k + 2, dtf, pu, health);
        if (k >= z0) faces_xy<T, SOLVER>(d, it, sm, k, urx, ury);
        __syncthreads();
        if (k + 4 <= last) issue(k + 4);
        // the owned cell's FP64 update of plane k+2 overlaps the work below
        apply_pending(d, Uout, pu, health);
        if (k < z0 - 2) continue;  // k + 1 < z0 - 1: nothing to reconstruct yet
        // phase B
        const W5 ulz_k = ulz;
        reconstruct<T, KIND>(d, it, sm, k + 1, urx, ury, ulz, urz);
        if (k >= z0 - 1 && it.own) {
            float UL[NV], UR[NV];
#pragma unroll
            for (int v = 0; v < NV; ++v) {
                UL[v] = ulz_k.v[v];
                UR[v] = urz.v[v];
            }
            fup[NV] = face_flux<SOLVER, 2>(d.mp, UL, UR, k + 1, d.kn[2], d.kper[2],
                                           (it.i0 + it.cx) + d.kn[0] * (it.j0 + it.cy), fup);
            if (k >= z0) residual3<T, SOLVER>(d, it, sm, Rout, k, fdn, fup, srmax, nrm);
#pragma unroll
            for (int v = 0; v <= NV; ++v) fdn[v] = fup[v];
        }
        __syncthreads();
    }
}

// The CTA's CFL maximum, health and residual norms into the problem's
// control word; the CTA that completes the problem's last item closes the
// step.
template <class T>
__device__ __forceinline__ void close3(const ProbDesc& d, int n_closes, float srmax, unsigned int health,
                                       float (&nrm)[NV], float* wmax, unsigned int* whealth) {
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    if (d.mp.norms) add_norms(d.ctl, nrm, 0xffffffffu, lane, 32);
    const unsigned int mbits = __reduce_max_sync(0xffffffffu, __float_as_uint(srmax));
    health = __reduce_or_sync(0xffffffffu, health);
    if (lane == 0) { wmax[wid] = __uint_as_float(mbits); whealth[wid] = health; }
    __syncthreads();
    if (threadIdx.x == 0) {
        float m = 0.0f;
        unsigned int hh = 0;
        for (int k = 0; k < T::NT / 32; ++k) { m = fmaxf(m, wmax[k]); hh |= whealth[k]; }
        Ctl* ctl = d.ctl;
        if (m > 0.0f) atomicMax(&ctl->srmax_bits, __float_as_uint(m));
        if (hh) atomicOr(&ctl->health, hh);
        __threadfence();
        if (atomicAdd(&ctl->blocks_done, 1u) == (unsigned)(n_closes - 1)) {
            __threadfence();
            finish_problem(ctl, d.mp.cfl);
        }
    }
}

template <int TX, int TY, int SOLVER, int KIND>
__global__ void __launch_bounds__(TX * TY, TX * TY <= 256 ? 2 : 1) k_mix3d(const __grid_constant__ ProbDesc d,
                                                      const __grid_constant__ Mix3dMaps maps) {
    using T = Tile3<TX, TY>;
    // all shared memory is dynamic, so the TMA stages start 128-byte aligned
    extern __shared__ __align__(1024) unsigned char smem[];
    float* wmax = reinterpret_cast<float*>(smem + T::OFF_RED);
    unsigned int* whealth = reinterpret_cast<unsigned int*>(smem + T::OFF_RED + 32 * 4);
    if (d.ctl->stop_req) return;
    const int par = d.ctl->parity;
    const float dtf = __double2float_rn(d.ctl->dt_apply);  // once per launch
    uint64_t* bar = reinterpret_cast<uint64_t*>(smem + T::OFF_BAR);
    if (threadIdx.x == 0) {
        *reinterpret_cast<volatile unsigned int*>(smem + T::OFF_FAIL) = 0u;
        mbar_init(&bar[0], 1);
        mbar_init(&bar[1], 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    }
    __syncthreads();
    unsigned int phase = 0;
    // every CTA closes once, after all its items (the CTA count is d.nq)
    float srmax = 0.0f, nrm[NV] = {0.0f, 0.0f, 0.0f, 0.0f, 0.0f};
    unsigned int health = 0;
    const int n_items = d.ncol * ((d.kn[2] + d.ch - 1) / d.ch);
    for (int q = blockIdx.x; q < n_items; q += gridDim.x) {
        __syncthreads();  // the previous item is finished with shared memory
        Item3 it;
        setup_item<T>(d, q, it);
        march<T, SOLVER, KIND>(d, maps, it, par, dtf, smem, bar, phase, srmax, health, nrm);
    }
    close3<T>(d, d.nq, srmax, health, nrm, wmax, whealth);
}

// ---------------------------------------------------------------------------
// Host side
// ---------------------------------------------------------------------------
#define TS_MIX3D_TILES(X) X(32, 8) X(16, 16) X(32, 16)

template <class F>
bool with3d(int tx, int ty, int solver, int kind, F&& f) {
    bool found = false;
#define TS_TRY3(TX_, TY_)                                                                                      \
    if (!found && tx == TX_ && ty == TY_) {                                                                   \
        found = true;                                                                                         \
        auto go = [&]<int S>() {                                                                              \
            switch (kind) {                                                                                   \
            case K_PWC: f.template operator()<TX_, TY_, S, K_PWC>(); break;                                   \
            case K_LINEAR: f.template operator()<TX_, TY_, S, K_LINEAR>(); break;                             \
            case K_ENO2: f.template operator()<TX_, TY_, S, K_ENO2>(); break;                                 \
            case K_LIM_VK: f.template operator()<TX_, TY_, S, K_LIM_VK>(); break;                             \
            default: f.template operator()<TX_, TY_, S, K_LIM_BJ>(); break;                                   \
            }                                                                                                 \
        };                                                                                                    \
        if (solver == TS_RS_HLLC) go.template operator()<TS_RS_HLLC>();                                       \
        else go.template operator()<TS_RS_ROE_PIKE>();                                                        \
    }
    TS_MIX3D_TILES(TS_TRY3)
#undef TS_TRY3
    return found;
}

PFN_cuTensorMapEncodeTiled_v12000 encode_fn() {
    static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
    static std::once_flag once;
    std::call_once(once, [] {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
    });
    return fn;
}

// 4D map over one SoA state buffer: x (the padded row), y, z (with ghost
// layers), variable; box = the tile plus its 2-cell halo, one plane, all
// five variables.
ts_status make_map(CUtensorMap* m, void* base, bool f64, const Layout& L, int bx, int by, std::string& err) {
    PFN_cuTensorMapEncodeTiled_v12000 fn = encode_fn();
    if (!fn) { err = "cuTensorMapEncodeTiled is not available"; return TS_ERR_CUDA; }
    const cuuint64_t es = f64 ? 8 : 4;
    const cuuint64_t dims[4] = {(cuuint64_t)L.px, (cuuint64_t)L.ey, (cuuint64_t)L.ez, (cuuint64_t)NV};
    const cuuint64_t strides[3] = {(cuuint64_t)L.px * es, (cuuint64_t)L.px * L.ey * es, (cuuint64_t)L.plane * es};
    const cuuint32_t box[4] = {(cuuint32_t)bx, (cuuint32_t)by, 1u, (cuuint32_t)NV};
    const cuuint32_t estr[4] = {1u, 1u, 1u, 1u};
    const CUresult r = fn(m, f64 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT64 : CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 4, base, dims,
                          strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                          CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) { err = "cuTensorMapEncodeTiled failed (" + std::to_string((int)r) + ")"; return TS_ERR_CUDA; }
    return TS_OK;
}

}  // namespace

bool mix3d_tile_info(int tx, int ty, int solver, int recon, int limiter, size_t* smem, int* per_sm) {
    MixPhys mp{};
    mp.recon = recon;
    mp.limiter = limiter;
    return with3d(tx, ty, solver, kind_of(mp), [&]<int TX, int TY, int S, int K>() {
        using T = Tile3<TX, TY>;
        *smem = T::BYTES;
        *per_sm = 0;
        if (cudaFuncSetAttribute(k_mix3d<TX, TY, S, K>, cudaFuncAttributeMaxDynamicSharedMemorySize, T::BYTES) !=
            cudaSuccess)
            return;
        cudaFuncSetAttribute(k_mix3d<TX, TY, S, K>, cudaFuncAttributePreferredSharedMemoryCarveout, 100);
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(per_sm, k_mix3d<TX, TY, S, K>, T::NT, T::BYTES);
    });
}

ts_status mix3d_make_maps(const ProbDesc& d, int tx, int ty, Mix3dMaps& maps, std::string& err) {
    const Layout& L = d.L;
    if (L.nd != 3 || L.gx != HB3 || L.gy != HB3 || L.gz != HB3) { err = "3D layout expected"; return TS_ERR_INVALID; }
    const int bx = tx + 2 * HB3, by = ty + 2 * HB3;
    ts_status s;
    for (int b = 0; b < 2; ++b) {
        if ((s = make_map(&maps.u[b], d.U[b], true, L, bx, by, err)) != TS_OK) return s;
        if ((s = make_map(&maps.r[b], d.R[b], false, L, bx, by, err)) != TS_OK) return s;
    }
    return TS_OK;
}

void mix3d_launch(int tx, int ty, int grid, const ProbDesc& d, const Mix3dMaps& maps, cudaStream_t st) {
    if (grid <= 0) return;
    with3d(tx, ty, d.mp.solver, kind_of(d.mp), [&]<int TX, int TY, int S, int K>() {
        using T = Tile3<TX, TY>;
        k_mix3d<TX, TY, S, K><<<grid, T::NT, T::BYTES, st>>>(d, maps);
    });
}

}  // namespace ts
