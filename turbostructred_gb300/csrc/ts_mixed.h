// Mixed-precision path: FP32 reconstruction, EOS and Riemann flux with FP64
// state, FP64 stage accumulation and FP64 dt.  One fused kernel advances a
// work list of (problem, tile column, z chunk) items of one or many problems
// by one stage.  See ts_mixed.cu.
#pragma once

#include <cuda.h>
#include <cuda_runtime.h>

#include <functional>
#include <string>

#include "ts_internal.h"

namespace ts {

// Per-axis geometry of one cell index (device, indexed i + ghost width).
struct AxisGeo {
    float h;      // cell size
    float hh;     // h / 2
    float ks;     // h / (2 (x[i+1] - x[i-1])): central slope -> half projection
    float il;     // 1 / (x[i] - x[i-1])
    float ir;     // 1 / (x[i+1] - x[i])
    float ih;     // 1 / h
};

// Physics constants of one problem for the FP32 flux path.
struct MixPhys {
    int nd, recon, limiter, solver, eos;
    int periodic[3];
    float gamma, gm1, pinf, einf, eps;
    double einf_d;        // gamma p_inf / (gamma - 1): energy shift, applied in FP64
    double cfl;
    // BC table: the six sides' own BCs (entries 0-5) inline; the extra kinds
    // a position-dependent side selects per face through `mark` (entries
    // 6..) in device memory, read only at such faces
    int bc_type[6];
    float bc_state[6][5];  // SubsonicInlet ghost state (shifted energy)
    float bc_vel[6][3];    // MovingWall velocity
    const uint8_t* mark[6];            // per-face kind of a position-dependent side (device), or null
    const struct MixBcKinds* kinds;    // entries 6.. (device), or null
    int force, accel;      // source terms on (kernel.h:941-989)
    float sigma[3], g[3];  // Sigma, UniformAcceleration
    int norms;             // form the residual norms sum V |R| (kernel.h:326)
};

// The extra BC kinds of position-dependent sides (table entries 6..).
struct MixBcKinds {
    int type[TS_MAX_BC_KINDS];
    float state[TS_MAX_BC_KINDS][5];
    float vel[TS_MAX_BC_KINDS][3];
};

// Everything the fused kernel needs about one problem (lives in device memory).
// The kernel works on kernel axes 0 (x), 1 (the tile's second axis, 3D
// only) and 2 (the marching axis: z in 3D, y in 2D); the k* fields map them
// to the problem's axes.  Inactive kernel axes have one cell.
struct ProbDesc {
    Layout L;
    double* U[2];          // NV FP64 planes each: U^n and U^{n+1}
    float* R[2];           // NV FP32 planes each: pending residual
    Ctl* ctl;              // per-problem step control word
    const AxisGeo* kgeo[3];  // geometry per kernel axis, indexed cell + kgoff
    int kgoff[3];
    int kn[3];             // cells along each kernel axis
    int kper[3];           // periodic
    int kphys[3];          // problem axis (momentum component; BC sides 2a, 2a+1)
    long long kstr[3];     // element strides
    long long kbase;       // element offset of cell (0, 0, 0)
    MixPhys mp;
    int ncx, ncol;         // tile columns along x, in total
    int ch, nq;            // planes per marching chunk, work items (columns x chunks)
};

// TMA descriptors of a 3D problem's state buffers (U[b] FP64, R[b] FP32),
// for the 3D fused kernel; kernel parameters.
struct Mix3dMaps {
    CUtensorMap u[2];
    CUtensorMap r[2];
};

struct MixedBufs {
    ProbDesc desc;                 // host copy
    Mix3dMaps maps;                // 3D problems: tensor maps of the state buffers
    ProbDesc* d_desc = nullptr;    // device copy
    int tx = 32, ty = 8;           // tile (one of the compiled shapes)
    int zchunks = 1;               // z chunks per column (3D)
    int grid = 0;                  // persistent CTAs
    size_t smem = 0;
    int sms = 0;
};

using DeviceAlloc = std::function<ts_status(size_t bytes, void** out)>;

// Geometry and physics of one problem (host work + uploads through `alloc`,
// queued on stream `st`: work queued there later sees them).
ts_status mixed_problem(const ts_config& c, const Layout& L, const Phys& ph, const HostGrid& g, Ctl* ctl,
                        const DeviceAlloc& alloc, ProbDesc& d, std::string& err, cudaStream_t st);
// Cells per tile along x and y of a compiled tile of tx x ty threads (one-row
// tiles of 1D and 2D problems own tx - 4 cells).
void mixed_tile_cells(int nd, int tx, int ty, int* cx, int* cy);
// Work items of a problem for a tile and chunking of the marching axis
// (0 = automatic, given the persistent grid size `slots`).
void mixed_items(ProbDesc& d, int tx, int ty, int zchunks, long long slots);
// Compiled tile lookup: smem bytes and resident CTAs per SM (of the batched
// kernel when `batch`), or false.
bool mixed_tile_info(int nd, int tx, int ty, int solver, size_t* smem, int* per_sm, bool batch = false);
// One stage of one problem (descriptor passed by value).
void mixed_launch_single(int nd, int tx, int ty, int solver, int grid, const ProbDesc& h_desc, cudaStream_t st);
// One stage of a list of (problem, item) pairs of 1D or 2D problems sharing
// the solver and tile (d_ctls[p] is problem p's control word); false when no
// batched kernel exists for (nd, tile).  The stage is closed afterwards by
// mixed_batch_finish over the listed problems, or, with close_in_kernel, by
// the CTA that completes each problem's last item (one launch per stage
// instead of two; the returned per-item atomics cost more than the saved
// launch when the list is long).
bool mixed_launch_batch(int nd, int tx, int ty, int solver, int grid, const ProbDesc* d_probs, const Ctl* d_ctls,
                        const int2* d_items, int n_items, cudaStream_t st, bool close_in_kernel = false);
void mixed_batch_finish(const ProbDesc* d_probs, const int* d_slots, int n, cudaStream_t st);

// Tail of a batch: n_problems 1D problems (d_list: their descriptor indices),
// each advanced by up to `budget` stages in one launch by a cluster of
// `cluster` CTAs that own mixed_tail_cells() cells each and keep the state
// on chip between stages (same arithmetic as the batched kernel).
constexpr int kTailMaxCluster = 16;
int mixed_tail_cells();
// The tail kernel can run clusters of this size on this device.
bool mixed_tail_ready(int solver, int cluster);
cudaError_t mixed_launch_tail(int solver, int cluster, int n_problems, const ProbDesc* d_probs, const int* d_list,
                              int budget, cudaStream_t st);

// Set-up of one problem's buffers; every upload and (with zero_buffers) the
// clearing of the state and residual buffers are queued on `st`.
ts_status mixed_init(const ts_config& c, const Layout& L, const Phys& ph, const HostGrid& g, Ctl* ctl,
                     const DeviceAlloc& alloc, MixedBufs& mb, std::string& err, cudaStream_t st,
                     bool zero_buffers = true);
// Choose the tile shape (tx, ty) and the z chunking (0 = automatic), and
// recompute the persistent grid (descriptor upload queued on `st`).
ts_status mixed_set_tile(MixedBufs& mb, int tx, int ty, int zchunks, std::string& err, cudaStream_t st);

// 3D problems: the TMA-staged fused kernel (ts_mix3d.cu).  Compiled tiles
// 32x8 and 16x16; smem bytes and resident CTAs per SM, or false.
bool mix3d_tile_info(int tx, int ty, int solver, int recon, int limiter, size_t* smem, int* per_sm);
// Tensor maps of the four state buffers for the tile's box.
ts_status mix3d_make_maps(const ProbDesc& d, int tx, int ty, Mix3dMaps& maps, std::string& err);
void mix3d_launch(int tx, int ty, int grid, const ProbDesc& d, const Mix3dMaps& maps, cudaStream_t st);

constexpr int kMixedMaxLaunches = 4;
void mixed_step(MixedBufs& mb, const Phys& ph, cudaStream_t st, cudaEvent_t* ev = nullptr, int* n_launch = nullptr,
                const char** names = nullptr);
// After a new state was written into U[parity]: no pending residual.
void mixed_reset(MixedBufs& mb, cudaStream_t st);
// Applies the pending residual so U[parity] holds the current state.
void mixed_materialize(MixedBufs& mb, const Phys& ph, cudaStream_t st);
// The same for problem p of a device descriptor array.
void mixed_apply(const ProbDesc* d_probs, int p, long long cells, cudaStream_t st);
// Current state buffer (host must have pulled ctl->parity).
double* mixed_state(MixedBufs& mb, int parity);

}  // namespace ts
