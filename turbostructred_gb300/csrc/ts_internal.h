// Internal types shared by the host code and the CUDA kernels of the
// GB300-native explicit FVM step.  Not part of the C ABI.
#pragma once

#include <cuda_runtime.h>

#include <cstddef>
#include <cstdint>
#include <string>
#include <vector>

#include "ts_fvm.h"

#ifdef __CUDACC__
#define TS_HD __host__ __device__ __forceinline__
#else
#define TS_HD inline
#endif

namespace ts {

// The device address, on `device`, of page-locked host memory allocated or
// registered against that device (cudaHostAlloc, cudaHostRegister, a pinned
// PyTorch tensor), or nullptr for any other pointer.  Kernels read and write
// such memory in place over the host link, so a state in it needs no staging
// copy through device memory; memory pinned for another device is staged
// (without cudaHostAllocPortable it is mapped for its own device only).
inline void* pinned_device_ptr(const void* p, int device) {
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    return a.type == cudaMemoryTypeHost && a.device == device ? a.devicePointer : nullptr;
}

constexpr int NV = 5;      // rho, rho*u, rho*v, rho*w, rho*E
constexpr int GHOST = 2;   // ghost layers per active axis in device arrays

// Device field layout: structure of arrays, one plane per variable, x fastest.
// Active axes carry GHOST ghost layers each side (the reference uses one;
// the second serves the fused mixed-precision stencil).  Rows are padded to
// a multiple of 8 elements so FP64 and FP32 rows start 64/32-byte aligned,
// and the first interior cell of a row sits at an even x offset, which keeps
// TMA boxes that start two cells before a tile 16-byte aligned.
struct Layout {
    int nd, nx, ny, nz;  // interior cells
    int gx, gy, gz;      // ghost widths (GHOST on active axes, else 0)
    int ex, ey, ez;      // extents including ghosts
    int px;              // row pitch in elements
    long long plane;     // elements per variable plane

    TS_HD long long at(int i, int j, int k) const {
        return ((long long)(k + gz) * ey + (j + gy)) * px + (i + gx);
    }
    TS_HD int n(int a) const { return a == 0 ? nx : (a == 1 ? ny : nz); }
    TS_HD long long stride(int a) const {
        return a == 0 ? 1LL : (a == 1 ? (long long)px : (long long)px * ey);
    }
    TS_HD long long cells() const { return (long long)nx * ny * nz; }
};

Layout make_layout(const ts_config& c);

// Boundary conditions: entries 0-5 are the six domain sides' own BCs (x-,
// x+, y-, y+, z-, z+), entries 6.. the extra kinds a position-dependent side
// selects face by face through its marker array (device memory; null for a
// side with one BC).
constexpr int kBcIds = 6 + TS_MAX_BC_KINDS;
struct BcSet {
    int type[kBcIds];
    double density[kBcIds];
    double vel[kBcIds][3];
    double pstatic[kBcIds];
    const uint8_t* mark[6];
};

// BC table entry of boundary face f of `side` (faces numbered by the side's
// tangential cell indices, lower axis fastest: x sides j + ny k, y sides
// i + nx k, z sides i + nx j).
TS_HD int bc_id(const uint8_t* const mark[6], int side, int f) {
    const uint8_t* m = mark[side];
    return m ? 6 + (int)m[f] : side;
}
TS_HD int face_index(int side, int i, int j, int k, int nx, int ny) {
    const int a = side >> 1;
    return a == 0 ? j + ny * k : (a == 1 ? i + nx * k : i + nx * j);
}

// Boundary faces of a side (the length of its marker array).
inline long long side_faces(const ts_config& c, int side) {
    const long long nx = c.nx, ny = c.n_dims > 1 ? c.ny : 1, nz = c.n_dims > 2 ? c.nz : 1;
    const int a = side >> 1;
    return a == 0 ? ny * nz : (a == 1 ? nx * nz : nx * ny);
}
// A config with at least one position-dependent side.
inline bool has_markers(const ts_config& c) {
    for (int s = 0; s < 6; ++s)
        if (c.bc_marker[s]) return true;
    return false;
}

// Physics and method selection passed by value to kernels.
struct Phys {
    int nd;
    int recon, limiter, solver, eos;
    int periodic[3];
    double gamma, p_inf, eps, cfl;
    BcSet bc;
    int force, accel;          // source terms on (kernel.h:941-989)
    double sigma[3], g[3];     // Sigma, UniformAcceleration
    int viscous;               // IsViscousFlow: viscous face fluxes
    double visc;               // Viscosity: also in the spectral radius
};

// Per-handle step control word in device memory (StepInfo, kernel.h:31-39).
struct Ctl {
    double time;
    double dt;
    double next_sol;
    double next_slice;
    double res[5];
    int iteration;
    unsigned int health;
    unsigned int blocks_done;  // last-block-done counter of the dt reduction
    int stop_req;              // sticky: later kernels of a finished Run exit
    int run_mode;              // 1 under Kernel::Run termination rules
    int max_iteration;
    double max_time;
    double save_sol, save_slice;
    double dt_min_raw;         // min(V/SR) before CFL and clipping
    // mixed-precision path (deferred stage update)
    double dt_apply;           // dt of the residual still waiting to be applied
    int parity;                // which of the two state/residual buffers is current
    unsigned int srmax_bits;   // running max of SR/V as FP32 bits (positive floats order as uints)
    double res_acc[5];         // residual norms of the stage in flight (moved to res when it closes)
};

// Host copy of the grid in the reference's layout (one ghost per active
// axis), grid.h:124-344.
struct HostGrid {
    std::vector<double> x, hx, y, hy, z, hz;
};

ts_status build_grid(const ts_config& c, HostGrid& g, std::string& err);

// The configuration a handle was created with (blocks point into the handle).
const ts_config& handle_config(const ts_handle* h);
// Joins a handle's pending asynchronous file writes; the first failure, if any.
void io_join_all(const ts_handle* h, ts_status* status, std::string* error);
ts_status validate_config(const ts_config& c, std::string& err);
Phys make_phys(const ts_config& c);

void set_error(const std::string& msg);
ts_status fail(ts_status s, const std::string& msg);

}  // namespace ts
