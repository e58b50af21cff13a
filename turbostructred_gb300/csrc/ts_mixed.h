// Mixed-precision path: FP32 reconstruction, EOS and Riemann flux with FP64
// state, FP64 stage accumulation and FP64 dt.  See ts_mixed.cu.
#pragma once

#include <cuda_runtime.h>

#include <functional>
#include <string>

#include "ts_internal.h"

namespace ts {

// Per-axis geometry of one cell index (device, indexed i + GHOST).
struct AxisGeo {
    float h;      // cell size
    float hh;     // h / 2
    float ks;     // h / (2 (x[i+1] - x[i-1])): central slope -> half projection
    float il;     // 1 / (x[i] - x[i-1])
    float ir;     // 1 / (x[i+1] - x[i])
    float ih;     // 1 / h
};

// Physics constants for the FP32 flux path, passed by value.
struct MixPhys {
    int nd, recon, limiter, solver, eos;
    int periodic[3];
    int uniform;          // every axis uniform: one volume for all cells
    float gamma, gm1, pinf, einf, eps;
    double einf_d;        // gamma p_inf / (gamma - 1): energy shift, applied in FP64
    double cfl;
    int bc_type[6];
    float bc_state[6][5];  // SubsonicInlet ghost state (shifted energy)
    float bc_vel[6][3];    // MovingWall velocity
};

struct MixedBufs {
    Layout L;
    double* U[2] = {nullptr, nullptr};  // NV FP64 planes each: U^n and U^{n+1}
    float* R[2] = {nullptr, nullptr};   // NV FP32 planes each: pending residual
    const AxisGeo* geo[3] = {nullptr, nullptr, nullptr};
    Ctl* ctl = nullptr;
    MixPhys mp;
    int tx = 32, ty = 8;   // tile (one of the compiled shapes)
    int zchunks = 1;       // z chunks per column (3D)
    int grid = 0;          // persistent CTAs
    size_t smem = 0;
    int sms = 0;
};

using DeviceAlloc = std::function<ts_status(size_t bytes, void** out)>;

ts_status mixed_init(const ts_config& c, const Layout& L, const Phys& ph, const HostGrid& g, Ctl* ctl,
                     const DeviceAlloc& alloc, MixedBufs& mb, std::string& err);
// Choose the tile shape (tx, ty) and the z chunking (0 = automatic), and
// recompute the persistent grid.
ts_status mixed_set_tile(MixedBufs& mb, int tx, int ty, int zchunks, std::string& err);

constexpr int kMixedMaxLaunches = 4;
void mixed_step(MixedBufs& mb, const Phys& ph, cudaStream_t st, cudaEvent_t* ev = nullptr, int* n_launch = nullptr,
                const char** names = nullptr);
// After a new state was written into U[parity]: no pending residual.
void mixed_reset(MixedBufs& mb, cudaStream_t st);
// Applies the pending residual so U[parity] holds the current state.
void mixed_materialize(MixedBufs& mb, const Phys& ph, cudaStream_t st);
// Current state buffer (host must have pulled ctl->parity).
double* mixed_state(MixedBufs& mb, int parity);

}  // namespace ts
