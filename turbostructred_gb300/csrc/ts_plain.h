// Plain FP64 path (bit-for-bit with the reference's CPU step): device buffers
// and the per-step launch sequence.  See ts_plain.cu.
#pragma once

#include <cuda_runtime.h>

#include "ts_internal.h"

namespace ts {

constexpr int kPlainBlock = 128;

struct PlainBufs {
    Layout L;
    double* U;           // NV planes: conserved state
    double* G;           // 3*NV planes: slopes, plane a*NV+v
    double* Lim;         // NV planes: limiter values
    double* F[3];        // NV planes per axis: face fluxes stored at the face's right cell
    double* Lam[3];      // 1 plane per axis: face max eigenvalue
    const double* cx[3]; // cell centres per axis, index i + ghost width
    const double* ch[3]; // cell sizes per axis
    const double* eps2;  // Venkatakrishnan eps^2 per cell (one plane) or null
    double* partial;     // per-block minima of V/SR
    Ctl* ctl;
    double* VG;          // viscous flow: 9 planes, d(velocity d)/d(axis e) at plane 3d+e
    double* VSR[3];      // viscosity > 0: 1 plane per axis, the face's viscous
                         // spectral-radius term, stored at the face's right cell
};

int plain_partial_blocks(const Layout& L);

// Enqueues one step.  With `ev` non-null, records ev[0] before the first
// launch and ev[i+1] after launch i (ev needs kPlainMaxLaunches+1 events);
// *n_launch receives the launch count and names[i] the kernel names.
constexpr int kPlainMaxLaunches = 14;
cudaError_t plain_step(const PlainBufs& b, const Phys& ph, cudaStream_t st, cudaEvent_t* ev = nullptr,
                       int* n_launch = nullptr, const char** names = nullptr);

}  // namespace ts
