// Mixed-precision path: FP32 reconstruction, EOS and Riemann flux with FP64
// state, stage accumulation and dt.  See ts_mixed.cu.
#pragma once

#include <cuda_runtime.h>

#include <functional>
#include <string>

#include "ts_internal.h"

namespace ts {

struct MixedBufs {
    Layout L;
    double* U = nullptr;  // NV FP64 planes: state U^n
    float* R = nullptr;   // NV FP32 planes: residual R^n, not yet applied
    int pending = 0;      // host flag: R^n awaits application
    Ctl* ctl = nullptr;
};

using DeviceAlloc = std::function<ts_status(size_t bytes, void** out)>;

ts_status mixed_init(const ts_config& c, const Layout& L, const Phys& ph, const HostGrid& g, Ctl* ctl,
                     const DeviceAlloc& alloc, MixedBufs& mb, std::string& err);
constexpr int kMixedMaxLaunches = 4;
void mixed_step(MixedBufs& mb, const Phys& ph, cudaStream_t st, cudaEvent_t* ev = nullptr, int* n_launch = nullptr,
                const char** names = nullptr);
void mixed_reset(MixedBufs& mb, cudaStream_t st);
void mixed_materialize(MixedBufs& mb, const Phys& ph, cudaStream_t st);

}  // namespace ts
