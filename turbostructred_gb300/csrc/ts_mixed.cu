// Mixed-precision path (placeholder until the fused kernel lands).
#include "ts_mixed.h"

namespace ts {

ts_status mixed_init(const ts_config&, const Layout&, const Phys&, const HostGrid&, Ctl*, const DeviceAlloc&,
                     MixedBufs&, std::string& err) {
    err = "mixed precision path not built yet";
    return TS_ERR_UNSUPPORTED;
}
void mixed_step(MixedBufs&, const Phys&, cudaStream_t, cudaEvent_t*, int* n, const char**) { if (n) *n = 0; }
void mixed_reset(MixedBufs&, cudaStream_t) {}
void mixed_materialize(MixedBufs&, const Phys&, cudaStream_t) {}

}  // namespace ts
