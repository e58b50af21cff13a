// C-ABI entry points (include/ts_fvm.h): handle life cycle, device memory,
// host<->device state transfer and the step/run loops.  Steps are enqueued on
// the handle's stream and replayed from captured CUDA graphs in chunks, so a
// run costs one host synchronisation per chunk, not per step.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <map>
#include <memory>
#include <string>
#include <tuple>
#include <vector>

#include "ts_internal.h"
#include "ts_mixed.h"
#include "ts_plain.h"

using namespace ts;

namespace {

struct DeviceGuard {
    int prev = -1;
    explicit DeviceGuard(int dev) {
        cudaGetDevice(&prev);
        if (prev != dev) cudaSetDevice(dev);
    }
    ~DeviceGuard() {
        int cur = -1;
        cudaGetDevice(&cur);
        if (prev >= 0 && cur != prev) cudaSetDevice(prev);
    }
};

#define TS_CUDA(call)                                                                            \
    do {                                                                                         \
        cudaError_t e_ = (call);                                                                 \
        if (e_ != cudaSuccess)                                                                   \
            return fail(e_ == cudaErrorMemoryAllocation ? TS_ERR_NO_MEMORY : TS_ERR_CUDA,        \
                        std::string(#call) + ": " + cudaGetErrorString(e_));                     \
    } while (0)

// Host AoS (interior or the reference's with-ghost array) <-> device SoA.
__global__ void k_scatter(const double* __restrict__ aos, Layout L, double* __restrict__ U, int with_ghosts,
                          long long n) {
    long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (t >= n) return;
    const int g1 = with_ghosts ? 1 : 0;
    const int sx = L.nx + 2 * g1, sy = L.ny + (L.nd > 1 ? 2 * g1 : 0);
    const int i = (int)(t % sx) - g1;
    const int j = (int)((t / sx) % sy) - (L.nd > 1 ? g1 : 0);
    const int k = (int)(t / ((long long)sx * sy)) - (L.nd > 2 ? g1 : 0);
    const long long c = L.at(i, j, k);
#pragma unroll
    for (int v = 0; v < NV; ++v) U[(long long)v * L.plane + c] = aos[t * NV + v];
}

__global__ void k_gather(double* __restrict__ aos, Layout L, const double* __restrict__ U, int with_ghosts,
                         long long n) {
    long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (t >= n) return;
    const int g1 = with_ghosts ? 1 : 0;
    const int sx = L.nx + 2 * g1, sy = L.ny + (L.nd > 1 ? 2 * g1 : 0);
    const int i = (int)(t % sx) - g1;
    const int j = (int)((t / sx) % sy) - (L.nd > 1 ? g1 : 0);
    const int k = (int)(t / ((long long)sx * sy)) - (L.nd > 2 ? g1 : 0);
    const long long c = L.at(i, j, k);
#pragma unroll
    for (int v = 0; v < NV; ++v) aos[t * NV + v] = U[(long long)v * L.plane + c];
}

}  // namespace

struct ts_handle {
    ts_config cfg{};
    std::vector<ts_block_node> blocks[3];
    std::vector<uint8_t> marks[6];  // copies of the per-face BC markers
    Layout L{};
    Phys ph{};
    HostGrid grid;
    int device = 0;
    cudaStream_t stream = nullptr;
    std::vector<void*> allocations;
    PlainBufs pb{};
    MixedBufs mb{};
    Ctl* ctl_d = nullptr;
    Ctl* ctl_h = nullptr;     // pinned mirror
    double* stage_d = nullptr;  // device AoS staging
    size_t stage_doubles = 0;
    std::map<int, cudaGraphExec_t> graphs;
    bool state_set = false;

    ~ts_handle() {
        DeviceGuard g(device);
        for (auto& kv : graphs) cudaGraphExecDestroy(kv.second);
        for (void* p : allocations) cudaFree(p);
        if (ctl_h) cudaFreeHost(ctl_h);
        if (stream) cudaStreamDestroy(stream);
    }

    template <class T>
    ts_status alloc(T** p, size_t count) {
        void* q = nullptr;
        cudaError_t e = cudaMalloc(&q, count * sizeof(T) + 256);
        if (e != cudaSuccess)
            return fail(TS_ERR_NO_MEMORY, std::string("device allocation failed: ") + cudaGetErrorString(e));
        allocations.push_back(q);
        *p = static_cast<T*>(q);
        return TS_OK;
    }

    ts_status upload_axis(int a, const double** cx, const double** chh) {
        // Device per-axis arrays with GHOST ghosts; the reference defines one
        // ghost cell per side, the outer layer continues its spacing.
        const std::vector<double>& X = a == 0 ? grid.x : (a == 1 ? grid.y : grid.z);
        const std::vector<double>& H = a == 0 ? grid.hx : (a == 1 ? grid.hy : grid.hz);
        const int n = L.n(a);
        const int g = a == 0 ? L.gx : (a == 1 ? L.gy : L.gz);
        std::vector<double> x(n + 2 * g), h(n + 2 * g);
        if (g == 0) {
            x[0] = X[0];
            h[0] = H[0];
        } else {
            for (int i = -1; i <= n; ++i) { x[i + g] = X[i + 1]; h[i + g] = H[i + 1]; }
            for (int l = 2; l <= g; ++l) {
                h[g - l] = h[g - l + 1];
                x[g - l] = x[g - l + 1] - h[g - l];
                h[n - 1 + l + g] = h[n - 2 + l + g];
                x[n - 1 + l + g] = x[n - 2 + l + g] + h[n - 1 + l + g];
            }
        }
        double *dx, *dh;
        ts_status s = alloc(&dx, x.size());
        if (s != TS_OK) return s;
        s = alloc(&dh, h.size());
        if (s != TS_OK) return s;
        // on the handle's stream (pageable sources are staged before return)
        TS_CUDA(cudaMemcpyAsync(dx, x.data(), x.size() * sizeof(double), cudaMemcpyHostToDevice, stream));
        TS_CUDA(cudaMemcpyAsync(dh, h.data(), h.size() * sizeof(double), cudaMemcpyHostToDevice, stream));
        *cx = dx;
        *chh = dh;
        return TS_OK;
    }

    ts_status init_plain() {
        const int nd = L.nd;
        const bool linear = cfg.reconstruction != TS_RECON_PIECEWISE_CONSTANT;
        const bool limited = cfg.reconstruction == TS_RECON_LINEAR_2POINTS_LIMITED;
        ts_status s;
        pb.L = L;
        if ((s = alloc(&pb.U, NV * L.plane)) != TS_OK) return s;
        TS_CUDA(cudaMemsetAsync(pb.U, 0, NV * L.plane * sizeof(double), stream));
        if (linear && (s = alloc(&pb.G, (size_t)nd * NV * L.plane)) != TS_OK) return s;
        if (limited && (s = alloc(&pb.Lim, NV * L.plane)) != TS_OK) return s;
        for (int a = 0; a < nd; ++a) {
            if ((s = alloc(&pb.F[a], NV * L.plane)) != TS_OK) return s;
            if ((s = alloc(&pb.Lam[a], L.plane)) != TS_OK) return s;
        }
        for (int a = 0; a < 3; ++a)
            if ((s = upload_axis(a, &pb.cx[a], &pb.ch[a])) != TS_OK) return s;
        if (limited && cfg.limiter == TS_LIM_VENKATAKRISHNAN) {
            // limVenkatar::SendCellInfo (Limiters.h:93-96) on the host, with the
            // same libm pow as the reference; one value per distinct cell shape.
            std::vector<double> e(L.plane, 0.0);
            std::map<std::tuple<double, double, double>, double> memo;
            for (int k = 0; k < L.nz; ++k)
                for (int j = 0; j < L.ny; ++j)
                    for (int i = 0; i < L.nx; ++i) {
                        const double hx = grid.hx[i + 1];
                        const double hy = nd > 1 ? grid.hy[j + 1] : grid.hy[0];
                        const double hz = nd > 2 ? grid.hz[k + 1] : grid.hz[0];
                        auto key = std::make_tuple(hx, hy, hz);
                        auto it = memo.find(key);
                        if (it == memo.end()) {
                            const double dx = std::pow(hx * hy * hz, 1.0 / nd);
                            it = memo.emplace(key, std::pow(5.0 * dx, 3.0)).first;
                        }
                        e[L.at(i, j, k)] = it->second;
                    }
            double* d;
            if ((s = alloc(&d, L.plane)) != TS_OK) return s;
            TS_CUDA(cudaMemcpyAsync(d, e.data(), L.plane * sizeof(double), cudaMemcpyHostToDevice, stream));
            pb.eps2 = d;
        }
        if ((s = alloc(&pb.partial, (size_t)plain_partial_blocks(L))) != TS_OK) return s;
        if (cfg.viscous) {
            if ((s = alloc(&pb.VG, (size_t)9 * L.plane)) != TS_OK) return s;
            TS_CUDA(cudaMemsetAsync(pb.VG, 0, (size_t)9 * L.plane * sizeof(double), stream));
        }
        if (cfg.viscosity != 0.0)
            for (int a = 0; a < nd; ++a)
                if ((s = alloc(&pb.VSR[a], L.plane)) != TS_OK) return s;
        pb.ctl = ctl_d;
        return TS_OK;
    }

    // Current state planes; for the mixed path the caller has pulled ctl.
    double* state_planes() { return cfg.precision == TS_PRECISION_MIXED ? mixed_state(mb, ctl_h->parity) : pb.U; }

    void enqueue_step() {
        if (cfg.precision == TS_PRECISION_MIXED) mixed_step(mb, ph, stream);
        else plain_step(pb, ph, stream);
    }

    ts_status graph_for(int k, cudaGraphExec_t* out) {
        auto it = graphs.find(k);
        if (it != graphs.end()) { *out = it->second; return TS_OK; }
        cudaGraph_t gph;
        TS_CUDA(cudaStreamBeginCapture(stream, cudaStreamCaptureModeThreadLocal));
        for (int s = 0; s < k; ++s) enqueue_step();
        cudaError_t le = cudaGetLastError();
        cudaError_t ee = cudaStreamEndCapture(stream, &gph);
        if (le != cudaSuccess) return fail(TS_ERR_CUDA, std::string("launch during capture: ") + cudaGetErrorString(le));
        if (ee != cudaSuccess) return fail(TS_ERR_CUDA, std::string("cudaStreamEndCapture: ") + cudaGetErrorString(ee));
        cudaGraphExec_t ex;
        cudaError_t ie = cudaGraphInstantiate(&ex, gph, 0);
        cudaGraphDestroy(gph);
        if (ie != cudaSuccess) return fail(TS_ERR_CUDA, std::string("cudaGraphInstantiate: ") + cudaGetErrorString(ie));
        graphs[k] = ex;
        *out = ex;
        return TS_OK;
    }

    ts_status launch_steps(int n) {
        static const int chunks[3] = {64, 8, 1};
        for (int c : chunks) {
            while (n >= c) {
                cudaGraphExec_t ex;
                ts_status s = graph_for(c, &ex);
                if (s != TS_OK) return s;
                TS_CUDA(cudaGraphLaunch(ex, stream));
                n -= c;
            }
        }
        return TS_OK;
    }

    ts_status push_ctl() {
        TS_CUDA(cudaMemcpyAsync(ctl_d, ctl_h, sizeof(Ctl), cudaMemcpyHostToDevice, stream));
        return TS_OK;
    }
    ts_status pull_ctl() {
        TS_CUDA(cudaMemcpyAsync(ctl_h, ctl_d, sizeof(Ctl), cudaMemcpyDeviceToHost, stream));
        TS_CUDA(cudaStreamSynchronize(stream));
        return TS_OK;
    }

    void fill_info(ts_step_info* info) const {
        if (!info) return;
        info->iteration = ctl_h->iteration;
        info->health = ctl_h->health;
        info->time = ctl_h->time;
        info->dt = ctl_h->dt;
        info->next_solution_time = ctl_h->next_sol;
        info->next_slice_time = ctl_h->next_slice;
        for (int v = 0; v < NV; ++v) info->residual[v] = ctl_h->res[v];
    }

    ts_status ensure_stage(size_t doubles) {
        if (stage_doubles >= doubles) return TS_OK;
        ts_status s = alloc(&stage_d, doubles);
        if (s != TS_OK) return s;
        stage_doubles = doubles;
        return TS_OK;
    }
};

namespace ts {
const ts_config& handle_config(const ts_handle* h) { return h->cfg; }
}  // namespace ts

extern "C" {

ts_status ts_create(const ts_config* cfg, ts_handle** out) {
    if (!cfg || !out) return fail(TS_ERR_INVALID, "NULL argument");
    *out = nullptr;
    std::unique_ptr<ts_handle> h(new ts_handle());
    h->cfg = *cfg;
    for (int sd = 0; sd < 6; ++sd) h->cfg.bc_marker[sd] = nullptr;  // copied once the sizes are checked
    for (int a = 0; a < 3; ++a) {
        if (cfg->n_blocks[a] > 0 && cfg->blocks[a]) {
            h->blocks[a].assign(cfg->blocks[a], cfg->blocks[a] + cfg->n_blocks[a]);
            h->cfg.blocks[a] = h->blocks[a].data();
        } else {
            h->cfg.n_blocks[a] = 0;
            h->cfg.blocks[a] = nullptr;
        }
    }
    std::string err;
    ts_status s = build_grid(h->cfg, h->grid, err);
    if (s != TS_OK) return fail(s, err);
    for (int sd = 0; sd < 6; ++sd) {
        if (!cfg->bc_marker[sd]) continue;
        if (sd >= 2 * h->cfg.n_dims || h->cfg.periodic[sd / 2])
            return fail(TS_ERR_INVALID, "bc_marker on a periodic or inactive side");
        h->marks[sd].assign(cfg->bc_marker[sd], cfg->bc_marker[sd] + side_faces(h->cfg, sd));
        h->cfg.bc_marker[sd] = h->marks[sd].data();
    }
    if ((s = validate_config(h->cfg, err)) != TS_OK) return fail(s, err);
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0)
        return fail(TS_ERR_CUDA, "no CUDA device available");
    if (cfg->device < 0 || cfg->device >= ndev) return fail(TS_ERR_INVALID, "device ordinal out of range");
    h->device = cfg->device;
    DeviceGuard g(h->device);
    h->L = make_layout(h->cfg);
    h->ph = make_phys(h->cfg);
    TS_CUDA(cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking));
    // per-face BC markers on the device (read by the ghost, face and
    // conversion code of both paths)
    for (int sd = 0; sd < 6; ++sd) {
        if (h->marks[sd].empty()) continue;
        uint8_t* dm = nullptr;
        if ((s = h->alloc(&dm, h->marks[sd].size())) != TS_OK) return s;
        TS_CUDA(cudaMemcpyAsync(dm, h->marks[sd].data(), h->marks[sd].size(), cudaMemcpyHostToDevice, h->stream));
        h->ph.bc.mark[sd] = dm;
    }
    TS_CUDA(cudaMallocHost(&h->ctl_h, sizeof(Ctl)));
    std::memset(h->ctl_h, 0, sizeof(Ctl));
    Ctl& c = *h->ctl_h;
    c.next_sol = cfg->save_solution_time;   // Kernel::Init, kernel.h:259-263
    c.next_slice = cfg->save_slice_time;
    c.max_iteration = cfg->max_iteration;
    c.max_time = cfg->max_time;
    c.save_sol = cfg->save_solution_time;
    c.save_slice = cfg->save_slice_time;
    if ((s = h->alloc(&h->ctl_d, 1)) != TS_OK) return s;
    if ((s = h->push_ctl()) != TS_OK) return s;
    if (cfg->precision == TS_PRECISION_MIXED) {
        s = mixed_init(h->cfg, h->L, h->ph, h->grid, h->ctl_d,
                       [&](size_t bytes, void** p) { return h->alloc(reinterpret_cast<char**>(p), bytes); },
                       h->mb, err, h->stream);
        if (s != TS_OK) return fail(s, err.empty() ? std::string(ts_last_error()) : err);
    } else {
        if ((s = h->init_plain()) != TS_OK) return s;
    }
    TS_CUDA(cudaStreamSynchronize(h->stream));
    *out = h.release();
    return TS_OK;
}

void ts_destroy(ts_handle* h) {
    if (!h) return;
    io_join_all(h, nullptr, nullptr);
    delete h;
}

static ts_status set_state_impl(ts_handle* h, const double* values, int32_t layout, bool device_ptr) {
    if (!h || !values) return fail(TS_ERR_INVALID, "NULL argument");
    if (layout != TS_LAYOUT_INTERIOR && layout != TS_LAYOUT_WITH_GHOSTS) return fail(TS_ERR_INVALID, "bad layout");
    DeviceGuard g(h->device);
    const size_t nd = ts_state_doubles(&h->cfg, layout);
    const long long ncell = (long long)(nd / NV);
    const double* src = values;
    ts_status s;
    if (h->cfg.precision == TS_PRECISION_MIXED) {
        // a fresh state has no pending residual and lives in buffer 0
        if ((s = h->pull_ctl()) != TS_OK) return s;
        h->ctl_h->parity = 0;
        h->ctl_h->dt_apply = 0.0;
        if ((s = h->push_ctl()) != TS_OK) return s;
    }
    if (!device_ptr) {
        if (const void* pd = pinned_device_ptr(values, h->device)) {
            src = static_cast<const double*>(pd);  // page-locked: read in place
        } else {
            if ((s = h->ensure_stage(nd)) != TS_OK) return s;
            TS_CUDA(cudaMemcpyAsync(h->stage_d, values, nd * sizeof(double), cudaMemcpyHostToDevice, h->stream));
            src = h->stage_d;
        }
    }
    const int blk = 256;
    k_scatter<<<(unsigned)((ncell + blk - 1) / blk), blk, 0, h->stream>>>(src, h->L, h->state_planes(),
                                                                           layout == TS_LAYOUT_WITH_GHOSTS, ncell);
    TS_CUDA(cudaGetLastError());
    if (h->cfg.precision == TS_PRECISION_MIXED) mixed_reset(h->mb, h->stream);
    TS_CUDA(cudaStreamSynchronize(h->stream));
    h->state_set = true;
    return TS_OK;
}

ts_status ts_set_state(ts_handle* h, const double* values, int32_t layout) {
    return set_state_impl(h, values, layout, false);
}

ts_status ts_set_state_device(ts_handle* h, const double* values, int32_t layout) {
    return set_state_impl(h, values, layout, true);
}

static ts_status get_state_impl(ts_handle* h, double* values, int32_t layout, bool device_ptr) {
    if (!h || !values) return fail(TS_ERR_INVALID, "NULL argument");
    if (layout != TS_LAYOUT_INTERIOR && layout != TS_LAYOUT_WITH_GHOSTS) return fail(TS_ERR_INVALID, "bad layout");
    DeviceGuard g(h->device);
    const size_t nd = ts_state_doubles(&h->cfg, layout);
    const long long ncell = (long long)(nd / NV);
    ts_status s;
    // page-locked host memory is written in place, like device memory
    double* pinned = device_ptr ? nullptr : static_cast<double*>(pinned_device_ptr(values, h->device));
    const bool staged = !device_ptr && !pinned;
    if (staged && (s = h->ensure_stage(nd)) != TS_OK) return s;
    if (h->cfg.precision == TS_PRECISION_MIXED) {
        if ((s = h->pull_ctl()) != TS_OK) return s;
        mixed_materialize(h->mb, h->ph, h->stream);
        h->ctl_h->dt_apply = 0.0;  // the device copy is cleared by the apply pass
    }
    double* dst = device_ptr ? values : (pinned ? pinned : h->stage_d);
    const int blk = 256;
    k_gather<<<(unsigned)((ncell + blk - 1) / blk), blk, 0, h->stream>>>(dst, h->L, h->state_planes(),
                                                                          layout == TS_LAYOUT_WITH_GHOSTS, ncell);
    TS_CUDA(cudaGetLastError());
    if (staged)
        TS_CUDA(cudaMemcpyAsync(values, h->stage_d, nd * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
    TS_CUDA(cudaStreamSynchronize(h->stream));
    return TS_OK;
}

ts_status ts_get_state(ts_handle* h, double* values, int32_t layout) {
    return get_state_impl(h, values, layout, false);
}

ts_status ts_get_state_device(ts_handle* h, double* values, int32_t layout) {
    return get_state_impl(h, values, layout, true);
}

ts_status ts_step(ts_handle* h, int32_t n_steps, ts_step_info* info) {
    if (!h) return fail(TS_ERR_INVALID, "NULL handle");
    if (n_steps < 0) return fail(TS_ERR_INVALID, "n_steps must be >= 0");
    if (!h->state_set) return fail(TS_ERR_INVALID, "state not set");
    DeviceGuard g(h->device);
    ts_status s;
    h->ctl_h->stop_req = 0;
    h->ctl_h->run_mode = 0;
    h->ctl_h->health = 0;
    if ((s = h->push_ctl()) != TS_OK) return s;
    if ((s = h->launch_steps(n_steps)) != TS_OK) return s;
    if ((s = h->pull_ctl()) != TS_OK) return s;
    h->fill_info(info);
    return TS_OK;
}

ts_status ts_step_timed(ts_handle* h, int32_t n_steps, ts_step_info* info, ts_timing* timing) {
    if (!h || !timing) return fail(TS_ERR_INVALID, "NULL argument");
    if (n_steps <= 0) return fail(TS_ERR_INVALID, "n_steps must be > 0");
    if (!h->state_set) return fail(TS_ERR_INVALID, "state not set");
    DeviceGuard g(h->device);
    ts_status s;
    h->ctl_h->stop_req = 0;
    h->ctl_h->run_mode = 0;
    h->ctl_h->health = 0;
    if ((s = h->push_ctl()) != TS_OK) return s;
    const bool mixed = h->cfg.precision == TS_PRECISION_MIXED;
    const int per = (mixed ? kMixedMaxLaunches : kPlainMaxLaunches) + 1;
    // per-launch events on at most kTimedSamples evenly spaced steps: an
    // event pair around every launch of every step slows short stages
    // (measured: 7-9 % on the 67 us stages of a 1024^2 2D problem)
    constexpr int kTimedSamples = 64;
    const int stride = std::max(1, n_steps / kTimedSamples);
    const int samples = (n_steps + stride - 1) / stride;
    std::vector<cudaEvent_t> ev((size_t)samples * per + 2, nullptr);
    for (auto& e : ev) TS_CUDA(cudaEventCreate(&e));
    struct Cleanup {
        std::vector<cudaEvent_t>& ev;
        ~Cleanup() { for (auto& e : ev) if (e) cudaEventDestroy(e); }
    } cleanup{ev};
    static_assert(kPlainMaxLaunches <= TS_MAX_KERNELS && kMixedMaxLaunches <= TS_MAX_KERNELS,
                  "every launch of a step has a kernel slot");
    const char* names[TS_MAX_KERNELS] = {};
    int nl = 0;
    TS_CUDA(cudaEventRecord(ev[0], h->stream));
    for (int st = 0; st < n_steps; ++st) {
        cudaEvent_t* e = st % stride ? nullptr : ev.data() + 1 + (size_t)(st / stride) * per;
        if (mixed) mixed_step(h->mb, h->ph, h->stream, e, &nl, names);
        else plain_step(h->pb, h->ph, h->stream, e, &nl, names);
    }
    TS_CUDA(cudaGetLastError());
    TS_CUDA(cudaEventRecord(ev.back(), h->stream));
    if ((s = h->pull_ctl()) != TS_OK) return s;
    TS_CUDA(cudaEventSynchronize(ev.back()));
    std::memset(timing, 0, sizeof(*timing));
    float ms = 0.f;
    TS_CUDA(cudaEventElapsedTime(&ms, ev[0], ev.back()));
    timing->total_ms = ms;
    timing->n_kernels = nl;
    timing->launches = nl * n_steps;
    for (int k = 0; k < nl && k < TS_MAX_KERNELS; ++k) {
        double acc = 0.0;
        for (int q = 0; q < samples; ++q) {
            cudaEvent_t* e = ev.data() + 1 + (size_t)q * per;
            TS_CUDA(cudaEventElapsedTime(&ms, e[k], e[k + 1]));
            acc += ms;
        }
        timing->kernel_ms[k] = acc / samples;
        std::strncpy(timing->kernel_name[k], names[k] ? names[k] : "?", 31);
    }
    h->fill_info(info);
    return TS_OK;
}

ts_status ts_run(ts_handle* h, ts_step_info* info) {
    if (!h) return fail(TS_ERR_INVALID, "NULL handle");
    if (!h->state_set) return fail(TS_ERR_INVALID, "state not set");
    DeviceGuard g(h->device);
    ts_status s;
    h->ctl_h->stop_req = 0;
    h->ctl_h->run_mode = 1;
    h->ctl_h->health = 0;
    if ((s = h->push_ctl()) != TS_OK) return s;
    // Steps past termination are no-ops on the device (stop_req), so chunks
    // may overshoot; the chunk grows while the run continues.
    int chunk = 8;
    for (;;) {
        if ((s = h->launch_steps(chunk)) != TS_OK) return s;
        if ((s = h->pull_ctl()) != TS_OK) return s;
        if (h->ctl_h->stop_req) break;
        if (chunk < 512) chunk *= 2;
    }
    h->fill_info(info);
    return TS_OK;
}

ts_status ts_get_step_info(ts_handle* h, ts_step_info* info) {
    if (!h || !info) return fail(TS_ERR_INVALID, "NULL argument");
    DeviceGuard g(h->device);
    ts_status s = h->pull_ctl();
    if (s != TS_OK) return s;
    h->fill_info(info);
    return TS_OK;
}

ts_status ts_set_step_info(ts_handle* h, const ts_step_info* info) {
    if (!h || !info) return fail(TS_ERR_INVALID, "NULL argument");
    DeviceGuard g(h->device);
    ts_status s = h->pull_ctl();
    if (s != TS_OK) return s;
    h->ctl_h->iteration = info->iteration;
    h->ctl_h->time = info->time;
    h->ctl_h->dt = info->dt;
    h->ctl_h->next_sol = info->next_solution_time;
    h->ctl_h->next_slice = info->next_slice_time;
    return h->push_ctl();
}

ts_status ts_set_tile(ts_handle* h, int32_t tx, int32_t ty, int32_t z_chunks) {
    if (!h) return fail(TS_ERR_INVALID, "NULL handle");
    if (h->cfg.precision != TS_PRECISION_MIXED) return fail(TS_ERR_UNSUPPORTED, "tiles apply to the mixed path");
    DeviceGuard g(h->device);
    TS_CUDA(cudaStreamSynchronize(h->stream));
    std::string err;
    ts_status s = mixed_set_tile(h->mb, tx, ty, z_chunks, err, h->stream);
    if (s != TS_OK) return fail(s, err);
    for (auto& kv : h->graphs) cudaGraphExecDestroy(kv.second);  // launch shape changed
    h->graphs.clear();
    return TS_OK;
}

ts_status ts_synchronize(ts_handle* h) {
    if (!h) return fail(TS_ERR_INVALID, "NULL handle");
    DeviceGuard g(h->device);
    TS_CUDA(cudaStreamSynchronize(h->stream));
    return TS_OK;
}

}  // extern "C"
