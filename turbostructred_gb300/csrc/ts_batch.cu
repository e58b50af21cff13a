// Batches of independent 1D/2D problems advanced by the fused mixed-precision
// kernel (include/ts_fvm.h, ts_batch_*).
//
// Memory: one device arena (the batch's budget) with a first-fit free list
// kept on the host; each problem takes its two FP64 state buffers, two FP32
// residual buffers and its per-axis geometry from it.  A slot table holds
// every problem's descriptor and control word in device memory.
//
// A stage is one launch of the batched kernel per Riemann solver present,
// over a work list of (slot, tile item) pairs sorted by problem size,
// largest first.  Finished problems' items skip themselves on the device;
// the list is rebuilt when membership changes or when most of it is idle.
// Chunks of stages are captured once into a CUDA graph and replayed while the
// list is unchanged (the list and descriptors live in device buffers, so
// replays see updated control words).
#include <cuda_runtime.h>

#include <algorithm>
#include <array>
#include <cmath>
#include <cstring>
#include <map>
#include <memory>
#include <string>
#include <vector>

#include "ts_mixed.h"

namespace ts {
namespace {

#define TB_CUDA(call)                                                                                   \
    do {                                                                                                \
        cudaError_t e_ = (call);                                                                        \
        if (e_ != cudaSuccess)                                                                          \
            return fail(e_ == cudaErrorMemoryAllocation ? TS_ERR_NO_MEMORY : TS_ERR_CUDA,               \
                        std::string(#call) + ": " + cudaGetErrorString(e_));                            \
    } while (0)

constexpr size_t kAlign = 256;

// First-fit allocator over one device allocation; bookkeeping on the host.
class Arena {
public:
    char* base = nullptr;
    size_t size = 0, used = 0, high = 0;
    std::map<size_t, size_t> free_;  // offset -> bytes
    std::map<size_t, size_t> taken_;

    cudaError_t init(size_t bytes) {
        size = (bytes + kAlign - 1) & ~(kAlign - 1);
        cudaError_t e = cudaMalloc(&base, size);
        if (e == cudaSuccess) free_[0] = size;
        return e;
    }
    ~Arena() { if (base) cudaFree(base); }
    void* take(size_t bytes) {
        bytes = (bytes + kAlign - 1) & ~(kAlign - 1);
        for (auto it = free_.begin(); it != free_.end(); ++it) {
            if (it->second < bytes) continue;
            const size_t off = it->first, len = it->second;
            free_.erase(it);
            if (len > bytes) free_[off + bytes] = len - bytes;
            taken_[off] = bytes;
            used += bytes;
            high = std::max(high, off + bytes);
            return base + off;
        }
        return nullptr;
    }
    void give(void* p) {
        const size_t off = (size_t)((char*)p - base);
        auto t = taken_.find(off);
        if (t == taken_.end()) return;
        size_t o = off, len = t->second;
        used -= len;
        taken_.erase(t);
        auto nx = free_.lower_bound(o);
        if (nx != free_.end() && nx->first == o + len) { len += nx->second; free_.erase(nx); }
        auto pv = free_.lower_bound(o);
        if (pv != free_.begin()) {
            --pv;
            if (pv->first + pv->second == o) { o = pv->first; len += pv->second; free_.erase(pv); }
        }
        free_[o] = len;
    }
};

__global__ void k_b_scatter(const double* __restrict__ aos, Layout L, double* __restrict__ U) {
    const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (t >= L.cells()) return;
    const int i = (int)(t % L.nx), j = (int)((t / L.nx) % L.ny), k = (int)(t / ((long long)L.nx * L.ny));
    const long long c = L.at(i, j, k);
#pragma unroll
    for (int v = 0; v < NV; ++v) U[(long long)v * L.plane + c] = aos[t * NV + v];
}

// Interior cells of problem p's current state to AoS order.
__global__ void k_b_gather(double* __restrict__ aos, const ProbDesc* __restrict__ probs, int p) {
    const ProbDesc& d = probs[p];
    const Layout& L = d.L;
    const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (t >= L.cells()) return;
    const int i = (int)(t % L.nx), j = (int)((t / L.nx) % L.ny), k = (int)(t / ((long long)L.nx * L.ny));
    const double* U = d.U[d.ctl->parity];
#pragma unroll
    for (int v = 0; v < NV; ++v) aos[t * NV + v] = U[(long long)v * L.plane + L.at(i, j, k)];
}

struct Slot {
    bool used = false;
    int id = -1;
    bool collected = false;   // reported by ts_batch_finished
    long long cells = 0;
    int tx = 0, ty = 0;       // tile of this problem
    std::vector<void*> mem;
    ts_config cfg;
};

struct Group {
    int nd = 0, solver = 0, tx = 0, ty = 0;
    int2* d_items = nullptr;
    int cap = 0, n = 0;
    int grid = 0;
};

// Launch policy of one dimension: a fixed tile or (tx = 0) a tile chosen per
// problem from its x extent; ctas = resident CTAs per SM (0: as many as fit).
struct Tune {
    int tx, ty, ctas;
};

// One-row tiles compiled for batched problems (threads along x).
const int kTiles1D[3] = {512, 256, 128};
const int kTiles2D[3] = {260, 132, 68};
constexpr int kRowsPerItem = 64;  // marching-axis rows per work item of a 2D problem
// Work lists of at most this many items close each problem's step inside the
// stage kernel; longer lists use the separate finish kernel.
constexpr long long kFusedCloseItems = 1024;

// The one-row tile of a problem with nx cells per row.  1D: the tile that
// covers the row with the fewest warp-slots per cell, charging each column
// ~4 warps of fixed cost (setup, barriers, close).
int pick_tile(int nd, int nx) {
    // 2D: the 132-thread tile (128 cells, five resident CTAs per SM) measured
    // fastest on mixed-size batches of 256^2-1024^2 problems (autotuner: 1.94e10
    // against 1.75e10 cell-updates/s for the 260-thread tile); the 68-thread
    // tile for rows that fit it
    if (nd == 2) return nx <= 64 ? 68 : 132;
    const int* c = kTiles1D;
    int best = c[0];
    double best_cost = 1e300;
    for (int k = 0; k < 3; ++k) {
        int cx, cy;
        mixed_tile_cells(nd, c[k], 1, &cx, &cy);
        const double cols = std::ceil((double)nx / cx);
        const double cost = cols * ((c[k] + 31) / 32 + 4) / (double)nx;
        if (cost < best_cost - 1e-12) { best_cost = cost; best = c[k]; }
    }
    return best;
}

}  // namespace
}  // namespace ts

using namespace ts;

struct ts_batch {
    int device = 0, sms = 0;
    cudaStream_t stream = nullptr;
    // groups beyond the first run concurrently on side streams (forked and
    // joined inside the captured stage graph)
    static constexpr int kSide = 4;
    cudaStream_t side[kSide] = {};
    cudaEvent_t fork = nullptr, join[kSide] = {};
    int* d_slots = nullptr;   // listed problems (closed by the finish kernel)
    int slots_cap = 0, n_listed = 0;
    // short work lists close each problem's step in the stage kernel itself
    // (the CTA finishing a problem's last item), saving the finish launch
    bool fused_close = false;
    // the last few long 1D problems run in the cluster tail kernel: many
    // stages per launch, state on chip (one list per Riemann solver)
    bool tail_enabled = true, tail_mode = false;
    int tail_cluster = 0;
    int* d_tail[2] = {nullptr, nullptr};
    int tail_n[2] = {0, 0}, tail_cap[2] = {0, 0};
    Arena arena;
    std::vector<Slot> slots;
    std::vector<ProbDesc> desc;
    ProbDesc* d_desc = nullptr;
    Ctl* d_ctl = nullptr;
    Ctl* h_ctl = nullptr;  // pinned mirror
    int capacity = 0;
    std::map<int, int> id2slot;
    int next_id = 0;
    std::vector<Group> groups;
    bool dirty = true;
    int stable = 0;  // launches since the work list last changed
    std::map<int, cudaGraphExec_t> graphs;
    Tune tune[4] = {{0, 0, 0}, {0, 1, 0}, {0, 1, 0}, {0, 0, 0}};
    // uploads of admitted problems and read-backs of finished ones run on
    // their own streams (with their own staging buffers), so they overlap
    // stages queued on the main stream
    cudaStream_t ustream = nullptr, dstream = nullptr;
    cudaEvent_t uploaded = nullptr;
    double* ustage = nullptr;
    size_t ustage_doubles = 0;
    double* dstage = nullptr;
    size_t dstage_doubles = 0;
    std::vector<int> quarantine;  // removed slots, reusable once the main stream has drained
    double done_cell_updates = 0.0;  // of removed problems
    long long stages = 0, launches = 0;

    ~ts_batch() {
        int prev = -1;
        cudaGetDevice(&prev);
        cudaSetDevice(device);
        drop_graphs();
        for (auto& g : groups) cudaFree(g.d_items);
        cudaFree(d_slots);
        cudaFree(d_tail[0]);
        cudaFree(d_tail[1]);
        for (int k = 0; k < kSide; ++k) {
            if (side[k]) cudaStreamDestroy(side[k]);
            if (join[k]) cudaEventDestroy(join[k]);
        }
        if (fork) cudaEventDestroy(fork);
        cudaFree(d_desc);
        cudaFree(d_ctl);
        cudaFreeHost(h_ctl);
        cudaFree(ustage);
        cudaFree(dstage);
        if (ustream) cudaStreamDestroy(ustream);
        if (dstream) cudaStreamDestroy(dstream);
        if (uploaded) cudaEventDestroy(uploaded);
        if (stream) cudaStreamDestroy(stream);
        if (prev >= 0) cudaSetDevice(prev);
    }

    void drop_graphs() {
        for (auto& kv : graphs) cudaGraphExecDestroy(kv.second);
        graphs.clear();
    }

    ts_status grow(int need) {
        if (need <= capacity) return TS_OK;
        int cap = std::max(64, capacity);
        while (cap < need) cap *= 2;
        ProbDesc* nd_ = nullptr;
        Ctl* nc = nullptr;
        Ctl* nh = nullptr;
        TB_CUDA(cudaMalloc(&nd_, sizeof(ProbDesc) * cap));
        TB_CUDA(cudaMalloc(&nc, sizeof(Ctl) * cap));
        TB_CUDA(cudaMallocHost(&nh, sizeof(Ctl) * cap));
        std::memset(nh, 0, sizeof(Ctl) * cap);
        TB_CUDA(cudaStreamSynchronize(stream));
        if (capacity) {
            TB_CUDA(cudaMemcpyAsync(nc, d_ctl, sizeof(Ctl) * capacity, cudaMemcpyDeviceToDevice, stream));
            std::memcpy(nh, h_ctl, sizeof(Ctl) * capacity);
            // the old control words are freed below: the copy out of them first
            TB_CUDA(cudaStreamSynchronize(stream));
        }
        cudaFree(d_desc);
        cudaFree(d_ctl);
        cudaFreeHost(h_ctl);
        d_desc = nd_;
        d_ctl = nc;
        h_ctl = nh;
        capacity = cap;
        slots.resize(cap);
        desc.resize(cap);
        // control-word pointers moved: re-point every descriptor
        for (int s = 0; s < cap; ++s) {
            if (!slots[s].used) continue;
            desc[s].ctl = d_ctl + s;
        }
        TB_CUDA(cudaMemcpyAsync(d_desc, desc.data(), sizeof(ProbDesc) * cap, cudaMemcpyHostToDevice, stream));
        dirty = true;
        return TS_OK;
    }

    int per_sm(const Group& g) const {
        size_t b;
        int n = 0;
        mixed_tile_info(g.nd, g.tx, g.ty, g.solver, &b, &n, true);
        if (tune[g.nd].ctas > 0) n = std::min(n, tune[g.nd].ctas);
        return std::max(n, 0);
    }

    // Tile of a problem under the current policy, and its work items.
    void place(int s) {
        ProbDesc& d = desc[s];
        const int nd = d.L.nd;
        slots[s].tx = tune[nd].tx > 0 ? tune[nd].tx : pick_tile(nd, d.kn[0]);
        slots[s].ty = 1;
        const int chunks = nd >= 2 ? std::max(1, d.kn[2] / kRowsPerItem) : 1;
        mixed_items(d, slots[s].tx, 1, chunks, (long long)sms);
    }

    // Work items of unfinished problems, grouped by (nd, solver), each group
    // sorted by problem size, largest first.
    ts_status rebuild() {
        std::map<std::array<int, 4>, std::vector<int>> bykey;
        for (int s = 0; s < capacity; ++s) {
            if (!slots[s].used || h_ctl[s].stop_req) continue;
            bykey[{desc[s].L.nd, desc[s].mp.solver, slots[s].tx, slots[s].ty}].push_back(s);
        }
        std::vector<Group> ng;
        for (auto& kv : bykey) {
            Group g;
            g.nd = kv.first[0];
            g.solver = kv.first[1];
            g.tx = kv.first[2];
            g.ty = kv.first[3];
            auto& v = kv.second;
            std::stable_sort(v.begin(), v.end(), [&](int a, int b2) { return slots[a].cells > slots[b2].cells; });
            std::vector<int2> items;
            for (int s : v)
                for (int q = 0; q < desc[s].nq; ++q) items.push_back(make_int2(s, q));
            g.n = (int)items.size();
            // reuse an old buffer of the same key when large enough
            for (auto& og : groups)
                if (og.d_items && og.cap >= g.n) {
                    g.d_items = og.d_items; g.cap = og.cap; og.d_items = nullptr;
                    break;
                }
            if (!g.d_items) {
                g.cap = std::max(1024, g.n);
                TB_CUDA(cudaMalloc(&g.d_items, sizeof(int2) * g.cap));
            }
            TB_CUDA(cudaMemcpyAsync(g.d_items, items.data(), sizeof(int2) * g.n, cudaMemcpyHostToDevice, stream));
            g.grid = std::min(g.n, std::max(1, per_sm(g)) * sms);
            ng.push_back(g);
        }
        for (auto& og : groups) cudaFree(og.d_items);
        groups.swap(ng);
        long long total = 0;
        for (auto& g : groups) total += g.n;
        fused_close = total <= kFusedCloseItems;
        ts_status ts = plan_tail();
        if (ts != TS_OK) return ts;
        // the listed problems, for the stage's finish kernel
        std::vector<int> listed;
        for (auto& kv : bykey) listed.insert(listed.end(), kv.second.begin(), kv.second.end());
        n_listed = (int)listed.size();
        if (n_listed > slots_cap) {
            cudaFree(d_slots);
            d_slots = nullptr;
            slots_cap = std::max(2 * slots_cap, std::max(n_listed, 256));
            TB_CUDA(cudaMalloc(&d_slots, sizeof(int) * slots_cap));
        }
        if (n_listed)
            TB_CUDA(cudaMemcpyAsync(d_slots, listed.data(), sizeof(int) * n_listed, cudaMemcpyHostToDevice, stream));
        TB_CUDA(cudaStreamSynchronize(stream));
        drop_graphs();
        dirty = false;
        return TS_OK;
    }

    // Tail mode when every unfinished problem is 1D, fits one cluster, and
    // all clusters together fit the GPU at once (one CTA per SM).
    ts_status plan_tail() {
        tail_mode = false;
        tail_n[0] = tail_n[1] = 0;
        if (!tail_enabled) return TS_OK;
        const int cells = mixed_tail_cells();
        std::vector<int> lists[2];
        int cmax = 0, nact = 0;
        for (int s = 0; s < capacity; ++s) {
            if (!slots[s].used || h_ctl[s].stop_req) continue;
            const ProbDesc& d = desc[s];
            const int items = (d.kn[0] + cells - 1) / cells;
            // the tail kernel forms no residual norms
            if (d.L.nd != 1 || items > kTailMaxCluster || d.mp.norms) return TS_OK;
            cmax = std::max(cmax, items);
            lists[d.mp.solver == TS_RS_HLLC ? 1 : 0].push_back(s);
            ++nact;
        }
        if (nact == 0 || (long long)nact * cmax > sms) return TS_OK;
        for (int k = 0; k < 2; ++k)
            if (!lists[k].empty() && !mixed_tail_ready(k ? TS_RS_HLLC : TS_RS_ROE_PIKE, cmax)) return TS_OK;
        for (int k = 0; k < 2; ++k) {
            tail_n[k] = (int)lists[k].size();
            if (!tail_n[k]) continue;
            if (tail_n[k] > tail_cap[k]) {
                cudaFree(d_tail[k]);
                d_tail[k] = nullptr;
                tail_cap[k] = std::max(64, tail_n[k]);
                TB_CUDA(cudaMalloc(&d_tail[k], sizeof(int) * tail_cap[k]));
            }
            TB_CUDA(cudaMemcpyAsync(d_tail[k], lists[k].data(), sizeof(int) * tail_n[k], cudaMemcpyHostToDevice,
                                    stream));
        }
        tail_cluster = cmax;
        tail_mode = true;
        return TS_OK;
    }

    // One stage: every group's launch (concurrently when there are several),
    // then the finish kernel that closes each listed problem's step.
    void enqueue_stage() {
        const int ng = (int)groups.size();
        if (ng > 1) cudaEventRecord(fork, stream);
        for (int k = 0; k < ng; ++k) {
            const Group& g = groups[k];
            cudaStream_t st = stream;
            if (k > 0) {
                st = side[(k - 1) % kSide];
                if (k - 1 < kSide) cudaStreamWaitEvent(st, fork, 0);
            }
            mixed_launch_batch(g.nd, g.tx, g.ty, g.solver, g.grid, d_desc, d_ctl, g.d_items, g.n, st, fused_close);
            ++launches;
        }
        for (int k = 0; k < std::min(ng - 1, kSide); ++k) {
            cudaEventRecord(join[k], side[k]);
            cudaStreamWaitEvent(stream, join[k], 0);
        }
        if (!fused_close) {
            mixed_batch_finish(d_desc, d_slots, n_listed, stream);
            ++launches;
        }
        ++stages;
    }

    // Stages are launched one by one right after the work list changed (a
    // capture costs more than it saves when membership keeps changing, as in
    // a served stream); once the list has been stable for a few launches,
    // chunks of stages are captured into graphs and replayed.
    ts_status launch(int n) {
        if (dirty) {
            ts_status s = rebuild();
            if (s != TS_OK) return s;
            stable = 0;
        }
        if (groups.empty()) return TS_OK;
        if (tail_mode) {
            // every tail problem advances up to n stages in one launch
            for (int k = 0; k < 2; ++k) {
                if (!tail_n[k]) continue;
                TB_CUDA(mixed_launch_tail(k ? TS_RS_HLLC : TS_RS_ROE_PIKE, tail_cluster, tail_n[k], d_desc, d_tail[k],
                                          n, stream));
                ++launches;
            }
            stages += n;
            return TS_OK;
        }
        if (stable < 2) {
            ++stable;
            for (int k = 0; k < n; ++k) enqueue_stage();
            TB_CUDA(cudaGetLastError());
            return TS_OK;
        }
        static const int chunks[3] = {32, 4, 1};
        for (int c : chunks) {
            while (n >= c) {
                auto it = graphs.find(c);
                cudaGraphExec_t ex;
                if (it == graphs.end()) {
                    cudaGraph_t gph;
                    const long long s0 = stages, l0 = launches;
                    TB_CUDA(cudaStreamBeginCapture(stream, cudaStreamCaptureModeThreadLocal));
                    for (int k = 0; k < c; ++k) enqueue_stage();
                    cudaError_t le = cudaGetLastError();
                    TB_CUDA(cudaStreamEndCapture(stream, &gph));
                    if (le != cudaSuccess) return fail(TS_ERR_CUDA, std::string("capture: ") + cudaGetErrorString(le));
                    stages = s0; launches = l0;
                    cudaError_t ie = cudaGraphInstantiate(&ex, gph, 0);
                    cudaGraphDestroy(gph);
                    if (ie != cudaSuccess) return fail(TS_ERR_CUDA, std::string("instantiate: ") + cudaGetErrorString(ie));
                    graphs[c] = ex;
                } else {
                    ex = it->second;
                }
                TB_CUDA(cudaGraphLaunch(ex, stream));
                stages += c;
                launches += (long long)c * (long long)(groups.size() + (fused_close ? 0 : 1));
                n -= c;
            }
        }
        return TS_OK;
    }

    // Control words to the host.  A problem whose state turned non-physical
    // (health flags) will not reach its end time: it is stopped here and
    // reported finished with its flags.
    ts_status pull() {
        TB_CUDA(cudaMemcpyAsync(h_ctl, d_ctl, sizeof(Ctl) * capacity, cudaMemcpyDeviceToHost, stream));
        TB_CUDA(cudaStreamSynchronize(stream));
        // the main stream has drained: removed slots can be reused
        for (int q : quarantine) slots[q].used = false;
        quarantine.clear();
        for (int s = 0; s < capacity; ++s) {
            if (!slots[s].used || h_ctl[s].stop_req || !h_ctl[s].health) continue;
            h_ctl[s].stop_req = 1;
            TB_CUDA(cudaMemcpyAsync(&d_ctl[s].stop_req, &h_ctl[s].stop_req, sizeof(int), cudaMemcpyHostToDevice,
                                    stream));
            dirty = true;
        }
        TB_CUDA(cudaStreamSynchronize(stream));
        return TS_OK;
    }

    int active(long long* items_active, long long* items_listed) const {
        int a = 0;
        long long ia = 0;
        for (int s = 0; s < capacity; ++s)
            if (slots[s].used && !h_ctl[s].stop_req) { ++a; ia += desc[s].nq; }
        long long il = 0;
        for (auto& g : groups) il += g.n;
        if (items_active) *items_active = ia;
        if (items_listed) *items_listed = il;
        return a;
    }

    double cell_updates() const {
        double c = done_cell_updates;
        for (int s = 0; s < capacity; ++s)
            if (slots[s].used) c += (double)slots[s].cells * (double)h_ctl[s].iteration;
        return c;
    }
};

namespace {

struct DevGuard {
    int prev = -1;
    explicit DevGuard(int d) { cudaGetDevice(&prev); if (prev != d) cudaSetDevice(d); }
    ~DevGuard() { int c = -1; cudaGetDevice(&c); if (prev >= 0 && c != prev) cudaSetDevice(prev); }
};

size_t problem_bytes(const Layout& L) {
    auto al = [](size_t b) { return (b + kAlign - 1) & ~(kAlign - 1); };
    size_t b = 2 * al(sizeof(double) * NV * L.plane) + 2 * al(sizeof(float) * NV * L.plane);
    b += al(sizeof(AxisGeo) * (L.nx + 2 * L.gx)) + al(sizeof(AxisGeo) * (L.ny + 2 * L.gy)) +
         al(sizeof(AxisGeo) * (L.nz + 2 * L.gz));
    return b;
}

}  // namespace

extern "C" {

ts_status ts_batch_create(int32_t device, size_t budget, ts_batch** out) {
    if (!out) return fail(TS_ERR_INVALID, "NULL argument");
    *out = nullptr;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return fail(TS_ERR_CUDA, "no CUDA device available");
    if (device < 0 || device >= ndev) return fail(TS_ERR_INVALID, "device ordinal out of range");
    if (budget < (1u << 20)) return fail(TS_ERR_INVALID, "memory budget below 1 MiB");
    std::unique_ptr<ts_batch> b(new ts_batch());
    b->device = device;
    DevGuard g(device);
    cudaDeviceGetAttribute(&b->sms, cudaDevAttrMultiProcessorCount, device);
    TB_CUDA(cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking));
    for (int k = 0; k < ts_batch::kSide; ++k) {
        TB_CUDA(cudaStreamCreateWithFlags(&b->side[k], cudaStreamNonBlocking));
        TB_CUDA(cudaEventCreateWithFlags(&b->join[k], cudaEventDisableTiming));
    }
    TB_CUDA(cudaEventCreateWithFlags(&b->fork, cudaEventDisableTiming));
    TB_CUDA(cudaStreamCreateWithFlags(&b->ustream, cudaStreamNonBlocking));
    TB_CUDA(cudaStreamCreateWithFlags(&b->dstream, cudaStreamNonBlocking));
    TB_CUDA(cudaEventCreateWithFlags(&b->uploaded, cudaEventDisableTiming));
    TB_CUDA(b->arena.init(budget));
    ts_status s = b->grow(64);
    if (s != TS_OK) return s;
    *out = b.release();
    return TS_OK;
}

void ts_batch_destroy(ts_batch* b) { delete b; }

size_t ts_batch_problem_bytes(const ts_config* cfg) {
    if (!cfg) return 0;
    std::string err;
    if (validate_config(*cfg, err) != TS_OK) return 0;
    if (cfg->n_dims > 2 || cfg->precision != TS_PRECISION_MIXED || has_markers(*cfg)) return 0;
    return problem_bytes(make_layout(*cfg));
}

ts_status ts_batch_add(ts_batch* b, const ts_config* cfg, const double* values, int32_t* id) {
    if (!b || !cfg || !values || !id) return fail(TS_ERR_INVALID, "NULL argument");
    if (cfg->precision != TS_PRECISION_MIXED) return fail(TS_ERR_UNSUPPORTED, "batches run the mixed-precision step");
    if (cfg->n_dims > 2) return fail(TS_ERR_UNSUPPORTED, "batches hold 1D and 2D problems");
    if (has_markers(*cfg)) return fail(TS_ERR_UNSUPPORTED, "batches take one boundary condition per side (no bc_marker)");
    HostGrid grid;
    std::string err;
    ts_status s = build_grid(*cfg, grid, err);
    if (s != TS_OK) return fail(s, err);
    DevGuard g(b->device);
    const Layout L = make_layout(*cfg);
    const Phys ph = make_phys(*cfg);
    if (b->arena.size - b->arena.used < problem_bytes(L))
        return fail(TS_ERR_NO_MEMORY, "batch memory budget exhausted");
    int slot = -1;
    for (int k = 0; k < b->capacity; ++k)
        if (!b->slots[k].used) { slot = k; break; }
    if (slot < 0) {
        slot = b->capacity;
        if ((s = b->grow(b->capacity + 1)) != TS_OK) return s;
    }
    Slot& sl = b->slots[slot];
    sl = Slot();
    auto take = [&](size_t bytes, void** p) -> ts_status {
        *p = b->arena.take(bytes);
        if (!*p) return fail(TS_ERR_NO_MEMORY, "batch memory budget exhausted");
        sl.mem.push_back(*p);
        return TS_OK;
    };
    auto undo = [&]() { for (void* p : sl.mem) b->arena.give(p); sl = Slot(); };
    ProbDesc& d = b->desc[slot];
    std::memset(&d, 0, sizeof d);
    if ((s = mixed_problem(*cfg, L, ph, grid, b->d_ctl + slot, take, d, err, b->ustream)) != TS_OK) {
        undo();
        return err.empty() ? s : fail(s, err);
    }
    for (int k = 0; k < 2; ++k) {
        if ((s = take(sizeof(double) * NV * L.plane, (void**)&d.U[k])) != TS_OK) { undo(); return s; }
        if ((s = take(sizeof(float) * NV * L.plane, (void**)&d.R[k])) != TS_OK) { undo(); return s; }
    }
    b->place(slot);
    // initial state: host -> staging -> U[0] (page-locked host memory is read
    // in place); no pending residual.  All on the upload stream; the main
    // stream waits for it before its next work, so stages already queued
    // there keep running meanwhile.
    const size_t nvals = (size_t)L.cells() * NV;
    const double* pinned = static_cast<const double*>(pinned_device_ptr(values, b->device));
    if (!pinned && b->ustage_doubles < nvals) {
        TB_CUDA(cudaStreamSynchronize(b->ustream));
        cudaFree(b->ustage);
        b->ustage = nullptr;
        b->ustage_doubles = 0;
        if (cudaMalloc(&b->ustage, nvals * sizeof(double)) != cudaSuccess) { undo(); return fail(TS_ERR_NO_MEMORY, "staging buffer"); }
        b->ustage_doubles = nvals;
    }
    cudaStream_t us = b->ustream;
    if (!pinned) TB_CUDA(cudaMemcpyAsync(b->ustage, values, nvals * sizeof(double), cudaMemcpyHostToDevice, us));
    k_b_scatter<<<(unsigned)((L.cells() + 255) / 256), 256, 0, us>>>(pinned ? pinned : b->ustage, L, d.U[0]);
    TB_CUDA(cudaMemsetAsync(d.R[0], 0, sizeof(float) * NV * L.plane, us));
    Ctl& c = b->h_ctl[slot];
    std::memset(&c, 0, sizeof c);
    c.next_sol = cfg->save_solution_time;
    c.next_slice = cfg->save_slice_time;
    c.save_sol = cfg->save_solution_time;
    c.save_slice = cfg->save_slice_time;
    c.max_iteration = cfg->max_iteration;
    c.max_time = cfg->max_time;
    c.run_mode = 1;
    TB_CUDA(cudaMemcpyAsync(b->d_ctl + slot, &c, sizeof(Ctl), cudaMemcpyHostToDevice, us));
    TB_CUDA(cudaMemcpyAsync(b->d_desc + slot, &d, sizeof(ProbDesc), cudaMemcpyHostToDevice, us));
    TB_CUDA(cudaEventRecord(b->uploaded, us));
    TB_CUDA(cudaStreamWaitEvent(b->stream, b->uploaded, 0));
    // the caller may reuse `values` on return; the upload stream only (not the
    // stages queued on the main stream) has to finish for that
    TB_CUDA(cudaStreamSynchronize(us));
    sl.used = true;
    sl.id = b->next_id++;
    sl.cells = L.cells();
    sl.cfg = *cfg;
    b->id2slot[sl.id] = slot;
    b->dirty = true;
    *id = sl.id;
    return TS_OK;
}

ts_status ts_batch_launch(ts_batch* b, int32_t n) {
    if (!b || n < 0) return fail(TS_ERR_INVALID, "bad argument");
    DevGuard g(b->device);
    long long ia, il;
    b->active(&ia, &il);
    if (2 * ia < il) b->dirty = true;  // most listed items belong to finished problems
    return b->launch(n);
}

ts_status ts_batch_wait(ts_batch* b, int32_t* active) {
    if (!b) return fail(TS_ERR_INVALID, "NULL batch");
    DevGuard g(b->device);
    ts_status s = b->pull();
    if (s != TS_OK) return s;
    if (active) *active = b->active(nullptr, nullptr);
    return TS_OK;
}

ts_status ts_batch_step(ts_batch* b, int32_t n) {
    if (!b || n < 0) return fail(TS_ERR_INVALID, "bad argument");
    DevGuard g(b->device);
    ts_status s = b->launch(n);
    if (s != TS_OK) return s;
    return b->pull();
}

ts_status ts_batch_run(ts_batch* b, int32_t max_stages, int32_t* active) {
    if (!b) return fail(TS_ERR_INVALID, "NULL batch");
    DevGuard g(b->device);
    ts_status s = b->pull();
    if (s != TS_OK) return s;
    long long done = 0;
    int chunk = 32;
    for (;;) {
        long long ia, il;
        const int a = b->active(&ia, &il);
        if (a == 0) break;
        if (max_stages > 0 && done >= max_stages) break;
        if (2 * ia < il) b->dirty = true;  // most listed items belong to finished problems
        int n = chunk;
        if (max_stages > 0) n = (int)std::min<long long>(n, max_stages - done);
        if ((s = b->launch(n)) != TS_OK) return s;
        if ((s = b->pull()) != TS_OK) return s;
        done += n;
        chunk = std::min(chunk * 2, 256);
    }
    if (active) *active = b->active(nullptr, nullptr);
    return TS_OK;
}

ts_status ts_batch_finished(ts_batch* b, int32_t* ids, int32_t cap, int32_t* n) {
    if (!b || !n) return fail(TS_ERR_INVALID, "NULL argument");
    int k = 0;
    for (int s = 0; s < b->capacity; ++s) {
        Slot& sl = b->slots[s];
        if (!sl.used || sl.id < 0 || sl.collected || !b->h_ctl[s].stop_req) continue;
        if (k < cap && ids) { ids[k] = sl.id; sl.collected = true; }
        ++k;
    }
    *n = std::min(k, cap);
    return TS_OK;
}

ts_status ts_batch_get(ts_batch* b, int32_t id, double* values, ts_step_info* info) {
    if (!b) return fail(TS_ERR_INVALID, "NULL batch");
    auto it = b->id2slot.find(id);
    if (it == b->id2slot.end()) return fail(TS_ERR_NOT_FOUND, "unknown problem id");
    const int slot = it->second;
    DevGuard g(b->device);
    const Layout& L = b->desc[slot].L;
    const unsigned blocks = (unsigned)((L.cells() + 255) / 256);
    // A finished problem is no longer touched by stages (its items skip), so
    // its read-back runs on the download stream beside whatever is queued on
    // the main stream; a running one is read in stream order.
    const bool finished = b->h_ctl[slot].stop_req != 0;
    cudaStream_t st = finished ? b->dstream : b->stream;
    mixed_apply(b->d_desc, slot, L.cells(), st);
    double* pinned = values ? static_cast<double*>(pinned_device_ptr(values, b->device)) : nullptr;
    if (values && pinned) {
        // page-locked host memory: gathered in place
        k_b_gather<<<blocks, 256, 0, st>>>(pinned, b->d_desc, slot);
        TB_CUDA(cudaGetLastError());
    } else if (values) {
        const size_t nvals = (size_t)L.cells() * NV;
        if (b->dstage_doubles < nvals) {
            cudaFree(b->dstage);
            b->dstage = nullptr;
            b->dstage_doubles = 0;
            TB_CUDA(cudaMalloc(&b->dstage, nvals * sizeof(double)));
            b->dstage_doubles = nvals;
        }
        k_b_gather<<<blocks, 256, 0, st>>>(b->dstage, b->d_desc, slot);
        TB_CUDA(cudaGetLastError());
        TB_CUDA(cudaMemcpyAsync(values, b->dstage, nvals * sizeof(double), cudaMemcpyDeviceToHost, st));
    }
    ts_status s = TS_OK;
    if (finished) TB_CUDA(cudaStreamSynchronize(st));
    else s = b->pull();
    if (s != TS_OK) return s;
    if (info) {
        const Ctl& c = b->h_ctl[slot];
        info->iteration = c.iteration;
        info->health = c.health;
        info->time = c.time;
        info->dt = c.dt;
        info->next_solution_time = c.next_sol;
        info->next_slice_time = c.next_slice;
        for (int v = 0; v < NV; ++v) info->residual[v] = c.res[v];  // zeros unless residual_norms
    }
    return TS_OK;
}

ts_status ts_batch_remove(ts_batch* b, int32_t id) {
    if (!b) return fail(TS_ERR_INVALID, "NULL batch");
    auto it = b->id2slot.find(id);
    if (it == b->id2slot.end()) return fail(TS_ERR_NOT_FOUND, "unknown problem id");
    DevGuard g(b->device);
    const int slot = it->second;
    // a running problem may still be read by queued stages: drain them first.
    // A finished one is skipped by them, so its memory is free at once; its
    // slot waits until the main stream has drained (the work lists queued
    // there still name it).
    if (!b->h_ctl[slot].stop_req) TB_CUDA(cudaStreamSynchronize(b->stream));
    TB_CUDA(cudaStreamSynchronize(b->dstream));
    Slot& sl = b->slots[slot];
    b->done_cell_updates += (double)sl.cells * (double)b->h_ctl[slot].iteration;
    for (void* p : sl.mem) b->arena.give(p);
    sl = Slot();
    sl.used = true;  // quarantined until the next drain
    b->quarantine.push_back(slot);
    std::memset(&b->h_ctl[slot], 0, sizeof(Ctl));
    b->h_ctl[slot].stop_req = 1;
    TB_CUDA(cudaMemcpyAsync(b->d_ctl + slot, &b->h_ctl[slot], sizeof(Ctl), cudaMemcpyHostToDevice, b->stream));
    b->id2slot.erase(it);
    b->dirty = true;
    return TS_OK;
}

ts_status ts_batch_set_tail(ts_batch* b, int32_t enable) {
    if (!b) return fail(TS_ERR_INVALID, "NULL batch");
    DevGuard g(b->device);
    TB_CUDA(cudaStreamSynchronize(b->stream));
    b->tail_enabled = enable != 0;
    b->dirty = true;
    return TS_OK;
}

ts_status ts_batch_set_tile(ts_batch* b, int32_t nd, int32_t tx, int32_t ty, int32_t ctas) {
    if (!b || nd < 1 || nd > 2 || ctas < 0) return fail(TS_ERR_INVALID, "bad argument");
    ty = 1;
    if (tx != 0) {
        size_t bytes;
        int per;
        if (!mixed_tile_info(nd, tx, ty, TS_RS_ROE_PIKE, &bytes, &per, true) || per < 1)
            return fail(TS_ERR_UNSUPPORTED, "no compiled tile of that shape");
    }
    DevGuard g(b->device);
    TB_CUDA(cudaStreamSynchronize(b->stream));
    b->tune[nd] = Tune{tx, ty, ctas};
    for (int s = 0; s < b->capacity; ++s) {
        if (!b->slots[s].used || b->slots[s].id < 0 || b->desc[s].L.nd != nd) continue;
        b->place(s);
        TB_CUDA(cudaMemcpyAsync(b->d_desc + s, &b->desc[s], sizeof(ProbDesc), cudaMemcpyHostToDevice, b->stream));
    }
    TB_CUDA(cudaStreamSynchronize(b->stream));
    b->dirty = true;
    return TS_OK;
}

ts_status ts_batch_autotune(ts_batch* b, int32_t stages, int32_t* tx_out, int32_t* ty_out, int32_t* ctas_out) {
    if (!b || stages < 1) return fail(TS_ERR_INVALID, "bad argument");
    DevGuard g(b->device);
    ts_status s = b->pull();
    if (s != TS_OK) return s;
    // dominant dimension by cells
    long long cells[3] = {0, 0, 0};
    for (int k = 0; k < b->capacity; ++k)
        if (b->slots[k].used && b->slots[k].id >= 0) cells[b->desc[k].L.nd] += b->slots[k].cells;
    const int nd = cells[2] > cells[1] ? 2 : 1;
    if (cells[nd] == 0) return fail(TS_ERR_INVALID, "empty batch");
    // snapshot: the arena up to its high-water mark and the control words
    char* snap = nullptr;
    Ctl* snap_ctl = nullptr;
    const size_t hb = b->arena.high;
    TB_CUDA(cudaMalloc(&snap, std::max<size_t>(hb, 1)));
    TB_CUDA(cudaMalloc(&snap_ctl, sizeof(Ctl) * b->capacity));
    auto restore = [&]() -> ts_status {
        TB_CUDA(cudaMemcpyAsync(b->arena.base, snap, hb, cudaMemcpyDeviceToDevice, b->stream));
        TB_CUDA(cudaMemcpyAsync(b->d_ctl, snap_ctl, sizeof(Ctl) * b->capacity, cudaMemcpyDeviceToDevice, b->stream));
        TB_CUDA(cudaStreamSynchronize(b->stream));
        return b->pull();
    };
    TB_CUDA(cudaMemcpyAsync(snap, b->arena.base, hb, cudaMemcpyDeviceToDevice, b->stream));
    TB_CUDA(cudaMemcpyAsync(snap_ctl, b->d_ctl, sizeof(Ctl) * b->capacity, cudaMemcpyDeviceToDevice, b->stream));
    // candidates: the per-problem policy, then every compiled one-row tile;
    // each with as many resident CTAs as fit, and capped at 2 and 1
    std::vector<Tune> cand;
    const int* tiles = nd == 1 ? kTiles1D : kTiles2D;
    for (int k = -1; k < 3; ++k) {
        const int tx = k < 0 ? 0 : tiles[k];
        size_t bytes;
        int per = 0;
        mixed_tile_info(nd, tx > 0 ? tx : tiles[0], 1, TS_RS_ROE_PIKE, &bytes, &per, true);
        if (per < 1) continue;
        cand.push_back(Tune{tx, 1, 0});
        for (int c : {2, 1})
            if (c < per) cand.push_back(Tune{tx, 1, c});
    }
    const Tune saved = b->tune[nd];
    const long long st0 = b->stages, la0 = b->launches;
    Tune best = saved;
    float best_ms = 1e30f;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    for (const Tune& t : cand) {
        if ((s = ts_batch_set_tile(b, nd, t.tx, t.ty, t.ctas)) != TS_OK) break;
        if ((s = b->launch(1)) != TS_OK) break;  // rebuild + warm-up
        if ((s = restore()) != TS_OK) break;
        cudaEventRecord(e0, b->stream);
        if ((s = b->launch(stages)) != TS_OK) break;
        cudaEventRecord(e1, b->stream);
        cudaEventSynchronize(e1);
        float ms = 0.f;
        cudaEventElapsedTime(&ms, e0, e1);
        if (ms < best_ms) { best_ms = ms; best = t; }
        if ((s = restore()) != TS_OK) break;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(snap);
    cudaFree(snap_ctl);
    b->stages = st0;
    b->launches = la0;
    if (s != TS_OK) return s;
    if ((s = ts_batch_set_tile(b, nd, best.tx, best.ty, best.ctas)) != TS_OK) return s;
    if (tx_out) *tx_out = best.tx;
    if (ty_out) *ty_out = best.ty;
    if (ctas_out) *ctas_out = best.ctas;
    return TS_OK;
}

ts_status ts_batch_stats(ts_batch* b, double* cell_updates, int64_t* stages, int64_t* launches) {
    if (!b) return fail(TS_ERR_INVALID, "NULL batch");
    if (cell_updates) *cell_updates = b->cell_updates();
    if (stages) *stages = b->stages;
    if (launches) *launches = b->launches;
    return TS_OK;
}

}  // extern "C"
