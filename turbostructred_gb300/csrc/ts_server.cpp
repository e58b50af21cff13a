// Served solves over one batch (include/ts_fvm.h, ts_server_*).
//
// Threads: callers submit and wait; one worker owns the batch.  The worker
// repeats: admit queued requests (in arrival order, or least work first)
// while the arena has room and the caps on admitted cells and solves allow,
// run one chunk of stages of everything admitted, retire what finished
// (state read back, slot and memory freed).  The cell cap keeps the admitted
// set near the size that saturates the GPU: beyond it, admitting more only
// stretches every admitted solve (all of them share each stage).  The chunk length adapts so one
// chunk takes about chunk_ms, which bounds how long a new arrival waits for
// the next admission point and how late a finished solve is noticed.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <condition_variable>
#include <cstdlib>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <unordered_map>
#include <vector>

#include "ts_fvm.h"
#include "ts_internal.h"

namespace {

using Clock = std::chrono::steady_clock;

// Page-locked host buffers for request states, kept by size and reused: the
// worker's uploads and read-backs then run as DMA transfers instead of
// through CUDA's staging of pageable memory (about 5 GB/s measured on the served
// stream, slow enough that the copies of one pass outlasted the chunk of
// stages in flight and left the GPU idle).  Past kPinnedCap bytes of pinned
// buffers, or when pinning fails, a buffer is ordinary memory.
class PinnedPool {
public:
    static constexpr size_t kPinnedCap = size_t(8) << 30;

    ~PinnedPool() {
        for (auto& kv : free_) cudaFreeHost(kv.second);
    }

    // A buffer of `bytes`; *pinned tells which kind.  nullptr when out of memory.
    void* take(size_t bytes, bool* pinned) {
        {
            std::lock_guard<std::mutex> lk(mu_);
            auto it = free_.find(bytes);
            if (it != free_.end()) {
                void* p = it->second;
                free_.erase(it);
                *pinned = true;
                return p;
            }
            if (pinned_ + bytes <= kPinnedCap) {
                void* p = nullptr;
                if (cudaHostAlloc(&p, bytes, cudaHostAllocPortable) == cudaSuccess) {
                    pinned_ += bytes;
                    *pinned = true;
                    return p;
                }
                cudaGetLastError();
            }
        }
        *pinned = false;
        return std::malloc(bytes);
    }

    void give(void* p, size_t bytes, bool pinned) {
        if (!p) return;
        if (!pinned) { std::free(p); return; }
        std::lock_guard<std::mutex> lk(mu_);
        free_.emplace(bytes, p);
    }

private:
    std::mutex mu_;
    std::multimap<size_t, void*> free_;
    size_t pinned_ = 0;  // bytes of all pinned buffers, free or taken
};

// A request's state in a pool buffer, returned to the pool with the request.
struct StateBuf {
    PinnedPool* pool = nullptr;
    double* p = nullptr;
    size_t n = 0;  // doubles
    bool pinned = false;

    StateBuf() = default;
    StateBuf(const StateBuf&) = delete;
    StateBuf& operator=(const StateBuf&) = delete;
    ~StateBuf() { reset(); }

    bool assign(PinnedPool* pl, const double* src, size_t count) {
        reset();
        pool = pl;
        p = static_cast<double*>(pl->take(count * sizeof(double), &pinned));
        if (!p) return false;
        n = count;
        std::memcpy(p, src, count * sizeof(double));
        return true;
    }
    void reset() {
        if (p) pool->give(p, n * sizeof(double), pinned);
        p = nullptr;
        n = 0;
    }
    double* data() { return p; }
};

struct Request {
    int32_t id = -1;
    double work = 0.0;  // admission key of TS_SERVE_SHORTEST_FIRST
    ts_config cfg{};
    std::vector<ts_block_node> blocks[3];
    StateBuf values;  // initial state; the final one when kept
    bool keep = true;
    size_t bytes = 0;
    double cells = 0.0;
    int32_t batch_id = -1;
    bool done = false;
    ts_status status = TS_OK;
    std::string error;
    ts_step_info info{};
    ts_request_times t{};
};

using Req = std::shared_ptr<Request>;

double percentile(std::vector<double> v, double p) {
    if (v.empty()) return 0.0;
    std::sort(v.begin(), v.end());
    // nearest rank
    size_t k = (size_t)std::ceil(p / 100.0 * (double)v.size());
    k = std::min(std::max<size_t>(k, 1), v.size());
    return v[k - 1];
}

}  // namespace

struct ts_server {
    // first member: destroyed last, after every request has returned its buffer
    PinnedPool pool;
    int device = 0;
    size_t budget = 0;
    int max_active = 0;
    int order = TS_SERVE_FIFO;
    long long max_cells = 0;
    double chunk_ms = 2.0;
    ts_batch* batch = nullptr;
    Clock::time_point t0 = Clock::now();

    std::mutex mu;
    std::condition_variable cv_work, cv_done;
    std::deque<Req> queue;
    std::unordered_map<int32_t, Req> requests;  // submitted and not yet collected
    std::unordered_map<int32_t, Req> running;   // by batch id
    std::vector<double> lat_ms, wait_ms;
    int64_t submitted = 0, admitted = 0, completed = 0, rejected = 0;
    int64_t stages = 0, launches = 0;
    double cell_updates = 0.0, busy_s = 0.0, admit_s = 0.0, retire_s = 0.0;
    size_t in_use = 0;
    double in_cells = 0.0;
    ts_status worker_status = TS_OK;
    std::string worker_error;
    bool stop = false;
    int32_t next_id = 0;
    std::thread worker;

    double now() const { return std::chrono::duration<double>(Clock::now() - t0).count(); }

    // Under the lock.
    void retire(const Req& r, ts_status st, const std::string& err) {
        r->status = st;
        r->error = err;
        r->done = true;
        r->t.finish_s = now();
        if (st == TS_OK) {
            ++completed;
            lat_ms.push_back(1e3 * (r->t.finish_s - r->t.submit_s));
        } else {
            ++rejected;
        }
    }

    void worker_failed(ts_status st) {
        std::lock_guard<std::mutex> lk(mu);
        worker_status = st;
        worker_error = ts_last_error();
        for (auto& kv : running) retire(kv.second, st, worker_error);
        running.clear();
        for (auto& r : queue) retire(r, st, worker_error);
        queue.clear();
        in_use = 0;
        in_cells = 0.0;
        cv_done.notify_all();
    }

    // One pass: admit (uploads overlap the chunk in flight), retire what the
    // last wait found finished (read-backs overlap it too), wait for the
    // chunk, launch the next one.
    void loop() {
        int chunk = 4;
        bool in_flight = false;
        int32_t active = 0;
        Clock::time_point launched = Clock::now();
        std::vector<int32_t> fin(1024), to_retire;
        for (;;) {
            std::vector<Req> admit;
            {
                std::unique_lock<std::mutex> lk(mu);
                if (running.empty() && !in_flight) cv_work.wait(lk, [&] { return stop || !queue.empty(); });
                if (stop) {
                    lk.unlock();
                    if (in_flight) ts_batch_wait(batch, &active);
                    return;
                }
                if (order == TS_SERVE_SHORTEST_FIRST)
                    std::stable_sort(queue.begin(), queue.end(),
                                     [](const Req& x, const Req& y) { return x.get()->work < y.get()->work; });
                size_t room = budget - in_use;
                double cells = in_cells;
                while (!queue.empty()) {
                    const Req& r = queue.front();
                    const bool idle = running.empty() && admit.empty();
                    if (max_active > 0 && running.size() + admit.size() >= (size_t)max_active) break;
                    if (max_cells > 0 && cells + r->cells > (double)max_cells && !idle) break;
                    if (r->bytes > room) break;  // the next in order waits for memory
                    room -= r->bytes;
                    cells += r->cells;
                    admit.push_back(r);
                    queue.pop_front();
                }
            }
            const Clock::time_point a0 = Clock::now();
            int added = 0;
            for (size_t k = 0; k < admit.size(); ++k) {
                const Req& r = admit[k];
                int32_t bid = -1;
                const ts_status s = ts_batch_add(batch, &r->cfg, r->values.data(), &bid);
                if (s == TS_ERR_NO_MEMORY) {
                    // the arena is fragmented: the rest goes back to the head, in order
                    std::lock_guard<std::mutex> lk(mu);
                    for (size_t j = admit.size(); j-- > k;) queue.push_front(admit[j]);
                    break;
                }
                std::lock_guard<std::mutex> lk(mu);
                if (s != TS_OK) {
                    retire(r, s, ts_last_error());
                    cv_done.notify_all();
                    continue;
                }
                ++added;
                r->batch_id = bid;
                r->t.admit_s = now();
                if (!r->keep) r->values.reset();
                running[bid] = r;
                in_use += r->bytes;
                in_cells += r->cells;
                ++admitted;
                wait_ms.push_back(1e3 * (r->t.admit_s - r->t.submit_s));
            }
            const Clock::time_point r0 = Clock::now();
            ts_status s = TS_OK;
            for (int32_t bid : to_retire) {
                Req r;
                {
                    std::lock_guard<std::mutex> lk(mu);
                    auto it = running.find(bid);
                    if (it == running.end()) continue;
                    r = it->second;
                }
                s = ts_batch_get(batch, bid, r->keep ? r->values.data() : nullptr, &r->info);
                if (s == TS_OK) s = ts_batch_remove(batch, bid);
                if (s != TS_OK) break;
                std::lock_guard<std::mutex> lk(mu);
                running.erase(bid);
                in_use -= r->bytes;
                in_cells -= r->cells;
                retire(r, TS_OK, "");
                cv_done.notify_all();
            }
            to_retire.clear();
            if (s != TS_OK) { worker_failed(s); return; }
            const Clock::time_point w0 = Clock::now();
            {
                std::lock_guard<std::mutex> lk(mu);
                admit_s += std::chrono::duration<double>(r0 - a0).count();
                retire_s += std::chrono::duration<double>(w0 - r0).count();
            }
            if (in_flight) {
                if ((s = ts_batch_wait(batch, &active)) != TS_OK) { worker_failed(s); return; }
                in_flight = false;
                const double el = std::chrono::duration<double>(Clock::now() - launched).count();
                // next chunk: about chunk_ms of stages at the current rate
                const double per_stage_ms = std::max(1e3 * el / chunk, 1e-3);
                chunk = std::min(std::max((int)(chunk_ms / per_stage_ms), 1), 4096);
                for (;;) {
                    int32_t n = 0;
                    if ((s = ts_batch_finished(batch, fin.data(), (int32_t)fin.size(), &n)) != TS_OK) break;
                    to_retire.insert(to_retire.end(), fin.begin(), fin.begin() + n);
                    if (n < (int32_t)fin.size()) break;
                }
                if (s != TS_OK) { worker_failed(s); return; }
                double cu = 0.0;
                int64_t st = 0, la = 0;
                ts_batch_stats(batch, &cu, &st, &la);
                std::lock_guard<std::mutex> lk(mu);
                busy_s += el;
                cell_updates = cu;
                stages = st;
                launches = la;
            }
            if (active > 0 || added > 0) {
                launched = Clock::now();
                if ((s = ts_batch_launch(batch, chunk)) != TS_OK) { worker_failed(s); return; }
                in_flight = true;
                active = std::max(active, added);
            }
        }
    }
};

extern "C" {

ts_status ts_server_create(const ts_server_config* cfg, ts_server** out) {
    if (!out || !cfg) return ts::fail(TS_ERR_INVALID, "NULL argument");
    *out = nullptr;
    if (cfg->max_active < 0 || cfg->chunk_ms < 0.0 || cfg->max_cells < 0 ||
        (cfg->order != TS_SERVE_FIFO && cfg->order != TS_SERVE_SHORTEST_FIRST))
        return ts::fail(TS_ERR_INVALID, "bad server configuration");
    std::unique_ptr<ts_server> s(new ts_server());
    ts_status st = ts_batch_create(cfg->device, cfg->memory_budget, &s->batch);
    if (st != TS_OK) return st;
    s->device = cfg->device;
    s->budget = cfg->memory_budget;
    s->max_active = cfg->max_active;
    s->order = cfg->order;
    s->max_cells = cfg->max_cells;
    s->chunk_ms = cfg->chunk_ms > 0.0 ? cfg->chunk_ms : 2.0;
    s->t0 = Clock::now();
    ts_server* p = s.get();
    s->worker = std::thread([p] { p->loop(); });
    *out = s.release();
    return TS_OK;
}

void ts_server_destroy(ts_server* s) {
    if (!s) return;
    {
        std::lock_guard<std::mutex> lk(s->mu);
        s->stop = true;
    }
    s->cv_work.notify_all();
    if (s->worker.joinable()) s->worker.join();
    ts_batch_destroy(s->batch);
    delete s;
}

ts_status ts_server_submit(ts_server* s, const ts_config* cfg, const double* values, int32_t keep_state,
                           int32_t* request_id) {
    if (!s || !cfg || !values || !request_id) return ts::fail(TS_ERR_INVALID, "NULL argument");
    const size_t bytes = ts_batch_problem_bytes(cfg);
    if (bytes == 0) {
        std::string err;
        if (ts::validate_config(*cfg, err) != TS_OK) return ts::fail(TS_ERR_INVALID, err);
        return ts::fail(TS_ERR_UNSUPPORTED,
                        "served solves are 1D/2D mixed precision with one boundary condition per side");
    }
    if (bytes > s->budget) return ts::fail(TS_ERR_NO_MEMORY, "solve larger than the server's memory budget");
    Req r = std::make_shared<Request>();
    r->cfg = *cfg;
    for (int a = 0; a < 3; ++a) {
        if (cfg->n_blocks[a] > 0 && cfg->blocks[a]) {
            r->blocks[a].assign(cfg->blocks[a], cfg->blocks[a] + cfg->n_blocks[a]);
            r->cfg.blocks[a] = r->blocks[a].data();
        }
    }
    const double ny = cfg->n_dims > 1 ? cfg->ny : 1, nz = cfg->n_dims > 2 ? cfg->nz : 1;
    r->cells = (double)cfg->nx * ny * nz;
    if (!r->values.assign(&s->pool, values, (size_t)r->cells * 5))
        return ts::fail(TS_ERR_NO_MEMORY, "no host memory for the request's state");
    r->keep = keep_state != 0;
    r->bytes = bytes;
    // work: cell-updates when MaxIteration bounds the run, else cells
    r->work = r->cells * (cfg->max_iteration > 0 && cfg->max_iteration < (1 << 30) ? cfg->max_iteration : 1.0);
    std::lock_guard<std::mutex> lk(s->mu);
    if (s->worker_status != TS_OK) return ts::fail(s->worker_status, "server stopped: " + s->worker_error);
    r->id = s->next_id++;
    r->t.submit_s = s->now();
    s->requests[r->id] = r;
    s->queue.push_back(r);
    ++s->submitted;
    *request_id = r->id;
    s->cv_work.notify_one();
    return TS_OK;
}

ts_status ts_server_wait(ts_server* s, int32_t id, int32_t timeout_ms, double* values, ts_step_info* info,
                         ts_request_times* times) {
    if (!s) return ts::fail(TS_ERR_INVALID, "NULL server");
    std::unique_lock<std::mutex> lk(s->mu);
    auto it = s->requests.find(id);
    if (it == s->requests.end()) return ts::fail(TS_ERR_NOT_FOUND, "unknown request id");
    Req r = it->second;
    if (timeout_ms < 0) {
        s->cv_done.wait(lk, [&] { return r->done; });
    } else if (!s->cv_done.wait_for(lk, std::chrono::milliseconds(timeout_ms), [&] { return r->done; })) {
        return ts::fail(TS_ERR_TIMEOUT, "request not finished");
    }
    s->requests.erase(id);
    if (r->status != TS_OK) return ts::fail(r->status, r->error);
    if (values && r->keep) std::memcpy(values, r->values.data(), r->values.n * sizeof(double));
    if (info) *info = r->info;
    if (times) *times = r->t;
    return TS_OK;
}

ts_status ts_server_drain(ts_server* s, int32_t timeout_ms) {
    if (!s) return ts::fail(TS_ERR_INVALID, "NULL server");
    std::unique_lock<std::mutex> lk(s->mu);
    auto idle = [&] { return s->queue.empty() && s->running.empty(); };
    if (timeout_ms < 0) {
        s->cv_done.wait(lk, idle);
    } else if (!s->cv_done.wait_for(lk, std::chrono::milliseconds(timeout_ms), idle)) {
        return ts::fail(TS_ERR_TIMEOUT, "server still busy");
    }
    return s->worker_status == TS_OK ? TS_OK : ts::fail(s->worker_status, s->worker_error);
}

ts_status ts_server_stats_get(ts_server* s, ts_server_stats* o) {
    if (!s || !o) return ts::fail(TS_ERR_INVALID, "NULL argument");
    std::lock_guard<std::mutex> lk(s->mu);
    o->submitted = s->submitted;
    o->admitted = s->admitted;
    o->completed = s->completed;
    o->rejected = s->rejected;
    o->queued = (int64_t)s->queue.size();
    o->active = (int64_t)s->running.size();
    o->stages = s->stages;
    o->launches = s->launches;
    o->cell_updates = s->cell_updates;
    o->busy_s = s->busy_s;
    o->admit_s = s->admit_s;
    o->retire_s = s->retire_s;
    o->latency_p50_ms = percentile(s->lat_ms, 50.0);
    o->latency_p99_ms = percentile(s->lat_ms, 99.0);
    o->latency_max_ms = s->lat_ms.empty() ? 0.0 : *std::max_element(s->lat_ms.begin(), s->lat_ms.end());
    o->wait_p50_ms = percentile(s->wait_ms, 50.0);
    o->wait_p99_ms = percentile(s->wait_ms, 99.0);
    o->bytes_budget = s->budget;
    o->bytes_in_use = s->in_use;
    o->worker_status = s->worker_status;
    return TS_OK;
}

}  // extern "C"
