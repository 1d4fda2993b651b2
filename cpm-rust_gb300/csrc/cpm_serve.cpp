// Serving loop (see cpm_serve.h).
#include "cpm_serve.h"

#include <algorithm>
#include <chrono>
#include <cstring>

#include "cpm_kernels.h"

namespace cpmhost {

struct Server::Req {
    Server* owner = nullptr;
    uint64_t ticket = 0;
    Config c;
    Initial init;
    ReadoutOptions ro;
    ReqState state = REQ_PLACING;
    bool cancel = false;
    std::string err;
    Result result;
    ReqTimes times;
    std::unique_ptr<DeviceSims> dev;
    cudaStream_t stream = nullptr;
    RunPlan full;
    int ns = 0, nt = 0;
    size_t est_bytes = 0;
};

namespace {

// Device bytes one simulation needs (the arena DeviceSims::create carves,
// with a margin for alignment), known before anything is allocated.
size_t estimate_bytes(const Config& c, const Initial& init, int ns, int ne, bool snapshots) {
    Geometry g;
    g.init(c);
    const size_t n1 = init.type_of.size() + 1, nt = c.types.size(), D = (size_t)c.D, t1 = nt + 1;
    uint32_t tmax = 0;
    for (auto& t : c.types) tmax = std::max({tmax, t.target_volume, t.target_interface});
    const size_t tab = std::min<size_t>(8192, 2 * (size_t)tmax + 128);
    size_t b = (size_t)g.n_padded * 4;
    b += n1 * (2 + 4 + 4 + 8 * D + 8 * D * D + 8);
    b += CPM_STAT_COUNT * 8 + t1 * t1 * 12 + nt * 24 + t1 * t1 * t1 * 12 + nt * tab * 32;
    if (c.active.act) b += nt * 12 + (size_t)g.n_padded * 4;  // Act parameters and acquisition MCS
    b += (size_t)std::max(1, ne) * 8;
    b += (size_t)ns * n1 * (8 + 8 * D + 8 * D * D);
    if (snapshots) b += (size_t)ns * (size_t)g.n_sites * 4;
    if (snapshots && ns > 0) b += topology_bytes(g.n_sites, (int)init.type_of.size());
    return b + 64 * 256 + sizeof(SimDesc) + 64;
}

}  // namespace

double Server::now() const {
    return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count() - t0_;
}

Server::Server() = default;
Server::~Server() { stop(); }

std::string Server::start(const ServeOptions& o) {
    std::lock_guard<std::mutex> lk(mu_);
    if (started_) return "server already started";
    opt_ = o;
    if (opt_.max_active <= 0) opt_.max_active = 128;
    if (opt_.hbm_budget == 0) opt_.hbm_budget = 150ull << 30;
    cudaError_t e = cudaGetDevice(&device_);
    if (e != cudaSuccess) return std::string("CUDA error: ") + cudaGetErrorString(e);
    t0_ = 0;
    t0_ = now();
    int np = opt_.placement_threads;
    if (np <= 0) np = (int)std::max(2u, std::min(16u, std::thread::hardware_concurrency()));
    for (int i = 0; i < np; ++i)
        pool_.emplace_back([this] {
            cudaSetDevice(device_);
            pool_loop();
        });
    scheduler_ = std::thread([this] {
        cudaSetDevice(device_);
        scheduler_loop();
    });
    started_ = true;
    return "";
}

std::string Server::submit(const Config& c, const ReadoutOptions& ro, uint64_t& ticket) {
    auto r = std::make_unique<Req>();
    r->owner = this;
    r->c = c;
    r->ro = ro;
    std::lock_guard<std::mutex> lk(mu_);
    if (!started_ || stopping_) return "server is not running";
    r->ticket = next_ticket_++;
    r->times.submitted = now();
    ticket = r->ticket;
    placing_.push_back(r.get());
    reqs_[ticket] = std::move(r);
    st_.submitted++;
    cv_pool_.notify_one();
    return "";
}

// Host pool: placements of new requests and read-backs of finished ones.
void Server::pool_loop() {
    for (;;) {
        Req* r = nullptr;
        bool place = false;
        {
            std::unique_lock<std::mutex> lk(mu_);
            cv_pool_.wait(lk, [&] { return stopping_ || !placing_.empty() || !finishing_.empty(); });
            if (!finishing_.empty()) {
                r = finishing_.front();
                finishing_.pop_front();
            } else if (stopping_) {
                return;
            } else {
                r = placing_.front();
                placing_.pop_front();
                place = true;
                if (r->cancel) {
                    r->state = REQ_CANCELLED;
                    st_.cancelled++;
                    cv_done_.notify_all();
                    continue;
                }
            }
        }
        if (!place) {
            finish(r);
            continue;
        }
        // placement (initialization.rs:39-330) and the window's sizes
        std::string e = initialize(r->c, r->init);
        const bool snapshots = r->ro.include_lattice || r->ro.topology;
        if (e.empty()) {
            r->full = plan_for(r->c, 0, snapshots);
            r->ns = r->full.n_samples;
            r->nt = trace_points(r->c.burn_in, r->c.interval, r->full.energy_sample_start);
            r->est_bytes = estimate_bytes(r->c, r->init, r->ns, r->ns + r->nt, snapshots);
        }
        std::lock_guard<std::mutex> lk(mu_);
        if (!e.empty()) {
            r->state = REQ_FAILED;
            r->err = e;
            r->times.finished = now();
            st_.failed++;
            cv_done_.notify_all();
        } else if (r->cancel) {
            r->state = REQ_CANCELLED;
            st_.cancelled++;
            cv_done_.notify_all();
        } else {
            r->state = REQ_QUEUED;
            ready_[r->ticket] = r;
            cv_work_.notify_one();
        }
    }
}

// Runs on a CUDA-internal thread when a simulation's stream reaches its end:
// no CUDA calls here, only the hand-over to the pool.
void CUDART_CB Server::device_done(void* ctx) {
    Req* r = static_cast<Req*>(ctx);
    Server* s = r->owner;
    std::lock_guard<std::mutex> lk(s->mu_);
    r->times.device_done = s->now();
    s->finishing_.push_back(r);
    s->cv_pool_.notify_one();
}

// Uploads an admitted simulation and enqueues its whole run window on its
// own stream (scheduler thread).
std::string Server::admit(Req& r) {
    cudaError_t ce = cudaStreamCreateWithFlags(&r.stream, cudaStreamNonBlocking);
    if (ce != cudaSuccess) return std::string("CUDA error: ") + cudaGetErrorString(ce);
    r.dev = std::make_unique<DeviceSims>();
    r.dev->set_stream_ordered(true);
    r.dev->set_tiled_grid_cap(opt_.tiled_grid_cap);
    const bool snapshots = r.ro.include_lattice || r.ro.topology;
    std::string e = r.dev->create({r.c}, {r.init}, {r.ns}, {r.ns + r.nt}, snapshots, r.stream);
    if (!e.empty()) return e;
    size_t bytes = r.dev->device_bytes();
    if (r.ro.topology && r.ns > 0) bytes += topology_bytes(r.dev->layout(0).g.n_sites, r.dev->layout(0).n_cells);
    e = r.dev->run({r.full});
    if (!e.empty()) return e;
    // The accounting moves from the estimate to the arena's actual size
    // before the hand-over is enqueued: from then on the pool may finish the
    // request (and a caller take it) at any moment.
    {
        std::lock_guard<std::mutex> lk(mu_);
        r.times.device_bytes = bytes;
        st_.bytes_in_use += bytes;
        st_.bytes_in_use -= r.est_bytes;
        st_.peak_bytes = std::max(st_.peak_bytes, st_.bytes_in_use);
        st_.launched++;
    }
    ce = cudaLaunchHostFunc(r.stream, &Server::device_done, &r);
    if (ce != cudaSuccess) {
        std::lock_guard<std::mutex> lk(mu_);
        st_.bytes_in_use += r.est_bytes;
        st_.bytes_in_use -= bytes;
        st_.launched--;
        return std::string("CUDA error: ") + cudaGetErrorString(ce);
    }
    return "";
}

void Server::release(Req& r) {
    r.dev.reset();  // stream-ordered frees on r.stream
    if (r.stream) cudaStreamDestroy(r.stream);
    r.stream = nullptr;
}

// Reads a finished simulation back, builds its result, frees it (pool).
void Server::finish(Req* rp) {
    Req& r = *rp;
    std::string e = r.dev->sync();  // stream done; tiled timeouts surface here
    bool cancelled;
    {
        std::lock_guard<std::mutex> lk(mu_);
        cancelled = r.cancel;
    }
    if (e.empty() && !cancelled) {
        std::vector<std::vector<Topo>> topo;
        if (r.ro.topology) e = r.dev->topology({0}, {r.ns}, topo);
        if (e.empty()) e = assemble_result(r.c, r.init, *r.dev, 0, r.ns, r.nt, r.ro, r.result);
        if (e.empty() && r.ro.topology) attach_topology(r.c, topo[0], r.result);
    }
    release(r);
    std::lock_guard<std::mutex> lk(mu_);
    st_.bytes_in_use -= r.times.device_bytes;
    active_--;
    if (active_ == 0 && busy_since_ >= 0) {
        st_.busy_seconds += now() - busy_since_;
        busy_since_ = -1;
    }
    r.times.finished = now();
    if (cancelled) {
        r.state = REQ_CANCELLED;
        st_.cancelled++;
    } else if (e.empty()) {
        r.state = REQ_DONE;
        st_.completed++;
    } else {
        r.state = REQ_FAILED;
        r.err = e;
        st_.failed++;
    }
    cv_done_.notify_all();
    cv_work_.notify_one();
}

void Server::scheduler_loop() {
    for (;;) {
        std::vector<Req*> admitted;
        {
            std::unique_lock<std::mutex> lk(mu_);
            auto can_admit = [&] {
                if (ready_.empty()) return false;
                const Req* r = ready_.begin()->second;
                if (r->cancel) return true;
                if ((int)active_ >= opt_.max_active) return false;
                return active_ == 0 || st_.bytes_in_use + r->est_bytes <= opt_.hbm_budget;
            };
            cv_work_.wait(lk, [&] { return stopping_ || can_admit(); });
            if (stopping_) break;
            // admission in ticket order under the slot and byte limits
            while (can_admit()) {
                Req* r = ready_.begin()->second;
                ready_.erase(ready_.begin());
                if (r->cancel) {
                    r->state = REQ_CANCELLED;
                    st_.cancelled++;
                    cv_done_.notify_all();
                    continue;
                }
                st_.bytes_in_use += r->est_bytes;
                active_++;
                if (busy_since_ < 0) busy_since_ = now();
                st_.peak_active = std::max<uint64_t>(st_.peak_active, active_);
                r->state = REQ_RUNNING;
                r->times.admitted = now();
                admitted.push_back(r);
            }
        }
        for (Req* r : admitted) {
            const std::string e = admit(*r);
            // running: the device callback hands it to the pool, which may
            // already have finished it and a caller taken (freed) it, so it
            // is not touched here any more
            if (e.empty()) continue;
            // nothing of it runs any more (no hand-over was enqueued): free it here
            if (r->stream) cudaStreamSynchronize(r->stream);
            release(*r);
            std::lock_guard<std::mutex> lk(mu_);
            st_.bytes_in_use -= r->est_bytes;
            r->state = REQ_FAILED;
            r->err = e;
            r->times.finished = now();
            st_.failed++;
            active_--;
            if (active_ == 0 && busy_since_ >= 0) {
                st_.busy_seconds += now() - busy_since_;
                busy_since_ = -1;
            }
            cv_done_.notify_all();
        }
    }
}

ReqState Server::poll(uint64_t ticket, bool take, Result* out, ReqTimes* t, std::string* err) {
    std::lock_guard<std::mutex> lk(mu_);
    auto it = reqs_.find(ticket);
    if (it == reqs_.end()) {
        if (err) *err = "unknown ticket " + std::to_string(ticket);
        return REQ_FAILED;
    }
    Req& r = *it->second;
    if (t) *t = r.times;
    if (err) *err = r.err;
    const ReqState s = r.state;
    if (take && (s == REQ_DONE || s == REQ_FAILED || s == REQ_CANCELLED)) {
        if (s == REQ_DONE && out) *out = std::move(r.result);
        reqs_.erase(it);
    }
    return s;
}

ReqState Server::wait(uint64_t ticket, double timeout_s, Result* out, ReqTimes* t, std::string* err) {
    {
        std::unique_lock<std::mutex> lk(mu_);
        auto finished = [&] {
            auto it = reqs_.find(ticket);
            if (it == reqs_.end()) return true;
            const ReqState s = it->second->state;
            return s == REQ_DONE || s == REQ_FAILED || s == REQ_CANCELLED;
        };
        if (timeout_s < 0) cv_done_.wait(lk, finished);
        else cv_done_.wait_for(lk, std::chrono::duration<double>(timeout_s), finished);
    }
    return poll(ticket, true, out, t, err);
}

bool Server::cancel(uint64_t ticket) {
    std::lock_guard<std::mutex> lk(mu_);
    auto it = reqs_.find(ticket);
    if (it == reqs_.end()) return false;
    Req& r = *it->second;
    if (r.state == REQ_DONE || r.state == REQ_FAILED || r.state == REQ_CANCELLED) return false;
    r.cancel = true;  // queued: dropped at admission; running: its result is discarded
    cv_work_.notify_one();
    return true;
}

ServeStats Server::stats() const {
    std::lock_guard<std::mutex> lk(mu_);
    ServeStats s = st_;
    s.active = active_;
    s.queued = ready_.size() + placing_.size();
    if (busy_since_ >= 0) s.busy_seconds += now() - busy_since_;
    return s;
}

void Server::stop() {
    {
        std::lock_guard<std::mutex> lk(mu_);
        if (!started_) return;
        stopping_ = true;
        for (auto& kv : reqs_) kv.second->cancel = true;
    }
    cv_work_.notify_all();
    if (scheduler_.joinable()) scheduler_.join();
    // the simulations already on the device finish and the pool frees them
    {
        std::unique_lock<std::mutex> lk(mu_);
        cv_done_.wait(lk, [&] { return active_ == 0; });
    }
    cv_pool_.notify_all();
    for (auto& t : pool_) t.join();
    pool_.clear();
    std::lock_guard<std::mutex> lk(mu_);
    for (auto& kv : reqs_) {
        Req& r = *kv.second;
        if (r.state == REQ_PLACING || r.state == REQ_QUEUED || r.state == REQ_RUNNING) r.state = REQ_CANCELLED;
    }
    cv_done_.notify_all();
    started_ = false;
}

}  // namespace cpmhost
