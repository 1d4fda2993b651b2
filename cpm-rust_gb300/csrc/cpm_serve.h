// Serving loop: continuous batching of whole simulations on one GPU.
//
// Requests (a configuration plus its run window) are placed on a host
// thread pool, then admitted to the device in submission order while the
// number of active simulations stays under `max_active` and their device
// bytes under the HBM budget. An admitted simulation gets its own stream,
// its state is uploaded with stream-ordered allocations (which, unlike
// cudaMalloc, do not serialise the other streams), and its whole run window
// is enqueued at once: the shared-memory-resident sweep as a one-CTA launch
// that keeps the lattice in one SM's shared memory for the whole window,
// larger lattices as tiled launches with a capped grid. The hardware
// schedules these launches side by side, so simulations of different sizes
// overlap and none waits for another's sampling interval. A host callback
// at the end of each stream hands the simulation to the pool, which reads
// it back, builds its run result and frees it; the freed slot and bytes
// admit the next request. A simulation's trajectory depends only on its
// configuration and seed (the sweep path is chosen from its own size, draws
// are keyed by (seed, MCS, site), and the tiled sweep's result does not
// depend on its grid), so each result is the same alone, in any mix and
// from `run`.
#pragma once
#include <cuda_runtime.h>

#include <condition_variable>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "cpm_engine.h"
#include "cpm_host.h"

namespace cpmhost {

struct ServeOptions {
    uint64_t hbm_budget = 150ull << 30;  // device bytes the admitted simulations may hold
    int max_active = 128;                // simulations on the device at once
    int placement_threads = 0;           // host threads for placements and read-backs (0: automatic)
    int tiled_grid_cap = 64;             // CTAs of one tiled simulation (leaves SMs to the others)
};

enum ReqState { REQ_PLACING = 0, REQ_QUEUED = 1, REQ_RUNNING = 2, REQ_DONE = 3, REQ_FAILED = 4, REQ_CANCELLED = 5 };

struct ReqTimes {
    double submitted = 0, admitted = 0, finished = 0;  // seconds since the server started
    double device_done = 0;                            // when its device work ended
    uint64_t device_bytes = 0;
};

struct ServeStats {
    uint64_t submitted = 0, completed = 0, failed = 0, cancelled = 0, launched = 0;
    uint64_t active = 0, queued = 0, peak_active = 0;
    uint64_t bytes_in_use = 0, peak_bytes = 0;
    double busy_seconds = 0;  // wall time with at least one simulation on the device
};

class Server {
   public:
    Server();
    ~Server();
    Server(const Server&) = delete;
    Server& operator=(const Server&) = delete;

    std::string start(const ServeOptions& o);
    // Enqueues a validated configuration; the placement runs on the pool.
    std::string submit(const Config& c, const ReadoutOptions& ro, uint64_t& ticket);
    // State of a ticket; for REQ_DONE with take, the result moves to *out
    // and the ticket is forgotten.
    ReqState poll(uint64_t ticket, bool take, Result* out, ReqTimes* t, std::string* err);
    // Blocks until the ticket is done, failed or cancelled, or timeout_s
    // elapses (negative: no limit); then as poll(take = true).
    ReqState wait(uint64_t ticket, double timeout_s, Result* out, ReqTimes* t, std::string* err);
    bool cancel(uint64_t ticket);
    ServeStats stats() const;
    // Cancels what has not finished, stops the threads and frees the device.
    void stop();

   private:
    struct Req;
    void pool_loop();
    void scheduler_loop();
    std::string admit(Req& r);
    void finish(Req* r);
    void release(Req& r);
    double now() const;
    static void CUDART_CB device_done(void* ctx);

    ServeOptions opt_;
    int device_ = 0;
    mutable std::mutex mu_;
    std::condition_variable cv_work_, cv_pool_, cv_done_;
    bool stopping_ = false, started_ = false;
    uint64_t next_ticket_ = 1;
    std::map<uint64_t, std::unique_ptr<Req>> reqs_;
    std::deque<Req*> placing_, finishing_;
    std::map<uint64_t, Req*> ready_;  // placed, waiting for admission (ticket order)
    size_t active_ = 0;
    std::vector<std::thread> pool_;
    std::thread scheduler_;
    ServeStats st_;
    double t0_ = 0, busy_since_ = -1;
};

}  // namespace cpmhost
