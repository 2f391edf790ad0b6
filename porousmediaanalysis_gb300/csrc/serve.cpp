// Serving: a request loop with continuous batching under a device-memory budget.
//
// Requests (one host volume each) queue in arrival order. Each lane - a child context with
// its own stream, scratch cache and host thread - takes the oldest request as soon as it is
// free and the request fits the budget, so requests that arrive while others run are
// admitted as lanes and memory free up, and their kernels overlap on the device with those
// of the requests in flight. All intermediate fields of a request stay on the device from
// the first stage to the last; only the input and the requested outputs cross the bus.
//
// Memory accounting. A request's footprint is estimated as bytes-per-voxel x voxels, where
// bytes-per-voxel is the largest ratio of a finished request's scratch demand (the sum of the
// largest size each named buffer was asked for) to its voxel count seen so far (the fields and
// work buffers of every stage are linear in the voxel count). A lane keeps its scratch between
// requests; the reservation of a lane is max(its scratch, footprint of its request). A
// request is admitted only if the lanes' reservations stay within the budget; idle lanes
// give their scratch back first when the budget is short, and a lane whose scratch exceeds
// twice its next request's footprint trims it before starting. Requests that exceed the
// budget on their own are rejected with PMA_ERR_MEMORY.
#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <deque>
#include <map>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "pma_internal.h"

using pma::guarded;

struct pma_server {
    pma_ctx* parent = nullptr;
    pma_options options{};
    uint64_t budget = 0;
    struct Request {
        uint64_t ticket;
        const uint8_t* solid;
        pma_dims dims;
        pma_outputs* out;
        std::chrono::steady_clock::time_point arrival;
    };
    struct Result {
        bool done = false;
        int status = PMA_OK;
        double latency_ms = 0;
        std::string message;
    };
    struct Lane {
        pma_ctx* ctx = nullptr;
        bool busy = false;
        uint64_t reserved = 0;
        std::thread thread;
    };
    std::mutex mu;
    std::condition_variable cv_work;  // lanes wait for requests or budget
    std::condition_variable cv_done;  // waiters wait for results
    std::deque<Request> queue;
    std::map<uint64_t, Result> results;
    std::vector<Lane> lanes;
    uint64_t next_ticket = 1;
    double bytes_per_voxel = 192.0;  // raised by measurement
    bool stopping = false;
    pma_server_stats stats{};
};

namespace pma {
namespace {

uint64_t footprint(const pma_server* s, pma_dims d) {
    return static_cast<uint64_t>(s->bytes_per_voxel * static_cast<double>(voxels(d))) + (64ull << 20);
}

uint64_t reserved_total(const pma_server* s) {
    uint64_t t = 0;
    for (const pma_server::Lane& l : s->lanes) t += l.busy ? l.reserved : pma_ctx_scratch_bytes(l.ctx);
    return t;
}

void lane_loop(pma_server* s, size_t li) {
    pma_server::Lane& me = s->lanes[li];
    cudaSetDevice(me.ctx->device);
    std::unique_lock<std::mutex> lock(s->mu);
    while (true) {
        if (s->queue.empty()) {
            if (s->stopping) return;
            s->cv_work.wait(lock);
            continue;
        }
        pma_server::Request r = s->queue.front();
        const uint64_t need = footprint(s, r.dims);
        const uint64_t mine = pma_ctx_scratch_bytes(me.ctx);
        // give back scratch this lane holds far beyond what the request needs
        if (mine > 2 * need) pma_ctx_trim(me.ctx);
        uint64_t others = reserved_total(s) - pma_ctx_scratch_bytes(me.ctx);
        uint64_t want = std::max<uint64_t>(pma_ctx_scratch_bytes(me.ctx), need);
        if (others + want > s->budget) {
            for (pma_server::Lane& l : s->lanes)  // idle lanes release their scratch
                if (!l.busy && &l != &me) pma_ctx_trim(l.ctx);
            others = reserved_total(s) - pma_ctx_scratch_bytes(me.ctx);
        }
        if (others + want > s->budget) {
            bool any_busy = false;
            for (const pma_server::Lane& l : s->lanes) any_busy |= l.busy;
            if (any_busy) {  // wait for a lane to finish and free its reservation
                s->cv_work.wait(lock);
                continue;
            }
            // nothing else runs: the request alone exceeds the budget
            s->queue.pop_front();
            pma_server::Result& res = s->results[r.ticket];
            res.done = true;
            res.status = PMA_ERR_MEMORY;
            res.message = "pma_server: request of " + std::to_string(need) +
                          " estimated device bytes exceeds the memory budget";
            s->stats.rejected++;
            s->cv_done.notify_all();
            continue;
        }
        s->queue.pop_front();
        me.busy = true;
        me.reserved = want;
        uint32_t in_flight = 0;
        for (const pma_server::Lane& l : s->lanes) in_flight += l.busy ? 1u : 0u;
        s->stats.max_in_flight = std::max(s->stats.max_in_flight, in_flight);
        s->stats.peak_reserved_bytes = std::max<uint64_t>(s->stats.peak_reserved_bytes, reserved_total(s));
        lock.unlock();

        me.ctx->reset_demand();
        const int status = guarded([&] { run_pipeline_host(me.ctx, r.solid, r.dims, s->options, r.out); });
        std::string message;
        if (status != PMA_OK) {
            char buf[1024];
            pma_last_error(buf, sizeof(buf));
            message = buf;
        }
        const double ms =
            std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - r.arrival).count();
        const uint64_t used = me.ctx->demand_bytes;

        lock.lock();
        if (status == PMA_OK) {
            const double ratio = static_cast<double>(used) / static_cast<double>(voxels(r.dims));
            if (voxels(r.dims) >= (1u << 20)) s->bytes_per_voxel = std::max(s->bytes_per_voxel, ratio);
            s->stats.completed++;
        } else {
            s->stats.failed++;
        }
        me.busy = false;
        me.reserved = 0;
        pma_server::Result& res = s->results[r.ticket];
        res.done = true;
        res.status = status;
        res.latency_ms = ms;
        res.message = message;
        s->cv_done.notify_all();
        s->cv_work.notify_all();
    }
}

}  // namespace
}  // namespace pma

extern "C" {

int pma_server_create(pma_ctx* ctx, const pma_server_config* cfg, pma_server** out) {
    return guarded([&] {
        PMA_REQUIRE(ctx && out, PMA_ERR_ARGUMENT, "pma_server_create: null argument");
        PMA_CUDA(cudaSetDevice(ctx->device));
        pma_server* s = new pma_server;
        s->parent = ctx;
        s->options = pma_options{PMA_D3Q27, 1, 1, 0};
        int lanes = 8;
        s->budget = 120ull << 30;
        if (cfg) {
            s->options = cfg->options;
            if (cfg->lanes) lanes = cfg->lanes;
            if (cfg->memory_budget) s->budget = cfg->memory_budget;
        }
        if (lanes < 1 || lanes > 64) {
            delete s;
            throw pma::Error(PMA_ERR_ARGUMENT, "pma_server_create: lanes must be 1..64");
        }
        s->lanes.resize(static_cast<size_t>(lanes));
        try {
            for (pma_server::Lane& l : s->lanes) {
                pma_ctx* c = nullptr;
                PMA_REQUIRE(pma_ctx_create(ctx->device, &c) == PMA_OK, PMA_ERR_CUDA,
                            "pma_server_create: lane context");
                c->blocking_sync = true;
                c->limits = ctx->limits;
                c->reference_throat_ids = ctx->reference_throat_ids;
                l.ctx = c;
            }
        } catch (...) {
            for (pma_server::Lane& l : s->lanes) pma_ctx_destroy(l.ctx);
            delete s;
            throw;
        }
        try {
            for (size_t i = 0; i < s->lanes.size(); ++i) s->lanes[i].thread = std::thread(pma::lane_loop, s, i);
        } catch (...) {  // stop the lanes already started before giving the server up
            {
                std::lock_guard<std::mutex> lock(s->mu);
                s->stopping = true;
                s->cv_work.notify_all();
            }
            for (pma_server::Lane& l : s->lanes)
                if (l.thread.joinable()) l.thread.join();
            for (pma_server::Lane& l : s->lanes) pma_ctx_destroy(l.ctx);
            delete s;
            throw pma::Error(PMA_ERR_CUDA, "pma_server_create: could not start the lane threads");
        }
        *out = s;
    });
}

int pma_server_submit(pma_server* s, const uint8_t* h_solid, pma_dims dims, pma_outputs* out,
                      uint64_t* ticket) {
    return guarded([&] {
        PMA_REQUIRE(s && h_solid && out && ticket, PMA_ERR_ARGUMENT, "pma_server_submit: null argument");
        pma::check_dims(dims);
        std::lock_guard<std::mutex> lock(s->mu);
        PMA_REQUIRE(!s->stopping, PMA_ERR_ARGUMENT, "pma_server_submit: server is stopping");
        const uint64_t t = s->next_ticket++;
        s->results[t] = pma_server::Result{};
        s->queue.push_back(pma_server::Request{t, h_solid, dims, out, std::chrono::steady_clock::now()});
        s->stats.submitted++;
        *ticket = t;
        s->cv_work.notify_all();
    });
}

int pma_server_wait(pma_server* s, uint64_t ticket, int64_t timeout_ms, int* status, double* latency_ms) {
    std::string message;
    int result = PMA_OK;
    const int rc = guarded([&] {
        PMA_REQUIRE(s && status, PMA_ERR_ARGUMENT, "pma_server_wait: null argument");
        std::unique_lock<std::mutex> lock(s->mu);
        auto it = s->results.find(ticket);
        PMA_REQUIRE(it != s->results.end(), PMA_ERR_ARGUMENT, "pma_server_wait: unknown ticket");
        auto ready = [&] { return s->results[ticket].done; };
        if (timeout_ms < 0) {
            s->cv_done.wait(lock, ready);
        } else if (!s->cv_done.wait_for(lock, std::chrono::milliseconds(timeout_ms), ready)) {
            throw pma::Error(PMA_ERR_LIMIT, "pma_server_wait: timed out");
        }
        pma_server::Result r = s->results[ticket];
        s->results.erase(ticket);
        *status = r.status;
        if (latency_ms) *latency_ms = r.latency_ms;
        message = r.message;
        result = r.status;
    });
    if (rc != PMA_OK) return rc;
    if (result != PMA_OK) pma::set_last_error(message);
    return PMA_OK;
}

int pma_server_get_stats(pma_server* s, pma_server_stats* out) {
    return guarded([&] {
        PMA_REQUIRE(s && out, PMA_ERR_ARGUMENT, "pma_server_get_stats: null argument");
        std::lock_guard<std::mutex> lock(s->mu);
        *out = s->stats;
        out->queued = s->queue.size();
        out->resident_bytes = 0;
        for (const pma_server::Lane& l : s->lanes) out->resident_bytes += pma_ctx_scratch_bytes(l.ctx);
        out->bytes_per_voxel = s->bytes_per_voxel;
    });
}

int pma_server_destroy(pma_server* s) {
    if (!s) return PMA_OK;
    return guarded([&] {
        {
            std::lock_guard<std::mutex> lock(s->mu);
            s->stopping = true;
            s->cv_work.notify_all();
        }
        for (pma_server::Lane& l : s->lanes)
            if (l.thread.joinable()) l.thread.join();
        for (pma_server::Lane& l : s->lanes) pma_ctx_destroy(l.ctx);
        delete s;
    });
}

}  // extern "C"
