// Header-only served form for C++ callers: the admission loop of the Python Server
// (poisson-surface-reconstruction-gpu_gb300/serve.py) over the C ABI's psr_submit /
// psr_poll.  The reference reconstructs one cloud per blocking call
// (mesh/PoissonReconstruction.cpp:195-245); here K handles, each with its own CUDA stream,
// are kept busy from one host thread: a request that arrives while others run is admitted
// as soon as a slot whose workspace takes it is free, and the slots' GPU work overlaps.
//
//   psr_gb300::Server srv(cfg, 8, 40ull << 30);        // slots bounded by a memory budget
//   psr_gb300::Server::Request r{points, options, &mesh};
//   srv.submit(&r);                                    // any time; arrival stamped here
//   while (srv.step() || srv.queued()) {}              // or interleave step() with other work
//   // r.status, r.mesh counts and outputs, r.latency_ms() once r.done is set
#pragma once

#include <cuda_runtime.h>

#include <chrono>
#include <deque>
#include <stdexcept>
#include <string>
#include <vector>

#include "psr.h"

namespace psr_gb300 {

class Server {
public:
    struct Request {
        psr_points points;        // host (pinned) or device arrays, alive until done
        psr_options options;
        psr_mesh* mesh;           // output buffers and capacities, filled on completion
        psr_status status = PSR_PENDING;
        bool done = false;
        double arrival = 0, admitted = 0, finished = 0;   // seconds on a steady clock
        double latency_ms() const { return 1000.0 * (finished - arrival); }
    };

    // `slots` handles of configuration `cfg`; with memory_budget > 0 only as many as their
    // device memory (psr_memory_bytes) fits, at least one.
    Server(const psr_config& cfg, int slots, size_t memory_budget = 0) : cfg_(cfg) {
        size_t used = 0;
        for (int k = 0; k < slots; ++k) {
            psr_handle* h = nullptr;
            psr_config c = cfg;
            c.concurrent_stages = 0;   // the slots overlap one another instead
            if (psr_create(&c, &h) != PSR_OK) {
                if (k == 0) throw std::runtime_error("psr_create failed");
                break;
            }
            size_t bytes = 0;
            psr_memory_bytes(h, &bytes);
            if (memory_budget && k > 0 && used + bytes > memory_budget) {
                psr_destroy(h);
                break;
            }
            used += bytes;
            cudaStream_t s = nullptr;
            if (cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking) != cudaSuccess) {
                psr_destroy(h);
                throw std::runtime_error("cudaStreamCreateWithFlags failed");
            }
            slots_.push_back(Slot{h, s, nullptr});
        }
    }
    ~Server() {
        for (auto& sl : slots_) {
            if (sl.req) psr_wait(sl.h);
            psr_destroy(sl.h);
            cudaStreamDestroy(sl.stream);
        }
    }
    Server(const Server&) = delete;
    Server& operator=(const Server&) = delete;

    void submit(Request* r) {
        r->arrival = now();
        r->done = false;
        r->status = PSR_PENDING;
        if (r->points.count > cfg_.max_points) {   // no slot takes it
            finish(r, PSR_OUT_OF_CAPACITY);
            return;
        }
        queue_.push_back(r);
    }

    // Collects finished slots and admits queued requests; returns the number of busy slots.
    int step() {
        int busy = 0;
        for (auto& sl : slots_) {
            if (sl.req) {
                const psr_status st = psr_poll(sl.h);
                if (st != PSR_PENDING) {
                    finish(sl.req, st);
                    sl.req = nullptr;
                }
            }
            if (!sl.req && !queue_.empty()) {
                Request* r = queue_.front();
                queue_.pop_front();
                r->admitted = now();
                const psr_status st = psr_submit(sl.h, &r->points, &r->options, r->mesh, sl.stream);
                if (st == PSR_OK) sl.req = r;
                else finish(r, st);
            }
            busy += sl.req != nullptr;
        }
        return busy;
    }

    size_t queued() const { return queue_.size(); }
    int slots() const { return (int)slots_.size(); }
    const std::vector<Request*>& completed() const { return done_; }

private:
    struct Slot {
        psr_handle* h;
        cudaStream_t stream;
        Request* req;
    };
    static double now() {
        return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
    }
    void finish(Request* r, psr_status st) {
        r->status = st;
        r->finished = now();
        r->done = true;
        done_.push_back(r);
    }
    psr_config cfg_;
    std::vector<Slot> slots_;
    std::deque<Request*> queue_;
    std::vector<Request*> done_;
};

}  // namespace psr_gb300
