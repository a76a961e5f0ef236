// Served form: a request loop with continuous batching on one GPU.
//
// Callers submit products of any registered point (N, W, q) with host
// buffers.  A scheduler thread forms batches (scheduler.hpp: oldest request
// first, same point and resident operand, up to the point's batch limit,
// admitted only if the batch's device bytes fit the free memory budget) and
// issues each one on a free slot stream: H2D copies, the launch chain, D2H
// copies, all stream-ordered, with the batch's device memory taken from a
// stream-ordered pool.  Several slots are in flight at once, so requests
// that arrive while others run join the next batch as soon as a slot and
// memory free up, and copies of one batch overlap kernels of another.  A
// completion thread retires batches as their events complete and records
// each request's latency (submission to completion on the host clock).
//
// Resident operands: add_operand() encodes an operand once and keeps its
// forward-transformed residue planes on the device; requests naming it skip
// its encode and forward transform (Context::multiply_spectral_device).
//
// No counterpart in the reference, which has no server (one product or one
// fixed batch per fherma_run call, native-smoke/solve.cu:506-525,
// native-batched/solve.cu:200-244).
#pragma once

#include <condition_variable>
#include <cstdint>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <unordered_map>
#include <vector>

#include "batch.hpp"
#include "engine.hpp"
#include "scheduler.hpp"

namespace bcg {

struct ServerOptions {
    uint64_t memory_bytes = 0;   // device memory budget; 0: 80% of the free memory at creation
    uint32_t slots = 3;          // batches in flight
    uint32_t max_batch = 0;      // products per batch; 0: the point's context group
    uint32_t max_queue = 1u << 16;   // waiting requests before submit() is refused
};

struct ServerStats {
    uint64_t submitted = 0, completed = 0, failed = 0, rejected = 0;
    uint64_t batches = 0, batched_products = 0, operands = 0;
    uint64_t memory_budget = 0, memory_used = 0, memory_peak = 0;
};

struct RequestResult {
    int status = 0;              // BCG_OK or a BCG_ERR_* code
    double latency_ms = 0;
    std::string error;
};

class Server {
public:
    Server(int device, const ServerOptions& opt);
    ~Server();   // finishes every submitted request, then stops
    Server(const Server&) = delete;
    Server& operator=(const Server&) = delete;

    uint32_t add_point(uint32_t N, uint32_t W, uint32_t L, const uint32_t* q);
    // Encodes and forward-transforms `a` (host buffer, [N][L]) once; synchronous.
    uint64_t add_operand(uint32_t point, const uint32_t* a);
    void remove_operand(uint64_t operand);
    // c = a * b for `point`; a == nullptr with operand != 0 uses the resident
    // operand.  Host buffers stay owned by the caller and must stay valid
    // (c unread) until wait() returns for the request.  Throws Busy when the
    // queue is full or the product can never fit the memory budget.
    uint64_t submit(uint32_t point, const uint32_t* a, uint64_t operand, const uint32_t* b, uint32_t* c);
    // Waits for a request (timeout_ms 0: no limit).  False on timeout.
    bool wait(uint64_t id, uint32_t timeout_ms, RequestResult* out);
    // Waits until every submitted request has completed.
    void drain();
    ServerStats stats() const;

private:
    struct Point {
        Context* ctx;
        uint32_t max_batch;
    };
    struct Operand {
        uint32_t point;
        DeviceBuffer planes;
    };
    struct Record {
        sched::Request req;
        const uint32_t* a;
        const uint32_t* b;
        uint32_t* c;
        bool done = false;
        RequestResult result;
    };
    struct Inflight {
        sched::Batch batch;
        Context* ctx = nullptr;
        const uint32_t* planes = nullptr;   // resident operand's spectral planes, or null
        std::vector<const uint32_t*> a, b;
        std::vector<uint32_t*> c;
        int slot = -1;
        void* mem = nullptr;
        cudaEvent_t done = nullptr;
        bool issued = false;
        int error_status = 0;   // BCG_* code if issuing the batch failed
        std::string error;
    };

    uint64_t product_bytes(const Point& p, bool resident) const;
    void schedule_loop();
    void complete_loop();
    void issue(Inflight& f);
    void retire(Inflight& f, int status, const std::string& error);
    static double now();

    int device_;
    ServerOptions opt_;
    PointRegistry reg_;
    std::vector<Point> points_;
    std::map<uint64_t, Operand> operands_;
    uint64_t next_operand_ = 1, next_request_ = 1;

    mutable std::mutex mu_;
    std::mutex launch_mu_;   // serialises launches on the contexts
    std::condition_variable cv_sched_, cv_done_;
    sched::Queue queue_;
    sched::Admission adm_;
    std::unordered_map<uint64_t, Record> records_;
    std::vector<std::unique_ptr<Inflight>> inflight_;
    std::vector<cudaStream_t> streams_;
    std::vector<bool> slot_busy_;
    std::vector<cudaEvent_t> event_pool_;
    cudaMemPool_t pool_ = nullptr;
    ServerStats stats_;
    uint64_t pending_ = 0;   // submitted and not yet completed
    bool stop_ = false, scheduler_done_ = false;
    std::thread scheduler_, completer_;
};

}  // namespace bcg
