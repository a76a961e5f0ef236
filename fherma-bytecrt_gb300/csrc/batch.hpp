// Batched form: many products of uneven points (N, W, q) in one CUDA graph.
//
// The reference batches B products of one point over four pipelined slots
// (native-batched/solve.cu:17-34, :200-244).  Here a Batch collects products
// of any registered points, groups them by (geometry, q), and captures the
// launch chains of every group, back to back on one stream, into one CUDA
// graph; each run() is one graph launch.  Contexts of the same geometry share
// the device tables (twiddles, twists, encode B operand); contexts of the
// same q share the CRT weights.  The products of a group run as chains of
// the context's group size on one shared workspace sized for the largest
// chain.
#pragma once

#include <cstdint>
#include <map>
#include <memory>
#include <vector>

#include "engine.hpp"

namespace bcg {

// Contexts keyed by point on one device (created on first use).
class PointRegistry {
public:
    explicit PointRegistry(int device) : device_(device) {}
    Context& get(uint32_t N, uint32_t W, uint32_t L, const uint32_t* q);
    int device() const { return device_; }
    size_t size() const { return ctxs_.size(); }

private:
    int device_;
    std::map<std::vector<uint32_t>, std::unique_ptr<Context>> ctxs_;
};

// Per-stage CUDA events recorded inside a captured graph (external event
// records, so every replay records them again).  Stages of every k-th chain
// are bracketed; after a replay the events hold that replay's times.
class GraphTimer : public StageTimer {
public:
    ~GraphTimer() override;
    void reset(uint32_t every);
    void next_chain() { timing_ = every_ != 0 && (chains_++ % every_) == 0; }
    void begin(int stage, cudaStream_t st) override;
    void end(cudaStream_t st) override;
    // Summed stage times of the last replay, launches and timed launches per
    // replay, per stage.
    void read(double* ms, uint64_t* launches, uint64_t* timed) const;
    void counts(uint64_t* launches) const {
        for (int s = 0; s < Context::kStages; ++s) launches[s] = launches_[s];
    }

private:
    struct Mark { int stage; cudaEvent_t begin, end; };
    std::vector<Mark> marks_;
    uint64_t launches_[Context::kStages] = {};
    uint32_t every_ = 0;
    uint64_t chains_ = 0;
    bool timing_ = false;
    bool open_ = false;
};

class Batch {
public:
    explicit Batch(int device);
    ~Batch();
    Batch(const Batch&) = delete;
    Batch& operator=(const Batch&) = delete;

    // `count` products of one point: a, b, c device buffers of [count][N][L]
    // words, 16-byte aligned.  Adding invalidates the captured graph.
    void add(uint32_t N, uint32_t W, uint32_t L, const uint32_t* q, const uint32_t* a, const uint32_t* b,
             uint32_t* c, uint32_t count);
    // Captures the graph if needed, then launches it on `st`.
    void run(cudaStream_t st);
    // Waits for the last run and reports a device-side wait timeout.
    void synchronize(cudaStream_t st);
    // Stage timing inside the graph: 0 off, k times every k-th chain (recaptures).
    void set_profiling(uint32_t every);
    // Launch chains alternate over `lanes` parallel branches of the graph (1 or
    // 2), each with its own workspace, so one chain's kernels can fill the
    // tail of another's (recaptures).  0 (the default) picks two branches when
    // the batch holds several (geometry, q) groups and one otherwise: measured
    // at N=65536/W=1747, two branches made the one-group B=128 batch 0.9%
    // slower and the six-group 96-product batch 1.8% faster.
    void set_lanes(uint32_t lanes);
    uint32_t lanes() const { return lanes_ ? lanes_ : (groups_.size() > 1 ? 2u : 1u); }
    void read_profile(double* ms, uint64_t* launches, uint64_t* timed, uint64_t* chains);
    // Launches per stage and chains of one run (captures the graph if needed).
    void read_counts(uint64_t* launches, uint64_t* chains);

    uint32_t groups() const { return uint32_t(groups_.size()); }
    uint64_t products() const { return products_; }

private:
    struct Entry { const uint32_t* a; const uint32_t* b; uint32_t* c; uint32_t count; };
    struct Group { Context* ctx; std::vector<Entry> entries; };
    void capture();
    void release_graph();

    PointRegistry reg_;
    std::vector<Group> groups_;
    uint64_t products_ = 0;
    DeviceBuffer ws_, ws2_;
    cudaStream_t capture_stream_ = nullptr, lane_stream_ = nullptr;
    cudaEvent_t fork_ = nullptr, join_ = nullptr;
    uint32_t lanes_ = 0;
    cudaGraph_t graph_ = nullptr;
    cudaGraphExec_t exec_ = nullptr;
    cudaStream_t last_stream_ = nullptr;   // stream of the last graph launch
    uint32_t profile_every_ = 0;
    GraphTimer timer_;
    uint64_t chains_ = 0;   // per run
};

}  // namespace bcg
