// Batched form: uneven products grouped by point, one CUDA graph per batch.
#include "batch.hpp"

#include <algorithm>

namespace bcg {

Context& PointRegistry::get(uint32_t N, uint32_t W, uint32_t L, const uint32_t* q) {
    if (!q) throw std::invalid_argument("null modulus");
    std::vector<uint32_t> key{N, W, L};
    key.insert(key.end(), q, q + L);
    auto it = ctxs_.find(key);
    if (it != ctxs_.end()) return *it->second;
    auto ctx = std::make_unique<Context>(N, W, L, q, device_);
    Context& ref = *ctx;
    ctxs_.emplace(std::move(key), std::move(ctx));
    return ref;
}

GraphTimer::~GraphTimer() { reset(0); }

void GraphTimer::reset(uint32_t every) {
    for (const Mark& m : marks_) { cudaEventDestroy(m.begin); cudaEventDestroy(m.end); }
    marks_.clear();
    for (auto& l : launches_) l = 0;
    every_ = every;
    chains_ = 0;
    timing_ = open_ = false;
}

void GraphTimer::begin(int stage, cudaStream_t st) {
    ++launches_[stage];
    open_ = false;
    if (!timing_) return;
    Mark m{stage, nullptr, nullptr};
    check(cudaEventCreate(&m.begin), "profile event");
    check(cudaEventCreate(&m.end), "profile event");
    marks_.push_back(m);
    // External records: nodes of the captured graph, recorded again on every replay.
    check(cudaEventRecordWithFlags(m.begin, st, cudaEventRecordExternal), "profile event");
    open_ = true;
}

void GraphTimer::end(cudaStream_t st) {
    if (!open_) return;
    check(cudaEventRecordWithFlags(marks_.back().end, st, cudaEventRecordExternal), "profile event");
    open_ = false;
}

void GraphTimer::read(double* ms, uint64_t* launches, uint64_t* timed) const {
    for (int s = 0; s < Context::kStages; ++s) { ms[s] = 0; timed[s] = 0; launches[s] = launches_[s]; }
    for (const Mark& m : marks_) {
        check(cudaEventSynchronize(m.end), "profile event");
        float t = 0;
        check(cudaEventElapsedTime(&t, m.begin, m.end), "profile elapsed");
        ms[m.stage] += t;
        ++timed[m.stage];
    }
}

Batch::Batch(int device) : reg_(device) {
    check(cudaSetDevice(device), "select device");
    check(cudaStreamCreateWithFlags(&capture_stream_, cudaStreamNonBlocking), "stream");
    check(cudaStreamCreateWithFlags(&lane_stream_, cudaStreamNonBlocking), "stream");
    check(cudaEventCreateWithFlags(&fork_, cudaEventDisableTiming), "event");
    check(cudaEventCreateWithFlags(&join_, cudaEventDisableTiming), "event");
}

Batch::~Batch() {
    release_graph();
    if (fork_) cudaEventDestroy(fork_);
    if (join_) cudaEventDestroy(join_);
    if (lane_stream_) cudaStreamDestroy(lane_stream_);
    if (capture_stream_) cudaStreamDestroy(capture_stream_);
}

void Batch::release_graph() {
    // A launched graph may still run on the caller's stream: let it finish
    // before its executable or its workspace go away.
    if (last_stream_) { cudaStreamSynchronize(last_stream_); last_stream_ = nullptr; }
    if (exec_) { cudaGraphExecDestroy(exec_); exec_ = nullptr; }
    if (graph_) { cudaGraphDestroy(graph_); graph_ = nullptr; }
}

void Batch::add(uint32_t N, uint32_t W, uint32_t L, const uint32_t* q, const uint32_t* a, const uint32_t* b,
                uint32_t* c, uint32_t count) {
    if (count == 0) return;
    if (!a || !b || !c) throw std::invalid_argument("null buffer");
    if ((reinterpret_cast<uintptr_t>(a) | reinterpret_cast<uintptr_t>(b) | reinterpret_cast<uintptr_t>(c)) & 15)
        throw std::invalid_argument("operand device pointers must be 16-byte aligned");
    Context& ctx = reg_.get(N, W, L, q);
    auto it = std::find_if(groups_.begin(), groups_.end(), [&](const Group& g) { return g.ctx == &ctx; });
    if (it == groups_.end()) {
        groups_.push_back(Group{&ctx, {}});
        it = groups_.end() - 1;
    }
    it->entries.push_back(Entry{a, b, c, count});
    products_ += count;
    release_graph();
}

void Batch::set_lanes(uint32_t lanes) {
    if (lanes > 2) throw std::invalid_argument("lanes must be 0 (automatic), 1 or 2");
    if (lanes == lanes_) return;
    lanes_ = lanes;
    release_graph();
}

void Batch::set_profiling(uint32_t every) {
    if (every == profile_every_) return;
    profile_every_ = every;
    release_graph();
}

void Batch::capture() {
    // One workspace, reused by every chain in stream order.
    size_t ws_bytes = 0;
    for (const Group& g : groups_)
        for (const Entry& e : g.entries)
            ws_bytes = std::max(ws_bytes, size_t(std::min(e.count, g.ctx->group())) *
                                              g.ctx->workspace_bytes_per_product());
    if (ws_bytes > ws_.bytes) ws_.allocate(ws_bytes);   // release_graph() waited for the last launch
    const uint32_t lanes = this->lanes();
    if (lanes > 1 && ws_bytes > ws2_.bytes) ws2_.allocate(ws_bytes);
    timer_.reset(profile_every_);
    chains_ = 0;
    check(cudaStreamBeginCapture(capture_stream_, cudaStreamCaptureModeThreadLocal), "graph capture");
    try {
        if (lanes > 1) {   // fork the second branch off the capture stream
            check(cudaEventRecord(fork_, capture_stream_), "graph fork");
            check(cudaStreamWaitEvent(lane_stream_, fork_, 0), "graph fork");
        }
        for (const Group& g : groups_) {
            Context& ctx = *g.ctx;
            const size_t cw = ctx.coeff_words();
            const uint32_t chunk = ctx.group();
            for (const Entry& e : g.entries) {
                for (uint32_t done = 0; done < e.count; done += chunk) {
                    const uint32_t n = std::min(chunk, e.count - done);
                    const bool second = lanes > 1 && (chains_ & 1);
                    timer_.next_chain();
                    ctx.chain(e.a + done * cw, e.b + done * cw, e.c + done * cw, n,
                              (second ? ws2_ : ws_).as<uint32_t>(), second ? lane_stream_ : capture_stream_, &timer_);
                    ++chains_;
                }
            }
        }
        if (lanes > 1) {   // join it back
            check(cudaEventRecord(join_, lane_stream_), "graph join");
            check(cudaStreamWaitEvent(capture_stream_, join_, 0), "graph join");
        }
    } catch (...) {
        cudaGraph_t partial = nullptr;
        cudaStreamEndCapture(capture_stream_, &partial);
        if (partial) cudaGraphDestroy(partial);
        throw;
    }
    check(cudaStreamEndCapture(capture_stream_, &graph_), "graph capture");
    check(cudaGraphInstantiate(&exec_, graph_, 0), "graph instantiate");
}

void Batch::run(cudaStream_t st) {
    if (groups_.empty()) return;
    if (!exec_) capture();
    st = st ? st : capture_stream_;
    if (last_stream_ && last_stream_ != st) check(cudaStreamSynchronize(last_stream_), "stream synchronize");
    check(cudaGraphLaunch(exec_, st), "graph launch");
    last_stream_ = st;
}

void Batch::synchronize(cudaStream_t st) {
    check(cudaStreamSynchronize(st ? st : capture_stream_), "stream synchronize");
    for (const Group& g : groups_) g.ctx->check_status();
}

void Batch::read_profile(double* ms, uint64_t* launches, uint64_t* timed, uint64_t* chains) {
    timer_.read(ms, launches, timed);
    *chains = chains_;
}

}  // namespace bcg

namespace bcg {

void Batch::read_counts(uint64_t* launches, uint64_t* chains) {
    if (!exec_ && !groups_.empty()) capture();
    timer_.counts(launches);
    *chains = chains_;
}

}  // namespace bcg
