// Served form: continuous batching over slot streams (see server.hpp).
#include "server.hpp"

#include <chrono>

#include "../../include/bytecrt_gb300.h"

namespace bcg {

double Server::now() {
    using namespace std::chrono;
    return duration<double>(steady_clock::now().time_since_epoch()).count();
}

Server::Server(int device, const ServerOptions& opt)
    : device_(device), opt_(opt), reg_(device), adm_(0) {
    if (opt_.slots == 0 || opt_.slots > 16) throw std::invalid_argument("slots must be in [1, 16]");
    check(cudaSetDevice(device_), "select device");
    uint64_t budget = opt_.memory_bytes;
    if (budget == 0) {
        size_t free_b = 0, total_b = 0;
        check(cudaMemGetInfo(&free_b, &total_b), "memory info");
        budget = uint64_t(free_b) / 5 * 4;
    }
    adm_ = sched::Admission(budget);
    stats_.memory_budget = budget;
    cudaMemPoolProps props{};
    props.allocType = cudaMemAllocationTypePinned;
    props.location.type = cudaMemLocationTypeDevice;
    props.location.id = device_;
    check(cudaMemPoolCreate(&pool_, &props), "memory pool");
    uint64_t keep = UINT64_MAX;   // freed batch memory stays in the pool for the next batch
    check(cudaMemPoolSetAttribute(pool_, cudaMemPoolAttrReleaseThreshold, &keep), "memory pool");
    streams_.resize(opt_.slots);
    for (auto& s : streams_) check(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking), "stream");
    slot_busy_.assign(opt_.slots, false);
    scheduler_ = std::thread([this] { schedule_loop(); });
    completer_ = std::thread([this] { complete_loop(); });
}

Server::~Server() {
    {
        std::lock_guard<std::mutex> lk(mu_);
        stop_ = true;
    }
    cv_sched_.notify_all();
    cv_done_.notify_all();
    if (scheduler_.joinable()) scheduler_.join();
    if (completer_.joinable()) completer_.join();
    cudaSetDevice(device_);
    for (auto s : streams_) { cudaStreamSynchronize(s); cudaStreamDestroy(s); }
    for (auto e : event_pool_) cudaEventDestroy(e);
    operands_.clear();
    if (pool_) cudaMemPoolDestroy(pool_);
}

uint32_t Server::add_point(uint32_t N, uint32_t W, uint32_t L, const uint32_t* q) {
    std::lock_guard<std::mutex> launch(launch_mu_);
    std::lock_guard<std::mutex> lk(mu_);
    Context& ctx = reg_.get(N, W, L, q);
    for (size_t i = 0; i < points_.size(); ++i)
        if (points_[i].ctx == &ctx) return uint32_t(i + 1);
    points_.push_back(Point{&ctx, opt_.max_batch ? opt_.max_batch : ctx.group()});
    return uint32_t(points_.size());
}

uint64_t Server::product_bytes(const Point& p, bool resident) const {
    const uint64_t cw = p.ctx->coeff_words(), pw = p.ctx->plane_words();
    return 4 * ((resident ? 0 : cw) + 2 * cw + (resident ? pw : 2 * pw));
}

uint64_t Server::add_operand(uint32_t point, const uint32_t* a) {
    if (!a) throw std::invalid_argument("null operand");
    Context* ctx;
    uint64_t bytes;
    {
        std::lock_guard<std::mutex> lk(mu_);
        if (point == 0 || point > points_.size()) throw std::invalid_argument("unknown point");
        ctx = points_[point - 1].ctx;
        bytes = ctx->plane_words() * 4;
        if (!adm_.fits(bytes)) throw Busy("no device memory left in the budget for a resident operand");
        adm_.take(bytes);
    }
    Operand op;
    op.point = point;
    try {
        check(cudaSetDevice(device_), "select device");
        op.planes.allocate(bytes);
        DeviceBuffer x;
        x.allocate(ctx->coeff_words() * 4);
        check(cudaMemcpy(x.ptr, a, ctx->coeff_words() * 4, cudaMemcpyHostToDevice), "operand copy");
        std::lock_guard<std::mutex> launch(launch_mu_);
        ctx->forward_spectral(x.as<uint32_t>(), op.planes.as<uint32_t>(), ctx->stream());
        ctx->synchronize(ctx->stream());
    } catch (...) {
        std::lock_guard<std::mutex> lk(mu_);
        adm_.give(bytes);
        throw;
    }
    std::lock_guard<std::mutex> lk(mu_);
    const uint64_t id = next_operand_++;
    operands_.emplace(id, std::move(op));
    ++stats_.operands;
    return id;
}

void Server::remove_operand(uint64_t operand) {
    std::unique_lock<std::mutex> lk(mu_);
    if (operands_.find(operand) == operands_.end()) throw std::invalid_argument("unknown operand");
    // Wait until no waiting or running request reads its planes; submit()
    // needs the lock, so none can name it between this check and the erase.
    cv_done_.wait(lk, [&] {
        for (const auto& kv : records_)
            if (!kv.second.done && kv.second.req.operand == operand) return false;
        return true;
    });
    auto it = operands_.find(operand);
    adm_.give(it->second.planes.bytes);
    operands_.erase(it);
    --stats_.operands;
}

uint64_t Server::submit(uint32_t point, const uint32_t* a, uint64_t operand, const uint32_t* b, uint32_t* c) {
    std::lock_guard<std::mutex> lk(mu_);
    if (point == 0 || point > points_.size()) throw std::invalid_argument("unknown point");
    if (!b || !c) throw std::invalid_argument("null buffer");
    if (operand != 0) {
        auto it = operands_.find(operand);
        if (it == operands_.end()) throw std::invalid_argument("unknown operand");
        if (it->second.point != point) throw std::invalid_argument("operand belongs to another point");
        if (a) throw std::invalid_argument("give either a or a resident operand, not both");
    } else if (!a) {
        throw std::invalid_argument("null buffer");
    }
    const uint64_t bytes = product_bytes(points_[point - 1], operand != 0);
    if (bytes > adm_.budget()) {
        ++stats_.rejected;
        throw Busy("product needs " + std::to_string(bytes) + " device bytes; the budget is " +
                   std::to_string(adm_.budget()));
    }
    if (queue_.size() >= opt_.max_queue) {
        ++stats_.rejected;
        throw Busy("request queue is full");
    }
    const uint64_t id = next_request_++;
    Record r;
    r.req = sched::Request{id, point, operand, bytes, now()};
    r.a = a; r.b = b; r.c = c;
    records_.emplace(id, r);
    queue_.push(r.req);
    ++stats_.submitted;
    ++pending_;
    cv_sched_.notify_one();
    return id;
}

bool Server::wait(uint64_t id, uint32_t timeout_ms, RequestResult* out) {
    std::unique_lock<std::mutex> lk(mu_);
    auto it = records_.find(id);
    if (it == records_.end()) throw std::invalid_argument("unknown request id");
    auto done = [&] { return records_.at(id).done; };
    if (timeout_ms == 0) cv_done_.wait(lk, done);
    else if (!cv_done_.wait_for(lk, std::chrono::milliseconds(timeout_ms), done)) return false;
    *out = records_.at(id).result;
    records_.erase(id);
    return true;
}

void Server::drain() {
    std::unique_lock<std::mutex> lk(mu_);
    cv_done_.wait(lk, [&] { return pending_ == 0; });
}

ServerStats Server::stats() const {
    std::lock_guard<std::mutex> lk(mu_);
    ServerStats s = stats_;
    s.memory_used = adm_.used();
    s.memory_peak = adm_.peak();
    return s;
}

void Server::schedule_loop() {
    cudaSetDevice(device_);
    std::unique_lock<std::mutex> lk(mu_);
    auto free_slot = [&]() -> int {
        for (size_t i = 0; i < slot_busy_.size(); ++i)
            if (!slot_busy_[i]) return int(i);
        return -1;
    };
    auto limit = [&](uint32_t point) { return points_[point - 1].max_batch; };
    for (;;) {
        cv_sched_.wait(lk, [&] { return (stop_ && queue_.empty()) || (!queue_.empty() && free_slot() >= 0); });
        if (queue_.empty()) break;   // stopping, nothing left
        const int slot = free_slot();
        auto f = std::make_unique<Inflight>();
        if (!queue_.next(adm_, limit, &f->batch)) {
            if (inflight_.empty()) {
                // Nothing running will free memory: resident operands hold the
                // rest of the budget.  Refuse the head instead of waiting forever.
                const sched::Request head = queue_.pop();
                Record& r = records_.at(head.id);
                r.done = true;
                r.result.status = BCG_ERR_BUSY;
                r.result.error = "resident operands leave too little of the memory budget for this product";
                ++stats_.failed;
                --pending_;
                cv_done_.notify_all();
            } else {
                cv_sched_.wait(lk);   // a retiring batch frees memory
            }
            continue;
        }
        Inflight& fr = *f;
        fr.slot = slot;
        fr.ctx = points_[fr.batch.point - 1].ctx;
        if (fr.batch.operand) fr.planes = operands_.at(fr.batch.operand).planes.as<uint32_t>();
        for (const sched::Request& q : fr.batch.requests) {
            const Record& r = records_.at(q.id);
            fr.a.push_back(r.a);
            fr.b.push_back(r.b);
            fr.c.push_back(r.c);
        }
        if (event_pool_.empty()) {
            cudaEvent_t e = nullptr;
            if (cudaEventCreateWithFlags(&e, cudaEventDisableTiming) != cudaSuccess) e = nullptr;
            event_pool_.push_back(e);
        }
        fr.done = event_pool_.back();
        event_pool_.pop_back();
        slot_busy_[slot] = true;
        inflight_.push_back(std::move(f));
        lk.unlock();
        try {
            issue(fr);
        } catch (const CudaError& e) {
            fr.error = e.what();
            fr.error_status = e.code == cudaErrorMemoryAllocation ? BCG_ERR_NOMEM : BCG_ERR_CUDA;
        } catch (const std::exception& e) {
            fr.error = e.what();
            fr.error_status = BCG_ERR_INVALID;
        }
        lk.lock();
        fr.issued = true;
        ++stats_.batches;
        stats_.batched_products += fr.batch.requests.size();
        cv_done_.notify_all();
    }
    scheduler_done_ = true;
    cv_done_.notify_all();
}

void Server::issue(Inflight& f) {
    if (!f.done) throw CudaError("completion event", cudaErrorMemoryAllocation);
    cudaStream_t st = streams_[f.slot];
    Context& ctx = *f.ctx;
    const uint32_t n = uint32_t(f.batch.requests.size());
    const size_t cw = ctx.coeff_words(), pw = ctx.plane_words();
    const bool resident = f.planes != nullptr;
    const size_t a_words = resident ? 0 : n * cw;
    const size_t ws_words = n * (resident ? pw : 2 * pw);
    const size_t bytes = 4 * (a_words + 2 * n * cw + ws_words);
    check(cudaMallocFromPoolAsync(&f.mem, bytes, pool_, st), "batch memory");
    try {
        uint32_t* A = static_cast<uint32_t*>(f.mem);
        uint32_t* B = A + a_words;
        uint32_t* C = B + n * cw;
        uint32_t* ws = C + n * cw;
        for (uint32_t i = 0; i < n; ++i) {
            if (!resident) check(cudaMemcpyAsync(A + i * cw, f.a[i], cw * 4, cudaMemcpyHostToDevice, st), "input copy");
            check(cudaMemcpyAsync(B + i * cw, f.b[i], cw * 4, cudaMemcpyHostToDevice, st), "input copy");
        }
        {
            std::lock_guard<std::mutex> launch(launch_mu_);
            if (resident) ctx.multiply_spectral_device(f.planes, B, C, n, ws, st);
            else ctx.chain(A, B, C, n, ws, st);
        }
        for (uint32_t i = 0; i < n; ++i)
            check(cudaMemcpyAsync(f.c[i], C + i * cw, cw * 4, cudaMemcpyDeviceToHost, st), "output copy");
    } catch (...) {
        cudaFreeAsync(f.mem, st);
        cudaEventRecord(f.done, st);
        throw;
    }
    check(cudaFreeAsync(f.mem, st), "batch memory");
    check(cudaEventRecord(f.done, st), "completion event");
}

void Server::retire(Inflight& f, int status, const std::string& error) {
    const double t = now();
    for (const sched::Request& q : f.batch.requests) {
        Record& r = records_.at(q.id);
        r.done = true;
        r.result.status = status;
        r.result.error = error;
        r.result.latency_ms = (t - q.submitted) * 1e3;
        if (status == BCG_OK) ++stats_.completed;
        else ++stats_.failed;
        --pending_;
    }
    adm_.give(f.batch.bytes);
    slot_busy_[f.slot] = false;
    if (f.done) event_pool_.push_back(f.done);
    cv_done_.notify_all();
    cv_sched_.notify_all();
}

void Server::complete_loop() {
    cudaSetDevice(device_);
    std::unique_lock<std::mutex> lk(mu_);
    for (;;) {
        if (inflight_.empty()) {
            if (scheduler_done_) break;
            cv_done_.wait(lk);
            continue;
        }
        bool progressed = false;
        for (size_t i = 0; i < inflight_.size();) {
            Inflight& f = *inflight_[i];
            if (!f.issued) { ++i; continue; }
            int status = f.error_status;
            std::string error = f.error;
            if (error.empty()) {
                const cudaError_t e = cudaEventQuery(f.done);
                if (e == cudaErrorNotReady) { ++i; continue; }
                if (e != cudaSuccess) {
                    error = cudaGetErrorString(e);
                    status = BCG_ERR_CUDA;
                }
            }
            if (error.empty()) {
                // A kernel's bounded wait that ran out leaves the context's status word set.
                Context* ctx = f.ctx;
                lk.unlock();
                try {
                    ctx->check_status();
                } catch (const DeviceTimeout& e) {
                    status = BCG_ERR_DEVICE_TIMEOUT;
                    error = e.what();
                } catch (const std::exception& e) {
                    status = BCG_ERR_CUDA;
                    error = e.what();
                }
                lk.lock();
            }
            retire(f, status, error);
            inflight_.erase(inflight_.begin() + long(i));
            progressed = true;
        }
        if (!progressed) {
            lk.unlock();
            std::this_thread::sleep_for(std::chrono::microseconds(20));
            lk.lock();
        }
    }
}

}  // namespace bcg
