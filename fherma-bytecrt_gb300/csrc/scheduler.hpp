// Request admission and batch formation for the serving loop (plain C++, no
// CUDA, so the policy is tested on the host against a mock executor).
//
// The reference has no server: it runs one product per fherma_run call
// (native-smoke/solve.cu:506-525) or one fixed batch per call
// (native-batched/solve.cu:200-244).  The serving loop admits products of
// different points as they arrive:
//   * the oldest waiting request always leads the next batch, so no request
//     waits behind later ones (head-of-line order, no starvation);
//   * the batch takes the later waiting requests of the same point and the
//     same resident operand, in arrival order, up to the point's batch limit;
//   * a batch is admitted only if its device bytes fit the free part of the
//     memory budget; otherwise the loop waits for running batches to finish.
#pragma once

#include <algorithm>
#include <cstdint>
#include <deque>
#include <functional>
#include <vector>

namespace bcg {
namespace sched {

struct Request {
    uint64_t id = 0;
    uint32_t point = 0;      // registered point (N, W, q)
    uint64_t operand = 0;    // resident left operand, 0 if a is sent with the request
    uint64_t bytes = 0;      // device bytes this product holds while in flight
    double submitted = 0;    // host clock at submission, seconds
};

struct Batch {
    uint32_t point = 0;
    uint64_t operand = 0;
    uint64_t bytes = 0;
    std::vector<Request> requests;
};

// Device-memory budget shared by in-flight batches and resident operands.
class Admission {
public:
    explicit Admission(uint64_t budget) : budget_(budget) {}
    bool fits(uint64_t bytes) const { return bytes <= budget_ - used_; }
    void take(uint64_t bytes) {
        used_ += bytes;
        if (used_ > peak_) peak_ = used_;
    }
    void give(uint64_t bytes) { used_ = bytes > used_ ? 0 : used_ - bytes; }
    uint64_t budget() const { return budget_; }
    uint64_t used() const { return used_; }
    uint64_t peak() const { return peak_; }

private:
    uint64_t budget_;
    uint64_t used_ = 0;
    uint64_t peak_ = 0;
};

class Queue {
public:
    void push(const Request& r) { q_.push_back(r); }
    size_t size() const { return q_.size(); }
    bool empty() const { return q_.empty(); }
    const Request& head() const { return q_.front(); }
    Request pop() {
        Request r = q_.front();
        q_.pop_front();
        return r;
    }

    // Forms the next batch and takes its bytes from `adm`.  Returns false
    // (queue unchanged) when the queue is empty or the head does not fit.
    bool next(Admission& adm, const std::function<uint32_t(uint32_t)>& max_batch, Batch* out) {
        if (q_.empty() || !adm.fits(q_.front().bytes)) return false;
        const Request head = q_.front();
        out->point = head.point;
        out->operand = head.operand;
        out->bytes = 0;
        out->requests.clear();
        const uint32_t limit = std::max<uint32_t>(1, max_batch(head.point));
        for (auto it = q_.begin(); it != q_.end() && out->requests.size() < limit;) {
            if (it->point == head.point && it->operand == head.operand && adm.fits(out->bytes + it->bytes)) {
                out->bytes += it->bytes;
                out->requests.push_back(*it);
                it = q_.erase(it);
            } else {
                ++it;
            }
        }
        adm.take(out->bytes);
        return true;
    }

private:
    std::deque<Request> q_;
};

}  // namespace sched
}  // namespace bcg
