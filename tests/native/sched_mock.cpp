// Host-only check of the serving loop's policy (scheduler.hpp) against a mock
// executor in virtual time: Poisson arrivals of three request sizes, a fixed
// number of slots, batch run time growing with the batch.  Exits non-zero on
// the first broken invariant.
#include "scheduler.hpp"

#include <cstdio>
#include <cstdlib>
#include <map>
#include <random>
#include <set>
#include <vector>

using namespace bcg::sched;

#define REQUIRE(cond)                                                              \
    do {                                                                           \
        if (!(cond)) {                                                             \
            std::fprintf(stderr, "invariant broken at line %d: %s\n", __LINE__, #cond); \
            std::exit(1);                                                          \
        }                                                                          \
    } while (0)

int main(int argc, char** argv) {
    const uint64_t seed = argc > 1 ? std::strtoull(argv[1], nullptr, 10) : 1;
    const int slots = argc > 2 ? std::atoi(argv[2]) : 3;
    std::mt19937_64 rng(seed);
    const uint64_t budget = 1000;
    // point -> (bytes per product, batch limit, run time of one product)
    std::map<uint32_t, uint64_t> bytes{{1, 60}, {2, 240}, {3, 900}};
    std::map<uint32_t, uint32_t> limit{{1, 8}, {2, 3}, {3, 1}};
    std::map<uint32_t, double> cost{{1, 1.0}, {2, 4.0}, {3, 16.0}};
    Admission adm(budget);
    Queue queue;
    struct Running { Batch b; double end; };
    std::vector<Running> running;
    std::set<uint64_t> waiting, done;
    std::exponential_distribution<double> gap(1.0 / 2.5);
    std::uniform_real_distribution<double> u(0, 1);
    const int total = 4000;
    double t = 0, next_arrival = 0, max_wait_big = 0;
    std::map<uint64_t, double> arrival;
    uint64_t next_id = 1, batches = 0;
    auto max_batch = [&](uint32_t p) { return limit[p]; };
    while (done.size() < size_t(total)) {
        // next event: an arrival or the earliest completion
        double next_done = 1e300;
        size_t which = 0;
        for (size_t i = 0; i < running.size(); ++i)
            if (running[i].end < next_done) { next_done = running[i].end; which = i; }
        const bool arrive = next_id <= uint64_t(total) && next_arrival <= next_done;
        if (!arrive && running.empty()) {
            REQUIRE(queue.empty());   // nothing runs, nothing arrives: the queue must be empty
            break;
        }
        if (arrive) {
            t = next_arrival;
            const double x = u(rng);
            const uint32_t p = x < 0.5 ? 1 : (x < 0.85 ? 2 : 3);
            const uint64_t operand = (p == 1 && u(rng) < 0.5) ? 7 : 0;
            Request r{next_id, p, operand, bytes[p], t};
            arrival[next_id] = t;
            waiting.insert(next_id);
            queue.push(r);
            ++next_id;
            next_arrival = t + gap(rng);
        } else {
            t = next_done;
            Running fin = running[which];
            running.erase(running.begin() + long(which));
            adm.give(fin.b.bytes);
            for (const Request& r : fin.b.requests) {
                REQUIRE(done.insert(r.id).second);   // completes exactly once
                if (r.point == 3 && t - arrival[r.id] > max_wait_big) max_wait_big = t - arrival[r.id];
            }
        }
        // admit while slots are free and the head fits
        while (int(running.size()) < slots && !queue.empty()) {
            const uint64_t oldest = *waiting.begin();
            REQUIRE(queue.head().id == oldest);       // head-of-line order
            Batch b;
            if (!queue.next(adm, max_batch, &b)) break;
            REQUIRE(!b.requests.empty());
            REQUIRE(b.requests.front().id == oldest); // the oldest leads the batch
            REQUIRE(b.requests.size() <= limit[b.point]);
            uint64_t sum = 0;
            for (size_t i = 0; i < b.requests.size(); ++i) {
                const Request& r = b.requests[i];
                REQUIRE(r.point == b.point && r.operand == b.operand);
                if (i) REQUIRE(r.id > b.requests[i - 1].id);   // arrival order inside the batch
                REQUIRE(waiting.erase(r.id) == 1);
                sum += r.bytes;
            }
            REQUIRE(sum == b.bytes);
            REQUIRE(adm.used() <= adm.budget());      // never over the budget
            running.push_back(Running{b, t + cost[b.point] * (0.5 + 0.5 * double(b.requests.size()))});
            ++batches;
        }
    }
    REQUIRE(done.size() == size_t(total));
    REQUIRE(waiting.empty());
    REQUIRE(adm.used() == 0);
    REQUIRE(adm.peak() <= budget);
    std::printf("ok requests=%d batches=%llu peak=%llu max_wait_big=%.1f\n", total,
                (unsigned long long)batches, (unsigned long long)adm.peak(), max_wait_big);
    return 0;
}
