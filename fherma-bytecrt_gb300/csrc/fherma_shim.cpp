// C++ plugin ABI (fherma_init / fherma_run / fherma_free) on top of the C ABI.
//
// Behaviour follows the reference's solve.cu: init builds everything that
// depends only on the point (native-smoke/solve.cu:295-397), run checks the
// input sizes and returns the owned product by value (native-smoke/solve.cu:
// 506-525), errors surface as std::runtime_error (solve.cu:46-49), free
// releases the state (solve.cu:527).  Built twice: libfherma_gb300.so (single
// product) and, with FHERMA_BATCHED, libfherma_gb300_batched.so (B <= 128,
// native-batched/solve.cu:160-244).
#include "fherma.h"
#include "bytecrt_gb300.h"

#include <cstdlib>
#include <cstring>
#include <exception>
#include <malloc.h>
#include <memory>
#include <mutex>
#include <omp.h>
// The owned output vector grows run by run as the library names each group's
// destination (bcg_multiply_dest): the vector's resize zero-fills the run, and
// the library writes the group straight into it (copy engine into page-locked
// runs in larger calls, SM stores through the host page tables in small ones),
// so the host writes each output byte once and no staging copy follows the
// device work.  B = 128 at N = 65536 took 38.2 ms per call when each group was
// staged and appended instead, 24-28 ms so.  std::vector copies with
// memmove/memcpy and fills with memset; this library is linked with --wrap for
// all three, so that large copies and fills (and the first touch of fresh
// pages) run on all cores, as the reference does for its output
// (native-smoke/vector-copy.cpp:19-56).
extern "C" void* __real_memcpy(void* dst, const void* src, size_t n);
extern "C" void* __real_memmove(void* dst, const void* src, size_t n);
extern "C" void* __real_memset(void* dst, int c, size_t n);

namespace {

constexpr size_t kParallelBytes = size_t(1) << 20;

void parallel_copy(char* dst, const char* src, size_t n) {
    const int workers = omp_get_num_procs() < 16 ? omp_get_num_procs() : 16;
    const size_t chunk = ((n + workers - 1) / workers + 63) & ~size_t(63);
#pragma omp parallel for num_threads(workers) schedule(static)
    for (int t = 0; t < workers; ++t) {
        const size_t begin = size_t(t) * chunk;
        if (begin < n) __real_memcpy(dst + begin, src + begin, n - begin < chunk ? n - begin : chunk);
    }
}

void parallel_fill(char* dst, int c, size_t n) {
    const int workers = omp_get_num_procs() < 16 ? omp_get_num_procs() : 16;
    const size_t chunk = ((n + workers - 1) / workers + 63) & ~size_t(63);
#pragma omp parallel for num_threads(workers) schedule(static)
    for (int t = 0; t < workers; ++t) {
        const size_t begin = size_t(t) * chunk;
        if (begin < n) __real_memset(dst + begin, c, n - begin < chunk ? n - begin : chunk);
    }
}

// The owned output of every call is a fresh vector of up to 1.8 GB.  glibc
// serves such blocks with mmap and unmaps them when they are freed, so every
// call would fault in fresh pages; while copies and kernels run, those faults
// cost 33 ms per B = 128 call on a GB300 host (9 ms on an idle one).  Serving
// large blocks from the heap and keeping freed heap memory mapped lets the next
// output land on pages that are already there.  Process-wide; switched off by
// BYTECRT_KEEP_HEAP=0 for processes that must hand memory back to the system.
void keep_heap_mapped() {
    static std::once_flag once;
    std::call_once(once, [] {
        const char* env = std::getenv("BYTECRT_KEEP_HEAP");
        if (env && env[0] == '0') return;
        mallopt(M_MMAP_MAX, 0);          // large blocks from the heap, not mmap
        mallopt(M_TRIM_THRESHOLD, -1);   // freed heap memory stays mapped
    });
}

bool disjoint(const void* dst, const void* src, size_t n) {
    const char* d = static_cast<const char*>(dst);
    const char* s = static_cast<const char*>(src);
    return d + n <= s || s + n <= d;
}

}  // namespace

extern "C" void* __wrap_memcpy(void* dst, const void* src, size_t n) {
    if (n >= kParallelBytes && !omp_in_parallel()) {
        parallel_copy(static_cast<char*>(dst), static_cast<const char*>(src), n);
        return dst;
    }
    return __real_memcpy(dst, src, n);
}

extern "C" void* __wrap_memset(void* dst, int c, size_t n) {
    if (n >= kParallelBytes && !omp_in_parallel()) {
        parallel_fill(static_cast<char*>(dst), c, n);
        return dst;
    }
    return __real_memset(dst, c, n);
}

extern "C" void* __wrap_memmove(void* dst, const void* src, size_t n) {
    if (n >= kParallelBytes && !omp_in_parallel() && disjoint(dst, src, n)) {
        parallel_copy(static_cast<char*>(dst), static_cast<const char*>(src), n);
        return dst;
    }
    return __real_memmove(dst, src, n);
}

namespace {

struct State {
    bcg_context* ctx = nullptr;
    uint32_t N = 0, L = 0, B = 1;
    ~State() { if (ctx) bcg_context_destroy(ctx); }
};

void check(int rc, const char* what) {
    if (rc != BCG_OK) throw std::runtime_error(std::string("bytecrt-gb300 ") + what + ": " + bcg_last_error());
}

}  // namespace

void* fherma_init(const fherma::Point& p) {
    keep_heap_mapped();
    auto s = std::make_unique<State>();
#ifdef FHERMA_BATCHED
    if (p.B == 0 || p.B > 128) throw std::runtime_error("bytecrt-gb300 batch coverage B=1..128");
    s->B = p.B;
#endif
    if (p.L != (p.W + 31) / 32) throw std::runtime_error("bytecrt-gb300 point L mismatch");
    if (p.q.data.size() != p.L) throw std::runtime_error("bytecrt-gb300 modulus limb count");
    s->N = p.N;
    s->L = p.L;
    check(bcg_context_create(p.N, p.W, p.L, p.q.data.data(), 0, &s->ctx), "init");
    return s.release();
}

fherma::Outputs fherma_run(void* state, const fherma::Inputs& in) {
    auto& s = *static_cast<State*>(state);
    const size_t words = size_t(s.N) * s.L;
    const size_t total = words * s.B;
    if (in.a.data.size() != total || in.b.data.size() != total)
        throw std::runtime_error("bytecrt-gb300 input coefficient count");
    fherma::Outputs out;
#ifdef FHERMA_BATCHED
    out.c.shape = {int64_t(s.B), int64_t(s.N), int64_t(s.L)};
#else
    out.c.shape = {int64_t(s.N), int64_t(s.L)};
#endif
    out.c.data.reserve(total);
    // The vector grows run by run (zero-filled on up to 16 threads) as the
    // library names each group's destination, and the library writes the
    // products straight into it.
    struct Grow {
        std::vector<uint32_t>* v;
        std::exception_ptr error;
    } grow{&out.c.data, nullptr};
    const int rc = bcg_multiply_dest(s.ctx, in.a.data.data(), in.b.data.data(), s.B,
                                     [](void* user, size_t n) -> uint32_t* {
                                         auto* g = static_cast<Grow*>(user);
                                         const size_t at = g->v->size();
                                         // Never past the reserved capacity: earlier runs keep their addresses.
                                         if (at + n > g->v->capacity()) return nullptr;
                                         try {
                                             g->v->resize(at + n);
                                         } catch (...) {
                                             g->error = std::current_exception();
                                             return nullptr;
                                         }
                                         return g->v->data() + at;
                                     },
                                     &grow);
    if (grow.error) std::rethrow_exception(grow.error);
    check(rc, "run");
    if (out.c.data.size() != total) throw std::runtime_error("bytecrt-gb300 output size");
    return out;
}

void fherma_free(void* state) { delete static_cast<State*>(state); }
