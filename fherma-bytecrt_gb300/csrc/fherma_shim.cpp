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

#include <memory>

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
    out.c.data.resize(total);
    check(bcg_multiply(s.ctx, in.a.data.data(), in.b.data.data(), out.c.data.data(), s.B), "run");
    return out;
}

void fherma_free(void* state) { delete static_cast<State*>(state); }
