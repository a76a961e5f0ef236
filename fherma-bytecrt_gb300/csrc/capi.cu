// extern "C" boundary (include/bytecrt_gb300.h): status codes in, exceptions
// never cross it.  The reference converts every CUDA error into a C++
// exception at the plugin boundary (native-smoke/solve.cu:46-49); here the C
// ABI returns a code and the C++ plugin shim turns it back into an exception.
#include "../../include/bytecrt_gb300.h"
#include "capi_internal.hpp"

#include <cstring>
#include <new>

using bcg::guarded;
using bcg::require;

namespace {

void fill_info(const bcg::HostPlan& p, bcg_info* out, uint32_t group) {
    const bcg::Geometry& g = p.g;
    std::memset(out, 0, sizeof *out);
    out->N = g.N; out->W = g.W; out->L = g.L; out->P = g.P; out->kpad = g.kpad;
    out->enc_k = g.enc_k; out->enc_cols = g.enc_cols; out->crt_k = g.crt_k_total; out->crt_n = g.crt_n;
    out->product_bits = g.product_bits;
    out->group = group;
    out->workspace_bytes_per_product = uint64_t(2) * g.P * g.N * 4;
}


}  // namespace

extern "C" {

const char* bcg_last_error(void) { return bcg::last_error(); }

int bcg_plan_create(uint32_t N, uint32_t W, uint32_t L, const uint32_t* q, bcg_plan** out) {
    return guarded([&] {
        require(q && out, "null argument");
        *out = nullptr;
        auto* p = new bcg_plan{bcg::make_plan(N, W, L, q)};
        *out = p;
    });
}

void bcg_plan_destroy(bcg_plan* plan) { delete plan; }

int bcg_plan_info(const bcg_plan* plan, bcg_info* out) {
    return guarded([&] {
        require(plan && out, "null argument");
        fill_info(plan->plan, out, 0);
    });
}

int bcg_plan_primes(const bcg_plan* plan, uint32_t* primes, uint32_t* psi, uint32_t* crt_inverse) {
    return guarded([&] {
        require(plan, "null argument");
        const auto& p = plan->plan;
        if (primes) std::memcpy(primes, p.primes.data(), p.primes.size() * 4);
        if (psi) std::memcpy(psi, p.psi.data(), p.psi.size() * 4);
        if (crt_inverse) std::memcpy(crt_inverse, p.crt_inverse.data(), p.crt_inverse.size() * 4);
    });
}

int bcg_plan_weights(const bcg_plan* plan, uint32_t* weights) {
    return guarded([&] {
        require(plan && weights, "null argument");
        std::memcpy(weights, plan->plan.weights.data(), plan->plan.weights.size() * 4);
    });
}

int bcg_context_create(uint32_t N, uint32_t W, uint32_t L, const uint32_t* q, int device, bcg_context** out) {
    return guarded([&] {
        require(q && out, "null argument");
        *out = nullptr;
        auto c = std::make_unique<bcg_context>();
        c->ctx = std::make_unique<bcg::Context>(N, W, L, q, device);
        *out = c.release();
    });
}

void bcg_context_destroy(bcg_context* ctx) { delete ctx; }

int bcg_context_info(const bcg_context* ctx, bcg_info* out) {
    return guarded([&] {
        require(ctx && out, "null argument");
        fill_info(ctx->ctx->plan(), out, ctx->ctx->group());
    });
}

int bcg_context_set_group(bcg_context* ctx, uint32_t group) {
    return guarded([&] {
        require(ctx && group >= 1 && group <= 4096, "group must be in [1, 4096]");
        ctx->ctx->set_group(group);
    });
}

int bcg_context_set_tuning(bcg_context* ctx, const char* knob, int64_t value) {
    return guarded([&] {
        require(ctx && knob, "null argument");
        const std::string k(knob);
        auto& c = *ctx->ctx;
        if (k == "group") {
            require(value >= 1 && value <= 4096, "group must be in [1, 4096]");
            c.set_group(uint32_t(value));
        } else if (k == "crt_tiles") {
            require(value == 1 || value == 2, "crt_tiles must be 1 or 2");
            bcg::Tuning t = c.tuning();
            t.crt_tiles = uint32_t(value);
            c.set_tuning(t);
        } else if (k == "row_local") {
            require(value == 0 || value == 3 || value == 4, "row_local must be 0, 3 or 4");
            bcg::Tuning t = c.tuning();
            t.row_local = uint32_t(value);
            c.set_tuning(t);
        } else if (k == "crt_gap_fold") {
            require(value == 0 || value == 1, "crt_gap_fold must be 0 or 1");
            bcg::Tuning t = c.tuning();
            t.crt_gap_fold = uint32_t(value);
            c.set_tuning(t);
        } else if (k == "crt_persistent") {
            require(value == 0 || value == 1, "crt_persistent must be 0 or 1");
            bcg::Tuning t = c.tuning();
            t.crt_persistent = uint32_t(value);
            c.set_tuning(t);
        } else if (k == "row_bits") {
            require(value >= 0 && value <= 8, "row_bits must be in [0, 8]");
            c.set_row_bits(uint32_t(value));
        } else if (k == "row_rows") {
            require(value >= 0 && value <= 4096, "row_rows must be in [0, 4096]");
            bcg::Tuning t = c.tuning();
            t.row_rows = uint32_t(value);
            c.set_tuning(t);
        } else if (k == "row_pass") {
            require(value == 0 || value == 1, "row_pass must be 0 or 1");
            bcg::Tuning t = c.tuning();
            t.row_pass = uint32_t(value);
            c.set_tuning(t);
        } else if (k == "encode_scalar") {
            require(value == 0 || value == 1, "encode_scalar must be 0 or 1");
            bcg::Tuning t = c.tuning();
            t.encode_scalar = uint32_t(value);
            c.set_tuning(t);
        } else if (k == "host_group") {
            require(value >= 0 && value <= 4096, "host_group must be in [0, 4096]");
            c.set_host_group(uint32_t(value));
        } else if (k == "host_direct") {
            require(value == 0 || value == 1, "host_direct must be 0 or 1");
            c.set_host_direct(value == 1);
        } else if (k == "wait_limit_ns") {
            require(value >= 0 && value <= 60000000000ll, "wait_limit_ns must be in [0, 6e10]");
            c.set_wait_limit_ns(uint64_t(value));
        } else {
            throw std::invalid_argument("unknown tuning knob: " + k);
        }
    });
}

int bcg_context_get_tuning(const bcg_context* ctx, const char* knob, int64_t* value) {
    return guarded([&] {
        require(ctx && knob && value, "null argument");
        const std::string k(knob);
        auto& c = *ctx->ctx;
        if (k == "group") *value = c.group();
        else if (k == "crt_tiles") *value = c.tuning().crt_tiles;
        else if (k == "row_rows") *value = c.tuning().row_rows;
        else if (k == "row_bits") *value = c.geom().r_bits;
        else if (k == "crt_persistent") *value = c.tuning().crt_persistent;
        else if (k == "crt_gap_fold") *value = c.tuning().crt_gap_fold;
        else if (k == "row_local") *value = c.tuning().row_local;
        else if (k == "row_pass") *value = c.tuning().row_pass;
        else if (k == "encode_scalar") *value = c.tuning().encode_scalar;
        else if (k == "gap") *value = c.plan().gap;
        else if (k == "wait_limit_ns") *value = int64_t(c.wait_limit_ns());
        else if (k == "host_direct") *value = c.host_direct() ? 1 : 0;
        else if (k == "host_group") *value = c.host_group();
        else throw std::invalid_argument("unknown tuning knob: " + k);
    });
}

int bcg_context_autotune(bcg_context* ctx, uint32_t max_group, bcg_autotune_report* out) {
    return guarded([&] {
        require(ctx && out, "null argument");
        const bcg::AutotuneReport r = bcg::autotune(*ctx->ctx, max_group);
        std::memset(out, 0, sizeof *out);
        out->group = r.group; out->crt_tiles = r.crt_tiles; out->row_rows = r.row_rows; out->row_bits = r.row_bits;
        out->candidates = r.candidates;
        out->crt_persistent = r.crt_persistent;
        out->row_local = r.row_local;
        out->row_pass = r.row_pass;
        out->encode_scalar = r.encode_scalar;
        out->us_per_product_default = r.us_per_product_default;
        out->us_per_product_tuned = r.us_per_product_tuned;
    });
}

int bcg_multiply_sink(bcg_context* ctx, const uint32_t* a, const uint32_t* b, uint32_t count, bcg_sink sink,
                      void* user) {
    return guarded([&] {
        require(ctx && sink, "null argument");
        if (count == 0) return;
        require(a && b, "null buffer");
        ctx->ctx->multiply_host(a, b, nullptr, count, sink, user);
    });
}

int bcg_multiply_dest(bcg_context* ctx, const uint32_t* a, const uint32_t* b, uint32_t count, bcg_dest dest,
                      void* user) {
    return guarded([&] {
        require(ctx && dest, "null argument");
        if (count == 0) return;
        require(a && b, "null buffer");
        ctx->ctx->multiply_host(a, b, nullptr, count, nullptr, user, dest);
    });
}

int bcg_host_alloc(size_t bytes, int device, void** out) {
    return guarded([&] {
        require(out, "null argument");
        *out = nullptr;
        require(bytes > 0, "zero-byte allocation");
        bcg::check(cudaSetDevice(device), "select device");
        bcg::check(cudaMallocHost(out, bytes), "pinned allocation");
    });
}

int bcg_host_free(void* p) {
    return guarded([&] {
        if (p) bcg::check(cudaFreeHost(p), "pinned free");
    });
}

int bcg_multiply(bcg_context* ctx, const uint32_t* a, const uint32_t* b, uint32_t* c, uint32_t count) {
    return guarded([&] {
        require(ctx, "null context");
        if (count == 0) return;
        require(a && b && c, "null buffer");
        ctx->ctx->multiply_host(a, b, c, count);
    });
}

int bcg_multiply_device(bcg_context* ctx, const uint32_t* a, const uint32_t* b, uint32_t* c, uint32_t count,
                        void* stream) {
    return guarded([&] {
        require(ctx, "null context");
        if (count == 0) return;
        require(a && b && c, "null buffer");
        ctx->ctx->multiply_device(a, b, c, count, static_cast<cudaStream_t>(stream));
    });
}

int bcg_encode_device(bcg_context* ctx, const uint32_t* a, const uint32_t* b, uint32_t* planes_a,
                      uint32_t* planes_b, size_t plane_stride, uint32_t count, void* stream) {
    return guarded([&] {
        require(ctx && a && b && planes_a && planes_b, "null argument");
        cudaStream_t st = stream ? static_cast<cudaStream_t>(stream) : ctx->ctx->stream();
        ctx->ctx->encode(a, b, planes_a, planes_b, plane_stride, count, st);
    });
}

int bcg_negacyclic_device(bcg_context* ctx, uint32_t* planes_a, uint32_t* planes_b, size_t plane_stride,
                          uint32_t count, void* stream) {
    return guarded([&] {
        require(ctx && planes_a && planes_b, "null argument");
        cudaStream_t st = stream ? static_cast<cudaStream_t>(stream) : ctx->ctx->stream();
        ctx->ctx->negacyclic(planes_a, planes_b, plane_stride, count, st);
    });
}

int bcg_crt_device(bcg_context* ctx, const uint32_t* terms, size_t plane_stride, uint32_t* c, uint32_t count,
                   void* stream) {
    return guarded([&] {
        require(ctx && terms && c, "null argument");
        cudaStream_t st = stream ? static_cast<cudaStream_t>(stream) : ctx->ctx->stream();
        ctx->ctx->crt(terms, plane_stride, c, count, st);
    });
}

int bcg_synchronize(bcg_context* ctx) {
    return guarded([&] {
        require(ctx, "null context");
        bcg::check(cudaDeviceSynchronize(), "device synchronize");
        ctx->ctx->check_status();
    });
}

int bcg_profile_enable(bcg_context* ctx, int enable) {
    return guarded([&] {
        require(ctx, "null context");
        require(enable >= 0, "profile sampling period must be >= 0");
        ctx->ctx->set_profiling(uint32_t(enable));
    });
}

int bcg_profile_read(bcg_context* ctx, bcg_profile* out, int reset) {
    return guarded([&] {
        require(ctx && out, "null argument");
        std::memset(out, 0, sizeof *out);
        ctx->ctx->read_profile(out->ms, out->launches, out->timed, &out->chains, reset != 0);
    });
}

}  // extern "C"
