// extern "C" boundary of the batched and served forms (include/bytecrt_gb300.h).
#include "../../include/bytecrt_gb300.h"
#include "capi_internal.hpp"
#include "batch.hpp"
#include "server.hpp"

#include <cstring>

using bcg::guarded;
using bcg::require;

struct bcg_batch {
    std::unique_ptr<bcg::Batch> batch;
};

struct bcg_server {
    std::unique_ptr<bcg::Server> server;
};

namespace {
cudaStream_t as_stream(void* s) { return static_cast<cudaStream_t>(s); }
}  // namespace

extern "C" {

int bcg_batch_create(int device, bcg_batch** out) {
    return guarded([&] {
        require(out, "null argument");
        *out = nullptr;
        auto* b = new bcg_batch{std::make_unique<bcg::Batch>(device)};
        *out = b;
    });
}

void bcg_batch_destroy(bcg_batch* batch) { delete batch; }

int bcg_batch_add(bcg_batch* batch, uint32_t N, uint32_t W, uint32_t L, const uint32_t* q, const uint32_t* a,
                  const uint32_t* b, uint32_t* c, uint32_t count) {
    return guarded([&] {
        require(batch, "null batch");
        batch->batch->add(N, W, L, q, a, b, c, count);
    });
}

int bcg_batch_run(bcg_batch* batch, void* stream) {
    return guarded([&] {
        require(batch, "null batch");
        batch->batch->run(as_stream(stream));
    });
}

int bcg_batch_synchronize(bcg_batch* batch, void* stream) {
    return guarded([&] {
        require(batch, "null batch");
        batch->batch->synchronize(as_stream(stream));
    });
}

int bcg_batch_get_info(bcg_batch* batch, bcg_batch_info* out) {
    return guarded([&] {
        require(batch && out, "null argument");
        std::memset(out, 0, sizeof *out);
        out->groups = batch->batch->groups();
        out->products = batch->batch->products();
        uint64_t launches[bcg::Context::kStages], chains = 0;
        batch->batch->read_counts(launches, &chains);
        out->chains = chains;
        for (int s = 0; s < bcg::Context::kStages; ++s) out->launches += launches[s];
    });
}

int bcg_batch_set_lanes(bcg_batch* batch, uint32_t lanes) {
    return guarded([&] {
        require(batch, "null batch");
        batch->batch->set_lanes(lanes);
    });
}

int bcg_batch_profile_enable(bcg_batch* batch, int every) {
    return guarded([&] {
        require(batch, "null batch");
        require(every >= 0, "profile sampling period must be >= 0");
        batch->batch->set_profiling(uint32_t(every));
    });
}

int bcg_batch_profile_read(bcg_batch* batch, bcg_profile* out) {
    return guarded([&] {
        require(batch && out, "null argument");
        std::memset(out, 0, sizeof *out);
        batch->batch->read_profile(out->ms, out->launches, out->timed, &out->chains);
    });
}

int bcg_server_create(int device, const bcg_server_options* opt, bcg_server** out) {
    return guarded([&] {
        require(out, "null argument");
        *out = nullptr;
        bcg::ServerOptions o;
        if (opt) {
            o.memory_bytes = opt->memory_bytes;
            if (opt->slots) o.slots = opt->slots;
            o.max_batch = opt->max_batch;
            if (opt->max_queue) o.max_queue = opt->max_queue;
        }
        auto* s = new bcg_server{std::make_unique<bcg::Server>(device, o)};
        *out = s;
    });
}

void bcg_server_destroy(bcg_server* server) { delete server; }

int bcg_server_add_point(bcg_server* server, uint32_t N, uint32_t W, uint32_t L, const uint32_t* q,
                         uint32_t* point) {
    return guarded([&] {
        require(server && point, "null argument");
        *point = server->server->add_point(N, W, L, q);
    });
}

int bcg_server_add_operand(bcg_server* server, uint32_t point, const uint32_t* a, uint64_t* operand) {
    return guarded([&] {
        require(server && operand, "null argument");
        *operand = server->server->add_operand(point, a);
    });
}

int bcg_server_remove_operand(bcg_server* server, uint64_t operand) {
    return guarded([&] {
        require(server, "null server");
        server->server->remove_operand(operand);
    });
}

int bcg_server_submit(bcg_server* server, uint32_t point, const uint32_t* a, uint64_t operand, const uint32_t* b,
                      uint32_t* c, uint64_t* request) {
    return guarded([&] {
        require(server && request, "null argument");
        *request = server->server->submit(point, a, operand, b, c);
    });
}

int bcg_server_wait(bcg_server* server, uint64_t request, uint32_t timeout_ms, double* latency_ms) {
    bcg::RequestResult r;
    bool done = false;
    const int rc = guarded([&] {
        require(server, "null server");
        done = server->server->wait(request, timeout_ms, &r);
    });
    if (rc != BCG_OK) return rc;
    if (!done) {
        bcg::set_last_error("request still pending");
        return BCG_ERR_TIMEOUT;
    }
    if (latency_ms) *latency_ms = r.latency_ms;
    if (r.status != BCG_OK) bcg::set_last_error(r.error);
    return r.status;
}

int bcg_server_drain(bcg_server* server) {
    return guarded([&] {
        require(server, "null server");
        server->server->drain();
    });
}

int bcg_server_get_stats(const bcg_server* server, bcg_server_stats* out) {
    return guarded([&] {
        require(server && out, "null argument");
        const bcg::ServerStats s = server->server->stats();
        out->submitted = s.submitted; out->completed = s.completed; out->failed = s.failed;
        out->rejected = s.rejected; out->batches = s.batches; out->batched_products = s.batched_products;
        out->operands = s.operands; out->memory_budget = s.memory_budget; out->memory_used = s.memory_used;
        out->memory_peak = s.memory_peak;
    });
}

}  // extern "C"
