// Per-geometry autotuner: picks the encode kernel, the NTT radix split, the CRT
// MMA tile shape, the row-pass CTA shape and the products per launch chain by
// timing whole launch chains on the device.
//
// The reference fixes its shapes per geometry by hand (native-smoke/solve.cu
// instantiates one kernel set per (N, P, Kpad)); here the search runs once per
// (device, N, W, L) in a process, and every Context of that geometry created
// afterwards starts from the result.
#include "engine.hpp"

#include <algorithm>
#include <map>
#include <mutex>
#include <tuple>
#include <vector>

namespace bcg {

namespace {

using Key = std::tuple<int, uint32_t, uint32_t, uint32_t>;
std::mutex g_tuned_mu;
std::map<Key, AutotuneReport>& tuned() {
    static std::map<Key, AutotuneReport> m;
    return m;
}

struct Settings {
    uint32_t row_bits, crt_tiles, crt_persistent, row_rows, row_local, group, row_pass, encode_scalar;
    bool operator==(const Settings& o) const {
        return row_bits == o.row_bits && crt_tiles == o.crt_tiles && crt_persistent == o.crt_persistent &&
               row_rows == o.row_rows && row_local == o.row_local && group == o.group && row_pass == o.row_pass &&
               encode_scalar == o.encode_scalar;
    }
};

void apply(Context& ctx, const Settings& s) {
    if (ctx.geom().r_bits != s.row_bits) ctx.set_row_bits(s.row_bits);
    Tuning t = ctx.tuning();
    t.crt_tiles = s.crt_tiles;
    t.crt_persistent = s.crt_persistent;
    t.row_rows = s.row_rows;
    t.row_local = s.row_local;
    t.row_pass = s.row_pass;
    t.encode_scalar = s.encode_scalar;
    ctx.set_tuning(t);
    ctx.set_group(s.group);
}

}  // namespace

bool cached_autotune(int device, uint32_t N, uint32_t W, uint32_t L, AutotuneReport* out) {
    std::lock_guard<std::mutex> lock(g_tuned_mu);
    auto it = tuned().find(Key{device, N, W, L});
    if (it == tuned().end()) return false;
    *out = it->second;
    return true;
}

void apply_autotune(Context& ctx, const AutotuneReport& r) {
    apply(ctx, Settings{r.row_bits, r.crt_tiles, r.crt_persistent, r.row_rows, r.row_local, r.group, r.row_pass,
                        r.encode_scalar});
}

AutotuneReport autotune(Context& ctx, uint32_t max_group) {
    const Geometry& g0 = ctx.geom();
    const uint32_t N = g0.N, L = g0.L;
    const size_t cw = ctx.coeff_words();
    max_group = std::max<uint32_t>(1, std::min<uint32_t>(max_group, 256));
    // Cap the timed chain at 4 GB of workspace.
    const size_t ws_pp = ctx.workspace_bytes_per_product();
    const uint32_t mem_cap = uint32_t(std::max<size_t>(1, (size_t(4) << 30) / ws_pp));
    const uint32_t gmax = std::min(max_group, mem_cap);

    // Canonical synthetic operands: pseudo-random limbs below 2^(W-1) < q.
    std::vector<uint32_t> host(cw);
    uint64_t x = 0x9e3779b97f4a7c15ull ^ (uint64_t(N) << 20) ^ g0.W;
    for (size_t i = 0; i < cw; ++i) {
        x ^= x << 13; x ^= x >> 7; x ^= x << 17;
        host[i] = uint32_t(x >> 16);
    }
    const uint32_t top_bits = (g0.W - 1) - 32 * (L - 1);
    const uint32_t top_mask = top_bits >= 32 ? 0xffffffffu : ((1u << top_bits) - 1);
    for (uint32_t n = 0; n < N; ++n) host[size_t(n) * L + L - 1] &= top_mask;
    DeviceBuffer io, ws;
    io.allocate(size_t(3) * gmax * cw * 4);
    ws.allocate(size_t(gmax) * ws_pp);
    uint32_t* a = io.as<uint32_t>();
    uint32_t* b = a + size_t(gmax) * cw;
    uint32_t* c = b + size_t(gmax) * cw;
    for (uint32_t i = 0; i < 2 * gmax; ++i)
        check(cudaMemcpy(a + size_t(i) * cw, host.data(), cw * 4, cudaMemcpyHostToDevice), "autotune input");

    cudaStream_t st = ctx.stream();
    cudaEvent_t e0, e1;
    check(cudaEventCreate(&e0), "event");
    check(cudaEventCreate(&e1), "event");
    uint32_t candidates = 0;
    // Device time of one product, best of three chains of `group` products.
    auto measure = [&](const Settings& s) {
        apply(ctx, s);
        ++candidates;
        const uint32_t n = std::min(s.group, gmax);
        ctx.chain(a, b, c, n, ws.as<uint32_t>(), st);   // warm (tables, L2)
        float best = 1e30f;
        for (int rep = 0; rep < 3; ++rep) {
            check(cudaEventRecord(e0, st), "event");
            ctx.chain(a, b, c, n, ws.as<uint32_t>(), st);
            check(cudaEventRecord(e1, st), "event");
            check(cudaEventSynchronize(e1), "autotune timing");
            float ms = 0;
            check(cudaEventElapsedTime(&ms, e0, e1), "event");
            best = std::min(best, ms);
        }
        ctx.check_status();
        return 1000.0 * best / n;
    };

    AutotuneReport r{};
    Settings cur{g0.r_bits, ctx.tuning().crt_tiles, ctx.tuning().crt_persistent, ctx.tuning().row_rows,
                 ctx.tuning().row_local, std::min(ctx.group(), gmax), ctx.tuning().row_pass,
                 ctx.tuning().encode_scalar};
    double cur_us = measure(cur);
    r.us_per_product_default = cur_us;
    auto consider = [&](Settings s) {
        if (s == cur) return;
        double us;
        try {
            us = measure(s);
        } catch (const std::invalid_argument&) {
            return;   // split not valid for this N
        }
        if (us < cur_us * 0.99) { cur = s; cur_us = us; }
    };
    // Coordinate search: encode kernel, radix split, CRT tile shape, row-pass kernel and CTA, chain length.
    if (L <= kScalarMaxLimbs)
        for (uint32_t es : {0u, 1u}) { Settings s = cur; s.encode_scalar = es; consider(s); }
    const uint32_t nb = g0.n_bits;
    for (uint32_t rb = (nb > 8 ? nb - 8 : 4); rb <= std::min<uint32_t>(8, nb); ++rb) {
        Settings s = cur; s.row_bits = rb; consider(s);
    }
    for (uint32_t t : {2u, 1u}) { Settings s = cur; s.crt_persistent = 0; s.crt_tiles = t; consider(s); }
    { Settings s = cur; s.crt_persistent = 1; consider(s); }
    for (uint32_t rl : {0u, 3u}) { Settings s = cur; s.row_local = rl; consider(s); }
    for (uint32_t rp : {0u, 1u}) { Settings s = cur; s.row_pass = rp; consider(s); }
    for (uint32_t rr : {0u, 8u, 16u, 64u, 128u}) { Settings s = cur; s.row_rows = rr; consider(s); }
    for (uint32_t gr : {1u, 2u, 4u, 8u, 16u, 32u, 64u}) {
        if (gr > gmax) break;
        Settings s = cur; s.group = gr; consider(s);
    }
    apply(ctx, cur);
    check(cudaEventDestroy(e0), "event");
    check(cudaEventDestroy(e1), "event");
    r.row_bits = cur.row_bits;
    r.crt_tiles = cur.crt_tiles;
    r.crt_persistent = cur.crt_persistent;
    r.row_rows = cur.row_rows;
    r.row_local = cur.row_local;
    r.row_pass = cur.row_pass;
    r.encode_scalar = cur.encode_scalar;
    r.group = cur.group;
    r.us_per_product_tuned = cur_us;
    r.candidates = candidates;
    std::lock_guard<std::mutex> lock(g_tuned_mu);
    tuned()[Key{ctx.device(), N, g0.W, L}] = r;
    return r;
}

}  // namespace bcg
