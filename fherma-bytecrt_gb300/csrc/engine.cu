// Host engine: device tables, workspace and the launch chain (see engine.hpp).
#include "engine.hpp"
#include "host_pages.hpp"

#include <algorithm>
#include <cstring>
#include <map>
#include <mutex>
#include <tuple>
#include <condition_variable>
#include <exception>
#include <functional>
#include <thread>
#include <omp.h>
#include <unistd.h>

namespace bcg {

namespace {
thread_local std::string g_last_error;

// Parallel host copy for the pinned staging of host-buffer calls (the
// reference packs operands with up to 12 OpenMP workers, native-smoke/io-copy.cpp:29-42).
void parallel_copy(void* dst, const void* src, size_t bytes) {
    if (bytes < (size_t(1) << 20)) { std::memcpy(dst, src, bytes); return; }
    const int workers = std::min(16, omp_get_num_procs());
    const size_t chunk = (bytes + workers - 1) / workers;
#pragma omp parallel for num_threads(workers) schedule(static)
    for (int t = 0; t < workers; ++t) {
        const size_t begin = size_t(t) * chunk;
        if (begin < bytes)
            std::memcpy(static_cast<char*>(dst) + begin, static_cast<const char*>(src) + begin,
                        std::min(chunk, bytes - begin));
    }
}
}  // namespace

std::shared_ptr<const GeometryTables> geometry_tables(int device, const HostPlan& plan) {
    // Weak entries: the tables live as long as some Context of the geometry does.
    static std::mutex mu;
    static std::map<std::tuple<int, uint32_t, uint32_t, uint32_t, uint32_t>, std::weak_ptr<const GeometryTables>> cache;
    const auto key = std::make_tuple(device, plan.g.N, plan.g.W, plan.g.L, plan.g.R);
    std::lock_guard<std::mutex> lock(mu);
    if (auto hit = cache[key].lock()) return hit;
    auto t = std::make_shared<GeometryTables>();
    auto upload = [&](DeviceBuffer& buf, const void* src, size_t bytes) {
        buf.allocate(bytes);
        check(cudaMemcpy(buf.ptr, src, bytes, cudaMemcpyHostToDevice), "table upload");
    };
    upload(t->consts, plan.prime_consts.data(), plan.prime_consts.size() * 4);
    upload(t->tables, plan.ntt_tables.data(), plan.ntt_tables.size() * 4);
    upload(t->enc_b, plan.enc_b.data(), plan.enc_b.size() * 2);
    upload(t->enc_pow, plan.enc_pow.data(), plan.enc_pow.size() * 4);
    cache[key] = t;
    return t;
}

void set_last_error(const std::string& msg) { g_last_error = msg; }
const char* last_error() { return g_last_error.c_str(); }

Context::Context(uint32_t N, uint32_t W, uint32_t L, const uint32_t* q, int device)
    : plan_(make_plan(N, W, L, q)), device_(device) {
    check(cudaSetDevice(device_), "select device");
    const Geometry& g = plan_.g;
    check(cudaStreamCreateWithFlags(&stream_, cudaStreamNonBlocking), "stream");
    check(cudaStreamCreateWithFlags(&copy_in_, cudaStreamNonBlocking), "stream");
    check(cudaStreamCreateWithFlags(&copy_out_, cudaStreamNonBlocking), "stream");
    for (uint32_t s = 0; s < kHostSlots; ++s) {
        check(cudaEventCreateWithFlags(&ev_in_[s], cudaEventDisableTiming), "event");
        check(cudaEventCreateWithFlags(&ev_done_[s], cudaEventDisableTiming), "event");
        check(cudaEventCreateWithFlags(&ev_out_[s], cudaEventDisableTiming), "event");
        // The output worker sleeps on this one instead of spinning (the cores go to its copies).  Only the
        // host waits on it: stream waits on blocking-sync events measured much slower (pinned e2e 6,243 ->
        // 3,466 products/s).
        check(cudaEventCreateWithFlags(&ev_host_[s], cudaEventDisableTiming | cudaEventBlockingSync), "event");
    }
    auto upload = [&](DeviceBuffer& buf, const void* src, size_t bytes) {
        buf.allocate(bytes);
        check(cudaMemcpy(buf.ptr, src, bytes, cudaMemcpyHostToDevice), "table upload");
    };
    geo_ = geometry_tables(device_, plan_);
    upload(crt_b_, plan_.crt_b.data(), plan_.crt_b.size() * 2);
    upload(q_, plan_.q.data(), plan_.q.size() * 4);
    status_.allocate(16);
    check(cudaMemset(status_.ptr, 0, 16), "status reset");
    {
        int pageable = 0, host_tables = 0;
        cudaDeviceGetAttribute(&pageable, cudaDevAttrPageableMemoryAccess, device_);
        cudaDeviceGetAttribute(&host_tables, cudaDevAttrPageableMemoryAccessUsesHostPageTables, device_);
        pageable_direct_ = pageable && host_tables;
    }

    bind_ntt();

    enc_.enc_b = geo_->enc_b.as<uint16_t>();
    enc_.enc_pow = geo_->enc_pow.as<uint32_t>();
    for (uint32_t j = 0; j < g.P; ++j)
        enc_.prime[j] = make_uint2(plan_.prime_consts[4 * j], plan_.prime_consts[4 * j + 1]);
    enc_.N = g.N; enc_.L = g.L; enc_.P = g.P; enc_.K = g.enc_k; enc_.cols = g.enc_cols; enc_.chunks = g.enc_chunks;
    enc_.status = status_.as<uint32_t>();
    enc_.wait_limit_ns = kWaitLimitNs;

    crt_.crt_b = crt_b_.as<uint16_t>();
    for (uint32_t j = 0; j < g.P; ++j) crt_.invp[j] = plan_.invp[j];
    for (uint32_t l = 0; l < g.L; ++l) crt_.q[l] = plan_.q[l];
    crt_.q_inv_scaled = plan_.q_inv_scaled;
    crt_.N = g.N; crt_.L = g.L; crt_.P = g.P; crt_.k_total = g.crt_k_total; crt_.kchunks = g.crt_kchunks;
    crt_.E = g.crt_e; crt_.NC = g.crt_n;
    crt_.gap = plan_.gap;
    crt_.top_bits = g.W - 32 * (g.L - 1);
    crt_.status = status_.as<uint32_t>();
    crt_.wait_limit_ns = kWaitLimitNs;

    // Products per launch chain: long chains amortise each kernel's launch and
    // tail (8 products per chain at N=65536 measured 16% faster than 1).
    group_ = std::min<uint32_t>(256, std::max<uint32_t>(1, 524288 / g.N));
    // A geometry the autotuner already measured in this process starts tuned.
    AutotuneReport tuned;
    if (cached_autotune(device_, g.N, g.W, g.L, &tuned)) apply_autotune(*this, tuned);
}

Context::~Context() {
    worker_.reset();
    if (stream_) cudaStreamSynchronize(stream_);
    for (const Mark& m : marks_) { cudaEventDestroy(m.begin); cudaEventDestroy(m.end); }
    for (cudaEvent_t e : event_pool_) cudaEventDestroy(e);
    for (uint32_t s = 0; s < kHostSlots; ++s) {
        if (ev_in_[s]) cudaEventDestroy(ev_in_[s]);
        if (ev_done_[s]) cudaEventDestroy(ev_done_[s]);
        if (ev_out_[s]) cudaEventDestroy(ev_out_[s]);
        if (ev_host_[s]) cudaEventDestroy(ev_host_[s]);
        for (cudaEvent_t e : piece_ev_[s]) cudaEventDestroy(e);
    }
    if (copy_in_) cudaStreamDestroy(copy_in_);
    if (copy_out_) cudaStreamDestroy(copy_out_);
    if (stream_) cudaStreamDestroy(stream_);
}

void Context::bind_ntt() {
    const Geometry& g = plan_.g;
    const TableOffsets off = table_offsets(g);
    const uint32_t row_rows = ntt_.row_rows, row_local = ntt_.row_local, row_pass = ntt_.row_pass;
    ntt_ = NttArgs{};
    ntt_.consts = geo_->consts.as<uint4>();
    ntt_.tables = geo_->tables.as<uint2>();
    ntt_.table_stride = g.table_stride;
    ntt_.off_col_f = off.col_f; ntt_.off_col_i = off.col_i;
    ntt_.off_row_f = off.row_f; ntt_.off_row_i = off.row_i;
    ntt_.off_tw_lo = off.tw_lo; ntt_.off_tw_hi = off.tw_hi;
    ntt_.off_itw_lo = off.itw_lo; ntt_.off_itw_hi = off.itw_hi;
    ntt_.N = g.N; ntt_.P = g.P; ntt_.c_bits = g.c_bits; ntt_.z_bits = g.z_bits; ntt_.Z = g.Z; ntt_.H = g.H;
    ntt_.R = g.R;
    ntt_.row_rows = row_rows;
    ntt_.row_local = row_local;
    ntt_.row_pass = row_pass;
}

void Context::set_row_bits(uint32_t row_bits) {
    // Only the NTT tables depend on the split; the encode and CRT operands stay.
    HostPlan p = make_plan(plan_.g.N, plan_.g.W, plan_.g.L, plan_.q.data(), row_bits);
    // The old tables may be freed below: no launch on any stream may still read them.
    check(cudaDeviceSynchronize(), "device synchronize");
    auto geo = geometry_tables(device_, p);
    plan_ = std::move(p);
    geo_ = std::move(geo);
    enc_.enc_b = geo_->enc_b.as<uint16_t>();
    enc_.enc_pow = geo_->enc_pow.as<uint32_t>();
    bind_ntt();
}

void Context::set_group(uint32_t g) { group_ = std::max<uint32_t>(1, g); }

void Context::set_wait_limit_ns(uint64_t ns) {
    enc_.wait_limit_ns = crt_.wait_limit_ns = ns ? ns : kWaitLimitNs;
}

uint32_t Context::host_group() const {
    // Host-buffer calls pipeline copies against compute in chunks of about
    // 128 MiB of inputs: the first copy in and the last copy out are not
    // overlapped, and the host link (~200 GB/s each way) makes them cost
    // more than the slightly shorter launch chains.  Pinned B = 128 calls at
    // N = 65536, median per call: 20.48 ms with 4 products per group, 20.55
    // with 2, 20.90 with 8, 22.04 with 16.
    if (host_group_) return host_group_;
    const size_t pair_bytes = 2 * coeff_words() * sizeof(uint32_t);
    const uint32_t g = uint32_t(std::max<size_t>(1, (size_t(128) << 20) / pair_bytes));
    return std::min(g, group_);
}

void Context::set_tuning(const Tuning& t) {
    if (t.crt_tiles != 1 && t.crt_tiles != 2) throw std::invalid_argument("crt_tiles must be 1 or 2");
    if (t.crt_persistent > 1) throw std::invalid_argument("crt_persistent must be 0 or 1");
    if (t.row_rows > 4096) throw std::invalid_argument("row_rows must be at most 4096");
    if (t.row_local != 0 && t.row_local != 3 && t.row_local != 4) throw std::invalid_argument("row_local must be 0, 3 or 4");
    if (t.row_pass > 1) throw std::invalid_argument("row_pass must be 0 or 1");
    if (t.encode_scalar > 1) throw std::invalid_argument("encode_scalar must be 0 or 1");
    if (t.encode_scalar && plan_.g.L > kScalarMaxLimbs)
        throw std::invalid_argument("encode_scalar needs L <= 32");
    tuning_ = t;
    enc_.scalar = t.encode_scalar;
    ntt_.row_rows = t.row_rows;
    ntt_.row_local = t.row_local;
    ntt_.row_pass = t.row_pass;
    crt_.gap = t.crt_gap_fold ? plan_.gap : 0u;
}

void Context::ensure_workspace(uint32_t products) {
    if (products <= ws_products_) return;
    cudaStreamSynchronize(stream_);
    ws_.allocate(size_t(products) * workspace_bytes_per_product());
    ws_products_ = products;
}

// Host-path slots, allocated only as far as a call uses them (a call of n
// groups uses min(n, kHostSlots) slots): device [A | B | C]; pinned A | B
// where operands are packed for the device (the GPU cannot read them in
// place); pinned C where products go to a sink or an unlocked output.
void Context::ensure_host_slots(uint32_t products, uint32_t slots, bool pack_in, bool stage_out) {
    const size_t unit = size_t(products) * coeff_words() * 4;
    auto grow = [&](auto& buf, size_t bytes, cudaStream_t st) {
        if (buf.bytes >= bytes) return;
        cudaStreamSynchronize(stream_);
        cudaStreamSynchronize(st);
        buf.allocate(bytes);
    };
    for (uint32_t s = 0; s < slots; ++s) {
        grow(io_dev_[s], 3 * unit, copy_out_);
        if (pack_in) grow(io_in_[s], 2 * unit, copy_in_);
        if (stage_out) grow(io_out_[s], unit, copy_out_);
    }
}

void Context::encode(const uint32_t* a, const uint32_t* b, uint32_t* pa, uint32_t* pb, size_t plane_stride,
                     uint32_t count, cudaStream_t st) {
    // The encode kernel bulk-copies input tiles: their addresses must be 16-byte aligned.
    if ((reinterpret_cast<uintptr_t>(a) | reinterpret_cast<uintptr_t>(b)) & 15)
        throw std::invalid_argument("operand device pointers must be 16-byte aligned");
    EncodeArgs e = enc_;
    e.in0 = a; e.in1 = b; e.in_stride = coeff_words();
    e.out0 = pa; e.out1 = pb; e.out_stride = plane_stride;
    check(launch_encode(e, count, st, 2), "encode launch");
}

void Context::negacyclic(uint32_t* pa, uint32_t* pb, size_t plane_stride, uint32_t count, cudaStream_t st) {
    check(launch_col_forward(ntt_, pa, plane_stride, count, st), "column pass launch");
    check(launch_col_forward(ntt_, pb, plane_stride, count, st), "column pass launch");
    check(launch_row_product(ntt_, pa, plane_stride, pb, plane_stride, pa, plane_stride, count, false, st),
          "row pass launch");
    check(launch_col_inverse(ntt_, pa, plane_stride, count, st), "inverse column pass launch");
}

void Context::crt(const uint32_t* terms, size_t plane_stride, uint32_t* c, uint32_t count, cudaStream_t st,
                  bool tiled) {
    CrtArgs a = crt_;
    a.terms = terms; a.terms_stride = plane_stride;
    a.out = c; a.out_stride = coeff_words();
    a.terms_tiled = tiled ? 1u : 0u;
    if (tuning_.crt_persistent || tiled) {
        // The persistent CRT moves terms and output tiles with bulk copies: 16-byte alignment.
        if ((reinterpret_cast<uintptr_t>(c) | reinterpret_cast<uintptr_t>(terms)) & 15)
            throw std::invalid_argument("terms and output device pointers must be 16-byte aligned");
        check(launch_crt_persistent(a, count, st), "CRT launch");
    }
    else check(launch_crt(a, count, st, tuning_.crt_tiles), "CRT launch");
}

void Context::mark_begin(int stage, cudaStream_t st) {
    ++stage_launches_[stage];
    ++launches_total_;
    if (!timing_chain_) return;
    ++stage_timed_[stage];
    auto take = [&]() {
        if (event_pool_.empty()) {
            cudaEvent_t e;
            check(cudaEventCreate(&e), "profile event");
            return e;
        }
        cudaEvent_t e = event_pool_.back();
        event_pool_.pop_back();
        return e;
    };
    Mark m{stage, take(), take()};
    check(cudaEventRecord(m.begin, st), "profile event");
    marks_.push_back(m);
}

void Context::mark_end(cudaStream_t st) {
    if (!timing_chain_ || marks_.empty()) return;
    check(cudaEventRecord(marks_.back().end, st), "profile event");
}

void Context::read_profile(double* ms, uint64_t* launches, uint64_t* timed, uint64_t* chains, bool reset) {
    for (int s = 0; s < kStages; ++s) ms[s] = 0;
    for (const Mark& m : marks_) {
        check(cudaEventSynchronize(m.end), "profile event");
        float t = 0;
        check(cudaEventElapsedTime(&t, m.begin, m.end), "profile elapsed");
        ms[m.stage] += t;
    }
    for (int s = 0; s < kStages; ++s) { launches[s] = stage_launches_[s]; timed[s] = stage_timed_[s]; }
    *chains = chains_;
    if (reset) {
        for (const Mark& m : marks_) { event_pool_.push_back(m.begin); event_pool_.push_back(m.end); }
        marks_.clear();
        for (auto& l : stage_launches_) l = 0;
        for (auto& l : stage_timed_) l = 0;
        chains_ = 0;
    }
}

void Context::chain(const uint32_t* a, const uint32_t* b, uint32_t* c, uint32_t count, uint32_t* ws,
                    cudaStream_t st, StageTimer* timer, const std::function<void()>& between) {
    // Workspace per product: [A planes | B planes]; the product overwrites A.
    const size_t pw = plane_words();
    uint32_t* pa = ws;
    uint32_t* pb = ws + pw;
    const size_t stride = 2 * pw;
    ++chains_;
    timing_chain_ = timer == nullptr && profile_every_ != 0 && (chains_ - 1) % profile_every_ == 0;
    auto begin = [&](int stage) {
        if (timer) { ++stage_launches_[stage]; ++launches_total_; timer->begin(stage, st); }
        else mark_begin(stage, st);
    };
    auto end = [&] {
        if (timer) timer->end(st);
        else mark_end(st);
    };
    if (between) {
        auto operand = [&](const uint32_t* x, uint32_t* planes) {
            if (reinterpret_cast<uintptr_t>(x) & 15)
                throw std::invalid_argument("operand device pointers must be 16-byte aligned");
            EncodeArgs e = enc_;
            e.in0 = x; e.in1 = x; e.in_stride = coeff_words();
            e.out0 = planes; e.out1 = planes; e.out_stride = stride;
            begin(kEncode);
            check(launch_encode(e, count, st, 1), "encode launch");
            end();
            if (geom().C > 1) {
                begin(kColForward);
                check(launch_col_forward(ntt_, planes, stride, count, st), "column pass launch");
                end();
            }
        };
        operand(a, pa);
        between();
        operand(b, pb);
    } else {
        begin(kEncode);
        encode(a, b, pa, pb, stride, count, st);
        end();
        // Both operands' column passes in one launch (sets alternate A, B).
        if (geom().C > 1) {
            begin(kColForward);
            check(launch_col_forward(ntt_, pa, pw, 2 * count, st), "column pass launch");
            end();
        }
    }
    begin(kRow);
    check(launch_row_product(ntt_, pa, stride, pb, stride, pa, stride, count, false, st), "row pass launch");
    end();
    // Tile-major terms for the persistent CRT go to B's planes, dead after the row pass.
    const bool tiled = tiled_terms();
    if (geom().C > 1) {
        begin(kColInverse);
        check(launch_col_inverse(ntt_, pa, stride, count, st, tiled ? pb : nullptr), "inverse column pass launch");
        end();
    }
    begin(kCrt);
    crt(tiled ? pb : pa, stride, c, count, st, tiled);
    end();
}

void Context::forward_spectral(const uint32_t* x, uint32_t* planes, cudaStream_t st) {
    EncodeArgs e = enc_;
    e.in0 = x; e.in1 = x; e.in_stride = 0;
    e.out0 = planes; e.out1 = planes; e.out_stride = 0;
    check(launch_encode(e, 1, st, 1), "encode launch");
    check(launch_col_forward(ntt_, planes, 0, 1, st), "column pass launch");
    check(launch_row_forward(ntt_, planes, 0, 1, st), "row forward launch");
}

void Context::multiply_spectral_device(const uint32_t* a_spectral, const uint32_t* b, uint32_t* c,
                                       uint32_t count, uint32_t* ws, cudaStream_t st) {
    const size_t pw = plane_words();
    EncodeArgs e = enc_;
    e.in0 = b; e.in1 = b; e.in_stride = coeff_words();
    e.out0 = ws; e.out1 = ws; e.out_stride = pw;
    check(launch_encode(e, count, st, 1), "encode launch");
    check(launch_col_forward(ntt_, ws, pw, count, st), "column pass launch");
    check(launch_row_product(ntt_, a_spectral, 0, ws, pw, ws, pw, count, true, st), "row pass launch");
    check(launch_col_inverse(ntt_, ws, pw, count, st), "inverse column pass launch");
    crt(ws, pw, c, count, st);
}

void Context::multiply_device(const uint32_t* a, const uint32_t* b, uint32_t* c, uint32_t count,
                              cudaStream_t st) {
    if (!st) st = stream_;
    const uint32_t g = std::min(group_, std::max<uint32_t>(count, 1));
    ensure_workspace(g);
    const size_t cw = coeff_words();
    for (uint32_t done = 0; done < count; done += g) {
        const uint32_t n = std::min(g, count - done);
        chain(a + done * cw, b + done * cw, c + done * cw, n, ws_.as<uint32_t>(), st);
    }
}

namespace {
bool is_pinned(const void* p) {
    cudaPointerAttributes attr{};
    if (cudaPointerGetAttributes(&attr, p) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return attr.type == cudaMemoryTypeHost;
}
}  // namespace

namespace {
// Page locking of the caller's buffers for one call.  Only pages that lie
// wholly inside a buffer are registered (host_pages.hpp says why); the
// partial pages at either end of a buffer (less than a page each) travel
// through a small pinned bounce buffer instead.  Registering 1.8 GB takes
// about 3 ms on a GB300 host, unregistering 0.04 ms.
uintptr_t page_size() {
    static const uintptr_t page = uintptr_t(sysconf(_SC_PAGESIZE));
    return page;
}

bool register_pages(uintptr_t lo, uintptr_t hi) {
    if (hi <= lo) return true;
    if (cudaHostRegister(reinterpret_cast<void*>(lo), size_t(hi - lo), cudaHostRegisterDefault) == cudaSuccess)
        return true;
    cudaGetLastError();
    return false;
}

// Page-locks an input buffer one group at a time, just ahead of its copies,
// so that locking overlaps the device's work on earlier groups instead of
// preceding the call (2 x 1.8 GB took 6.1 ms up front).  The chunks and the
// cut of each group's copy are ChunkPlan's.
class ChunkLock {
public:
    ChunkLock(const void* p, size_t total, size_t step, bool enable) {
        if (!p || !total) return;
        pinned_ = is_pinned(p);
        if (pinned_ || !enable) return;
        plan_ = ChunkPlan(uintptr_t(p), total, step, page_size());
        regs_.assign(plan_.chunks, false);
        active_ = true;
    }
    ~ChunkLock() {
        for (size_t k = 0; k < regs_.size(); ++k)
            if (regs_[k]) cudaHostUnregister(reinterpret_cast<void*>(plan_.bound(k)));
    }
    ChunkLock(const ChunkLock&) = delete;
    ChunkLock& operator=(const ChunkLock&) = delete;
    // Locks every chunk up to k (stops for good at the first refusal).
    void lock_through(size_t k) {
        if (!active_) return;
        for (; ok_ && next_ <= k && next_ < plan_.chunks; ++next_) {
            const uintptr_t lo = plan_.bound(next_), hi = plan_.bound(next_ + 1);
            if (hi <= lo) continue;
            if (register_pages(lo, hi)) regs_[next_] = true;
            else ok_ = false;
        }
    }
    // The buffer is pinned or being locked: its copies go through copy_to_device.
    bool engaged() const { return pinned_ || active_; }
    // Copies group k (bytes from src): its pieces in locked chunks
    // asynchronously, its pieces in the buffer's partial end pages through
    // `bounce` (pinned, two pages: head, tail), and pieces in chunks that
    // could not be locked as pageable copies (the call returns once they are
    // read).  The bounce pages mirror the buffer's partial pages byte for
    // byte, so groups that share one of them use disjoint bytes of it.
    void copy_to_device(char* dst, const char* src, size_t k, size_t bytes, cudaStream_t st, char* bounce) {
        if (pinned_) {
            check(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, st), "input copy");
            return;
        }
        const uintptr_t b = uintptr_t(src);
        group_pieces(plan_, k, pieces_);
        for (const CopyPiece& c : pieces_) {
            const char* from = reinterpret_cast<const char*>(c.lo);
            if (c.kind != PieceKind::chunk) {
                char* h = c.kind == PieceKind::head ? bounce + (c.lo - plan_.base)
                                                    : bounce + page_size() + (c.lo - plan_.span.hi);
                std::memcpy(h, from, size_t(c.hi - c.lo));
                from = h;
            }
            check(cudaMemcpyAsync(dst + (c.lo - b), from, size_t(c.hi - c.lo), cudaMemcpyHostToDevice, st),
                  "input copy");
        }
    }
private:
    ChunkPlan plan_;
    size_t next_ = 0;
    bool pinned_ = false, active_ = false, ok_ = true;
    std::vector<bool> regs_;
    std::vector<CopyPiece> pieces_;
};

// Page-locks the output runs of one call as they are named (a caller's
// destination, or the groups of a pageable output): each run's whole pages,
// so neighbouring runs never share a registration.  prepare() says which part
// the copy engine may write directly; the partial pages at either end of the
// run come back through staging.
class OutLock {
public:
    OutLock() = default;
    ~OutLock() {
        for (uintptr_t lo : regs_) cudaHostUnregister(reinterpret_cast<void*>(lo));
    }
    OutLock(const OutLock&) = delete;
    OutLock& operator=(const OutLock&) = delete;
    // [*lo, *hi): the bytes of [d, d + bytes) (offsets) that may be written
    // directly; the rest, before and after, goes through staging.
    void prepare(char* d, size_t bytes, size_t* lo, size_t* hi) {
        const uintptr_t b = uintptr_t(d);
        bool ours = false;
        for (const auto& r : spans_) ours = ours || (b >= r.first && b < r.second);
        if (!ours && is_pinned(d)) {   // memory the caller pinned itself (one allocation per run)
            *lo = 0;
            *hi = bytes;
            return;
        }
        const PageSpan sp = whole_pages(b, bytes, page_size());
        if (sp.hi > sp.lo && register_pages(sp.lo, sp.hi)) {
            regs_.push_back(sp.lo);
            spans_.push_back({sp.lo, sp.hi});
            *lo = size_t(sp.lo - b);
            *hi = size_t(sp.hi - b);
        } else {
            *lo = *hi = 0;
        }
    }
private:
    std::vector<uintptr_t> regs_;
    std::vector<std::pair<uintptr_t, uintptr_t>> spans_;
};
}  // namespace

// One long-lived thread per context for the host side of the output: its
// OpenMP team (the parallel copies and page faulting of the sink) is created
// once, not on every call.
class HostWorker {
public:
    HostWorker() : thread_([this] { loop(); }) {}
    ~HostWorker() {
        {
            std::lock_guard<std::mutex> lk(mu_);
            quit_ = true;
        }
        cv_.notify_all();
        thread_.join();
    }
    // Runs f on the worker; wait() returns once it has returned.  f must not throw.
    void post(std::function<void()> f) {
        std::lock_guard<std::mutex> lk(mu_);
        task_ = std::move(f);
        busy_ = true;
        cv_.notify_all();
    }
    void wait() {
        std::unique_lock<std::mutex> lk(mu_);
        cv_.wait(lk, [&] { return !busy_; });
    }
private:
    void loop() {
        std::unique_lock<std::mutex> lk(mu_);
        for (;;) {
            cv_.wait(lk, [&] { return quit_ || busy_; });
            if (busy_) {
                std::function<void()> f = std::move(task_);
                lk.unlock();
                f();
                lk.lock();
                busy_ = false;
                cv_.notify_all();
            } else if (quit_) {
                return;
            }
        }
    }
    std::mutex mu_;
    std::condition_variable cv_;
    std::function<void()> task_;
    bool busy_ = false, quit_ = false;
    std::thread thread_;
};

// Host buffers.  Products move in groups of host_group() through kHostSlots
// device slots ([A | B | C] each), so that one group's copies overlap the
// compute of the others.
//  - Inputs: pinned ones go in with asynchronous copy-engine copies.  In calls
//    of three or more groups, pageable ones are page-locked chunk by chunk
//    just ahead of their copies.  In smaller calls the SMs read them in place
//    where the GPU uses the host's page tables (coherent CPU-GPU systems, such
//    as the GB300's Grace hosts); elsewhere they are packed into pinned staging.
//  - Outputs: a pinned output receives its products directly.  A pageable
//    output, or destinations a callback names group by group, is page-locked
//    run by run in larger calls and written straight, and written by the SMs
//    in smaller calls where the GPU uses the host's page tables.  A sink gets
//    each group from pinned staging, in order: in larger calls on the output
//    worker while the calling thread issues the next groups.
void Context::multiply_host(const uint32_t* a, const uint32_t* b, uint32_t* c, uint32_t count, Sink sink,
                            void* user, Dest dest) {
    if (count == 0) return;
    const size_t cw = coeff_words();
    const size_t all = size_t(count) * cw * 4;
    // Locking pays where the groups overlap one another's copies; a call of one
    // or two groups is not locked (one product through the plugin: 0.50 ms
    // unlocked against 0.81 ms locked, 0.42 ms with the copy kernels below).
    const uint32_t g = std::min(host_group(), count);
    const size_t gbytes = size_t(g) * cw * 4;
    const bool lock = count > 2 * g;
    ChunkLock lock_a(a, all, gbytes, lock), lock_b(b != a ? b : nullptr, all, gbytes, lock);
    ChunkLock& lock_b_or_a = b != a ? lock_b : lock_a;
    OutLock lock_out;
    // Leaving early (an error), no copy may still read or write the locked
    // buffers when they are unlocked: this guard is destroyed before them.
    struct Quiesce {
        cudaStream_t s0, s1, s2;
        ~Quiesce() { cudaStreamSynchronize(s0); cudaStreamSynchronize(s1); cudaStreamSynchronize(s2); }
    } quiesce{copy_in_, stream_, copy_out_};
    const bool out_pinned = !sink && !dest && is_pinned(c);
    ensure_workspace(g);
    const uint32_t ngroups = (count + g - 1) / g;
    const uint32_t slots = std::min(kHostSlots, ngroups);

    constexpr size_t kPiece = size_t(4) << 20;
    const bool host_direct = pageable_direct_ && host_direct_;
    ensure_host_slots(g, slots, !host_direct && !(is_pinned(a) && is_pinned(b)), !out_pinned);
    if (edge_.bytes < 4 * page_size()) edge_.allocate(4 * page_size());
    char* bounce_a = edge_.as<char>();
    char* bounce_b = b != a ? bounce_a + 2 * page_size() : bounce_a;
    const size_t max_pieces = (size_t(g) * cw * 4 + kPiece - 1) / kPiece;
    for (uint32_t s = 0; s < slots; ++s)
        while (piece_ev_[s].size() < max_pieces) {
            cudaEvent_t e;
            check(cudaEventCreateWithFlags(&e, cudaEventDisableTiming), "event");
            piece_ev_[s].push_back(e);
        }
    auto group_size = [&](uint32_t gi) { return std::min(g, count - gi * g); };
    auto stage_in = [&](ChunkLock& lk, uint32_t gi, char* h, char* d, const char* x, size_t bytes, char* bounce) {
        if (lk.engaged()) {                    // pinned or locked: asynchronous
            lk.copy_to_device(d, x, gi, bytes, copy_in_, bounce);
            return;
        }
        if (host_direct) {                     // the SMs read it in place, asynchronously
            check(launch_host_copy(reinterpret_cast<uint32_t*>(d), reinterpret_cast<const uint32_t*>(x), bytes / 4,
                                   copy_in_), "input copy");
            return;
        }
        for (size_t off = 0; off < bytes; off += kPiece) {
            const size_t n = std::min(kPiece, bytes - off);
            parallel_copy(h + off, x + off, n);
            check(cudaMemcpyAsync(d + off, h + off, n, cudaMemcpyHostToDevice, copy_in_), "input copy");
        }
    };

    // The output worker drains group gi once the calling thread has issued it.
    std::mutex mu;
    std::condition_variable cv;
    uint32_t issued = 0, drained = 0;
    bool stop = false;
    std::exception_ptr out_error;
    // One or two groups leave nothing to overlap on the host: their products
    // come back in 4 MiB pieces that this thread hands over as each lands (one
    // product through the plugin: 0.71 ms through the worker, 0.5 ms so).
    const bool inline_out = !out_pinned && ngroups <= 2;
    // Small calls into memory the GPU can write through the host's page
    // tables (a caller's destination or a pageable output): the SMs write
    // the product there directly, right after the chain; the destination is
    // named while the device computes.
    const bool direct_out = inline_out && !sink && host_direct;
    // Larger calls into a pageable output or a caller's destinations lock each
    // group's run of the output as it is issued and copy straight into it.
    const bool run_out = !out_pinned && !inline_out && !sink;
    const bool worker_out = !out_pinned && !inline_out && sink;
    // The parts of a run that are not locked (its partial end pages, or all
    // of it where locking fails) come back through the slot's staging; the
    // calling thread moves them before the slot's staging is reused and at
    // the end.
    struct Staged { char* dst = nullptr; size_t lo = 0, hi = 0, bytes = 0; } staged[kHostSlots];
    auto settle_staged = [&](uint32_t s) {
        Staged& st = staged[s];
        if (!st.dst) return;
        check(cudaEventSynchronize(ev_host_[s]), "output copy");
        const char* h = reinterpret_cast<const char*>(io_out_[s].as<uint32_t>());
        parallel_copy(st.dst, h, st.lo);
        parallel_copy(st.dst + st.hi, h + st.hi, st.bytes - st.hi);
        st.dst = nullptr;
    };
    auto named = [&](uint32_t gi, size_t words) {
        if (!dest) return reinterpret_cast<char*>(c + size_t(gi) * g * cw);
        uint32_t* p = dest(user, words);
        if (!p) throw std::invalid_argument("the output destination callback returned no memory");
        return reinterpret_cast<char*>(p);
    };
    if (worker_out) {
        if (!worker_) worker_ = std::make_unique<HostWorker>();
        worker_->post([&] {
            try {
                for (uint32_t gi = 0; gi < ngroups; ++gi) {
                    {
                        std::unique_lock<std::mutex> lk(mu);
                        cv.wait(lk, [&] { return issued > gi || stop; });
                        if (issued <= gi) return;
                    }
                    const uint32_t s = gi % slots;
                    const size_t bytes = size_t(group_size(gi)) * cw * 4;
                    const uint32_t* src = io_out_[s].as<uint32_t>();
                    // The products of this group are on their way: the sink may prepare room for them.
                    if (sink) sink(user, nullptr, bytes / 4);
                    check(cudaEventSynchronize(ev_host_[s]), "output copy");
                    if (sink) sink(user, src, bytes / 4);
                    else parallel_copy(c + size_t(gi) * g * cw, src, bytes);
                    std::lock_guard<std::mutex> lk(mu);
                    drained = gi + 1;
                    cv.notify_all();
                }
            } catch (...) {
                std::lock_guard<std::mutex> lk(mu);
                out_error = std::current_exception();
                stop = true;
                cv.notify_all();
            }
        });
    }
    // Whatever happens below, the worker's task ends before this frame does.
    struct Settle {
        HostWorker* w; std::mutex& mu; std::condition_variable& cv; bool& stop;
        ~Settle() {
            if (!w) return;
            { std::lock_guard<std::mutex> lk(mu); stop = true; }
            cv.notify_all();
            w->wait();
        }
    } settle{worker_out ? worker_.get() : nullptr, mu, cv, stop};

    for (uint32_t gi = 0; gi < ngroups; ++gi) {
        const uint32_t s = gi % slots;
        const uint32_t n = group_size(gi);
        const size_t off = size_t(gi) * g * cw, bytes = size_t(n) * cw * 4;
        if (worker_out && gi >= slots) {
            // The slot's previous group has left its staging (and so its device output).
            std::unique_lock<std::mutex> lk(mu);
            cv.wait(lk, [&] { return drained + slots > gi || out_error; });
            if (out_error) break;
        }
        lock_a.lock_through(gi);
        lock_b_or_a.lock_through(gi);
        uint32_t* d = io_dev_[s].as<uint32_t>();
        uint32_t* h = io_in_[s].ptr ? io_in_[s].as<uint32_t>() : nullptr;
        // Packing into the slot's staging: its previous inputs have left for the device.
        const bool packs = !host_direct && !(lock_a.engaged() && lock_b_or_a.engaged());
        if (packs && gi >= slots) check(cudaEventSynchronize(ev_in_[s]), "slot reuse");
        if (gi >= slots) check(cudaStreamWaitEvent(copy_in_, ev_done_[s], 0), "slot reuse");
        // Operand A first: the device encodes it while operand B comes in.
        stage_in(lock_a, gi, reinterpret_cast<char*>(h), reinterpret_cast<char*>(d),
                 reinterpret_cast<const char*>(a + off), bytes, bounce_a);
        check(cudaEventRecord(ev_in_[s], copy_in_), "event");
        check(cudaStreamWaitEvent(stream_, ev_in_[s], 0), "event wait");
        if (gi >= slots) check(cudaStreamWaitEvent(stream_, ev_out_[s], 0), "slot reuse");
        chain(d, d + g * cw, d + 2 * g * cw, n, ws_.as<uint32_t>(), stream_, nullptr, [&] {
            stage_in(lock_b_or_a, gi, reinterpret_cast<char*>(h ? h + g * cw : nullptr),
                     reinterpret_cast<char*>(d + g * cw), reinterpret_cast<const char*>(b + off), bytes, bounce_b);
            check(cudaEventRecord(ev_in_[s], copy_in_), "event");
            check(cudaStreamWaitEvent(stream_, ev_in_[s], 0), "event wait");
        });
        check(cudaEventRecord(ev_done_[s], stream_), "event");
        check(cudaStreamWaitEvent(copy_out_, ev_done_[s], 0), "event wait");
        if (direct_out) {
            char* dst = named(gi, bytes / 4);
            check(launch_host_copy(reinterpret_cast<uint32_t*>(dst), d + 2 * g * cw, bytes / 4, copy_out_),
                  "output copy");
        } else if (inline_out) {
            char* hs = reinterpret_cast<char*>(io_out_[s].as<uint32_t>());
            const char* ds = reinterpret_cast<const char*>(d + 2 * g * cw);
            for (size_t k = 0, po = 0; po < bytes; ++k, po += kPiece) {
                check(cudaMemcpyAsync(hs + po, ds + po, std::min(kPiece, bytes - po), cudaMemcpyDeviceToHost,
                                      copy_out_), "output copy");
                check(cudaEventRecord(piece_ev_[s][k], copy_out_), "event");
            }
        } else if (run_out) {
            settle_staged(s);
            char* dst = named(gi, bytes / 4);
            const char* ds = reinterpret_cast<const char*>(d + 2 * g * cw);
            char* hs = reinterpret_cast<char*>(io_out_[s].as<uint32_t>());
            size_t lo = 0, hi = 0;
            lock_out.prepare(dst, bytes, &lo, &hi);
            if (hi > lo)
                check(cudaMemcpyAsync(dst + lo, ds + lo, hi - lo, cudaMemcpyDeviceToHost, copy_out_), "output copy");
            if (lo > 0 || hi < bytes) {
                if (lo > 0) check(cudaMemcpyAsync(hs, ds, lo, cudaMemcpyDeviceToHost, copy_out_), "output copy");
                if (hi < bytes)
                    check(cudaMemcpyAsync(hs + hi, ds + hi, bytes - hi, cudaMemcpyDeviceToHost, copy_out_),
                          "output copy");
                check(cudaEventRecord(ev_host_[s], copy_out_), "event");
                staged[s] = Staged{dst, lo, hi, bytes};
            }
        } else {
            check(cudaMemcpyAsync(out_pinned ? c + off : io_out_[s].as<uint32_t>(), d + 2 * g * cw, bytes,
                                  cudaMemcpyDeviceToHost, copy_out_), "output copy");
        }
        check(cudaEventRecord(ev_out_[s], copy_out_), "event");
        // Lock the next group's inputs while the device works on this one.  (On
        // a helper thread running ahead, locking measured slower: 30.9 against
        // 24.2 ms per B = 128 plugin call; the driver serialises it against
        // this thread's calls.)
        lock_a.lock_through(gi + 1);
        lock_b_or_a.lock_through(gi + 1);
        if (!worker_out) continue;
        check(cudaEventRecord(ev_host_[s], copy_out_), "event");
        std::lock_guard<std::mutex> lk(mu);
        issued = gi + 1;
        cv.notify_all();
    }
    if (direct_out) {
        check(cudaStreamSynchronize(copy_out_), "output copy");
    } else if (inline_out) {
        for (uint32_t gi = 0; gi < ngroups; ++gi) {
            const uint32_t s = gi % slots;
            const size_t bytes = size_t(group_size(gi)) * cw * 4;
            const char* src = reinterpret_cast<const char*>(io_out_[s].as<uint32_t>());
            char* dst = named(gi, bytes / 4);
            if (sink) sink(user, nullptr, bytes / 4);
            for (size_t k = 0, po = 0; po < bytes; ++k, po += kPiece) {
                const size_t pn = std::min(kPiece, bytes - po);
                check(cudaEventSynchronize(piece_ev_[s][k]), "output copy");
                if (sink) sink(user, reinterpret_cast<const uint32_t*>(src + po), pn / 4);
                else parallel_copy(dst + po, src + po, pn);
            }
        }
    } else if (worker_out) {
        {
            std::unique_lock<std::mutex> lk(mu);
            cv.wait(lk, [&] { return drained == ngroups || out_error; });
        }
        if (out_error) std::rethrow_exception(out_error);
    } else {
        check(cudaStreamSynchronize(copy_out_), "output copy");
        for (uint32_t s = 0; s < slots; ++s) settle_staged(s);
    }
    check_status();
}

void Context::check_status() {
    uint32_t st = 0;
    check(cudaMemcpy(&st, status_.ptr, 4, cudaMemcpyDeviceToHost), "status read");
    if (st != kStatusOk) {
        check(cudaMemset(status_.ptr, 0, 4), "status reset");
        raise_device_status(st);
    }
}

void Context::synchronize(cudaStream_t st) {
    check(cudaStreamSynchronize(st ? st : stream_), "stream synchronize");
    check_status();
}

}  // namespace bcg
