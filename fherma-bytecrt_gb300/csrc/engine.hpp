// Host engine: one Context per point (N, W, q) on one GPU.  It owns the
// device copies of the plan tables, a plane workspace for `group` products,
// pinned staging for host-buffer calls, and the launch chain
//   encode -> column pass (A,B) -> row pass (product) -> inverse column pass -> CRT.
#pragma once

#include <cstdint>
#include <functional>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "kernels.hpp"
#include "ntt.cuh"
#include "plan.hpp"

namespace bcg {

class CudaError : public std::runtime_error {
public:
    CudaError(const std::string& what, cudaError_t e)
        : std::runtime_error(what + ": " + cudaGetErrorString(e)), code(e) {}
    cudaError_t code;
};

class DeviceTimeout : public std::runtime_error {
public:
    using std::runtime_error::runtime_error;
};

// Admission refused by the serving loop (queue full, or a request larger
// than the memory budget).
class Busy : public std::runtime_error {
public:
    using std::runtime_error::runtime_error;
};

inline void check(cudaError_t e, const char* what) {
    if (e != cudaSuccess) throw CudaError(what, e);
}

// The device status word a context's kernels write (common.cuh DeviceStatus)
// as the host reports it: any value but kStatusOk is a wait that ran out.
inline void raise_device_status(uint32_t st) {
    if (st != 0)
        throw DeviceTimeout("a kernel's bounded wait ran out (device status " + std::to_string(st) + ")");
}

struct DeviceBuffer {
    void* ptr = nullptr;
    size_t bytes = 0;
    DeviceBuffer() = default;
    DeviceBuffer(const DeviceBuffer&) = delete;
    DeviceBuffer& operator=(const DeviceBuffer&) = delete;
    DeviceBuffer(DeviceBuffer&& o) noexcept : ptr(o.ptr), bytes(o.bytes) { o.ptr = nullptr; o.bytes = 0; }
    ~DeviceBuffer() { if (ptr) cudaFree(ptr); }
    void allocate(size_t n) {
        if (ptr) { cudaFree(ptr); ptr = nullptr; bytes = 0; }
        if (n) { check(cudaMalloc(&ptr, n), "device allocation"); bytes = n; }
    }
    template <class T> T* as() const { return static_cast<T*>(ptr); }
};

struct PinnedBuffer {
    void* ptr = nullptr;
    size_t bytes = 0;
    PinnedBuffer() = default;
    PinnedBuffer(const PinnedBuffer&) = delete;
    PinnedBuffer& operator=(const PinnedBuffer&) = delete;
    ~PinnedBuffer() { if (ptr) cudaFreeHost(ptr); }
    void allocate(size_t n) {
        if (ptr) { cudaFreeHost(ptr); ptr = nullptr; bytes = 0; }
        if (n) { check(cudaMallocHost(&ptr, n), "pinned allocation"); bytes = n; }
    }
    template <class T> T* as() const { return static_cast<T*>(ptr); }
};

// Device tables that depend only on the geometry (N, W, L) and the device:
// prime constants, NTT twiddle/twist tables and the encode B operand.
// Every Context of the same geometry on a device shares one copy (moduli of a
// geometry differ only in the CRT weights and q, which stay per Context).
struct GeometryTables {
    DeviceBuffer consts, tables, enc_b, enc_pow;
};
std::shared_ptr<const GeometryTables> geometry_tables(int device, const HostPlan& plan);

// Receives the stage boundaries of a launch chain (per-stage CUDA-event timing).
class StageTimer {
public:
    virtual ~StageTimer() = default;
    virtual void begin(int stage, cudaStream_t st) = 0;
    virtual void end(cudaStream_t st) = 0;
};

class HostWorker;

class Context {
public:
    Context(uint32_t N, uint32_t W, uint32_t L, const uint32_t* q, int device);
    ~Context();
    Context(const Context&) = delete;
    Context& operator=(const Context&) = delete;

    const HostPlan& plan() const { return plan_; }
    const Geometry& geom() const { return plan_.g; }
    int device() const { return device_; }
    cudaStream_t stream() const { return stream_; }
    uint32_t group() const { return group_; }
    // Products per copy/compute chunk of the host-buffer paths.
    uint32_t host_group() const;
    // Products per host-path group (0: about 128 MiB of operands, at most the chain length).
    void set_host_group(uint32_t g) { host_group_ = g; }
    uint32_t host_group_setting() const { return host_group_; }
    void set_group(uint32_t g);
    size_t plane_words() const { return size_t(plan_.g.P) * plan_.g.N; }
    size_t coeff_words() const { return size_t(plan_.g.N) * plan_.g.L; }
    size_t workspace_bytes_per_product() const { return 2 * plane_words() * sizeof(uint32_t); }

    // Stages (device pointers, asynchronous on st).
    void encode(const uint32_t* a, const uint32_t* b, uint32_t* pa, uint32_t* pb, size_t plane_stride,
                uint32_t count, cudaStream_t st);
    void negacyclic(uint32_t* pa, uint32_t* pb, size_t plane_stride, uint32_t count, cudaStream_t st);
    // terms in the natural [P][N] layout, or tile-major ([N/128][P][128], from
    // launch_col_inverse(..., tiled = true)) when tiled is set.
    void crt(const uint32_t* terms, size_t plane_stride, uint32_t* c, uint32_t count, cudaStream_t st,
             bool tiled = false);
    // The launch chain hands the CRT tile-major terms when the persistent CRT runs.
    bool tiled_terms() const { return tuning_.crt_persistent && plan_.g.C > 1 && plan_.g.N >= 128; }
    // Spectral form of an operand: encode + column pass + forward row pass.
    void forward_spectral(const uint32_t* x, uint32_t* planes, cudaStream_t st);
    // c = a * b where a is given in spectral form (planes, shared by all count products).
    void multiply_spectral_device(const uint32_t* a_spectral, const uint32_t* b, uint32_t* c, uint32_t count,
                                  uint32_t* workspace, cudaStream_t st);

    // Whole products.
    void multiply_device(const uint32_t* a, const uint32_t* b, uint32_t* c, uint32_t count, cudaStream_t st);
    // Host buffers.  With a sink, c is unused: the product goes to
    // sink(user, words, n) in order, one staged piece at a time.  With a
    // destination, c is unused too: dest(user, n) names, in order, where each
    // run of n words goes, and the library copies the run there.
    using Sink = void (*)(void* user, const uint32_t* words, size_t n);
    using Dest = uint32_t* (*)(void* user, size_t n);
    void multiply_host(const uint32_t* a, const uint32_t* b, uint32_t* c, uint32_t count,
                       Sink sink = nullptr, void* user = nullptr, Dest dest = nullptr);

    // Throws DeviceTimeout (after clearing it) if a kernel reported a wait timeout.
    void synchronize(cudaStream_t st);
    void check_status();

    // One product chain on a caller-provided workspace of >= count products.
    // `timer` (optional) replaces the context's own sampled profiler for this chain.
    // With `between`, operand A is encoded and column-transformed on its own,
    // then between() runs on the host (it may bring operand B in and make st
    // wait for it), then operand B follows: the device works on A while B is
    // still on its way.
    void chain(const uint32_t* a, const uint32_t* b, uint32_t* c, uint32_t count, uint32_t* ws, cudaStream_t st,
               StageTimer* timer = nullptr, const std::function<void()>& between = nullptr);

    NttArgs ntt_args() const { return ntt_; }
    const Tuning& tuning() const { return tuning_; }
    void set_tuning(const Tuning& t);
    // Limit of the kernels' waits on another role's arrival (0: the default,
    // kWaitLimitNs).  A wait that runs out makes the call report
    // DeviceTimeout; waits on a thread's own copies and MMAs keep kWaitLimitNs.
    void set_wait_limit_ns(uint64_t ns);
    uint64_t wait_limit_ns() const { return enc_.wait_limit_ns; }
    // Whether host-buffer calls may read and write pageable memory through the
    // host page tables where the device supports it (default on).
    void set_host_direct(bool on) { host_direct_ = on; }
    bool host_direct() const { return host_direct_ && pageable_direct_; }
    // NTT split N = C * 2^row_bits (0: the default R = min(N, 256)); re-plans the NTT tables.
    void set_row_bits(uint32_t row_bits);

    // Per-stage timing with CUDA events recorded on the launching stream.
    enum Stage { kEncode = 0, kColForward, kRow, kColInverse, kCrt, kStages };
    // every: 0 off, k > 0 brackets the stages of every k-th launch chain with events.
    void set_profiling(uint32_t every) { profile_every_ = every; }
    // Sums the elapsed time of every recorded stage (synchronizes on them).
    void read_profile(double* ms, uint64_t* launches, uint64_t* timed, uint64_t* chains, bool reset);
    uint64_t launches() const { return launches_total_; }

private:
    struct Mark { int stage; cudaEvent_t begin, end; };
    void mark_begin(int stage, cudaStream_t st);
    void mark_end(cudaStream_t st);
    uint32_t profile_every_ = 0;
    bool timing_chain_ = false;
    std::vector<Mark> marks_;
    std::vector<cudaEvent_t> event_pool_;
    uint64_t stage_launches_[kStages] = {};
    uint64_t stage_timed_[kStages] = {};
    uint64_t launches_total_ = 0, chains_ = 0;

    void ensure_workspace(uint32_t products);
    void ensure_host_slots(uint32_t products, uint32_t slots, bool pack_in, bool stage_out);
    void bind_ntt();

    HostPlan plan_;
    int device_ = 0;
    // The copy engines read pageable host memory through the host page tables
    // (coherent CPU-GPU systems): host inputs then skip the pinned staging copy.
    bool pageable_direct_ = false;   // the device reads and writes pageable memory through the host page tables
    bool host_direct_ = true;        // the host path may use that (knob host_direct)
    uint32_t host_group_ = 0;        // products per host-path group (knob host_group; 0: automatic)
    cudaStream_t stream_ = nullptr;
    cudaStream_t copy_in_ = nullptr, copy_out_ = nullptr;
    uint32_t group_ = 1;
    std::shared_ptr<const GeometryTables> geo_;
    DeviceBuffer crt_b_, q_, status_;
    DeviceBuffer ws_;
    size_t ws_products_ = 0;
    // Host-buffer path: kHostSlots device slots for inputs/outputs and pinned staging.
    // Six: a slot's round trip (inputs in, compute, product out, handed over)
    // took about 2.9 ms per 4-product group at N = 65536, and three slots left
    // the link idle between groups (1.04 ms per group against 0.58 of input
    // transfer).
    static constexpr uint32_t kHostSlots = 6;
    DeviceBuffer io_dev_[kHostSlots];
    PinnedBuffer io_in_[kHostSlots], io_out_[kHostSlots];
    PinnedBuffer edge_;   // partial end pages of the operands (two pages per operand)
    cudaEvent_t ev_in_[kHostSlots] = {}, ev_done_[kHostSlots] = {}, ev_out_[kHostSlots] = {};
    cudaEvent_t ev_host_[kHostSlots] = {};   // staged output landed (host waits only: the output worker, and
                                             // the calling thread for a run's staged end pages)
    std::vector<cudaEvent_t> piece_ev_[kHostSlots];   // 4 MiB output pieces of small calls
    std::unique_ptr<HostWorker> worker_;   // output side of the host path (created on first use)
    NttArgs ntt_{};
    EncodeArgs enc_{};
    CrtArgs crt_{};
    Tuning tuning_{};
};

// Autotuner (autotune.cu): times candidate shapes for ctx's geometry, applies
// the fastest and records it for later Contexts of the same geometry.
struct AutotuneReport {
    uint32_t group = 0, crt_tiles = 0, crt_persistent = 0, row_rows = 0, row_local = 0, row_bits = 0, candidates = 0;
    uint32_t row_pass = 0, encode_scalar = 0;
    double us_per_product_default = 0, us_per_product_tuned = 0;
};
AutotuneReport autotune(Context& ctx, uint32_t max_group);
bool cached_autotune(int device, uint32_t N, uint32_t W, uint32_t L, AutotuneReport* out);
void apply_autotune(Context& ctx, const AutotuneReport& r);

// Thread-local last error message for the C ABI.
void set_last_error(const std::string& msg);
const char* last_error();

}  // namespace bcg
