// Device helpers shared by the sm_103a kernels: modular arithmetic on the
// INT32 pipe, and thin inline-PTX wrappers for tcgen05 (TMEM allocation, MMA,
// commit, loads), mbarriers and bulk async copies.
//
// Every wait on an mbarrier is bounded by a wall-clock limit read from
// %globaltimer.  A wait that runs out records an error code in the context's
// device status word and returns false; the kernel then skips its remaining
// work, drains what it started and frees its TMEM, so the CUDA context stays
// usable and the host reports the status.
//
// Two kinds of wait:
//   mbar_wait      waits for another role's arrival (a producer's tile, the
//                  MMA's commit).  Its limit is a kernel argument (the
//                  context's wait limit, 2 s by default) and it also gives up
//                  as soon as another thread of the CTA has given up;
//   mbar_wait_own  waits for this thread's own asynchronous work (its bulk
//                  copies, its MMAs) before the CTA may leave or free TMEM.
//                  It keeps the fixed 2 s limit and ignores the abort flag.
#pragma once

#include <cstdint>
#include <cuda_fp16.h>

namespace bcg {

// ---------------------------------------------------------------- status ---
enum DeviceStatus : uint32_t {
    kStatusOk = 0,
    kStatusWaitTimeout = 1,
};

// Generous: legitimate waits last microseconds.
constexpr uint64_t kWaitLimitNs = 2000000000ull;

__device__ __forceinline__ uint64_t global_ns() {
    uint64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// ------------------------------------------------------ modular arithmetic --
// Primes satisfy 2^30 < p < 2^31, so 2p < 2^32 and residues kept in [0, 2p)
// fit a uint32.  Twiddles are stored with Shoup companions w' = floor(w*2^32/p).

// x in [0, 2p) -> [0, p).  For x < p, x - p wraps above x.
__device__ __forceinline__ uint32_t reduce_once(uint32_t x, uint32_t p) {
    return min(x, x - p);
}

// Shoup product: y any uint32, w < p with companion wq.  Result in [0, 2p).
__device__ __forceinline__ uint32_t mul_shoup(uint32_t y, uint32_t w, uint32_t wq, uint32_t p) {
    const uint32_t q = __umulhi(y, wq);
    return y * w - q * p;
}

// Montgomery product a*b*2^-32 mod p for a < p, b < 2p.  Result in [0, 2p).
// np = -p^-1 mod 2^32.
__device__ __forceinline__ uint32_t mul_mont(uint32_t a, uint32_t b, uint32_t p, uint32_t np) {
    const uint64_t x = uint64_t(a) * b;
    const uint32_t lo = uint32_t(x), hi = uint32_t(x >> 32);
    const uint32_t m = lo * np;
    // lo + lo(m*p) == 0 mod 2^32: the carry out of the low word is (lo != 0).
    return hi + __umulhi(m, p) + (lo != 0);
}

// Forward Cooley-Tukey butterfly, inputs and outputs in [0, 2p).
__device__ __forceinline__ void bfly_ct(uint32_t& x, uint32_t& y, uint2 w, uint32_t p) {
    const uint32_t t = reduce_once(mul_shoup(y, w.x, w.y, p), p);
    const uint32_t xr = reduce_once(x, p);
    x = xr + t;
    y = xr - t + p;
}

// Inverse Gentleman-Sande butterfly, inputs and outputs in [0, 2p).
__device__ __forceinline__ void bfly_gs(uint32_t& x, uint32_t& y, uint2 w, uint32_t p) {
    const uint32_t xr = reduce_once(x, p), yr = reduce_once(y, p);
    x = xr + yr;
    y = mul_shoup(xr - yr + p, w.x, w.y, p);
}

// The same butterflies for a twiddle of 1: no multiply.
__device__ __forceinline__ void bfly_ct_unit(uint32_t& x, uint32_t& y, uint32_t p) {
    const uint32_t t = reduce_once(y, p);
    const uint32_t xr = reduce_once(x, p);
    x = xr + t;
    y = xr - t + p;
}
__device__ __forceinline__ void bfly_gs_unit(uint32_t& x, uint32_t& y, uint32_t p) {
    const uint32_t xr = reduce_once(x, p), yr = reduce_once(y, p);
    x = xr + yr;
    y = xr - yr + p;
}

// ---------------------------------------------------- fp16 byte digits -----
// Balanced base-256 digits in [-128, 128] are exact in fp16.  0x64XX is the
// fp16 bit pattern of 1024 + XX, so a byte b becomes fp16(b - bias) with one
// byte permute and one packed subtraction.
__device__ __forceinline__ uint32_t prmt(uint32_t a, uint32_t b, uint32_t sel) {
    uint32_t r;
    asm("prmt.b32 %0, %1, %2, %3;" : "=r"(r) : "r"(a), "r"(b), "r"(sel));
    return r;
}

// Bytes (b0, b1) of w as half2 (b0 - bias0, b1 - bias1); bias as half2 of 1024+bias.
__device__ __forceinline__ uint32_t bytes01_to_half2(uint32_t w, uint32_t bias) {
    const uint32_t h = prmt(w, 0x64u, 0x4140u);
    __half2 r = __hsub2(*reinterpret_cast<const __half2*>(&h), *reinterpret_cast<const __half2*>(&bias));
    return *reinterpret_cast<uint32_t*>(&r);
}
__device__ __forceinline__ uint32_t bytes23_to_half2(uint32_t w, uint32_t bias) {
    const uint32_t h = prmt(w, 0x64u, 0x4342u);
    __half2 r = __hsub2(*reinterpret_cast<const __half2*>(&h), *reinterpret_cast<const __half2*>(&bias));
    return *reinterpret_cast<uint32_t*>(&r);
}
// half2 bit patterns of (1024+128, 1024+128) and (1024+128, 1024+0).
constexpr uint32_t kBias128x2 = 0x64806480u;
constexpr uint32_t kBias128_0 = 0x64006480u;

// An exact integer |v| < 2^22 held in fp32 -> int32 without a conversion unit:
// v + 1.5*2^23 lies in [2^23, 2^24), where the ulp is 1.
__device__ __forceinline__ int32_t small_float_to_int(float v) {
    return __float_as_int(v + 12582912.0f) - 0x4B400000;
}

__device__ __forceinline__ uint32_t bit_reverse_dev(uint32_t x, uint32_t bits) {
    return bits ? (__brev(x) >> (32 - bits)) : 0u;
}

// ---------------------------------------------------------- shared memory --
__device__ __forceinline__ uint32_t smem_u32(const void* p) {
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

// ---------------------------------------------------------------- mbarrier --
__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" :: "r"(smem_u32(bar)), "r"(count));
}
__device__ __forceinline__ void mbar_fence_init() {
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
    asm volatile("{\n\t.reg .b64 st;\n\tmbarrier.arrive.shared::cta.b64 st, [%0];\n\t}"
                 :: "r"(smem_u32(bar)) : "memory");
}
__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* bar, uint32_t bytes) {
    asm volatile("{\n\t.reg .b64 st;\n\tmbarrier.arrive.expect_tx.shared::cta.b64 st, [%0], %1;\n\t}"
                 :: "r"(smem_u32(bar)), "r"(bytes) : "memory");
}
// suspend_ns > 0: a thread whose phase has not completed may sleep in
// hardware for up to that long per poll (it wakes when the phase completes),
// so many waiting warps do not keep the shared-memory pipe busy with polls.
__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity, uint32_t suspend_ns = 0) {
    uint32_t done;
    if (suspend_ns)
        asm volatile("{\n\t.reg .pred p;\n\t"
                     "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, %3;\n\t"
                     "selp.u32 %0, 1, 0, p;\n\t}"
                     : "=r"(done) : "r"(smem_u32(bar)), "r"(parity), "r"(suspend_ns) : "memory");
    else
        asm volatile("{\n\t.reg .pred p;\n\t"
                     "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
                     "selp.u32 %0, 1, 0, p;\n\t}"
                     : "=r"(done) : "r"(smem_u32(bar)), "r"(parity) : "memory");
    return done != 0;
}
// Non-blocking test of the phase with the given parity.
__device__ __forceinline__ bool mbar_test_wait(uint64_t* bar, uint32_t parity) {
    uint32_t done;
    asm volatile("{\n\t.reg .pred p;\n\t"
                 "mbarrier.test_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
                 "selp.u32 %0, 1, 0, p;\n\t}"
                 : "=r"(done) : "r"(smem_u32(bar)), "r"(parity) : "memory");
    return done != 0;
}

// Bounded wait for another role's arrival.  Returns false (and records the
// timeout) if the phase with the given parity did not complete within
// limit_ns, or if another thread of the CTA already gave up (abort flag in
// shared memory).  Threads of one warp can see different outcomes (one sees
// the phase complete, another the abort flag): vote before a warp-collective
// step.  The first poll is the whole fast path: the limit is read only once
// the phase is found incomplete (the CRT's chunk hand-offs are latency bound;
// a parameter load, a non-blocking test or a flag test ahead of the first poll
// measured 18.4 -> 20.0-21.4 us per product there).  The clock is then read
// every 64 polls and a poll may suspend the thread (up to suspend_ns, or a time
// the hardware chooses), so a wait can overrun its limit by that much: the
// limit is a lower bound.
//
// QUICK (kernels launched with a limit under 1 us, finer than %globaltimer
// resolves): one non-blocking test, and the wait gives up if the phase is
// incomplete; a blocking poll may suspend the thread long enough to cover a
// short wait.
template <bool QUICK = false>
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity,
                                          volatile uint32_t* abort_flag,
                                          uint32_t* status, uint64_t limit_ns, uint32_t suspend_ns = 0) {
    if constexpr (QUICK) {
        if (mbar_test_wait(bar, parity)) return true;
        if (*abort_flag) return false;
    } else {
        if (mbar_try_wait(bar, parity, suspend_ns)) return true;
        const uint64_t start = global_ns();
        for (uint32_t spin = 0;; ++spin) {
            if (mbar_try_wait(bar, parity, suspend_ns)) return true;
            if ((spin & 63) == 0) {
                if (*abort_flag) return false;
                if (global_ns() - start > limit_ns) break;
            }
        }
    }
    *abort_flag = 1;
    atomicExch(status, kStatusWaitTimeout);
    return false;
}

// Kernels are instantiated for both wait forms; launches with a limit under 1 us use QUICK.
inline bool quick_waits(uint64_t limit_ns) { return limit_ns < 1000ull; }

// Waits for this thread's own asynchronous work (copies, MMAs) to land before
// the CTA leaves: bounded by the same limit, but not cut short by the abort
// flag (an aborted CTA must still not exit with its copies in flight).
__device__ __forceinline__ bool mbar_wait_own(uint64_t* bar, uint32_t parity, uint32_t* status,
                                              uint32_t suspend_ns = 0) {
    if (mbar_try_wait(bar, parity, suspend_ns)) return true;
    const uint64_t start = global_ns();
    for (uint32_t spin = 0;; ++spin) {
        if (mbar_try_wait(bar, parity, suspend_ns)) return true;
        if ((spin & 63) == 0 && global_ns() - start > kWaitLimitNs) {
            atomicExch(status, kStatusWaitTimeout);
            return false;
        }
    }
}

// Named barrier `id` over `threads` threads that also returns whether `pred`
// holds in every one of them: a group of warps takes one decision together,
// so none of them is left waiting at a later barrier for a thread that left.
__device__ __forceinline__ bool named_sync_all(uint32_t id, uint32_t threads, bool pred) {
    uint32_t r;
    asm volatile("{\n\t.reg .pred p, q;\n\t"
                 "setp.ne.u32 p, %1, 0;\n\t"
                 "bar.red.and.pred q, %2, %3, p;\n\t"
                 "selp.u32 %0, 1, 0, q;\n\t}"
                 : "=r"(r) : "r"(pred ? 1u : 0u), "r"(id), "r"(threads) : "memory");
    return r != 0;
}

// ------------------------------------------------------- bulk async copy --
// 1-D global -> shared copy completing on an mbarrier (transaction bytes).
// Both addresses 16-byte aligned, bytes a multiple of 16.
__device__ __forceinline__ void bulk_load(void* smem_dst, const void* gmem_src, uint32_t bytes,
                                          uint64_t* bar) {
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
        :: "r"(smem_u32(smem_dst)), "l"(gmem_src), "r"(bytes), "r"(smem_u32(bar)) : "memory");
}

// 1-D shared -> global bulk copy (bulk-group completion).  Both addresses
// 16-byte aligned, bytes a multiple of 16; the writes to smem_src must be made
// visible to the async proxy first (fence_proxy_async + a barrier).
__device__ __forceinline__ void bulk_store(void* gmem_dst, const void* smem_src, uint32_t bytes) {
    asm volatile("cp.async.bulk.global.shared::cta.bulk_group [%0], [%1], %2;"
                 :: "l"(gmem_dst), "r"(smem_u32(smem_src)), "r"(bytes) : "memory");
    asm volatile("cp.async.bulk.commit_group;" ::: "memory");
}
// The sources of this thread's bulk stores have been read (smem reusable).
__device__ __forceinline__ void bulk_store_wait_read() {
    asm volatile("cp.async.bulk.wait_group.read 0;" ::: "memory");
}
// This thread's bulk stores are complete.
__device__ __forceinline__ void bulk_store_wait_all() {
    asm volatile("cp.async.bulk.wait_group 0;" ::: "memory");
}

// Hint: bring [src, src + bytes) into L2 ahead of a later bulk copy.
__device__ __forceinline__ void bulk_prefetch_l2(const void* gmem_src, uint32_t bytes) {
    asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" :: "l"(gmem_src), "r"(bytes) : "memory");
}

// Generic-proxy writes to shared memory become visible to the async proxy
// (tensor core operand reads) after this fence.
__device__ __forceinline__ void fence_proxy_async() {
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

// ---------------------------------------------------------------- tcgen05 --
__device__ __forceinline__ void tmem_alloc(uint32_t* smem_result, uint32_t ncols) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;"
                 :: "r"(smem_u32(smem_result)), "r"(ncols) : "memory");
}
__device__ __forceinline__ void tmem_relinquish() {
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" :: "r"(taddr), "r"(ncols) : "memory");
}
__device__ __forceinline__ void tc_fence_before() {
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void tc_fence_after() {
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}

// Shared-memory matrix descriptor, no swizzle, K-major canonical layout:
// 8-row x 16-byte core matrices; lbo = byte stride between core matrices
// along K, sbo = byte stride between 8-row groups.  Bits 46-47 hold the
// descriptor version (1) required by tcgen05.
__device__ __forceinline__ uint64_t smem_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
    uint64_t d = 0;
    d |= uint64_t((saddr >> 4) & 0x3FFFu);
    d |= uint64_t((lbo >> 4) & 0x3FFFu) << 16;
    d |= uint64_t((sbo >> 4) & 0x3FFFu) << 32;
    d |= uint64_t(1) << 46;
    return d;
}

// Instruction descriptor for kind::f16: fp16 A and B (both K-major), fp32 D.
__host__ __device__ constexpr uint32_t idesc_f16_f32(uint32_t M, uint32_t N) {
    return (1u << 4)                 // D format: f32
         | (0u << 7) | (0u << 10)    // A, B format: f16
         | ((N >> 3) << 17)
         | ((M >> 4) << 24);
}

// D[tmem] (+)= A[smem] * B[smem]^T, issued by one thread.
__device__ __forceinline__ void mma_f16(uint32_t tmem_d, uint64_t adesc, uint64_t bdesc,
                                        uint32_t idesc, uint32_t accumulate) {
    asm volatile("{\n\t.reg .pred p;\n\t"
                 "setp.ne.b32 p, %4, 0;\n\t"
                 "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}"
                 :: "r"(tmem_d), "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate) : "memory");
}

// Arrive once on bar when all previously issued tcgen05 async ops of this thread finish.
__device__ __forceinline__ void mma_commit(uint64_t* bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];"
                 :: "r"(smem_u32(bar)) : "memory");
}

// Each thread of the warp reads 32 consecutive fp32 columns of its TMEM lane.
__device__ __forceinline__ void tmem_ld32(uint32_t taddr, float (&v)[32]) {
    uint32_t r[32];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x32.b32 "
        "{%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
        "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]),
          "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]),
          "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int i = 0; i < 32; ++i) v[i] = __uint_as_float(r[i]);
}

// Issue half of a pipelined TMEM read: the registers are valid only after
// tmem_ld32_wait() on the same array (which names them as operands, so no use
// can move above the wait).
__device__ __forceinline__ void tmem_ld32_issue(uint32_t taddr, uint32_t (&r)[32]) {
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x32.b32 "
        "{%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
        "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]),
          "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]),
          "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
        : "r"(taddr));
}
__device__ __forceinline__ void tmem_ld32_wait(uint32_t (&r)[32]) {
    asm volatile("tcgen05.wait::ld.sync.aligned;"
                 : "+r"(r[0]), "+r"(r[1]), "+r"(r[2]), "+r"(r[3]), "+r"(r[4]), "+r"(r[5]), "+r"(r[6]), "+r"(r[7]),
                   "+r"(r[8]), "+r"(r[9]), "+r"(r[10]), "+r"(r[11]), "+r"(r[12]), "+r"(r[13]), "+r"(r[14]), "+r"(r[15]),
                   "+r"(r[16]), "+r"(r[17]), "+r"(r[18]), "+r"(r[19]), "+r"(r[20]), "+r"(r[21]), "+r"(r[22]), "+r"(r[23]),
                   "+r"(r[24]), "+r"(r[25]), "+r"(r[26]), "+r"(r[27]), "+r"(r[28]), "+r"(r[29]), "+r"(r[30]), "+r"(r[31])
                 :: "memory");
}

__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float (&v)[16]) {
    uint32_t r[16];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 "
        "{%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}

// Byte offset of element (row, k) in a K-major no-swizzle fp16 tile whose
// core matrices are laid out [row/8][k/8][row%8][k%8] (lbo = 128 bytes,
// sbo = (K/8)*128 bytes).
__host__ __device__ constexpr uint32_t kmajor_offset(uint32_t row, uint32_t k, uint32_t K) {
    return (row >> 3) * (K >> 3) * 128u + (k >> 3) * 128u + (row & 7u) * 16u + (k & 7u) * 2u;
}

}  // namespace bcg
