// RNS encode on the 5th-generation tensor cores (tcgen05, kind::f16).
//
// For a tile of 128 coefficients and a group of primes p_j:
//     x_j = sum_k digit_k(coefficient) * (2^(8k+32) mod p_j)
// as a GEMM [128 x K] x [K x 4G] where both operands are balanced base-256
// digits (|digit| <= 128, exact in fp16) and the 4 output columns of a prime
// are the 4 balanced digits of 2^(8k+32) mod p_j.  Every digit sum is an
// integer of magnitude <= K*128*128 < 2^22, exact in the fp32 accumulator.
// The epilogue reassembles x_j = sum_d S_d 256^d (|x| < 2^46) and applies one
// signed Montgomery reduction, which removes the 2^32 folded into the powers:
// the result is the coefficient mod p_j, in [0, 2p_j).
//
// The reference computes the same residues with u8 mma.sync byte dots and a
// u64 Barrett (native-smoke/rns-encode-mma.cuh:15-52, 148-252).  Balanced
// digits make the fp16 path exact; it replaces the int8 path, which sm_103a
// does not have (ptxas rejects tcgen05.mma .kind::i8 for this target).
//
// Persistent kernel.  The primes are split into NG groups (NG = 2 for P > 16)
// so that one group's byte-power matrix stays resident in shared memory for
// the whole launch (one bulk copy per CTA); CTAs of group g loop over all
// 128-row tiles of all operands and products.  A tiles and TMEM accumulators
// are double buffered: builders fill tile i+1 while the MMA of tile i runs
// and the epilogue warps drain tile i-1.  Warp roles:
//   warps 0-7    A-tile builders in two groups, one per A buffer (thread = row:
//                balanced fp16 digits of one row each); a group issues its
//                buffer's input copy as soon as the MMA has released it, so
//                one buffer's copy overlaps the other's conversion
//   warps 8-23   epilogue, four warps per TMEM lane quarter, each a quarter of the columns
//   warp 24      TMEM allocation, B load, MMA issue (one thread)
// The epilogue bounds the job rate (per-job globaltimer traces: the MMA waits
// for the accumulator the epilogue hands back); four warps per quarter
// rather than three measured 3.6% faster at N = 65536.
#include "common.cuh"
#include "kernels.hpp"

namespace bcg {
namespace {

constexpr uint32_t kTileRows = 128;
constexpr uint32_t kBuildGroupWarps = 4;   // one builder thread per tile row
constexpr uint32_t kBuildWarps = 2 * kBuildGroupWarps;   // one builder group per A buffer
constexpr uint32_t kEpiPerQuarter = 4;      // epilogue warps per TMEM lane quarter
constexpr uint32_t kEpiWarps = 4 * kEpiPerQuarter;
constexpr uint32_t kCtlWarp = kBuildWarps + kEpiWarps;
constexpr uint32_t kEncThreads = (kCtlWarp + 1) * 32;
// The MMA-issuing thread sleeps up to this long per mbarrier poll (30.65 ->
// 30.49 us per product at N=65536); the builders' and epilogue's waits
// measured slower with it and keep polling.
constexpr uint32_t kCtlSuspendNs = 20000;

struct EncodeSmem {
    uint64_t bfull, afull[2], aempty[2], accfull[2], accempty[2], infull[2];
    uint32_t tmem_base;
    uint32_t abort_flag;
};

// Digits of one coefficient row into the K-major A tile: every input byte b
// becomes fp16(b - 128) independently (no carries); the digit at k = 4L is
// the constant 1 that adds back C = 0x80..80 through the B matrix.
template <int LT>
__device__ __forceinline__ void digits_row(uint8_t* tile, uint32_t r, const uint32_t* w, uint32_t L, uint32_t K) {
    const uint32_t words = LT ? uint32_t(LT) : L;
    uint32_t h[4] = {0, 0, 0, 0};
#pragma unroll
    for (uint32_t l = 0; l < (LT ? uint32_t(LT) : 64u); ++l) {
        if (!LT && l >= words) break;
        h[2 * (l & 1)] = bytes01_to_half2(w[l], kBias128x2);
        h[2 * (l & 1) + 1] = bytes23_to_half2(w[l], kBias128x2);
        if (l & 1)
            *reinterpret_cast<uint4*>(tile + kmajor_offset(r, 8 * (l >> 1), K)) = make_uint4(h[0], h[1], h[2], h[3]);
    }
    // Tail: the constant digit right after the last word, then zero padding.
    uint32_t kc = words / 2;
    if (words & 1) {
        h[2] = 0x00003C00u;                       // fp16 1.0 at k = 4L
        h[3] = 0;
    } else {
        h[0] = 0x00003C00u;
        h[1] = h[2] = h[3] = 0;
    }
    *reinterpret_cast<uint4*>(tile + kmajor_offset(r, 8 * kc, K)) = make_uint4(h[0], h[1], h[2], h[3]);
    for (++kc; kc < K / 8; ++kc)
        *reinterpret_cast<uint4*>(tile + kmajor_offset(r, 8 * kc, K)) = make_uint4(0u, 0u, 0u, 0u);
}

// x = sum_d S_d 256^d from four exact fp32 digit sums, then (x - m p) / 2^32.
// With |S_d| < 2^22: u = S_3*256 + S_2 and v = S_1*256 + S_0 fit int32 and
// x = u * 2^16 + v is one wide multiply-add.  The signed Montgomery quotient
// t = hi(x) - hi(m p) lies in (-p - 2^14, 2^14]; min(t + p, t + 2p) taken as
// unsigned picks the representative in [0, 2p).
__device__ __forceinline__ uint32_t encode_residue(float s0, float s1, float s2, float s3, uint2 pc) {
    // Bit patterns of S + 1.5*2^23 carry S + 0x4B400000; wrapping unsigned
    // arithmetic removes the bias exactly (the true u and v fit int32).
    const uint32_t b0 = __float_as_uint(s0 + 12582912.0f), b1 = __float_as_uint(s1 + 12582912.0f);
    const uint32_t b2 = __float_as_uint(s2 + 12582912.0f), b3 = __float_as_uint(s3 + 12582912.0f);
    constexpr uint32_t kBias257 = 0x4B400000u * 257u;
    const int32_t u = int32_t(b3 * 256u + b2 - kBias257);
    const int32_t v = int32_t(b1 * 256u + b0 - kBias257);
    const int64_t x = int64_t(u) * 65536 + v;
    const uint32_t m = uint32_t(x) * pc.y;
    const uint32_t t = uint32_t(int32_t(x >> 32)) - __umulhi(m, pc.x);
    return min(t + pc.x, t + 2 * pc.x);
}

template <int LT, bool QUICK>
__global__ void __launch_bounds__(kEncThreads, 1)
encode_kernel(const __grid_constant__ EncodeArgs a) {
    extern __shared__ __align__(1024) uint8_t smem[];
    const uint32_t K = a.K, L = LT ? uint32_t(LT) : a.L;
    const uint32_t ng = a.groups;
    const uint32_t g = blockIdx.x % ng;                       // prime group of this CTA
    const uint32_t slot = blockIdx.x / ng, nslots = gridDim.x / ng;
    const uint32_t col0 = g * a.group_cols;                   // first B column of the group
    const uint32_t gcols = min(a.group_cols, a.cols - col0);  // multiple of 16
    const uint32_t tile_bytes = kTileRows * K * 2;
    uint8_t* tiles = smem;                                    // 2 x tile_bytes
    uint8_t* bres = smem + 2 * tile_bytes;                    // gcols x K fp16, resident
    EncodeSmem* ctl = reinterpret_cast<EncodeSmem*>(bres + a.group_cols * K * 2);
    volatile uint32_t* abort_flag = &ctl->abort_flag;

    const uint32_t warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const uint32_t ntiles = (a.N + kTileRows - 1) / kTileRows;
    const uint32_t njobs = a.nprod * a.operands * ntiles;

    if (threadIdx.x == 0) {
        mbar_init(&ctl->bfull, 1);
        for (int i = 0; i < 2; ++i) {
            mbar_init(&ctl->afull[i], kTileRows);
            mbar_init(&ctl->aempty[i], 1);
            mbar_init(&ctl->accfull[i], 1);
            mbar_init(&ctl->accempty[i], kEpiWarps * 32);
            mbar_init(&ctl->infull[i], 1);
        }
        ctl->abort_flag = 0;
        mbar_fence_init();
    }
    if (warp == kCtlWarp) {
        tmem_alloc(&ctl->tmem_base, 512);
        tmem_relinquish();
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = ctl->tmem_base;

    if (warp == kCtlWarp) {
        if (lane == 0) {
            // The group's columns are one contiguous K-major range (8-row groups are contiguous).
            const uint32_t bbytes = gcols * K * 2;
            mbar_arrive_expect_tx(&ctl->bfull, bbytes);
            bulk_load(bres, a.enc_b + size_t(col0) * K, bbytes, &ctl->bfull);
            // This thread's own copy: it must land before the CTA can leave.
            bool ok = mbar_wait_own(&ctl->bfull, 0, a.status, kCtlSuspendNs);
            const uint32_t sbo = (K / 8) * 128;
            const uint32_t idesc = idesc_f16_f32(kTileRows, gcols);
            const uint32_t b_addr = smem_u32(bres);
            uint32_t ii = 0;
            for (uint32_t job = slot; ok && job < njobs; job += nslots, ++ii) {
                const uint32_t s = ii & 1, use = ii >> 1;
                ok = mbar_wait<QUICK>(&ctl->afull[s], use & 1, abort_flag, a.status, a.wait_limit_ns, kCtlSuspendNs);
                if (ok && ii >= 2)
                    ok = mbar_wait<QUICK>(&ctl->accempty[s], (use - 1) & 1, abort_flag, a.status, a.wait_limit_ns, kCtlSuspendNs);
                if (!ok) break;
                tc_fence_after();
                const uint32_t a_addr = smem_u32(tiles + s * tile_bytes);
                for (uint32_t ks = 0; ks < K / 16; ++ks)
                    mma_f16(tmem + s * 256, smem_desc(a_addr + ks * 256, 128, sbo),
                            smem_desc(b_addr + ks * 256, 128, sbo), idesc, ks > 0);
                mma_commit(&ctl->accfull[s]);
                mma_commit(&ctl->aempty[s]);
            }
            // This thread's own MMAs (ii jobs issued) retire before TMEM is freed.
            for (uint32_t back = 1; back <= 2 && back <= ii; ++back) {
                const uint32_t jj = ii - back;
                mbar_wait_own(&ctl->aempty[jj & 1], (jj >> 1) & 1, a.status, kCtlSuspendNs);
            }
        }
        __syncwarp();
    } else if (warp < kBuildWarps) {
        // ---- builders: thread = row of the tile.  The tile's input rows are
        // contiguous: one bulk copy stages them in the tail of the A buffer
        // being filled; every builder reads its row before any digit is
        // written (named barrier), so the in-place conversion is race free.
        const uint32_t grp = warp / kBuildGroupWarps;           // = the A buffer this group fills
        const uint32_t r = threadIdx.x - grp * kBuildGroupWarps * 32;
        const uint32_t stage_off = (tile_bytes - kTileRows * L * 4) & ~15u;
        const uint32_t bar_id = 1 + grp;                        // named barriers 1 and 2
        const uint32_t vote_id = 3 + grp;                       // 3 and 4: the group's joint decision
        uint32_t ii = grp;
        for (uint32_t job = slot + grp * nslots; job < njobs; job += 2 * nslots, ii += 2) {
            const uint32_t s = ii & 1, use = ii >> 1;
            // The MMA has released this buffer.  The group leaves together or
            // not at all: a thread that gave up alone would strand the others
            // at the group's named barrier below.
            const bool free_ok = ii < 2 || mbar_wait<QUICK>(&ctl->aempty[s], (use - 1) & 1, abort_flag, a.status,
                                                     a.wait_limit_ns);
            if (!named_sync_all(vote_id, kBuildGroupWarps * 32, free_ok)) break;
            const uint32_t tile = job % ntiles, operand = (job / ntiles) % a.operands;
            const uint32_t prod = job / (ntiles * a.operands);
            const uint32_t rows = min(kTileRows, a.N - tile * kTileRows);
            uint8_t* buf = tiles + s * tile_bytes;
            const uint32_t* staged = reinterpret_cast<const uint32_t*>(buf + stage_off);
            if (r == 0) {
                // Warm L2 with the input of the job after next.
                const uint32_t pj = job + 2 * nslots;
                if (pj < njobs) {
                    const uint32_t pt = pj % ntiles, po = (pj / ntiles) % a.operands, pp = pj / (ntiles * a.operands);
                    const uint32_t prow = min(kTileRows, a.N - pt * kTileRows);
                    bulk_prefetch_l2((po ? a.in1 : a.in0) + size_t(pp) * a.in_stride + size_t(pt) * kTileRows * L,
                                     prow * L * 4);
                }
                const uint32_t bytes = rows * L * 4;
                mbar_arrive_expect_tx(&ctl->infull[s], bytes);
                bulk_load(buf + stage_off,
                          (operand ? a.in1 : a.in0) + size_t(prod) * a.in_stride + size_t(tile) * kTileRows * L,
                          bytes, &ctl->infull[s]);
            }
            const bool valid = r < rows;
            // The group's own copy: every builder waits for it to land (never
            // cut short by the abort flag, so no copy is left in flight).
            const bool ok_in = mbar_wait_own(&ctl->infull[s], use & 1, a.status);
            uint32_t w[LT ? LT : 64];
#pragma unroll
            for (uint32_t l = 0; l < (LT ? uint32_t(LT) : 64u); ++l) {
                if (!LT && l >= L) break;
                w[l] = (valid && ok_in) ? staged[r * L + l] : 0u;
            }
            // Every row is read before any digit is written over the staging.
            asm volatile("bar.sync %0, %1;" :: "r"(bar_id), "r"(kBuildGroupWarps * 32) : "memory");
            if (valid) {
                digits_row<LT>(buf, r, w, L, K);
            } else {
                for (uint32_t kc = 0; kc < K / 8; ++kc)
                    *reinterpret_cast<uint4*>(buf + kmajor_offset(r, 8 * kc, K)) = make_uint4(0u, 0u, 0u, 0u);
            }
            fence_proxy_async();
            mbar_arrive(&ctl->afull[s]);
        }
    } else {
        // ---- epilogue: quarter of TMEM lanes, a quarter of the group's primes.
        const uint32_t e = warp - kBuildWarps;
        const uint32_t quarter = e & 3, part = e >> 2;        // part 0..kEpiPerQuarter-1
        const uint32_t r = quarter * 32 + lane;
        const uint32_t gp = gcols / 4;                        // primes in this group (incl. padding)
        const uint32_t per = (gp + kEpiPerQuarter - 1) / kEpiPerQuarter;
        const uint32_t p0 = part * per, p1 = min(gp, p0 + per);
        uint32_t ii = 0;
        for (uint32_t job = slot; job < njobs; job += nslots, ++ii) {
            const uint32_t s = ii & 1, use = ii >> 1;
            const bool ok = mbar_wait<QUICK>(&ctl->accfull[s], use & 1, abort_flag, a.status, a.wait_limit_ns);
            // The TMEM loads below are warp-collective: the warp leaves as one.
            if (!__all_sync(0xffffffffu, ok)) break;
            tc_fence_after();
            const uint32_t tile = job % ntiles, operand = (job / ntiles) % a.operands;
            const uint32_t prod = job / (ntiles * a.operands);
            const uint32_t i = tile * kTileRows + r;
            const bool valid = i < a.N;
            uint32_t* planes = (operand ? a.out1 : a.out0) + size_t(prod) * a.out_stride;
            const uint32_t taddr = tmem + ((quarter * 32) << 16) + s * 256;
            // Up to 60 primes per group (240 columns): at most 15 primes (60
            // columns) per warp, read 32 columns (8 primes) at a time.
#pragma unroll 1
            for (uint32_t cb = 0; cb < 2; ++cb) {
                if (cb * 8 >= p1 - p0) break;                       // warp-uniform
                float v[32];
                tmem_ld32(taddr + 4 * p0 + cb * 32, v);
                if (valid) {
#pragma unroll
                    for (uint32_t jj = 0; jj < 8; ++jj) {
                        const uint32_t lp = p0 + cb * 8 + jj;                 // prime within the group
                        const uint32_t j = g * (a.group_cols / 4) + lp;        // global prime
                        if (lp < p1 && j < a.P)
                            planes[size_t(j) * a.N + i] =
                                encode_residue(v[4 * jj], v[4 * jj + 1], v[4 * jj + 2], v[4 * jj + 3], a.prime[j]);
                    }
                }
            }
            tc_fence_before();
            mbar_arrive(&ctl->accempty[s]);
        }
    }
    tc_fence_before();
    __syncthreads();
    if (warp == kCtlWarp) {
        tc_fence_after();
        tmem_dealloc(tmem, 512);
    }
}

}  // namespace

// Column groups: the resident B of one group plus two A tiles must fit the
// 227 KB of shared memory; each group is at most 256 columns (one MMA).
uint32_t encode_group_cols(uint32_t cols, uint32_t K) {
    const uint32_t budget = 227 * 1024 - 2 * kTileRows * K * 2 - 1024 - sizeof(EncodeSmem);
    uint32_t groups = 1;
    while (true) {
        const uint32_t gc = ((cols + groups - 1) / groups + 15) / 16 * 16;
        if (gc <= 240 && gc * K * 2 <= budget) return gc;
        ++groups;
    }
}

size_t encode_smem_bytes(uint32_t K, uint32_t group_cols) {
    return size_t(2) * kTileRows * K * 2 + size_t(group_cols) * K * 2 + sizeof(EncodeSmem) + 1024;
}

static int sm_count() {
    static int n = 0;
    if (!n) {
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
        if (n <= 0) n = 1;
    }
    return n;
}

template <int LT>
static cudaError_t launch_encode_t(EncodeArgs a, uint32_t nprod, cudaStream_t st, uint32_t operands) {
    a.group_cols = encode_group_cols(a.cols, a.K);
    a.groups = (a.cols + a.group_cols - 1) / a.group_cols;
    a.nprod = nprod;
    a.operands = operands;
    const size_t smem = encode_smem_bytes(a.K, a.group_cols);
    auto* kern = quick_waits(a.wait_limit_ns) ? encode_kernel<LT, true> : encode_kernel<LT, false>;
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem));
    if (e != cudaSuccess) return e;
    const uint32_t ntiles = (a.N + kTileRows - 1) / kTileRows;
    const uint32_t jobs = nprod * operands * ntiles;
    uint32_t slots = uint32_t(sm_count()) / a.groups;
    if (slots < 1) slots = 1;
    if (slots > jobs) slots = jobs;
    kern<<<slots * a.groups, kEncThreads, smem, st>>>(a);
    return cudaGetLastError();
}

cudaError_t launch_encode(const EncodeArgs& a, uint32_t nprod, cudaStream_t st, uint32_t operands) {
    if (a.scalar) return launch_encode_scalar(a, nprod, st, operands);
    switch (a.L) {
        case 14: return launch_encode_t<14>(a, nprod, st, operands);
        case 28: return launch_encode_t<28>(a, nprod, st, operands);
        case 55: return launch_encode_t<55>(a, nprod, st, operands);
        default: return launch_encode_t<0>(a, nprod, st, operands);
    }
}

}  // namespace bcg
