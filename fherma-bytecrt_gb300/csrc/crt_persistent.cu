// Persistent, warp-specialised CRT reconstruction (same arithmetic as crt.cu).
//
// One CTA per SM walks the (product, 128-row tile) jobs.  Roles:
//   warp 0      loader: per K chunk, one bulk copy of the weight-digit chunk and
//               the 8 t_j plane rows of the tile into a stage (6 stages);
//   warp 1      MMA: tcgen05 kind::f16 into one of two TMEM accumulators;
//   warps 2-9   producers in two groups of four warps that take alternate
//               chunks: each thread turns its row's 8 terms of the chunk into
//               balanced fp16 digits and keeps its group's partial alpha sum;
//   warps 10-13 epilogue: carry chain, reduction mod q, one bulk store per tile.
// The two accumulators let the epilogue of tile i run while tile i+1 goes
// through the MMA loop; the epilogue hands its accumulator back as soon as
// its TMEM reads finish.  Stages flow across tile boundaries, so the copies of
// the next tile start while the current one is still in the MMA loop.
//
// alpha is the nearest integer to sum_j t_j / p_j; the plan's bound
// (|c/Prod| < 1/4 and P*gamma_(P+4) < 1/4) makes every summation order give
// that integer, so the two groups' partial sums per row (each in the
// reference's fp32 round-to-nearest arithmetic) give the reference's alpha.
//
// Every wait is bounded.  Roles never leave their loops early: once a wait
// gives up (ok = false) a thread skips its work but still reaches every named
// barrier its partners wait at; at the end the loader waits for its own
// copies and the MMA warp for its own MMAs before the TMEM is freed.
#include <algorithm>

#include "common.cuh"
#include "crt_common.cuh"
#include "kernels.hpp"

namespace bcg {
namespace {

using namespace crt_detail;

// Stages of the chunk ring: 7 where they fit in shared memory, else 6 (7 measured
// 18.8 -> 18.3 us per product at N=65536 with the waits' suspend hints; 5: 19.6).
constexpr uint32_t kMaxStages = 7;
constexpr uint32_t kLoadWarp = 0, kMmaWarp = 1, kProdWarp0 = 2, kEpiWarp0 = 10;
constexpr uint32_t kProdThreads = 8 * 32;
constexpr uint32_t kEpiThreads = 4 * 32;
constexpr uint32_t kPThreads = 14 * 32;
constexpr uint32_t kAccCols = 256;             // one accumulator (NC <= 256 fp32 columns)
// Waiting threads sleep up to this long per poll (14 warps wait at once; the
// epilogue's waits last a whole tile).  CRT 20.0 -> 18.9 us per product at N=65536.
constexpr uint32_t kSuspendNs = 20000;

struct PSmem {
    uint64_t bfull[kMaxStages], afull[kMaxStages], sempty[kMaxStages];
    uint64_t accfull[2], accempty[2], mma_done;
    uint32_t tmem_base;
    uint32_t abort_flag;
    float alpha_part[2][kTileRows];
};

__host__ __device__ constexpr uint32_t stage_bytes_for(uint32_t NC) {
    return kTileRows * kCrtChunkK * 2 + NC * kCrtChunkK * 2 + kTermsPerChunk * kTileRows * 4;
}
__host__ __device__ constexpr uint32_t zstage_bytes_for(uint32_t L) {
    return (kTileRows * L * 4 + 1023) / 1024 * 1024;        // rows at stride L, as in the output
}

size_t smem_bytes_for(uint32_t NC, uint32_t L, uint32_t stages) {
    return size_t(stages) * stage_bytes_for(NC) + zstage_bytes_for(L) + sizeof(PSmem) + 1024;
}
// The device's opt-in shared memory per block (227 KB on GB300), read once.
size_t smem_optin_bytes() {
    static int bytes = 0;
    if (!bytes) {
        int dev = 0, v = 0;
        if (cudaGetDevice(&dev) != cudaSuccess ||
            cudaDeviceGetAttribute(&v, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev) != cudaSuccess || v <= 0) {
            cudaGetLastError();
            v = 227 * 1024;
        }
        bytes = v;
    }
    return size_t(bytes);
}
uint32_t stages_for(uint32_t NC, uint32_t L) {
    return smem_bytes_for(NC, L, kMaxStages) <= smem_optin_bytes() ? kMaxStages : kMaxStages - 1;
}

__device__ __forceinline__ void named_sync(uint32_t id, uint32_t threads) {
    asm volatile("bar.sync %0, %1;" :: "r"(id), "r"(threads) : "memory");
}

template <int LT, int GAP, int kPStages, bool QUICK>
__global__ void __launch_bounds__(kPThreads, 1)
crt_persistent_kernel(const __grid_constant__ CrtArgs a, uint32_t nprod) {
    extern __shared__ __align__(1024) uint8_t smem[];
    const uint32_t NC = a.NC, N = a.N, P = a.P;
    const uint32_t L = LT ? uint32_t(LT) : a.L;
    const uint32_t nkc = a.kchunks;
    const uint32_t a_bytes = kTileRows * kCrtChunkK * 2;
    const uint32_t b_bytes = NC * kCrtChunkK * 2;
    const uint32_t stage_bytes = stage_bytes_for(NC);
    uint32_t* zstage = reinterpret_cast<uint32_t*>(smem + kPStages * stage_bytes);
    PSmem* ctl = reinterpret_cast<PSmem*>(smem + kPStages * stage_bytes + zstage_bytes_for(L));
    volatile uint32_t* abort_flag = &ctl->abort_flag;
    auto stageA = [&](uint32_t s) { return smem + s * stage_bytes; };
    auto stageB = [&](uint32_t s) { return smem + s * stage_bytes + a_bytes; };
    auto stageT = [&](uint32_t s) { return reinterpret_cast<uint32_t*>(smem + s * stage_bytes + a_bytes + b_bytes); };

    const uint32_t warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const uint32_t ntiles = (N + kTileRows - 1) / kTileRows;
    const uint32_t njobs = nprod * ntiles;
    const uint32_t alpha_chunk = P / kTermsPerChunk;      // the last chunk: terms up to P (alpha)

    if (threadIdx.x == 0) {
        for (uint32_t i = 0; i < kPStages; ++i) {
            mbar_init(&ctl->bfull[i], 1);
            mbar_init(&ctl->afull[i], kProdThreads / 2);   // one producer group per chunk
            mbar_init(&ctl->sempty[i], 1);
        }
        for (uint32_t b = 0; b < 2; ++b) {
            mbar_init(&ctl->accfull[b], 1);
            mbar_init(&ctl->accempty[b], kEpiThreads);
        }
        mbar_init(&ctl->mma_done, 1);
        ctl->abort_flag = 0;
        mbar_fence_init();
    }
    if (warp == kMmaWarp) {
        tmem_alloc(&ctl->tmem_base, 2 * kAccCols);
        tmem_relinquish();
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = ctl->tmem_base;

    if (warp == kLoadWarp) {
        if (lane == 0) {
            bool ok = true;
            uint32_t g = 0;
            for (uint32_t job = blockIdx.x; ok && job < njobs; job += gridDim.x) {
                const uint32_t prod = job / ntiles, row0 = (job % ntiles) * kTileRows;
                const uint32_t rows = min(kTileRows, N - row0);
                // Natural layout: the chunk's t_j rows are N words apart (one copy each);
                // tile-major: they are contiguous (one copy per chunk).
                const uint32_t* terms = a.terms + size_t(prod) * a.terms_stride +
                                        (a.terms_tiled ? size_t(row0) * P : size_t(row0));
                for (uint32_t kc = 0; kc < nkc; ++kc, ++g) {
                    const uint32_t s = g % kPStages;
                    if (g >= kPStages && !mbar_wait<QUICK>(&ctl->sempty[s], ((g / kPStages) - 1) & 1, abort_flag, a.status, a.wait_limit_ns, kSuspendNs)) {
                        ok = false;
                        break;
                    }
                    const uint32_t bb = NC * chunk_k(a.k_total, kc) * 2;
                    const uint32_t j0 = kc * kTermsPerChunk;
                    const uint32_t nj = j0 < P ? min(kTermsPerChunk, P - j0) : 0u;
                    mbar_arrive_expect_tx(&ctl->bfull[s], bb + nj * rows * 4);
                    bulk_load(stageB(s), a.crt_b + size_t(kc) * kCrtChunkK * NC, bb, &ctl->bfull[s]);
                    if (a.terms_tiled) {
                        if (nj) bulk_load(stageT(s), terms + size_t(j0) * kTileRows, nj * kTileRows * 4, &ctl->bfull[s]);
                    } else {
                        for (uint32_t jj = 0; jj < nj; ++jj)
                            bulk_load(stageT(s) + jj * kTileRows, terms + size_t(j0 + jj) * N, rows * 4, &ctl->bfull[s]);
                    }
                }
            }
            // Let the last copy into every stage land before the CTA can exit.
            for (uint32_t back = 1; back <= kPStages && back <= g; ++back) {
                const uint32_t gg = g - back;
                mbar_wait_own(&ctl->bfull[gg % kPStages], (gg / kPStages) & 1, a.status, kSuspendNs);
            }
        }
        __syncwarp();
    } else if (warp == kMmaWarp) {
        if (lane == 0) {
            const uint32_t idesc = idesc_f16_f32(kTileRows, NC);
            bool ok = true;
            uint32_t g = 0, it = 0;
            for (uint32_t job = blockIdx.x; ok && job < njobs; job += gridDim.x, ++it) {
                const uint32_t buf = it & 1;
                if (it >= 2 && !mbar_wait<QUICK>(&ctl->accempty[buf], ((it / 2) - 1) & 1, abort_flag, a.status, a.wait_limit_ns, kSuspendNs)) {
                    ok = false;
                    break;
                }
                tc_fence_after();
                for (uint32_t kc = 0; kc < nkc; ++kc, ++g) {
                    const uint32_t s = g % kPStages;
                    if (!mbar_wait<QUICK>(&ctl->afull[s], (g / kPStages) & 1, abort_flag, a.status, a.wait_limit_ns, kSuspendNs)) {
                        ok = false;
                        break;
                    }
                    tc_fence_after();
                    const uint32_t kl = chunk_k(a.k_total, kc);
                    const uint32_t sbo = (kl / 8) * 128;
                    const uint32_t a_addr = smem_u32(stageA(s)), b_addr = smem_u32(stageB(s));
                    for (uint32_t ks = 0; ks < kl / 16; ++ks)
                        mma_f16(tmem + buf * kAccCols, smem_desc(a_addr + ks * 256, 128, sbo),
                                smem_desc(b_addr + ks * 256, 128, sbo), idesc, (kc | ks) != 0);
                    mma_commit(&ctl->sempty[s]);   // stage s (A, B, t) free once these MMAs retire
                }
                if (ok) mma_commit(&ctl->accfull[buf]);
            }
            // Every MMA issued by this thread has retired once mma_done completes.
            mma_commit(&ctl->mma_done);
            mbar_wait_own(&ctl->mma_done, 0, a.status, kSuspendNs);
        }
        __syncwarp();
    } else if (warp < kEpiWarp0) {
        // ---- producers: two groups of four warps take alternate chunks (g even
        // or odd); in a group, thread = row, all 8 terms of the chunk.  One
        // group's chunk latency (wait, loads, conversion, fence, arrival)
        // overlaps the other's.  With an odd stage count a stage passes from
        // one group to the other between uses; a group still never falls two
        // phases behind a stage's bfull, because refilling the stage needs the
        // MMA of this group's chunk, hence this group's arrival.
        const uint32_t pt = threadIdx.x - kProdWarp0 * 32;
        const uint32_t row = pt % kTileRows, grp = pt / kTileRows;
        bool ok = true;
        uint32_t g = 0;
        for (uint32_t job = blockIdx.x; job < njobs; job += gridDim.x) {
            const uint32_t row0 = (job % ntiles) * kTileRows;
            const bool valid = row < min(kTileRows, N - row0);
            float acc = 0.0f;
            for (uint32_t kc = 0; kc < nkc; ++kc, ++g) {
                const bool mine = (g & 1u) == grp;
                if (kc == alpha_chunk && !mine) {
                    // Every term below P lies in a chunk before this one: hand
                    // the partial sum to the group that builds alpha's digits.
                    // Both groups pass this barrier once per tile (a blocking
                    // sync on both sides keeps the pairing exact even when
                    // waits have given up and threads run ahead).
                    ctl->alpha_part[grp][row] = acc;
                    named_sync(2, kProdThreads);
                }
                if (!mine) continue;
                const uint32_t s = g % kPStages;
                if (ok) ok = mbar_wait<QUICK>(&ctl->bfull[s], (g / kPStages) & 1, abort_flag, a.status, a.wait_limit_ns, kSuspendNs);
                const uint32_t kl = chunk_k(a.k_total, kc);
                const uint32_t* ts = stageT(s) + row;
                uint32_t t[kTermsPerChunk];
#pragma unroll
                for (uint32_t jj = 0; jj < kTermsPerChunk; ++jj) {
                    const uint32_t u = kc * kTermsPerChunk + jj;
                    t[jj] = (ok && u < P && valid) ? ts[jj * kTileRows] : 0u;
                }
#pragma unroll
                for (uint32_t jj = 0; jj < kTermsPerChunk; ++jj) {
                    const uint32_t u = kc * kTermsPerChunk + jj;
                    if (u < P) acc = __fadd_rn(acc, __fmul_rn(__uint2float_rn(t[jj]), a.invp[u]));
                }
                uint32_t alpha = 0;
                if (kc == alpha_chunk) {
                    // alpha = round(own partial + the other group's), the digits of term P.
                    named_sync(2, kProdThreads);
                    alpha = __float2uint_rn(__fadd_rn(acc, ctl->alpha_part[grp ^ 1u][row]));
                }
                if (ok) {
                    uint8_t* tileA = stageA(s);
#pragma unroll
                    for (uint32_t pp = 0; pp < kTermsPerChunk / 2; ++pp) {
                        const uint32_t kpos = 8 * pp;                      // first of this pair's 8 digits
                        if (kpos >= kl) break;
                        uint32_t h[4];
#pragma unroll
                        for (uint32_t hh = 0; hh < 2; ++hh) {
                            const uint32_t u = kc * kTermsPerChunk + 2 * pp + hh;
                            const uint32_t tb = (u == P ? alpha : t[2 * pp + hh]) + 0x808080u;
                            const bool live = u <= P && valid;
                            h[2 * hh] = live ? bytes01_to_half2(tb, kBias128x2) : 0u;
                            h[2 * hh + 1] = live ? bytes23_to_half2(tb, kBias128_0) : 0u;
                        }
                        *reinterpret_cast<uint4*>(tileA + kmajor_offset(row, kpos, kl)) =
                            make_uint4(h[0], h[1], h[2], h[3]);
                    }
                    fence_proxy_async();
                    mbar_arrive(&ctl->afull[s]);
                }
            }
        }
    } else {
        // ---- epilogue: TMEM lane quarter (warp % 4), one row per thread.  The
        // tile's rows are contiguous in the output, so they leave the staging
        // buffer with one bulk copy issued by the first epilogue thread.
        const uint32_t quarter = warp & 3;
        const uint32_t row = quarter * 32 + lane;
        const bool leader = threadIdx.x == kEpiWarp0 * 32;
        bool ok = true;
        uint32_t it = 0;
        for (uint32_t job = blockIdx.x; job < njobs; job += gridDim.x, ++it) {
            const uint32_t buf = it & 1;
            const uint32_t prod = job / ntiles, row0 = (job % ntiles) * kTileRows;
            const uint32_t rows = min(kTileRows, N - row0);
            const bool valid = row < rows;
            if (ok) ok = mbar_wait<QUICK>(&ctl->accfull[buf], (it / 2) & 1, abort_flag, a.status, a.wait_limit_ns, kSuspendNs);
            // The TMEM loads are warp-collective: a warp reads its lanes only if
            // every thread of it saw the accumulator complete.
            ok = __all_sync(0xffffffffu, ok);
            uint32_t z[LT ? LT : 1];
            int64_t top = 0;
            if (ok) {
                tc_fence_after();
                const uint32_t taddr = tmem + ((quarter * 32) << 16) + buf * kAccCols;
                if constexpr (LT > 0) {
                    top = crt_row_carry<LT>(a, taddr, z);
                    tc_fence_before();
                    mbar_arrive(&ctl->accempty[buf]);          // accumulator read: hand it back
                    if (valid) reduce_mod_q<LT, GAP>(z, top, a, LT);
                }
            }
            // The previous tile's bulk store has read the staging buffer.
            if (leader) bulk_store_wait_read();
            named_sync(1, kEpiThreads);
            uint32_t* zrow = zstage + row * L;
            if (ok) {
                if constexpr (LT > 0) {
#pragma unroll
                    for (uint32_t l = 0; l < LT; ++l) zrow[l] = z[l];
                } else {
                    const uint32_t taddr = tmem + ((quarter * 32) << 16) + buf * kAccCols;
                    top = crt_row_carry<0>(a, taddr, zrow);
                    tc_fence_before();
                    mbar_arrive(&ctl->accempty[buf]);
                    if (valid) reduce_mod_q<0, GAP>(zrow, top, a, L);
                }
            }
            fence_proxy_async();
            named_sync(1, kEpiThreads);
            if (leader && ok)
                bulk_store(a.out + size_t(prod) * a.out_stride + size_t(row0) * L, zstage, rows * L * 4);
        }
        if (leader) bulk_store_wait_all();
    }
    tc_fence_before();
    __syncthreads();
    if (warp == kMmaWarp) {
        tc_fence_after();
        tmem_dealloc(tmem, 2 * kAccCols);
    }
}

int sm_count_of_current_device() {
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    return sms > 0 ? sms : 1;
}

template <int LT, int GAP, int ST>
cudaError_t launch_persistent_t(const CrtArgs& a, uint32_t nprod, cudaStream_t st) {
    const size_t smem = smem_bytes_for(a.NC, a.L, ST);
    auto* kern = quick_waits(a.wait_limit_ns) ? crt_persistent_kernel<LT, GAP, ST, true>
                                              : crt_persistent_kernel<LT, GAP, ST, false>;
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem));
    if (e != cudaSuccess) return e;
    const uint32_t jobs = nprod * ((a.N + kTileRows - 1) / kTileRows);
    const uint32_t grid = std::min<uint32_t>(jobs, uint32_t(sm_count_of_current_device()));
    kern<<<grid, kPThreads, smem, st>>>(a, nprod);
    return cudaGetLastError();
}

// One instantiation per reducer: carrying both would raise register pressure.
template <int LT>
cudaError_t launch_persistent_l(const CrtArgs& a, uint32_t nprod, cudaStream_t st) {
    if (stages_for(a.NC, a.L) == kMaxStages)
        return a.gap ? launch_persistent_t<LT, 1, kMaxStages>(a, nprod, st) : launch_persistent_t<LT, 0, kMaxStages>(a, nprod, st);
    return a.gap ? launch_persistent_t<LT, 1, kMaxStages - 1>(a, nprod, st)
                 : launch_persistent_t<LT, 0, kMaxStages - 1>(a, nprod, st);
}

}  // namespace

size_t crt_persistent_smem_bytes(uint32_t NC, uint32_t L) {
    return smem_bytes_for(NC, L, stages_for(NC, L));
}

cudaError_t launch_crt_persistent(const CrtArgs& a, uint32_t nprod, cudaStream_t st) {
    if (a.NC > kAccCols) return cudaErrorInvalidValue;
    if (reinterpret_cast<uintptr_t>(a.out) & 15) return cudaErrorMisalignedAddress;   // bulk stores
    if (a.terms_tiled && (a.N < kTileRows || a.N % kTileRows)) return cudaErrorInvalidValue;
    switch (a.L) {
        case 14: return launch_persistent_l<14>(a, nprod, st);
        case 28: return launch_persistent_l<28>(a, nprod, st);
        case 55: return launch_persistent_l<55>(a, nprod, st);
        default: return launch_persistent_l<0>(a, nprod, st);
    }
}

}  // namespace bcg
