// Byte-matrix CRT reconstruction on tcgen05 (kind::f16), one fused kernel.
//
// Per coefficient, the terms are the P weighted residues t_j (canonical,
// t_j = c_j * inv(Prod/p_j) mod p_j) and alpha = round(sum_j t_j / p_j),
// computed in FP32 with separately rounded products and sums exactly as the
// reference does (native-smoke/g1-crt.cuh:249-257); the two-guard-bit bound
// |c/Prod| < 1/4 plus P*gamma_(P+4) < 1/4 makes it the exact nearest integer.
// With weights W_u = (Prod/p_u) mod q and W_P = (-Prod) mod q,
//     z = sum_u t_u * W_u = c (mod q).
// Each term is split into 4 balanced byte digits and each (256^a * W_u) mod q
// into crt_e balanced byte digits, so z = sum_e S_e 256^e where the digit sums
// S_e (|S_e| <= 4(P+1)*128*128 < 2^24) come exact from one fp32-accumulating
// MMA [256 x 4(P+1)] x [4(P+1) x crt_e].  This is the reference's four-column
// B4 algebra (native-smoke/README.md, g1-crt.cuh:201-335) with signed digits.
//
// Per K chunk (16 terms) one thread issues two bulk copies into a stage: the
// chunk of the weight-digit matrix, and the 16 t_j plane rows of the CTA's 256
// coefficients (1 KB each).  Eight producer warps (thread = coefficient row)
// turn the staged t_j into fp16 digits of the A tile and accumulate alpha.
//
// Epilogue per row (TMEM lane): signed 64-bit carry chain over the limbs, then
// a generic reduction mod q (the reference's reducer only handles
// q = 2^W - gap): a double-precision quotient estimate from the top words, one
// multiply-subtract of k*q and at most one correction.  Only canonical limbs
// are written, through a shared-memory staging tile for coalesced stores.
#include "common.cuh"
#include "crt_common.cuh"
#include "kernels.hpp"

namespace bcg {
namespace {

using namespace crt_detail;

// A CTA covers TILES M tiles of 128 coefficient rows: with 2 tiles every
// staged weight-digit chunk feeds two MMAs (half the L2 traffic for B); with
// 1 tile a CTA needs half the TMEM and shared memory, so two CTAs share an SM
// and one's epilogue overlaps the other's MMA loop.
constexpr uint32_t kStages = 4;
template <int TILES> struct CrtShape {
    static constexpr uint32_t kRows = kTileRows * TILES;
    static constexpr uint32_t kProdWarps = 4 * TILES;
    static constexpr uint32_t kThreads = (kProdWarps + 1) * 32;
    static constexpr uint32_t kMinBlocks = TILES == 1 ? 2 : 1;
};

struct CrtSmem {
    uint64_t afull[kStages], bfull[kStages], sempty[kStages], accfull;
    uint32_t tmem_base;
    uint32_t abort_flag;
};

template <int LT, int TILES, bool QUICK>
__global__ void __launch_bounds__(CrtShape<TILES>::kThreads, CrtShape<TILES>::kMinBlocks)
crt_kernel(const __grid_constant__ CrtArgs a) {
    constexpr uint32_t kTiles = TILES;
    constexpr uint32_t kRows = CrtShape<TILES>::kRows;
    constexpr uint32_t kProdWarps = CrtShape<TILES>::kProdWarps;
    extern __shared__ __align__(1024) uint8_t smem[];
    const uint32_t NC = a.NC;
    const uint32_t a_bytes = kRows * kCrtChunkK * 2;              // both tiles
    const uint32_t b_bytes = NC * kCrtChunkK * 2;
    const uint32_t t_bytes = kTermsPerChunk * kRows * 4;
    const uint32_t stage_bytes = a_bytes + b_bytes + t_bytes;
    CrtSmem* ctl = reinterpret_cast<CrtSmem*>(smem + kStages * stage_bytes);
    uint32_t* zbuf = reinterpret_cast<uint32_t*>(smem);          // epilogue staging (after all MMAs)
    volatile uint32_t* abort_flag = &ctl->abort_flag;
    auto stageA = [&](uint32_t s) { return smem + s * stage_bytes; };
    auto stageB = [&](uint32_t s) { return smem + s * stage_bytes + a_bytes; };
    auto stageT = [&](uint32_t s) { return reinterpret_cast<uint32_t*>(smem + s * stage_bytes + a_bytes + b_bytes); };

    const uint32_t warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const uint32_t prod = blockIdx.y;
    const uint32_t row0 = blockIdx.x * kRows;
    const uint32_t* terms = a.terms + size_t(prod) * a.terms_stride;
    uint32_t* out = a.out + size_t(prod) * a.out_stride;
    const uint32_t L = a.L, P = a.P, N = a.N;
    const uint32_t nkc = a.kchunks;
    const uint32_t rows = N - row0 < kRows ? N - row0 : kRows;

    if (threadIdx.x == 0) {
        for (int i = 0; i < int(kStages); ++i) {
            mbar_init(&ctl->afull[i], kRows);
            mbar_init(&ctl->bfull[i], 1);
            mbar_init(&ctl->sempty[i], 1);
        }
        mbar_init(&ctl->accfull, 1);
        ctl->abort_flag = 0;
        mbar_fence_init();
    }
    // One accumulator of NC fp32 columns per tile.
    const uint32_t tile_cols = NC <= 128 ? 128u : 256u;
    if (warp == kProdWarps) {
        tmem_alloc(&ctl->tmem_base, kTiles * tile_cols);
        tmem_relinquish();
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = ctl->tmem_base;

    if (warp == kProdWarps) {
        if (lane == 0) {
            // Stage s for chunk kc: weight digits + the staged t_j rows, one barrier.
            auto load = [&](uint32_t kc) {
                const uint32_t s = kc % kStages;
                const uint32_t bb = NC * chunk_k(a.k_total, kc) * 2;
                const uint32_t j0 = kc * kTermsPerChunk;
                const uint32_t nj = j0 < P ? min(kTermsPerChunk, P - j0) : 0u;
                mbar_arrive_expect_tx(&ctl->bfull[s], bb + nj * rows * 4);
                bulk_load(stageB(s), a.crt_b + size_t(kc) * kCrtChunkK * NC, bb, &ctl->bfull[s]);
                for (uint32_t jj = 0; jj < nj; ++jj)
                    bulk_load(stageT(s) + jj * kRows, terms + size_t(j0 + jj) * N + row0, rows * 4, &ctl->bfull[s]);
            };
            uint32_t loaded = 0;                       // chunks 0..loaded-1 were copied
            for (; loaded < kStages && loaded < nkc; ++loaded) load(loaded);
            const uint32_t idesc = idesc_f16_f32(kTileRows, NC);
            bool ok = true;
            uint32_t used = 0;                         // chunks whose bfull this thread saw complete
            for (uint32_t kc = 0; ok && kc < nkc; ++kc) {
                const uint32_t s = kc % kStages, sp = (kc / kStages) & 1;
                ok = mbar_wait<QUICK>(&ctl->afull[s], sp, abort_flag, a.status, a.wait_limit_ns);
                if (ok) ok = mbar_wait<QUICK>(&ctl->bfull[s], sp, abort_flag, a.status, a.wait_limit_ns);
                if (!ok) break;
                used = kc + 1;
                tc_fence_after();
                const uint32_t kl = chunk_k(a.k_total, kc);
                const uint32_t sbo = (kl / 8) * 128;
                const uint32_t b_addr = smem_u32(stageB(s));
                for (uint32_t t = 0; t < kTiles; ++t) {
                    const uint32_t a_addr = smem_u32(stageA(s)) + t * kTileRows * kl * 2;
                    for (uint32_t ks = 0; ks < kl / 16; ++ks)
                        mma_f16(tmem + t * tile_cols, smem_desc(a_addr + ks * 256, 128, sbo),
                                smem_desc(b_addr + ks * 256, 128, sbo), idesc, (kc | ks) != 0);
                }
                mma_commit(&ctl->sempty[s]);
                if (kc >= 1 && kc - 1 + kStages < nkc) {
                    // Chunk kc-1's MMAs retired: its stage (A, B and t_j) takes chunk kc-1+kStages.
                    const uint32_t pc = kc - 1;
                    ok = mbar_wait<QUICK>(&ctl->sempty[pc % kStages], (pc / kStages) & 1, abort_flag, a.status, a.wait_limit_ns);
                    if (ok) load(loaded++);
                }
            }
            // This thread's own work must finish before the CTA leaves: the
            // copies of chunks it never consumed (distinct stages), then every
            // MMA it issued (accfull completes when they have all retired).
            for (uint32_t c = used; c < loaded; ++c)
                mbar_wait_own(&ctl->bfull[c % kStages], (c / kStages) & 1, a.status);
            mma_commit(&ctl->accfull);
            mbar_wait_own(&ctl->accfull, 0, a.status);
        }
        __syncwarp();
    } else {
        const uint32_t r = threadIdx.x;                    // 0..kRows-1
        const uint32_t tile = r / kTileRows, trow = r % kTileRows;
        const bool valid = r < rows;
        float acc = 0.0f;
        bool ok = true;
        // ---- producer: balanced digits of t_j and alpha, 16 terms per K chunk.
        for (uint32_t kc = 0; ok && kc < nkc; ++kc) {
            const uint32_t s = kc % kStages;
            // bfull(kc) also implies chunk kc-kStages retired, so the A stage is free.
            ok = mbar_wait<QUICK>(&ctl->bfull[s], (kc / kStages) & 1, abort_flag, a.status, a.wait_limit_ns);
            if (!ok) break;
            const uint32_t kl = chunk_k(a.k_total, kc);
            uint8_t* tileA = stageA(s) + tile * kTileRows * kl * 2;
            const uint32_t* ts = stageT(s) + r;
            uint32_t t[kTermsPerChunk];
#pragma unroll
            for (uint32_t jj = 0; jj < kTermsPerChunk; ++jj) {
                const uint32_t u = kc * kTermsPerChunk + jj;
                t[jj] = (u < P && valid) ? ts[jj * kRows] : 0u;
            }
#pragma unroll
            for (uint32_t jj = 0; jj < kTermsPerChunk; ++jj) {
                const uint32_t u = kc * kTermsPerChunk + jj;
                if (u < P) acc = __fadd_rn(acc, __fmul_rn(__uint2float_rn(t[jj]), a.invp[u]));
                else if (u == P) t[jj] = __float2uint_rn(acc);
            }
#pragma unroll
            for (uint32_t pp = 0; pp < kTermsPerChunk / 2; ++pp) {
                if (16 * pp >= 2 * kl) break;
                uint32_t h[4];
#pragma unroll
                for (int half = 0; half < 2; ++half) {
                    const uint32_t u = kc * kTermsPerChunk + 2 * pp + half;
                    const uint32_t tb = t[2 * pp + half] + 0x808080u;
                    const bool live = u <= P;
                    h[2 * half] = live ? bytes01_to_half2(tb, kBias128x2) : 0u;
                    h[2 * half + 1] = live ? bytes23_to_half2(tb, kBias128_0) : 0u;
                }
                if (!valid) { h[0] = h[1] = h[2] = h[3] = 0; }
                *reinterpret_cast<uint4*>(tileA + kmajor_offset(trow, 8 * pp, kl)) = make_uint4(h[0], h[1], h[2], h[3]);
            }
            fence_proxy_async();
            mbar_arrive(&ctl->afull[s]);
        }

        // ---- epilogue.
        if (ok) ok = mbar_wait<QUICK>(&ctl->accfull, 0, abort_flag, a.status, a.wait_limit_ns);
        ok = __all_sync(0xffffffffu, ok);                   // the TMEM loads are warp-collective
        const uint32_t st = L | 1u;                        // odd staging stride
        if (ok) {
            tc_fence_after();
            const uint32_t taddr = tmem + (((warp & 3) * 32) << 16) + tile * tile_cols;
            crt_row_epilogue<LT>(a, taddr, zbuf + r * st, valid);
        }
        tc_fence_before();
        // Coalesced store of the staged rows (producer warps only).
        asm volatile("bar.sync 1, %0;" :: "r"(kProdWarps * 32) : "memory");
        for (uint32_t rr = warp; rr < rows; rr += kProdWarps) {
            uint32_t* dst = out + size_t(row0 + rr) * L;
            const uint32_t* srow = zbuf + rr * st;
            for (uint32_t l = lane; l < L; l += 32) dst[l] = srow[l];
        }
    }
    tc_fence_before();
    __syncthreads();
    if (warp == kProdWarps) {
        tc_fence_after();
        tmem_dealloc(tmem, kTiles * tile_cols);
    }
}

}  // namespace

size_t crt_smem_bytes(uint32_t NC, uint32_t tiles) {
    const size_t rows = size_t(kTileRows) * tiles;
    const size_t stage = rows * kCrtChunkK * 2 + size_t(NC) * kCrtChunkK * 2 + kTermsPerChunk * rows * 4;
    return kStages * stage + sizeof(CrtSmem) + 1024;
}

template <int LT, int TILES>
static cudaError_t launch_crt_t(const CrtArgs& a, uint32_t nprod, cudaStream_t st) {
    const size_t smem = crt_smem_bytes(a.NC, TILES);
    auto* kern = quick_waits(a.wait_limit_ns) ? crt_kernel<LT, TILES, true> : crt_kernel<LT, TILES, false>;
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem));
    if (e != cudaSuccess) return e;
    constexpr uint32_t rows = CrtShape<TILES>::kRows;
    const dim3 grid((a.N + rows - 1) / rows, nprod);
    kern<<<grid, CrtShape<TILES>::kThreads, smem, st>>>(a);
    return cudaGetLastError();
}

template <int TILES>
static cudaError_t launch_crt_tiles(const CrtArgs& a, uint32_t nprod, cudaStream_t st) {
    switch (a.L) {
        case 14: return launch_crt_t<14, TILES>(a, nprod, st);
        case 28: return launch_crt_t<28, TILES>(a, nprod, st);
        case 55: return launch_crt_t<55, TILES>(a, nprod, st);
        default: return launch_crt_t<0, TILES>(a, nprod, st);
    }
}

cudaError_t launch_crt(const CrtArgs& a, uint32_t nprod, cudaStream_t st, uint32_t tiles) {
    if (tiles == 1) return launch_crt_tiles<1>(a, nprod, st);
    if (tiles == 2) return launch_crt_tiles<2>(a, nprod, st);
    return cudaErrorInvalidValue;
}

}  // namespace bcg
