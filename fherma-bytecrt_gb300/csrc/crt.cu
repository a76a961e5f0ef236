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
// MMA [128 x 4(P+1)] x [4(P+1) x crt_e].  This is the reference's four-column
// B4 algebra (native-smoke/README.md, g1-crt.cuh:201-335) with signed digits.
//
// Epilogue per row (TMEM lane): signed 64-bit carry chain over the limbs, then
// a generic reduction mod q (the reference's reducer only handles
// q = 2^W - gap): a double-precision quotient estimate from the top words, one
// multiply-subtract of k*q and at most one correction.  Only canonical limbs
// are written, through a shared-memory staging tile for coalesced stores.
#include "common.cuh"
#include "kernels.hpp"

namespace bcg {
namespace {

constexpr uint32_t kTileRows = 128;
constexpr uint32_t kCrtThreads = 160;
constexpr uint32_t kCrtTmemCols = 256;

struct CrtSmem {
    uint64_t afull[2], bfull[2], sempty[2], accfull;
    uint32_t tmem_base;
    uint32_t abort_flag;
    uint32_t q[64];
};

__device__ __forceinline__ uint32_t chunk_k(uint32_t k_total, uint32_t kc) {
    const uint32_t rem = k_total - kc * kCrtChunkK;
    return rem >= kCrtChunkK ? kCrtChunkK : (rem + 15) / 16 * 16;
}

__global__ void __launch_bounds__(kCrtThreads, 1)
crt_kernel(CrtArgs a) {
    extern __shared__ __align__(1024) uint8_t smem[];
    const uint32_t NC = a.NC;
    const uint32_t a_bytes = kTileRows * kCrtChunkK * 2;
    const uint32_t b_bytes = NC * kCrtChunkK * 2;
    uint8_t* stageA = smem;                          // 2 x a_bytes
    uint8_t* stageB = smem + 2 * a_bytes;            // 2 x b_bytes
    CrtSmem* ctl = reinterpret_cast<CrtSmem*>(stageB + 2 * b_bytes);
    uint32_t* zbuf = reinterpret_cast<uint32_t*>(smem);   // epilogue staging (after all MMAs)
    volatile uint32_t* abort_flag = &ctl->abort_flag;

    const uint32_t warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const uint32_t prod = blockIdx.y;
    const uint32_t row0 = blockIdx.x * kTileRows;
    const uint32_t* terms = a.terms + size_t(prod) * a.terms_stride;
    uint32_t* out = a.out + size_t(prod) * a.out_stride;
    const uint32_t L = a.L, P = a.P, N = a.N;
    const uint32_t nkc = a.kchunks;

    if (threadIdx.x == 0) {
        for (int i = 0; i < 2; ++i) {
            mbar_init(&ctl->afull[i], kTileRows);
            mbar_init(&ctl->bfull[i], 1);
            mbar_init(&ctl->sempty[i], 1);
        }
        mbar_init(&ctl->accfull, 1);
        ctl->abort_flag = 0;
        mbar_fence_init();
    }
    for (uint32_t l = threadIdx.x; l < L; l += blockDim.x) ctl->q[l] = a.q[l];
    if (warp == 4) {
        tmem_alloc(&ctl->tmem_base, kCrtTmemCols);
        tmem_relinquish();
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = ctl->tmem_base;

    if (warp == 4) {
        if (lane == 0) {
            auto load_b = [&](uint32_t kc) {
                const uint32_t bytes = NC * chunk_k(a.k_total, kc) * 2;
                mbar_arrive_expect_tx(&ctl->bfull[kc & 1], bytes);
                bulk_load(stageB + (kc & 1) * b_bytes, a.crt_b + size_t(kc) * kCrtChunkK * NC, bytes,
                          &ctl->bfull[kc & 1]);
            };
            load_b(0);
            if (nkc > 1) load_b(1);
            const uint32_t idesc = idesc_f16_f32(kTileRows, NC);
            bool ok = true;
            for (uint32_t kc = 0; ok && kc < nkc; ++kc) {
                ok = mbar_wait(&ctl->afull[kc & 1], (kc >> 1) & 1, abort_flag, a.status);
                if (ok) ok = mbar_wait(&ctl->bfull[kc & 1], (kc >> 1) & 1, abort_flag, a.status);
                if (!ok) break;
                tc_fence_after();
                const uint32_t kl = chunk_k(a.k_total, kc);
                const uint32_t sbo = (kl / 8) * 128;
                const uint32_t a_addr = smem_u32(stageA + (kc & 1) * a_bytes);
                const uint32_t b_addr = smem_u32(stageB + (kc & 1) * b_bytes);
                for (uint32_t ks = 0; ks < kl / 16; ++ks)
                    mma_f16(tmem, smem_desc(a_addr + ks * 256, 128, sbo), smem_desc(b_addr + ks * 256, 128, sbo),
                            idesc, (kc | ks) != 0);
                mma_commit(&ctl->sempty[kc & 1]);
                if (kc >= 1 && kc + 1 < nkc) {
                    ok = mbar_wait(&ctl->sempty[(kc - 1) & 1], ((kc - 1) >> 1) & 1, abort_flag, a.status);
                    if (ok) load_b(kc + 1);
                }
            }
            mma_commit(&ctl->accfull);
        }
        __syncwarp();
    } else {
        const uint32_t r = threadIdx.x;
        const uint32_t i = row0 + r;
        const bool valid = i < N;
        float acc = 0.0f;
        bool ok = true;
        // ---- producer: balanced digits of t_j and alpha, 16 terms per K chunk.
        for (uint32_t kc = 0; kc < nkc; ++kc) {
            if (kc >= 2) ok = mbar_wait(&ctl->sempty[kc & 1], ((kc >> 1) - 1) & 1, abort_flag, a.status);
            if (!ok) break;
            uint8_t* tile = stageA + (kc & 1) * a_bytes;
            const uint32_t kl = chunk_k(a.k_total, kc);
            for (uint32_t pp = 0; pp < kl / 8; ++pp) {
                uint32_t h[4];
#pragma unroll
                for (int half = 0; half < 2; ++half) {
                    const uint32_t u = kc * 16 + 2 * pp + half;
                    uint32_t t = 0;
                    bool live = true;
                    if (u < P) {
                        t = valid ? __ldg(terms + size_t(u) * N + i) : 0u;
                        acc = __fadd_rn(acc, __fmul_rn(__uint2float_rn(t), __ldg(a.invp + u)));
                    } else if (u == P) {
                        t = __float2uint_rn(acc);
                    } else {
                        live = false;
                    }
                    const uint32_t tb = t + 0x808080u;
                    h[2 * half] = live ? bytes01_to_half2(tb, kBias128x2) : 0u;
                    h[2 * half + 1] = live ? bytes23_to_half2(tb, kBias128_0) : 0u;
                }
                if (!valid) { h[0] = h[1] = h[2] = h[3] = 0; }
                *reinterpret_cast<uint4*>(tile + kmajor_offset(r, 8 * pp, kl)) = make_uint4(h[0], h[1], h[2], h[3]);
            }
            fence_proxy_async();
            mbar_arrive(&ctl->afull[kc & 1]);
        }

        // ---- epilogue.
        if (ok) ok = mbar_wait(&ctl->accfull, 0, abort_flag, a.status);
        // All threads of the warp execute the TMEM loads (sync.aligned).
        const uint32_t st = L | 1u;                       // odd staging stride
        uint32_t* z = zbuf + r * st;
        int64_t carry = 0;
        if (ok) {
            tc_fence_after();
            const uint32_t taddr = tmem + ((warp * 32) << 16);
            const uint32_t ncol = a.E;
            for (uint32_t cb = 0; cb < (ncol + 31) / 32; ++cb) {
                float v[32];
                tmem_ld32(taddr + cb * 32, v);
#pragma unroll
                for (uint32_t q4 = 0; q4 < 8; ++q4) {
                    const uint32_t l = cb * 8 + q4;
                    if (l < L) {
                        const int64_t s = int64_t(__float2int_rn(v[4 * q4])) +
                                          (int64_t(__float2int_rn(v[4 * q4 + 1])) << 8) +
                                          (int64_t(__float2int_rn(v[4 * q4 + 2])) << 16) +
                                          (int64_t(__float2int_rn(v[4 * q4 + 3])) << 24) + carry;
                        z[l] = uint32_t(s);
                        carry = s >> 32;
                    } else if (l == L && ncol == 4 * L + 1) {
                        // Extra digit at 256^(4L) = 2^(32L) adds to the top word.
                        carry += int64_t(__float2int_rn(v[4 * q4]));
                    }
                }
            }
        }
        tc_fence_before();
        if (ok && valid) {
            // ---- generic reduction mod q.
            const uint32_t T = L < 3 ? L : 3;
            double zhi = double(carry);
            for (uint32_t t = 0; t < T; ++t) zhi = zhi * 4294967296.0 + double(z[L - 1 - t]);
            const int64_t k = int64_t(floor(zhi * a.q_inv_scaled));
            int64_t c = 0;
            for (uint32_t l = 0; l < L; ++l) {
                const int64_t s = int64_t(z[l]) - k * int64_t(ctl->q[l]) + c;
                z[l] = uint32_t(s);
                c = s >> 32;
            }
            const int64_t top = carry + c;
            if (top < 0) {
                uint64_t cc = 0;
                for (uint32_t l = 0; l < L; ++l) {
                    const uint64_t s = uint64_t(z[l]) + ctl->q[l] + cc;
                    z[l] = uint32_t(s);
                    cc = s >> 32;
                }
            } else {
                bool ge = top > 0;
                if (!ge) {
                    ge = true;
                    for (int l = int(L) - 1; l >= 0; --l) {
                        if (z[l] != ctl->q[l]) { ge = z[l] > ctl->q[l]; break; }
                    }
                }
                if (ge) {
                    int64_t b = 0;
                    for (uint32_t l = 0; l < L; ++l) {
                        const int64_t s = int64_t(z[l]) - int64_t(ctl->q[l]) + b;
                        z[l] = uint32_t(s);
                        b = s >> 32;
                    }
                }
            }
        }
        // Coalesced store of the staged tile (warps 0-3 only).
        asm volatile("bar.sync 1, 128;" ::: "memory");
        const uint32_t rows = N - row0 < kTileRows ? N - row0 : kTileRows;
        for (uint32_t rr = warp; rr < rows; rr += 4) {
            uint32_t* dst = out + size_t(row0 + rr) * L;
            const uint32_t* srow = zbuf + rr * st;
            for (uint32_t l = lane; l < L; l += 32) dst[l] = srow[l];
        }
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 4) {
        tc_fence_after();
        tmem_dealloc(tmem, kCrtTmemCols);
    }
}

}  // namespace

size_t crt_smem_bytes(uint32_t NC) {
    return size_t(2) * kTileRows * kCrtChunkK * 2 + size_t(2) * NC * kCrtChunkK * 2 + sizeof(CrtSmem) + 1024;
}

cudaError_t launch_crt(const CrtArgs& a, uint32_t nprod, cudaStream_t st) {
    const size_t smem = crt_smem_bytes(a.NC);
    cudaError_t e = cudaFuncSetAttribute(crt_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem));
    if (e != cudaSuccess) return e;
    const dim3 grid((a.N + kTileRows - 1) / kTileRows, nprod);
    crt_kernel<<<grid, kCrtThreads, smem, st>>>(a);
    return cudaGetLastError();
}

}  // namespace bcg
