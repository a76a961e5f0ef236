// RNS encode on the 5th-generation tensor cores (tcgen05, kind::f16).
//
// For one tile of 128 coefficients and every prime p_j:
//     x_j = sum_k digit_k(coefficient) * (2^(8k+32) mod p_j)
// as a GEMM [128 x K] x [K x 4P'] where both operands are balanced base-256
// digits (|digit| <= 128, exact in fp16) and the 4 output columns of a prime
// are the 4 balanced digits of 2^(8k+32) mod p_j.  Every digit sum is an
// integer of magnitude <= K*128*128 < 2^22, exact in the fp32 accumulator.
// The epilogue reassembles x_j = sum_d S_d 256^d (|x| < 2^46) and applies one
// signed Montgomery reduction, which removes the 2^32 folded into the powers:
// the result is the coefficient mod p_j, in [0, 2p_j).
//
// The reference computes the same residues with u8 mma.sync byte dots and a
// u64 Barrett (native-smoke/rns-encode-mma.cuh:15-52, 148-252).  Balanced
// digits make the fp16 path exact; it replaces the int8 path, whose tensor
// rate on GB300 is far below the fp16 rate.
//
// Warp roles (160 threads): warps 0-3 build the A tile (thread = row) and run
// the epilogue for their TMEM lane quarter; warp 4 allocates TMEM, streams the
// B chunks (64 columns = 16 primes) through two shared-memory stages with
// bulk async copies, and issues the MMAs from one thread.  TMEM holds two
// 64-column accumulators so the epilogue of chunk c overlaps the MMAs of c+1.
#include "common.cuh"
#include "kernels.hpp"

namespace bcg {
namespace {

constexpr uint32_t kTileRows = 128;
constexpr uint32_t kEncThreads = 160;
constexpr uint32_t kEncTmemCols = 128;

struct EncodeSmem {
    uint64_t bfull[2], bempty[2], accfull[2], accempty[2], afull;
    uint32_t tmem_base;
    uint32_t abort_flag;
};

__global__ void __launch_bounds__(kEncThreads, 1)
encode_kernel(EncodeArgs a) {
    extern __shared__ __align__(1024) uint8_t smem[];
    const uint32_t K = a.K;
    uint8_t* tileA = smem;                                           // 128 x K fp16
    uint8_t* stageB = smem + kTileRows * K * 2;                      // 2 x 64 x K fp16
    EncodeSmem* ctl = reinterpret_cast<EncodeSmem*>(stageB + 2 * kEncChunkCols * K * 2);
    volatile uint32_t* abort_flag = &ctl->abort_flag;

    const uint32_t warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const uint32_t operand = blockIdx.y, prod = blockIdx.z;
    const uint32_t row0 = blockIdx.x * kTileRows;
    const uint32_t* in = (operand ? a.in1 : a.in0) + size_t(prod) * a.in_stride;
    uint32_t* planes = (operand ? a.out1 : a.out0) + size_t(prod) * a.out_stride;

    if (threadIdx.x == 0) {
        for (int i = 0; i < 2; ++i) {
            mbar_init(&ctl->bfull[i], 1);
            mbar_init(&ctl->bempty[i], 1);
            mbar_init(&ctl->accfull[i], 1);
            mbar_init(&ctl->accempty[i], kTileRows);
        }
        mbar_init(&ctl->afull, kTileRows);
        ctl->abort_flag = 0;
        mbar_fence_init();
    }
    if (warp == 4) {
        tmem_alloc(&ctl->tmem_base, kEncTmemCols);
        tmem_relinquish();
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = ctl->tmem_base;
    const uint32_t nchunks = a.chunks;

    if (warp == 4) {
        if (lane == 0) {
            auto chunk_cols = [&](uint32_t c) { return min(kEncChunkCols, a.cols - c * kEncChunkCols); };
            auto load_chunk = [&](uint32_t c) {
                const uint32_t bytes = chunk_cols(c) * K * 2;
                mbar_arrive_expect_tx(&ctl->bfull[c & 1], bytes);
                bulk_load(stageB + (c & 1) * kEncChunkCols * K * 2,
                          a.enc_b + size_t(c) * kEncChunkCols * K, bytes, &ctl->bfull[c & 1]);
            };
            load_chunk(0);
            if (nchunks > 1) load_chunk(1);
            bool ok = mbar_wait(&ctl->afull, 0, abort_flag, a.status);
            for (uint32_t c = 0; ok && c < nchunks; ++c) {
                if (c >= 2) ok = mbar_wait(&ctl->accempty[c & 1], ((c >> 1) - 1) & 1, abort_flag, a.status);
                if (ok) ok = mbar_wait(&ctl->bfull[c & 1], (c >> 1) & 1, abort_flag, a.status);
                if (!ok) break;
                tc_fence_after();
                const uint32_t n = chunk_cols(c);
                const uint32_t idesc = idesc_f16_f32(kTileRows, n);
                const uint32_t a_addr = smem_u32(tileA);
                const uint32_t b_addr = smem_u32(stageB + (c & 1) * kEncChunkCols * K * 2);
                const uint32_t sbo = (K / 8) * 128;
                for (uint32_t ks = 0; ks < K / 16; ++ks) {
                    const uint64_t ad = smem_desc(a_addr + ks * 256, 128, sbo);
                    const uint64_t bd = smem_desc(b_addr + ks * 256, 128, sbo);
                    mma_f16(tmem + (c & 1) * 64, ad, bd, idesc, ks > 0);
                }
                mma_commit(&ctl->accfull[c & 1]);
                mma_commit(&ctl->bempty[c & 1]);
                if (c >= 1 && c + 1 < nchunks) {
                    // Stage of chunk c-1 is free once its MMAs retired; refill with c+1.
                    ok = mbar_wait(&ctl->bempty[(c - 1) & 1], ((c - 1) >> 1) & 1, abort_flag, a.status);
                    if (ok) load_chunk(c + 1);
                }
            }
            // Drain: the last commits must land before TMEM is freed.
            if (nchunks >= 1) mbar_wait(&ctl->bempty[(nchunks - 1) & 1], ((nchunks - 1) >> 1) & 1, abort_flag, a.status);
            if (nchunks >= 2) mbar_wait(&ctl->bempty[(nchunks - 2) & 1], ((nchunks - 2) >> 1) & 1, abort_flag, a.status);
        }
        __syncwarp();
    } else {
        // ---- A tile: balanced digits of this thread's coefficient row.
        const uint32_t r = threadIdx.x;                 // 0..127
        const uint32_t i = row0 + r;
        const bool valid = i < a.N;
        const uint32_t* src = in + size_t(i) * a.L;
        uint32_t carry = 0;
        const uint32_t L = a.L;
        for (uint32_t kc = 0; kc < K / 8; ++kc) {       // 8 digits = 2 input words per store
            uint32_t h[4];
#pragma unroll
            for (int half = 0; half < 2; ++half) {
                const uint32_t l = 2 * kc + half;
                uint32_t lo0 = 0, lo1 = 0;
                if (l < L) {
                    const uint32_t w = valid ? __ldg(src + l) : 0u;
                    const uint64_t s = uint64_t(w) + 0x80808080u + carry;
                    const uint32_t v = uint32_t(s);
                    carry = uint32_t(s >> 32);
                    lo0 = bytes01_to_half2(v, kBias128x2);
                    lo1 = bytes23_to_half2(v, kBias128x2);
                } else if (l == L && valid && carry) {
                    lo0 = 0x00003C00u;      // fp16 1.0 in the low half: the carry digit
                    carry = 0;
                }
                h[2 * half] = lo0;
                h[2 * half + 1] = lo1;
            }
            if (!valid) { h[0] = h[1] = h[2] = h[3] = 0; }
            *reinterpret_cast<uint4*>(tileA + kmajor_offset(r, 8 * kc, K)) = make_uint4(h[0], h[1], h[2], h[3]);
        }
        fence_proxy_async();
        mbar_arrive(&ctl->afull);

        // ---- Epilogue: residues for this thread's row, chunk by chunk.
        const uint32_t quarter = warp;                  // TMEM lanes 32*warp .. +31
        for (uint32_t c = 0; c < nchunks; ++c) {
            if (!mbar_wait(&ctl->accfull[c & 1], (c >> 1) & 1, abort_flag, a.status)) break;
            tc_fence_after();
            const uint32_t n = min(kEncChunkCols, a.cols - c * kEncChunkCols);
            float v[64];
            {
                float t0[32];
                tmem_ld32(tmem + ((quarter * 32) << 16) + (c & 1) * 64, t0);
#pragma unroll
                for (int q = 0; q < 32; ++q) v[q] = t0[q];
                if (n > 32) {
                    tmem_ld32(tmem + ((quarter * 32) << 16) + (c & 1) * 64 + 32, t0);
#pragma unroll
                    for (int q = 0; q < 32; ++q) v[32 + q] = t0[q];
                }
            }
            tc_fence_before();
            mbar_arrive(&ctl->accempty[c & 1]);
            if (valid) {
#pragma unroll
                for (uint32_t jj = 0; jj < 16; ++jj) {
                    if (4 * jj >= n) break;
                    const uint32_t j = c * 16 + jj;
                    if (j >= a.P) break;
                    const uint4 pc = __ldg(a.consts + j);
                    const int32_t y0 = small_float_to_int(v[4 * jj]);
                    const int32_t y1 = small_float_to_int(v[4 * jj + 1]);
                    const int32_t y2 = small_float_to_int(v[4 * jj + 2]);
                    const int32_t y3 = small_float_to_int(v[4 * jj + 3]);
                    const int64_t x = int64_t(y0) + (int64_t(y1) << 8) + (int64_t(y2) << 16) + (int64_t(y3) << 24);
                    // Signed Montgomery: (x - m p) / 2^32 with m = x * p^-1 mod 2^32.
                    const uint32_t m = uint32_t(x) * pc.y;
                    const int32_t t = int32_t(x >> 32) - int32_t(__umulhi(m, pc.x));
                    int32_t res = t + int32_t(pc.x);
                    res = res < 0 ? res + int32_t(pc.x) : res;
                    planes[size_t(j) * a.N + i] = uint32_t(res);
                }
            }
        }
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 4) {
        tc_fence_after();
        tmem_dealloc(tmem, kEncTmemCols);
    }
}

}  // namespace

size_t encode_smem_bytes(uint32_t K) {
    return size_t(kTileRows) * K * 2 + size_t(2) * kEncChunkCols * K * 2 + sizeof(EncodeSmem) + 1024;
}

cudaError_t launch_encode(const EncodeArgs& a, uint32_t nprod, cudaStream_t st, uint32_t operands) {
    const size_t smem = encode_smem_bytes(a.K);
    cudaError_t e = cudaFuncSetAttribute(encode_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem));
    if (e != cudaSuccess) return e;
    const dim3 grid((a.N + kTileRows - 1) / kTileRows, operands, nprod);
    encode_kernel<<<grid, kEncThreads, smem, st>>>(a);
    return cudaGetLastError();
}

}  // namespace bcg
