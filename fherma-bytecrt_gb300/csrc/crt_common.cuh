// CRT helpers shared by the per-tile kernel (crt.cu) and the persistent
// warp-specialised kernel (crt_persistent.cu): K-chunk geometry, the signed
// carry chain over the TMEM digit sums, and the generic reduction mod q.
#pragma once

#include "common.cuh"
#include "kernels.hpp"

namespace bcg {
namespace crt_detail {

constexpr uint32_t kTileRows = 128;                      // coefficient rows per MMA tile (TMEM lanes)
constexpr uint32_t kTermsPerChunk = kCrtChunkK / 4;      // 8 terms x 4 digits per K chunk

__device__ __forceinline__ uint32_t chunk_k(uint32_t k_total, uint32_t kc) {
    const uint32_t rem = k_total - kc * kCrtChunkK;
    return rem >= kCrtChunkK ? kCrtChunkK : (rem + 15) / 16 * 16;
}


// One limb of the carry chain: S_0 + 256 S_1 + 2^16 S_2 + 2^24 S_3 + carry.
// With |S| < 2^23 and P < 127 the partial sums u, v fit int32; otherwise 64-bit.
__device__ __forceinline__ int64_t limb_value(float f0, float f1, float f2, float f3, bool narrow) {
    const int32_t s0 = __float2int_rn(f0), s1 = __float2int_rn(f1);
    const int32_t s2 = __float2int_rn(f2), s3 = __float2int_rn(f3);
    if (narrow) {
        const int32_t u = s3 * 256 + s2, v = s1 * 256 + s0;
        return int64_t(u) * 65536 + v;
    }
    return (int64_t(s3) << 24) + (int64_t(s2) << 16) + (int64_t(s1) << 8) + s0;
}

// Reduces the signed (L+1)-word value (z, top) mod q in place.  k is the
// floor of the quotient estimated in double precision from the top words
// (error far below 1), so after z - k q at most one correction remains.
template <int LT>
__device__ __forceinline__ void reduce_mod_q(uint32_t* z, int64_t top, const CrtArgs& a, uint32_t L) {
    double zhi = double(top);
    const uint32_t T = L < 3 ? L : 3;     // q_inv_scaled = 2^(32(L-T)) / q
#pragma unroll
    for (uint32_t tt = 0; tt < 3; ++tt)
        if (tt < T) zhi = zhi * 4294967296.0 + double(z[L - 1 - tt]);
    const int64_t k = int64_t(floor(zhi * a.q_inv_scaled));
    const bool neg = k < 0;
    const uint32_t ka = uint32_t(neg ? -k : k);
    int64_t c = 0;
#pragma unroll
    for (uint32_t l = 0; l < (LT ? LT : L); ++l) {
        const int64_t prod = int64_t(uint64_t(ka) * a.q[l]);
        const int64_t sum = int64_t(z[l]) + (neg ? prod : -prod) + c;
        z[l] = uint32_t(sum);
        c = sum >> 32;
    }
    top += c;
    if (top < 0) {
        uint64_t cc = 0;
#pragma unroll
        for (uint32_t l = 0; l < (LT ? LT : L); ++l) {
            const uint64_t sum = uint64_t(z[l]) + a.q[l] + cc;
            z[l] = uint32_t(sum);
            cc = sum >> 32;
        }
    } else {
        // d = z - q; keep d unless it borrowed out of the top word.
        int64_t b = 0;
        uint32_t d[LT ? LT : 1];
        if constexpr (LT > 0) {
#pragma unroll
            for (uint32_t l = 0; l < LT; ++l) {
                const int64_t sum = int64_t(z[l]) - int64_t(a.q[l]) + b;
                d[l] = uint32_t(sum);
                b = sum >> 32;
            }
            if (top + b >= 0) {
#pragma unroll
                for (uint32_t l = 0; l < LT; ++l) z[l] = d[l];
            }
        } else {
            bool ge = top > 0;
            if (!ge) {
                ge = true;
                for (int l = int(L) - 1; l >= 0; --l)
                    if (z[l] != a.q[l]) { ge = z[l] > a.q[l]; break; }
            }
            if (ge) {
                for (uint32_t l = 0; l < L; ++l) {
                    const int64_t sum = int64_t(z[l]) - int64_t(a.q[l]) + b;
                    z[l] = uint32_t(sum);
                    b = sum >> 32;
                }
            }
        }
    }
}

// Carry chain over one row's TMEM digit sums (TMEM address taddr): writes the
// low L limbs to z and returns the signed top word.  LT > 0: z is a register
// array (all indices fold after unrolling) and the TMEM reads are
// double-buffered; LT == 0: z is memory and L comes from the arguments.
template <int LT>
__device__ __forceinline__ int64_t crt_row_carry(const CrtArgs& a, uint32_t taddr, uint32_t* z) {
    const uint32_t L = LT ? uint32_t(LT) : a.L;
    const bool narrow = uint64_t(4) * (a.P + 1) * 16384u * 257u < (uint64_t(1) << 31);
    const bool extra = a.E == 4 * L + 1;
    int64_t carry = 0;
    if constexpr (LT > 0) {
        constexpr uint32_t NB = (4 * LT + 1 + 31) / 32;
        // Batch cb+1 is in flight while batch cb goes through the carry chain.
        uint32_t ra[32], rb[32];
        tmem_ld32_issue(taddr, ra);
        tmem_ld32_wait(ra);
#pragma unroll
        for (uint32_t cb = 0; cb < NB; ++cb) {
            uint32_t (&cur)[32] = (cb & 1) ? rb : ra;
            uint32_t (&nxt)[32] = (cb & 1) ? ra : rb;
            if (cb + 1 < NB) tmem_ld32_issue(taddr + (cb + 1) * 32, nxt);
#pragma unroll
            for (uint32_t q4 = 0; q4 < 8; ++q4) {
                const uint32_t l = cb * 8 + q4;
                if (l < LT) {
                    const int64_t sum = limb_value(__uint_as_float(cur[4 * q4]), __uint_as_float(cur[4 * q4 + 1]),
                                                   __uint_as_float(cur[4 * q4 + 2]), __uint_as_float(cur[4 * q4 + 3]),
                                                   narrow) + carry;
                    z[l] = uint32_t(sum);
                    carry = sum >> 32;
                } else if (l == LT && extra) {
                    carry += int64_t(__float2int_rn(__uint_as_float(cur[4 * q4])));
                }
            }
            if (cb + 1 < NB) tmem_ld32_wait(nxt);
        }
    } else {
        for (uint32_t cb = 0; cb < (a.E + 31) / 32; ++cb) {
            float v[32];
            tmem_ld32(taddr + cb * 32, v);
#pragma unroll
            for (uint32_t q4 = 0; q4 < 8; ++q4) {
                const uint32_t l = cb * 8 + q4;
                if (l < L) {
                    const int64_t sum = limb_value(v[4 * q4], v[4 * q4 + 1], v[4 * q4 + 2], v[4 * q4 + 3], narrow) + carry;
                    z[l] = uint32_t(sum);
                    carry = sum >> 32;
                } else if (l == L && extra) {
                    carry += int64_t(__float2int_rn(v[4 * q4]));
                }
            }
        }
    }
    return carry;
}

// Carry chain, reduction mod q, result to the shared staging row.
template <int LT>
__device__ __forceinline__ void crt_row_epilogue(const CrtArgs& a, uint32_t taddr, uint32_t* zrow, bool valid) {
    if constexpr (LT > 0) {
        uint32_t z[LT];
        const int64_t top = crt_row_carry<LT>(a, taddr, z);
        if (valid) reduce_mod_q<LT>(z, top, a, LT);
#pragma unroll
        for (uint32_t l = 0; l < LT; ++l) zrow[l] = z[l];
    } else {
        const int64_t top = crt_row_carry<0>(a, taddr, zrow);
        if (valid) reduce_mod_q<0>(zrow, top, a, a.L);
    }
}

}  // namespace crt_detail
}  // namespace bcg
