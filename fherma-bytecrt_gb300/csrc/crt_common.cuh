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

// q = 2^W - gap with 0 < gap < 2^32 and W > 70 (the form the reference's
// only reducer handles, native-smoke/g1-crt.cuh:13-68).  Here the CRT sum z
// is signed (balanced digits times weights in [0, q)), |z| < 2^17 q, so the
// fold works with the signed high part h = floor(z / 2^W), |h| <= 2^17:
// z <- (z mod 2^W) + h gap.  A first fold leaves z in [-2^49, 2^W + 2^49);
// a negative z then has h = -1 and the second fold gives z + q; otherwise z
// ends below 2q, and z >= q exactly when z + gap >= 2^W, in which case
// z - q = z + gap - 2^W.  Carries and borrows past the second limb are rare,
// so each propagation stops as soon as it dies out.
template <int LT>
__device__ __forceinline__ void reduce_gap_form(uint32_t* z, int64_t top, const CrtArgs& a, uint32_t L) {
    const uint32_t r = a.top_bits;                       // 1..32
    const uint32_t mask = r == 32 ? 0xffffffffu : (1u << r) - 1u;
    constexpr uint32_t LB = LT ? uint32_t(LT) : 64u;     // compile-time loop bounds keep z in registers
    int64_t over = top;                                  // signed value of the words above limb L-1
#pragma unroll
    for (int fold = 0; fold < 2; ++fold) {
        const int64_t high = r == 32 ? over : over * (int64_t(1) << (32 - r)) + int64_t(z[L - 1] >> r);
        z[L - 1] &= mask;
        const uint64_t m = uint64_t(high < 0 ? -high : high) * a.gap;       // < 2^49: two words
        const uint32_t w0 = uint32_t(m), w1 = uint32_t(m >> 32);
        if (high >= 0) {
            uint64_t s = uint64_t(z[0]) + w0;
            z[0] = uint32_t(s);
            s = uint64_t(z[1]) + w1 + (s >> 32);
            z[1] = uint32_t(s);
            uint32_t carry = uint32_t(s >> 32);
#pragma unroll
            for (uint32_t l = 2; l < LB; ++l) {
                if (!LT && l >= L) break;
                if (!carry) break;
                s = uint64_t(z[l]) + carry;
                z[l] = uint32_t(s);
                carry = uint32_t(s >> 32);
            }
            over = carry;
        } else {
            int64_t s = int64_t(z[0]) - int64_t(w0);
            z[0] = uint32_t(s);
            uint32_t borrow = s < 0;
            s = int64_t(z[1]) - int64_t(w1) - borrow;
            z[1] = uint32_t(s);
            borrow = s < 0;
#pragma unroll
            for (uint32_t l = 2; l < LB; ++l) {
                if (!LT && l >= L) break;
                if (!borrow) break;
                s = int64_t(z[l]) - 1;
                z[l] = uint32_t(s);
                borrow = s < 0;
            }
            over = -int64_t(borrow);
        }
    }
    // Now 0 <= z < 2q.  ge: z >= q, either bit W or above is set, or the low W
    // bits are at least 2^W - gap = [mask][all ones...][2^32 - gap].
    const int64_t high = r == 32 ? over : over * (int64_t(1) << (32 - r)) + int64_t(z[L - 1] >> r);
    bool ge = high != 0;
    if (!ge && (z[L - 1] & mask) == mask && z[0] >= 0u - a.gap) {
        ge = true;
#pragma unroll
        for (uint32_t l = 1; l + 1 < LB; ++l) {
            if (!LT && l + 1 >= L) break;
            if (z[l] != 0xffffffffu) { ge = false; break; }
        }
    }
    if (ge) {
        uint64_t s = uint64_t(z[0]) + a.gap;
        z[0] = uint32_t(s);
        uint32_t carry = uint32_t(s >> 32);
#pragma unroll
        for (uint32_t l = 1; l < LB; ++l) {
            if (!LT && l >= L) break;
            if (!carry) break;
            s = uint64_t(z[l]) + carry;
            z[l] = uint32_t(s);
            carry = uint32_t(s >> 32);
        }
        z[L - 1] &= mask;                                 // subtract 2^W
    }
}

// Reduces the signed (L+1)-word value (z, top) mod q in place.  k is the
// floor of the quotient estimated in double precision from the top words
// (error far below 1), so after z - k q at most one correction remains.
// GAP: -1 decide from a.gap at run time (uniform: a kernel argument), 0 generic
// only, 1 gap form only (a kernel instantiated per reducer keeps only one).
template <int LT, int GAP = -1>
__device__ __forceinline__ void reduce_mod_q(uint32_t* z, int64_t top, const CrtArgs& a, uint32_t L) {
    if (GAP == 1 || (GAP == -1 && a.gap)) {
        reduce_gap_form<LT>(z, top, a, L);
        return;
    }
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
