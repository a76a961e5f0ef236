// Negacyclic NTT product per RNS prime, on the INT32 pipe.
//
// A residue plane holds one prime's N coefficients in natural order, viewed as
// C rows of R = min(N, 256) contiguous words (N = C * R).  The length-N
// negacyclic transform splits into
//   * a column pass: levels 0..c-1 of the merged (twist-free) Cooley-Tukey
//     negacyclic NTT, whose butterflies pair rows of the same column and whose
//     twiddles psi^(R * brv_c(2^l + blk)) are shared by every column;
//   * a row pass: after it, row i2 holds a(X) mod (X^R - tau^R) with
//     tau = psi^(2*brv_c(i2)+1); twisting element s by tau^s turns it into a
//     cyclic R-point NTT with fixed twiddles.
// The row kernel fuses the twisted forward transforms of A and B, their
// pointwise Montgomery product, the inverse cyclic transform and the untwist
// (whose table also carries N^-1 * inv(Prod/p_j) * 2^32, so the final plane
// holds the CRT terms t_j).  The inverse column pass then finishes the
// transform and leaves canonical t_j in [0, p).
//
// This replaces the reference's closed staged NTT (native-smoke/ntt-pipeline.cuh,
// ntt-weighted.cuh); only the per-prime negacyclic product and the t_j
// weighting are the same (native-smoke/ntt-smoke.cu:111-129,
// native-smoke/ntt-weighted.cuh:26-35).
#pragma once

#include "common.cuh"

namespace bcg {

struct NttArgs {
    const uint4* consts;       // per prime: p, p^-1, -p^-1, N^-1 * inv(Prod/p) * 2^32 mod p
    const uint2* tables;       // per prime: table_stride entries (value, Shoup companion)
    uint32_t table_stride;
    uint32_t off_col_f, off_col_i, off_row_f, off_row_i;
    uint32_t off_tw_lo, off_tw_hi, off_itw_lo, off_itw_hi;
    uint32_t N, P, c_bits, z_bits, Z, H;
    uint32_t R;                // row length of the split N = C * R
    uint32_t row_rows;         // rows of the row pass per CTA (0: the launcher's default)
    uint32_t row_local;        // log2 elements per thread in the row pass (0: 4 for R = 256, else 3)
    uint32_t row_pass;         // 0: row_kernel; 1: row_sliced_kernel (per-row twist tables)
};

// Bit positions handled inside one thread during phase `phase` of a transform
// over `bits` index bits with 2^LOCAL elements per thread: LOCAL positions
// (levels LOCAL*phase .. LOCAL*phase+LOCAL-1 pair bits bits-1-level; short
// phases are padded with the highest unused positions).
__host__ __device__ constexpr int phase_count(int bits, int local = 3) { return (bits + local - 1) / local; }

template <int BITS, int LOCAL>
struct PhaseMap {
    int local_pos[4];          // position for k bit LOCAL-1 .. 0 (only LOCAL used, LOCAL <= 4)
    int thread_pos[BITS];      // positions of thread-index bits, ascending
    int levels;                // levels in this phase
    int first_level;
    __host__ __device__ constexpr PhaseMap(int phase)
        : local_pos{0, 0, 0, 0}, thread_pos{}, levels(0), first_level(LOCAL * phase) {
        bool used[BITS > 0 ? BITS : 1] = {};
        int n = 0;
        for (int l = first_level; l < first_level + LOCAL && l < BITS; ++l) {
            local_pos[n++] = BITS - 1 - l;
            used[BITS - 1 - l] = true;
        }
        levels = n;
        for (int pos = BITS - 1; n < LOCAL && pos >= 0; --pos)
            if (!used[pos]) { local_pos[n++] = pos; used[pos] = true; }
        int m = 0;
        for (int pos = 0; pos < BITS; ++pos)
            if (!used[pos]) thread_pos[m++] = pos;
    }
    // Index of local element k (LOCAL bits) for thread t.
    __host__ __device__ constexpr uint32_t index(uint32_t t, uint32_t k) const {
        uint32_t s = 0;
        for (int i = 0; i < LOCAL; ++i) s |= ((k >> (LOCAL - 1 - i)) & 1u) << local_pos[i];
        for (int m = 0; m < BITS - LOCAL; ++m) s |= ((t >> m) & 1u) << thread_pos[m];
        return s;
    }
};

// Shared-memory word of element s inside a row buffer: XOR swizzle that keeps
// all three phase layouts of a 256-word row free of bank conflicts.
__device__ __forceinline__ uint32_t swz(uint32_t s) {
    const uint32_t h = (s >> 5) & 7u;
    return s ^ ((h << 2) | (h & 3u));
}

// In the first phase the block index of level l is k >> (LOCAL - l), known at
// compile time.  UNIT0: the transform's block-0 twiddles are 1 (the cyclic row
// transforms), so those butterflies skip the multiply.
template <int LOCAL>
__device__ __forceinline__ constexpr bool unit_block(int first_level, int li, uint32_t k) {
    return first_level == 0 && (k >> (LOCAL - li)) == 0;
}

// Forward CT levels of one phase on a thread's LOCAL elements; `twiddle(level, s)`.
template <int BITS, int LOCAL, bool UNIT0 = false, class Tw>
__device__ __forceinline__ void phase_ct(uint32_t (&x)[1 << LOCAL], const PhaseMap<BITS, LOCAL>& map,
                                         uint32_t t, uint32_t p, Tw twiddle) {
#pragma unroll
    for (int li = 0; li < map.levels; ++li) {
        const int level = map.first_level + li;
        const uint32_t bit = 1u << (LOCAL - 1 - li);
#pragma unroll
        for (uint32_t k = 0; k < (1u << LOCAL); ++k) {
            if (k & bit) continue;
            if (UNIT0 && unit_block<LOCAL>(map.first_level, li, k)) { bfly_ct_unit(x[k], x[k | bit], p); continue; }
            const uint32_t s = map.index(t, k);
            const uint2 w = twiddle(level, s);
            bfly_ct(x[k], x[k | bit], w, p);
        }
    }
}

template <int BITS, int LOCAL, bool UNIT0 = false, class Tw>
__device__ __forceinline__ void phase_gs(uint32_t (&x)[1 << LOCAL], const PhaseMap<BITS, LOCAL>& map,
                                         uint32_t t, uint32_t p, Tw twiddle) {
#pragma unroll
    for (int li = map.levels - 1; li >= 0; --li) {
        const int level = map.first_level + li;
        const uint32_t bit = 1u << (LOCAL - 1 - li);
#pragma unroll
        for (uint32_t k = 0; k < (1u << LOCAL); ++k) {
            if (k & bit) continue;
            if (UNIT0 && unit_block<LOCAL>(map.first_level, li, k)) { bfly_gs_unit(x[k], x[k | bit], p); continue; }
            const uint32_t s = map.index(t, k);
            const uint2 w = twiddle(level, s);
            bfly_gs(x[k], x[k | bit], w, p);
        }
    }
}

}  // namespace bcg
