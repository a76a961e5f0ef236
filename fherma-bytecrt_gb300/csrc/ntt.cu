// NTT kernels (see ntt.cuh for the decomposition).
#include <algorithm>

#include "ntt.cuh"
#include "kernels.hpp"

namespace bcg {
namespace {

// Column pass: 16 elements per thread, 4 levels per phase (C = 256 takes two
// phases and one exchange; three-level phases took three and two, and
// measured slower).
__host__ __device__ constexpr int local_bits(int bits) { return bits < 4 ? bits : 4; }

// ------------------------------------------------------------ column pass --
// One CTA: 32 adjacent columns (lane = column) of one plane and one prime.
// Each thread keeps 16 elements of its column in registers per phase of four
// levels; between phases the tile goes through shared memory, one 128-byte
// row per warp access (conflict free).
template <int CB, bool INVERSE, int PH>
__device__ __forceinline__ void col_phase(uint32_t (&x)[1 << local_bits(CB)], uint32_t w, uint32_t p,
                                          const uint2* __restrict__ tw) {
    constexpr int LOCAL = local_bits(CB);
    constexpr PhaseMap<CB, LOCAL> map(PH);
    auto twiddle = [&](int level, uint32_t s) { return __ldg(tw + (1u << level) + (s >> (CB - level))); };
    if constexpr (INVERSE) phase_gs<CB, LOCAL>(x, map, w, p, twiddle);
    else phase_ct<CB, LOCAL>(x, map, w, p, twiddle);
}

template <int CB, int FROM, int TO>
__device__ __forceinline__ void col_exchange(uint32_t (&x)[1 << local_bits(CB)], uint32_t* buf,
                                             uint32_t w, uint32_t lane) {
    constexpr int LOCAL = local_bits(CB);
    constexpr PhaseMap<CB, LOCAL> from(FROM), to(TO);
#pragma unroll
    for (uint32_t k = 0; k < (1u << LOCAL); ++k) buf[from.index(w, k) * 32 + lane] = x[k];
    __syncthreads();
#pragma unroll
    for (uint32_t k = 0; k < (1u << LOCAL); ++k) x[k] = buf[to.index(w, k) * 32 + lane];
    __syncthreads();
}

// TILED (inverse only): the terms leave in the CRT's tile-major layout, the
// 128 coefficients of a tile contiguous per prime, [N/128][P][128], in a
// separate buffer `out` (a CTA's tile-major positions are other CTAs' inputs).
template <int CB, bool INVERSE, bool TILED = false>
__global__ void __launch_bounds__(32 * ((1 << CB) >> local_bits(CB)))
col_kernel(NttArgs a, uint32_t* __restrict__ planes, size_t plane_stride, uint32_t* __restrict__ out) {
    constexpr int LOCAL = local_bits(CB);
    constexpr int NPH = phase_count(CB, LOCAL);
    static_assert(NPH <= 2, "the column pass handles C <= 256 in at most two phases");
    const uint32_t R = a.R;                 // column stride: the row length
    __shared__ uint32_t buf[(1 << CB) * 32];
    const uint32_t lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const uint32_t j = blockIdx.y;
    const uint32_t p = a.consts[j].x;
    uint32_t* col = planes + size_t(blockIdx.z) * plane_stride + size_t(j) * a.N + blockIdx.x * 32 + lane;
    const uint2* tw = a.tables + size_t(j) * a.table_stride + (INVERSE ? a.off_col_i : a.off_col_f);
    uint32_t x[1 << LOCAL];
    constexpr int first = INVERSE ? NPH - 1 : 0;
    constexpr int last = INVERSE ? 0 : NPH - 1;
    {
        constexpr PhaseMap<CB, LOCAL> m(first);
#pragma unroll
        for (uint32_t k = 0; k < (1u << LOCAL); ++k) x[k] = col[size_t(m.index(w, k)) * R];
    }
    if constexpr (!INVERSE) {
        col_phase<CB, false, 0>(x, w, p, tw);
        if constexpr (NPH > 1) { col_exchange<CB, 0, 1>(x, buf, w, lane); col_phase<CB, false, 1>(x, w, p, tw); }
        if constexpr (NPH > 2) { col_exchange<CB, 1, 2>(x, buf, w, lane); col_phase<CB, false, 2>(x, w, p, tw); }
    } else {
        if constexpr (NPH > 2) { col_phase<CB, true, 2>(x, w, p, tw); col_exchange<CB, 2, 1>(x, buf, w, lane); }
        if constexpr (NPH > 1) { col_phase<CB, true, 1>(x, w, p, tw); col_exchange<CB, 1, 0>(x, buf, w, lane); }
        col_phase<CB, true, 0>(x, w, p, tw);
#pragma unroll
        for (uint32_t k = 0; k < (1u << LOCAL); ++k) x[k] = reduce_once(x[k], p);
    }
    {
        constexpr PhaseMap<CB, LOCAL> m(last);
        if constexpr (TILED) {
            uint32_t* base = out + size_t(blockIdx.z) * plane_stride + (size_t(j) << 7);
#pragma unroll
            for (uint32_t k = 0; k < (1u << LOCAL); ++k) {
                const uint32_t i = blockIdx.x * 32 + lane + m.index(w, k) * R;
                base[size_t(i >> 7) * (size_t(a.P) << 7) + (i & 127u)] = x[k];
            }
        } else {
#pragma unroll
            for (uint32_t k = 0; k < (1u << LOCAL); ++k) col[size_t(m.index(w, k)) * R] = x[k];
        }
    }
}

// --------------------------------------------------------------- row pass --
// TPR = R / 2^RL threads per row, 2^RL elements each; a warp holds 32/TPR
// rows.  Per row: twist A and B, forward cyclic NTTs, Montgomery pointwise
// product, inverse cyclic NTT, untwist (with the CRT weight), store into A's
// plane.  RL = 4 (R = 256: two phases of four levels, one exchange per
// transform) or RL = 3 (three-level phases, for the shorter rows).
constexpr int kRowWarps = 8;

// Row buffer geometry: 16 words of padding per row when RL = 4 put the two
// rows of a warp on opposite bank halves.
template <int RB, int RL> struct RowShape {
    static constexpr uint32_t R = 1u << RB;
    static constexpr uint32_t TPR = R >> RL;
    static constexpr uint32_t RPW = 32 / TPR;
    static constexpr uint32_t kPad = RL == 4 ? 16u : 0u;
    static constexpr uint32_t kWarpWords = RPW * (R + kPad);   // one operand's rows of a warp
};

// Shared-memory word of element s inside a row buffer.  RL = 3: swz() keeps
// the three phase layouts conflict free.  RL = 4: phase 0 writes s = 16k + t
// and phase 1 reads s = 16t + k; XOR-ing the low nibble with the high one
// spreads both over distinct banks.
template <int RL>
__device__ __forceinline__ uint32_t row_word(uint32_t s) {
    if constexpr (RL == 4) return s ^ ((s >> 4) & 15u);
    else return swz(s);
}

// Row twiddle tables in shared memory.  Level l uses entries 2^l + u,
// u = s >> (RB - l).  With R = 256 and 16 elements per thread, phase 1
// (levels 4-7) holds s = 16t + k, so u = t * 2^(l-4) + c with c from k: in
// natural order the 16 threads of a row would read entries 2^(l-4) apart
// (up to 8-way bank conflicts on the 8-byte entries).  Those levels are
// stored c-major instead, entry 2^l + c*16 + t, so the threads of a row read
// 16 consecutive entries.  Phase 0 reads one entry per level for all threads
// (a broadcast) and keeps the natural order.
template <int RB, int RL>
__host__ __device__ constexpr bool row_tw_cmajor() { return RB == 8 && RL == 4; }

// Position of natural entry i (1 <= i < R) in the shared-memory table.
template <int RB, int RL>
__device__ __forceinline__ uint32_t row_tw_slot(uint32_t i) {
    if constexpr (row_tw_cmajor<RB, RL>()) {
        if (i < 16) return i;
        const uint32_t l = 31u - __clz(i), u = i - (1u << l);
        return (1u << l) + ((u & ((1u << (l - 4)) - 1u)) << 4) + (u >> (l - 4));
    } else {
        return i;
    }
}

template <int RB, int RL>
__device__ __forceinline__ uint2 row_twiddle(const uint2* tab, int level, uint32_t s) {
    const uint32_t u = s >> (RB - level);
    if constexpr (row_tw_cmajor<RB, RL>()) {
        if (level >= 4) return tab[(1u << level) + ((u & ((1u << (level - 4)) - 1u)) << 4) + (s >> 4)];
    }
    return tab[(1u << level) + u];
}

template <int RB, int RL, int PH>
__device__ __forceinline__ void row_fwd_phase(uint32_t (&x)[1 << RL], uint32_t t, uint32_t p, const uint2* rf) {
    constexpr PhaseMap<RB, RL> map(PH);
    phase_ct<RB, RL, true>(x, map, t, p, [&](int level, uint32_t s) { return row_twiddle<RB, RL>(rf, level, s); });
}
template <int RB, int RL, int PH>
__device__ __forceinline__ void row_inv_phase(uint32_t (&x)[1 << RL], uint32_t t, uint32_t p, const uint2* ri) {
    constexpr PhaseMap<RB, RL> map(PH);
    phase_gs<RB, RL, true>(x, map, t, p, [&](int level, uint32_t s) { return row_twiddle<RB, RL>(ri, level, s); });
}
template <int RB, int RL, int FROM, int TO>
__device__ __forceinline__ void row_exchange(uint32_t (&x)[1 << RL], uint32_t* rowbuf, uint32_t t) {
    constexpr PhaseMap<RB, RL> from(FROM), to(TO);
#pragma unroll
    for (uint32_t k = 0; k < (1u << RL); ++k) rowbuf[row_word<RL>(from.index(t, k))] = x[k];
    __syncwarp();
#pragma unroll
    for (uint32_t k = 0; k < (1u << RL); ++k) x[k] = rowbuf[row_word<RL>(to.index(t, k))];
    __syncwarp();
}

template <int RB, int RL>
__device__ __forceinline__ void row_forward(uint32_t (&x)[1 << RL], uint32_t* rowbuf, uint32_t t, uint32_t p,
                                            const uint2* rf) {
    constexpr int NPH = phase_count(RB, RL);
    row_fwd_phase<RB, RL, 0>(x, t, p, rf);
    if constexpr (NPH > 1) { row_exchange<RB, RL, 0, 1>(x, rowbuf, t); row_fwd_phase<RB, RL, 1>(x, t, p, rf); }
    if constexpr (NPH > 2) { row_exchange<RB, RL, 1, 2>(x, rowbuf, t); row_fwd_phase<RB, RL, 2>(x, t, p, rf); }
}
template <int RB, int RL>
__device__ __forceinline__ void row_inverse(uint32_t (&x)[1 << RL], uint32_t* rowbuf, uint32_t t, uint32_t p,
                                            const uint2* ri) {
    constexpr int NPH = phase_count(RB, RL);
    if constexpr (NPH > 2) { row_inv_phase<RB, RL, 2>(x, t, p, ri); row_exchange<RB, RL, 2, 1>(x, rowbuf, t); }
    if constexpr (NPH > 1) { row_inv_phase<RB, RL, 1>(x, t, p, ri); row_exchange<RB, RL, 1, 0>(x, rowbuf, t); }
    row_inv_phase<RB, RL, 0>(x, t, p, ri);
}

template <int RB, int RL>
__global__ void __launch_bounds__(32 * kRowWarps)
row_kernel(NttArgs a, const uint32_t* planes_a, size_t a_stride, const uint32_t* planes_b, size_t b_stride,
           uint32_t* planes_out, size_t out_stride, uint32_t rows_per_cta, uint32_t a_spectral) {
    using S = RowShape<RB, RL>;
    constexpr uint32_t R = S::R, TPR = S::TPR, RPW = S::RPW, E = 1u << RL;
    extern __shared__ uint4 smem_raw[];
    uint2* tabs = reinterpret_cast<uint2*>(smem_raw);
    const uint32_t Z = a.Z, H = a.H;
    uint2* s_row_f = tabs;
    uint2* s_row_i = s_row_f + R;
    uint2* s_tw_lo = s_row_i + R;
    uint2* s_tw_hi = s_tw_lo + Z;
    uint2* s_itw_lo = s_tw_hi + H;
    uint2* s_itw_hi = s_itw_lo + Z;
    uint32_t* xbuf = reinterpret_cast<uint32_t*>(s_itw_hi + H);   // kRowWarps x 2 x kWarpWords words

    const uint32_t j = blockIdx.y;
    const uint4 pc = a.consts[j];
    const uint32_t p = pc.x, np = pc.z;
    {
        const uint2* g = a.tables + size_t(j) * a.table_stride;
        for (uint32_t i = threadIdx.x; i < R; i += blockDim.x) {
            const uint32_t slot = i ? row_tw_slot<RB, RL>(i) : 0u;
            s_row_f[slot] = g[a.off_row_f + i];
            s_row_i[slot] = g[a.off_row_i + i];
        }
        for (uint32_t i = threadIdx.x; i < Z; i += blockDim.x) {
            s_tw_lo[i] = g[a.off_tw_lo + i];
            s_itw_lo[i] = g[a.off_itw_lo + i];
        }
        for (uint32_t i = threadIdx.x; i < H; i += blockDim.x) {
            s_tw_hi[i] = g[a.off_tw_hi + i];
            s_itw_hi[i] = g[a.off_itw_hi + i];
        }
    }
    __syncthreads();

    const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const uint32_t t = lane % TPR, rw = lane / TPR;
    uint32_t* bufa = xbuf + warp * 2 * S::kWarpWords + rw * (R + S::kPad);
    uint32_t* bufb = bufa + S::kWarpWords;
    const uint32_t C = a.N / R;
    const uint32_t zmask = Z - 1;
    const size_t z = blockIdx.z, jn = size_t(j) * a.N;
    constexpr PhaseMap<RB, RL> m0(0);
    constexpr PhaseMap<RB, RL> ml(phase_count(RB, RL) - 1);

    for (uint32_t it = 0; it * (kRowWarps * RPW) < rows_per_cta; ++it) {
        const uint32_t i2 = blockIdx.x * rows_per_cta + it * (kRowWarps * RPW) + warp * RPW + rw;
        const bool valid = i2 < C && it * (kRowWarps * RPW) + warp * RPW + rw < rows_per_cta;
        const uint32_t e0 = 2 * bit_reverse_dev(i2, a.c_bits) + 1;
        const uint32_t* rowa = planes_a + z * a_stride + jn + size_t(i2) * R;
        const uint32_t* rowb = planes_b + z * b_stride + jn + size_t(i2) * R;
        uint32_t* rowo = planes_out + z * out_stride + jn + size_t(i2) * R;
        uint32_t x[E], xb[E];
#pragma unroll
        for (uint32_t k = 0; k < E; ++k) {
            // A cached in spectral form is stored in natural order (element s at s).
            x[k] = valid ? rowa[a_spectral ? ml.index(t, k) : m0.index(t, k)] : 0u;
            xb[k] = valid ? rowb[m0.index(t, k)] : 0u;
        }
#pragma unroll
        for (uint32_t k = 0; k < E; ++k) {
            const uint32_t e = e0 * m0.index(t, k);
            const uint2 lo = s_tw_lo[e & zmask], hi = s_tw_hi[e >> a.z_bits];
            if (!a_spectral) x[k] = mul_shoup(mul_shoup(x[k], lo.x, lo.y, p), hi.x, hi.y, p);
            xb[k] = mul_shoup(mul_shoup(xb[k], lo.x, lo.y, p), hi.x, hi.y, p);
        }
        if (!a_spectral) row_forward<RB, RL>(x, bufa, t, p, s_row_f);
        row_forward<RB, RL>(xb, bufb, t, p, s_row_f);
        // Both operands now sit in the last phase's layout: pointwise product.
#pragma unroll
        for (uint32_t k = 0; k < E; ++k) x[k] = mul_mont(reduce_once(x[k], p), xb[k], p, np);
        row_inverse<RB, RL>(x, bufa, t, p, s_row_i);
#pragma unroll
        for (uint32_t k = 0; k < E; ++k) {
            const uint32_t s = m0.index(t, k);
            const uint32_t e = e0 * s;
            const uint2 lo = s_itw_lo[e & zmask], hi = s_itw_hi[e >> a.z_bits];
            uint32_t v = mul_shoup(mul_shoup(x[k], lo.x, lo.y, p), hi.x, hi.y, p);
            // With a single row there is no inverse column pass: emit canonical terms here.
            if (C == 1) v = reduce_once(v, p);
            if (valid) rowo[s] = v;
        }
    }
}

// ---------------------------------------------- twisted row pass, sliced --
// row_kernel's arithmetic with its twist factors taken from per-row tables:
// tw[s] = tau^s and uw[s] = K tau^-s (K = N^-1 inv(Prod/p) 2^32, consts.w),
// each with its Shoup companion, built once per CTA for its rows in flight and
// shared by every product of its slice.  A twist is then one Shoup product
// instead of two (tau^s = T_lo[e mod Z] T_hi[e / Z]), and the threads of a row
// read consecutive entries instead of scattered table words.  The cyclic
// twiddles (and their twiddle-1 butterflies) are row_kernel's.

// floor(w * 2^32 / p) for w < p, 2^30 < p < 2^31, mu = floor(2^62 / p) < 2^32:
// the estimate floor(w mu / 2^30) is at most 2 below, and the remainder
// w 2^32 - q p tells how far.
__device__ __forceinline__ uint32_t shoup_companion(uint32_t w, uint32_t p, uint32_t mu) {
    uint32_t q = uint32_t((uint64_t(w) * mu) >> 30);
    uint64_t r = (uint64_t(w) << 32) - uint64_t(q) * p;
    if (r >= p) { r -= p; ++q; }
    if (r >= p) ++q;
    return q;
}

// One row's twist (tw) and untwist (uw) factors, built by the row's TPR
// threads (thread t): entry s starts at tau^t (K tau^-t) and steps by
// tau^TPR (tau^-TPR).
template <int RB, int RL>
__device__ __forceinline__ void build_row_twists(uint2* tw, uint2* uw, uint32_t i2, uint32_t t, const NttArgs& a,
                                                 const uint2* g, uint32_t p, uint32_t mu, uint32_t K, uint32_t Kq) {
    constexpr uint32_t R = 1u << RB, TPR = R >> RL;
    const uint32_t two_n = 2 * a.N, zmask = a.Z - 1;
    auto psi_pow = [&](uint32_t ex) {           // psi^ex for 0 <= ex < 2N
        const uint2 lo = __ldg(g + a.off_tw_lo + (ex & zmask)), hi = __ldg(g + a.off_tw_hi + (ex >> a.z_bits));
        return reduce_once(mul_shoup(lo.x, hi.x, hi.y, p), p);
    };
    const uint32_t e = 2 * bit_reverse_dev(i2, a.c_bits) + 1;          // tau = psi^e; e * R < 2N
    const uint32_t et = e * t, es = e * TPR;
    uint32_t x = psi_pow(et);                                          // tau^t
    uint32_t y = reduce_once(mul_shoup(psi_pow(et ? two_n - et : 0u), K, Kq, p), p);   // K tau^-t
    const uint32_t st = psi_pow(es), sti = psi_pow(two_n - es);        // tau^TPR, tau^-TPR
    const uint32_t stq = shoup_companion(st, p, mu), stiq = shoup_companion(sti, p, mu);
    for (uint32_t sidx = t; sidx < R; sidx += TPR) {
        tw[sidx] = make_uint2(x, shoup_companion(x, p, mu));
        uw[sidx] = make_uint2(y, shoup_companion(y, p, mu));
        x = reduce_once(mul_shoup(x, st, stq, p), p);
        y = reduce_once(mul_shoup(y, sti, stiq, p), p);
    }
}

// Grid (row blocks, P, product slices): a CTA walks rows_per_cta rows of one
// prime, RIF rows at a time, and for each such set the products
// [blockIdx.z * prod_per_cta, ...) of the chain.
template <int RB, int RL>
__global__ void __launch_bounds__(32 * kRowWarps)
row_sliced_kernel(NttArgs a, const uint32_t* planes_a, size_t a_stride, const uint32_t* planes_b, size_t b_stride,
                  uint32_t* planes_out, size_t out_stride, uint32_t rows_per_cta, uint32_t a_spectral,
                  uint32_t nprod, uint32_t prod_per_cta) {
    using S = RowShape<RB, RL>;
    constexpr uint32_t R = S::R, TPR = S::TPR, RPW = S::RPW, E = 1u << RL;
    constexpr uint32_t RIF = kRowWarps * RPW;                 // rows in flight per CTA
    extern __shared__ uint4 smem_raw[];
    uint2* s_row_f = reinterpret_cast<uint2*>(smem_raw);
    uint2* s_row_i = s_row_f + R;
    uint2* s_tabs = s_row_i + R;                               // RIF rows x (twist R, untwist R)
    uint32_t* xbuf = reinterpret_cast<uint32_t*>(s_tabs + 2 * RIF * R);   // kRowWarps x 2 x kWarpWords words

    const uint32_t j = blockIdx.y;
    const uint4 pc = a.consts[j];
    const uint32_t p = pc.x, np = pc.z;
    const uint32_t mu = uint32_t((uint64_t(1) << 62) / p);
    const uint32_t K = pc.w, Kq = shoup_companion(K, p, mu);
    const uint2* g = a.tables + size_t(j) * a.table_stride;
    for (uint32_t i = threadIdx.x; i < R; i += blockDim.x) {
        const uint32_t slot = i ? row_tw_slot<RB, RL>(i) : 0u;
        s_row_f[slot] = g[a.off_row_f + i];
        s_row_i[slot] = g[a.off_row_i + i];
    }
    __syncthreads();

    const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const uint32_t t = lane % TPR, rw = lane / TPR;
    const uint32_t rslot = warp * RPW + rw;                    // this thread's row among the rows in flight
    uint2* tw = s_tabs + size_t(rslot) * 2 * R;                // written and read by this row's warp only
    uint2* uw = tw + R;
    uint32_t* bufa = xbuf + warp * 2 * S::kWarpWords + rw * (R + S::kPad);
    uint32_t* bufb = bufa + S::kWarpWords;
    const uint32_t C = a.N / R;
    const size_t jn = size_t(j) * a.N;
    const uint32_t z0 = blockIdx.z * prod_per_cta;
    const uint32_t z1 = min(nprod, z0 + prod_per_cta);
    constexpr PhaseMap<RB, RL> m0(0);
    constexpr PhaseMap<RB, RL> ml(phase_count(RB, RL) - 1);

    for (uint32_t it = 0; it * RIF < rows_per_cta; ++it) {
        const uint32_t i2 = blockIdx.x * rows_per_cta + it * RIF + rslot;
        const bool valid = i2 < C && it * RIF + rslot < rows_per_cta;
        __syncwarp();                                          // the previous rows' tables are read out
        if (valid) build_row_twists<RB, RL>(tw, uw, i2, t, a, g, p, mu, K, Kq);
        __syncwarp();
        for (uint32_t z = z0; z < z1; ++z) {
            const uint32_t* rowa = planes_a + z * a_stride + jn + size_t(i2) * R;
            const uint32_t* rowb = planes_b + z * b_stride + jn + size_t(i2) * R;
            uint32_t* rowo = planes_out + z * out_stride + jn + size_t(i2) * R;
            uint32_t x[E], xb[E];
#pragma unroll
            for (uint32_t k = 0; k < E; ++k) {
                // A cached in spectral form is stored in natural order (element s at s).
                x[k] = valid ? rowa[a_spectral ? ml.index(t, k) : m0.index(t, k)] : 0u;
                xb[k] = valid ? rowb[m0.index(t, k)] : 0u;
            }
#pragma unroll
            for (uint32_t k = 0; k < E; ++k) {
                const uint2 w = tw[m0.index(t, k)];
                if (!a_spectral) x[k] = mul_shoup(x[k], w.x, w.y, p);
                xb[k] = mul_shoup(xb[k], w.x, w.y, p);
            }
            if (!a_spectral) row_forward<RB, RL>(x, bufa, t, p, s_row_f);
            row_forward<RB, RL>(xb, bufb, t, p, s_row_f);
#pragma unroll
            for (uint32_t k = 0; k < E; ++k) x[k] = mul_mont(reduce_once(x[k], p), xb[k], p, np);
            row_inverse<RB, RL>(x, bufa, t, p, s_row_i);
#pragma unroll
            for (uint32_t k = 0; k < E; ++k) {
                const uint32_t sidx = m0.index(t, k);
                const uint2 w = uw[sidx];
                uint32_t v = mul_shoup(x[k], w.x, w.y, p);
                // With a single row there is no inverse column pass: emit canonical terms here.
                if (C == 1) v = reduce_once(v, p);
                if (valid) rowo[sidx] = v;
            }
        }
    }
}

// Forward row transform only (twist + cyclic NTT), in place: leaves an operand
// in the spectral form that row_kernel accepts with a_spectral = 1.
template <int RB, int RL>
__global__ void __launch_bounds__(32 * kRowWarps)
row_forward_kernel(NttArgs a, uint32_t* __restrict__ planes, size_t plane_stride, uint32_t rows_per_cta) {
    using S = RowShape<RB, RL>;
    constexpr uint32_t R = S::R, TPR = S::TPR, RPW = S::RPW, E = 1u << RL;
    extern __shared__ uint4 smem_raw[];
    uint2* tabs = reinterpret_cast<uint2*>(smem_raw);
    const uint32_t Z = a.Z, H = a.H;
    uint2* s_row_f = tabs;
    uint2* s_tw_lo = s_row_f + R;
    uint2* s_tw_hi = s_tw_lo + Z;
    uint32_t* xbuf = reinterpret_cast<uint32_t*>(s_tw_hi + H);
    const uint32_t j = blockIdx.y;
    const uint32_t p = a.consts[j].x;
    {
        const uint2* g = a.tables + size_t(j) * a.table_stride;
        for (uint32_t i = threadIdx.x; i < R; i += blockDim.x) s_row_f[i ? row_tw_slot<RB, RL>(i) : 0u] = g[a.off_row_f + i];
        for (uint32_t i = threadIdx.x; i < Z; i += blockDim.x) s_tw_lo[i] = g[a.off_tw_lo + i];
        for (uint32_t i = threadIdx.x; i < H; i += blockDim.x) s_tw_hi[i] = g[a.off_tw_hi + i];
    }
    __syncthreads();
    const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const uint32_t t = lane % TPR, rw = lane / TPR;
    uint32_t* buf = xbuf + warp * S::kWarpWords + rw * (R + S::kPad);
    const uint32_t C = a.N / R;
    const uint32_t zmask = Z - 1;
    const size_t plane_off = size_t(blockIdx.z) * plane_stride + size_t(j) * a.N;
    constexpr PhaseMap<RB, RL> m0(0);
    constexpr PhaseMap<RB, RL> ml(phase_count(RB, RL) - 1);
    for (uint32_t it = 0; it * (kRowWarps * RPW) < rows_per_cta; ++it) {
        const uint32_t i2 = blockIdx.x * rows_per_cta + it * (kRowWarps * RPW) + warp * RPW + rw;
        const bool valid = i2 < C && it * (kRowWarps * RPW) + warp * RPW + rw < rows_per_cta;
        const uint32_t e0 = 2 * bit_reverse_dev(i2, a.c_bits) + 1;
        uint32_t* row = planes + plane_off + size_t(i2) * R;
        uint32_t x[E];
#pragma unroll
        for (uint32_t k = 0; k < E; ++k) {
            const uint32_t s = m0.index(t, k);
            const uint32_t v = valid ? row[s] : 0u;
            const uint32_t e = e0 * s;
            const uint2 lo = s_tw_lo[e & zmask], hi = s_tw_hi[e >> a.z_bits];
            x[k] = mul_shoup(mul_shoup(v, lo.x, lo.y, p), hi.x, hi.y, p);
        }
        row_forward<RB, RL>(x, buf, t, p, s_row_f);
        // Spectral values are stored in natural (bit-reversed evaluation) order.
#pragma unroll
        for (uint32_t k = 0; k < E; ++k)
            if (valid) row[ml.index(t, k)] = x[k];
    }
}

}  // namespace

// ---------------------------------------------------------------- launchers --
template <bool INVERSE, bool TILED = false>
static cudaError_t launch_col(const NttArgs& a, uint32_t* planes, size_t stride, uint32_t nplanes, cudaStream_t st,
                              uint32_t* out = nullptr) {
    const uint32_t C = a.N / a.R;
    if (C <= 1) return cudaSuccess;
    if (TILED && (a.N < 128 || a.N % 128 || !out || out == planes)) return cudaErrorInvalidValue;
    const dim3 grid(a.R / 32, a.P, nplanes);
    switch (a.c_bits) {
#define BCG_COL(CBV) case CBV: col_kernel<CBV, INVERSE, TILED><<<grid, 32 * ((1 << CBV) >> local_bits(CBV)), 0, st>>>(a, planes, stride, out); break;
        BCG_COL(1) BCG_COL(2) BCG_COL(3) BCG_COL(4) BCG_COL(5) BCG_COL(6) BCG_COL(7) BCG_COL(8)
#undef BCG_COL
        default: return cudaErrorInvalidValue;
    }
    return cudaGetLastError();
}

cudaError_t launch_col_forward(const NttArgs& a, uint32_t* planes, size_t stride, uint32_t nplanes, cudaStream_t st) {
    return launch_col<false>(a, planes, stride, nplanes, st);
}
cudaError_t launch_col_inverse(const NttArgs& a, uint32_t* planes, size_t stride, uint32_t nplanes, cudaStream_t st,
                               uint32_t* tiled_out) {
    return tiled_out ? launch_col<true, true>(a, planes, stride, nplanes, st, tiled_out)
                     : launch_col<true, false>(a, planes, stride, nplanes, st);
}

// Elements per thread of the row pass: 2^3, or 2^4 for R = 256 unless the
// row_local knob asks for 3.
static uint32_t row_local_bits(const NttArgs& a) { return (a.R == 256 && a.row_local != 3) ? 4u : 3u; }

static uint32_t sm_count() {
    static int n = 0;
    if (!n) {
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
        if (n <= 0) n = 1;
    }
    return uint32_t(n);
}

// Rows one CTA walks through.  Default 32, or 128 with 16 elements per thread,
// where a CTA holds 16 rows at a time and the longer walk amortises its table
// loads (N = 65536, 16 products: 44.5 against 47.5 us per product).  A default
// is halved while the grid would give fewer than four CTAs per SM (one
// product per launch: N = 32768 has only 57 rows of CTAs at 128 rows each).
static uint32_t row_rows_per_cta(const NttArgs& a, uint32_t C, uint32_t rows_per_iter, uint32_t nprod) {
    uint32_t rows = a.row_rows ? a.row_rows : (row_local_bits(a) == 4 ? 128 : 32);
    if (!a.row_rows) {
        const uint64_t want = 4ull * sm_count();
        while (rows > rows_per_iter && uint64_t((C + rows - 1) / rows) * a.P * nprod < want) rows /= 2;
    }
    if (rows > C) rows = C;
    if (rows < rows_per_iter) rows = rows_per_iter;
    return rows;
}

size_t row_smem_bytes(const NttArgs& a, bool forward_only) {
    const uint32_t R = a.R;
    const uint32_t rl = row_local_bits(a);
    const uint32_t rpw = 32 / (R >> rl);
    const size_t warp_words = size_t(rpw) * (R + (rl == 4 ? 16 : 0));
    const size_t tabs = forward_only ? (R + a.Z + a.H) : (2 * R + 2 * a.Z + 2 * a.H);
    return tabs * sizeof(uint2) + (forward_only ? 1 : 2) * kRowWarps * warp_words * sizeof(uint32_t);
}

size_t row_sliced_smem_bytes(const NttArgs& a) {
    const uint32_t R = a.R;
    const uint32_t rl = row_local_bits(a);
    const uint32_t rpw = 32 / (R >> rl);
    const size_t warp_words = size_t(rpw) * (R + (rl == 4 ? 16 : 0));
    const size_t rif = size_t(kRowWarps) * rpw;
    return (2 * R + 2 * rif * R) * sizeof(uint2) + 2 * kRowWarps * warp_words * sizeof(uint32_t);
}

// The sliced row pass: a CTA per (row set, prime, product slice); slices of
// at least two products, so that each row's tables serve several products,
// and enough CTAs for four per SM where the chain allows.
static cudaError_t launch_row_sliced(const NttArgs& a, const uint32_t* planes_a, size_t a_stride,
                                     const uint32_t* planes_b, size_t b_stride, uint32_t* planes_out,
                                     size_t out_stride, uint32_t nprod, bool a_spectral, cudaStream_t st) {
    const uint32_t R = a.R;
    const uint32_t C = a.N / R;
    const uint32_t rif = kRowWarps * (32 / (R >> row_local_bits(a)));
    uint32_t rows = a.row_rows ? (a.row_rows + rif - 1) / rif * rif : rif;
    if (rows > (C + rif - 1) / rif * rif) rows = (C + rif - 1) / rif * rif;
    const uint32_t xy = (C + rows - 1) / rows * a.P;
    const uint32_t want = 4 * sm_count();
    uint32_t slices = std::max<uint32_t>(1, std::min<uint32_t>(nprod / 2, (want + xy - 1) / xy));
    const uint32_t per = (nprod + slices - 1) / slices;
    slices = (nprod + per - 1) / per;
    const dim3 grid((C + rows - 1) / rows, a.P, slices);
    const size_t smem = row_sliced_smem_bytes(a);
    const uint32_t rb = 31 - __builtin_clz(R) + (row_local_bits(a) == 4 ? 8 : 0);
    switch (rb) {
#define BCG_ROWS(RBV, RLV) case RBV + (RLV == 4 ? 8 : 0): { \
        cudaError_t e = cudaFuncSetAttribute(row_sliced_kernel<RBV, RLV>, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem)); \
        if (e != cudaSuccess) return e; \
        row_sliced_kernel<RBV, RLV><<<grid, 32 * kRowWarps, smem, st>>>(a, planes_a, a_stride, planes_b, b_stride, \
            planes_out, out_stride, rows, a_spectral ? 1u : 0u, nprod, per); break; }
        BCG_ROWS(4, 3) BCG_ROWS(5, 3) BCG_ROWS(6, 3) BCG_ROWS(7, 3) BCG_ROWS(8, 3) BCG_ROWS(8, 4)
#undef BCG_ROWS
        default: return cudaErrorInvalidValue;
    }
    return cudaGetLastError();
}

cudaError_t launch_row_product(const NttArgs& a, const uint32_t* planes_a, size_t a_stride,
                               const uint32_t* planes_b, size_t b_stride, uint32_t* planes_out,
                               size_t out_stride, uint32_t nprod, bool a_spectral, cudaStream_t st) {
    if (a.row_pass == 1)
        return launch_row_sliced(a, planes_a, a_stride, planes_b, b_stride, planes_out, out_stride, nprod,
                                 a_spectral, st);
    const uint32_t R = a.R;
    const uint32_t C = a.N / R;
    const uint32_t rpi = kRowWarps * (32 / (R >> row_local_bits(a)));
    const uint32_t rows = row_rows_per_cta(a, C, rpi, nprod);
    const dim3 grid((C + rows - 1) / rows, a.P, nprod);
    const size_t smem = row_smem_bytes(a, false);
    const uint32_t rb = 31 - __builtin_clz(R) + (row_local_bits(a) == 4 ? 8 : 0);   // 16: R = 256, 16 elements
    switch (rb) {
#define BCG_ROW(RBV, RLV) case RBV + (RLV == 4 ? 8 : 0): \
        cudaFuncSetAttribute(row_kernel<RBV, RLV>, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem)); \
        row_kernel<RBV, RLV><<<grid, 32 * kRowWarps, smem, st>>>(a, planes_a, a_stride, planes_b, b_stride, planes_out, out_stride, rows, a_spectral ? 1u : 0u); break;
        BCG_ROW(4, 3) BCG_ROW(5, 3) BCG_ROW(6, 3) BCG_ROW(7, 3) BCG_ROW(8, 3) BCG_ROW(8, 4)
#undef BCG_ROW
        default: return cudaErrorInvalidValue;
    }
    return cudaGetLastError();
}

cudaError_t launch_row_forward(const NttArgs& a, uint32_t* planes, size_t stride, uint32_t nplanes, cudaStream_t st) {
    const uint32_t R = a.R;
    const uint32_t C = a.N / R;
    const uint32_t rpi = kRowWarps * (32 / (R >> row_local_bits(a)));
    const uint32_t rows = row_rows_per_cta(a, C, rpi, nplanes);
    const dim3 grid((C + rows - 1) / rows, a.P, nplanes);
    const size_t smem = row_smem_bytes(a, true);
    const uint32_t rb = 31 - __builtin_clz(R) + (row_local_bits(a) == 4 ? 8 : 0);
    switch (rb) {
#define BCG_ROWF(RBV, RLV) case RBV + (RLV == 4 ? 8 : 0): \
        cudaFuncSetAttribute(row_forward_kernel<RBV, RLV>, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem)); \
        row_forward_kernel<RBV, RLV><<<grid, 32 * kRowWarps, smem, st>>>(a, planes, stride, rows); break;
        BCG_ROWF(4, 3) BCG_ROWF(5, 3) BCG_ROWF(6, 3) BCG_ROWF(7, 3) BCG_ROWF(8, 3) BCG_ROWF(8, 4)
#undef BCG_ROWF
        default: return cudaErrorInvalidValue;
    }
    return cudaGetLastError();
}

}  // namespace bcg
