// Host plan construction.  The prime rule, roots and CRT weights follow the
// reference's plan (native-smoke/rns-plan.hpp:174-324, reference.py:39-54),
// generalised to any odd W-bit q with the top bit set and any power-of-two N
// in [16, 65536].  The device tables are this project's own layouts.
#include "plan.hpp"
#include "common.cuh"

#include <algorithm>
#include <cmath>
#include <stdexcept>

namespace bcg {
namespace {

// ---------------------------------------------------------------- big ints --
// Little-endian base-2^32; the empty vector is zero.
using Big = std::vector<uint32_t>;

void trim(Big& a) { while (!a.empty() && a.back() == 0) a.pop_back(); }

uint32_t bitlen(const Big& a) {
    if (a.empty()) return 0;
    uint32_t top = 32 - __builtin_clz(a.back());
    return 32u * uint32_t(a.size() - 1) + top;
}

int cmp(const Big& a, const Big& b) {
    if (a.size() != b.size()) return a.size() < b.size() ? -1 : 1;
    for (size_t i = a.size(); i-- > 0;)
        if (a[i] != b[i]) return a[i] < b[i] ? -1 : 1;
    return 0;
}

void sub_in_place(Big& a, const Big& b) {
    uint64_t borrow = 0;
    for (size_t i = 0; i < a.size(); ++i) {
        const uint64_t s = (i < b.size() ? uint64_t(b[i]) : 0) + borrow;
        const uint64_t w = a[i];
        a[i] = uint32_t(w - s);
        borrow = w < s;
    }
    trim(a);
}

void mul_small(Big& a, uint32_t m) {
    uint64_t carry = 0;
    for (auto& w : a) {
        const uint64_t t = uint64_t(w) * m + carry;
        w = uint32_t(t);
        carry = t >> 32;
    }
    if (carry) a.push_back(uint32_t(carry));
    trim(a);
}

Big mul(const Big& a, const Big& b) {
    Big r(a.size() + b.size(), 0);
    for (size_t i = 0; i < a.size(); ++i) {
        uint64_t carry = 0;
        for (size_t j = 0; j < b.size(); ++j) {
            const uint64_t t = uint64_t(a[i]) * b[j] + r[i + j] + carry;
            r[i + j] = uint32_t(t);
            carry = t >> 32;
        }
        r[i + b.size()] = uint32_t(carry);
    }
    trim(r);
    return r;
}

Big div_small(const Big& a, uint32_t d) {
    Big r(a.size(), 0);
    uint64_t rem = 0;
    for (size_t i = a.size(); i-- > 0;) {
        const uint64_t num = (rem << 32) | a[i];
        r[i] = uint32_t(num / d);
        rem = num % d;
    }
    trim(r);
    return r;
}

uint32_t mod_small(const Big& a, uint32_t d) {
    uint64_t rem = 0;
    for (size_t i = a.size(); i-- > 0;) rem = ((rem << 32) | a[i]) % d;
    return uint32_t(rem);
}

// Remainder by shift-and-subtract over the bits of a (set-up only).
Big mod(const Big& a, const Big& m) {
    Big r;
    for (uint32_t bit = bitlen(a); bit-- > 0;) {
        uint32_t carry = (a[bit / 32] >> (bit % 32)) & 1u;
        for (auto& w : r) {
            const uint32_t top = w >> 31;
            w = (w << 1) | carry;
            carry = top;
        }
        if (carry) r.push_back(carry);
        if (cmp(r, m) >= 0) sub_in_place(r, m);
    }
    return r;
}

// ------------------------------------------------------------ 32-bit math --
uint32_t pow_mod(uint64_t b, uint64_t e, uint32_t m) {
    uint64_t r = 1;
    b %= m;
    for (; e; e >>= 1) {
        if (e & 1) r = r * b % m;
        b = b * b % m;
    }
    return uint32_t(r);
}

bool is_prime32(uint32_t p) {
    if (p < 2) return false;
    for (uint32_t s : {2u, 3u, 5u, 7u, 11u, 13u, 17u}) {
        if (p == s) return true;
        if (p % s == 0) return false;
    }
    uint32_t d = p - 1, s = 0;
    while (!(d & 1)) { d >>= 1; ++s; }
    for (uint32_t a : {2u, 7u, 61u}) {
        uint32_t x = pow_mod(a, d, p);
        if (x == 1 || x == p - 1) continue;
        bool witness = true;
        for (uint32_t i = 1; i < s && witness; ++i) {
            x = uint32_t(uint64_t(x) * x % p);
            if (x == p - 1) witness = false;
        }
        if (witness) return false;
    }
    return true;
}

uint32_t shoup(uint32_t w, uint32_t p) { return uint32_t((uint64_t(w) << 32) / p); }

// fp16 bit pattern of an integer with |v| <= 2048 (exact).
uint16_t half_bits(int v) {
    if (v == 0) return 0;
    const uint16_t sign = v < 0 ? 0x8000 : 0;
    uint32_t m = uint32_t(v < 0 ? -v : v);
    int e = 31 - __builtin_clz(m);               // m = 2^e * 1.f
    const uint32_t frac = (m << (10 - e)) & 0x3FF;
    return uint16_t(sign | ((e + 15) << 10) | frac);
}

// Four digits of a value below 2^31: three balanced bytes in [-128, 127] and a
// top digit in [0, 128], value = sum d_i 256^i.
void digits31(uint32_t v, int out[4]) {
    const uint32_t t = v + 0x808080u;
    out[0] = int(t & 255) - 128;
    out[1] = int((t >> 8) & 255) - 128;
    out[2] = int((t >> 16) & 255) - 128;
    out[3] = int(t >> 24);
}

// Balanced base-256 digits of an L-word value: 4L digits in [-128, 127] and a
// carry digit (0 or 1) at position 4L.
void digits_wide(const uint32_t* v, uint32_t L, int* out) {
    uint64_t carry = 0;
    for (uint32_t l = 0; l < L; ++l) {
        const uint64_t s = uint64_t(v[l]) + 0x80808080u + carry;
        const uint32_t w = uint32_t(s);
        carry = s >> 32;
        for (int d = 0; d < 4; ++d) out[4 * l + d] = int((w >> (8 * d)) & 255) - 128;
    }
    out[4 * L] = int(carry);
}

}  // namespace

uint32_t bit_reverse(uint32_t x, uint32_t bits) {
    uint32_t r = 0;
    for (uint32_t i = 0; i < bits; ++i) { r = (r << 1) | (x & 1); x >>= 1; }
    return r;
}

TableOffsets table_offsets(const Geometry& g) {
    TableOffsets o;
    o.col_f = 0;
    o.col_i = o.col_f + g.C;
    o.row_f = o.col_i + g.C;
    o.row_i = o.row_f + g.R;
    o.tw_lo = o.row_i + g.R;
    o.tw_hi = o.tw_lo + g.Z;
    o.itw_lo = o.tw_hi + g.H;
    o.itw_hi = o.itw_lo + g.Z;
    return o;
}

HostPlan make_plan(uint32_t N, uint32_t W, uint32_t L, const uint32_t* qw, uint32_t row_bits) {
    if (N < 16 || N > 65536 || (N & (N - 1)))
        throw std::invalid_argument("N must be a power of two in [16, 65536]");
    if (W < 2 || L != (W + 31) / 32)
        throw std::invalid_argument("L must equal ceil(W/32)");
    if (L > 63) throw std::invalid_argument("W above 2016 bits is not supported");
    Big q(qw, qw + L);
    trim(q);
    if (bitlen(q) != W) throw std::invalid_argument("q must have exactly W bits (top bit set)");
    if (!(qw[0] & 1)) throw std::invalid_argument("q must be odd");

    HostPlan plan;
    Geometry& g = plan.g;
    g.N = N; g.W = W; g.L = L;
    g.n_bits = 31 - __builtin_clz(N);
    g.R = row_bits ? (1u << row_bits) : std::min<uint32_t>(N, 256);
    if (row_bits > 8 || g.R > N || g.R < 16 || N / g.R > 256 || (N / g.R > 1 && g.R < 32))
        throw std::invalid_argument("row_bits gives an unsupported NTT split for this N");
    g.C = N / g.R;
    g.r_bits = 31 - __builtin_clz(g.R);
    g.c_bits = 31 - __builtin_clz(g.C);
    g.z_bits = (g.n_bits + 2) / 2;               // ceil((n+1)/2)
    g.Z = 1u << g.z_bits;
    g.H = (2 * N) / g.Z;
    plan.q.assign(qw, qw + L);

    // Prime rule of the reference plan (rns-plan.hpp:200-221): descending
    // p = 1 mod 2N from below 2^31 until bitlen(prod) >= 2W + bitlen(N) + 2.
    const uint32_t guard = 2 * W + (g.n_bits + 1) + 2;
    const uint32_t step = 2 * N;
    uint32_t p = ((1u << 31) - 2) / step * step + 1;
    Big prod{1};
    while (bitlen(prod) < guard) {
        while (p > (1u << 30) && !is_prime32(p)) p -= step;
        if (p <= (1u << 30)) throw std::invalid_argument("RNS prime search exhausted for this N");
        plan.primes.push_back(p);
        mul_small(prod, p);
        p -= step;
    }
    g.P = uint32_t(plan.primes.size());
    g.product_bits = bitlen(prod);
    {   // prod > 4N(q-1)^2: the centred CRT value is exact (rns-plan.hpp:222-226).
        Big qm1 = q;
        sub_in_place(qm1, Big{1});
        Big bound = mul(qm1, qm1);
        mul_small(bound, 4 * N);
        if (cmp(prod, bound) <= 0) throw std::invalid_argument("prime product below 4N(q-1)^2");
    }
    g.crt_terms = g.P + 1;
    if (g.crt_terms > 255) throw std::invalid_argument("too many RNS primes for the byte CRT");
    g.kpad = (4 * g.crt_terms + 31) / 32 * 32;

    // FP32 alpha: |c/Prod| < 1/4 and the accumulated rounding error of
    // P products and P sums stays below P*gamma_(P+4) (g1-crt.cuh:249-257).
    {
        const double u = std::ldexp(1.0, -24);
        const double n = double(g.P + 4);
        const double gamma = n * u / (1.0 - n * u);
        plan.alpha_error_bound = float(g.P * gamma);
        if (!(g.P * gamma < 0.2)) throw std::invalid_argument("fp32 alpha bound fails for this prime count");
    }

    // Encode GEMM shape: the 4L input bytes enter as b - 128 (no carries), and
    // one extra K row with A digit 1 adds back C = 0x80..80 (4L bytes).
    g.enc_k_real = 4 * L + 1;
    // The CRT output digits of a weight below q < 2^W need a carry digit only
    // when W > 32L - 2 (then w + 0x80..80 can reach 2^(32L)).
    const uint32_t extra = W > 32 * L - 2 ? 1 : 0;
    g.enc_k = (g.enc_k_real + 15) / 16 * 16;
    if (g.enc_k_real > 256) throw std::invalid_argument("encode digit sums exceed the fp32 exact range");
    const uint32_t p4 = (g.P + 3) / 4 * 4;
    g.enc_cols = 4 * p4;
    g.enc_chunks = (g.enc_cols + kEncChunkCols - 1) / kEncChunkCols;
    // CRT GEMM shape.
    g.crt_k_total = 4 * g.crt_terms;
    g.crt_kchunks = (g.crt_k_total + kCrtChunkK - 1) / kCrtChunkK;
    g.crt_e = 4 * L + extra;
    g.crt_n = (g.crt_e + 15) / 16 * 16;
    if (g.crt_n > 256) throw std::invalid_argument("CRT output digits exceed one MMA");

    const TableOffsets off = table_offsets(g);
    g.table_stride = off.itw_hi + g.H;

    plan.psi.resize(g.P);
    plan.crt_inverse.resize(g.P);
    plan.n_inverse.resize(g.P);
    plan.weights.assign(size_t(g.crt_terms) * L, 0);
    plan.prime_consts.assign(size_t(4) * g.P, 0);
    plan.ntt_tables.assign(size_t(g.P) * g.table_stride * 2, 0);
    plan.invp.resize(g.P);

    for (uint32_t j = 0; j < g.P; ++j) {
        const uint32_t pj = plan.primes[j];
        // psi: first a >= 2 whose power a^((p-1)/2N) has order 2N (rns-plan.hpp:161-168).
        const uint32_t e = (pj - 1) / (2 * N);
        uint32_t psi = 0;
        for (uint32_t a = 2; a < pj; ++a) {
            const uint32_t s = pow_mod(a, e, pj);
            if (pow_mod(s, N, pj) == pj - 1) { psi = s; break; }
        }
        if (!psi) throw std::runtime_error("primitive 2N-th root search failed");
        plan.psi[j] = psi;
        plan.n_inverse[j] = pow_mod(N, pj - 2, pj);
        const Big base = div_small(prod, pj);
        plan.crt_inverse[j] = pow_mod(mod_small(base, pj), pj - 2, pj);
        const Big wj = mod(base, q);
        std::copy(wj.begin(), wj.end(), plan.weights.begin() + size_t(j) * L);
        plan.invp[j] = float(1.0 / double(pj));

        uint32_t pinv = 1;                       // p^-1 mod 2^32 by Newton
        for (int it = 0; it < 5; ++it) pinv *= 2 - pj * pinv;
        plan.prime_consts[4 * j + 0] = pj;
        plan.prime_consts[4 * j + 1] = pinv;
        plan.prime_consts[4 * j + 2] = 0u - pinv;

        // NTT tables.
        uint32_t* tb = plan.ntt_tables.data() + size_t(j) * g.table_stride * 2;
        const uint64_t two_n = 2ull * N;
        auto put = [&](uint32_t idx, uint64_t exponent, uint32_t scale = 1) {
            uint32_t w = pow_mod(psi, exponent % two_n, pj);
            if (scale != 1) w = uint32_t(uint64_t(w) * scale % pj);
            tb[2 * idx] = w;
            tb[2 * idx + 1] = shoup(w, pj);
        };
        for (uint32_t k = 1; k < g.C; ++k) {
            const uint64_t ex = uint64_t(g.R) * bit_reverse(k, g.c_bits);   // k = 2^l + blk
            put(off.col_f + k, ex);
            put(off.col_i + k, two_n - ex);
        }
        for (uint32_t l = 0; l < g.r_bits; ++l) {
            for (uint32_t blk = 0; blk < (1u << l); ++blk) {
                // omega_R^(brv_l(blk) * R / 2^(l+1)) with omega_R = psi^(2C).
                const uint64_t ex = uint64_t(N) * bit_reverse(blk, l) >> l;
                put(off.row_f + (1u << l) + blk, ex);
                put(off.row_i + (1u << l) + blk, two_n - ex);
            }
        }
        // Inverse twist carries N^-1 * crt_inverse * 2^32 (the Montgomery
        // pointwise product divides by 2^32).
        const uint32_t r32 = uint32_t((uint64_t(1) << 32) % pj);
        const uint32_t K = uint32_t(uint64_t(plan.n_inverse[j]) * plan.crt_inverse[j] % pj * r32 % pj);
        // The sliced row pass builds its untwist factors K tau^-s from this constant.
        plan.prime_consts[4 * j + 3] = K;
        for (uint32_t lo = 0; lo < g.Z; ++lo) {
            put(off.tw_lo + lo, lo);
            put(off.itw_lo + lo, two_n - lo);
        }
        for (uint32_t hi = 0; hi < g.H; ++hi) {
            put(off.tw_hi + hi, uint64_t(g.Z) * hi);
            put(off.itw_hi + hi, two_n - uint64_t(g.Z) * hi % two_n, K);
        }
    }
    {   // alpha weight (-Prod) mod q.
        const Big pm = mod(prod, q);
        Big neg;
        if (!pm.empty()) { neg = q; sub_in_place(neg, pm); }
        std::copy(neg.begin(), neg.end(), plan.weights.begin() + size_t(g.P) * L);
    }

    // Encode B: chunk c holds columns [64c, 64c + cols_c) in K-major core-matrix
    // order over K = enc_k.  Column n = 4*j + d: digit d of 2^(8k+32) mod p_j for
    // k < 4L, and at k = 4L digit d of C * 2^32 mod p_j with C = sum_k 128 * 256^k.
    plan.enc_b.assign(size_t(g.enc_cols) * g.enc_k, 0);
    for (uint32_t col = 0; col < g.enc_cols; ++col) {
        const uint32_t j = col / 4, d = col % 4;
        if (j >= g.P) continue;
        const uint32_t pj = plan.primes[j];
        const uint32_t chunk = col / kEncChunkCols, n = col % kEncChunkCols;
        uint16_t* dst = plan.enc_b.data() + size_t(chunk) * kEncChunkCols * g.enc_k;
        uint32_t w = pow_mod(2, 32, pj);
        uint64_t cterm = 0;                          // C * 2^32 mod p_j
        for (uint32_t k = 0; k < 4 * L; ++k) {
            int dg[4];
            digits31(w, dg);
            dst[kmajor_offset(n, k, g.enc_k) / 2] = half_bits(dg[d]);
            cterm = (cterm + 128ull * w) % pj;
            w = uint32_t(uint64_t(w) * 256 % pj);
        }
        int dg[4];
        digits31(uint32_t(cterm), dg);
        dst[kmajor_offset(n, 4 * L, g.enc_k) / 2] = half_bits(dg[d]);
    }

    // CUDA-core encoder powers: half-limb m (16 bits) weighs 2^(16m) * R mod p_j
    // (R = 2^32), so one Montgomery reduction of the weighted sum is x mod p_j.
    plan.enc_pow.assign(size_t(g.P) * 2 * L, 0);
    for (uint32_t j = 0; j < g.P; ++j) {
        const uint32_t pj = plan.primes[j];
        uint64_t w = pow_mod(2, 32, pj);
        for (uint32_t m = 0; m < 2 * L; ++m) {
            plan.enc_pow[size_t(j) * 2 * L + m] = uint32_t(w);
            w = w * 65536 % pj;
        }
    }

    // CRT B: K chunk kc holds k = 4u + a for terms u in [16kc, 16kc + 16), rows
    // (MMA N) e < crt_n.  Entry = digit e of (256^a * weight_u) mod q.
    plan.crt_b.assign(size_t(g.crt_kchunks) * kCrtChunkK * g.crt_n, 0);
    std::vector<int> dg(4 * L + 1);
    for (uint32_t u = 0; u < g.crt_terms; ++u) {
        Big v(plan.weights.begin() + size_t(u) * L, plan.weights.begin() + size_t(u + 1) * L);
        trim(v);
        for (uint32_t a = 0; a < 4; ++a) {
            std::vector<uint32_t> words(L, 0);
            std::copy(v.begin(), v.end(), words.begin());
            digits_wide(words.data(), L, dg.data());
            const uint32_t k = 4 * u + a, kc = k / kCrtChunkK, kl = k % kCrtChunkK;
            const uint32_t kc_len = std::min(kCrtChunkK, (g.crt_k_total - kc * kCrtChunkK + 15) / 16 * 16);
            uint16_t* dst = plan.crt_b.data() + size_t(kc) * kCrtChunkK * g.crt_n;
            for (uint32_t e = 0; e < g.crt_e; ++e)
                dst[kmajor_offset(e, kl, kc_len) / 2] = half_bits(dg[e]);
            mul_small(v, 256);
            v = mod(v, q);
        }
    }

    {   // Quotient estimate constant for the generic mod-q epilogue.
        const uint32_t T = std::min<uint32_t>(L, 3);
        long double top = 0;
        for (uint32_t i = 0; i < L; ++i) {
            const int shift = 32 * int(i) - 32 * int(L - T);
            if (shift >= -64) top += std::ldexp((long double)plan.q[i], shift);
        }
        plan.q_inv_scaled = double(1.0L / top);
    }
    {   // Gap form q = 2^W - gap (gap < 2^32): the CRT can reduce by two folds.
        Big two_w(L, 0);
        two_w.push_back(0);
        two_w[(W) / 32] |= 1u << (W % 32);
        trim(two_w);
        Big gap = two_w;
        sub_in_place(gap, q);
        trim(gap);
        if (W > 70 && gap.size() == 1) plan.gap = gap[0];
    }
    return plan;
}

}  // namespace bcg
