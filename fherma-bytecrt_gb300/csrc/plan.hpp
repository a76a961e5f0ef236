// Host plan for one point (N, W, q): the RNS prime set, roots, CRT weights and
// every constant table the sm_103a kernels read.  Built once per point, off the
// timed path, like the reference's make_rns_plan (native-smoke/rns-plan.hpp:174-324).
#pragma once

#include <cstdint>
#include <string>
#include <vector>

namespace bcg {

// Column/row split of the length-N negacyclic transform: N = C * R with
// R = min(N, 256) contiguous coefficients per row and C rows.
struct Geometry {
    uint32_t N = 0, W = 0, L = 0, P = 0;
    uint32_t n_bits = 0;          // log2 N
    uint32_t C = 0, R = 0, c_bits = 0, r_bits = 0;
    uint32_t Z = 0, H = 0, z_bits = 0;     // twist exponent split: e = h*Z + lo, h < H
    uint32_t table_stride = 0;    // uint2 entries of NTT tables per prime
    // Encode GEMM: A = balanced byte digits of a coefficient (K = enc_k),
    // B = balanced byte digits of 2^(8k+32) mod p_j, 4 columns per prime.
    uint32_t enc_k_real = 0, enc_k = 0, enc_cols = 0, enc_chunks = 0;
    // CRT GEMM: A = balanced digits of t_j and alpha (4 per term),
    // B = balanced digits of (256^a * weight_u) mod q over crt_e positions.
    uint32_t crt_terms = 0, crt_k_total = 0, crt_kchunks = 0, crt_e = 0, crt_n = 0;
    uint32_t kpad = 0;            // the reference's padded CRT inner axis, pad32(4(P+1))
    uint32_t product_bits = 0;
};

constexpr uint32_t kEncChunkCols = 64;   // 16 primes x 4 digits per MMA chunk
constexpr uint32_t kCrtChunkK = 32;      // 8 terms x 4 digits per K chunk

struct HostPlan {
    Geometry g;
    std::vector<uint32_t> q;               // L words
    std::vector<uint32_t> primes, psi, crt_inverse, n_inverse;
    std::vector<uint32_t> weights;         // (P+1) x L words: (Prod/p_j) mod q, then (-Prod) mod q
    std::vector<uint32_t> prime_consts;    // 4 words per prime: p, p^-1 mod 2^32, -p^-1 mod 2^32,
                                           // N^-1 * inv(Prod/p) * 2^32 mod p
    std::vector<uint32_t> ntt_tables;      // P x table_stride x (value, Shoup companion)
    std::vector<uint16_t> enc_b;           // fp16 bit patterns, chunked core-matrix order
    std::vector<uint32_t> enc_pow;         // [P][2L]: 2^(16m) * 2^32 mod p_j (CUDA-core encoder)
    std::vector<uint16_t> crt_b;           // fp16 bit patterns, chunked core-matrix order
    std::vector<float> invp;               // float(1.0 / p_j)
    double q_inv_scaled = 0;               // 2^(32*(L-T)) / q, T = min(L, 3)
    uint32_t gap = 0;                      // q = 2^W - gap with 0 < gap < 2^32 and W > 70, else 0
    float alpha_error_bound = 0;           // proven bound on |alpha_sum - exact|
};

// Offsets (in uint2 entries) inside one prime's NTT table block.
struct TableOffsets {
    uint32_t col_f, col_i, row_f, row_i, tw_lo, tw_hi, itw_lo, itw_hi;
};
TableOffsets table_offsets(const Geometry& g);

// Throws std::invalid_argument for an unsupported point.  row_bits picks the
// NTT split N = C * R with R = 2^row_bits (0: R = min(N, 256)); it needs
// C <= 256, 16 <= R <= 256, and R >= 32 when C > 1.
HostPlan make_plan(uint32_t N, uint32_t W, uint32_t L, const uint32_t* q, uint32_t row_bits = 0);

uint32_t bit_reverse(uint32_t x, uint32_t bits);

}  // namespace bcg
