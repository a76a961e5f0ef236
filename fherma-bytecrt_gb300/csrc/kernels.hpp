// Launch interfaces of the sm_103a kernels (host side of csrc/*.cu).
#pragma once

#include <cstddef>
#include <cstdint>
#include <cuda_runtime.h>

#include "plan.hpp"

namespace bcg {

constexpr uint32_t kMaxPrimes = 256;
constexpr uint32_t kMaxLimbs = 64;
constexpr uint32_t kScalarMaxLimbs = 32;   // the CUDA-core encoder (encode_scalar.cu) takes L <= 32

// Kernel arguments are passed by value; the small per-point constants ride in
// the parameter space (constant bank), where warp-uniform reads are free.
struct EncodeArgs {
    const uint32_t* in0;     // operand A coefficients [N][L] (product z at + z*in_stride)
    const uint32_t* in1;     // operand B
    size_t in_stride;
    uint32_t* out0;          // residue planes [P][N] of A (product z at + z*out_stride)
    uint32_t* out1;
    size_t out_stride;
    const uint16_t* enc_b;   // fp16 byte-power matrix, chunked
    const uint32_t* enc_pow; // [P][2L] 2^(16m) * 2^32 mod p_j (the CUDA-core encoder's half-limb weights)
    uint32_t scalar;         // 1: CUDA-core encoder (L <= 32), 0: tcgen05 encoder
    uint32_t N, L, P, K, cols, chunks;
    uint32_t* status;
    uint64_t wait_limit_ns;  // limit of waits on other roles (the context's wait limit)
    uint32_t groups, group_cols, nprod, operands;   // set by the launcher
    uint2 prime[kMaxPrimes]; // p, p^-1 mod 2^32
};

struct CrtArgs {
    const uint32_t* terms;   // t_j planes [P][N] (product z at + z*terms_stride)
    size_t terms_stride;
    uint32_t* out;           // [N][L] canonical limbs
    size_t out_stride;
    const uint16_t* crt_b;   // fp16 weight-digit matrix, chunked over K
    double q_inv_scaled;
    uint32_t N, L, P, k_total, kchunks, E, NC;
    uint32_t* status;
    uint64_t wait_limit_ns;  // limit of waits on other roles (the context's wait limit)
    uint32_t q[kMaxLimbs];
    float invp[256];         // float(1/p_j): warp-uniform reads from the constant cache
    uint32_t terms_tiled;    // persistent CRT only: terms tile-major, [N/128][P][128]
    uint32_t gap;            // q = 2^W - gap: reduce by two folds (0: generic reduction)
    uint32_t top_bits;       // W - 32 (L - 1): bits of q's top limb
};

struct NttArgs;   // ntt.cuh

// Kernel shape knobs (the autotuner's search space, bcg_context_set_tuning).
struct Tuning {
    uint32_t crt_tiles = 2;   // 128-row M tiles per CRT CTA: 2 (shared B chunks) or 1 (two CTAs per SM)
    uint32_t crt_persistent = 1;   // 1: persistent warp-specialised CRT (crt_tiles unused); measured
                                   // fastest at N = 16384, 32768 and 65536
    uint32_t row_rows = 0;    // rows of the row pass per CTA; 0: 128 (16 elements per thread) or 32,
                              // halved while the grid holds fewer than four CTAs per SM
    uint32_t crt_gap_fold = 1;   // 1: gap-form q (2^W - gap) reduces by folding; 0: generic reduction
    uint32_t row_local = 0;      // row pass elements per thread: 0 default, 3 (8 elements) or 4 (16, R = 256)
    uint32_t row_pass = 0;       // row pass kernel: 0 row_kernel, 1 row_sliced_kernel (per-row twist tables
                                 // shared by the products of a CTA's slice); an autotuner candidate
    uint32_t encode_scalar = 0;  // encode kernel: 0 tcgen05 digit GEMM, 1 CUDA-core Montgomery (L <= 32)
};

size_t encode_smem_bytes(uint32_t K, uint32_t group_cols);
uint32_t encode_group_cols(uint32_t cols, uint32_t K);
size_t crt_smem_bytes(uint32_t NC, uint32_t tiles);

// Encodes operand A (and operand B when operands == 2) of nprod products (grid.y = operand);
// a.scalar selects the CUDA-core encoder.
cudaError_t launch_encode(const EncodeArgs& a, uint32_t nprod, cudaStream_t st, uint32_t operands = 2);
// CUDA-core encoder (encode_scalar.cu): same residues, canonical in [0, p).
cudaError_t launch_encode_scalar(const EncodeArgs& a, uint32_t nprod, cudaStream_t st, uint32_t operands);
cudaError_t launch_crt(const CrtArgs& a, uint32_t nprod, cudaStream_t st, uint32_t tiles = 2);
// Persistent warp-specialised CRT (crt_persistent.cu): same results, overlapped epilogue.
cudaError_t launch_crt_persistent(const CrtArgs& a, uint32_t nprod, cudaStream_t st);
size_t crt_persistent_smem_bytes(uint32_t NC, uint32_t L);

// Column passes over nplanes prime-plane sets, set z at planes + z*stride.
cudaError_t launch_col_forward(const NttArgs& a, uint32_t* planes, size_t stride, uint32_t nplanes, cudaStream_t st);
// tiled_out: write the terms tile-major, [N/128][P][128] per set (N >= 128), into that separate
// buffer (same stride) for the persistent CRT; null: in place, natural layout.
cudaError_t launch_col_inverse(const NttArgs& a, uint32_t* planes, size_t stride, uint32_t nplanes, cudaStream_t st,
                               uint32_t* tiled_out = nullptr);
cudaError_t launch_row_product(const NttArgs& a, const uint32_t* planes_a, size_t a_stride,
                               const uint32_t* planes_b, size_t b_stride, uint32_t* planes_out,
                               size_t out_stride, uint32_t nprod, bool a_spectral, cudaStream_t st);
cudaError_t launch_row_forward(const NttArgs& a, uint32_t* planes, size_t stride, uint32_t nplanes, cudaStream_t st);
size_t row_smem_bytes(const NttArgs& a, bool forward_only);

// Word copy with SM loads and stores (host_copy.cu); either side may be
// pageable host memory where the GPU uses the host's page tables.
cudaError_t launch_host_copy(uint32_t* dst, const uint32_t* src, size_t words, cudaStream_t st);

}  // namespace bcg
