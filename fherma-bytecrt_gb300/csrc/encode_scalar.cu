// CUDA-core encoder for points with few limbs (L <= 32): coefficient limbs to
// residues mod every prime with integer multiply-adds, no tensor cores.
//
// It computes what the reference's scalar encoder computes
// (native-smoke/rns-encode.cuh:30-77: x mod p_j from the limbs and the powers
// 2^(32 limb) mod p_j) in fewer multiplies.  Each limb splits into two 16-bit
// halves h_m (m < 2L) and the table holds w_m = 2^(16m) R mod p_j (R = 2^32),
// so s = sum_m h_m w_m is one 32 x 32 + 64-bit multiply-add per half and stays
// below 2L 2^47 <= 2^53 < R p; s = x R mod p_j, and one Montgomery reduction
// of s gives x mod p_j in [0, 2p) (s + m p < 2^64), one subtraction makes it
// canonical.  The reference's form costs three multiplies and a conditional
// subtraction per limb; this one two multiply-adds per limb and one
// reduction per prime.
//
// Shape: one thread per coefficient, 128 coefficients per CTA.  The CTA copies
// its 128 L-word rows (contiguous in [N][L]) into shared memory with coalesced
// loads (row stride L | 1: the 32 rows a warp reads sit in 32 distinct banks),
// keeps each thread's half-limbs in registers, and walks a group of primes
// whose weight rows sit in shared memory (broadcast reads, two weights per
// 8-byte load).  Each prime's 128 residues leave as one coalesced 512-byte
// store into the plane [P][N].  The tcgen05 encoder (encode.cu) is faster from
// about eight limbs up; this one is the autotuner's alternative below that.
#include "kernels.hpp"

#include <algorithm>

namespace bcg {

namespace {

constexpr uint32_t kScalarRows = 128;

int sm_count_cached() {
    static int n = [] {
        int dev = 0, v = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev);
        return v > 0 ? v : 1;
    }();
    return n;
}

template <uint32_t LMAX>
__global__ void __launch_bounds__(kScalarRows) encode_scalar_kernel(const EncodeArgs a, uint32_t group_primes) {
    extern __shared__ __align__(16) uint32_t smem[];
    const uint32_t L = a.L, stride = L | 1u;
    uint32_t* pw = smem;                                 // [group_primes][2L] weights (8-byte aligned rows)
    uint32_t* tile = smem + group_primes * 2 * L;        // [128][L | 1] input limbs
    const uint32_t z = blockIdx.z;                       // product * operands + operand
    const uint32_t prod = z / a.operands, op = z - prod * a.operands;
    const uint32_t* in = (op ? a.in1 : a.in0) + size_t(prod) * a.in_stride;
    uint32_t* out = (op ? a.out1 : a.out0) + size_t(prod) * a.out_stride;
    const uint32_t n0 = blockIdx.x * kScalarRows;
    const uint32_t rows = min(kScalarRows, a.N - n0);
    const uint32_t j0 = blockIdx.y * group_primes;
    const uint32_t nj = min(group_primes, a.P - j0);

    const uint32_t* src = in + size_t(n0) * L;
    for (uint32_t w = threadIdx.x; w < rows * L; w += kScalarRows) {
        const uint32_t r = w / L;
        tile[r * stride + (w - r * L)] = src[w];
    }
    for (uint32_t w = threadIdx.x; w < nj * 2 * L; w += kScalarRows) pw[w] = a.enc_pow[size_t(j0) * 2 * L + w];
    __syncthreads();
    const uint32_t t = threadIdx.x;
    if (t >= rows) return;

    uint32_t half[2 * LMAX];
#pragma unroll
    for (uint32_t k = 0; k < LMAX; ++k) {
        const uint32_t v = k < L ? tile[t * stride + k] : 0u;
        half[2 * k] = v & 0xffffu;
        half[2 * k + 1] = v >> 16;
    }
    uint32_t* dst = out + n0 + t;
    for (uint32_t jj = 0; jj < nj; ++jj) {
        const uint2 pr = a.prime[j0 + jj];               // p, p^-1 mod 2^32
        const uint32_t p = pr.x;
        const uint2* row = reinterpret_cast<const uint2*>(pw + jj * 2 * L);
        uint64_t s = 0;
#pragma unroll
        for (uint32_t k = 0; k < LMAX; ++k)
            if (k < L) {
                const uint2 w = row[k];
                s += uint64_t(half[2 * k]) * w.x;
                s += uint64_t(half[2 * k + 1]) * w.y;
            }
        // Montgomery reduction with -p^-1: s + m p is a multiple of 2^32 below 2^64.
        const uint32_t m = uint32_t(s) * (0u - pr.y);
        uint32_t r = uint32_t((s + uint64_t(m) * p) >> 32);
        if (r >= p) r -= p;
        dst[size_t(j0 + jj) * a.N] = r;
    }
}

template <uint32_t LMAX>
cudaError_t launch_scalar_t(const EncodeArgs& a, uint32_t nprod, cudaStream_t st, uint32_t operands,
                            uint32_t group_primes) {
    EncodeArgs e = a;
    e.nprod = nprod;
    e.operands = operands;
    const uint32_t tiles = (a.N + kScalarRows - 1) / kScalarRows;
    const dim3 grid(tiles, (a.P + group_primes - 1) / group_primes, nprod * operands);
    const size_t smem = (size_t(kScalarRows) * (a.L | 1u) + size_t(group_primes) * 2 * a.L) * 4;
    encode_scalar_kernel<LMAX><<<grid, kScalarRows, smem, st>>>(e, group_primes);
    return cudaGetLastError();
}

}  // namespace

cudaError_t launch_encode_scalar(const EncodeArgs& a, uint32_t nprod, cudaStream_t st, uint32_t operands) {
    if (a.L == 0 || a.L > kScalarMaxLimbs || !a.enc_pow || a.P == 0) return cudaErrorInvalidValue;
    if (nprod == 0) return cudaSuccess;
    if (size_t(nprod) * operands > 65535) return cudaErrorInvalidValue;   // grid.z
    // Primes per CTA: enough CTAs for about two waves of 8 resident CTAs per
    // SM, and at least 4 primes per reload of the CTA's input rows.
    const size_t tiles = (a.N + kScalarRows - 1) / kScalarRows;
    const size_t units = size_t(a.P) * tiles * nprod * operands;
    const size_t target = size_t(sm_count_cached()) * 16;
    uint32_t group = uint32_t(std::min<size_t>(a.P, std::max<size_t>(4, (units + target - 1) / target)));
    group = std::min<uint32_t>(group, 32);
    if (a.L <= 4) return launch_scalar_t<4>(a, nprod, st, operands, group);
    if (a.L <= 16) return launch_scalar_t<16>(a, nprod, st, operands, group);
    return launch_scalar_t<32>(a, nprod, st, operands, group);
}

}  // namespace bcg
