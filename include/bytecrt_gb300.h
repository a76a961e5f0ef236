/*
 * bytecrt_gb300.h — C ABI of the GB300-native exact negacyclic multiplier.
 *
 *   c = a * b  mod (X^N + 1)  mod q,
 *
 * every coefficient as L = ceil(W/32) little-endian uint32 limbs, [N][L] row
 * major per product (the tensor layout of fherma::Inputs / fherma::Outputs,
 * native-smoke/fherma.h:15-41).  Products of a batch are contiguous:
 * [count][N][L].  q is any odd W-bit modulus with its top bit set; N is a
 * power of two in [16, 65536]; W <= 2016.
 *
 * Plain pointers and sizes only.  Every function returns BCG_OK (0) or a
 * BCG_ERR_* code; bcg_last_error() gives a message for the calling thread.
 * Device-pointer entry points take a cudaStream_t passed as void* (NULL means
 * the context's own stream); they are asynchronous.  Host-pointer entry points
 * are synchronous.
 *
 * The C++ plugin ABI of the reference (fherma_init / fherma_run / fherma_free,
 * native-smoke/fherma.h:46-48, native-batched/fherma.h:47-49) is provided on
 * top of these functions by libfherma_gb300.so (fherma_shim.cpp).
 */
#ifndef BYTECRT_GB300_H
#define BYTECRT_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define BCG_OK 0
#define BCG_ERR_INVALID 1        /* bad argument or unsupported point */
#define BCG_ERR_CUDA 2           /* CUDA runtime error */
#define BCG_ERR_NOMEM 3          /* device or pinned allocation failed */
#define BCG_ERR_DEVICE_TIMEOUT 4 /* a kernel's bounded wait ran out (context stays usable) */
#define BCG_ERR_BUSY 5           /* admission refused (server) */

typedef struct bcg_plan bcg_plan;        /* host-only plan (no GPU needed) */
typedef struct bcg_context bcg_context;  /* plan + device tables + workspace */

typedef struct bcg_info {
    uint32_t N, W, L;
    uint32_t P;             /* RNS primes */
    uint32_t kpad;          /* the reference's padded CRT inner axis, pad32(4(P+1)) */
    uint32_t enc_k;         /* encode MMA K (padded digits per coefficient) */
    uint32_t enc_cols;      /* encode MMA columns (4 per prime, padded) */
    uint32_t crt_k;         /* CRT MMA K = 4(P+1) */
    uint32_t crt_n;         /* CRT MMA N (padded output digits) */
    uint32_t product_bits;  /* bit length of the prime product */
    uint32_t group;         /* products per launch chain (autotuned) */
    uint32_t reserved;
    uint64_t workspace_bytes_per_product;
} bcg_info;

const char* bcg_last_error(void);

/* ---- host-only plan: replaces bytecrt::make_rns_plan (native-smoke/rns-plan.hpp:174-324) */
int bcg_plan_create(uint32_t N, uint32_t W, uint32_t L, const uint32_t* q, bcg_plan** out);
void bcg_plan_destroy(bcg_plan* plan);
int bcg_plan_info(const bcg_plan* plan, bcg_info* out);
/* primes, psi roots, CRT inverses inv(Prod/p_j): P words each */
int bcg_plan_primes(const bcg_plan* plan, uint32_t* primes, uint32_t* psi, uint32_t* crt_inverse);
/* (P+1) x L words: (Prod/p_j) mod q, then (-Prod) mod q */
int bcg_plan_weights(const bcg_plan* plan, uint32_t* weights);

/* ---- context: replaces fherma_init / fherma_free (native-smoke/solve.cu:295-397, :527) */
int bcg_context_create(uint32_t N, uint32_t W, uint32_t L, const uint32_t* q, int device, bcg_context** out);
void bcg_context_destroy(bcg_context* ctx);
int bcg_context_info(const bcg_context* ctx, bcg_info* out);
/* Products per launch chain (grid.z of every stage).  The default fills the
 * GPU for the point; the autotuner may change it. */
int bcg_context_set_group(bcg_context* ctx, uint32_t group);
/* Kernel shape knobs (the autotuner's search space), by name:
 *   "group"           products per launch chain, 1..4096
 *   "encode_bstages"  B-operand shared-memory stages of the encode MMA loop, 2 or 3
 *   "encode_accbuf"   TMEM accumulator buffers of the encode kernel, 2 or 4 */
int bcg_context_set_tuning(bcg_context* ctx, const char* knob, int64_t value);
int bcg_context_get_tuning(const bcg_context* ctx, const char* knob, int64_t* value);

/* ---- whole products.
 * bcg_multiply: host buffers, synchronous; replaces fherma_run
 * (native-smoke/solve.cu:506-525; batched native-batched/solve.cu:200-244). */
int bcg_multiply(bcg_context* ctx, const uint32_t* a, const uint32_t* b, uint32_t* c, uint32_t count);
/* device buffers, asynchronous on `stream` */
int bcg_multiply_device(bcg_context* ctx, const uint32_t* a, const uint32_t* b, uint32_t* c,
                        uint32_t count, void* stream);
/* Same product as bcg_multiply_device, for callers that cannot allocate
 * device memory at call time (a caller-owned memory pool, a framework that
 * forbids cudaMalloc on its hot path, an allocator already at its limit).
 * No counterpart in the reference.  It allocates nothing: its residue-plane
 * scratch is a 16 MiB array compiled into the library, held by every GPU that
 * loads it.  A product needs 2*P*N words of it, so points up to N=32768 with
 * W around 868 bits fit; larger points return BCG_ERR_INVALID.  The first call
 * on a device looks up the array's device address (make it before any stream
 * capture).  Calls that overlap on the GPU race on the shared array. */
int bcg_multiply_device_static(bcg_context* ctx, const uint32_t* a, const uint32_t* b, uint32_t* c,
                               uint32_t count, void* stream);

/* ---- pipeline stages (device buffers, asynchronous).  A residue plane set is
 * [P][N] uint32 per operand per product; sets of a batch are `plane_stride`
 * words apart.
 * bcg_encode_device: coefficients -> residues in [0, 2p_j); replaces
 *   launch_encode_mma32_transposed[_range] (native-smoke/rns-encode-mma.cuh:302-345). */
int bcg_encode_device(bcg_context* ctx, const uint32_t* a, const uint32_t* b, uint32_t* planes_a,
                      uint32_t* planes_b, size_t plane_stride, uint32_t count, void* stream);
/* bcg_negacyclic_device: residues of A and B -> canonical CRT terms
 *   t_j = (a*b mod (X^N+1) mod p_j) * inv(Prod/p_j) mod p_j, written over planes_a;
 *   replaces forward_first_coalesced + fused_middle + inverse_weighted
 *   (native-smoke/ntt-pipeline.cuh:73-120, native-smoke/ntt-weighted.cuh:10-44).
 *   planes_b is overwritten (forward transform). */
int bcg_negacyclic_device(bcg_context* ctx, uint32_t* planes_a, uint32_t* planes_b, size_t plane_stride,
                          uint32_t count, void* stream);
/* bcg_crt_device: CRT terms -> canonical [N][L] limbs mod q; replaces
 *   launch_g1_crt32_transposed (native-smoke/g1-crt.cuh:373-387). */
int bcg_crt_device(bcg_context* ctx, const uint32_t* terms, size_t plane_stride, uint32_t* c,
                   uint32_t count, void* stream);

/* Waits for the context's stream and reports a device-side wait timeout. */
int bcg_synchronize(bcg_context* ctx);

/* ---- measurement.  Stage order: 0 encode, 1 column pass, 2 row pass,
 * 3 inverse column pass, 4 CRT.  With profiling on, every stage launch is
 * bracketed by CUDA events on its own stream (the reference times its phases
 * the same way on warm-up calls, native-smoke/solve.cu:406-503). */
#define BCG_STAGES 5
typedef struct bcg_profile {
    double ms[8];           /* summed device time per stage */
    uint64_t launches[8];   /* kernel launches per stage */
    uint64_t chains;        /* launch chains issued */
} bcg_profile;
int bcg_profile_enable(bcg_context* ctx, int enable);
int bcg_profile_read(bcg_context* ctx, bcg_profile* out, int reset);

#ifdef __cplusplus
}
#endif

#endif /* BYTECRT_GB300_H */
