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
 * are synchronous.  Device buffers must be 16-byte aligned (the kernels move
 * them with bulk copies).
 *
 * Threads: a plan is read-only and may be shared.  A context, a batch and the
 * stage entry points that use them are not thread-safe: use one per thread,
 * or serialise calls on it (as the reference's single-threaded harness does,
 * native-smoke/main.cpp).  Contexts never share mutable state, so different
 * contexts may run on different threads.  A server is thread-safe: any thread
 * may submit and wait.
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
#define BCG_ERR_TIMEOUT 6        /* bcg_server_wait: the request has not completed yet */

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
 *   "group"      products per launch chain, 1..4096
 *   "crt_tiles"  CRT MMA tile shape: 128-row M tiles per CTA, 2 (each staged
 *                weight-digit chunk feeds both) or 1 (two CTAs per SM)
 *   "crt_persistent"  1: persistent warp-specialised CRT (one CTA per SM,
 *                double-buffered accumulators, epilogue overlapping the MMA loop)
 *   "crt_gap_fold"  1 (default): for q = 2^W - gap (gap < 2^32, W > 70, the
 *                reference's form) the CRT reduces by two folds instead of the
 *                generic quotient estimate; 0: always generic
 *   "gap"        (read only) the gap of a gap-form q, else 0
 *   "row_local"  row pass elements per thread: 0 (default: 16 for R = 256, else 8),
 *                3 (8) or 4 (16, R = 256 only)
 *   "row_rows"   rows per row-pass CTA; 0: up to 128 with 16 elements per thread, else 32
 *                (row_pass 1: one set of rows in flight, 16 with 16 elements per thread)
 *   "row_pass"   0 (default): the row pass twists each element by tau^s with two
 *                table products; 1: the sliced row pass, whose CTAs build each
 *                row's twist and untwist factors once and share them with every
 *                product of their slice (one product per twist)
 *   "encode_scalar"  0 (default): the encode is an exact fp16 digit GEMM on
 *                the tensor cores; 1: a CUDA-core encoder with one Montgomery
 *                product per limb and prime (the reference's scalar encoder,
 *                native-smoke/rns-encode.cuh:30-77), for L <= 32 only
 *   "row_bits"   NTT radix split N = C * 2^row_bits (C <= 256); 0: R = min(N, 256).
 *                Re-plans the twiddle and twist tables (the primes stay).
 *   "host_group"  products per group of a host-buffer call (copies of one
 *                group overlap the compute of others); 0 (default): about
 *                128 MiB of operands, at most the chain length.  Reads back the
 *                value in use
 *   "host_direct"  1 (default): where the device reads and writes pageable
 *                memory through the host's page tables (Grace-based systems),
 *                small host-buffer calls use copy kernels on it; 0: they pack
 *                into pinned staging, as on systems without (reads as 0 there)
 *   "wait_limit_ns"  limit of a kernel's wait on another warp role's arrival,
 *                in ns (0: the default, 2 s).  A lower bound: a wait reads the
 *                clock every 64 polls and a poll may sleep up to 20 us, so it
 *                can overrun by about a millisecond.  Under 1000 (finer than
 *                the device clock resolves) a wait gives up at once if the
 *                arrival is missing.  A wait that runs out makes the
 *                kernel skip its remaining work, drain its own copies and MMAs
 *                and return; the call then reports BCG_ERR_DEVICE_TIMEOUT and
 *                the context stays usable.  Waits on a thread's own copies and
 *                MMAs always keep 2 s.  The reference reports CUDA failures
 *                through check() (native-smoke/solve.cu:46-49); it has no
 *                bounded device waits. */
int bcg_context_set_tuning(bcg_context* ctx, const char* knob, int64_t value);
int bcg_context_get_tuning(const bcg_context* ctx, const char* knob, int64_t* value);
/* Autotuner: times whole launch chains on synthetic operands for both encode
 * kernels (L <= 32), every value of row_bits, then the CRT kernel and tile
 * shape, row_local, row_pass, row_rows and group (coordinate search, at most
 * max_group products per chain and 4 GB of workspace), keeps the fastest, and
 * records it so that contexts of the same geometry created later in the
 * process (including those of bcg_batch and bcg_server) start from it.  The
 * reference fixes these shapes per geometry at compile time. */
typedef struct bcg_autotune_report {
    uint32_t group, crt_tiles, row_rows, row_bits;
    uint32_t candidates;    /* settings timed */
    uint32_t crt_persistent;
    uint32_t row_local, row_pass;
    uint32_t encode_scalar;
    uint32_t reserved;
    double us_per_product_default, us_per_product_tuned;
} bcg_autotune_report;
int bcg_context_autotune(bcg_context* ctx, uint32_t max_group, bcg_autotune_report* out);

/* ---- pinned host memory for the fastest host-buffer calls: bcg_multiply copies
 * pinned operands and outputs with asynchronous copy-engine copies, overlapped
 * with the device's work, and locks nothing.  The reference keeps pinned
 * staging of its own (native-smoke/solve.cu:191-247).  Free with bcg_host_free. */
int bcg_host_alloc(size_t bytes, int device, void** out);
int bcg_host_free(void* p);

/* ---- whole products.
 * bcg_multiply: host buffers, synchronous; replaces fherma_run
 * (native-smoke/solve.cu:506-525; batched native-batched/solve.cu:200-244).
 * In calls of three or more groups of products, pageable buffers are
 * page-locked as the call reaches them (the whole pages inside each buffer
 * only; the partial pages at its ends go through pinned staging) and
 * unlocked before it returns, so that the copies are asynchronous.  Pinned
 * buffers are copied directly. */
int bcg_multiply(bcg_context* ctx, const uint32_t* a, const uint32_t* b, uint32_t* c, uint32_t count);
/* Like bcg_multiply, but the product ([count][N][L] words) is handed over in
 * order, in consecutive runs, to sink(user, words, n) as each run arrives on
 * the host; `words` is valid only during the call, and the sink must not
 * throw.  The products travel in groups; before the runs of each group the
 * sink is called with words == NULL and n = the group's words: a chance to
 * prepare the destination (fault in or reserve its memory).  The sink is
 * called one call at a time, in order: from a library thread in calls of three
 * or more groups (while the calling thread issues the next groups), on the
 * calling thread in smaller ones.  For callers that append to a container of
 * their own without filling it first (bcg_multiply_dest below writes into
 * named memory instead; the plugin shim uses that).  No counterpart in the
 * reference. */
typedef void (*bcg_sink)(void* user, const uint32_t* words, size_t n);
int bcg_multiply_sink(bcg_context* ctx, const uint32_t* a, const uint32_t* b, uint32_t count, bcg_sink sink,
                      void* user);
/* Like bcg_multiply, but the caller names the output memory run by run: the
 * product ([count][N][L] words) travels in groups, and for each group, in
 * order, dest(user, n) is called on the calling thread with the group's word
 * count n and returns where those n words go (host memory that the caller
 * neither reads nor writes until the call returns; NULL fails the call with
 * BCG_ERR_INVALID).  Every run is named before any of its words is written.
 * In calls of three or more groups the library page-locks the whole pages of
 * each run as it is named and copies the product straight into them (the
 * partial pages at a run's ends, and runs that cannot be locked, come back
 * through pinned staging).  In smaller calls, where the GPU uses the host's
 * page tables, the SMs write the product straight into the run.
 * For callers that grow their own output run by run while earlier groups
 * compute (the plugin's owned std::vector: its zero fill overlaps the device
 * work instead of a staging copy after it).  No counterpart in the reference. */
typedef uint32_t* (*bcg_dest)(void* user, size_t n);
int bcg_multiply_dest(bcg_context* ctx, const uint32_t* a, const uint32_t* b, uint32_t count, bcg_dest dest,
                      void* user);
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
 * capture; the address is kept, so do not use this entry point across a
 * cudaDeviceReset).  Calls that overlap on the GPU race on the shared array. */
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
 * 3 inverse column pass, 4 CRT.  bcg_profile_enable(ctx, k): k = 0 turns
 * profiling off; k > 0 brackets every stage launch of every k-th launch chain
 * with CUDA events on its own stream (the reference times its phases the same
 * way on warm-up calls, native-smoke/solve.cu:406-503).  A period above 1
 * keeps the event records from stretching the region being timed. */
#define BCG_STAGES 5
typedef struct bcg_profile {
    double ms[8];           /* summed device time of the timed launches, per stage */
    uint64_t launches[8];   /* kernel launches per stage */
    uint64_t timed[8];      /* launches per stage that carried events */
    uint64_t chains;        /* launch chains issued */
} bcg_profile;
int bcg_profile_enable(bcg_context* ctx, int every);
int bcg_profile_read(bcg_context* ctx, bcg_profile* out, int reset);

/* ---- batched form.  The reference's batched plugin runs B products of one
 * point per fherma_run over four pipelined slots (native-batched/solve.cu:
 * 17-34, :200-244).  A bcg_batch takes products of any points (device
 * buffers), groups them by (geometry, q), and captures the launch chains of
 * every group into one CUDA graph on the first run; every run is then one
 * graph launch.  Contexts of one geometry share the twiddle, twist and encode
 * tables; contexts of one q share the CRT weights.  Runs of one batch must
 * not overlap (they share one workspace). */
typedef struct bcg_batch bcg_batch;
typedef struct bcg_batch_info {
    uint32_t groups;        /* distinct (geometry, q) groups */
    uint32_t reserved;
    uint64_t products;
    uint64_t chains;        /* launch chains per run */
    uint64_t launches;      /* kernel launches per run */
} bcg_batch_info;
int bcg_batch_create(int device, bcg_batch** out);
void bcg_batch_destroy(bcg_batch* batch);
/* `count` products of one point: a, b, c device buffers [count][N][L], 16-byte
 * aligned, kept valid while the batch runs.  Invalidates the captured graph. */
int bcg_batch_add(bcg_batch* batch, uint32_t N, uint32_t W, uint32_t L, const uint32_t* q,
                  const uint32_t* a, const uint32_t* b, uint32_t* c, uint32_t count);
int bcg_batch_run(bcg_batch* batch, void* stream);
int bcg_batch_synchronize(bcg_batch* batch, void* stream);
int bcg_batch_get_info(bcg_batch* batch, bcg_batch_info* out);   /* captures the graph if needed */
/* Chains alternate over `lanes` (1 or 2) parallel branches of the graph, each
 * with its own workspace, so that one chain's kernels fill another's tail.
 * 0 (the default): two branches when the batch holds several (geometry, q)
 * groups, one otherwise. */
int bcg_batch_set_lanes(bcg_batch* batch, uint32_t lanes);
/* Stage events inside the graph for every k-th chain (recaptures); the
 * profile holds the stage times of the last completed run. */
int bcg_batch_profile_enable(bcg_batch* batch, int every);
int bcg_batch_profile_read(bcg_batch* batch, bcg_profile* out);

/* ---- served form (no counterpart in the reference, which has no server).
 * A request loop on one GPU with continuous batching: submitted products of
 * any registered point wait in arrival order; whenever a slot stream is free
 * the oldest request leads a batch with the later requests of the same point
 * and resident operand, admitted only if its device bytes fit the free part
 * of the memory budget; batches on different slots overlap.  Resident
 * operands keep their forward-transformed residues on the device, so a
 * request that names one skips its encode and forward transform.  Host
 * buffers stay caller-owned and valid until the request is waited for. */
typedef struct bcg_server bcg_server;
typedef struct bcg_server_options {
    uint64_t memory_bytes;  /* device memory budget; 0: 80% of the free memory */
    uint32_t slots;         /* batches in flight (1..16); 0: 3 */
    uint32_t max_batch;     /* products per batch; 0: the point's group */
    uint32_t max_queue;     /* waiting requests before submit returns BCG_ERR_BUSY; 0: 65536 */
    uint32_t reserved;
} bcg_server_options;
typedef struct bcg_server_stats {
    uint64_t submitted, completed, failed, rejected;
    uint64_t batches, batched_products, operands;
    uint64_t memory_budget, memory_used, memory_peak;
} bcg_server_stats;
int bcg_server_create(int device, const bcg_server_options* opt, bcg_server** out);
/* Finishes every submitted request, then stops. */
void bcg_server_destroy(bcg_server* server);
int bcg_server_add_point(bcg_server* server, uint32_t N, uint32_t W, uint32_t L, const uint32_t* q,
                         uint32_t* point);
/* Encodes and forward-transforms host operand a ([N][L]) once, synchronously. */
int bcg_server_add_operand(bcg_server* server, uint32_t point, const uint32_t* a, uint64_t* operand);
int bcg_server_remove_operand(bcg_server* server, uint64_t operand);
/* c = a*b; pass a = NULL and operand != 0 to use a resident operand.  The
 * server keeps each request's result until bcg_server_wait() collects it (or
 * the server is destroyed): wait for every request you submit. */
int bcg_server_submit(bcg_server* server, uint32_t point, const uint32_t* a, uint64_t operand,
                      const uint32_t* b, uint32_t* c, uint64_t* request);
/* Returns the request's own status (BCG_OK or its error), or BCG_ERR_TIMEOUT
 * after timeout_ms (0: no limit) with the request still pending.  latency_ms:
 * submission to completion on the host clock. */
int bcg_server_wait(bcg_server* server, uint64_t request, uint32_t timeout_ms, double* latency_ms);
int bcg_server_drain(bcg_server* server);
int bcg_server_get_stats(const bcg_server* server, bcg_server_stats* out);

#ifdef __cplusplus
}
#endif

#endif /* BYTECRT_GB300_H */
