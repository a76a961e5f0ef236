/*
 * ORACLE — test infrastructure only. Nothing in the product links, loads or
 * calls this file; only tests/, __graft_entry__.smoke() and bench.py's CPU
 * baseline leg use it, and only as the checker.
 *
 * A plain-C restatement of the ByteCRT algorithm for the exact negacyclic
 * product c = a*b mod (X^N+1) mod q (blucca/fherma-bytecrt), CPU only:
 *
 *   plan    : native-smoke/rns-plan.hpp:174-324 and reference.py:39-54
 *             (prime search, roots, CRT inverses, weights, B4 byte matrix),
 *             generalised to any odd W-bit q with the top bit set and any
 *             power-of-two N >= 16 (the reference only accepts q = 2^W - gap
 *             at two fixed geometries, rns-plan.hpp:177-197).
 *   encode  : native-smoke/rns-encode-mma.cuh:15-52 — x = sum_k byte_k *
 *             (2^(8k) mod p) as u64, then the u64 Barrett with
 *             mu = floor((2^64-1)/p) and one conditional subtraction.
 *   product : native-smoke/ntt-smoke.cu:86-129 — psi twist, radix-2 DIT
 *             cyclic NTT with explicit bit reversal, pointwise product,
 *             inverse NTT, N^-1 and psi^-i untwist, all with ordinary u64 %.
 *   crt     : t_j = c_j * inv(P/p_j) mod p_j (native-smoke/ntt-weighted.cuh:
 *             26-35); FP32 round-to-nearest alpha (native-smoke/g1-crt.cuh:
 *             249-257); B4 byte-column dots and the u64 carry chain
 *             (native-smoke/g1-crt.cuh:263-318, native-smoke/README.md
 *             "Four-column byte-weighted CRT"); then a generic z mod q by
 *             binary long division (new: the reference's reducer,
 *             g1-crt.cuh:13-68, only handles q = 2^W - gap).
 *
 * Build: gcc -O2 -fopenmp -ffp-contract=off -shared -fPIC (see oracle/build.py).
 * -ffp-contract=off matters: alpha must be computed with separately rounded
 * fp32 multiply and add, as the reference's __fmul_rn/__fadd_rn do.
 */
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#include <stdio.h>
#include <math.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define ORC_MAX_WORDS 512

/* ---------------- little-endian base-2^32 big integers ---------------- */
/* Follows the helpers of native-smoke/rns-plan.hpp:25-129. */

typedef struct { uint32_t w[ORC_MAX_WORDS]; int n; } bn_t;

static void bn_trim(bn_t *a) { while (a->n > 0 && a->w[a->n - 1] == 0) a->n--; }

static unsigned bn_bitlen(const bn_t *a) {
    if (a->n == 0) return 0;
    unsigned top = 0;
    for (uint32_t t = a->w[a->n - 1]; t; t >>= 1) top++;
    return 32u * (unsigned)(a->n - 1) + top;
}

static int bn_cmp(const bn_t *a, const bn_t *b) {
    if (a->n != b->n) return a->n < b->n ? -1 : 1;
    for (int i = a->n; i > 0; --i)
        if (a->w[i - 1] != b->w[i - 1]) return a->w[i - 1] < b->w[i - 1] ? -1 : 1;
    return 0;
}

static void bn_sub(bn_t *a, const bn_t *b) {  /* a -= b, requires a >= b */
    uint64_t borrow = 0;
    for (int i = 0; i < a->n; ++i) {
        uint64_t s = (i < b->n ? (uint64_t)b->w[i] : 0) + borrow;
        uint64_t w = a->w[i];
        a->w[i] = (uint32_t)(w - s);
        borrow = w < s;
    }
    bn_trim(a);
}

static void bn_mul_small(bn_t *a, uint32_t m) {
    uint64_t carry = 0;
    for (int i = 0; i < a->n; ++i) {
        uint64_t t = (uint64_t)a->w[i] * m + carry;
        a->w[i] = (uint32_t)t;
        carry = t >> 32;
    }
    if (carry) a->w[a->n++] = (uint32_t)carry;
    bn_trim(a);
}

static void bn_mul(bn_t *out, const bn_t *a, const bn_t *b) {
    bn_t r; memset(&r, 0, sizeof r);
    r.n = a->n + b->n;
    for (int i = 0; i < a->n; ++i) {
        uint64_t carry = 0;
        for (int j = 0; j < b->n; ++j) {
            uint64_t t = (uint64_t)a->w[i] * b->w[j] + r.w[i + j] + carry;
            r.w[i + j] = (uint32_t)t;
            carry = t >> 32;
        }
        r.w[i + b->n] = (uint32_t)carry;
    }
    bn_trim(&r);
    *out = r;
}

static uint32_t bn_div_small(bn_t *q, const bn_t *a, uint32_t d) {
    uint64_t rem = 0;
    bn_t r; memset(&r, 0, sizeof r); r.n = a->n;
    for (int i = a->n; i > 0; --i) {
        uint64_t num = (rem << 32) | a->w[i - 1];
        r.w[i - 1] = (uint32_t)(num / d);
        rem = num % d;
    }
    bn_trim(&r);
    *q = r;
    return (uint32_t)rem;
}

static uint32_t bn_mod_small(const bn_t *a, uint32_t d) {
    uint64_t rem = 0;
    for (int i = a->n; i > 0; --i) rem = ((rem << 32) | a->w[i - 1]) % d;
    return (uint32_t)rem;
}

/* Bit-serial remainder, as rns-plan.hpp:112-129 (init only). */
static void bn_mod(bn_t *out, const bn_t *a, const bn_t *q) {
    bn_t r; memset(&r, 0, sizeof r);
    for (unsigned bit = bn_bitlen(a); bit != 0;) {
        --bit;
        uint64_t carry = (a->w[bit / 32] >> (bit % 32)) & 1u;
        for (int i = 0; i < r.n; ++i) {
            uint64_t t = ((uint64_t)r.w[i] << 1) | carry;
            r.w[i] = (uint32_t)t;
            carry = t >> 32;
        }
        if (carry) r.w[r.n++] = (uint32_t)carry;
        if (bn_cmp(&r, q) >= 0) bn_sub(&r, q);
    }
    *out = r;
}

/* ---------------- 32-bit modular helpers ---------------- */

static uint32_t pow_mod(uint32_t base, uint32_t e, uint32_t m) {
    uint64_t r = 1, b = base % m;
    for (; e; e >>= 1) {
        if (e & 1) r = r * b % m;
        b = b * b % m;
    }
    return (uint32_t)r;
}

/* Deterministic Miller-Rabin for u32 (bases 2, 7, 61), reference.py:11-36. */
static int prime32(uint32_t p) {
    static const uint32_t small[] = {2, 3, 5, 7, 11, 13, 17};
    if (p < 2) return 0;
    for (int i = 0; i < 7; ++i) {
        if (p == small[i]) return 1;
        if (p % small[i] == 0) return 0;
    }
    uint32_t d = p - 1, s = 0;
    while ((d & 1) == 0) { d >>= 1; ++s; }
    static const uint32_t bases[] = {2, 7, 61};
    for (int i = 0; i < 3; ++i) {
        uint32_t a = bases[i];
        if (a % p == 0) continue;
        uint32_t x = pow_mod(a, d, p);
        if (x == 1 || x == p - 1) continue;
        int ok = 0;
        for (uint32_t r = 1; r < s; ++r) {
            x = (uint32_t)((uint64_t)x * x % p);
            if (x == p - 1) { ok = 1; break; }
        }
        if (!ok) return 0;
    }
    return 1;
}

/* Montgomery product with R = 2^32, native-smoke/rns-encode.cuh:15-22. */
uint32_t orc_mont_mul_word(uint32_t a, uint32_t b, uint32_t p, uint32_t neg_inverse) {
    uint64_t x = (uint64_t)a * b;
    uint32_t t = (uint32_t)x * neg_inverse;
    uint32_t u = (uint32_t)((x + (uint64_t)t * p) >> 32);
    return u >= p ? u - p : u;
}

/* ---------------- plan ---------------- */

typedef struct {
    uint32_t n, w, l, pcount, kpad;
    uint32_t *primes, *psi, *crt_inverse, *n_inverse;
    double *invp;
    uint32_t *weights;      /* (pcount+1) x l words: (P/p_j) mod q, then (-P) mod q */
    uint32_t *q;            /* l words */
    uint8_t *b4;            /* 4l columns x kpad bytes, column-major (rns-plan.hpp:301-322) */
    uint32_t product_bits;
} orc_plan;

static char orc_err[256];
const char *orc_last_error(void) { return orc_err; }

void orc_plan_free(orc_plan *p) {
    if (!p) return;
    free(p->primes); free(p->psi); free(p->crt_inverse); free(p->n_inverse);
    free(p->invp); free(p->weights); free(p->q); free(p->b4);
    free(p);
}

/*
 * Plan for N (power of two, >= 16), W-bit odd q with the top bit set, L limbs.
 * Prime rule: native-smoke/rns-plan.hpp:200-226 / reference.py:40-49.
 */
orc_plan *orc_plan_create(uint32_t N, uint32_t W, uint32_t L, const uint32_t *qw) {
    orc_err[0] = 0;
    if (N < 2 || (N & (N - 1))) { snprintf(orc_err, sizeof orc_err, "N must be a power of two"); return NULL; }
    if (L == 0 || L > 200 || (W + 31) / 32 != L) { snprintf(orc_err, sizeof orc_err, "L must be ceil(W/32)"); return NULL; }
    bn_t q; memset(&q, 0, sizeof q);
    q.n = (int)L; memcpy(q.w, qw, L * 4); bn_trim(&q);
    if (bn_bitlen(&q) != W) { snprintf(orc_err, sizeof orc_err, "bitlen(q) != W"); return NULL; }
    if ((qw[0] & 1) == 0) { snprintf(orc_err, sizeof orc_err, "q must be odd"); return NULL; }

    orc_plan *pl = calloc(1, sizeof *pl);
    pl->n = N; pl->w = W; pl->l = L;
    unsigned nbits = 0;
    for (uint32_t v = N; v; v >>= 1) ++nbits;
    unsigned guard = 2 * W + nbits + 2;
    uint32_t step = 2 * N;
    uint32_t p = ((1u << 31) - 2) / step * step + 1;
    bn_t prod; memset(&prod, 0, sizeof prod); prod.n = 1; prod.w[0] = 1;
    uint32_t primes[1024]; unsigned count = 0;
    while (bn_bitlen(&prod) < guard) {
        while (p > (1u << 30) && !prime32(p)) p -= step;
        if (p <= (1u << 30) || count >= 1024) {
            snprintf(orc_err, sizeof orc_err, "prime search exhausted");
            orc_plan_free(pl); return NULL;
        }
        primes[count++] = p;
        bn_mul_small(&prod, p);
        p -= step;
    }
    pl->pcount = count;
    pl->product_bits = bn_bitlen(&prod);
    /* Exact centred-CRT guard P > 4N(q-1)^2 (rns-plan.hpp:222-226). */
    bn_t qm1 = q, one; memset(&one, 0, sizeof one); one.n = 1; one.w[0] = 1;
    bn_sub(&qm1, &one);
    bn_t bound; bn_mul(&bound, &qm1, &qm1); bn_mul_small(&bound, 4 * N);
    if (bn_cmp(&prod, &bound) <= 0) {
        snprintf(orc_err, sizeof orc_err, "prime product below 4N(q-1)^2");
        orc_plan_free(pl); return NULL;
    }
    unsigned terms = count + 1;
    pl->kpad = (4 * terms + 31) / 32 * 32;
    pl->primes = malloc(count * 4); pl->psi = malloc(count * 4);
    pl->crt_inverse = malloc(count * 4); pl->n_inverse = malloc(count * 4);
    pl->invp = malloc(count * sizeof(double));
    pl->weights = calloc((size_t)terms * L, 4);
    pl->q = malloc(L * 4); memcpy(pl->q, qw, L * 4);
    for (unsigned j = 0; j < count; ++j) {
        uint32_t pj = primes[j];
        pl->primes[j] = pj;
        /* First a >= 2 with psi = a^((p-1)/2N) of order 2N (rns-plan.hpp:161-168). */
        uint32_t e = (pj - 1) / (2 * N), psi = 0;
        for (uint32_t a = 2; a < pj; ++a) {
            uint32_t s = pow_mod(a, e, pj);
            if (pow_mod(s, N, pj) == pj - 1) { psi = s; break; }
        }
        pl->psi[j] = psi;
        pl->n_inverse[j] = pow_mod(N % pj, pj - 2, pj);
        bn_t base; uint32_t rem = bn_div_small(&base, &prod, pj);
        (void)rem;
        uint32_t bm = bn_mod_small(&base, pj);
        pl->crt_inverse[j] = pow_mod(bm, pj - 2, pj);
        pl->invp[j] = 1.0 / (double)pj;
        bn_t wq; bn_mod(&wq, &base, &q);
        memcpy(pl->weights + (size_t)j * L, wq.w, (size_t)wq.n * 4);
    }
    bn_t pm; bn_mod(&pm, &prod, &q);
    if (pm.n) {  /* (-P) mod q = q - (P mod q) */
        bn_t neg = q; bn_sub(&neg, &pm);
        memcpy(pl->weights + (size_t)count * L, neg.w, (size_t)neg.n * 4);
    }
    /* B4: column 4l+d, input byte 4j+a holds byte_d(word_l((256^a * weight_j) mod q)). */
    pl->b4 = calloc((size_t)4 * L * pl->kpad, 1);
    for (unsigned j = 0; j < terms; ++j) {
        bn_t sh; memset(&sh, 0, sizeof sh); sh.n = (int)L;
        memcpy(sh.w, pl->weights + (size_t)j * L, L * 4); bn_trim(&sh);
        for (unsigned a = 0; a < 4; ++a) {
            for (unsigned l = 0; l < L; ++l) {
                uint32_t word = (int)l < sh.n ? sh.w[l] : 0;
                for (unsigned d = 0; d < 4; ++d)
                    pl->b4[(size_t)(4 * l + d) * pl->kpad + 4 * j + a] = (uint8_t)(word >> (8 * d));
            }
            if (a < 3) { bn_mul_small(&sh, 256); bn_t t; bn_mod(&t, &sh, &q); sh = t; }
        }
    }
    return pl;
}

uint32_t orc_plan_pcount(const orc_plan *p) { return p->pcount; }
uint32_t orc_plan_kpad(const orc_plan *p) { return p->kpad; }
uint32_t orc_plan_product_bits(const orc_plan *p) { return p->product_bits; }
void orc_plan_primes(const orc_plan *p, uint32_t *out) { memcpy(out, p->primes, p->pcount * 4); }
void orc_plan_psi(const orc_plan *p, uint32_t *out) { memcpy(out, p->psi, p->pcount * 4); }
void orc_plan_crt_inverse(const orc_plan *p, uint32_t *out) { memcpy(out, p->crt_inverse, p->pcount * 4); }
void orc_plan_weights(const orc_plan *p, uint32_t *out) { memcpy(out, p->weights, (size_t)(p->pcount + 1) * p->l * 4); }
void orc_plan_b4(const orc_plan *p, uint8_t *out) { memcpy(out, p->b4, (size_t)4 * p->l * p->kpad); }

/* ---------------- encode (rns-encode-mma.cuh:15-52) ---------------- */

/* in: [N][L] limbs; out: [P][N] canonical residues. */
void orc_encode(const orc_plan *pl, const uint32_t *in, uint32_t *out, int threads) {
    const uint32_t N = pl->n, L = pl->l, P = pl->pcount;
#pragma omp parallel for num_threads(threads) schedule(static)
    for (int64_t j = 0; j < (int64_t)P; ++j) {
        const uint32_t p = pl->primes[j];
        uint32_t pw[4 * ORC_MAX_WORDS];
        uint32_t power = 1;
        for (uint32_t k = 0; k < 4 * L; ++k) { pw[k] = power; power = (uint32_t)((uint64_t)power * 256 % p); }
        const uint64_t mu = UINT64_MAX / p;
        for (uint32_t i = 0; i < N; ++i) {
            const uint32_t *row = in + (size_t)i * L;
            uint64_t x = 0;
            for (uint32_t l = 0; l < L; ++l) {
                uint32_t v = row[l];
                x += (uint64_t)(v & 255) * pw[4 * l] + (uint64_t)((v >> 8) & 255) * pw[4 * l + 1]
                   + (uint64_t)((v >> 16) & 255) * pw[4 * l + 2] + (uint64_t)(v >> 24) * pw[4 * l + 3];
            }
            uint64_t qh = (uint64_t)(((__uint128_t)x * mu) >> 64);
            uint64_t r = x - qh * p;
            out[(size_t)j * N + i] = (uint32_t)(r >= p ? r - p : r);
        }
    }
}

/* ---------------- per-prime negacyclic product (ntt-smoke.cu:86-129) ---------------- */

static uint32_t mm(uint32_t a, uint32_t b, uint32_t p) { return (uint32_t)((uint64_t)a * b % p); }

static void cyclic_ntt(uint32_t *a, uint32_t n, uint32_t p, uint32_t root) {
    for (uint32_t i = 1, j = 0; i < n; ++i) {
        uint32_t bit = n >> 1;
        while (j & bit) { j ^= bit; bit >>= 1; }
        j ^= bit;
        if (i < j) { uint32_t t = a[i]; a[i] = a[j]; a[j] = t; }
    }
    for (uint32_t len = 2; len <= n; len <<= 1) {
        uint32_t step = pow_mod(root, n / len, p);
        for (uint32_t start = 0; start < n; start += len) {
            uint32_t w = 1;
            for (uint32_t j = 0; j < len / 2; ++j) {
                uint32_t u = a[start + j], v = mm(a[start + j + len / 2], w, p);
                uint64_t s = (uint64_t)u + v;
                a[start + j] = (uint32_t)(s >= p ? s - p : s);
                a[start + j + len / 2] = u >= v ? u - v : (uint32_t)((uint64_t)u + p - v);
                w = mm(w, step, p);
            }
        }
    }
}

/* x, y: canonical residues of one prime; out = x*y mod (X^N+1) mod p_j. */
void orc_prime_product(const orc_plan *pl, uint32_t j, const uint32_t *x, const uint32_t *y, uint32_t *out) {
    const uint32_t N = pl->n, p = pl->primes[j], psi = pl->psi[j];
    const uint32_t psi_inv = pow_mod(psi, p - 2, p), omega = mm(psi, psi, p);
    const uint32_t omega_inv = pow_mod(omega, p - 2, p), ninv = pl->n_inverse[j];
    uint32_t *a = malloc((size_t)N * 4), *b = malloc((size_t)N * 4);
    uint32_t pw = 1;
    for (uint32_t i = 0; i < N; ++i) { a[i] = mm(x[i], pw, p); b[i] = mm(y[i], pw, p); pw = mm(pw, psi, p); }
    cyclic_ntt(a, N, p, omega);
    cyclic_ntt(b, N, p, omega);
    for (uint32_t i = 0; i < N; ++i) a[i] = mm(a[i], b[i], p);
    cyclic_ntt(a, N, p, omega_inv);
    pw = 1;
    for (uint32_t i = 0; i < N; ++i) { out[i] = mm(mm(a[i], ninv, p), pw, p); pw = mm(pw, psi_inv, p); }
    free(a); free(b);
}

/* ---------------- CRT of one coefficient ---------------- */

/*
 * terms: P canonical t_j (already multiplied by inv(P/p_j)).
 * alpha: FP32 RN sum (g1-crt.cuh:249-257); wide: L+2 words of the B4 sum
 * with the u64 carry chain (g1-crt.cuh:304-318); out: L words of wide mod q.
 */
static void crt_one(const orc_plan *pl, const uint32_t *terms, uint32_t *alpha_out,
                    uint32_t *wide_out, uint32_t *out) {
    const uint32_t P = pl->pcount, L = pl->l, K = pl->kpad;
    /* __fadd_rn(sum, __fmul_rn(__uint2float_rn(t), (float)invp)); no FMA contraction. */
    float sum = 0.0f;
    for (uint32_t j = 0; j < P; ++j) {
        float prod = (float)terms[j] * (float)pl->invp[j];
        sum = sum + prod;
    }
    /* __float2uint_rn: round to nearest even (the default FP environment). */
    uint32_t alpha = (uint32_t)lrintf(sum);
    uint8_t abytes[4 * 257];
    memset(abytes, 0, sizeof abytes);
    for (uint32_t j = 0; j < P; ++j)
        for (int d = 0; d < 4; ++d) abytes[4 * j + d] = (uint8_t)(terms[j] >> (8 * d));
    for (int d = 0; d < 4; ++d) abytes[4 * P + d] = (uint8_t)(alpha >> (8 * d));
    uint64_t carry = 0;
    uint32_t digits[ORC_MAX_WORDS + 2];
    for (uint32_t l = 0; l < L; ++l) {
        uint32_t c[4];
        for (int d = 0; d < 4; ++d) {
            const uint8_t *col = pl->b4 + (size_t)(4 * l + d) * K;
            uint32_t s = 0;
            for (uint32_t k = 0; k < 4 * (P + 1); ++k) s += (uint32_t)abytes[k] * col[k];
            c[d] = s;
        }
        uint64_t lo = (uint64_t)c[0] + ((uint64_t)c[1] << 8) + ((uint64_t)c[2] << 16) + ((uint64_t)c[3] << 24);
        uint64_t total = carry + lo;
        digits[l] = (uint32_t)total;
        carry = total >> 32;
    }
    digits[L] = (uint32_t)carry;
    digits[L + 1] = (uint32_t)(carry >> 32);
    if (alpha_out) *alpha_out = alpha;
    if (wide_out) memcpy(wide_out, digits, (L + 2) * 4);
    /* Generic z mod q by binary long division (new; replaces g1-crt.cuh:13-68). */
    bn_t z; memset(&z, 0, sizeof z); z.n = (int)L + 2; memcpy(z.w, digits, (L + 2) * 4); bn_trim(&z);
    bn_t q; memset(&q, 0, sizeof q); q.n = (int)L; memcpy(q.w, pl->q, L * 4); bn_trim(&q);
    bn_t r; bn_mod(&r, &z, &q);
    memset(out, 0, L * 4);
    memcpy(out, r.w, (size_t)r.n * 4);
}

void orc_crt_terms(const orc_plan *pl, const uint32_t *terms, uint32_t *alpha, uint32_t *wide, uint32_t *out) {
    crt_one(pl, terms, alpha, wide, out);
}

/* res: [P][N] canonical per-prime products c_j; out: [N][L]. */
void orc_crt(const orc_plan *pl, const uint32_t *res, uint32_t *out, int threads) {
    const uint32_t N = pl->n, P = pl->pcount, L = pl->l;
#pragma omp parallel for num_threads(threads) schedule(static)
    for (int64_t i = 0; i < (int64_t)N; ++i) {
        uint32_t terms[1024];
        for (uint32_t j = 0; j < P; ++j)
            terms[j] = mm(res[(size_t)j * N + i], pl->crt_inverse[j], pl->primes[j]);
        crt_one(pl, terms, NULL, NULL, out + (size_t)i * L);
    }
}

/* Whole product: a, b, c are [N][L]. */
int orc_multiply(const orc_plan *pl, const uint32_t *a, const uint32_t *b, uint32_t *c, int threads) {
    const uint32_t N = pl->n, P = pl->pcount;
    uint32_t *ra = malloc((size_t)P * N * 4), *rb = malloc((size_t)P * N * 4), *rc = malloc((size_t)P * N * 4);
    if (!ra || !rb || !rc) { free(ra); free(rb); free(rc); return -1; }
    orc_encode(pl, a, ra, threads);
    orc_encode(pl, b, rb, threads);
#pragma omp parallel for num_threads(threads) schedule(dynamic)
    for (int64_t j = 0; j < (int64_t)P; ++j)
        orc_prime_product(pl, (uint32_t)j, ra + (size_t)j * N, rb + (size_t)j * N, rc + (size_t)j * N);
    orc_crt(pl, rc, c, threads);
    free(ra); free(rb); free(rc);
    return 0;
}

int orc_max_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}
