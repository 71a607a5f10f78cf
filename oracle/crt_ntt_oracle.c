/*
 * crt_ntt_oracle.c — CPU restatement of the reference CRT-NTT big-integer
 * multiply, used ONLY as test infrastructure.
 *
 * This file is the checker. Only tests/, __graft_entry__.smoke() and the
 * CPU-baseline leg of bench.py may load it. The product (the CUDA library in
 * cryptography_gb300/) never links, calls or falls back to it.
 *
 * What it restates (reference paths inside cecoppola/cryptography):
 *   - prime set and primitive roots ......... ntt/lib/primes.h:36-48
 *     (the build uses the 3 primes P0, P2, P3; P1 has 2-adicity 24 and
 *      cannot reach N = 2^29)
 *   - Solinas reductions reduce_p0/p2/p3 .... ntt/lib/primes.h:57-163
 *   - addmod / submod / mulmod .............. ntt/lib/primes.h:193-217
 *   - modpow ................................ ntt/lib/primes.h:269-279
 *   - scatter (limb -> residue, zero pad) ... ntt/lib/arith/bigint.c:286-294
 *   - radix-2 DIT NTT with bit reversal ..... ntt/lib/arith/test_e2e_oracle.c:120-143
 *                                             and ntt/ref/ntt_cpu.c:158-204
 *   - roots omega = g^((p-1)/N) .............. ntt/lib/arith/ntt_mul.hip:189-308
 *   - cyclic convolution + n^-1 scale ....... ntt/lib/arith/test_e2e_oracle.c:146-162
 *   - Garner mixed radix, k residues ........ ntt/lib/garner.hip:105-173
 *   - gather with carry sweep ............... ntt/lib/arith/bigint.c:333-357
 *   - schoolbook product (column sums) ...... ntt/app/compute_e/test_polymul_sweep.hip:48-65
 *   - GMP mpz_mul through hand-declared ABI . ntt/app/compute_e/test_gmp_oracle.c:30-38
 *
 * Differences from the reference that the build makes on purpose: limbs are
 * 32-bit (one limb per NTT coefficient; a little-endian uint64 limb array is
 * the same bytes as a uint32 array of twice the length) and the CRT uses the
 * three primes {P0, P2, P3}.
 */
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#include <stdio.h>
#include <dlfcn.h>
#ifdef _OPENMP
#include <omp.h>
#endif

typedef unsigned __int128 u128;

/* Prime index 0,1,2 of this engine = reference P0, P2, P3. */
static const uint64_t ORC_P[3] = {
    UINT64_C(0xffffffff00000001),   /* 2^64 - 2^32 + 1 */
    UINT64_C(0xfffffffc00000001),   /* 2^64 - 2^34 + 1 */
    UINT64_C(0xffffff0000000001),   /* 2^64 - 2^40 + 1 */
};
static const uint64_t ORC_G[3] = { 7, 10, 19 };   /* reference PRIM_ROOT[0,2,3] */
static const int      ORC_B[3] = { 32, 34, 40 };

uint64_t oracle_prime(int i)      { return ORC_P[i]; }
uint64_t oracle_generator(int i)  { return ORC_G[i]; }

/* ---- exact reduction of a 128-bit value mod p = 2^64 - 2^b + 1 ----------
 * 2^64 == 2^b - 1 (mod p). Fold the high word down until it is zero, then
 * one conditional subtract. Same fold as reduce_p2/reduce_p3; for b = 32 the
 * reference does the fold in one explicit step (reduce_p0), which gives the
 * same value. */
static inline uint64_t orc_reduce(u128 x, int pi)
{
    const uint64_t p = ORC_P[pi];
    const uint64_t c = (UINT64_C(1) << ORC_B[pi]) - 1;
    while ((uint64_t)(x >> 64) != 0)
        x = (u128)(uint64_t)(x >> 64) * c + (uint64_t)x;
    uint64_t r = (uint64_t)x;
    if (r >= p) r -= p;
    return r;
}

uint64_t oracle_reduce(int pi, uint64_t lo, uint64_t hi)
{
    return orc_reduce(((u128)hi << 64) | lo, pi);
}

static inline uint64_t orc_add(uint64_t a, uint64_t b, int pi)
{
    const uint64_t p = ORC_P[pi];
    uint64_t r = a + b;
    if (r < a) r -= p;          /* wrapped past 2^64: r + 2^64 - p */
    if (r >= p) r -= p;
    return r;
}
static inline uint64_t orc_sub(uint64_t a, uint64_t b, int pi)
{
    return a >= b ? a - b : a + ORC_P[pi] - b;
}
static inline uint64_t orc_mul(uint64_t a, uint64_t b, int pi)
{
    return orc_reduce((u128)a * b, pi);
}
uint64_t oracle_mulmod(int pi, uint64_t a, uint64_t b) { return orc_mul(a, b, pi); }
uint64_t oracle_addmod(int pi, uint64_t a, uint64_t b) { return orc_add(a, b, pi); }
uint64_t oracle_submod(int pi, uint64_t a, uint64_t b) { return orc_sub(a, b, pi); }

static uint64_t orc_pow(uint64_t b, uint64_t e, int pi)
{
    uint64_t r = 1;
    b = orc_reduce(b, pi);
    while (e) {
        if (e & 1) r = orc_mul(r, b, pi);
        b = orc_mul(b, b, pi);
        e >>= 1;
    }
    return r;
}
uint64_t oracle_powmod(int pi, uint64_t b, uint64_t e) { return orc_pow(b, e, pi); }

/* Primitive 2^log_n-th root g^((p-1)/N) (or its inverse). */
uint64_t oracle_root(int pi, int log_n, int inverse)
{
    uint64_t w = orc_pow(ORC_G[pi], (ORC_P[pi] - 1) >> log_n, pi);
    if (inverse) w = orc_pow(w, ORC_P[pi] - 2, pi);
    return w;
}

/* ---- NTT: natural order in, natural order out -------------------------- */
static void orc_bitrev(uint64_t *a, size_t n)
{
    for (size_t i = 1, j = 0; i < n; i++) {
        size_t bit = n >> 1;
        for (; j & bit; bit >>= 1) j ^= bit;
        j ^= bit;
        if (i < j) { uint64_t t = a[i]; a[i] = a[j]; a[j] = t; }
    }
}

/* In-place X[k] = sum_n x[n] w^(nk), w = oracle_root(pi, log_n, inverse).
 * The inverse direction is NOT scaled here. */
void oracle_ntt(int pi, uint64_t *a, int log_n, int inverse)
{
    size_t n = (size_t)1 << log_n;
    if (n < 2) return;
    uint64_t w = oracle_root(pi, log_n, inverse);
    uint64_t *tw = (uint64_t *)malloc((n / 2) * sizeof(uint64_t));
    tw[0] = 1;
    for (size_t j = 1; j < n / 2; j++) tw[j] = orc_mul(tw[j - 1], w, pi);
    orc_bitrev(a, n);
    for (size_t len = 2; len <= n; len <<= 1) {
        size_t half = len >> 1, stride = n / len;
        long nblk = (long)(n / len);
        #pragma omp parallel for schedule(static) if (n >= 65536)
        for (long blk = 0; blk < nblk; blk++) {
            uint64_t *x = a + (size_t)blk * len;
            for (size_t j = 0; j < half; j++) {
                uint64_t u = x[j];
                uint64_t t = orc_mul(x[j + half], tw[j * stride], pi);
                x[j]        = orc_add(u, t, pi);
                x[j + half] = orc_sub(u, t, pi);
            }
        }
    }
    free(tw);
}

/* ---- Garner mixed-radix CRT over k = 3 residues ------------------------
 * x = a0 + a1*q0 + a2*q0*q1 with a_i in [0, q_i); returns x as four
 * little-endian 64-bit words (x < q0*q1*q2 < 2^192, so w[3] == 0). */
void oracle_garner3(uint64_t r0, uint64_t r1, uint64_t r2, uint64_t out[4])
{
    const uint64_t q0 = ORC_P[0], q1 = ORC_P[1];
    /* constants: inverses by Fermat, as garner_precompute does */
    static uint64_t inv_q0_q1 = 0, inv_q0_q2, inv_q1_q2, q0_q2, q0q1_q2;
    if (!inv_q0_q1) {
        inv_q0_q2 = orc_pow(orc_reduce(q0, 2), ORC_P[2] - 2, 2);
        inv_q1_q2 = orc_pow(orc_reduce(q1, 2), ORC_P[2] - 2, 2);
        q0_q2     = orc_reduce(q0, 2);
        q0q1_q2   = orc_mul(orc_reduce(q0, 2), orc_reduce(q1, 2), 2);
        inv_q0_q1 = orc_pow(orc_reduce(q0, 1), ORC_P[1] - 2, 1);
    }
    uint64_t a0 = r0;
    uint64_t a1 = orc_mul(orc_sub(r1, orc_reduce(a0, 1), 1), inv_q0_q1, 1);
    uint64_t base2 = orc_add(orc_reduce(a0, 2), orc_mul(a1, q0_q2, 2), 2);
    uint64_t a2 = orc_mul(orc_mul(orc_sub(r2, base2, 2), inv_q0_q2, 2), inv_q1_q2, 2);
    (void)q0q1_q2;
    /* assemble: x = a0 + a1*q0 + a2*(q0*q1) */
    u128 q0q1 = (u128)q0 * q1;
    uint64_t w[4] = { a0, 0, 0, 0 };
    u128 t = (u128)a1 * q0 + w[0];
    w[0] = (uint64_t)t; t >>= 64;
    w[1] = (uint64_t)t;
    /* + a2 * q0q1 (128-bit constant) */
    u128 m0 = (u128)a2 * (uint64_t)q0q1;
    u128 m1 = (u128)a2 * (uint64_t)(q0q1 >> 64);
    u128 s = (u128)w[0] + (uint64_t)m0;
    w[0] = (uint64_t)s; s >>= 64;
    s += (u128)w[1] + (uint64_t)(m0 >> 64) + (uint64_t)m1;
    w[1] = (uint64_t)s; s >>= 64;
    s += (uint64_t)(m1 >> 64);
    w[2] = (uint64_t)s;
    w[3] = (uint64_t)(s >> 64);
    memcpy(out, w, sizeof w);
}

/* ---- gather: value = sum_i coeff[i] * 2^(32 i), carry swept ------------
 * coeffs: n_coeffs entries of 4 little-endian 64-bit words (eight 32-bit
 * words each). out must hold out_cap 32-bit limbs and is overwritten.
 * Returns the trimmed limb count. */
long oracle_gather_u32(const uint64_t *coeffs, long n_coeffs,
                       uint32_t *out, long out_cap)
{
    memset(out, 0, (size_t)out_cap * sizeof(uint32_t));
    for (long i = 0; i < n_coeffs; i++) {
        uint64_t carry = 0;
        for (int w = 0; w < 8; w++) {
            long pos = i + w;
            if (pos >= out_cap) break;
            uint32_t word = (uint32_t)(coeffs[4 * i + w / 2] >> (32 * (w & 1)));
            uint64_t s = (uint64_t)out[pos] + word + carry;
            out[pos] = (uint32_t)s;
            carry = s >> 32;
        }
        for (long j = i + 8; carry && j < out_cap; j++) {
            uint64_t s = (uint64_t)out[j] + carry;
            out[j] = (uint32_t)s;
            carry = s >> 32;
        }
    }
    long n = out_cap;
    while (n > 0 && out[n - 1] == 0) n--;
    return n;
}

/* ---- full CRT-NTT product ------------------------------------------------
 * c (na + nb limbs, fully written) = a * b. Returns the trimmed length.
 * Transform length: smallest power of two >= na + nb - 1. */
long oracle_mul_u32(const uint32_t *a, long na, const uint32_t *b, long nb,
                    uint32_t *c)
{
    long nc = na + nb;
    if (na == 0 || nb == 0) { if (nc) memset(c, 0, (size_t)nc * 4); return 0; }
    long need = na + nb - 1;
    int log_n = 0;
    while (((long)1 << log_n) < need) log_n++;
    size_t N = (size_t)1 << log_n;
    int square = (a == b && na == nb);
    uint64_t *res[3];
    for (int pi = 0; pi < 3; pi++) {
        uint64_t *A = (uint64_t *)calloc(N, sizeof(uint64_t));
        uint64_t *B = square ? A : (uint64_t *)calloc(N, sizeof(uint64_t));
        /* scatter: a 32-bit limb is already below every prime */
        for (long i = 0; i < na; i++) A[i] = a[i];
        if (!square) for (long i = 0; i < nb; i++) B[i] = b[i];
        oracle_ntt(pi, A, log_n, 0);
        if (!square) oracle_ntt(pi, B, log_n, 0);
        #pragma omp parallel for schedule(static) if (N >= 65536)
        for (long k = 0; k < (long)N; k++) A[k] = orc_mul(A[k], B[k], pi);
        oracle_ntt(pi, A, log_n, 1);
        uint64_t ninv = orc_pow((uint64_t)N, ORC_P[pi] - 2, pi);
        #pragma omp parallel for schedule(static) if (N >= 65536)
        for (long k = 0; k < (long)N; k++) A[k] = orc_mul(A[k], ninv, pi);
        if (!square) free(B);
        res[pi] = A;
    }
    uint64_t *co = (uint64_t *)malloc((size_t)need * 4 * sizeof(uint64_t));
    #pragma omp parallel for schedule(static) if (need >= 65536)
    for (long k = 0; k < need; k++)
        oracle_garner3(res[0][k], res[1][k], res[2][k], co + 4 * k);
    long n = oracle_gather_u32(co, need, c, nc);
    free(co);
    for (int pi = 0; pi < 3; pi++) free(res[pi]);
    return n;
}

/* ---- schoolbook column-sum product (small operands) -------------------- */
long oracle_schoolbook_u32(const uint32_t *a, long na, const uint32_t *b, long nb,
                           uint32_t *c)
{
    long nc = na + nb;
    u128 *col = (u128 *)calloc((size_t)nc + 1, sizeof(u128));
    for (long i = 0; i < na; i++)
        for (long j = 0; j < nb; j++)
            col[i + j] += (u128)a[i] * b[j];
    u128 carry = 0;
    for (long k = 0; k < nc; k++) {
        u128 v = col[k] + carry;
        c[k] = (uint32_t)v;
        carry = v >> 32;
    }
    free(col);
    long n = nc;
    while (n > 0 && c[n - 1] == 0) n--;
    return n;
}

/* ---- value of a limb vector modulo a 64-bit modulus (checksums) -------- */
uint64_t oracle_mod_u32(const uint32_t *a, long n, uint64_t q)
{
    u128 r = 0;
    for (long i = n - 1; i >= 0; i--)
        r = ((r << 32) | a[i]) % q;
    return (uint64_t)r;
}

/* Same value with OpenMP: chunk values mod q combined with 2^(32 len) mod q. */
uint64_t oracle_mod_u32_par(const uint32_t *a, long n, uint64_t q)
{
    const long chunk = 1L << 20;
    long nch = (n + chunk - 1) / chunk;
    if (nch <= 1) return oracle_mod_u32(a, n, q);
    uint64_t *val = (uint64_t *)malloc((size_t)nch * sizeof(uint64_t));
    #pragma omp parallel for schedule(dynamic)
    for (long c = 0; c < nch; c++) {
        long s = c * chunk, m = (s + chunk <= n) ? chunk : n - s;
        val[c] = oracle_mod_u32(a + s, m, q);
    }
    /* shift = 2^(32 chunk) mod q */
    u128 sh = 1, b = ((u128)1 << 32) % q;
    for (long e = chunk; e; e >>= 1) { if (e & 1) sh = sh * b % q; b = b * b % q; }
    u128 r = 0;
    for (long c = nch - 1; c >= 0; c--) r = (r * sh + val[c]) % q;
    free(val);
    return (uint64_t)r;
}

/* ---- GMP ground truth through the public mpz ABI (dlopen) -------------- */
typedef struct { int alloc, size; void *d; } orc_mpz;
static void (*g_init)(orc_mpz *);
static void (*g_clear)(orc_mpz *);
static void (*g_import)(orc_mpz *, size_t, int, size_t, int, size_t, const void *);
static void *(*g_export)(void *, size_t *, int, size_t, int, size_t, const orc_mpz *);
static void (*g_mul)(orc_mpz *, const orc_mpz *, const orc_mpz *);
static int g_gmp_state = 0;   /* 0 unknown, 1 ok, -1 missing */

int oracle_gmp_available(void)
{
    if (g_gmp_state) return g_gmp_state > 0;
    void *h = dlopen("libgmp.so.10", RTLD_NOW | RTLD_LOCAL);
    if (!h) h = dlopen("libgmp.so", RTLD_NOW | RTLD_LOCAL);
    if (!h) { g_gmp_state = -1; return 0; }
    g_init   = (void (*)(orc_mpz *))dlsym(h, "__gmpz_init");
    g_clear  = (void (*)(orc_mpz *))dlsym(h, "__gmpz_clear");
    g_import = (void (*)(orc_mpz *, size_t, int, size_t, int, size_t, const void *))
               dlsym(h, "__gmpz_import");
    g_export = (void *(*)(void *, size_t *, int, size_t, int, size_t, const orc_mpz *))
               dlsym(h, "__gmpz_export");
    g_mul    = (void (*)(orc_mpz *, const orc_mpz *, const orc_mpz *))
               dlsym(h, "__gmpz_mul");
    g_gmp_state = (g_init && g_clear && g_import && g_export && g_mul) ? 1 : -1;
    return g_gmp_state > 0;
}

/* c must hold na + nb limbs; returns the trimmed length, or -1 without GMP. */
long oracle_gmp_mul_u32(const uint32_t *a, long na, const uint32_t *b, long nb,
                        uint32_t *c)
{
    if (!oracle_gmp_available()) return -1;
    orc_mpz x, y, z;
    g_init(&x); g_init(&y); g_init(&z);
    g_import(&x, (size_t)na, -1, 4, 0, 0, a);
    g_import(&y, (size_t)nb, -1, 4, 0, 0, b);
    g_mul(&z, &x, &y);
    memset(c, 0, (size_t)(na + nb) * 4);
    size_t cnt = 0;
    g_export(c, &cnt, -1, 4, 0, 0, &z);
    g_clear(&x); g_clear(&y); g_clear(&z);
    return (long)cnt;
}

int oracle_num_threads(void)
{
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

/* Thread count of the OpenMP regions that follow (the CPU-baseline timing
 * runs the port on all cores but one while GMP uses the last). */
void oracle_set_threads(int n)
{
#ifdef _OPENMP
    if (n > 0) omp_set_num_threads(n);
#else
    (void)n;
#endif
}
