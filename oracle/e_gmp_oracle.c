/*
 * e_gmp_oracle.c — CPU oracle and CPU baseline of the reference's compute_e
 * path (TEST INFRASTRUCTURE ONLY), with GMP doing the arithmetic.
 *
 * Restates, on GMP integers:
 *   split_terms_needed   ntt/app/compute_e/binary_split.c:96-108
 *   binary_split         ntt/app/compute_e/binary_split.c:26-86 (same
 *                        midpoint recursion, leaf P = 1, B = a)
 *   the result           ntt/app/compute_e/main.c:167-296:
 *                        floor((B + P) 10^(D+20) / B)
 *   the printed string   ntt/app/compute_e/main.c:340-345: d0 "." d1..d(D-1)
 * GMP's mpz functions are declared by hand (no gmp.h), as the reference's
 * own ntt/app/compute_e/test_gmp_oracle.c:30-38 does; libgmp.so.10 provides
 * them. One thread.
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

typedef struct {
    int alloc, size;
    void *d;
} gmpz;
extern void __gmpz_init(gmpz *);
extern void __gmpz_clear(gmpz *);
extern void __gmpz_set_ui(gmpz *, unsigned long);
extern void __gmpz_mul(gmpz *, const gmpz *, const gmpz *);
extern void __gmpz_add(gmpz *, const gmpz *, const gmpz *);
extern void __gmpz_ui_pow_ui(gmpz *, unsigned long, unsigned long);
extern void __gmpz_tdiv_q(gmpz *, const gmpz *, const gmpz *);
extern char *__gmpz_get_str(char *, int, const gmpz *);
extern size_t __gmpz_sizeinbase(const gmpz *, int);

long oracle_split_terms_needed(long n_digits)
{
    const double target = (double)n_digits * log(10.0);
    double N = target / log(target);
    for (int i = 0; i < 50; i++) {
        const double logN = log(N);
        if (logN <= 1.0) {
            N = target;
            break;
        }
        N = target / (logN - 1.0);
    }
    return (long)(N * 1.05) + 64;
}

static void split(gmpz *P, gmpz *B, unsigned long a, unsigned long b)
{
    if (b <= a) {
        __gmpz_set_ui(P, 0);
        __gmpz_set_ui(B, 1);
        return;
    }
    if (b - a == 1) {
        __gmpz_set_ui(P, 1);
        __gmpz_set_ui(B, a);
        return;
    }
    const unsigned long m = a + (b - a) / 2;
    gmpz pl, bl, pr, br;
    __gmpz_init(&pl);
    __gmpz_init(&bl);
    __gmpz_init(&pr);
    __gmpz_init(&br);
    split(&pl, &bl, a, m);
    split(&pr, &br, m, b);
    __gmpz_mul(B, &bl, &br);
    __gmpz_mul(P, &pl, &br);
    __gmpz_add(P, P, &pr);
    __gmpz_clear(&pl);
    __gmpz_clear(&bl);
    __gmpz_clear(&pr);
    __gmpz_clear(&br);
}

static double now(void)
{
    struct timespec t;
    clock_gettime(CLOCK_MONOTONIC, &t);
    return t.tv_sec + 1e-9 * t.tv_nsec;
}

/* "2.718..." with `digits` digits into out (cap >= digits + 2); seconds
 * receives the wall time. Returns 0 on success. */
int oracle_e_digits(long digits, char *out, size_t cap, double *seconds)
{
    if (digits < 1 || cap < (size_t)digits + 2) return 1;
    const double t0 = now();
    const long n_total = digits + 20;
    const long K = oracle_split_terms_needed(n_total);
    gmpz P, B, t, q;
    __gmpz_init(&P);
    __gmpz_init(&B);
    __gmpz_init(&t);
    __gmpz_init(&q);
    split(&P, &B, 1, (unsigned long)K + 1);
    __gmpz_add(&P, &P, &B);                 /* numerator = B + P */
    __gmpz_ui_pow_ui(&t, 10, (unsigned long)n_total);
    __gmpz_mul(&P, &P, &t);
    __gmpz_tdiv_q(&q, &P, &B);
    char *s = __gmpz_get_str(NULL, 10, &q);
    const size_t n = strlen(s);
    int rc = n < (size_t)digits;
    if (!rc) {
        out[0] = s[0];
        out[1] = '.';
        memcpy(out + 2, s + 1, (size_t)digits - 1);
        out[digits + 1] = 0;
    }
    free(s);
    __gmpz_clear(&P);
    __gmpz_clear(&B);
    __gmpz_clear(&t);
    __gmpz_clear(&q);
    if (seconds) *seconds = now() - t0;
    return rc;
}
