/*
 * ref_e_gmp_shim.c — the engine half of the reference's host compute_e,
 * served by GMP instead of a GPU (test infrastructure only). Linked with the
 * reference's own main.c / binary_split.c / mem_pool.c / bigint.c /
 * multiply.c / newton.c / base_convert.c, compiled by path (oracle/build.py),
 * it reproduces the reference CPU path whose digits the GPU e pipeline must
 * match. Implements the symbols of ntt/app/compute_e/ntt_stub.c:19-31 with
 * ntt_bigint_mul = mpz_mul through the public mpz ABI (the hand-declared
 * prototypes of ntt/app/compute_e/test_gmp_oracle.c:30-38).
 */
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#include "bigint.h"

typedef struct { int alloc, size; void *d; } shim_mpz;
extern void __gmpz_init(shim_mpz *);
extern void __gmpz_clear(shim_mpz *);
extern void __gmpz_import(shim_mpz *, size_t, int, size_t, int, size_t, const void *);
extern void *__gmpz_export(void *, size_t *, int, size_t, int, size_t, const shim_mpz *);
extern void __gmpz_mul(shim_mpz *, const shim_mpz *, const shim_mpz *);

static unsigned long g_calls = 0;

void ntt_bigint_mul(BigInt *c, const BigInt *a, const BigInt *b)
{
    shim_mpz x, y, z;
    g_calls++;
    __gmpz_init(&x); __gmpz_init(&y); __gmpz_init(&z);
    __gmpz_import(&x, (size_t)a->n_limbs, -1, 8, 0, 0, a->limbs);
    __gmpz_import(&y, (size_t)b->n_limbs, -1, 8, 0, 0, b->limbs);
    __gmpz_mul(&z, &x, &y);
    int need = a->n_limbs + b->n_limbs + 4;
    bigint_resize(c, need);
    memset(c->limbs, 0, (size_t)c->cap * 8);
    size_t cnt = 0;
    __gmpz_export(c->limbs, &cnt, -1, 8, 0, 0, &z);
    c->n_limbs = (int)cnt;
    __gmpz_clear(&x); __gmpz_clear(&y); __gmpz_clear(&z);
}

void ntt_mul_init_impl(int max_log_n) { (void)max_log_n; }
void ntt_mul_teardown_impl(void) {}
unsigned long ntt_get_gpu_dispatch_count(void) { return g_calls; }
void ntt_gpu_emergency_reset(void) {}
