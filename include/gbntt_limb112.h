/* gbntt_limb112.h — the reference-compatible entry points of libgbntt112.so,
 * the flavour of the library for the reference's LIMB_BITS=112 BigInt
 * build (ntt/lib/arith/bigint.h:30-43, :69-74): limbs are 16-byte words
 * holding 112 bits each, value = sum limbs[i] * 2^(112 i). The symbols are
 * the same as libgbntt.so's (ntt_bigint_mul and the rest), so a reference
 * build with LIMB_BITS=112 links against libgbntt112.so instead; the native
 * API (gbntt_*) is the same in both libraries. */
#pragma once
#define GBNTT_LIMB112_ABI 1
#include "gbntt.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef unsigned __int128 gbntt_limb112;   /* 112 valid bits, the top 16 zero */

/* Layout-identical to the reference BigInt with LIMB_BITS == 112. */
typedef struct {
    gbntt_limb112 *limbs;
    int n_limbs;
    int cap;
    int managed;
} gbntt_bigint112;

/* Replaces ntt_mul_init_impl (ntt/lib/arith/ntt_mul.hip:379) for 112-bit
 * limbs: products of up to 2^max_log_n 112-bit coefficients
 * (n_a + n_b - 1 <= 2^max_log_n, 3.5 32-bit limbs per coefficient, so the
 * engine is sized for 2^(max_log_n + 2) 32-bit coefficients); valid range
 * [3, cap], cap 28 (the engine's 2^30 limit), lowered by NTT_MAX_LOGN
 * (3..28). Out of range: message + exit(1). */
void ntt_mul_init_impl(int max_log_n);
void ntt_mul_teardown_impl(void);

/* Replaces ntt_bigint_mul (ntt/lib/arith/ntt_mul.hip:995): c = a * b, the
 * same guards and growth rules as the 64-bit flavour (c grown to
 * n_a + n_b + 4 limbs, a managed c too small aborts, the cyclic wrap guard
 * exits). */
void ntt_bigint_mul(gbntt_bigint112 *c, const gbntt_bigint112 *a, const gbntt_bigint112 *b);
unsigned long ntt_get_gpu_dispatch_count(void);
void ntt_gpu_emergency_reset(void);
gbntt_bigint112 bigint_alloc_managed(int cap);
void hip_free_limbs(gbntt_limb112 *p);
void ntt_bigint_sqr(gbntt_bigint112 *c, const gbntt_bigint112 *a);
int ntt_bigint_mul_checked(gbntt_bigint112 *c, const gbntt_bigint112 *a, const gbntt_bigint112 *b);

#ifdef __cplusplus
}
#endif
