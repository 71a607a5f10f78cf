/* ref_negacyclic_shim.c — TEST INFRASTRUCTURE ONLY.
 *
 * One C entry point around the reference's own CPU negacyclic multiply,
 * polymul_ntt_negacyclic (ntt/ref/ntt_polymul_negacyclic.c:178-213), which
 * oracle/build.py compiles by path from the reference checkout (library
 * form, -DNTT_NEGACYC_NO_MAIN) and links with this file into
 * oracle/_ref/libref_nega.so. The set-up follows the reference's own
 * self-test (ntt_polymul_negacyclic.c:252-330): omega = psi^2,
 * ntt_params_init, the forward/inverse twiddles and the psi^i / psi^-i
 * twist tables. Nothing of the reference is copied: its header ntt.h is
 * included by path.
 */
#include <stdint.h>
#include <stdlib.h>
#include "ntt.h"

static uint64_t shim_pow(uint64_t b, uint64_t e, uint64_t m)
{
    uint64_t r = 1;
    b %= m;
    for (; e; e >>= 1) {
        if (e & 1) r = (uint64_t)((__uint128_t)r * b % m);
        b = (uint64_t)((__uint128_t)b * b % m);
    }
    return r;
}

/* c = f * g mod (X^n + 1) mod q for coefficients in [0, q); psi a primitive
 * 2n-th root of unity mod q. Returns 0, or -1 when the reference rejects
 * the parameters (its lazy-overflow guard needs q <= 2^64 / 2n). */
int ref_negacyclic_mul(const uint64_t *f, const uint64_t *g, uint64_t *c, uint64_t n, uint64_t q, uint64_t psi)
{
    ntt_params_t p = {0};
    p.n = n;
    p.q = q;
    p.omega = shim_pow(psi, 2, q);
    if (ntt_params_init(&p) != 0) return -1;
    uint64_t *tw = ntt_alloc_twiddles(&p);
    uint64_t *twi = ntt_alloc_twiddles_inv(&p);
    uint64_t *twist = alloc_twist(n, q, psi);
    uint64_t *twist_inv = alloc_twist_inv(n, q, psi);
    int rc = -1;
    if (tw && twi && twist && twist_inv) {
        polymul_ntt_negacyclic(f, g, c, tw, twi, twist, twist_inv, &p);
        rc = 0;
    }
    free(tw);
    free(twi);
    free(twist);
    free(twist_inv);
    return rc;
}
