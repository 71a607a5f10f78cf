/*
 * ref_shim.cpp — exposes the REFERENCE's own host code (compiled from its
 * sources where they lie, never copied) through a small C ABI so the oracle
 * restatement can be pinned against it. Test infrastructure only.
 *
 * Built by oracle/build.py into oracle/_ref/libref.so with
 *   -I <reference>/ntt/lib -I <reference>/ntt/lib/arith
 * and linked with the reference's ntt/lib/arith/bigint.c.
 *
 * Wrapped reference functions:
 *   reduce_p0/p1/p2/p3 ...... ntt/lib/primes.h:57-163
 *   addmod/submod/mulmod .... ntt/lib/primes.h:193-217
 *   make_shoup/shoup_mul .... ntt/lib/shoup.h:45-112
 *   garner_precompute +
 *   garner_reconstruct ...... ntt/lib/garner.hip:105-173, :302-332 (4 primes)
 *   bigint_scatter .......... ntt/lib/arith/bigint.c:286-294
 *   bigint_gather ........... ntt/lib/arith/bigint.c:333-397
 */
#include <stdint.h>
#include <string.h>
#include "primes.h"
#include "shoup.h"
#include "crt_ntt.h"
#include "bigint.h"
#include "garner.hip"

extern "C" {

uint64_t ref_reduce(int pidx, uint64_t lo, uint64_t hi)
{
    __uint128_t x = ((__uint128_t)hi << 64) | lo;
    switch (pidx) {
    case 0: return reduce_p0(x);
    case 1: return reduce_p1(x);
    case 2: return reduce_p2(x);
    default: return reduce_p3(x);
    }
}

uint64_t ref_mulmod(int pidx, uint64_t a, uint64_t b)
{
    switch (pidx) {
    case 0: return mulmod<0>(a, b);
    case 1: return mulmod<1>(a, b);
    case 2: return mulmod<2>(a, b);
    default: return mulmod<3>(a, b);
    }
}

uint64_t ref_addmod(int pidx, uint64_t a, uint64_t b)
{
    switch (pidx) {
    case 0: return addmod<0>(a, b);
    case 1: return addmod<1>(a, b);
    case 2: return addmod<2>(a, b);
    default: return addmod<3>(a, b);
    }
}

uint64_t ref_submod(int pidx, uint64_t a, uint64_t b)
{
    switch (pidx) {
    case 0: return submod<0>(a, b);
    case 1: return submod<1>(a, b);
    case 2: return submod<2>(a, b);
    default: return submod<3>(a, b);
    }
}

uint64_t ref_shoup_mul(int pidx, uint64_t t, uint64_t w)
{
    ShoupPair sp = make_shoup(w, PRIMES[pidx]);
    switch (pidx) {
    case 0: return shoup_mul<0>(t, sp.w, sp.w_inv);
    case 1: return shoup_mul<1>(t, sp.w, sp.w_inv);
    case 2: return shoup_mul<2>(t, sp.w, sp.w_inv);
    default: return shoup_mul<3>(t, sp.w, sp.w_inv);
    }
}

uint64_t ref_prime(int pidx) { return PRIMES[pidx]; }
uint64_t ref_prim_root(int pidx) { return PRIM_ROOT[pidx]; }

/* Garner over the reference's 4 primes for n residue tuples. */
void ref_garner4(const uint64_t *r0, const uint64_t *r1, const uint64_t *r2,
                 const uint64_t *r3, uint64_t *out_words, int n)
{
    GarnerConsts g = garner_precompute();
    garner_reconstruct(r0, r1, r2, r3, (U256 *)out_words, n, &g);
}

/* bigint_scatter over 64-bit limbs. */
void ref_scatter(const uint64_t *limbs, int n_limbs, uint64_t *coeffs,
                 int n_coeffs, int pidx)
{
    BigInt a;
    a.limbs = (limb_t *)limbs;
    a.n_limbs = n_limbs;
    a.cap = n_limbs;
    a.managed = 0;
    bigint_scatter(&a, coeffs, n_coeffs, pidx);
}

/* bigint_gather: U256 coefficients at 64-bit limb offsets -> 64-bit limbs.
 * out must hold cap limbs; returns the trimmed limb count. */
int ref_gather(const uint64_t *coeff_words, int n_coeffs, uint64_t *out, int cap)
{
    BigInt a = bigint_alloc(cap > n_coeffs + 4 ? cap : n_coeffs + 4);
    bigint_gather(&a, (const U256 *)coeff_words, n_coeffs);
    int n = a.n_limbs;
    memset(out, 0, (size_t)cap * sizeof(uint64_t));
    memcpy(out, a.limbs, (size_t)(n < cap ? n : cap) * sizeof(uint64_t));
    bigint_free(&a);
    return n;
}

}  /* extern "C" */
