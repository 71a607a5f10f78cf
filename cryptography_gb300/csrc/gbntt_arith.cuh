// gbntt_arith.cuh — modular arithmetic for the three CRT primes on sm_103a.
//
// Prime set (reference ntt/lib/primes.h:36-48, indices 0, 2 and 3 there):
//   q0 = 2^64 - 2^32 + 1, q1 = 2^64 - 2^34 + 1, q2 = 2^64 - 2^40 + 1.
// Every prime has the form p = 2^64 - 2^b + 1, so
//   2^64 == 2^b - 1 (mod p)     and     p^-1 == 1 + 2^b (mod 2^64)  (b >= 32).
// The second identity makes Montgomery reduction (R = 2^64) free of
// multiplies: m = T_lo * p^-1 = T_lo + (T_lo << b), and the high half of m*p
// is m - (m >> (64-b)) - [(m << b) mod 2^64 > m]. The reference reduces the
// full 128-bit product with Solinas folds (primes.h:57-163) and uses Shoup
// multiplication for twiddles (shoup.h:69-112); both give the same residues.
//
// Value ranges: add_mod/sub_mod take and return canonical values in [0, p).
// mont_mul(a, b) takes a in [0, 2^64) and b in [0, p) and returns the
// canonical a*b*2^-64 mod p.
#pragma once
#include <stdint.h>

namespace gbntt {

template <int PI> struct Prime;
template <> struct Prime<0> { static constexpr int B = 32; static constexpr uint64_t P = 0xFFFFFFFF00000001ull; };
template <> struct Prime<1> { static constexpr int B = 34; static constexpr uint64_t P = 0xFFFFFFFC00000001ull; };
template <> struct Prime<2> { static constexpr int B = 40; static constexpr uint64_t P = 0xFFFFFF0000000001ull; };

// 2^64 mod p = 2^b - 1.
template <int PI> __host__ __device__ constexpr uint64_t fold_const() { return (1ull << Prime<PI>::B) - 1; }

template <int PI>
__device__ __forceinline__ uint64_t add_mod(uint64_t a, uint64_t b)
{
    constexpr uint64_t C = fold_const<PI>();
    uint64_t s = a + b;          // wraps past 2^64 at most once
    uint64_t t = s + C;          // s - p (mod 2^64); carries out iff s >= p
    return (s < a || t < s) ? t : s;
}

template <int PI>
__device__ __forceinline__ uint64_t sub_mod(uint64_t a, uint64_t b)
{
    constexpr uint64_t C = fold_const<PI>();
    uint64_t d = a - b;
    return (a < b) ? d - C : d;  // d + p (mod 2^64) when a < b
}

// Montgomery product a*b/2^64 mod p for the special primes.
template <int PI>
__device__ __forceinline__ uint64_t mont_mul(uint64_t a, uint64_t b)
{
    constexpr int B = Prime<PI>::B;
    constexpr uint64_t C = fold_const<PI>();
    uint64_t lo = a * b;
    uint64_t hi = __umul64hi(a, b);
    uint64_t m = lo + (lo << B);                           // lo * p^-1 mod 2^64
    uint64_t e = (m >> (64 - B)) + (uint64_t)((m << B) > m);
    uint64_t d = hi - m;                                   // u = hi - m + e in (-p, p)
    uint64_t r = d + e;
    if (hi < m && r >= d) r -= C;                          // negative: add p
    return r;
}

// Runtime prime dispatch helpers used by host-side tables.
__host__ __device__ inline uint64_t prime_value(int pi)
{
    return pi == 0 ? 0xFFFFFFFF00000001ull : (pi == 1 ? 0xFFFFFFFC00000001ull : 0xFFFFFF0000000001ull);
}
__host__ __device__ inline int prime_b(int pi) { return pi == 0 ? 32 : (pi == 1 ? 34 : 40); }

}  // namespace gbntt
