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

// hi word of p (p = P1 * 2^32 + 1 for all three primes) and 2^32 - P1.
template <int PI> __host__ __device__ constexpr uint32_t p_hi() { return (uint32_t)(Prime<PI>::P >> 32); }
template <int PI> __host__ __device__ constexpr uint32_t p_hi_neg() { return (uint32_t)(0x100000000ull - p_hi<PI>()); }

// The three operations below are written with 32-bit carry chains so that
// the corrections by +-p are multiply-adds by a 0/-1 borrow mask (IMAD, on
// the FMA pipe) instead of 64-bit compares and selects (ALU pipe): integer
// NTT passes are bound by the ALU pipe otherwise.

template <int PI>
__device__ __forceinline__ uint64_t add_mod(uint64_t a, uint64_t b)
{
    // s = a + b; c2 = [s >= p or a + b >= 2^64] (the carry of s + (2^64 - p));
    // result = s + c2 * (2^64 - p) mod 2^64.
    constexpr uint32_t C1 = (uint32_t)(fold_const<PI>() >> 32);
    uint64_t r;
    asm("{\n\t"
        ".reg .u32 a0, a1, b0, b1, s0, s1, c, c2, x0, x1, r0, r1;\n\t"
        "mov.b64 {a0, a1}, %1;\n\t"
        "mov.b64 {b0, b1}, %2;\n\t"
        "add.cc.u32 s0, a0, b0;\n\t"
        "addc.cc.u32 s1, a1, b1;\n\t"
        "addc.u32 c, 0, 0;\n\t"
        "add.cc.u32 x0, s0, 0xFFFFFFFF;\n\t"
        "addc.cc.u32 x1, s1, %3;\n\t"
        "addc.u32 c2, c, 0;\n\t"
        "mad.lo.cc.u32 r0, c2, 0xFFFFFFFF, s0;\n\t"
        "madc.lo.u32 r1, c2, %3, s1;\n\t"
        "mov.b64 %0, {r0, r1};\n\t"
        "}"
        : "=l"(r) : "l"(a), "l"(b), "n"(C1));
    return r;
}

template <int PI>
__device__ __forceinline__ uint64_t sub_mod(uint64_t a, uint64_t b)
{
    // d = a - b; on borrow add p = P1 * 2^32 + 1 via the mask bw = -borrow.
    uint64_t r;
    asm("{\n\t"
        ".reg .u32 a0, a1, b0, b1, d0, d1, bw, r0, r1;\n\t"
        "mov.b64 {a0, a1}, %1;\n\t"
        "mov.b64 {b0, b1}, %2;\n\t"
        "sub.cc.u32 d0, a0, b0;\n\t"
        "subc.cc.u32 d1, a1, b1;\n\t"
        "subc.u32 bw, 0, 0;\n\t"
        "mad.lo.cc.u32 r0, bw, 0xFFFFFFFF, d0;\n\t"
        "madc.lo.u32 r1, bw, %3, d1;\n\t"
        "mov.b64 %0, {r0, r1};\n\t"
        "}"
        : "=l"(r) : "l"(a), "l"(b), "n"(p_hi_neg<PI>()));
    return r;
}

// Montgomery product a*b/2^64 mod p for the special primes.
//   T = a*b from five 32x32->64 multiply-adds.
//   m = T_lo * p^-1 mod 2^64: m0 = t0, m1 = t1 + t0 * 2^(b-32).
//   hi(m*p) = m1*P1 + ((m0*P1 + m1) >> 32)   (p's low word is 1).
//   u = T_hi - hi(m*p) in (-p, p); add p on borrow.
template <int PI>
__device__ __forceinline__ uint64_t mont_mul(uint64_t a, uint64_t b)
{
    constexpr uint32_t SHM = 1u << (Prime<PI>::B - 32);
    uint64_t r;
    asm("{\n\t"
        ".reg .u32 a0, a1, b0, b1, t0, t1, h0, h1, z, m1, k0, k1, u0, u1, bw, r0, r1, l00, h00, l01, h01, l10, h10;\n\t"
        ".reg .u64 p00, p01, p10, p11, th, k, hh, w;\n\t"
        "mov.b64 {a0, a1}, %1;\n\t"
        "mov.b64 {b0, b1}, %2;\n\t"
        "mov.u32 z, 0;\n\t"
        "mul.wide.u32 p00, a0, b0;\n\t"
        "mov.b64 {l00, h00}, p00;\n\t"
        "mov.b64 w, {h00, z};\n\t"
        "mad.wide.u32 p01, a0, b1, w;\n\t"
        "mov.b64 {l01, h01}, p01;\n\t"
        "mov.b64 w, {l01, z};\n\t"
        "mad.wide.u32 p10, a1, b0, w;\n\t"
        "mov.b64 {l10, h10}, p10;\n\t"
        "mov.b64 w, {h01, z};\n\t"
        "mad.wide.u32 p11, a1, b1, w;\n\t"
        "mad.wide.u32 th, h10, 1, p11;\n\t"
        "mov.b64 {h0, h1}, th;\n\t"
        "mad.lo.u32 m1, l00, %3, l10;\n\t"
        "mov.b64 w, {m1, z};\n\t"
        "mad.wide.u32 k, l00, %4, w;\n\t"
        "mov.b64 {k0, k1}, k;\n\t"
        "mov.b64 w, {k1, z};\n\t"
        "mad.wide.u32 hh, m1, %4, w;\n\t"
        "mov.b64 {k0, k1}, hh;\n\t"
        "sub.cc.u32 u0, h0, k0;\n\t"
        "subc.cc.u32 u1, h1, k1;\n\t"
        "subc.u32 bw, 0, 0;\n\t"
        "mad.lo.cc.u32 r0, bw, 0xFFFFFFFF, u0;\n\t"
        "madc.lo.u32 r1, bw, %5, u1;\n\t"
        "mov.b64 %0, {r0, r1};\n\t"
        "}"
        : "=l"(r) : "l"(a), "l"(b), "n"(SHM), "n"(p_hi<PI>()), "n"(p_hi_neg<PI>()));
    return r;
}

// Reference forms of the same three operations in plain C++ (64-bit compares
// and selects); kept for the device self-test that pins the PTX forms.
template <int PI>
__device__ __forceinline__ uint64_t add_mod_ref(uint64_t a, uint64_t b)
{
    constexpr uint64_t C = fold_const<PI>();
    uint64_t s = a + b;
    uint64_t t = s + C;
    return (s < a || t < s) ? t : s;
}
template <int PI>
__device__ __forceinline__ uint64_t sub_mod_ref(uint64_t a, uint64_t b)
{
    constexpr uint64_t C = fold_const<PI>();
    uint64_t d = a - b;
    return (a < b) ? d - C : d;
}
template <int PI>
__device__ __forceinline__ uint64_t mont_mul_ref(uint64_t a, uint64_t b)
{
    constexpr int B = Prime<PI>::B;
    constexpr uint64_t C = fold_const<PI>();
    uint64_t lo = a * b;
    uint64_t hi = __umul64hi(a, b);
    uint64_t m = lo + (lo << B);
    uint64_t e = (m >> (64 - B)) + (uint64_t)((m << B) > m);
    uint64_t d = hi - m;
    uint64_t r = d + e;
    if (hi < m && r >= d) r -= C;
    return r;
}

// Runtime prime dispatch helpers used by host-side tables.
__host__ __device__ inline uint64_t prime_value(int pi)
{
    return pi == 0 ? 0xFFFFFFFF00000001ull : (pi == 1 ? 0xFFFFFFFC00000001ull : 0xFFFFFF0000000001ull);
}
__host__ __device__ inline int prime_b(int pi) { return pi == 0 ? 32 : (pi == 1 ? 34 : 40); }

}  // namespace gbntt
