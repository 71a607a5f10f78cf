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

// q0 = 2^64 - 2^32 + 1 specialisations with the corrections on the ALU pipe.
// With small passes the q0 kernels saturate the FMA-heavy pipe (IMAD) and
// leave the ALU pipe about a fifth idle, so for q0 the +-p corrections are
// borrow-chain subtractions of EPS = 2^32 - 1 (adding q0 mod 2^64 is
// subtracting EPS) or selects, and the Montgomery reduction needs no
// multiply at all: with m = T_lo (1 + 2^32) = (m1 : m0), m0 = t0,
// m1 = t1 + t0, the high half of m q0 is m - m1 - [m1 < m0], so
//   u = T_hi - m + m1 + [m1 < m0]   in (-q0, q0), minus EPS when negative.
#ifndef GBNTT_Q0_ALU
// bit 0: add/sub as pure borrow chains (fewer instructions: a butterfly of
// 13.4 instead of 17.4, a 16-point register DFT of 683 instead of 856, but
// all on the ALU pipe, which binds: 2^28-limb multiply 52.9 against 51.9 ms),
// bit 1: multiply-free Montgomery reduction, bit 2: power-of-two reduction;
// 2^29 transform pairs: 65.4 ms with none, 61.6 ms with bits 1 and 2.
// bit 3: the 64 x 64 product as 32-bit multiply-add carry chains instead of
// wide multiplies with zero-extended addends (61.6 -> 60.9 ms).
#define GBNTT_Q0_ALU 14
#endif
#if GBNTT_Q0_ALU & 1
template <>
__device__ __forceinline__ uint64_t add_mod<0>(uint64_t a, uint64_t b)
{
    // a + b = a - (q0 - b): q0 - b = (0xFFFFFFFF : 1) - b needs no borrow out
    // (b < q0); a borrow of a - (q0 - b) means a + b < q0, and adding q0
    // back is subtracting EPS = 2^64 - q0 with the borrow mask (bw = EPS).
    // Borrow chains only: the multiply-add corrections of the generic form
    // cost negated moves besides the multiply-adds.
    uint64_t r;
    asm("{\n\t"
        ".reg .u32 a0, a1, b0, b1, n0, n1, d0, d1, bw, r0, r1;\n\t"
        "mov.b64 {a0, a1}, %1;\n\t"
        "mov.b64 {b0, b1}, %2;\n\t"
        "sub.cc.u32 n0, 1, b0;\n\t"
        "subc.u32 n1, 0xFFFFFFFF, b1;\n\t"
        "sub.cc.u32 d0, a0, n0;\n\t"
        "subc.cc.u32 d1, a1, n1;\n\t"
        "subc.u32 bw, 0, 0;\n\t"
        "sub.cc.u32 r0, d0, bw;\n\t"
        "subc.u32 r1, d1, 0;\n\t"
        "mov.b64 %0, {r0, r1};\n\t"
        "}"
        : "=l"(r) : "l"(a), "l"(b));
    return r;
}

template <>
__device__ __forceinline__ uint64_t sub_mod<0>(uint64_t a, uint64_t b)
{
    // d = a - b; on borrow (bw = 0xFFFFFFFF) subtract EPS = bw
    uint64_t r;
    asm("{\n\t"
        ".reg .u32 a0, a1, b0, b1, d0, d1, bw, r0, r1;\n\t"
        "mov.b64 {a0, a1}, %1;\n\t"
        "mov.b64 {b0, b1}, %2;\n\t"
        "sub.cc.u32 d0, a0, b0;\n\t"
        "subc.cc.u32 d1, a1, b1;\n\t"
        "subc.u32 bw, 0, 0;\n\t"
        "sub.cc.u32 r0, d0, bw;\n\t"
        "subc.u32 r1, d1, 0;\n\t"
        "mov.b64 %0, {r0, r1};\n\t"
        "}"
        : "=l"(r) : "l"(a), "l"(b));
    return r;
}
#endif

#if GBNTT_Q0_ALU & 2
template <>
__device__ __forceinline__ uint64_t mont_mul<0>(uint64_t a, uint64_t b)
{
    uint64_t r;
    asm("{\n\t"
        ".reg .u32 a0, a1, b0, b1, z, l00, h00, l01, h01, l10, h10, t2, t3, m1, s, v0, v1, bw, w0, w1, cy, r0, r1;\n\t"
        ".reg .u64 p00, p01, p10, p11, w;\n\t"
        ".reg .pred lt;\n\t"
        "mov.b64 {a0, a1}, %1;\n\t"
        "mov.b64 {b0, b1}, %2;\n\t"
#if GBNTT_Q0_ALU & 8
        // T = (t3 : t2 : l10 : l00) through 32-bit carry chains
        "mul.lo.u32 l00, a0, b0;\n\t"
        "mul.hi.u32 l10, a0, b0;\n\t"
        "mad.lo.cc.u32 l10, a0, b1, l10;\n\t"
        "madc.hi.u32 t2, a0, b1, 0;\n\t"
        "mad.lo.cc.u32 l10, a1, b0, l10;\n\t"
        "madc.hi.cc.u32 t2, a1, b0, t2;\n\t"
        "addc.u32 t3, 0, 0;\n\t"
        "mad.lo.cc.u32 t2, a1, b1, t2;\n\t"
        "madc.hi.u32 t3, a1, b1, t3;\n\t"
#else
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
        "mov.b64 {t2, t3}, p11;\n\t"
        "add.cc.u32 t2, t2, h10;\n\t"           // T_hi = (t3 : t2)
        "addc.u32 t3, t3, 0;\n\t"
#endif
        "add.u32 m1, l10, l00;\n\t"              // m = (m1 : l00)
        "setp.lt.u32 lt, m1, l00;\n\t"
        "selp.u32 s, 1, 0, lt;\n\t"
        "add.u32 s, s, m1;\n\t"                  // s = m1 + [m1 < m0] < 2^32
        "sub.cc.u32 v0, t2, l00;\n\t"            // v = T_hi - m
        "subc.cc.u32 v1, t3, m1;\n\t"
        "subc.u32 bw, 0, 0;\n\t"
        "add.cc.u32 w0, v0, s;\n\t"              // w = v + s
        "addc.cc.u32 w1, v1, 0;\n\t"
        "addc.u32 cy, bw, 0;\n\t"               // 0xFFFFFFFF: u < 0
        "sub.cc.u32 r0, w0, cy;\n\t"             // u + q0 = w - EPS
        "subc.u32 r1, w1, 0;\n\t"
        "mov.b64 %0, {r0, r1};\n\t"
        "}"
        : "=l"(r) : "l"(a), "l"(b));
    return r;
}
#endif

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

// ---------------------------------------------------------------------------
// The 32-bit prime p3 = 3 * 2^30 + 1 (2-adicity 30, the only prime below
// 2^32 with roots of unity of order 2^29 and 2^30). Together with q0 it
// gives a CRT modulus q0 p3 ~ 2^95.6, above every coefficient of a product
// of 32-bit limbs with up to 2^29 limbs in the shorter operand (< 2^93): the
// 32-bit-coefficient products need only these two primes. p3 > 2^31, so
// sums need 33 bits; the forms below never form them.
//   add: a + b = a - (p - b), plus p on borrow.
//   mul: signed Montgomery, R = 2^32: m = lo(a b) p^-1 mod 2^32 makes
//        lo(m p) = lo(a b), so (a b - m p) / 2^32 = hi(a b) - hi(m p)
//        exactly, in (-p, p); add p on borrow. Output canonical.
// ---------------------------------------------------------------------------
constexpr uint32_t kP3 = 0xC0000001u;          // 3 * 2^30 + 1
constexpr uint32_t kP3Inv = 0x40000001u;       // p3^-1 mod 2^32
constexpr uint32_t kP3Neg = 0x3FFFFFFFu;       // -p3 mod 2^32

#ifndef GBNTT_P3_ALU
#define GBNTT_P3_ALU 0   // p3 corrections as and + add (ALU pipe) instead of IMAD (measured +0.6 ms at 2^29)
#endif
#if GBNTT_P3_ALU
__device__ __forceinline__ uint32_t p3_add(uint32_t a, uint32_t b)
{
    uint32_t r;
    asm("{\n\t"
        ".reg .u32 nb, d, bw, k;\n\t"
        "sub.u32 nb, %3, %2;\n\t"
        "sub.cc.u32 d, %1, nb;\n\t"
        "subc.u32 bw, 0, 0;\n\t"
        "and.b32 k, bw, %3;\n\t"
        "add.u32 %0, d, k;\n\t"
        "}"
        : "=r"(r) : "r"(a), "r"(b), "n"(kP3));
    return r;
}

__device__ __forceinline__ uint32_t p3_sub(uint32_t a, uint32_t b)
{
    uint32_t r;
    asm("{\n\t"
        ".reg .u32 d, bw, k;\n\t"
        "sub.cc.u32 d, %1, %2;\n\t"
        "subc.u32 bw, 0, 0;\n\t"
        "and.b32 k, bw, %3;\n\t"
        "add.u32 %0, d, k;\n\t"
        "}"
        : "=r"(r) : "r"(a), "r"(b), "n"(kP3));
    return r;
}

__device__ __forceinline__ uint32_t p3_mul(uint32_t a, uint32_t b)
{
    uint32_t r;
    asm("{\n\t"
        ".reg .u32 t0, t1, m, h, d, bw, k;\n\t"
        ".reg .u64 t;\n\t"
        "mul.wide.u32 t, %1, %2;\n\t"
        "mov.b64 {t0, t1}, t;\n\t"
        "mul.lo.u32 m, t0, %3;\n\t"
        "mul.hi.u32 h, m, %4;\n\t"
        "sub.cc.u32 d, t1, h;\n\t"
        "subc.u32 bw, 0, 0;\n\t"
        "and.b32 k, bw, %4;\n\t"
        "add.u32 %0, d, k;\n\t"
        "}"
        : "=r"(r) : "r"(a), "r"(b), "n"(kP3Inv), "n"(kP3));
    return r;
}
#else
__device__ __forceinline__ uint32_t p3_add(uint32_t a, uint32_t b)
{
    uint32_t r;
    asm("{\n\t"
        ".reg .u32 nb, d, bw;\n\t"
        "sub.u32 nb, %3, %2;\n\t"
        "sub.cc.u32 d, %1, nb;\n\t"
        "subc.u32 bw, 0, 0;\n\t"
        "mad.lo.u32 %0, bw, %4, d;\n\t"
        "}"
        : "=r"(r) : "r"(a), "r"(b), "n"(kP3), "n"(kP3Neg));
    return r;
}

__device__ __forceinline__ uint32_t p3_sub(uint32_t a, uint32_t b)
{
    uint32_t r;
    asm("{\n\t"
        ".reg .u32 d, bw;\n\t"
        "sub.cc.u32 d, %1, %2;\n\t"
        "subc.u32 bw, 0, 0;\n\t"
        "mad.lo.u32 %0, bw, %3, d;\n\t"
        "}"
        : "=r"(r) : "r"(a), "r"(b), "n"(kP3Neg));
    return r;
}

// a * b * 2^-32 mod p3 for a < 2^32, b < p3 (then hi(a b) < p3).
__device__ __forceinline__ uint32_t p3_mul(uint32_t a, uint32_t b)
{
    uint32_t r;
    asm("{\n\t"
        ".reg .u32 t0, t1, m, h, d, bw;\n\t"
        ".reg .u64 t;\n\t"
        "mul.wide.u32 t, %1, %2;\n\t"
        "mov.b64 {t0, t1}, t;\n\t"
        "mul.lo.u32 m, t0, %3;\n\t"
        "mul.hi.u32 h, m, %4;\n\t"
        "sub.cc.u32 d, t1, h;\n\t"
        "subc.u32 bw, 0, 0;\n\t"
        "mad.lo.u32 %0, bw, %5, d;\n\t"
        "}"
        : "=r"(r) : "r"(a), "r"(b), "n"(kP3Inv), "n"(kP3), "n"(kP3Neg));
    return r;
}
#endif

// plain C++ forms for the device self-test
__device__ __forceinline__ uint32_t p3_add_ref(uint32_t a, uint32_t b)
{
    const uint64_t s = (uint64_t)a + b;
    return (uint32_t)(s >= kP3 ? s - kP3 : s);
}
__device__ __forceinline__ uint32_t p3_sub_ref(uint32_t a, uint32_t b) { return a >= b ? a - b : a + (kP3 - b); }
__device__ __forceinline__ uint32_t p3_mul_ref(uint32_t a, uint32_t b)
{
    // a b 2^-32 mod p3 through the 64-bit remainder and 2^-32 mod p3
    const uint64_t t = (uint64_t)a * b % kP3;
    constexpr uint64_t kRinv = 0x90000000ull;   // 2^-32 mod p3
    return (uint32_t)(t * kRinv % kP3);
}

// ---------------------------------------------------------------------------
// q0 = 2^64 - 2^32 + 1 in normal form with lazy residues: any 64-bit word x
// stands for x mod q0 (EPS = 2^64 mod q0 = 2^32 - 1, 2^96 == -1). Products
// fold the 128-bit result without multiplies:
//   t = t0 + t1 2^32 + t2 2^64 + t3 2^96 == (t1:t0) - t3 + t2 EPS,
// sums and differences fold their carry or borrow by EPS (at most twice).
// Outputs lie in [0, 2^64); the Garner stage reduces them.
// ---------------------------------------------------------------------------
__device__ __forceinline__ uint64_t gl_add(uint64_t a, uint64_t b)
{
    uint64_t r;
    asm("{\n\t"
        ".reg .u32 a0, a1, b0, b1, s0, s1, c, c2;\n\t"
        "mov.b64 {a0, a1}, %1;\n\t"
        "mov.b64 {b0, b1}, %2;\n\t"
        "add.cc.u32 s0, a0, b0;\n\t"
        "addc.cc.u32 s1, a1, b1;\n\t"
        "addc.u32 c, 0, 0;\n\t"
        "mad.lo.cc.u32 s0, c, 0xFFFFFFFF, s0;\n\t"
        "addc.cc.u32 s1, s1, 0;\n\t"
        "addc.u32 c2, 0, 0;\n\t"
        "mad.lo.cc.u32 s0, c2, 0xFFFFFFFF, s0;\n\t"
        "addc.u32 s1, s1, 0;\n\t"
        "mov.b64 %0, {s0, s1};\n\t"
        "}"
        : "=l"(r) : "l"(a), "l"(b));
    return r;
}

__device__ __forceinline__ uint64_t gl_sub(uint64_t a, uint64_t b)
{
    // on borrow the wrapped difference is 2^64 too large: subtract EPS (== 2^64),
    // and once more if that wraps as well
    uint64_t r;
    asm("{\n\t"
        ".reg .u32 a0, a1, b0, b1, d0, d1, bw, bw2;\n\t"
        "mov.b64 {a0, a1}, %1;\n\t"
        "mov.b64 {b0, b1}, %2;\n\t"
        "sub.cc.u32 d0, a0, b0;\n\t"
        "subc.cc.u32 d1, a1, b1;\n\t"
        "subc.u32 bw, 0, 0;\n\t"
        "sub.cc.u32 d0, d0, bw;\n\t"
        "subc.cc.u32 d1, d1, 0;\n\t"
        "subc.u32 bw2, 0, 0;\n\t"
        "sub.cc.u32 d0, d0, bw2;\n\t"
        "subc.u32 d1, d1, 0;\n\t"
        "mov.b64 %0, {d0, d1};\n\t"
        "}"
        : "=l"(r) : "l"(a), "l"(b));
    return r;
}

__device__ __forceinline__ uint64_t gl_mul(uint64_t a, uint64_t b)
{
    uint64_t r;
    asm("{\n\t"
        ".reg .u32 a0, a1, b0, b1, z, l00, h00, l01, h01, l10, h10, t2, t3, x0, x1, bw, y0, y1, r0, r1, c;\n\t"
        ".reg .u64 p00, p01, p10, p11, th, w;\n\t"
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
        "mov.b64 {t2, t3}, th;\n\t"
        // x = (l10:l00) - t3, + q0 on borrow (add 0xFFFFFFFF00000001 = -EPS)
        "sub.cc.u32 x0, l00, t3;\n\t"
        "subc.cc.u32 x1, l10, 0;\n\t"
        "subc.u32 bw, 0, 0;\n\t"
        "mad.lo.cc.u32 x0, bw, 0xFFFFFFFF, x0;\n\t"
        "madc.lo.u32 x1, bw, 1, x1;\n\t"
        // y = t2 * EPS = (t2 << 32) - t2
        "sub.cc.u32 y0, 0, t2;\n\t"
        "subc.u32 y1, t2, 0;\n\t"
        // r = x + y, + EPS on carry (no second carry)
        "add.cc.u32 r0, x0, y0;\n\t"
        "addc.cc.u32 r1, x1, y1;\n\t"
        "addc.u32 c, 0, 0;\n\t"
        "mad.lo.cc.u32 r0, c, 0xFFFFFFFF, r0;\n\t"
        "addc.u32 r1, r1, 0;\n\t"
        "mov.b64 %0, {r0, r1};\n\t"
        "}"
        : "=l"(r) : "l"(a), "l"(b));
    return r;
}

// (v1:v0) + v2 EPS - v3 mod q0 (the value of v0 + v1 2^32 + v2 2^64 +
// v3 2^96), canonical.
#if GBNTT_Q0_ALU & 4
// corrections as borrow chains and selects (ALU pipe)
__device__ __forceinline__ uint64_t gl_reduce4(uint32_t v0, uint32_t v1, uint32_t v2, uint32_t v3)
{
    uint64_t r;
    asm("{\n\t"
        ".reg .u32 x0, x1, bw, y0, y1, r0, r1, c, m, t0, t1, c2;\n\t"
        ".reg .pred p;\n\t"
        "sub.cc.u32 x0, %1, %4;\n\t"            // x = (v1:v0) - v3, + q0 (= - EPS) on borrow
        "subc.cc.u32 x1, %2, 0;\n\t"
        "subc.u32 bw, 0, 0;\n\t"
        "sub.cc.u32 x0, x0, bw;\n\t"
        "subc.u32 x1, x1, 0;\n\t"
        "sub.cc.u32 y0, 0, %3;\n\t"             // y = v2 EPS = (v2 << 32) - v2
        "subc.u32 y1, %3, 0;\n\t"
        "add.cc.u32 r0, x0, y0;\n\t"            // r = x + y, + EPS on carry
        "addc.cc.u32 r1, x1, y1;\n\t"
        "addc.u32 c, 0, 0;\n\t"
        "neg.s32 m, c;\n\t"
        "add.cc.u32 r0, r0, m;\n\t"
        "addc.u32 r1, r1, 0;\n\t"
        "add.cc.u32 t0, r0, 0xFFFFFFFF;\n\t"     // canonical: r - q0 = r + EPS when r >= q0
        "addc.cc.u32 t1, r1, 0;\n\t"
        "addc.u32 c2, 0, 0;\n\t"
        "setp.ne.u32 p, c2, 0;\n\t"
        "selp.u32 r0, t0, r0, p;\n\t"
        "selp.u32 r1, t1, r1, p;\n\t"
        "mov.b64 %0, {r0, r1};\n\t"
        "}"
        : "=l"(r) : "r"(v0), "r"(v1), "r"(v2), "r"(v3));
    return r;
}
#else
__device__ __forceinline__ uint64_t gl_reduce4(uint32_t v0, uint32_t v1, uint32_t v2, uint32_t v3)
{
    uint64_t r;
    asm("{\n\t"
        ".reg .u32 x0, x1, bw, y0, y1, r0, r1, c, t0, t1, c2;\n\t"
        "sub.cc.u32 x0, %1, %4;\n\t"
        "subc.cc.u32 x1, %2, 0;\n\t"
        "subc.u32 bw, 0, 0;\n\t"
        "mad.lo.cc.u32 x0, bw, 0xFFFFFFFF, x0;\n\t"
        "madc.lo.u32 x1, bw, 1, x1;\n\t"
        "sub.cc.u32 y0, 0, %3;\n\t"
        "subc.u32 y1, %3, 0;\n\t"
        "add.cc.u32 r0, x0, y0;\n\t"
        "addc.cc.u32 r1, x1, y1;\n\t"
        "addc.u32 c, 0, 0;\n\t"
        "mad.lo.cc.u32 r0, c, 0xFFFFFFFF, r0;\n\t"
        "addc.u32 r1, r1, 0;\n\t"
        "add.cc.u32 t0, r0, 0xFFFFFFFF;\n\t"
        "addc.cc.u32 t1, r1, 0;\n\t"
        "addc.u32 c2, 0, 0;\n\t"
        "mad.lo.cc.u32 r0, c2, 0xFFFFFFFF, r0;\n\t"
        "addc.u32 r1, r1, 0;\n\t"
        "mov.b64 %0, {r0, r1};\n\t"
        "}"
        : "=l"(r) : "r"(v0), "r"(v1), "r"(v2), "r"(v3));
    return r;
}
#endif

#ifndef GBNTT_Q0_POW2
#define GBNTT_Q0_POW2 1   // 1: the shorter per-range forms below; 0: the general fold gl_reduce4
#endif

// Canonical form of w = (w1:w0) < 2^64: w >= q0 exactly when w1 is all ones
// and w0 is nonzero, and then w - q0 = (0 : w0 - 1).
#define GBNTT_GL_CANON_W                                  \
    "setp.eq.u32 p, w1, 0xFFFFFFFF;\n\t"                  \
    "setp.ne.and.u32 p, w0, 0, p;\n\t"                   \
    "@p sub.u32 w0, w0, 1;\n\t"                          \
    "@p mov.u32 w1, 0;\n\t"

// x 2^r for r < 32 as u = (u2 : u1 : u0), u2 < 2^r: (u1:u0) + u2 EPS
// = (u1:u0) - u2 + (u2 << 32) is below 2^64 + 2^63 (carry c in {0, 1}),
// folded once by c EPS (no second carry), then made canonical.
__device__ __forceinline__ uint64_t gl_pow2_q0(uint32_t u0, uint32_t u1, uint32_t u2)
{
    uint64_t r;
    asm("{\n\t"
        ".reg .u32 s0, s1, b, c, w0, w1;\n\t"
        ".reg .pred p;\n\t"
        "sub.cc.u32 s0, %1, %3;\n\t"
        "subc.cc.u32 s1, %2, 0;\n\t"
        "subc.u32 b, 0, 0;\n\t"
        "add.cc.u32 s1, s1, %3;\n\t"
        "addc.u32 c, b, 0;\n\t"
        "mad.lo.cc.u32 w0, c, 0xFFFFFFFF, s0;\n\t"
        "addc.u32 w1, s1, 0;\n\t"
        GBNTT_GL_CANON_W
        "mov.b64 %0, {w0, w1};\n\t"
        "}"
        : "=l"(r) : "r"(u0), "r"(u1), "r"(u2));
    return r;
}

// x 2^(32 + r) for r < 32, u as above: u0 2^32 + u1 2^64 + u2 2^96
// == (u0 + u1) 2^32 - (u1 + u2) = v2 2^64 + (v1:v0) with v2 in {-1, 0, 1};
// folding v2 EPS leaves a canonical value unless v2 = 0, so one check.
__device__ __forceinline__ uint64_t gl_pow2_q1(uint32_t u0, uint32_t u1, uint32_t u2)
{
    uint64_t r;
    asm("{\n\t"
        ".reg .u32 h, hc, s, sc, v0, v1, v2, n, sg, w0, w1;\n\t"
        ".reg .pred p;\n\t"
        "add.cc.u32 h, %1, %2;\n\t"
        "addc.u32 hc, 0, 0;\n\t"
        "add.cc.u32 s, %2, %3;\n\t"
        "addc.u32 sc, 0, 0;\n\t"
        "sub.cc.u32 v0, 0, s;\n\t"
        "subc.cc.u32 v1, h, sc;\n\t"
        "subc.u32 v2, hc, 0;\n\t"
        "neg.s32 n, v2;\n\t"
        "shr.s32 sg, v2, 31;\n\t"
        "add.cc.u32 w0, v0, n;\n\t"
        "addc.u32 w1, v1, sg;\n\t"
        GBNTT_GL_CANON_W
        "mov.b64 %0, {w0, w1};\n\t"
        "}"
        : "=l"(r) : "r"(u0), "r"(u1), "r"(u2));
    return r;
}

// x * 2^e mod q0 for canonical x and 0 <= e < 96 (e folds to a constant
// after unrolling, so the shifts and the branch on e / 32 vanish). In q0
// every 64th root of unity is a power of two (2^96 == -1, 2^192 == 1), so
// the register DFTs multiply by these instead of full products.
__device__ __forceinline__ uint64_t gl_mul_pow2(uint64_t x, int e)
{
    if (e == 0) return x;
    const uint32_t x0 = (uint32_t)x, x1 = (uint32_t)(x >> 32);
    const int q = e >> 5, r = e & 31;
    const uint32_t u0 = x0 << r;
    const uint32_t u1 = r ? ((x1 << r) | (x0 >> (32 - r))) : x1;
    const uint32_t u2 = r ? (x1 >> (32 - r)) : 0u;
#if GBNTT_Q0_POW2
    if (q == 0) return gl_pow2_q0(u0, u1, u2);
    if (q == 1) return gl_pow2_q1(u0, u1, u2);
#else
    if (q == 0) return gl_reduce4(u0, u1, u2, 0u);
    if (q == 1) return gl_reduce4(0u, u0, u1, u2);
#endif
    // q == 2: u0 2^64 + u1 2^96 + u2 2^128 == u0 EPS - (u2 2^32 + u1), the
    // subtrahend below 2^63 < q0
    const uint64_t y = ((uint64_t)u0 << 32) - (uint64_t)u0;   // u0 EPS < q0
    return sub_mod<0>(y, ((uint64_t)u2 << 32) | u1);
}

// canonical representative in [0, q0)
__host__ __device__ __forceinline__ uint64_t gl_canon(uint64_t x)
{
    return x >= 0xFFFFFFFF00000001ull ? x - 0xFFFFFFFF00000001ull : x;
}

// plain C++ forms for the device self-test (canonical results)
__device__ __forceinline__ uint64_t gl_add_ref(uint64_t a, uint64_t b)
{
    constexpr uint64_t P = 0xFFFFFFFF00000001ull;
    return (uint64_t)(((unsigned __int128)a + b) % P);
}
__device__ __forceinline__ uint64_t gl_sub_ref(uint64_t a, uint64_t b)
{
    constexpr uint64_t P = 0xFFFFFFFF00000001ull;
    return (uint64_t)(((unsigned __int128)(a % P) + P - (b % P)) % P);
}
__device__ __forceinline__ uint64_t gl_mul_ref(uint64_t a, uint64_t b)
{
    constexpr uint64_t P = 0xFFFFFFFF00000001ull;
    return (uint64_t)(((unsigned __int128)a * b) % P);
}

// ---------------------------------------------------------------------------
// Field policies for the pass kernels: prime index PI -> residue word T,
// slot in the per-launch argument arrays, and the three operations. Primes
// 0..2 are the 64-bit Montgomery primes above (slots 0..2); prime 3 is p3
// and prime 4 is lazy normal-form q0 (slots 1 and 0 of the two-prime set).
// ---------------------------------------------------------------------------
// Beside add/sub/mul every policy converts from a 32-bit limb (from_u32)
// and from the 64-bit form host code uses (from_u64), gives zero() and the
// low 32 bits of a residue (low32).
template <int PI>
struct Field {
    typedef uint64_t T;
    static constexpr int SLOT = PI;
    static constexpr uint64_t P = Prime<PI>::P;
    static __device__ __forceinline__ T add(T a, T b) { return add_mod<PI>(a, b); }
    static __device__ __forceinline__ T sub(T a, T b) { return sub_mod<PI>(a, b); }
    static __device__ __forceinline__ T mul(T a, T b) { return mont_mul<PI>(a, b); }
    static __device__ __forceinline__ T from_u32(uint32_t v) { return v; }   // v < 2^32 < p
    static __device__ __forceinline__ T from_u64(uint64_t v) { return v; }
    static __device__ __forceinline__ T zero() { return 0; }
    static __device__ __forceinline__ uint32_t low32(T v) { return (uint32_t)v; }
};

template <>
struct Field<3> {
    typedef uint32_t T;
    static constexpr int SLOT = 1;
    static constexpr uint64_t P = kP3;
    static __device__ __forceinline__ T add(T a, T b) { return p3_add(a, b); }
    static __device__ __forceinline__ T sub(T a, T b) { return p3_sub(a, b); }
    static __device__ __forceinline__ T mul(T a, T b) { return p3_mul(a, b); }
    static __device__ __forceinline__ T from_u32(uint32_t v) { return v >= kP3 ? v - kP3 : v; }   // 2^32 < 2 p3
    static __device__ __forceinline__ T from_u64(uint64_t v) { return (uint32_t)v; }
    static __device__ __forceinline__ T zero() { return 0; }
    static __device__ __forceinline__ uint32_t low32(T v) { return v; }
};

// Prime 4 is q0 again, in normal form with lazy residues (slot 0 of the
// two-prime set); prime 0 (Montgomery q0) stays in the three-prime set.
template <>
struct Field<4> {
    typedef uint64_t T;
    static constexpr int SLOT = 0;
    static constexpr uint64_t P = 0xFFFFFFFF00000001ull;
    static __device__ __forceinline__ T add(T a, T b) { return gl_add(a, b); }
    static __device__ __forceinline__ T sub(T a, T b) { return gl_sub(a, b); }
    static __device__ __forceinline__ T mul(T a, T b) { return gl_mul(a, b); }
    static __device__ __forceinline__ T from_u32(uint32_t v) { return v; }
    static __device__ __forceinline__ T from_u64(uint64_t v) { return v; }
    static __device__ __forceinline__ T zero() { return 0; }
    static __device__ __forceinline__ uint32_t low32(T v) { return (uint32_t)v; }
};

// Runtime prime dispatch helpers used by host-side tables.
__host__ __device__ inline uint64_t prime_value(int pi)
{
    return (pi == 0 || pi == 4) ? 0xFFFFFFFF00000001ull
                                : (pi == 1 ? 0xFFFFFFFC00000001ull : (pi == 2 ? 0xFFFFFF0000000001ull : (uint64_t)kP3));
}
__host__ __device__ inline int prime_b(int pi) { return pi == 0 ? 32 : (pi == 1 ? 34 : 40); }

}  // namespace gbntt
