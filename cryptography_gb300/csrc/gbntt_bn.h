// gbntt_bn.h — host big-integer helpers used by the e pipeline (the
// reference's arith layer, ntt/lib/arith/bigint.c and newton.c, restated on
// 32-bit limbs). Multiplication of large operands is not here: it goes to
// the GPU engine; these are the O(n) operations and the small products that
// the reference also keeps on the CPU (its schoolbook threshold,
// ntt/lib/arith/multiply.h:23-25).
#pragma once
#include <stdint.h>
#include <string.h>
#include <algorithm>
#include <vector>

namespace gbntt {
namespace bn {

typedef std::vector<uint32_t> Num;   // little-endian, trimmed (zero = empty)

inline void trim(Num &a)
{
    while (!a.empty() && a.back() == 0) a.pop_back();
}

inline size_t bits(const Num &a)
{
    if (a.empty()) return 0;
    return 32 * (a.size() - 1) + (32 - __builtin_clz(a.back()));
}

inline int cmp(const Num &a, const Num &b)
{
    if (a.size() != b.size()) return a.size() < b.size() ? -1 : 1;
    for (size_t i = a.size(); i-- > 0;)
        if (a[i] != b[i]) return a[i] < b[i] ? -1 : 1;
    return 0;
}

inline Num add(const Num &a, const Num &b)
{
    const Num &x = a.size() >= b.size() ? a : b;
    const Num &y = a.size() >= b.size() ? b : a;
    Num r(x.size() + 1);
    uint64_t c = 0;
    for (size_t i = 0; i < x.size(); i++) {
        c += (uint64_t)x[i] + (i < y.size() ? y[i] : 0);
        r[i] = (uint32_t)c;
        c >>= 32;
    }
    r[x.size()] = (uint32_t)c;
    trim(r);
    return r;
}

// a - b, requires a >= b
inline Num sub(const Num &a, const Num &b)
{
    Num r(a.size());
    int64_t br = 0;
    for (size_t i = 0; i < a.size(); i++) {
        int64_t v = (int64_t)a[i] - (i < b.size() ? b[i] : 0) - br;
        br = v < 0;
        r[i] = (uint32_t)(v + (br << 32));
    }
    trim(r);
    return r;
}

inline Num shl(const Num &a, size_t n)
{
    if (a.empty()) return a;
    const size_t w = n / 32, s = n % 32;
    Num r(a.size() + w + 1, 0);
    for (size_t i = 0; i < a.size(); i++) {
        const uint64_t v = (uint64_t)a[i] << s;
        r[i + w] |= (uint32_t)v;
        r[i + w + 1] |= (uint32_t)(v >> 32);
    }
    trim(r);
    return r;
}

inline Num shr(const Num &a, size_t n)
{
    const size_t w = n / 32, s = n % 32;
    if (w >= a.size()) return Num();
    Num r(a.size() - w);
    for (size_t i = 0; i < r.size(); i++) {
        uint64_t v = a[i + w];
        if (i + w + 1 < a.size()) v |= (uint64_t)a[i + w + 1] << 32;
        r[i] = (uint32_t)(v >> s);
    }
    trim(r);
    return r;
}

// a = a * m + c
inline void mul_small_add(Num &a, uint32_t m, uint32_t c)
{
    uint64_t carry = c;
    for (size_t i = 0; i < a.size(); i++) {
        carry += (uint64_t)a[i] * m;
        a[i] = (uint32_t)carry;
        carry >>= 32;
    }
    if (carry) a.push_back((uint32_t)carry);
    trim(a);
}

// schoolbook product (column sums in 64-bit halves), small operands only
inline Num mul_school(const Num &a, const Num &b)
{
    if (a.empty() || b.empty()) return Num();
    Num r(a.size() + b.size(), 0);
    for (size_t i = 0; i < a.size(); i++) {
        uint64_t carry = 0;
        const uint64_t ai = a[i];
        for (size_t j = 0; j < b.size(); j++) {
            carry += ai * b[j] + r[i + j];
            r[i + j] = (uint32_t)carry;
            carry >>= 32;
        }
        size_t k = i + b.size();
        while (carry) {
            carry += r[k];
            r[k++] = (uint32_t)carry;
            carry >>= 32;
        }
    }
    trim(r);
    return r;
}

inline Num from_u64(uint64_t v)
{
    Num r;
    while (v) { r.push_back((uint32_t)v); v >>= 32; }
    return r;
}

// a / d for a 32-bit divisor, remainder returned
inline uint32_t divmod_small(Num &a, uint32_t d)
{
    uint64_t rem = 0;
    for (size_t i = a.size(); i-- > 0;) {
        const uint64_t cur = (rem << 32) | a[i];
        a[i] = (uint32_t)(cur / d);
        rem = cur % d;
    }
    trim(a);
    return (uint32_t)rem;
}

// floor(u / v) for v != 0: long division with a two-limb quotient estimate
// on the normalised divisor, corrected by at most one add-back per limb
// (Knuth, TAOCP vol. 2, 4.3.1, Algorithm D).
inline Num div_floor(const Num &u, const Num &v)
{
    if (cmp(u, v) < 0) return Num();
    if (v.size() == 1) {
        Num q = u;
        divmod_small(q, v[0]);
        return q;
    }
    const size_t n = v.size(), m = u.size() - n;
    const int s = __builtin_clz(v.back());
    Num vn = shl(v, s);
    Num un = shl(u, s);
    un.resize(u.size() + 1, 0);
    Num q(m + 1, 0);
    for (size_t j = m + 1; j-- > 0;) {
        const uint64_t num = ((uint64_t)un[j + n] << 32) | un[j + n - 1];
        uint64_t qh = num / vn[n - 1], rh = num % vn[n - 1];
        while ((qh >> 32) || qh * vn[n - 2] > ((rh << 32) | un[j + n - 2])) {
            qh--;
            rh += vn[n - 1];
            if (rh >> 32) break;
        }
        uint64_t k = 0;
        uint32_t br = 0;
        for (size_t i = 0; i < n; i++) {
            const uint64_t p = qh * vn[i] + k;
            k = p >> 32;
            const uint64_t t = (uint64_t)un[i + j] - (uint32_t)p - br;
            un[i + j] = (uint32_t)t;
            br = (t >> 32) ? 1u : 0u;
        }
        const uint64_t t = (uint64_t)un[j + n] - k - br;
        un[j + n] = (uint32_t)t;
        if (t >> 32) {   // qh was one too large: add v back
            qh--;
            uint64_t c = 0;
            for (size_t i = 0; i < n; i++) {
                c += (uint64_t)un[i + j] + vn[i];
                un[i + j] = (uint32_t)c;
                c >>= 32;
            }
            un[j + n] += (uint32_t)c;
        }
        q[j] = (uint32_t)qh;
    }
    trim(q);
    return q;
}

}  // namespace bn
}  // namespace gbntt
