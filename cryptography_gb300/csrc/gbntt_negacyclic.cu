// gbntt_negacyclic.cu — negacyclic polynomial products, mod X^N + 1.
//
// The reference's crt_ntt benchmark multiplies polynomials modulo X^N + 1
// with a twist / cyclic NTT / pointwise product / inverse NTT / untwist
// pipeline per CRT prime followed by Garner (ntt/lib/main.hip:557-684,
// twist and untwist kernels). Here the cyclic part is the engine's own
// pass chain over the three 64-bit primes; this file holds the two
// elementwise kernels around it:
//   twist:  residue i of prime k = (f_i mod p_k) psi_k^i, psi_k a primitive
//           2N-th root of unity (psi^N = -1), written where the first
//           forward pass reads residues;
//   finish: multiplies the inverse transform's output by psi_k^-i (so the
//           cyclic convolution of the twisted sequences becomes the
//           negacyclic one), reconstructs the coefficient modulo
//           M = q0 q1 q2 (~2^192) by Garner, and writes it as a signed
//           256-bit two's complement integer (|c| < N 2^128 < M / 2).
#include <cuda_runtime.h>
#include <stdint.h>

#include "gbntt_arith.cuh"
#include "gbntt_internal.h"

namespace gbntt {

namespace {

// psi^i = w^(i << shift), w the primitive 2^30-th root of the tables
template <int PI>
__device__ __forceinline__ uint64_t nega_tw(const NegaArgs &a, long long i)
{
    const uint32_t e = (uint32_t)((unsigned long long)i << a.shift);
    return mont_mul<PI>(__ldg(a.hi[PI] + (e >> kTwBits)), __ldg(a.lo[PI] + (e & (kTwSize - 1))));
}

template <int PI>
__device__ __forceinline__ void twist_one(const NegaArgs &a, long long i, uint64_t v)
{
    constexpr uint64_t P = Prime<PI>::P;
    const uint64_t r = v >= P ? v - P : v;   // v < 2^64 < 2p
    a.spec[PI][i] = mont_mul<PI>(r, nega_tw<PI>(a, i));
}

__global__ void nega_twist_kernel(NegaArgs a)
{
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < a.n; i += stride) {
        const uint64_t v = __ldg(a.coef + i);
        twist_one<0>(a, i, v);
        twist_one<1>(a, i, v);
        twist_one<2>(a, i, v);
    }
}

// (w2 : w1 : w0) - (b2 : b1 : b0) over 256 bits (w3 = 0), in place
__device__ __forceinline__ void sub256(uint64_t &w0, uint64_t &w1, uint64_t &w2, uint64_t &w3, uint64_t b0,
                                       uint64_t b1, uint64_t b2)
{
    const uint64_t d0 = w0 - b0;
    const uint64_t c0 = w0 < b0;
    const uint64_t t1 = w1 - b1;
    const uint64_t c1 = (w1 < b1) + (t1 < c0);
    const uint64_t d1 = t1 - c0;
    const uint64_t t2 = w2 - b2;
    const uint64_t c2 = (w2 < b2) + (t2 < c1);
    const uint64_t d2 = t2 - c1;
    w0 = d0;
    w1 = d1;
    w2 = d2;
    w3 = 0 - c2;
}

__global__ void nega_finish_kernel(NegaArgs a)
{
    typedef unsigned __int128 u128;
    constexpr uint64_t q0 = Prime<0>::P, q1 = Prime<1>::P, q2 = Prime<2>::P;
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < a.n; i += stride) {
        // untwist: the residues of the negacyclic coefficient
        const uint64_t r0 = mont_mul<0>(a.spec[0][i], nega_tw<0>(a, i));
        const uint64_t r1 = mont_mul<1>(a.spec[1][i], nega_tw<1>(a, i));
        const uint64_t r2 = mont_mul<2>(a.spec[2][i], nega_tw<2>(a, i));
        // mixed-radix digits: c = a0 + q0 a1 + q0 q1 a2
        const uint64_t a0 = r0;
        const uint64_t a1 = mont_mul<1>(sub_mod<1>(r1, a0 >= q1 ? a0 - q1 : a0), a.garner[0]);
        uint64_t t = sub_mod<2>(r2, a0 >= q2 ? a0 - q2 : a0);
        t = sub_mod<2>(t, mont_mul<2>(a1, a.garner[1]));
        const uint64_t a2 = mont_mul<2>(t, a.garner[2]);
        // c in three 64-bit words: (a1 q0 + a0) + (q0 q1) a2
        const u128 lowp = (u128)a1 * q0 + a0;   // < q0 q1 < 2^128
        const u128 x = (u128)a.q01_lo * a2;
        const u128 y = (u128)a.q01_hi * a2;
        const u128 s = lowp + x;
        const uint64_t cs = s < lowp ? 1u : 0u;
        uint64_t w0 = (uint64_t)s;
        const uint64_t mid = (uint64_t)(s >> 64);
        uint64_t w1 = mid + (uint64_t)y;
        const uint64_t cm = w1 < mid ? 1u : 0u;
        uint64_t w2 = (uint64_t)(y >> 64) + cs + cm;
        uint64_t w3 = 0;
        // signed representative: c - M when c > (M - 1) / 2
        const bool neg = w2 != a.half[2] ? w2 > a.half[2] : (w1 != a.half[1] ? w1 > a.half[1] : w0 > a.half[0]);
        if (neg) sub256(w0, w1, w2, w3, a.m[0], a.m[1], a.m[2]);
        uint64_t *o = a.out + 4 * i;
        o[0] = w0;
        o[1] = w1;
        o[2] = w2;
        o[3] = w3;
    }
}

int grid_for(long long n)
{
    long long g = (n + 255) / 256;
    return (int)(g > 152 * 16 ? 152 * 16 : (g < 1 ? 1 : g));
}

}  // namespace

cudaError_t launch_nega_twist(const NegaArgs &a, cudaStream_t st)
{
    nega_twist_kernel<<<grid_for(a.n), 256, 0, st>>>(a);
    return cudaGetLastError();
}

cudaError_t launch_nega_finish(const NegaArgs &a, cudaStream_t st)
{
    nega_finish_kernel<<<grid_for(a.n), 256, 0, st>>>(a);
    return cudaGetLastError();
}

}  // namespace gbntt
