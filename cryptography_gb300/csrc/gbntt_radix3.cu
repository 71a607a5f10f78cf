// gbntt_radix3.cu — the outer radix-3 stage of transforms of length
// N = 3 M, M = 2^k (both CRT primes have roots of order 3 2^30: 3 divides
// q0 - 1 and p3 - 1 = 3 2^30). A product whose coefficients fit 3 M but
// not 2^(k+1) runs as three M-point transforms of the existing pass chain
// between these two kernels, a quarter fewer points than the next power of
// two.
//
// Forward (decimation in frequency), for j < M, with x_r = x[j + r M] and
// w = w_N = g^((p-1)/N) (om = w^M a cube root of unity,
// c = (om - om^2) / 2):
//   s = x_1 + x_2, d = x_1 - x_2, t = x_0 - s / 2
//   y_0[j] = x_0 + s, y_1[j] = (t + c d) w^j, y_2[j] = (t - c d) w^(2j)
// (y_m[j] = w^(jm) sum_r x_r om^(rm), the coefficients of
// A(w^m X) mod (X^M - 1), A reduced mod X^M - om^m); each y_m then goes
// through the M-point pass chain (any primitive M-th root: it only has to
// give cyclic convolutions of length M), and the pointwise products pair
// them up.
// Inverse (decimation in time), in place, after the three M-point inverse
// transforms (which scale by 1/(3 M): the 1/3 rides on their scale):
//   t_0 = z_0[j], t_m = z_m[j] w^(-jm), s = t_1 + t_2, d = t_1 - t_2
//   x[j] = t_0 + s, x[j + M] = t_0 - s / 2 - c d, x[j + 2M] = t_0 - s / 2 + c d.
// Halving is a shift and a conditional add of (p + 1) / 2, not a multiply.
// A thread's first power of w comes from two-level tables of
// rho = g^((p-1)/(3 2^30)): w^j = rho^(j 2^(30-k)) = hi[e >> 15]
// lo[e & (2^15 - 1)], e < 3 2^30; its later ones by one multiply each.
// Residues stay in the pass chain's forms (plain values; constants and
// table entries in each field's multiply form).
#include <cuda_runtime.h>
#include <stdint.h>

#include "gbntt_arith.cuh"
#include "gbntt_internal.h"

namespace gbntt {

namespace {

constexpr long long kR3Order = 3LL << 30;   // order of rho

// x / 2 mod p for a residue x of the field's range: x >> 1, plus (p + 1) / 2
// when x is odd ((x - 1) / 2 + (p + 1) / 2 = (x + p) / 2, no overflow; a
// canonical x gives a canonical result, and lazy q0 values below 2^64 stay
// below 2^64).
template <int PI>
__device__ __forceinline__ typename Field<PI>::T r3_half(typename Field<PI>::T x)
{
    using V = typename Field<PI>::T;
    constexpr V kHalfUp = PI == 3 ? (V)((kP3 + 1u) / 2u) : (V)(0xFFFFFFFF00000001ull / 2 + 1);
    return (x >> 1) + ((x & 1) ? kHalfUp : (V)0);
}

template <int PI>
__device__ __forceinline__ typename Field<PI>::T r3_pow(const R3Args &a, long long e)
{
    using V = typename Field<PI>::T;
    const V *hi = (const V *)a.hi, *lo = (const V *)a.lo;
    return Field<PI>::mul(hi[e >> 15], lo[e & 32767]);
}

// Thread t of the grid takes j = t, t + G, t + 2 G, ... (G = blocks x 256:
// a warp's 32 consecutive j keep every load and store coalesced), kR3Unroll
// of them per loop step with all their loads issued first. Its twiddle w^j
// comes from the tables once and is then multiplied by w^G per j.
template <int PI>
__global__ void __launch_bounds__(256, 4) radix3_fwd_kernel(const R3Args a)
{
    using F = Field<PI>;
    using V = typename F::T;
    constexpr int U = kR3Unroll;
    const long long M = a.M, w = blockIdx.y;
    const long long G = (long long)gridDim.x * blockDim.x;
    const uint32_t *x = a.limb_tab ? a.limb_tab[w] : a.limbs;
    const long long n = a.len_tab ? a.len_tab[w] : a.n_limbs;
    V *out = (V *)a.spec + w * 3 * M;
    const V c = (V)a.c, step = (V)a.step;
    long long j = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (j >= M) return;
    V w1 = r3_pow<PI>(a, j << a.shift);
    for (; j < M; j += U * G) {
        uint32_t v[U][3];
#pragma unroll
        for (int u = 0; u < U; u++) {
            const long long jj = j + u * G;
#pragma unroll
            for (int r = 0; r < 3; r++) {
                const long long i = jj + r * M;
                v[u][r] = (jj < M && i < n) ? __ldcs(x + i) : 0u;
            }
        }
#pragma unroll
        for (int u = 0; u < U; u++) {
            const long long jj = j + u * G;
            if (jj < M) {
                const V x0 = F::from_u32(v[u][0]), x1 = F::from_u32(v[u][1]), x2 = F::from_u32(v[u][2]);
                const V s = F::add(x1, x2), d = F::sub(x1, x2);
                const V t = F::sub(x0, r3_half<PI>(s)), e = F::mul(d, c);
                const V w2 = F::mul(w1, w1);
                out[jj] = F::add(x0, s);
                out[M + jj] = F::mul(F::add(t, e), w1);
                out[2 * M + jj] = F::mul(F::sub(t, e), w2);
            }
            w1 = F::mul(w1, step);
        }
    }
}

template <int PI>
__global__ void __launch_bounds__(256, 4) radix3_inv_kernel(const R3Args a)
{
    using F = Field<PI>;
    using V = typename F::T;
    constexpr int U = kR3Unroll;
    const long long M = a.M, w = blockIdx.y;
    const long long G = (long long)gridDim.x * blockDim.x;
    V *z = (V *)a.spec + w * 3 * M;
    const V c = (V)a.c, step = (V)a.step;
    long long j = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (j >= M) return;
    const long long ex = j << a.shift;
    V w1 = r3_pow<PI>(a, ex ? kR3Order - ex : 0);   // w^(-j)
    for (; j < M; j += U * G) {
        V v[U][3];
#pragma unroll
        for (int u = 0; u < U; u++) {
            const long long jj = j + u * G;
#pragma unroll
            for (int r = 0; r < 3; r++) v[u][r] = jj < M ? z[jj + r * M] : F::zero();
        }
#pragma unroll
        for (int u = 0; u < U; u++) {
            const long long jj = j + u * G;
            if (jj < M) {
                const V w2 = F::mul(w1, w1);
                const V t1 = F::mul(v[u][1], w1), t2 = F::mul(v[u][2], w2);
                const V s = F::add(t1, t2), d = F::sub(t1, t2);
                const V t0 = v[u][0], q = F::sub(t0, r3_half<PI>(s)), e = F::mul(d, c);
                z[jj] = F::add(t0, s);
                z[M + jj] = F::sub(q, e);
                z[2 * M + jj] = F::add(q, e);
            }
            w1 = F::mul(w1, step);
        }
    }
}

template <int PI>
cudaError_t launch_r3(bool inverse, const R3Args &a, cudaStream_t st)
{
    const dim3 grid((unsigned)a.blocks, (unsigned)a.W);
    if (inverse) radix3_inv_kernel<PI><<<grid, 256, 0, st>>>(a);
    else radix3_fwd_kernel<PI><<<grid, 256, 0, st>>>(a);
    return cudaGetLastError();
}

}  // namespace

cudaError_t launch_radix3(int pi, bool inverse, const R3Args &a, cudaStream_t st)
{
    if (a.W < 1 || a.W > 65535 || a.blocks < 1 || a.blocks > 65535) return cudaErrorInvalidValue;
    switch (pi) {
    case 0: return launch_r3<0>(inverse, a, st);
    case 3: return launch_r3<3>(inverse, a, st);
    case 4: return launch_r3<4>(inverse, a, st);
    default: return cudaErrorInvalidValue;
    }
}

}  // namespace gbntt
