// gbntt_kernels.cu — sm_103a kernels of the CRT-NTT multiply.
//
// 1. The NTT pass kernels live in gbntt_pass.cuh (one translation unit per
//    prime). Fused into the passes: limb -> residue decomposition (first
//    forward pass reads 32-bit limbs; reference scatter kernel
//    ntt/lib/arith/ntt_mul.hip:117-160), the pointwise product (first
//    inverse pass; reference hadamard_kernel ntt/lib/ntt_kernel.hip:386-399
//    and stockham_kernel_had :739-780) and the N^-1 scale (last inverse pass).
// 2. garner_carry_kernel: CRT reconstruction of every coefficient from its
//    three residues, the limb sums w0(c_j) + w1(c_{j-1}) + w2(c_{j-2}), and
//    the carry propagation over all product limbs as one decoupled look-back
//    scan (bounded waits). Replaces garner_kernel (ntt/lib/garner.hip:
//    187-260) plus the host carry sweep bigint_gather
//    (ntt/lib/arith/bigint.c:333-397); the carry monoid follows the CLA
//    cells of ntt/lib/transfer_core.h:165-251, generalised to carries in
//    {0, 1, 2}.
#include "gbntt_arith.cuh"
#include "gbntt_carry.cuh"
#include "gbntt_internal.h"

namespace gbntt {

// ---------------------------------------------------------------------------
// Element-wise modular operations over device arrays (self-test of the
// arithmetic, as the reference's test_modops.hip pins primes.h / shoup.h).
// op: 0 add_mod, 1 sub_mod, 2 mont_mul, 3..5 the plain C++ forms;
// q0 only: 6 a * 2^(b mod 96) through gl_mul_pow2 (the register DFTs'
// power-of-two twiddles; here with the exponent known only at run time).
// ---------------------------------------------------------------------------
template <int PI>
__device__ __forceinline__ uint64_t modop(int op, uint64_t a, uint64_t b)
{
    switch (op) {
    case 0: return add_mod<PI>(a, b);
    case 1: return sub_mod<PI>(a, b);
    case 2: return mont_mul<PI>(a, b);
    case 3: return add_mod_ref<PI>(a, b);
    case 4: return sub_mod_ref<PI>(a, b);
    default: return mont_mul_ref<PI>(a, b);
    }
}

__global__ void modops_kernel(int prime, int op, const uint64_t *a, const uint64_t *b, uint64_t *out, long long n)
{
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const uint64_t x = a[i], y = b[i];
    if (prime == 4) {   // lazy normal-form q0 (operands any 64-bit words)
        uint64_t r;
        switch (op) {
        case 0: r = gl_add(x, y); break;
        case 1: r = gl_sub(x, y); break;
        case 2: r = gl_mul(x, y); break;
        case 3: r = gl_add_ref(x, y); break;
        case 4: r = gl_sub_ref(x, y); break;
        default: r = gl_mul_ref(x, y); break;
        }
        out[i] = r;
        return;
    }
    if (prime == 3) {   // the 32-bit prime (operands in the low words)
        const uint32_t u = (uint32_t)x, v = (uint32_t)y;
        uint32_t r;
        switch (op) {
        case 0: r = p3_add(u, v); break;
        case 1: r = p3_sub(u, v); break;
        case 2: r = p3_mul(u, v); break;
        case 3: r = p3_add_ref(u, v); break;
        case 4: r = p3_sub_ref(u, v); break;
        default: r = p3_mul_ref(u, v); break;
        }
        out[i] = r;
        return;
    }
    if (prime == 0 && op == 6) {
        out[i] = gl_mul_pow2(x, (int)(y % 96));
        return;
    }
    out[i] = prime == 0 ? modop<0>(op, x, y) : (prime == 1 ? modop<1>(op, x, y) : modop<2>(op, x, y));
}

cudaError_t launch_modops(int prime, int op, const uint64_t *a, const uint64_t *b, uint64_t *out, long long n,
                          cudaStream_t stream)
{
    if (n <= 0) return cudaSuccess;
    const long long grid = (n + 255) / 256;
    modops_kernel<<<(unsigned)grid, 256, 0, stream>>>(prime, op, a, b, out, n);
    return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// Garner + carry
// ---------------------------------------------------------------------------
// ---------------------------------------------------------------------------
// Seeded synthetic operands on the device: limb i is the low 32 bits of
// splitmix64 at seed + (i + 1) * 0x9E3779B97F4A7C15, the top limb gets bit 31
// (the same limbs as cryptography_gb300/synth.py produces on the host).
// ---------------------------------------------------------------------------
__global__ void fill_splitmix_kernel(uint32_t *d, long long n, uint64_t seed)
{
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
        uint64_t z = seed + (uint64_t)(i + 1) * 0x9E3779B97F4A7C15ull;
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
        z ^= z >> 31;
        uint32_t v = (uint32_t)z;
        if (i == n - 1) v |= 0x80000000u;
        d[i] = v;
    }
}

// Copy n 32-bit words from (mapped pinned) host memory to device memory in
// 16-byte words where both addresses allow it: one coalesced sweep over
// NVLink-C2C, driven by the SMs instead of a copy engine.
__global__ void copy_words_kernel(uint32_t *__restrict__ dst, const uint32_t *__restrict__ src, long long n)
{
    const long long stride = (long long)gridDim.x * blockDim.x;
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if ((((uintptr_t)dst | (uintptr_t)src) & 15) == 0) {
        const long long n4 = n >> 2;
        const uint4 *s4 = reinterpret_cast<const uint4 *>(src);
        uint4 *d4 = reinterpret_cast<uint4 *>(dst);
        for (long long i = t; i < n4; i += stride) d4[i] = s4[i];
        for (long long i = (n4 << 2) + t; i < n; i += stride) dst[i] = src[i];
    } else {
        for (long long i = t; i < n; i += stride) dst[i] = src[i];
    }
}

cudaError_t launch_copy_words(uint32_t *dst, const uint32_t *src, long long n, int grid, cudaStream_t st)
{
    if (n <= 0) return cudaSuccess;
    copy_words_kernel<<<grid, 512, 0, st>>>(dst, src, n);
    return cudaGetLastError();
}

cudaError_t launch_fill_splitmix(uint32_t *d, long long n, uint64_t seed, cudaStream_t st)
{
    if (n <= 0) return cudaSuccess;
    long long grid = (n + 255) / 256;
    if (grid > 152 * 64) grid = 152 * 64;
    fill_splitmix_kernel<<<(unsigned)grid, 256, 0, st>>>(d, n, seed);
    return cudaGetLastError();
}

constexpr int kCarryThreads = 256;
constexpr int kCarryPerThread = 8;
constexpr int kCarryTile = kCarryThreads * kCarryPerThread;   // limbs per tile

long long carry_tiles(long long n_out) { return (n_out + kCarryTile - 1) / kCarryTile; }

// c_j from its residues (mixed radix, Garner): returns the three 32-bit words
// of c_j < 2^96 and flags a nonzero third digit (c_j >= q0*q1 means the
// residues are corrupted: a true coefficient is below 2^93).
__device__ __forceinline__ void garner_coef(const CarryArgs &a, long long j, uint32_t &w0, uint32_t &w1,
                                            uint32_t &w2, unsigned &err)
{
    if (j < 0 || j >= a.n_coef) { w0 = w1 = w2 = 0; return; }
    constexpr uint64_t q0 = Prime<0>::P, q1 = Prime<1>::P, q2 = Prime<2>::P;
    const uint64_t r0 = a.res[0][j], r1 = a.res[1][j], r2 = a.res[2][j];
    const uint64_t a0 = r0;
    const uint64_t a0_1 = a0 >= q1 ? a0 - q1 : a0;
    const uint64_t a1 = mont_mul<1>(sub_mod<1>(r1, a0_1), a.garner[0]);
    const uint64_t a0_2 = a0 >= q2 ? a0 - q2 : a0;
    uint64_t t = sub_mod<2>(r2, a0_2);
    t = sub_mod<2>(t, mont_mul<2>(a1, a.garner[1]));
    const uint64_t a2 = mont_mul<2>(t, a.garner[2]);
    uint64_t lo = a1 * q0;
    uint64_t hi = __umul64hi(a1, q0);
    lo += a0;
    hi += (lo < a0);
    if (a2 != 0 || (hi >> 32) != 0) err |= ERR_GARNER_DIGIT;
    w0 = (uint32_t)lo;
    w1 = (uint32_t)(lo >> 32);
    w2 = (uint32_t)hi;
}

typedef unsigned __int128 u128;

// Two-prime form (lazy q0 and the 32-bit p3): c_j = r0 + q0 a1 with
// a1 = (r1 - r0) q0^-1 mod p3, c_j < q0 p3 < 2^96. garner[0] = q0^-1 mod p3
// and garner[1] = 2^64 mod p3, both as p3 Montgomery multipliers. A true
// coefficient is below N 2^64 (N = the transform length, above the shorter
// operand's limb count): a larger top word means corrupted residues.
__device__ __forceinline__ void garner_coef2(const CarryArgs &a, long long j, uint32_t &w0, uint32_t &w1,
                                             uint32_t &w2, unsigned &err)
{
    if (j < 0 || j >= a.n_coef) { w0 = w1 = w2 = 0; return; }
    constexpr uint64_t q0 = Prime<0>::P;
    const uint64_t r0 = gl_canon(a.res[0][j]);   // lazy residues reach [0, 2^64)
    const uint32_t r1 = ((const uint32_t *)a.res[1])[j];
    const uint32_t lo = (uint32_t)r0;
    const uint32_t r0m = p3_add(p3_mul((uint32_t)(r0 >> 32), (uint32_t)a.garner[1]), lo >= kP3 ? lo - kP3 : lo);
    const uint32_t a1 = p3_mul(p3_sub(r1, r0m), (uint32_t)a.garner[0]);
    const u128 c = (u128)a1 * q0 + r0;
    w0 = (uint32_t)c;
    w1 = (uint32_t)(c >> 32);
    const uint64_t top = (uint64_t)(c >> 64);
    w2 = (uint32_t)top;
    if (top >= (uint64_t)a.n_coef) err |= ERR_GARNER_DIGIT;
}

// The two-prime Garner step on residues already loaded (r0 of q0, r1 of p3;
// (0, 0) gives 0). c = r0 + a1 q0 = r0 + a1 + a1 2^64 - a1 2^32 through add
// and borrow chains instead of a 128-bit multiply.
__device__ __forceinline__ void garner2_vals(const CarryArgs &a, uint64_t r0, uint32_t r1, uint32_t &w0,
                                             uint32_t &w1, uint32_t &w2, unsigned &err)
{
    r0 = gl_canon(r0);   // lazy residues reach [0, 2^64)
    const uint32_t lo = (uint32_t)r0;
    const uint32_t r0m = p3_add(p3_mul((uint32_t)(r0 >> 32), (uint32_t)a.garner[1]), lo >= kP3 ? lo - kP3 : lo);
    const uint32_t a1 = p3_mul(p3_sub(r1, r0m), (uint32_t)a.garner[0]);
    const uint64_t x = r0 + (uint64_t)a1;
    const uint32_t ca = x < r0 ? 1u : 0u;
    const uint64_t sh = (uint64_t)a1 << 32;
    const uint64_t y = x - sh;
    const uint32_t bb = x < sh ? 1u : 0u;
    const uint32_t top = a1 + ca - bb;
    w0 = (uint32_t)y;
    w1 = (uint32_t)(y >> 32);
    w2 = top;
    if ((long long)top >= a.n_coef) err |= ERR_GARNER_DIGIT;
}

template <bool MIXED>
__device__ __forceinline__ void garner_any(const CarryArgs &a, long long j, uint32_t &w0, uint32_t &w1, uint32_t &w2,
                                           unsigned &err)
{
    if (MIXED) garner_coef2(a, j, w0, w1, w2, err);
    else garner_coef(a, j, w0, w1, w2, err);
}

#ifndef GBNTT_CARRY_MIN_BLOCKS
#define GBNTT_CARRY_MIN_BLOCKS 6   // resident carry CTAs per SM the register budget targets (2^29: 5 -> 2.39 ms, 6 -> 2.21, 8 -> 2.34)
#endif
template <bool BATCH, bool MIXED>
__global__ void __launch_bounds__(kCarryThreads, GBNTT_CARRY_MIN_BLOCKS) garner_carry_kernel_t(CarryArgs a)
{
    constexpr int T = kCarryThreads, K = kCarryPerThread, TILE = kCarryTile;
    constexpr int SW = TILE + 2 + (TILE + 2) / 32 + 1;
    __shared__ uint32_t W0[SW], W1[SW], W2[SW];
    __shared__ unsigned s_warp[T / 32];
    __shared__ unsigned s_tile, s_cin;
    __shared__ long long s_prod;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    if (tid == 0) {
        s_tile = atomicAdd(a.ticket, 1u);
        if (BATCH) {
            // product owning this global tile (binary search of tile_start)
            long long lo = 0, hi = a.nprod;   // tile_start[lo] <= t < tile_start[hi]
            const long long t = s_tile;
            while (hi - lo > 1) {
                const long long mid = (lo + hi) >> 1;
                if (a.tile_start[mid] <= t) lo = mid; else hi = mid;
            }
            s_prod = t < a.tile_start[a.nprod] ? lo : -1;
        }
    }
    __syncthreads();
    if (BATCH) {
        // tickets beyond the batch's tiles (the grid is an upper bound) exit
        if (s_prod < 0) return;
        const long long b = s_prod;
        const long long n_prod = (a.radix3 ? 3LL : 1LL) << a.log_n_prod;
        const long long off = b * n_prod;
        if (MIXED) {
            a.res[0] += off;
            a.res[1] = (const uint64_t *)((const uint32_t *)a.res[1] + off);
        } else {
            for (int pi = 0; pi < 3; pi++) a.res[pi] += off;
        }
        a.out = a.out_tab[b];
        a.n_out = a.nout_tab[b];
        a.n_coef = n_prod;
        a.status += a.tile_start[b];
    }
    const long long tile = BATCH ? (long long)s_tile - a.tile_start[s_prod] : (long long)s_tile;
    const long long base = tile * TILE;
    unsigned err = 0;

    // phase 1: coefficients of positions base-2 .. base+TILE-1 (slot q+2)
    if constexpr (MIXED) {
        // all of this thread's residue loads first (beyond the transform:
        // zero), then the arithmetic
        const uint64_t *res0 = a.res[0];
        const uint32_t *res1 = (const uint32_t *)a.res[1];
        uint64_t v0[K];
        uint32_t v1[K];
#pragma unroll
        for (int r = 0; r < K; r++) {
            const long long j = base + r * T + tid;
            const bool in = j < a.n_coef;
            v0[r] = in ? __ldcs(res0 + j) : 0ull;
            v1[r] = in ? __ldcs(res1 + j) : 0u;
        }
#pragma unroll
        for (int r = 0; r < K; r++) {
            const int q = r * T + tid;
            uint32_t w0, w1, w2;
            garner2_vals(a, v0[r], v1[r], w0, w1, w2, err);
            W0[spad(q + 2)] = w0; W1[spad(q + 2)] = w1; W2[spad(q + 2)] = w2;
        }
    } else {
#pragma unroll
        for (int r = 0; r < K; r++) {
            const int q = r * T + tid;
            uint32_t w0, w1, w2;
            garner_any<MIXED>(a, base + q, w0, w1, w2, err);
            W0[spad(q + 2)] = w0; W1[spad(q + 2)] = w1; W2[spad(q + 2)] = w2;
        }
    }
    if (tid < 2) {
        uint32_t w0, w1, w2;
        garner_any<MIXED>(a, base - 2 + tid, w0, w1, w2, err);
        W0[spad(tid)] = w0; W1[spad(tid)] = w1; W2[spad(tid)] = w2;
    }
    __syncthreads();

    // phase 2: limb sums of this thread's K consecutive limbs, carry-in 0
    const int q0 = tid * K;
    uint64_t s[K];
#pragma unroll
    for (int k = 0; k < K; k++) {
        const int q = q0 + k;
        s[k] = (uint64_t)W0[spad(q + 2)] + W1[spad(q + 1)] + W2[spad(q)];
    }
    unsigned fn;
    {
        uint64_t c = 0;
        bool all_max = true, rest_max = true, low_ge = false;
#pragma unroll
        for (int k = 0; k < K; k++) {
            const uint64_t v = s[k] + c;
            const uint32_t limb = (uint32_t)v;
            c = v >> 32;
            if (limb != 0xFFFFFFFFu) all_max = false;
            if (k == 0) low_ge = limb >= 0xFFFFFFFEu;
            else if (limb != 0xFFFFFFFFu) rest_max = false;
        }
        const unsigned f0 = (unsigned)c;
        const unsigned f1 = f0 + (all_max ? 1u : 0u);
        const unsigned f2 = f0 + ((rest_max && low_ge) ? 1u : 0u);
        fn = f0 | (f1 << 2) | (f2 << 4);
    }

    // phase 3: block scan of transfer functions (thread order = limb order)
    unsigned inc = fn;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        const unsigned o = __shfl_up_sync(0xFFFFFFFFu, inc, d);
        if (lane >= d) inc = fn_compose(inc, o);
    }
    if (lane == 31) s_warp[warp] = inc;
    __syncthreads();
    unsigned warp_prefix = kFnIdentity, block_agg = kFnIdentity;
#pragma unroll
    for (int w = 0; w < T / 32; w++) {
        if (w == warp) warp_prefix = block_agg;
        block_agg = fn_compose(s_warp[w], block_agg);
    }
    unsigned lane_excl = __shfl_up_sync(0xFFFFFFFFu, inc, 1);
    if (lane == 0) lane_excl = kFnIdentity;
    const unsigned thread_prefix = fn_compose(lane_excl, warp_prefix);

    // phase 4: decoupled look-back for this tile's carry-in (bounded waits)
    if (tid == 0) s_cin = lookback_carry(a.status, tile, block_agg, err);
    __syncthreads();

    // phase 5: final limbs with this thread's carry-in, coalesced store
    uint64_t c = fn_apply(thread_prefix, s_cin);
    uint32_t *out_s = W0;   // W0 is dead after phase 2
#pragma unroll
    for (int k = 0; k < K; k++) {
        const uint64_t v = s[k] + c;
        c = v >> 32;
        out_s[spad(q0 + k)] = (uint32_t)v;
    }
    __syncthreads();
#pragma unroll
    for (int r = 0; r < K; r++) {
        const int q = r * T + tid;
        const long long pos = base + q;
        if (pos < a.n_out) a.out[pos] = out_s[spad(q)];
    }
    if (err) atomicOr(a.error, err);
}

// ---------------------------------------------------------------------------
// Garner + carry for 64-bit coefficients (packed mode): one 64-bit limb per
// coefficient, as the reference engine does (ntt/lib/arith/bigint.h:30-43).
// A coefficient is below n * 2^128 < 2^158 and needs all three mixed-radix
// digits: c = a0 + a1 q0 + a2 q0 q1 < 2^192, three 64-bit words w0..w2.
// Product limb j = w0(c_j) + w1(c_{j-1}) + w2(c_{j-2}) + carry; the carry
// into a limb is again 0, 1 or 2, so the scan monoid is the one above.
// ---------------------------------------------------------------------------
constexpr int kCarry64Threads = 256;
constexpr int kCarry64PerThread = 4;
constexpr int kCarry64Tile = kCarry64Threads * kCarry64PerThread;

long long carry_tiles64(long long n_out) { return (n_out + kCarry64Tile - 1) / kCarry64Tile; }

__device__ __forceinline__ void garner_coef64(const CarryArgs &a, long long j, uint64_t &w0, uint64_t &w1,
                                              uint64_t &w2, unsigned &err)
{
    if (j < 0 || j >= a.n_coef) { w0 = w1 = w2 = 0; return; }
    constexpr uint64_t q0 = Prime<0>::P, q1 = Prime<1>::P, q2 = Prime<2>::P;
    const uint64_t r0 = a.res[0][j], r1 = a.res[1][j], r2 = a.res[2][j];
    const uint64_t a0 = r0;
    const uint64_t a0_1 = a0 >= q1 ? a0 - q1 : a0;
    const uint64_t a1 = mont_mul<1>(sub_mod<1>(r1, a0_1), a.garner[0]);
    const uint64_t a0_2 = a0 >= q2 ? a0 - q2 : a0;
    uint64_t t = sub_mod<2>(r2, a0_2);
    t = sub_mod<2>(t, mont_mul<2>(a1, a.garner[1]));
    const uint64_t a2 = mont_mul<2>(t, a.garner[2]);
    // c = a0 + a1 q0 + a2 (q0 q1)
    u128 lo = (u128)a1 * q0 + a0;                     // < 2^128
    const u128 x = (u128)a2 * a.q01_lo;
    const u128 y = (u128)a2 * a.q01_hi;
    u128 s0 = (u128)(uint64_t)lo + (uint64_t)x;
    w0 = (uint64_t)s0;
    u128 s1 = (s0 >> 64) + (uint64_t)(lo >> 64) + (uint64_t)(x >> 64) + (uint64_t)y;
    w1 = (uint64_t)s1;
    w2 = (uint64_t)(s1 >> 64) + (uint64_t)(y >> 64);
    // a true coefficient is below 2^158: a larger top word means corrupted residues
    if ((w2 >> 31) != 0) err |= ERR_GARNER_DIGIT;
}

__global__ void __launch_bounds__(kCarry64Threads) garner_carry64_kernel(CarryArgs a)
{
    constexpr int T = kCarry64Threads, K = kCarry64PerThread, TILE = kCarry64Tile;
    constexpr int SW = TILE + 2 + (TILE + 2) / 32 + 1;
    __shared__ uint64_t W0[SW], W1[SW], W2[SW];
    __shared__ unsigned s_warp[T / 32];
    __shared__ unsigned s_tile, s_cin;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    if (tid == 0) s_tile = atomicAdd(a.ticket, 1u);
    __syncthreads();
    const long long tile = s_tile;
    const long long base = tile * TILE;
    unsigned err = 0;

#pragma unroll
    for (int r = 0; r < K; r++) {
        const int q = r * T + tid;
        uint64_t w0, w1, w2;
        garner_coef64(a, base + q, w0, w1, w2, err);
        W0[spad(q + 2)] = w0; W1[spad(q + 2)] = w1; W2[spad(q + 2)] = w2;
    }
    if (tid < 2) {
        uint64_t w0, w1, w2;
        garner_coef64(a, base - 2 + tid, w0, w1, w2, err);
        W0[spad(tid)] = w0; W1[spad(tid)] = w1; W2[spad(tid)] = w2;
    }
    __syncthreads();

    const int q0 = tid * K;
    u128 s[K];
#pragma unroll
    for (int k = 0; k < K; k++) {
        const int q = q0 + k;
        s[k] = (u128)W0[spad(q + 2)] + W1[spad(q + 1)] + W2[spad(q)];
    }
    unsigned fn;
    {
        u128 c = 0;
        bool all_max = true, rest_max = true, low_ge = false;
#pragma unroll
        for (int k = 0; k < K; k++) {
            const u128 v = s[k] + c;
            const uint64_t limb = (uint64_t)v;
            c = v >> 64;
            if (limb != ~0ull) all_max = false;
            if (k == 0) low_ge = limb >= ~0ull - 1;
            else if (limb != ~0ull) rest_max = false;
        }
        const unsigned f0 = (unsigned)c;
        const unsigned f1 = f0 + (all_max ? 1u : 0u);
        const unsigned f2 = f0 + ((rest_max && low_ge) ? 1u : 0u);
        fn = f0 | (f1 << 2) | (f2 << 4);
    }

    unsigned inc = fn;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        const unsigned o = __shfl_up_sync(0xFFFFFFFFu, inc, d);
        if (lane >= d) inc = fn_compose(inc, o);
    }
    if (lane == 31) s_warp[warp] = inc;
    __syncthreads();
    unsigned warp_prefix = kFnIdentity, block_agg = kFnIdentity;
#pragma unroll
    for (int w = 0; w < T / 32; w++) {
        if (w == warp) warp_prefix = block_agg;
        block_agg = fn_compose(s_warp[w], block_agg);
    }
    unsigned lane_excl = __shfl_up_sync(0xFFFFFFFFu, inc, 1);
    if (lane == 0) lane_excl = kFnIdentity;
    const unsigned thread_prefix = fn_compose(lane_excl, warp_prefix);

    if (tid == 0) s_cin = lookback_carry(a.status, tile, block_agg, err);
    __syncthreads();

    u128 c = fn_apply(thread_prefix, s_cin);
    uint64_t *out_s = W0;
#pragma unroll
    for (int k = 0; k < K; k++) {
        const u128 v = s[k] + c;
        c = v >> 64;
        out_s[spad(q0 + k)] = (uint64_t)v;
    }
    __syncthreads();
#pragma unroll
    for (int r = 0; r < K; r++) {
        const int q = r * T + tid;
        const long long pos = base + q;
        if (pos < a.n_out) a.out64[pos] = out_s[spad(q)];
    }
    if (err) atomicOr(a.error, err);
}

cudaError_t launch_garner_carry64(const CarryArgs &args, cudaStream_t stream, long long *ntiles_out)
{
    const long long nt = carry_tiles64(args.n_out);
    if (ntiles_out) *ntiles_out = nt;
    if (nt == 0) return cudaSuccess;
    garner_carry64_kernel<<<(unsigned)nt, kCarry64Threads, 0, stream>>>(args);
    return cudaGetLastError();
}

// the carry kernels' tiles live in shared memory: ask for the largest
// shared-memory carveout so that shared memory does not cap their residency
static void carry_carveout()
{
    static bool done = false;
    if (done) return;
    done = true;
    cudaFuncSetAttribute(garner_carry_kernel_t<false, true>, cudaFuncAttributePreferredSharedMemoryCarveout, 100);
    cudaFuncSetAttribute(garner_carry_kernel_t<false, false>, cudaFuncAttributePreferredSharedMemoryCarveout, 100);
    cudaFuncSetAttribute(garner_carry_kernel_t<true, true>, cudaFuncAttributePreferredSharedMemoryCarveout, 100);
    cudaFuncSetAttribute(garner_carry_kernel_t<true, false>, cudaFuncAttributePreferredSharedMemoryCarveout, 100);
    (void)cudaGetLastError();
}

cudaError_t launch_garner_carry(const CarryArgs &args, cudaStream_t stream, long long *ntiles_out)
{
    carry_carveout();
    const long long nt = carry_tiles(args.n_out);
    if (ntiles_out) *ntiles_out = nt;
    if (nt == 0) return cudaSuccess;
    if (args.mixed) garner_carry_kernel_t<false, true><<<(unsigned)nt, kCarryThreads, 0, stream>>>(args);
    else garner_carry_kernel_t<false, false><<<(unsigned)nt, kCarryThreads, 0, stream>>>(args);
    return cudaGetLastError();
}

cudaError_t launch_garner_carry_batch(const CarryArgs &args, long long grid_tiles, cudaStream_t stream)
{
    carry_carveout();
    if (grid_tiles <= 0) return cudaSuccess;
    if (args.mixed) garner_carry_kernel_t<true, true><<<(unsigned)grid_tiles, kCarryThreads, 0, stream>>>(args);
    else garner_carry_kernel_t<true, false><<<(unsigned)grid_tiles, kCarryThreads, 0, stream>>>(args);
    return cudaGetLastError();
}

}  // namespace gbntt
