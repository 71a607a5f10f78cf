// gbntt_pass.cuh — one NTT pass of 2^l points (l = 5..10) for one prime.
//
// The transform of N = 2^L points is a chain of 1-4 passes (outermost
// first). Pass i owns sub-problems of M_i points; inside each, element
// (j, m) sits at j + S_i m (column j < S_i, row m < 2^l, S_i = M_i / 2^l).
// A forward (decimation-in-frequency) pass computes, for every column, the
// 2^l-point DFT over m, multiplies output k by w_M^(j k) and stores it at
// j + S_i k; the next pass then works on the contiguous blocks of S_i points.
// The inverse pass is the exact transpose: input k of column j is first
// multiplied by w_M^-(j k), then the inverse 2^l-point DFT is stored back in
// natural order. Spectra therefore come out digit-reversed by pass and go
// back to natural order, with no transposes. The reference reaches the same
// structure with explicit transposes (Bailey four-step,
// ntt/lib/ntt_kernel.hip:835-925, :1172-1375).
//
// The kernels are generic over the prime's field policy (Field<PI> in
// gbntt_arith.cuh): 64-bit Montgomery residues for q0..q2, 32-bit residues
// for p3. Argument arrays are indexed by the policy's slot.
//
// Inside a CTA (128 threads, G columns): the 2^l-point DFT is A x B with
// A = 2^ceil(l/2), B = 2^floor(l/2): step 1 runs one A-point register DFT
// per (column, b), multiplies by w_L^(b k_a), step 2 runs A/B B-point
// register DFTs per thread. Shared memory holds the G x 2^l tile with an odd
// row stride and one pad word per B words, so both steps are free of bank
// conflicts. Two address layouts:
//   STRIDED (S >= G): the CTA's G columns are adjacent in every row, so each
//     thread walks one column with a constant pointer increment;
//   CONTIG (S == 1): the CTA's columns are G consecutive rows of 2^l words.
#pragma once
#include <algorithm>
#include "gbntt_arith.cuh"
#include "gbntt_internal.h"

namespace gbntt {

enum PassLayout { LAYOUT_STRIDED = 0, LAYOUT_CONTIG = 1 };

#ifndef GBNTT_PASS_MIN_BLOCKS
#define GBNTT_PASS_MIN_BLOCKS 5   // resident CTAs per SM the register budget targets, 2^9/2^10-point passes (measured best of 3..6)
#endif
#ifndef GBNTT_PASS_MIN_BLOCKS_SMALL
#define GBNTT_PASS_MIN_BLOCKS_SMALL 7   // the same for passes of up to 2^8 points (2^29: 5 -> 59.9 ms, 7 -> 59.4 ms)
#endif
#ifndef GBNTT_PASS_MIN_BLOCKS32
#define GBNTT_PASS_MIN_BLOCKS32 8  // the same for the 32-bit prime (measured 5..10 at 2^29: 8 within 1%, no spills of note)
#endif
template <int PI, int LOG_L>
struct PassMinBlocks {
    static constexpr int value = sizeof(typename Field<PI>::T) == 4
                                     ? GBNTT_PASS_MIN_BLOCKS32
                                     : (LOG_L <= 8 ? GBNTT_PASS_MIN_BLOCKS_SMALL : GBNTT_PASS_MIN_BLOCKS);
};
constexpr int kPassThreads = 128;
constexpr int kLogPassThreads = 7;

template <int LOG_L, int WORD = 8>
struct PassShape {
    static constexpr int L = 1 << LOG_L;
    static constexpr int LOG_A = (LOG_L + 1) / 2, LOG_B = LOG_L / 2;
    static constexpr int A = 1 << LOG_A, B = 1 << LOG_B;
    static constexpr int T = kPassThreads;
    static constexpr int LOG_G = kLogPassThreads - LOG_B;
    static constexpr int G = 1 << LOG_G;          // columns per CTA
    // row stride in words: odd for 8-byte words; for 4-byte words the pad
    // that minimises bank conflicts over the load/store and both DFT steps
    // (searched exhaustively per l; conflict-free at l = 10)
    static constexpr int PAD4 = LOG_L == 5 ? 5 : LOG_L == 6 ? 2 : LOG_L == 7 ? 6 : LOG_L == 10 ? 8 : 4;
    static constexpr int RS = L + A + (WORD == 4 ? PAD4 : 1);
    static constexpr size_t SMEM = (size_t)G * RS * WORD;
};

__host__ __device__ constexpr int bitrev(int x, int bits)
{
    int r = 0;
    for (int i = 0; i < bits; i++) r = (r << 1) | ((x >> i) & 1);
    return r;
}

// w^E from the two-level tables (Montgomery form), E < 2^30.
template <int PI>
__device__ __forceinline__ typename Field<PI>::T tw_exp(const typename Field<PI>::T *hi,
                                                        const typename Field<PI>::T *lo, uint32_t e)
{
    return Field<PI>::mul(__ldg(hi + (e >> kTwBits)), __ldg(lo + (e & (kTwSize - 1))));
}

// In-register radix-2 DIF DFT of 2^LOG_R points: natural order in,
// bit-reversed order out (X[k] ends in x[bitrev(k)]). w64 = Montgomery forms
// of the primitive 64th root's powers.
template <int PI, int LOG_R, int DIR>
__device__ __forceinline__ void dft_reg(typename Field<PI>::T (&x)[1 << LOG_R], const uint64_t *w64)
{
    using F = Field<PI>;
    using T = typename F::T;
    constexpr int R = 1 << LOG_R;
#pragma unroll
    for (int s = R / 2; s >= 1; s >>= 1) {
#pragma unroll
        for (int blk = 0; blk < R; blk += 2 * s) {
#pragma unroll
            for (int i = 0; i < s; i++) {
                const T u = x[blk + i], v = x[blk + i + s];
                x[blk + i] = F::add(u, v);
                // w_{2s}^i = w_64^(i * 32 / s)
                const int k = i * (32 / s);
                if constexpr (PI == 0) {
                    // q0's w_64 is 2^39 (inverse: 2^-39 = 2^153); 2^96 == -1,
                    // so a power 2^e with e >= 96 is -2^(e-96): swap u and v
                    const int e = (DIR == 0 ? 39 * k : 153 * k) % 192;
                    if (k == 0) x[blk + i + s] = F::sub(u, v);
                    else if (e < 96) x[blk + i + s] = gl_mul_pow2(F::sub(u, v), e);
                    else x[blk + i + s] = gl_mul_pow2(F::sub(v, u), e - 96);
                } else {
                    const T d = F::sub(u, v);
                    x[blk + i + s] = (k == 0) ? d : F::mul(d, (T)w64[k]);
                }
            }
        }
    }
}

// Residue of a 64-bit limb (zero beyond n_limbs): limb < 2^64 < 2p, so one
// conditional subtract reduces it (the reference reduces with a 128-bit %,
// ntt/lib/arith/bigint.c:286-294).
template <int PI>
__device__ __forceinline__ uint64_t limb64_residue(const PassArgs &a, long long addr)
{
    uint64_t v = addr < a.n_limbs ? __ldg(a.limbs64 + addr) : 0ull;
    return v >= Field<PI>::P ? v - Field<PI>::P : v;
}

// 32-bit limb of coefficient `addr` (zero beyond the operand): one flat
// operand, or, in a batch, the operand of product addr >> log_n_prod.
__device__ __forceinline__ uint64_t limb32_at(const PassArgs &a, long long addr)
{
    if (a.limb_tab) {
        const long long b = addr >> a.log_n_prod;
        const long long local = addr & ((1LL << a.log_n_prod) - 1);
        return local < __ldg(a.len_tab + b) ? (uint64_t)__ldg(a.limb_tab[b] + local) : 0ull;
    }
    return addr < a.n_limbs ? (uint64_t)__ldg(a.limbs + addr) : 0ull;
}

#ifndef GBNTT_PASS_SHARED_DFT
#define GBNTT_PASS_SHARED_DFT 1   // even l: one loop body for both DFT steps
#endif
#ifndef GBNTT_PASS_CPASYNC
#define GBNTT_PASS_CPASYNC 1   // plain residue loads go global -> shared through cp.async
#endif
#ifndef GBNTT_PASS_PW_ASYNC
#define GBNTT_PASS_PW_ASYNC 1  // pointwise pass: one spectrum through cp.async, the other in registers (2^29: 8.8 -> 8.1 ms)
#endif

// asynchronous global -> shared copy of one residue word (no register
// staging, so every load of a thread can be in flight at once)
template <int BYTES>
__device__ __forceinline__ void cp_async_word(void *smem, const void *gmem)
{
    const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
    asm volatile("cp.async.ca.shared.global [%0], [%1], %2;\n" ::"r"(s), "l"(gmem), "n"(BYTES) : "memory");
}
__device__ __forceinline__ void cp_async_wait_all()
{
    asm volatile("cp.async.commit_group;\n\tcp.async.wait_group 0;\n" ::: "memory");
}
// 4-byte asynchronous copy that reads src_bytes (4 or 0) from gmem and
// zero-fills the rest
__device__ __forceinline__ void cp_async_u32_zfill(void *smem, const void *gmem, int src_bytes)
{
    const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4, %2;\n" ::"r"(s), "l"(gmem), "r"(src_bytes) : "memory");
}

#ifndef GBNTT_PASS_LIMB_ASYNC
#define GBNTT_PASS_LIMB_ASYNC 1   // first forward pass: limbs go to the tile through cp.async (all in flight)
#endif

// Tile word as the first DFT step reads it. In a first forward pass (LD_U32)
// the slot holds a 32-bit limb in its low word (the rest of an 8-byte slot
// is not written), reduced here: the limb itself for a 64-bit prime, one
// conditional subtract for p3. A slot that already holds the reduced value
// reads the same.
template <int PI, int LD>
__device__ __forceinline__ typename Field<PI>::T tile_in(const typename Field<PI>::T *p)
{
    if constexpr (LD == LD_U32) return Field<PI>::from_u32(*(const uint32_t *)p);
    else return *p;
}

// Position in the second spectra of element addr of the product spectra: the
// same, within the one shared spectrum (other_log), or within the spectrum
// a pair of products shares (other_pair_log); for transforms of 3 2^k
// points (other_r3) the same per sub-transform of 2^k points.
__device__ __forceinline__ long long other_index(const PassArgs &a, long long addr)
{
    const int k = a.other_log ? a.other_log : a.other_pair_log;
    if (a.other_r3 && k) {   // sub-transform s = 3 p + m of product p (2^k points each)
        const long long s = addr >> k, p = s / 3, m = s - 3 * p;
        const long long bs = a.other_log ? m : 3 * (p >> 1) + m;
        return (bs << k) | (addr & ((1LL << k) - 1));
    }
    if (a.other_log) return addr & ((1LL << a.other_log) - 1);
    if (a.other_pair_log) {
        const int L = a.other_pair_log;
        return ((addr >> (L + 1)) << L) | (addr & ((1LL << L) - 1));
    }
    return addr;
}

// The second spectra for a contiguous tile [base, base + span) of the
// product spectra: when the tile lies within one product (one sub-transform
// for other_r3), other_index is a constant offset off over it (returns true;
// off = 0 without a shared spectrum), else it must be applied per element
// (returns false).
__device__ __forceinline__ bool other_tile_offset(const PassArgs &a, long long base, long long span, long long &off)
{
    off = 0;
    const int L = a.other_log ? a.other_log : a.other_pair_log;
    if (!L) return true;
    if ((base >> L) != ((base + span - 1) >> L)) return false;
    off = other_index(a, base) - base;
    return true;
}

// value of tile element at address addr for the load kind LD
template <int PI, int LD>
__device__ __forceinline__ typename Field<PI>::T load_elem(const PassArgs &a, const typename Field<PI>::T *data,
                                                           const typename Field<PI>::T *other, long long addr)
{
    using F = Field<PI>;
    if constexpr (LD == LD_U32) {
        return F::from_u32((uint32_t)limb32_at(a, addr));
    } else if constexpr (LD == LD_U64LIMB) {
        if constexpr (sizeof(typename F::T) == 8) return F::from_u64(limb64_residue<PI>(a, addr));
        else return F::zero();
    } else if constexpr (LD == LD_PW) {
        return F::mul(data[addr], other[other_index(a, addr)]);
    } else {
        return data[addr];
    }
}

// Issue (without waiting) the cp.async copies of the residue tile whose first
// column is col0 into sm: tile element (g, m) -> sm[g*RS + m + m/B]; rows of
// a contiguous tile beyond the pass are zero-filled with plain stores.
template <int PI, int LOG_L, int LAYOUT, bool OTHER = false>
__device__ __forceinline__ void issue_tile_loads_from(const PassArgs &a, const typename Field<PI>::T *data,
                                                      typename Field<PI>::T *sm, long long col0)
{
    using F = Field<PI>;
    using V = typename F::T;
    using S_ = PassShape<LOG_L, sizeof(V)>;
    constexpr int L = S_::L, A = S_::A, B = S_::B, LOG_B = S_::LOG_B, G = S_::G, LOG_G = S_::LOG_G;
    constexpr int T = S_::T, RS = S_::RS;
    const int t = threadIdx.x;
    const int log_s = a.log_s, log_m = a.log_m;
    if (LAYOUT == LAYOUT_STRIDED) {
        const uint64_t j0 = (uint64_t)(col0 & ((1LL << log_s) - 1));
        const int g = t & (G - 1), m0 = t >> LOG_G;
        const long long S = 1LL << log_s;
        const long long base = ((col0 >> log_s) << log_m) + (long long)j0 + g + (long long)m0 * S;
        const long long stepg = (long long)B * S;
        V *dst = sm + g * RS + m0;
#pragma unroll
        for (int it = 0; it < A; it++) cp_async_word<sizeof(V)>(dst + it * (B + 1), data + base + it * stepg);
    } else {
        const long long rows_left = a.ncols - col0;
        const long long base = col0 << LOG_L;
        long long off = 0;
        if (!OTHER || other_tile_offset(a, base, (long long)G << LOG_L, off)) {
            const V *src = data + off + base;
#pragma unroll
            for (int it = 0; it < A; it++) {
                const int e = t + it * T;
                const int g = e >> LOG_L, m = e & (L - 1);
                V *d = sm + g * RS + m + (m >> LOG_B);
                if (g < rows_left) cp_async_word<sizeof(V)>(d, src + e);
                else *d = F::zero();
            }
        } else {   // a tile over several products sharing second spectra
#pragma unroll
            for (int it = 0; it < A; it++) {
                const int e = t + it * T;
                const int g = e >> LOG_L, m = e & (L - 1);
                V *d = sm + g * RS + m + (m >> LOG_B);
                if (g < rows_left) cp_async_word<sizeof(V)>(d, data + other_index(a, base + e));
                else *d = F::zero();
            }
        }
    }
}

template <int PI, int LOG_L, int LAYOUT>
__device__ __forceinline__ void issue_tile_loads(const PassArgs &a, typename Field<PI>::T *sm, long long col0)
{
    issue_tile_loads_from<PI, LOG_L, LAYOUT>(a, (const typename Field<PI>::T *)a.data[Field<PI>::SLOT], sm, col0);
}

// The 2^l-point DFT of every column of a tile in shared memory, in place:
// tile element (g, m) at sm[g RS + m + m/B] in natural order in, output k
// at the same index out (forward: DIF, inverse: its transpose). Starts with
// the tile complete in shared memory (after a barrier) and ends with a
// barrier.
template <int PI, int LOG_L, int DIR, int LD>
__device__ __forceinline__ void tile_steps(typename Field<PI>::T *sm, const uint64_t *w64,
                                           const typename Field<PI>::T *st1)
{
    using F = Field<PI>;
    using V = typename F::T;
    using S_ = PassShape<LOG_L, sizeof(V)>;
    constexpr int A = S_::A, B = S_::B, LOG_B = S_::LOG_B, RS = S_::RS;
    const int t = threadIdx.x;
    if constexpr (S_::A == S_::B && GBNTT_PASS_SHARED_DFT) {
        // Even l: both steps are A-point DFTs whose outputs go to
        // sm[g RS + k (B + 1) + lane]; only the read differs (column, then
        // row). One loop body keeps a single copy of the unrolled DFT code.
        const int g = t >> LOG_B, lane = t & (B - 1);
#pragma unroll 1
        for (int phase = 0; phase < 2; phase++) {
            V x[A];
            const int rbase = g * RS + (phase == 0 ? lane : lane * (B + 1));
            const int rstride = phase == 0 ? (B + 1) : 1;
            if (phase == 0) {
#pragma unroll
                for (int i = 0; i < A; i++) x[i] = tile_in<PI, LD>(&sm[rbase + i * rstride]);
            } else {
#pragma unroll
                for (int i = 0; i < A; i++) x[i] = sm[rbase + i * rstride];
            }
            dft_reg<PI, S_::LOG_A, DIR>(x, w64);
            if (phase == 0) {
                if (lane > 0) {   // w_L^(lane ka)
#pragma unroll
                    for (int ka = 1; ka < A; ka++) {
                        const int idx = bitrev(ka, S_::LOG_A);
                        x[idx] = F::mul(x[idx], __ldg(st1 + ka * B + lane));
                    }
                }
            }
            __syncthreads();
#pragma unroll
            for (int k = 0; k < A; k++) sm[g * RS + k * (B + 1) + lane] = x[bitrev(k, S_::LOG_A)];
            __syncthreads();
        }
    } else {
    // ---- step 1: one A-point DFT per (g, b) over the high digit
    {
        const int g = t >> LOG_B, b = t & (B - 1);
        V x[A];
#pragma unroll
        for (int i = 0; i < A; i++) x[i] = tile_in<PI, LD>(&sm[g * RS + i * (B + 1) + b]);
        dft_reg<PI, S_::LOG_A, DIR>(x, w64);
#pragma unroll
        for (int ka = 0; ka < A; ka++) {
            V v = x[bitrev(ka, S_::LOG_A)];
            if (ka > 0 && b > 0)   // w_L^(b ka)
                v = F::mul(v, __ldg(st1 + ka * B + b));
            sm[g * RS + ka * (B + 1) + b] = v;
        }
    }
    __syncthreads();

    // ---- step 2: A/B B-point DFTs per thread over the low digit
    {
        constexpr int R = A / B;
        const int g = t >> LOG_B, q = t & (B - 1);
        if constexpr (R == 2 && GBNTT_PASS_SHARED_DFT) {
            // odd l: the two B-point DFTs of a thread run through one loop
            // body (one copy of the unrolled code); the first result waits
            // in y0 until the barrier, the second stays in z
            V y0[B], z[B];
#pragma unroll 1
            for (int r = 0; r < 2; r++) {
                const int ka = q + r * B;
#pragma unroll
                for (int i = 0; i < B; i++) z[i] = sm[g * RS + ka * (B + 1) + i];
                dft_reg<PI, LOG_B, DIR>(z, w64);
                if (r == 0) {
#pragma unroll
                    for (int i = 0; i < B; i++) y0[i] = z[i];
                }
            }
            __syncthreads();
#pragma unroll
            for (int kb = 0; kb < B; kb++) {
                const int k0 = q + A * kb, k1 = q + B + A * kb;
                sm[g * RS + k0 + (k0 >> LOG_B)] = y0[bitrev(kb, LOG_B)];
                sm[g * RS + k1 + (k1 >> LOG_B)] = z[bitrev(kb, LOG_B)];
            }
        } else {
            V y[R][B];
#pragma unroll
            for (int r = 0; r < R; r++) {
                const int ka = q + r * B;
#pragma unroll
                for (int i = 0; i < B; i++) y[r][i] = sm[g * RS + ka * (B + 1) + i];
                dft_reg<PI, LOG_B, DIR>(y[r], w64);
            }
            __syncthreads();
#pragma unroll
            for (int r = 0; r < R; r++) {
                const int ka = q + r * B;
#pragma unroll
                for (int kb = 0; kb < B; kb++) {
                    const int k = ka + A * kb;
                    sm[g * RS + k + (k >> LOG_B)] = y[r][bitrev(kb, LOG_B)];
                }
            }
        }
    }
    __syncthreads();
    }
}

// One tile of a pass: load (unless PRELOADED: the caller has already
// brought this thread's words of the tile into sm), DFT steps, store.
template <int PI, int LOG_L, int DIR, int LD, int LAYOUT, bool PRELOADED = false>
__device__ __forceinline__ void pass_tile(const PassArgs &a, typename Field<PI>::T *sm, const uint64_t *w64,
                                          long long col0)
{
    using F = Field<PI>;
    using V = typename F::T;
    using S_ = PassShape<LOG_L, sizeof(V)>;
    constexpr int L = S_::L, A = S_::A, B = S_::B, LOG_B = S_::LOG_B, G = S_::G, LOG_G = S_::LOG_G;
    constexpr int T = S_::T, RS = S_::RS;
    const int t = threadIdx.x;
    const int log_s = a.log_s, log_m = a.log_m;
    V *data = (V *)a.data[F::SLOT];
    const V *other = (const V *)a.other[F::SLOT];
    const V *twhi = (const V *)a.tw.hi[F::SLOT];
    const V *twlo = (const V *)a.tw.lo[F::SLOT];
    const V *st1 = (const V *)a.tw.st1[F::SLOT] + (L - 32);   // w_L^(ka b) at [ka B + b]
    const int sh = kMaxLog - log_m;
    // column index within the sub-problem of the first column of this CTA
    const uint64_t j0 = LAYOUT == LAYOUT_STRIDED ? (uint64_t)(col0 & ((1LL << log_s) - 1)) : 0ull;

    // ---- load: tile element (g, m) -> sm[g*RS + m + m/B]
    if constexpr (PRELOADED) {
    } else if constexpr (LD == LD_U64 && GBNTT_PASS_CPASYNC) {
        issue_tile_loads<PI, LOG_L, LAYOUT>(a, sm, col0);
        cp_async_wait_all();
    } else if (LAYOUT == LAYOUT_STRIDED) {
        const int g = t & (G - 1), m0 = t >> LOG_G;            // m = m0 + it*B
        const long long S = 1LL << log_s;
        const long long base = ((col0 >> log_s) << log_m) + (long long)j0 + g + (long long)m0 * S;
        const long long stepg = (long long)B * S;
        V *dst = sm + g * RS + m0;
        bool loaded = false;
        if constexpr (LD == LD_U32 && GBNTT_PASS_LIMB_ASYNC) {
            if (!a.limb_tab) {
                // one operand's limbs: every copy of the thread in flight at
                // once, zero-filled beyond the operand (the slot's low word;
                // tile_in reduces it when step 1 reads it)
                const uint32_t *limbs = a.limbs;
#pragma unroll
                for (int it = 0; it < A; it++) {
                    const long long addr = base + it * stepg;
                    const bool in = addr < a.n_limbs;
                    cp_async_u32_zfill(dst + it * (B + 1), limbs + (in ? addr : 0), in ? 4 : 0);
                }
                cp_async_wait_all();
                loaded = true;
            }
        }
        if (!loaded) {
            if constexpr (sizeof(V) == 4) {   // all A loads in flight (registers allow it)
#pragma unroll
                for (int it = 0; it < A; it++) dst[it * (B + 1)] = load_elem<PI, LD>(a, data, other, base + it * stepg);
            } else {
#pragma unroll 8
                for (int it = 0; it < A; it++) dst[it * (B + 1)] = load_elem<PI, LD>(a, data, other, base + it * stepg);
            }
        }
        if constexpr (LD == LD_U32 && sizeof(V) == 8) {
            // staged first pass (64-bit prime, whose residue of a limb is
            // the limb): copy the limbs just read to stage_out in HBM
            if (a.stage_out) {
#pragma unroll 4
                for (int it = 0; it < A; it++) {
                    const long long addr = base + it * stepg;
                    if (addr < a.n_limbs) a.stage_out[addr] = F::low32(dst[it * (B + 1)]);
                }
            }
        }
    } else if constexpr (LD == LD_PW && GBNTT_PASS_PW_ASYNC) {
        // pointwise product: this spectrum's words go to the tile through
        // cp.async while the other spectrum's words are loaded into
        // registers, all in flight at once; each thread then multiplies the
        // words it copied (visible to it after the wait)
        const long long rows_left = a.ncols - col0;
        const long long base = col0 << LOG_L;
        // a shared second spectrum (one operand common to the whole batch,
        // or to a pair of products) is read at the position other_index gives
        V o[A];
        long long off = 0;
        const bool flat = other_tile_offset(a, base, (long long)G << LOG_L, off);
        const V *osrc = other + off + base;
#pragma unroll
        for (int it = 0; it < A; it++) {
            const int e = t + it * T;
            const int g = e >> LOG_L, m = e & (L - 1);
            V *d = sm + g * RS + m + (m >> LOG_B);
            if (g < rows_left) {
                cp_async_word<sizeof(V)>(d, data + base + e);
                o[it] = __ldg(flat ? osrc + e : other + other_index(a, base + e));
            } else {
                *d = F::zero();
                o[it] = F::zero();
            }
        }
        cp_async_wait_all();
#pragma unroll
        for (int it = 0; it < A; it++) {
            const int e = t + it * T;
            const int m = e & (L - 1);
            V *d = sm + (e >> LOG_L) * RS + m + (m >> LOG_B);
            *d = F::mul(*d, o[it]);
        }
    } else {
        const long long rows_left = a.ncols - col0;
        const long long base = col0 << LOG_L;
#pragma unroll 8
        for (int it = 0; it < A; it++) {
            const int e = t + it * T;
            const int g = e >> LOG_L, m = e & (L - 1);
            V v = F::zero();
            if (g < rows_left) v = load_elem<PI, LD>(a, data, other, base + e);
            sm[g * RS + m + (m >> LOG_B)] = v;
        }
        if constexpr (LD == LD_U32 && sizeof(V) == 8) {
            if (a.stage_out) {   // staged first pass, as in the strided layout
#pragma unroll 4
                for (int it = 0; it < A; it++) {
                    const int e = t + it * T;
                    const int g = e >> LOG_L, m = e & (L - 1);
                    if (g < rows_left && base + e < a.n_limbs) a.stage_out[base + e] = F::low32(sm[g * RS + m + (m >> LOG_B)]);
                }
            }
        }
    }
    if (DIR == 1 && (a.twiddle || a.use_scale)) {
        // inverse pass: input row m of column j gets w_M^-(j m), times the
        // scale in the last pass; each thread scales the words it loaded (a
        // partly rolled loop instead of the unrolled register step)
        if (LAYOUT == LAYOUT_STRIDED) {
            const int g = t & (G - 1), m0 = t >> LOG_G;
            const uint64_t j = j0 + (uint64_t)g;
            V *dst = sm + g * RS + m0;
            const V *ptw = (const V *)a.ptw[F::SLOT];
            if (a.twiddle && ptw) {
                // table entry j + m S (the scale already folded in)
                const long long S = 1LL << log_s;
                const V *tp = ptw + (long long)j + (long long)m0 * S;
                const long long stepg = (long long)B * S;
#pragma unroll 4
                for (int it = 0; it < A; it++) dst[it * (B + 1)] = F::mul(dst[it * (B + 1)], __ldg(tp + it * stepg));
            } else if (a.twiddle) {
                V tw = tw_exp<PI>(twhi, twlo, (uint32_t)(((uint64_t)m0 * j) << sh));
                const V step = tw_exp<PI>(twhi, twlo, (uint32_t)(((uint64_t)B * j) << sh));
                if (a.use_scale) tw = F::mul(tw, F::from_u64(a.scale[F::SLOT]));
#pragma unroll 4
                for (int it = 0; it < A; it++) {
                    dst[it * (B + 1)] = F::mul(dst[it * (B + 1)], tw);
                    tw = F::mul(tw, step);
                }
            } else {
                const V sc = F::from_u64(a.scale[F::SLOT]);
#pragma unroll 4
                for (int it = 0; it < A; it++) dst[it * (B + 1)] = F::mul(dst[it * (B + 1)], sc);
            }
        } else {   // contiguous: no twiddle (S = 1), only the scale
            const long long rows_left = a.ncols - col0;
            const V sc = F::from_u64(a.scale[F::SLOT]);
#pragma unroll 4
            for (int it = 0; it < A; it++) {
                const int e = t + it * T;
                const int g = e >> LOG_L, m = e & (L - 1);
                if (g < rows_left) {
                    V *d = sm + g * RS + m + (m >> LOG_B);
                    *d = F::mul(*d, sc);
                }
            }
        }
    }
    __syncthreads();

    tile_steps<PI, LOG_L, DIR, LD>(sm, w64, st1);

    // ---- store: same addressing as the load
    if (LAYOUT == LAYOUT_STRIDED) {
        const int g = t & (G - 1), m0 = t >> LOG_G;
        const long long S = 1LL << log_s;
        const long long base = ((col0 >> log_s) << log_m) + (long long)j0 + g + (long long)m0 * S;
        const long long stepg = (long long)B * S;
        const V *src = sm + g * RS + m0;
        const V *ptw = (const V *)a.ptw[F::SLOT];
        if (DIR == 0 && a.twiddle && ptw) {
            // forward pass, twiddle w_M^(j k) from the pass table (entry
            // j + k S, the element's offset within its sub-problem)
            const V *tp = ptw + (long long)(j0 + (uint64_t)g) + (long long)m0 * S;
#pragma unroll 4
            for (int it = 0; it < A; it++) data[base + it * stepg] = F::mul(src[it * (B + 1)], __ldg(tp + it * stepg));
        } else if (DIR == 0 && a.twiddle) {
            // forward pass: output k = m0 + it B of column j gets w_M^(j k),
            // applied here (a partly rolled loop) instead of in the
            // unrolled register step
            const uint64_t j = j0 + (uint64_t)g;
            V tw = tw_exp<PI>(twhi, twlo, (uint32_t)(((uint64_t)m0 * j) << sh));
            const V step = tw_exp<PI>(twhi, twlo, (uint32_t)(((uint64_t)B * j) << sh));
#pragma unroll 4
            for (int it = 0; it < A; it++) {
                data[base + it * stepg] = F::mul(src[it * (B + 1)], tw);
                tw = F::mul(tw, step);
            }
        } else {
#pragma unroll 8
            for (int it = 0; it < A; it++) data[base + it * stepg] = src[it * (B + 1)];
        }
    } else {
        const long long rows_left = a.ncols - col0;
        const long long base = col0 << LOG_L;
#pragma unroll 8
        for (int it = 0; it < A; it++) {
            const int e = t + it * T;
            const int g = e >> LOG_L, m = e & (L - 1);
            if (g < rows_left) data[base + e] = sm[g * RS + m + (m >> LOG_B)];
        }
    }
}

template <int PI, int LOG_L, int DIR, int LD, int LAYOUT>
__global__ void __launch_bounds__(kPassThreads, PassMinBlocks<PI, LOG_L>::value) ntt_pass_kernel(PassArgs a)
{
    extern __shared__ uint64_t sm[];
    using S_ = PassShape<LOG_L, sizeof(typename Field<PI>::T)>;
    pass_tile<PI, LOG_L, DIR, LD, LAYOUT>(a, reinterpret_cast<typename Field<PI>::T *>(sm), a.w64,
                                          (long long)blockIdx.x * S_::G);
}

// Persistent form of a residue pass (software pipelined): each CTA walks
// tiles blockIdx.x, blockIdx.x + gridDim.x, ... with two shared-memory tile
// buffers; the next tile's cp.async copies are in flight while the current
// tile is transformed and stored, so global-load latency is hidden behind
// the DFTs instead of being waited out by every CTA.
template <int PI, int LOG_L, int DIR, int LAYOUT>
__global__ void __launch_bounds__(kPassThreads, PassMinBlocks<PI, LOG_L>::value) ntt_pass_kernel_pipe(PassArgs a)
{
    extern __shared__ uint64_t smraw[];
    using V = typename Field<PI>::T;
    using S_ = PassShape<LOG_L, sizeof(V)>;
    constexpr size_t TW = S_::SMEM / sizeof(V);   // words per tile buffer
    V *const buf0 = reinterpret_cast<V *>(smraw), *const buf1 = buf0 + TW;
    const long long ntiles = (a.ncols + S_::G - 1) / S_::G;
    long long tile = blockIdx.x;
    if (tile >= ntiles) return;
    issue_tile_loads<PI, LOG_L, LAYOUT>(a, buf0, tile * S_::G);
    asm volatile("cp.async.commit_group;\n" ::: "memory");
    int cur = 0;
    for (; tile < ntiles; tile += gridDim.x) {
        const long long next = tile + gridDim.x;
        if (next < ntiles) issue_tile_loads<PI, LOG_L, LAYOUT>(a, cur ? buf0 : buf1, next * S_::G);
        asm volatile("cp.async.commit_group;\n\tcp.async.wait_group 1;\n" ::: "memory");
        pass_tile<PI, LOG_L, DIR, LD_U64, LAYOUT, true>(a, cur ? buf1 : buf0, a.w64, tile * S_::G);
        __syncthreads();   // buf[cur] is refilled by the next iteration's prefetch
        cur ^= 1;
    }
}

#ifndef GBNTT_PASS_PIPE32
#define GBNTT_PASS_PIPE32 0   // pipelined residue passes for the 32-bit prime (measured slower: 99 ms against 82 ms)
#endif
#ifndef GBNTT_PASS_PIPE64
#define GBNTT_PASS_PIPE64 0   // and for the 64-bit primes (measured slower still: 110 ms)
#endif

// Launch a pipelined residue pass: as many resident CTAs as fit, each with
// two tile buffers.
template <int PI, int LOG_L, int DIR, int LAYOUT>
static cudaError_t launch_pipe(const PassArgs &a, cudaStream_t st)
{
    using S_ = PassShape<LOG_L, sizeof(typename Field<PI>::T)>;
    static int grid_cap = 0;
    auto fn = ntt_pass_kernel_pipe<PI, LOG_L, DIR, LAYOUT>;
    const size_t smem = 2 * S_::SMEM;
    if (grid_cap == 0) {
        cudaError_t e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return e;
        int dev = 0, sms = 0, per = 0;
        if ((e = cudaGetDevice(&dev)) != cudaSuccess) return e;
        if ((e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev)) != cudaSuccess) return e;
        if ((e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, fn, kPassThreads, smem)) != cudaSuccess) return e;
        grid_cap = std::max(1, sms * per);
    }
    const long long ntiles = (a.ncols + S_::G - 1) / S_::G;
    const long long grid = std::min<long long>(ntiles, grid_cap);
    fn<<<(unsigned)grid, kPassThreads, smem, st>>>(a);
    return cudaGetLastError();
}

// Launcher for one prime (explicitly instantiated, one translation unit per
// prime so the three are compiled in parallel).
template <int PI, int LOG_L>
static cudaError_t launch_pass_l(int dir, int ld, const PassArgs &a, cudaStream_t st)
{
    using S_ = PassShape<LOG_L, sizeof(typename Field<PI>::T)>;
    const int layout = a.log_s == 0 ? LAYOUT_CONTIG : LAYOUT_STRIDED;
    constexpr bool kPipe = sizeof(typename Field<PI>::T) == 4 ? GBNTT_PASS_PIPE32 : GBNTT_PASS_PIPE64;
    if constexpr (kPipe && GBNTT_PASS_CPASYNC) {
        if (ld == LD_U64) {
            if (dir == 0)
                return layout == LAYOUT_STRIDED ? launch_pipe<PI, LOG_L, 0, LAYOUT_STRIDED>(a, st)
                                                : launch_pipe<PI, LOG_L, 0, LAYOUT_CONTIG>(a, st);
            if (layout == LAYOUT_STRIDED) return launch_pipe<PI, LOG_L, 1, LAYOUT_STRIDED>(a, st);
        }
    }
    void (*fn)(PassArgs) = nullptr;
    if (dir == 0) {
        if (ld == LD_U32)
            fn = layout == LAYOUT_STRIDED ? ntt_pass_kernel<PI, LOG_L, 0, LD_U32, LAYOUT_STRIDED>
                                          : ntt_pass_kernel<PI, LOG_L, 0, LD_U32, LAYOUT_CONTIG>;
        else if (ld == LD_U64LIMB) {
            if constexpr (sizeof(typename Field<PI>::T) == 8)   // packed limbs: 64-bit primes only
                fn = layout == LAYOUT_STRIDED ? ntt_pass_kernel<PI, LOG_L, 0, LD_U64LIMB, LAYOUT_STRIDED>
                                              : ntt_pass_kernel<PI, LOG_L, 0, LD_U64LIMB, LAYOUT_CONTIG>;
        } else
            fn = layout == LAYOUT_STRIDED ? ntt_pass_kernel<PI, LOG_L, 0, LD_U64, LAYOUT_STRIDED>
                                          : ntt_pass_kernel<PI, LOG_L, 0, LD_U64, LAYOUT_CONTIG>;
    } else {
        // the pointwise pass is always the innermost (contiguous) one and the
        // other inverse passes are strided
        if (ld == LD_PW && layout == LAYOUT_CONTIG) fn = ntt_pass_kernel<PI, LOG_L, 1, LD_PW, LAYOUT_CONTIG>;
        else if (ld == LD_U64 && layout == LAYOUT_STRIDED) fn = ntt_pass_kernel<PI, LOG_L, 1, LD_U64, LAYOUT_STRIDED>;
    }
    if (!fn) return cudaErrorInvalidValue;
    const long long gx = (a.ncols + S_::G - 1) / S_::G;
    fn<<<(unsigned)gx, kPassThreads, S_::SMEM, st>>>(a);
    return cudaGetLastError();
}

#ifndef GBNTT_FUSED_MIN_BLOCKS
#define GBNTT_FUSED_MIN_BLOCKS 6   // resident CTAs the fused kernel's registers target (64-bit primes; two tiles of shared memory each)
#endif
template <int PI, int LOG_L>
struct FusedMinBlocks {
    // 2^9- and 2^10-point tiles of 64-bit words: two of them take 54-68 KB
    // of shared memory, so at most three CTAs are resident anyway
    static constexpr int value = sizeof(typename Field<PI>::T) == 4 ? GBNTT_PASS_MIN_BLOCKS32
                                                                    : (LOG_L <= 8 ? GBNTT_FUSED_MIN_BLOCKS : 3);
};

// Innermost passes of a product in one launch. The innermost forward pass
// of each operand, the pointwise product and the innermost inverse pass all
// work on the same contiguous blocks of 2^l points, so a CTA loads G blocks
// of both spectra (as they are before their last forward pass), runs both
// forward DFTs, multiplies, runs the inverse DFT and stores the blocks of
// the product spectrum: three words of traffic per point instead of seven
// over three launches. No pass twiddle and no scale occur in these passes
// (plans of two or more passes). a.other == a.data: a square.
// PAIRED: products 2i and 2i + 1 share the second spectrum i (a separate
// instantiation, so that the unpaired kernel keeps its code as it is).
template <int PI, int LOG_L, bool PAIRED>
__global__ void __launch_bounds__(kPassThreads, FusedMinBlocks<PI, LOG_L>::value) ntt_inner_fused_kernel(PassArgs a)
{
    extern __shared__ uint64_t smraw[];
    using F = Field<PI>;
    using V = typename F::T;
    using S_ = PassShape<LOG_L, sizeof(V)>;
    constexpr int L = S_::L, A = S_::A, LOG_B = S_::LOG_B, LOG_L_ = LOG_L, T = S_::T, RS = S_::RS;
    constexpr size_t TW = S_::SMEM / sizeof(V);   // words per tile buffer
    V *const smA = reinterpret_cast<V *>(smraw);
    V *const smB = smA + TW;
    const long long col0 = (long long)blockIdx.x * S_::G;
    const bool square = a.other[F::SLOT] == a.data[F::SLOT];
    const int t = threadIdx.x;
    // both tiles' copies in flight at once
    issue_tile_loads_from<PI, LOG_L, LAYOUT_CONTIG>(a, (const V *)a.data[F::SLOT], smA, col0);
    if (!square) issue_tile_loads_from<PI, LOG_L, LAYOUT_CONTIG, PAIRED>(a, (const V *)a.other[F::SLOT], smB, col0);
    cp_async_wait_all();
    __syncthreads();
    const V *st1f = (const V *)a.tw.st1[F::SLOT] + (L - 32);
    const V *st1i = (const V *)a.st1_inv[F::SLOT] + (L - 32);
#pragma unroll 1
    for (int op = 0; op < (square ? 1 : 2); op++) tile_steps<PI, LOG_L, 0, LD_U64>(op ? smB : smA, a.w64, st1f);
    // pointwise product (Montgomery: leaves R^-1, folded into the scale of
    // the outermost inverse pass as in the unfused pointwise pass)
#pragma unroll 4
    for (int it = 0; it < A; it++) {
        const int e = t + it * T;
        const int g = e >> LOG_L_, m = e & (L - 1);
        const int idx = g * RS + m + (m >> LOG_B);
        smA[idx] = F::mul(smA[idx], square ? smA[idx] : smB[idx]);
    }
    __syncthreads();
    tile_steps<PI, LOG_L, 1, LD_U64>(smA, a.w64_inv, st1i);
    V *data = (V *)a.data[F::SLOT];
    const long long rows_left = a.ncols - col0;
    const long long base = col0 << LOG_L;
#pragma unroll 8
    for (int it = 0; it < A; it++) {
        const int e = t + it * T;
        const int g = e >> LOG_L_, m = e & (L - 1);
        if (g < rows_left) data[base + e] = smA[g * RS + m + (m >> LOG_B)];
    }
}

template <int PI, int LOG_L, bool PAIRED>
static cudaError_t launch_inner_fused_lp(const PassArgs &a, cudaStream_t st)
{
    using S_ = PassShape<LOG_L, sizeof(typename Field<PI>::T)>;
    const long long gx = (a.ncols + S_::G - 1) / S_::G;
    const size_t smem = 2 * S_::SMEM;
    auto fn = ntt_inner_fused_kernel<PI, LOG_L, PAIRED>;
    static bool attr_set = false;   // once per instantiation (before any graph capture uses it)
    if (smem > 48 * 1024 && !attr_set) {
        const cudaError_t e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return e;
        attr_set = true;
    }
    fn<<<(unsigned)gx, kPassThreads, smem, st>>>(a);
    return cudaGetLastError();
}

template <int PI, int LOG_L>
static cudaError_t launch_inner_fused_l(const PassArgs &a, cudaStream_t st)
{
    return a.other_pair_log ? launch_inner_fused_lp<PI, LOG_L, true>(a, st) : launch_inner_fused_lp<PI, LOG_L, false>(a, st);
}

template <int PI>
cudaError_t launch_inner_fused_prime(int log_l, const PassArgs &a, cudaStream_t st)
{
    switch (log_l) {
    case 5: return launch_inner_fused_l<PI, 5>(a, st);
    case 6: return launch_inner_fused_l<PI, 6>(a, st);
    case 7: return launch_inner_fused_l<PI, 7>(a, st);
    case 8: return launch_inner_fused_l<PI, 8>(a, st);
    case 9: return launch_inner_fused_l<PI, 9>(a, st);
    case 10: return launch_inner_fused_l<PI, 10>(a, st);
    default: return cudaErrorInvalidValue;
    }
}

// Pass twiddle table: entry e = j + m S (m < 2^(log_m - log_s), j < S) is
// w_M^(j m) from the two-level tables of the wanted direction, times scale
// when use_scale is set.
template <int PI>
__global__ void build_pass_twiddles_kernel(typename Field<PI>::T *table, const typename Field<PI>::T *hi,
                                           const typename Field<PI>::T *lo, int log_m, int log_s, int use_scale,
                                           uint64_t scale64)
{
    const typename Field<PI>::T scale = Field<PI>::from_u64(scale64);
    const long long M = 1LL << log_m;
    const int sh = kMaxLog - log_m;
    for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < M; e += (long long)gridDim.x * blockDim.x) {
        const uint64_t m = (uint64_t)e >> log_s, j = (uint64_t)e & ((1ull << log_s) - 1);
        typename Field<PI>::T w = tw_exp<PI>(hi, lo, (uint32_t)((m * j) << sh));
        if (use_scale) w = Field<PI>::mul(w, scale);
        table[e] = w;
    }
}

template <int PI>
cudaError_t launch_build_pass_twiddles(uint64_t *table, const uint64_t *hi, const uint64_t *lo, int log_m, int log_s,
                                       int use_scale, uint64_t scale, cudaStream_t st)
{
    using V = typename Field<PI>::T;
    const long long M = 1LL << log_m;
    const long long grid = std::min<long long>((M + 255) / 256, 152 * 16);
    build_pass_twiddles_kernel<PI><<<(unsigned)grid, 256, 0, st>>>((V *)table, (const V *)hi, (const V *)lo, log_m,
                                                                   log_s, use_scale, scale);
    return cudaGetLastError();
}

template <int PI>
cudaError_t launch_pass_prime(int log_l, int dir, int ld, const PassArgs &a, cudaStream_t st)
{
    switch (log_l) {
    case 5: return launch_pass_l<PI, 5>(dir, ld, a, st);
    case 6: return launch_pass_l<PI, 6>(dir, ld, a, st);
    case 7: return launch_pass_l<PI, 7>(dir, ld, a, st);
    case 8: return launch_pass_l<PI, 8>(dir, ld, a, st);
    case 9: return launch_pass_l<PI, 9>(dir, ld, a, st);
    case 10: return launch_pass_l<PI, 10>(dir, ld, a, st);
    default: return cudaErrorInvalidValue;
    }
}

}  // namespace gbntt
