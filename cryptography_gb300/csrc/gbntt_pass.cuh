// gbntt_pass.cuh — one NTT pass of 2^l points (l = 5..10) for one prime.
//
// The transform of N = 2^L points is a chain of 1-3 passes (outermost
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
#include "gbntt_arith.cuh"
#include "gbntt_internal.h"

namespace gbntt {

enum PassLayout { LAYOUT_STRIDED = 0, LAYOUT_CONTIG = 1 };

#ifndef GBNTT_PASS_MIN_BLOCKS
#define GBNTT_PASS_MIN_BLOCKS 5   // resident CTAs per SM the register budget targets
#endif
constexpr int kPassThreads = 128;
constexpr int kLogPassThreads = 7;

template <int LOG_L>
struct PassShape {
    static constexpr int L = 1 << LOG_L;
    static constexpr int LOG_A = (LOG_L + 1) / 2, LOG_B = LOG_L / 2;
    static constexpr int A = 1 << LOG_A, B = 1 << LOG_B;
    static constexpr int T = kPassThreads;
    static constexpr int LOG_G = kLogPassThreads - LOG_B;
    static constexpr int G = 1 << LOG_G;          // columns per CTA
    static constexpr int RS = L + A + 1;          // odd row stride in 8-byte words
    static constexpr size_t SMEM = (size_t)G * RS * 8;
};

__host__ __device__ constexpr int bitrev(int x, int bits)
{
    int r = 0;
    for (int i = 0; i < bits; i++) r = (r << 1) | ((x >> i) & 1);
    return r;
}

// w^E from the two-level tables (Montgomery form), E < 2^30.
template <int PI>
__device__ __forceinline__ uint64_t tw_exp(const uint64_t *hi, const uint64_t *lo, uint32_t e)
{
    return mont_mul<PI>(__ldg(hi + (e >> kTwBits)), __ldg(lo + (e & (kTwSize - 1))));
}

// In-register radix-2 DIF DFT of 2^LOG_R points: natural order in,
// bit-reversed order out (X[k] ends in x[bitrev(k)]). w64 = Montgomery forms
// of the primitive 64th root's powers.
template <int PI, int LOG_R>
__device__ __forceinline__ void dft_reg(uint64_t (&x)[1 << LOG_R], const uint64_t *w64)
{
    constexpr int R = 1 << LOG_R;
#pragma unroll
    for (int s = R / 2; s >= 1; s >>= 1) {
#pragma unroll
        for (int blk = 0; blk < R; blk += 2 * s) {
#pragma unroll
            for (int i = 0; i < s; i++) {
                const uint64_t u = x[blk + i], v = x[blk + i + s];
                x[blk + i] = add_mod<PI>(u, v);
                const uint64_t d = sub_mod<PI>(u, v);
                // w_{2s}^i = w_64^(i * 32 / s)
                x[blk + i + s] = (i == 0) ? d : mont_mul<PI>(d, w64[i * (32 / s)]);
            }
        }
    }
}

// cp.async helpers (8-byte / 4-byte copies, zero-filled when src_bytes == 0).
__device__ __forceinline__ void cp_async8(void *dst, const void *src, int src_bytes)
{
    const unsigned d = (unsigned)__cvta_generic_to_shared(dst);
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8, %2;\n" ::"r"(d), "l"(src), "r"(src_bytes));
}
__device__ __forceinline__ void cp_async4(void *dst, const void *src, int src_bytes)
{
    const unsigned d = (unsigned)__cvta_generic_to_shared(dst);
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4, %2;\n" ::"r"(d), "l"(src), "r"(src_bytes));
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::); }
template <int N>
__device__ __forceinline__ void cp_async_wait() { asm volatile("cp.async.wait_group %0;\n" ::"n"(N)); }

// Shared-memory plan of one CTA (in 8-byte words):
//   [0, L)              in-CTA twiddles twm[ka*B + b] = w_L^(b ka)
//   then, by load kind:
//   LD_U64: two tile buffers (double buffering)
//   LD_U32: one 8-byte work tile + two 4-byte input tiles
//   LD_PW : two 8-byte tiles (both spectra, single buffered)
template <int LOG_L, int LD>
struct PassSmem {
    using S_ = PassShape<LOG_L>;
    static constexpr int TILE = S_::G * S_::RS;     // words of one 8-byte tile
    static constexpr int TW = S_::L;
    static constexpr size_t BYTES = 8 * (size_t)(TW + (LD == LD_U32 ? TILE + TILE : 2 * TILE));
};

// Element (g, m) of tile `tile` -> global index, for both layouts.
template <int LOG_L, int LAYOUT>
struct TileAddr {
    using S_ = PassShape<LOG_L>;
    long long base;    // address of (g_thread, m_thread(it = 0))
    long long step;    // address increment per iteration
    __device__ __forceinline__ TileAddr(long long col0, int log_s, int log_m, int t)
    {
        if (LAYOUT == LAYOUT_STRIDED) {
            const int g = t & (S_::G - 1), m0 = t >> S_::LOG_G;
            const long long S = 1LL << log_s;
            base = ((col0 >> log_s) << log_m) + (col0 & (S - 1)) + g + (long long)m0 * S;
            step = (long long)S_::B * S;
        } else {
            base = (col0 << LOG_L) + t;
            step = S_::T;
        }
    }
};

// Shared-memory word of iteration `it` of thread t (same mapping as TileAddr).
template <int LOG_L, int LAYOUT>
__device__ __forceinline__ int tile_slot(int t, int it)
{
    using S_ = PassShape<LOG_L>;
    if (LAYOUT == LAYOUT_STRIDED) {
        const int g = t & (S_::G - 1), m0 = t >> S_::LOG_G;
        return g * S_::RS + m0 + it * (S_::B + 1);
    } else {
        const int e = t + it * S_::T;
        const int g = e >> LOG_L, m = e & (S_::L - 1);
        return g * S_::RS + m + (m >> S_::LOG_B);
    }
}

// Row (column group member) of iteration `it` of thread t, for bounds checks
// of the contiguous layout.
template <int LOG_L, int LAYOUT>
__device__ __forceinline__ int tile_row(int t, int it)
{
    using S_ = PassShape<LOG_L>;
    return LAYOUT == LAYOUT_STRIDED ? (t & (S_::G - 1)) : ((t + it * S_::T) >> LOG_L);
}

// Issue the asynchronous loads of one tile (A copies per thread).
template <int LOG_L, int LD, int LAYOUT>
__device__ __forceinline__ void tile_load_async(const PassArgs &a, const uint64_t *src64, long long col0, void *dst,
                                                int t)
{
    using S_ = PassShape<LOG_L>;
    const TileAddr<LOG_L, LAYOUT> ad(col0, a.log_s, a.log_m, t);
    const long long rows_left = a.ncols - col0;
#pragma unroll 8
    for (int it = 0; it < S_::A; it++) {
        const long long addr = ad.base + it * ad.step;
        const int slot = tile_slot<LOG_L, LAYOUT>(t, it);
        const bool row_ok = LAYOUT == LAYOUT_STRIDED || tile_row<LOG_L, LAYOUT>(t, it) < rows_left;
        if (LD == LD_U32) {
            const bool ok = row_ok && addr < a.n_limbs;
            cp_async4((uint32_t *)dst + slot, ok ? (const void *)(a.limbs + addr) : (const void *)a.limbs, ok ? 4 : 0);
        } else {
            cp_async8((uint64_t *)dst + slot, row_ok ? (const void *)(src64 + addr) : (const void *)src64,
                      row_ok ? 8 : 0);
        }
    }
}

// Steps 1 and 2 of one tile, in place in `w` (8-byte words); `in32` is the
// 4-byte input tile of the first forward pass, `inB` the second spectrum of
// the pointwise pass.
template <int PI, int LOG_L, int DIR, int LD, int LAYOUT>
__device__ __forceinline__ void tile_compute(const PassArgs &a, uint64_t *w, const uint32_t *in32,
                                             const uint64_t *inB, const uint64_t *twm, const uint64_t *w64,
                                             long long col0, int t)
{
    using S_ = PassShape<LOG_L>;
    constexpr int A = S_::A, B = S_::B, LOG_B = S_::LOG_B, RS = S_::RS;
    const uint64_t *twhi = a.tw.hi[PI];
    const uint64_t *twlo = a.tw.lo[PI];
    const int sh = kMaxLog - a.log_m;
    const uint64_t j0 = LAYOUT == LAYOUT_STRIDED ? (uint64_t)(col0 & ((1LL << a.log_s) - 1)) : 0ull;

    // ---- step 1: one A-point DFT per (g, b) over the high digit
    {
        const int g = t >> LOG_B, b = t & (B - 1);
        uint64_t x[A];
#pragma unroll
        for (int i = 0; i < A; i++) {
            const int idx = g * RS + i * (B + 1) + b;
            if (LD == LD_U32) x[i] = in32[idx];
            else if (LD == LD_PW) x[i] = mont_mul<PI>(w[idx], inB[idx]);
            else x[i] = w[idx];
        }
        if (DIR == 1 && (a.twiddle || a.use_scale)) {
            // inverse pass: input twiddle w_M^-((iB + b) j), times the scale
            const uint64_t j = j0 + (uint64_t)(LAYOUT == LAYOUT_STRIDED ? g : 0);
            uint64_t base = tw_exp<PI>(twhi, twlo, (uint32_t)(((uint64_t)b * j) << sh));
            const uint64_t step = tw_exp<PI>(twhi, twlo, (uint32_t)(((uint64_t)B * j) << sh));
            if (a.use_scale) base = mont_mul<PI>(base, a.scale[PI]);
#pragma unroll
            for (int i = 0; i < A; i++) {
                x[i] = mont_mul<PI>(x[i], base);
                if (i + 1 < A) base = mont_mul<PI>(base, step);
            }
        }
        dft_reg<PI, S_::LOG_A>(x, w64);
#pragma unroll
        for (int ka = 0; ka < A; ka++) {
            uint64_t v = x[bitrev(ka, S_::LOG_A)];
            if (ka > 0 && b > 0) v = mont_mul<PI>(v, twm[ka * B + b]);   // w_L^(b ka)
            w[g * RS + ka * (B + 1) + b] = v;
        }
    }
    __syncthreads();

    // ---- step 2: A/B B-point DFTs per thread over the low digit
    {
        constexpr int R = A / B;
        const int g = t >> LOG_B, q = t & (B - 1);
        uint64_t y[R][B];
        uint64_t step = 0;
        if (DIR == 0 && LAYOUT == LAYOUT_STRIDED && a.twiddle) {
            const uint64_t j = j0 + (uint64_t)g;
            step = tw_exp<PI>(twhi, twlo, (uint32_t)(((uint64_t)A * j) << sh));
        }
#pragma unroll
        for (int r = 0; r < R; r++) {
            const int ka = q + r * B;
#pragma unroll
            for (int i = 0; i < B; i++) y[r][i] = w[g * RS + ka * (B + 1) + i];
            dft_reg<PI, LOG_B>(y[r], w64);
            if (DIR == 0 && LAYOUT == LAYOUT_STRIDED && a.twiddle) {
                // forward pass: output twiddle w_M^((ka + A kb) j)
                const uint64_t j = j0 + (uint64_t)g;
                uint64_t base = tw_exp<PI>(twhi, twlo, (uint32_t)(((uint64_t)ka * j) << sh));
#pragma unroll
                for (int kb = 0; kb < B; kb++) {
                    const int idx = bitrev(kb, LOG_B);
                    y[r][idx] = mont_mul<PI>(y[r][idx], base);
                    if (kb + 1 < B) base = mont_mul<PI>(base, step);
                }
            }
        }
        __syncthreads();
#pragma unroll
        for (int r = 0; r < R; r++) {
            const int ka = q + r * B;
#pragma unroll
            for (int kb = 0; kb < B; kb++) {
                const int k = ka + A * kb;
                w[g * RS + k + (k >> LOG_B)] = y[r][bitrev(kb, LOG_B)];
            }
        }
    }
    __syncthreads();
}

// Global stores of one finished tile from `w`.
template <int LOG_L, int LAYOUT>
__device__ __forceinline__ void tile_store(const PassArgs &a, uint64_t *dst64, long long col0, const uint64_t *w, int t)
{
    using S_ = PassShape<LOG_L>;
    const TileAddr<LOG_L, LAYOUT> ad(col0, a.log_s, a.log_m, t);
    const long long rows_left = a.ncols - col0;
#pragma unroll 8
    for (int it = 0; it < S_::A; it++) {
        if (LAYOUT == LAYOUT_STRIDED || tile_row<LOG_L, LAYOUT>(t, it) < rows_left)
            dst64[ad.base + it * ad.step] = w[tile_slot<LOG_L, LAYOUT>(t, it)];
    }
}

// Persistent pass kernel: each CTA walks tiles blockIdx.x, +gridDim.x, ...;
// the next tile's loads (cp.async) are in flight while the current one is
// computed (not for the pointwise pass, which stages two spectra).
template <int PI, int LOG_L, int DIR, int LD, int LAYOUT>
__device__ __forceinline__ void pass_persistent(const PassArgs &a, uint64_t *sm, const uint64_t *w64)
{
    using S_ = PassShape<LOG_L>;
    using P_ = PassSmem<LOG_L, LD>;
    const int t = threadIdx.x;
    const long long ntiles = (a.ncols + S_::G - 1) / S_::G;
    uint64_t *twm = sm;
    uint64_t *data = a.data[PI];
    const uint64_t *twhi = a.tw.hi[PI];

    // in-CTA twiddles, once per CTA: twm[ka*B + b] = w_L^(b ka)
    for (int idx = t; idx < S_::L; idx += S_::T) {
        const int ka = idx >> S_::LOG_B, b = idx & (S_::B - 1);
        twm[idx] = __ldg(twhi + ((b * ka) << (kTwBits - LOG_L)));
    }

    long long tile = blockIdx.x;
    if (LD == LD_PW) {
        uint64_t *wA = sm + P_::TW, *wB = wA + P_::TILE;
        for (; tile < ntiles; tile += gridDim.x) {
            const long long col0 = tile * S_::G;
            tile_load_async<LOG_L, LD_U64, LAYOUT>(a, data, col0, wA, t);
            tile_load_async<LOG_L, LD_U64, LAYOUT>(a, a.other[PI], col0, wB, t);
            cp_async_commit();
            cp_async_wait<0>();
            __syncthreads();
            tile_compute<PI, LOG_L, DIR, LD, LAYOUT>(a, wA, nullptr, wB, twm, w64, col0, t);
            tile_store<LOG_L, LAYOUT>(a, data, col0, wA, t);
            __syncthreads();
        }
        return;
    }

    if (LD == LD_U32) {
        uint64_t *work = sm + P_::TW;
        uint32_t *in0 = (uint32_t *)(work + P_::TILE), *in1 = in0 + P_::TILE;
        int cur = 0;
        if (tile < ntiles) tile_load_async<LOG_L, LD_U32, LAYOUT>(a, nullptr, tile * S_::G, in0, t);
        cp_async_commit();
        for (; tile < ntiles; tile += gridDim.x) {
            const long long col0 = tile * S_::G;
            const long long next = tile + gridDim.x;
            if (next < ntiles) tile_load_async<LOG_L, LD_U32, LAYOUT>(a, nullptr, next * S_::G, cur ? in0 : in1, t);
            cp_async_commit();
            cp_async_wait<1>();
            __syncthreads();
            tile_compute<PI, LOG_L, DIR, LD_U32, LAYOUT>(a, work, cur ? in1 : in0, nullptr, twm, w64, col0, t);
            tile_store<LOG_L, LAYOUT>(a, data, col0, work, t);
            __syncthreads();
            cur ^= 1;
        }
        cp_async_wait<0>();
        return;
    }

    uint64_t *buf0 = sm + P_::TW, *buf1 = buf0 + P_::TILE;
    int cur = 0;
    if (tile < ntiles) tile_load_async<LOG_L, LD_U64, LAYOUT>(a, data, tile * S_::G, buf0, t);
    cp_async_commit();
    for (; tile < ntiles; tile += gridDim.x) {
        const long long col0 = tile * S_::G;
        const long long next = tile + gridDim.x;
        if (next < ntiles) tile_load_async<LOG_L, LD_U64, LAYOUT>(a, data, next * S_::G, cur ? buf0 : buf1, t);
        cp_async_commit();
        cp_async_wait<1>();
        __syncthreads();
        uint64_t *w = cur ? buf1 : buf0;
        tile_compute<PI, LOG_L, DIR, LD_U64, LAYOUT>(a, w, nullptr, nullptr, twm, w64, col0, t);
        tile_store<LOG_L, LAYOUT>(a, data, col0, w, t);
        __syncthreads();
        cur ^= 1;
    }
    cp_async_wait<0>();
}

template <int PI, int LOG_L, int DIR, int LD, int LAYOUT>
__global__ void __launch_bounds__(kPassThreads, GBNTT_PASS_MIN_BLOCKS) ntt_pass_kernel(PassArgs a)
{
    extern __shared__ uint64_t sm[];
    pass_persistent<PI, LOG_L, DIR, LD, LAYOUT>(a, sm, a.w64);
}

// Launcher for one prime (explicitly instantiated, one translation unit per
// prime so the three are compiled in parallel).
template <int PI, int LOG_L>
static cudaError_t launch_pass_l(int dir, int ld, const PassArgs &a, cudaStream_t st)
{
    using S_ = PassShape<LOG_L>;
    const int layout = a.log_s == 0 ? LAYOUT_CONTIG : LAYOUT_STRIDED;
    void (*fn)(PassArgs) = nullptr;
    if (dir == 0) {
        if (ld == LD_U32)
            fn = layout == LAYOUT_STRIDED ? ntt_pass_kernel<PI, LOG_L, 0, LD_U32, LAYOUT_STRIDED>
                                          : ntt_pass_kernel<PI, LOG_L, 0, LD_U32, LAYOUT_CONTIG>;
        else
            fn = layout == LAYOUT_STRIDED ? ntt_pass_kernel<PI, LOG_L, 0, LD_U64, LAYOUT_STRIDED>
                                          : ntt_pass_kernel<PI, LOG_L, 0, LD_U64, LAYOUT_CONTIG>;
    } else {
        // the pointwise pass is always the innermost (contiguous) one and the
        // other inverse passes are strided
        if (ld == LD_PW && layout == LAYOUT_CONTIG) fn = ntt_pass_kernel<PI, LOG_L, 1, LD_PW, LAYOUT_CONTIG>;
        else if (ld == LD_U64 && layout == LAYOUT_STRIDED) fn = ntt_pass_kernel<PI, LOG_L, 1, LD_U64, LAYOUT_STRIDED>;
    }
    if (!fn) return cudaErrorInvalidValue;
    size_t smem = 0;
    if (ld == LD_U32) smem = PassSmem<LOG_L, LD_U32>::BYTES;
    else if (ld == LD_PW) smem = PassSmem<LOG_L, LD_PW>::BYTES;
    else smem = PassSmem<LOG_L, LD_U64>::BYTES;
    // per-kernel one-time setup: shared-memory limit and resident CTAs per SM
    struct Slot { void (*fn)(PassArgs); int per_sm; };
    static Slot cache[8] = {};
    int per_sm = 0;
    for (auto &c : cache) {
        if (c.fn == fn) { per_sm = c.per_sm; break; }
    }
    if (per_sm == 0) {
        cudaError_t e = cudaFuncSetAttribute((const void *)fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return e;
        e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, kPassThreads, smem);
        if (e != cudaSuccess) return e;
        if (per_sm < 1) return cudaErrorInvalidConfiguration;
        for (auto &c : cache) {
            if (!c.fn) { c.fn = fn; c.per_sm = per_sm; break; }
        }
    }
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const long long ntiles = (a.ncols + S_::G - 1) / S_::G;
    const long long cap = (long long)sms * per_sm;
    const long long gx = ntiles < cap ? ntiles : cap;
    fn<<<(unsigned)gx, kPassThreads, smem, st>>>(a);
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
