// gbntt_e.cu — e to D decimal digits, every large product on the GPU engine.
//
// The reference application (ntt/app/compute_e/main.c:150-345) computes
//   K   = split_terms_needed(D + 20)                (binary_split.c:96-108)
//   P,B = binary_split(1, K + 1)                    (binary_split.c:26-86)
//   R   = floor((B + P) * 10^(D+20) / B)            (main.c:262-296, newton.c)
// and prints the first D decimal digits of R as "2.718..." (main.c:340-345,
// base_convert.c). Since floor(floor(x) / 10^21) = floor(x / 10^21), those
// digits are exactly the decimal digits of Q = floor((B + P) 10^(D-1) / B),
// which is what this file computes, with the reference's K.
//
// GB300 design. All integers stay in HBM as 32-bit limbs; the host only
// plans, launches and reads lengths and flags.
//  * Product tree: leaf groups of up to 64 consecutive terms are folded by
//    one thread each (P = P k + 1, B = B k) and the first five levels of 32
//    groups merged in shared memory by one CTA (bs_block_kernel); above
//    that the tree is merged level by level, each level's 2 m products
//    (B_L B_R and P_L B_R) going to the engine as ONE batch
//    (gbntt_batch_mul_u32: waves of equal-length transforms), P_L B_R + P_R
//    as one batched add kernel.
//    Any tree shape gives the same P and B: P / B = sum_{k=a}^{b-1}
//    (a-1)!/k! with B = (b-1)!/(a-1)!.
//  * 10^(D-1) = 5^(D-1) 2^(D-1): 5^(D-1) by GPU squarings; the power of two
//    is a bit shift (extract_kernel).
//  * Division (reference newton.c): reciprocal Y = floor(beta^2k / T) of the
//    normalised divisor by Newton iteration with precision doubling (two
//    GPU products per step, from an exact host division at 64 limbs), made
//    exact by a bounded correction; the quotient estimate multiplies only
//    the dividend's top limbs by Y and is at most three below, fixed by
//    conditional subtracts (add/subtract kernel with decoupled look-back
//    carry); remainders come from cyclic products where those are shorter.
//  * Decimal conversion (reference base_convert.c, divide and conquer on
//    powers of ten): pieces are split by d_j = 10^(9 2^j) level by level; a
//    level's pieces are divided together (batched products against one
//    reciprocal, each level's derived from the level above's) and leading
//    pieces known to be zero are skipped, down to pieces of 9 2^12 digits;
//    below that one CTA per piece finishes the splits in shared memory and
//    prints the digits (dec_block_kernel).
#include <cuda_runtime.h>
#include <math.h>
#include <stdarg.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <algorithm>
#include <chrono>
#include <mutex>
#include <vector>

#include "gbntt.h"
#include "gbntt_bn.h"
#include "gbntt_carry.cuh"
#include "gbntt_internal.h"

namespace gbntt {

constexpr unsigned ERR_E_OVERFLOW = 4u;   // conditional increment ran off the top
constexpr unsigned ERR_E_WRAP = 16u;      // a cyclic remainder out of its bound

// ---------------------------------------------------------------------------
// Device kernels
// ---------------------------------------------------------------------------

// out = x + y or x - y (mod beta^nout) for a batch of items (the launch
// picks one, or an item's sel word on the device). Limb i of the operands
// reads as 0 at or beyond nx / ny. Subtraction adds the complement
// of y plus one, so the carry out of the top limb is 1 exactly when x >= y;
// that carry is stored in *flag. In-place use (out == x or out == y) is safe:
// a limb is read and written by the same thread.
struct AddItem {
    const uint32_t *x, *y;
    uint32_t *out;
    unsigned *flag;
    long long nx, ny, nout;
    long long tile_start;
    const uint32_t *sel = nullptr;   // when set: subtract iff (*sel != 0) == sub_if_nonzero (else the launch's mode)
    int sub_if_nonzero = 1;
};

constexpr int kAddThreads = 256, kAddPer = 8, kAddTile = kAddThreads * kAddPer;

__global__ void __launch_bounds__(kAddThreads)
    addsub_kernel(const AddItem *items, int nitems, int sub, unsigned *ticket, unsigned *status, unsigned *error)
{
    constexpr int T = kAddThreads, K = kAddPer;
    __shared__ unsigned s_warp[T / 32];
    __shared__ long long s_t;
    __shared__ int s_item;
    __shared__ unsigned s_cin;
    const int tid = threadIdx.x;
    if (tid == 0) {
        const long long t = atomicAdd(ticket, 1u);
        int lo = 0, hi = nitems;
        while (hi - lo > 1) {
            const int mid = (lo + hi) >> 1;
            if (items[mid].tile_start <= t) lo = mid; else hi = mid;
        }
        s_t = t;
        s_item = lo;
    }
    __syncthreads();
    const AddItem it = items[s_item];
    if (it.sel) sub = ((*it.sel != 0u) ? 1 : 0) == it.sub_if_nonzero;
    const long long tile = s_t - it.tile_start;
    const long long base = tile * kAddTile + (long long)tid * K;
    uint64_t s[K];
#pragma unroll
    for (int k = 0; k < K; k++) {
        const long long pos = base + k;
        uint64_t v = 0;
        if (pos < it.nout) {
            const uint32_t xv = pos < it.nx ? it.x[pos] : 0u;
            uint32_t yv = pos < it.ny ? it.y[pos] : 0u;
            if (sub) yv = ~yv;
            v = (uint64_t)xv + yv + ((sub && pos == 0) ? 1u : 0u);
        }
        s[k] = v;
    }
    unsigned block_agg;
    const unsigned prefix = block_scan_transfer<T>(run_transfer<K>(s), s_warp, &block_agg);
    unsigned err = 0;
    if (tid == 0) s_cin = lookback_carry(status + it.tile_start, tile, block_agg, err);
    __syncthreads();
    uint64_t c = fn_apply(prefix, s_cin);
#pragma unroll
    for (int k = 0; k < K; k++) {
        const long long pos = base + k;
        const uint64_t v = s[k] + c;
        c = v >> 32;
        if (pos < it.nout) {
            it.out[pos] = (uint32_t)v;
            if (pos == it.nout - 1 && it.flag) *it.flag = (unsigned)c;
        }
    }
    if (err) atomicOr(error, err);
}

// out limb i = bits [off + 32 i, off + 32 i + 32) of x (bits outside
// [0, 32 nx) read as 0), for i < nout: shifts, truncations, zero-padded
// copies. An item with a condition word runs only when it is nonzero. out
// must not overlap x unless off == 0.
struct ExtractItem {
    const uint32_t *x;
    uint32_t *out;
    const unsigned *cond;
    long long nx, nout, off;
    long long blk_start;
};

constexpr int kExtThreads = 256, kExtPer = 4, kExtBlock = kExtThreads * kExtPer;

__global__ void __launch_bounds__(kExtThreads) extract_kernel(const ExtractItem *items, int nitems)
{
    __shared__ int s_item;
    if (threadIdx.x == 0) {
        const long long b = blockIdx.x;
        int lo = 0, hi = nitems;
        while (hi - lo > 1) {
            const int mid = (lo + hi) >> 1;
            if (items[mid].blk_start <= b) lo = mid; else hi = mid;
        }
        s_item = lo;
    }
    __syncthreads();
    const ExtractItem it = items[s_item];
    if (it.cond && *it.cond == 0) return;
    const long long i0 = ((long long)blockIdx.x - it.blk_start) * kExtBlock;
#pragma unroll
    for (int r = 0; r < kExtPer; r++) {
        const long long i = i0 + r * kExtThreads + threadIdx.x;
        if (i >= it.nout) continue;
        const long long bit = it.off + 32 * i;
        const long long w = bit >> 5;          // floor division (arithmetic shift)
        const int sh = (int)(bit & 31);
        const uint32_t lo = (w >= 0 && w < it.nx) ? it.x[w] : 0u;
        const uint32_t hi = (w + 1 >= 0 && w + 1 < it.nx) ? it.x[w + 1] : 0u;
        it.out[i] = sh ? ((lo >> sh) | (hi << (32 - sh))) : lo;
    }
}

// Exact limb count (leading zero limbs dropped) of each item.
struct TrimItem {
    const uint32_t *x;
    long long n;
};

__global__ void trim_kernel(const TrimItem *items, int nitems, long long *lens)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nitems) return;
    const uint32_t *x = items[i].x;
    long long n = items[i].n;
    while (n > 0 && x[n - 1] == 0) n--;
    lens[i] = n;
}

// x += 1 (mod beta^n) where *cond is nonzero; running off the top sets an
// error bit.
struct IncItem {
    uint32_t *x;
    const unsigned *cond;
    long long n;
};

__global__ void cond_inc_kernel(const IncItem *items, int nitems, unsigned *error)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nitems) return;
    const IncItem it = items[i];
    if (it.cond && *it.cond == 0) return;
    long long j = 0;
    for (; j < it.n; j++)
        if (++it.x[j] != 0) break;
    if (j == it.n) atomicOr(error, ERR_E_OVERFLOW);
}

// Remainders from cyclic products (Pipe::wrap_remainders). With M = beta^W
// - 1, r = x - P (mod M) is assembled from S1 = x_lo + x_hi (carry f1),
// S2 = P_lo + P_top (carry f2, in place in P) and D = S1 - S2 (f3 = 1 when
// S1 >= S2, no borrow): r == D + e (mod M) with e = f1 - f2 - (1 - f3) in
// -2 .. 1. For a remainder below beta^(W-1), D + e >= 0 (a value in
// [-2, 0) would be congruent to one in [M - 2, M)), and D + e is r itself
// unless it reached M or M + 1, for r = 0 or 1.
struct WrapFix {
    uint32_t *D;
    const unsigned *f;   // f1, f2, f3
    long long W;
};

// D += e, one thread per item (the carry or borrow rarely passes a limb);
// D + 1 = beta^W is stored as 1, D = M stays (the copy reads it as 0).
__global__ void wrap_fix_kernel(const WrapFix *items, int nitems, unsigned *error)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nitems) return;
    const WrapFix it = items[i];
    const int e = (int)it.f[0] - (int)it.f[1] - (1 - (int)it.f[2]);
    if (e > 0) {
        long long j = 0;
        for (; j < it.W; j++)
            if (++it.D[j] != 0) break;
        if (j == it.W) it.D[0] = 1;
    } else if (e < 0) {
        uint32_t b = (uint32_t)(-e);
        for (long long j = 0; j < it.W && b; j++) {
            const uint32_t v = it.D[j];
            it.D[j] = v - b;
            b = v < b ? 1u : 0u;
        }
        if (b) atomicOr(error, ERR_E_WRAP);
    }
}

struct WrapCopy {
    const uint32_t *D;
    uint32_t *r;
    long long W, nr;
    long long tile_start;   // first tile of the item; tiles of kWrapTile limbs cover [0, W)
};
constexpr int kWrapThreads = 256, kWrapTile = 4 * kWrapThreads;

// r = D (0 when D = M, all ones), nr limbs; the limbs of D from nr up must
// be zero.
__global__ void __launch_bounds__(kWrapThreads)
    wrap_copy_kernel(const WrapCopy *items, int nitems, unsigned *error)
{
    int lo = 0, hi = nitems - 1;
    while (lo < hi) {   // the item whose tiles hold this block
        const int mid = (lo + hi + 1) >> 1;
        if (items[mid].tile_start <= (long long)blockIdx.x) lo = mid;
        else hi = mid - 1;
    }
    const WrapCopy it = items[lo];
    const long long j0 = ((long long)blockIdx.x - it.tile_start) * kWrapTile;
    const bool all_ones = it.D[it.W - 1] == 0xffffffffu;
    bool bad = false;
    for (long long j = j0 + threadIdx.x; j < j0 + kWrapTile && j < it.W; j += kWrapThreads) {
        if (j < it.nr) it.r[j] = all_ones ? 0u : it.D[j];
        else bad |= !all_ones && it.D[j] != 0;
    }
    if (bad) atomicOr(error, ERR_E_WRAP);
}

// Leaf groups of the product tree: group i folds the terms
// [a + i G, min(a + (i+1) G, b)) as P <- P k + 1, B <- B k (the reference's
// leaf P = 1, B = a merged term by term, binary_split.c:44-51 and :60-71);
// G is picked so that a group's B stays below 2^(32 (kLeafLimbs - 2)).
constexpr int kLeafLimbs = 64;

// Newton reciprocals of at most this many limbs are computed exactly on the
// host (long division) instead of by further GPU steps.
constexpr size_t kRecipHostLimbs = 64;

// ---------------------------------------------------------------------------
// Decimal conversion of the lower levels in one kernel (dec_block_kernel).
//
// d_j = 10^(9 2^j) has n_j 32-bit limbs; a piece of level j is below d_j^2
// and is stored in 2 n_j + 1 limbs (level -1: 2 limbs). Splitting a level-j
// piece x gives its two level-(j-1) pieces q = floor(x / d_j) (the leading
// digits) and r = x - q d_j. One CTA takes one piece of level `top` and
// splits it level by level down to `low`, all in shared memory, then prints
// the pieces of level low - 1 (9 2^low digits each, one thread per piece).
//
// A split is Barrett's reduction with mu_j = floor(beta^(2n) / d_j) (n + 1
// limbs, beta = 2^32; HAC algorithm 14.42): q^ = floor(floor(x / beta^(n-1))
// mu / beta^(n+1)) satisfies q - 2 <= q^ <= q for x < beta^(2n). The product
// is summed from column n - 1 up only; the columns left out add less than
// beta^(n+1) (a column is below (n + 1) beta^2), so the estimate q' from the
// partial sum is q^ or q^ - 1 and r' = x - q' d_j lies in [0, 4 d_j): it is
// exact modulo beta^(n+1), and at most three subtractions of d_j finish it.
// The products are schoolbook column sums (5 adjacent columns per thread,
// 96-bit accumulators, the d_j or mu_j operand slid through registers); one
// warp per piece then carries the column blocks into limbs, subtracts and
// corrects (warp_resolve, warp_addsub).
// ---------------------------------------------------------------------------
constexpr int kDecThreads = 128;
constexpr int kDecWarps = kDecThreads / 32;
constexpr int kDecCols = 5;          // product columns per thread item; odd, so that the
                                     // lanes' operand reads (stride kDecCols) hit distinct banks
constexpr int kDecPad = kDecCols;    // zero limbs on either side of d_j and mu_j in the table
constexpr int kDecMaxTop = 12;       // highest level whose constants exist
constexpr int kDecLeafLog = 7;       // at most 2^7 = kDecThreads printed pieces per CTA
constexpr unsigned ERR_E_DECIMAL = 8u;   // a split's quotient or correction out of bounds

struct DecLevel {
    int n;             // limbs of d_j
    int stride;        // limbs per stored piece of level j
    int nblk;          // column blocks per piece of the quotient product, ceil((n + 3) / kDecCols)
    long long off_d;   // d_j at ctab + off_d (kDecPad zeros before and after)
    long long off_mu;  // mu_j at ctab + off_mu, n + 1 limbs (padded likewise)
};

struct DecArgs {
    const uint32_t *pieces;   // pieces of level `top`, stride lv[top].stride
    long long first;          // CTA b converts piece first + b
    int top, low;
    int leaf_stride;          // stride of a level low - 1 piece
    int buf_limbs;            // limbs of each of the two piece buffers
    int blk_items;            // column blocks of the largest level (limbs / kDecCols of the block area)
    const uint32_t *ctab;
    DecLevel lv[kDecMaxTop + 1];
    char *digits;             // piece i's 9 2^(top+1) digits at digits + i 9 2^(top+1)
    unsigned *err;
};

// (s0, s1, s2) += x y as one carry chain
__device__ __forceinline__ void dec_mac(uint32_t &s0, uint32_t &s1, uint32_t &s2, uint32_t x, uint32_t y)
{
    asm("mad.lo.cc.u32 %0, %3, %4, %0;\n\t"
        "madc.hi.cc.u32 %1, %3, %4, %1;\n\t"
        "addc.u32 %2, %2, 0;"
        : "+r"(s0), "+r"(s1), "+r"(s2)
        : "r"(x), "r"(y));
}

// Columns c0 .. c0 + kDecCols - 1 of a (na limbs, shared memory) times b (nb
// limbs, zero padded by kDecPad on both sides; global memory when
// B_GLOBAL, else shared): their sum
// sum_k col_k beta^k as kDecCols limbs at L and a two-limb carry at K
// (below beta^2 for na < 2^30).
template <bool B_GLOBAL = true>
__device__ __forceinline__ void dec_colblock(const uint32_t *a, int na, const uint32_t *__restrict__ b, int nb, int c0,
                                             uint32_t *L, uint32_t *K)
{
    uint32_t s0[kDecCols], s1[kDecCols], s2[kDecCols];
#pragma unroll
    for (int k = 0; k < kDecCols; k++) s0[k] = s1[k] = s2[k] = 0;
    const int ihi = min(c0 + kDecCols - 1, na - 1), ilo = max(0, c0 - nb + 1);
    if (ihi >= ilo) {
        uint32_t w[kDecCols];   // w[k] = b[c0 + k - i]
#pragma unroll
        for (int k = 0; k < kDecCols; k++) w[k] = B_GLOBAL ? __ldg(b + (c0 + k - ihi)) : b[c0 + k - ihi];
        for (int i = ihi; i >= ilo; --i) {
            const uint32_t ai = a[i];
#pragma unroll
            for (int k = 0; k < kDecCols; k++) dec_mac(s0[k], s1[k], s2[k], ai, w[k]);
#pragma unroll
            for (int k = 0; k + 1 < kDecCols; k++) w[k] = w[k + 1];
            w[kDecCols - 1] = B_GLOBAL ? __ldg(b + (c0 + kDecCols - i)) : b[c0 + kDecCols - i];
        }
    }
    uint64_t cy = 0;   // carry into the current column, below 2^64
#pragma unroll
    for (int k = 0; k < kDecCols; k++) {
        // v = col_k + cy < 2^96; limb = low word, carry = v >> 32
        const uint64_t lo = (uint64_t)s0[k] + (uint32_t)cy;
        const uint64_t hi = ((uint64_t)s2[k] << 32 | s1[k]) + (cy >> 32) + (lo >> 32);
        L[k] = (uint32_t)lo;
        cy = hi;
    }
    K[0] = (uint32_t)cy;
    K[1] = (uint32_t)(cy >> 32);
}

// Warp-wide carry propagation. Lane i of a chunk owns one block of limbs;
// with G = lanes whose block generates a carry (with no carry in) and X = G
// or lanes whose block passes a carry on (all ones, or all zeros for a
// borrow), the carries into the lanes are (X + G) ^ X ^ G: the carry chain
// of the sum X + G is exactly "generate, or propagate a carry from below".
// A carry into the chunk enters as a generating lane below lane 0.
// Returns the carries into lanes 0 .. 31 (bits 1 .. 32) and out of the
// chunk's lane `last` (bit last + 2).
__device__ __forceinline__ uint64_t warp_carries(bool g, bool p, uint32_t cin)
{
    const uint64_t G = (uint64_t)__ballot_sync(0xffffffffu, g) << 1 | cin;
    const uint64_t X = (uint64_t)__ballot_sync(0xffffffffu, g || p) << 1 | cin;
    return (X + G) ^ X ^ G;
}

// Carry a product's column blocks into limbs, in place (one warp): block t
// holds kDecCols limbs at L + t kDecCols and a carry below beta^2 into block
// t + 1 at K + 2 t. Returns the carry out of the last block (its K plus the
// propagated bit).
__device__ __forceinline__ uint64_t warp_resolve(uint32_t *L, const uint32_t *K, int nblk, int lane)
{
    uint64_t cin = 0;   // into the chunk's first block
    for (int b0 = 0; b0 < nblk; b0 += 32) {
        const int b = b0 + lane, last = min(31, nblk - 1 - b0);
        const bool act = b < nblk;
        uint32_t v[kDecCols];
        bool g = false, p = false;
        if (act) {
            uint64_t c = lane ? ((uint64_t)K[2 * (b - 1) + 1] << 32 | K[2 * (b - 1)]) : cin;
            p = true;
#pragma unroll
            for (int k = 0; k < kDecCols; k++) {   // L_b + K_(b-1): a carry of 0 or 1 leaves the block
                const uint64_t s = (uint64_t)L[b * kDecCols + k] + (uint32_t)c;
                v[k] = (uint32_t)s;
                c = (c >> 32) + (s >> 32);
                p = p && v[k] == 0xffffffffu;
            }
            g = c != 0;
        }
        const uint64_t cv = warp_carries(g, p, 0);
        if (act) {
            uint32_t c = (uint32_t)(cv >> (lane + 1)) & 1u;
#pragma unroll
            for (int k = 0; k < kDecCols; k++) {
                const uint64_t s = (uint64_t)v[k] + c;
                L[b * kDecCols + k] = (uint32_t)s;
                c = (uint32_t)(s >> 32);
            }
        }
        const int bl = b0 + last;
        cin = ((uint64_t)K[2 * bl + 1] << 32 | K[2 * bl]) + ((cv >> (last + 2)) & 1);
    }
    return cin;
}

// dst[0 .. n) = x + y or x - y modulo beta^n (one warp), x and y read as 0 at
// or beyond nx, ny; lane i of a chunk owns limbs i kDecCols .. + kDecCols.
// In-place use (dst == x or dst == y) is safe. Returns the carry (borrow)
// out of limb n - 1.
__device__ __forceinline__ uint32_t warp_addsub(uint32_t *dst, const uint32_t *x, int nx, const uint32_t *y, int ny,
                                                int n, bool sub, int lane)
{
    uint32_t cin = 0;
    for (int i0 = 0; i0 < n; i0 += 32 * kDecCols) {
        const int i = i0 + lane * kDecCols, last = min(31, (n - 1 - i0) / kDecCols);
        uint32_t v[kDecCols];
        bool g = false, p = i < n;
        uint32_t c = 0;
#pragma unroll
        for (int k = 0; k < kDecCols; k++) {
            const int j = i + k;
            if (j < n) {
                const uint32_t a = j < nx ? x[j] : 0u, e = j < ny ? y[j] : 0u;
                const uint64_t s = sub ? (uint64_t)a - e - c : (uint64_t)a + e + c;
                v[k] = (uint32_t)s;
                c = sub ? (uint32_t)(s >> 63) : (uint32_t)(s >> 32);
                p = p && v[k] == (sub ? 0u : 0xffffffffu);
            }
        }
        g = c != 0;
        const uint64_t cv = warp_carries(g, p, cin);
        c = (uint32_t)(cv >> (lane + 1)) & 1u;
#pragma unroll
        for (int k = 0; k < kDecCols; k++) {
            const int j = i + k;
            if (j < n) {
                const uint64_t s = sub ? (uint64_t)v[k] - c : (uint64_t)v[k] + c;
                dst[j] = (uint32_t)s;
                c = sub ? (uint32_t)(s >> 63) : (uint32_t)(s >> 32);
            }
        }
        cin = (uint32_t)(cv >> (last + 2)) & 1u;
    }
    return cin;
}

__global__ void __launch_bounds__(kDecThreads) dec_block_kernel(const DecArgs A)
{
    extern __shared__ uint32_t dsm[];
    uint32_t *cur = dsm, *nxt = dsm + A.buf_limbs;
    uint32_t *BL = dsm + 2 * A.buf_limbs;                 // column block limbs
    uint32_t *BK = BL + (size_t)A.blk_items * kDecCols;   // column block carries
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const long long piece = A.first + blockIdx.x;
    {
        const int S = A.lv[A.top].stride;
        const uint32_t *src = A.pieces + piece * S;
        for (int i = tid; i < S; i += kDecThreads) cur[i] = src[i];
    }
    __syncthreads();
    for (int j = A.top; j >= A.low; j--) {
        const DecLevel lv = A.lv[j];
        const int n = lv.n, S = lv.stride, Sc = j > 0 ? A.lv[j - 1].stride : 2, nb = lv.nblk;
        const int m = 1 << (A.top - j);
        const uint32_t *d = A.ctab + lv.off_d, *mu = A.ctab + lv.off_mu;
        // quotient estimate: columns n - 1 .. of floor(x / beta^(n-1)) mu
        for (int it = tid; it < m * nb; it += kDecThreads) {
            const int p = it / nb, t = it - p * nb;
            dec_colblock(cur + p * S + (n - 1), n + 1, mu, n + 1, n - 1 + t * kDecCols, BL + (size_t)it * kDecCols,
                         BK + 2 * (size_t)it);
        }
        __syncthreads();
        for (int p = warp; p < m; p += kDecWarps) {   // one warp per piece
            uint32_t *L = BL + (size_t)p * nb * kDecCols;
            const uint64_t over = warp_resolve(L, BK + 2 * (size_t)p * nb, nb, lane);
            uint32_t *q = nxt + (2 * p) * Sc;   // limb u of q' is column n + 1 + u
            for (int u = lane; u < Sc; u += 32) q[u] = u < n ? L[u + 2] : 0u;
            if (lane == 0 && (over || L[n + 2])) atomicOr(A.err, ERR_E_DECIMAL);
        }
        __syncthreads();
        // r' = x - q' d_j modulo beta^(n+1): columns 0 .. n of q' d_j
        const int nbr = (n + 1 + kDecCols - 1) / kDecCols;
        for (int it = tid; it < m * nbr; it += kDecThreads) {
            const int p = it / nbr, t = it - p * nbr;
            const int o = p * nb + t;
            dec_colblock(nxt + (2 * p) * Sc, n, d, n, t * kDecCols, BL + (size_t)o * kDecCols, BK + 2 * (size_t)o);
        }
        __syncthreads();
        for (int p = warp; p < m; p += kDecWarps) {
            uint32_t *L = BL + (size_t)p * nb * kDecCols;
            warp_resolve(L, BK + 2 * (size_t)p * nb, nbr, lane);
            const uint32_t *x = cur + p * S;
            uint32_t *r = nxt + (2 * p + 1) * Sc, *q = nxt + (2 * p) * Sc;
            warp_addsub(r, x, n + 1, L, n + 1, n + 1, true, lane);   // r' = x - q' d_j mod beta^(n+1)
            for (int u = n + 1 + lane; u < Sc; u += 32) r[u] = 0;
            __syncwarp();
            int t = 0;
            for (;;) {   // while r' >= d_j: r' -= d_j, q' += 1 (r' - d_j goes to the block area first)
                const uint32_t br = warp_addsub(L, r, n + 1, d, n, n + 1, true, lane);
                if (br) break;
                if (t == 3) {
                    if (lane == 0) atomicOr(A.err, ERR_E_DECIMAL);
                    break;
                }
                __syncwarp();
                for (int u = lane; u <= n; u += 32) r[u] = L[u];
                __syncwarp();
                t++;
            }
            if (t) {
                if (lane == 0) L[0] = (uint32_t)t;
                __syncwarp();
                warp_addsub(q, q, n, L, 1, n, false, lane);
            }
        }
        __syncthreads();
        uint32_t *sw = cur;
        cur = nxt;
        nxt = sw;
    }
    // print the level low - 1 pieces: 9 2^low digits each, by repeated
    // division by 10^9 in place
    const int groups = 1 << A.low, npr = 1 << (A.top - A.low + 1), W = A.leaf_stride;
    char *out = A.digits + piece * (9LL << (A.top + 1));
    for (int p = tid; p < npr; p += kDecThreads) {
        uint32_t *x = cur + p * W;
        int nl = W;
        while (nl > 0 && x[nl - 1] == 0) nl--;
        char *o = out + (long long)p * groups * 9;
        for (int g = groups - 1; g >= 0; g--) {
            uint64_t rem = 0;
            for (int u = nl - 1; u >= 0; u--) {
                const uint64_t c = (rem << 32) | x[u];
                x[u] = (uint32_t)(c / 1000000000u);
                rem = c % 1000000000u;
            }
            while (nl > 0 && x[nl - 1] == 0) nl--;
            uint32_t v = (uint32_t)rem;
            for (int k = 8; k >= 0; k--) {
                o[g * 9 + k] = (char)('0' + v % 10u);
                v /= 10u;
            }
        }
    }
}

// ---------------------------------------------------------------------------
// Product tree bottom in one kernel (bs_block_kernel). CTA c folds the leaf
// groups c 2^t .. c 2^t + 2^t - 1 (G terms each; groups past the end are
// empty: P = 0, B = 1) and merges them t levels up in
// shared memory, P = P_L B_R + P_R, B = B_L B_R (binary_split.c:73-84),
// with schoolbook column blocks (dec_colblock) and one warp per product
// carrying them into limbs (warp_resolve). A node of level l spans G 2^l terms below
// 2^kbits, so B < 2^(kbits G 2^l) and P < 2 B: cap[l] limbs hold either.
// Layout of a level: the P of its nodes, then their B, each node's cap[l]
// limbs preceded by kDecCols zeros, and kDecCols zeros at the end; the
// zeros are the padding dec_colblock reads past an operand.
// ---------------------------------------------------------------------------
constexpr int kBsThreads = 128;
constexpr int kBsMaxLevels = 8;

struct BsArgs {
    unsigned long long a, b;       // terms [a, b)
    int G, t;
    int cap[kBsMaxLevels + 1];     // limbs of a node's P or B at level l
    int region;                    // limbs of one level's node area
    uint32_t *out;                 // node c: P at out + 2 c cap[t], B at out + (2 c + 1) cap[t]
    long long *lens;               // limb counts of P and B of node c at lens[2 c], lens[2 c + 1]
    unsigned *err;
};

__global__ void __launch_bounds__(kBsThreads) bs_block_kernel(const BsArgs A)
{
    extern __shared__ uint32_t bsm[];
    uint32_t *cur = bsm, *nxt = bsm + A.region;
    uint32_t *BK = bsm + 2 * A.region;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5, t = A.t, n0 = 1 << t;
    for (int i = tid; i < A.region; i += kBsThreads) cur[i] = 0;
    __syncthreads();
    {   // leaves: thread 2u folds P of group u, thread 2u + 1 its B
        const int cap = A.cap[0], s0 = cap + kDecCols;
        for (int w = tid; w < 2 * n0; w += kBsThreads) {
            const int u = w >> 1, isB = w & 1;
            uint32_t *x = cur + (isB ? n0 * s0 : 0) + kDecCols + u * s0;
            const unsigned long long lo = A.a + ((unsigned long long)blockIdx.x * n0 + u) * (unsigned long long)A.G;
            const unsigned long long hi = lo + A.G < A.b ? lo + A.G : A.b;
            int n = 0;
            if (isB) x[n++] = 1;
            for (unsigned long long k = lo; k < hi; k++) {
                const uint32_t m = (uint32_t)k;
                uint64_t c = isB ? 0 : 1;
                for (int j = 0; j < n; j++) {
                    c += (uint64_t)x[j] * m;
                    x[j] = (uint32_t)c;
                    c >>= 32;
                }
                if (c) {
                    if (n < cap) x[n++] = (uint32_t)c;
                    else atomicOr(A.err, ERR_E_OVERFLOW);
                }
            }
        }
    }
    __syncthreads();
    for (int l = 1; l <= t; l++) {
        const int N = 1 << (t - l);
        const int cp = A.cap[l - 1], sp = cp + kDecCols, cl = A.cap[l], sl = cl + kDecCols;
        const int nb = (cl + kDecCols - 1) / kDecCols;
        for (int i = tid; i < A.region; i += kBsThreads) nxt[i] = 0;
        __syncthreads();
        const uint32_t *Pp = cur + kDecCols, *Bp = cur + 2 * N * sp + kDecCols;
        uint32_t *Pn = nxt + kDecCols, *Bn = nxt + N * sl + kDecCols;
        // product e of pair v: e = 0 B_L B_R, e = 1 P_L B_R; block t2 of it
        for (int it = tid; it < 2 * N * nb; it += kBsThreads) {
            const int pe = it / nb, t2 = it - pe * nb, v = pe >> 1, e = pe & 1;
            const uint32_t *x = (e ? Pp : Bp) + (2 * v) * sp;
            uint32_t *o = (e ? Pn : Bn) + v * sl;
            dec_colblock<false>(x, cp, Bp + (2 * v + 1) * sp, cp, t2 * kDecCols, o + t2 * kDecCols,
                                BK + 2 * (size_t)it);
        }
        __syncthreads();
        for (int pe = warp; pe < 2 * N; pe += kBsThreads / 32) {   // one warp per product
            const int v = pe >> 1, e = pe & 1;
            uint32_t *o = (e ? Pn : Bn) + v * sl;
            bool bad = warp_resolve(o, BK + 2 * (size_t)pe * nb, nb, lane) != 0;
            if (e) bad |= warp_addsub(o, o, cl, Pp + (2 * v + 1) * sp, cp, cl, false, lane) != 0;   // + P_R
            for (int j = cl + lane; j < nb * kDecCols; j += 32) {   // the overhang is the next node's zero padding
                bad |= o[j] != 0;
                o[j] = 0;
            }
            if (__any_sync(0xffffffffu, bad) && lane == 0) atomicOr(A.err, ERR_E_OVERFLOW);
        }
        __syncthreads();
        uint32_t *sw = cur;
        cur = nxt;
        nxt = sw;
    }
    const int ct = A.cap[t];
    const uint32_t *P = cur + kDecCols, *B = cur + ct + 2 * kDecCols;
    uint32_t *oP = A.out + 2 * (size_t)blockIdx.x * ct, *oB = oP + ct;
    for (int i = tid; i < ct; i += kBsThreads) {
        oP[i] = P[i];
        oB[i] = B[i];
    }
    if (tid < 2) {
        const uint32_t *x = tid ? B : P;
        int n = ct;
        while (n > 0 && x[n - 1] == 0) n--;
        A.lens[2 * (size_t)blockIdx.x + tid] = n;
    }
}

// Batched limb additions for the engine's split products (gbntt_engine.cu):
// out_i = x_i + y_i over n_i limbs each, on stream st; the sums fit in n_i
// limbs (no carry leaves the top). Item table and tile status come from the
// stream-ordered pool. Look-back wait failures set bits in *err.
int batch_add_limbs(const uint32_t *const *x, const uint32_t *const *y, uint32_t *const *out, const long long *n,
                    int count, cudaStream_t st, unsigned *err)
{
    std::vector<AddItem> run;
    run.reserve((size_t)count);
    long long tiles = 0;
    for (int i = 0; i < count; i++) {
        if (n[i] <= 0) continue;
        run.push_back({x[i], y[i], out[i], nullptr, n[i], n[i], n[i], tiles});
        tiles += (n[i] + kAddTile - 1) / kAddTile;
    }
    if (run.empty()) return GBNTT_OK;
    if (tiles > 0x7FFFFFFFLL) return GBNTT_ERR_SIZE;
    void *d = nullptr, *ctl = nullptr;
    if (cudaMallocAsync(&d, run.size() * sizeof(AddItem), st) != cudaSuccess ||
        cudaMallocAsync(&ctl, ((size_t)tiles + 1) * sizeof(unsigned), st) != cudaSuccess) {
        if (d) cudaFreeAsync(d, st);
        (void)cudaGetLastError();
        return GBNTT_ERR_ALLOC;
    }
    cudaError_t e = cudaMemcpyAsync(d, run.data(), run.size() * sizeof(AddItem), cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) e = cudaMemsetAsync(ctl, 0, ((size_t)tiles + 1) * sizeof(unsigned), st);
    if (e == cudaSuccess) {
        addsub_kernel<<<(unsigned)tiles, kAddThreads, 0, st>>>((const AddItem *)d, (int)run.size(), 0, (unsigned *)ctl,
                                                               (unsigned *)ctl + 1, err);
        e = cudaGetLastError();
    }
    cudaFreeAsync(d, st);
    cudaFreeAsync(ctl, st);
    return e == cudaSuccess ? GBNTT_OK : GBNTT_ERR_CUDA;
}

// ---------------------------------------------------------------------------
// Host orchestration
// ---------------------------------------------------------------------------
namespace {

struct Stopwatch {
    std::chrono::steady_clock::time_point t0 = std::chrono::steady_clock::now();
    double lap()
    {
        const auto t = std::chrono::steady_clock::now();
        const double s = std::chrono::duration<double>(t - t0).count();
        t0 = t;
        return s;
    }
};

struct EFail {
    int code;
};

[[noreturn]] void efail(int code, const char *fmt, ...)
{
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    set_error_message(buf);
    throw EFail{code};
}

#define ECK(expr)                                                                                            \
    do {                                                                                                     \
        cudaError_t _e = (expr);                                                                             \
        if (_e != cudaSuccess)                                                                               \
            efail(GBNTT_ERR_CUDA, "CUDA error %d (%s) at %s:%d: %s", (int)_e, cudaGetErrorString(_e), __FILE__, \
                  __LINE__, #expr);                                                                          \
    } while (0)

#define ERC(expr)                                                                                            \
    do {                                                                                                     \
        const int _r = (expr);                                                                               \
        if (_r != GBNTT_OK) efail(_r, "%s", gbntt_last_error());                                             \
    } while (0)

cudaStream_t g_st = nullptr;   // stream of the running pipeline call

// Device limb buffer, stream-ordered allocation on g_st.
struct DBuf {
    uint32_t *p = nullptr;
    size_t cap = 0;
    DBuf() = default;
    explicit DBuf(size_t n) { alloc(n); }
    DBuf(const DBuf &) = delete;
    DBuf &operator=(const DBuf &) = delete;
    DBuf(DBuf &&o) noexcept : p(o.p), cap(o.cap) { o.p = nullptr; o.cap = 0; }
    DBuf &operator=(DBuf &&o) noexcept
    {
        if (this != &o) {
            release();
            p = o.p;
            cap = o.cap;
            o.p = nullptr;
            o.cap = 0;
        }
        return *this;
    }
    ~DBuf() { release(); }
    void alloc(size_t n)
    {
        release();
        void *q = nullptr;
        ECK(cudaMallocAsync(&q, std::max<size_t>(n, 1) * sizeof(uint32_t), g_st));
        p = (uint32_t *)q;
        cap = n;
    }
    void release()
    {
        if (p) cudaFreeAsync(p, g_st);
        p = nullptr;
        cap = 0;
    }
};

// Host vector mirrored to a stream-ordered device array (upload on creation).
template <class T>
struct DTab {
    T *p = nullptr;
    explicit DTab(const std::vector<T> &v)
    {
        void *q = nullptr;
        ECK(cudaMallocAsync(&q, std::max<size_t>(v.size(), 1) * sizeof(T), g_st));
        p = (T *)q;
        if (!v.empty()) ECK(cudaMemcpyAsync(p, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice, g_st));
    }
    explicit DTab(size_t n)
    {
        void *q = nullptr;
        ECK(cudaMallocAsync(&q, std::max<size_t>(n, 1) * sizeof(T), g_st));
        p = (T *)q;
    }
    DTab(const DTab &) = delete;
    DTab &operator=(const DTab &) = delete;
    ~DTab()
    {
        if (p) cudaFreeAsync(p, g_st);
    }
};

// d_j = 10^(9 2^j) and mu_j = floor(beta^(2 n_j) / d_j) for j = 0 ..
// kDecMaxTop, laid out for dec_block_kernel. They depend on nothing but j:
// computed once per process on the host (long division, checked by
// multiplication), uploaded per call.
struct DecConst {
    std::vector<uint32_t> tab;
    DecLevel lv[kDecMaxTop + 1];
    bn::Num d[kDecMaxTop + 1];
};

const DecConst &dec_constants()
{
    static DecConst C;
    static std::once_flag once;
    std::call_once(once, [] {
        bn::Num d = bn::from_u64(1000000000u);
        for (int j = 0; j <= kDecMaxTop; j++) {
            if (j) d = bn::mul_school(d, d);
            const size_t n = d.size();
            bn::Num b(2 * n + 1, 0);
            b[2 * n] = 1;
            const bn::Num mu = bn::div_floor(b, d);
            const bn::Num lo = bn::mul_school(mu, d), hi = bn::add(lo, d);
            if (mu.size() != n + 1 || bn::cmp(lo, b) > 0 || bn::cmp(hi, b) <= 0) {
                fprintf(stderr, "gbntt: reciprocal of 10^(9 2^%d) failed its check\n", j);
                abort();
            }
            DecLevel &L = C.lv[j];
            L.n = (int)n;
            L.stride = (int)(2 * n + 1);
            L.nblk = (int)((n + 3 + kDecCols - 1) / kDecCols);
            C.tab.insert(C.tab.end(), kDecPad, 0u);
            L.off_d = (long long)C.tab.size();
            C.tab.insert(C.tab.end(), d.begin(), d.end());
            C.tab.insert(C.tab.end(), 2 * kDecPad, 0u);
            L.off_mu = (long long)C.tab.size();
            C.tab.insert(C.tab.end(), mu.begin(), mu.end());
            C.tab.insert(C.tab.end(), kDecPad, 0u);
            C.d[j] = d;
        }
    });
    return C;
}

// Reciprocals of the lower powers of ten from the one above (default), or
// each by its own Newton iteration (GBNTT_E_DERIVE_RECIP=0).
bool derive_reciprocals()
{
    const char *e = getenv("GBNTT_E_DERIVE_RECIP");
    return !e || atoi(e) != 0;
}

// Product tree levels merged inside bs_block_kernel (GBNTT_BS_BLOCK_LEVELS,
// 0 .. kBsMaxLevels).
int bs_block_levels()
{
    const char *e = getenv("GBNTT_BS_BLOCK_LEVELS");
    const int v = e ? atoi(e) : 5;
    return std::max(0, std::min(kBsMaxLevels, v));
}

// The top decimal level's reciprocal only as precise as its quotient needs,
// from the squared reciprocal of the level below (default), or a full-length
// Newton reciprocal (GBNTT_E_SHORT_TOP=0).
bool short_top_reciprocal()
{
    const char *e = getenv("GBNTT_E_SHORT_TOP");
    return !e || atoi(e) != 0;
}

// Division remainders from cyclic products where their transform is shorter
// (default), or always from full products (GBNTT_E_WRAP=0).
bool wrap_remainders_enabled()
{
    const char *e = getenv("GBNTT_E_WRAP");
    return !e || atoi(e) != 0;
}

// Highest level dec_block_kernel takes (GBNTT_DEC_TOP, 0 .. kDecMaxTop).
int dec_top_level()
{
    const char *e = getenv("GBNTT_DEC_TOP");
    const int v = e ? atoi(e) : 11;
    return std::max(0, std::min(kDecMaxTop, v));
}

struct Pipe {
    unsigned *d_err = nullptr;   // sticky device error bits of this call

    Pipe()
    {
        void *q = nullptr;
        ECK(cudaMallocAsync(&q, sizeof(unsigned), g_st));
        d_err = (unsigned *)q;
        ECK(cudaMemsetAsync(d_err, 0, sizeof(unsigned), g_st));
    }
    ~Pipe()
    {
        if (d_err) cudaFreeAsync(d_err, g_st);
    }

    void sync() { ECK(cudaStreamSynchronize(g_st)); }

    void check_errors()
    {
        unsigned e = 0;
        ECK(cudaMemcpyAsync(&e, d_err, sizeof e, cudaMemcpyDeviceToHost, g_st));
        sync();
        if (e) efail(GBNTT_ERR_DEVICE, "e pipeline device check failed (flags 0x%x)", e);
    }

    uint32_t read_limb(const uint32_t *p)
    {
        uint32_t v = 0;
        ECK(cudaMemcpyAsync(&v, p, sizeof v, cudaMemcpyDeviceToHost, g_st));
        sync();
        return v;
    }

    // exact limb count of p[0 .. n)
    size_t trim_top(const uint32_t *p, size_t n)
    {
        while (n > 0 && read_limb(p + n - 1) == 0) n--;
        return n;
    }

    DBuf upload(const bn::Num &v, size_t n_out)
    {
        DBuf d(n_out);
        ECK(cudaMemsetAsync(d.p, 0, n_out * sizeof(uint32_t), g_st));
        if (!v.empty()) ECK(cudaMemcpyAsync(d.p, v.data(), std::min(v.size(), n_out) * 4, cudaMemcpyHostToDevice, g_st));
        sync();   // v may be a temporary
        return d;
    }

    // ---- kernel wrappers ----
    void addsub(std::vector<AddItem> &items, bool sub)
    {
        std::vector<AddItem> run;
        run.reserve(items.size());
        long long tiles = 0;
        for (auto it : items) {
            if (it.nout <= 0) continue;
            it.tile_start = tiles;
            tiles += (it.nout + kAddTile - 1) / kAddTile;
            run.push_back(it);
        }
        if (run.empty()) return;
        if (tiles > 0x7FFFFFFFLL) efail(GBNTT_ERR_SIZE, "add/subtract batch too large");
        DTab<AddItem> d(run);
        DTab<unsigned> ctl((size_t)tiles + 1);
        ECK(cudaMemsetAsync(ctl.p, 0, ((size_t)tiles + 1) * sizeof(unsigned), g_st));
        addsub_kernel<<<(unsigned)tiles, kAddThreads, 0, g_st>>>(d.p, (int)run.size(), sub ? 1 : 0, ctl.p, ctl.p + 1,
                                                                 d_err);
        ECK(cudaGetLastError());
    }
    void add1(uint32_t *out, size_t nout, const uint32_t *x, size_t nx, const uint32_t *y, size_t ny, bool sub,
              unsigned *flag = nullptr)
    {
        std::vector<AddItem> v{{x, y, out, flag, (long long)nx, (long long)ny, (long long)nout, 0}};
        addsub(v, sub);
    }

    void extract(std::vector<ExtractItem> &items)
    {
        std::vector<ExtractItem> run;
        run.reserve(items.size());
        long long blks = 0;
        for (auto it : items) {
            if (it.nout <= 0) continue;
            it.blk_start = blks;
            blks += (it.nout + kExtBlock - 1) / kExtBlock;
            run.push_back(it);
        }
        if (run.empty()) return;
        if (blks > 0x7FFFFFFFLL) efail(GBNTT_ERR_SIZE, "extract batch too large");
        DTab<ExtractItem> d(run);
        extract_kernel<<<(unsigned)blks, kExtThreads, 0, g_st>>>(d.p, (int)run.size());
        ECK(cudaGetLastError());
    }
    void extract1(uint32_t *out, size_t nout, const uint32_t *x, size_t nx, long long off)
    {
        std::vector<ExtractItem> v{{x, out, nullptr, (long long)nx, (long long)nout, off, 0}};
        extract(v);
    }

    std::vector<long long> trim(const std::vector<TrimItem> &items)
    {
        std::vector<long long> lens(items.size());
        if (items.empty()) return lens;
        DTab<TrimItem> d(items);
        DTab<long long> dl(items.size());
        trim_kernel<<<(unsigned)((items.size() + 255) / 256), 256, 0, g_st>>>(d.p, (int)items.size(), dl.p);
        ECK(cudaGetLastError());
        ECK(cudaMemcpyAsync(lens.data(), dl.p, items.size() * sizeof(long long), cudaMemcpyDeviceToHost, g_st));
        sync();
        return lens;
    }

    void cond_inc(const std::vector<IncItem> &items)
    {
        if (items.empty()) return;
        DTab<IncItem> d(items);
        cond_inc_kernel<<<(unsigned)((items.size() + 255) / 256), 256, 0, g_st>>>(d.p, (int)items.size(), d_err);
        ECK(cudaGetLastError());
    }

    void mul(uint32_t *c, const uint32_t *a, size_t na, const uint32_t *b, size_t nb)
    {
        ERC(gbntt_mul_u32(c, a, na, b, nb, (void *)g_st));
    }

    struct Prod {
        uint32_t *c;
        const uint32_t *a, *b;
        size_t na, nb;
    };
    void batch_mul(const std::vector<Prod> &v)
    {
        if (v.empty()) return;
        std::vector<uint32_t *> c(v.size());
        std::vector<const uint32_t *> a(v.size()), b(v.size());
        std::vector<size_t> na(v.size()), nb(v.size());
        for (size_t i = 0; i < v.size(); i++) {
            c[i] = v[i].c;
            a[i] = v[i].a;
            b[i] = v[i].b;
            na[i] = v[i].na;
            nb[i] = v[i].nb;
        }
        ERC(gbntt_batch_mul_u32(c.data(), a.data(), na.data(), b.data(), nb.data(), (int)v.size(), (void *)g_st));
    }

    // Products with cyclic items (wl[i] > 0: c = a b mod (beta^(2^wl) - 1),
    // 2^wl + 3 limbs, the top 3 unfolded).
    void batch_mul_wrap(const std::vector<Prod> &v, const std::vector<int> &wl)
    {
        if (v.empty()) return;
        std::vector<uint32_t *> c(v.size());
        std::vector<const uint32_t *> a(v.size()), b(v.size());
        std::vector<size_t> na(v.size()), nb(v.size());
        for (size_t i = 0; i < v.size(); i++) {
            c[i] = v[i].c;
            a[i] = v[i].a;
            b[i] = v[i].b;
            na[i] = v[i].na;
            nb[i] = v[i].nb;
        }
        ERC(gbntt::batch_mul_wrap(c.data(), a.data(), na.data(), b.data(), nb.data(), wl.data(), (int)v.size(), g_st));
    }

    // r_i = x_i - P_i (mod beta^W_i - 1) for remainders known to be below
    // beta^(W_i - 1), where P_i (W_i + 3 limbs, overwritten) is a cyclic
    // product; x_i has at most 2 W_i limbs. r_i gets nr_i limbs (nr_i <= W_i;
    // the remainder must fit them).
    struct WrapItem {
        const uint32_t *x;
        size_t nx;
        uint32_t *P;
        size_t W;
        uint32_t *r;
        size_t nr;
    };
    void wrap_remainders(const std::vector<WrapItem> &v)
    {
        const size_t n = v.size();
        if (!n) return;
        size_t tot = 0;
        for (auto &w : v) {
            if (w.nx > 2 * w.W || w.nr > w.W) efail(GBNTT_ERR_ARG, "cyclic remainder operands out of range");
            tot += w.W;
        }
        DBuf S(tot);
        DTab<unsigned> f(3 * n);
        std::vector<AddItem> a1, a2, a3;
        std::vector<WrapFix> fx;
        std::vector<WrapCopy> cp;
        size_t o = 0;
        long long tiles = 0;
        for (size_t i = 0; i < n; i++) {
            const WrapItem &w = v[i];
            const long long W = (long long)w.W;
            uint32_t *s1 = S.p + o;
            a1.push_back({w.x, w.x + std::min(w.nx, w.W), s1, f.p + 3 * i, (long long)std::min(w.nx, w.W),
                          (long long)(w.nx > w.W ? w.nx - w.W : 0), W, 0});
            a2.push_back({w.P, w.P + w.W, w.P, f.p + 3 * i + 1, W, 3, W, 0});
            a3.push_back({s1, w.P, s1, f.p + 3 * i + 2, W, W, W, 0});
            fx.push_back({s1, f.p + 3 * i, W});
            cp.push_back({s1, w.r, W, (long long)w.nr, tiles});
            tiles += (W + kWrapTile - 1) / kWrapTile;
            o += w.W;
        }
        addsub(a1, false);
        addsub(a2, false);
        addsub(a3, true);
        {
            DTab<WrapFix> d(fx);
            wrap_fix_kernel<<<(unsigned)((n + 127) / 128), 128, 0, g_st>>>(d.p, (int)n, d_err);
            ECK(cudaGetLastError());
        }
        if (tiles > 0x7fffffffLL) efail(GBNTT_ERR_SIZE, "cyclic remainders too long");
        DTab<WrapCopy> d(cp);
        wrap_copy_kernel<<<(unsigned)tiles, kWrapThreads, 0, g_st>>>(d.p, (int)n, d_err);
        ECK(cudaGetLastError());
    }

    // ---- binary splitting (reference binary_split.c) ----
    // P and B of [a, b) on the device, exact limb counts.
    void binary_split(unsigned long long a, unsigned long long b, DBuf &P, size_t &nP, DBuf &B, size_t &nB)
    {
        if (b <= a) {   // empty range: P = 0, B = 1 (binary_split.c:37-43)
            P = upload(bn::Num(), 1);
            nP = 0;
            B = upload(bn::from_u64(1), 1);
            nB = 1;
            return;
        }
        if (b - 1 > 0xFFFFFFFFull) efail(GBNTT_ERR_ARG, "binary_split: terms must stay below 2^32");
        const int kbits = 64 - __builtin_clzll(b - 1);
        const int G = std::max(1, std::min(64, (kLeafLimbs - 2) * 32 / kbits));
        const long long nleaf = (long long)((b - a + G - 1) / G);
        // the first t levels in shared memory (bs_block_kernel), 2^t groups per CTA
        int t = 0;
        while (t < bs_block_levels() && (1LL << t) < nleaf) t++;
        BsArgs ba{};
        ba.a = a;
        ba.b = b;
        ba.G = G;
        ba.t = t;
        long long region = 0, items = 0;
        for (int l = 0; l <= t; l++) {
            ba.cap[l] = (int)(((long long)kbits * G << l) / 32 + 3) | 1;   // >= 2 spare limbs, odd node stride
            const long long nodes = 1LL << (t - l), sl = ba.cap[l] + kDecCols;
            region = std::max(region, 2 * nodes * sl + kDecCols);
            if (l) items = std::max(items, 2 * nodes * ((ba.cap[l] + kDecCols - 1) / kDecCols));
        }
        ba.region = (int)region;
        const size_t smem = (size_t)(2 * region + 2 * items) * sizeof(uint32_t);
        if (smem > 48 * 1024) {
            int dev = 0, cap = 0;
            ECK(cudaGetDevice(&dev));
            ECK(cudaDeviceGetAttribute(&cap, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
            if (smem > (size_t)cap) efail(GBNTT_ERR_SIZE, "product tree block needs %zu bytes of shared memory", smem);
            ECK(cudaFuncSetAttribute(bs_block_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        }
        const long long ncta = (nleaf + (1LL << t) - 1) >> t;
        const size_t ct = (size_t)ba.cap[t];
        DBuf lev((size_t)ncta * 2 * ct);
        std::vector<long long> lens((size_t)ncta * 2);
        {
            Stopwatch sw;
            DTab<long long> dl((size_t)ncta * 2);
            ba.out = lev.p;
            ba.lens = dl.p;
            ba.err = d_err;
            bs_block_kernel<<<(unsigned)ncta, kBsThreads, smem, g_st>>>(ba);
            ECK(cudaGetLastError());
            ECK(cudaMemcpyAsync(lens.data(), dl.p, lens.size() * sizeof(long long), cudaMemcpyDeviceToHost, g_st));
            sync();
            if (getenv("GBNTT_E_PROFILE"))
                fprintf(stderr, "binary_split leaves and levels 1..%d in one kernel: %lld CTAs, %zu bytes shared, "
                        "%.2f ms\n", t, ncta, smem, sw.lap() * 1e3);
        }
        struct Node {
            uint32_t *P, *B;
            size_t nP, nB;
        };
        std::vector<Node> nodes((size_t)ncta);
        for (long long i = 0; i < ncta; i++)
            nodes[i] = {lev.p + 2 * i * ct, lev.p + (2 * i + 1) * ct, (size_t)lens[2 * i], (size_t)lens[2 * i + 1]};
        const bool prof = getenv("GBNTT_E_PROFILE") != nullptr;
        int level = 0;
        while (nodes.size() > 1) {
            Stopwatch sw;
            const size_t m = nodes.size() / 2;
            const bool odd = nodes.size() & 1;
            std::vector<size_t> capB(m), capP(m);
            size_t total = 0;
            for (size_t i = 0; i < m; i++) {
                const Node &L = nodes[2 * i], &R = nodes[2 * i + 1];
                capB[i] = L.nB + R.nB;
                capP[i] = std::max(L.nP + R.nB, R.nP) + 1;
                total += capB[i] + capP[i];
            }
            if (odd) total += nodes.back().nP + nodes.back().nB;
            DBuf next(total);
            std::vector<Node> out(m + (odd ? 1 : 0));
            std::vector<Prod> prods;
            prods.reserve(2 * m);
            std::vector<AddItem> adds;
            adds.reserve(m);
            size_t off = 0;
            for (size_t i = 0; i < m; i++) {
                const Node &L = nodes[2 * i], &R = nodes[2 * i + 1];
                Node &o = out[i];
                o.B = next.p + off;
                off += capB[i];
                o.P = next.p + off;
                off += capP[i];
                o.nB = capB[i];
                o.nP = capP[i];
                prods.push_back({o.B, L.B, R.B, L.nB, R.nB});   // B = B_L B_R
                prods.push_back({o.P, L.P, R.B, L.nP, R.nB});   // P_L B_R
            }
            batch_mul(prods);
            for (size_t i = 0; i < m; i++) {   // P = P_L B_R + P_R (in place)
                const Node &L = nodes[2 * i], &R = nodes[2 * i + 1];
                adds.push_back({out[i].P, R.P, out[i].P, nullptr, (long long)(L.nP + R.nB), (long long)R.nP,
                                (long long)capP[i], 0});
            }
            addsub(adds, false);
            if (odd) {   // the last node moves up unchanged
                const Node &L = nodes.back();
                Node &o = out[m];
                o.P = next.p + off;
                o.B = o.P + L.nP;
                o.nP = L.nP;
                o.nB = L.nB;
                std::vector<ExtractItem> cp{{L.P, o.P, nullptr, (long long)L.nP, (long long)L.nP, 0, 0},
                                            {L.B, o.B, nullptr, (long long)L.nB, (long long)L.nB, 0, 0}};
                extract(cp);
            }
            std::vector<TrimItem> tr;
            tr.reserve(2 * out.size());
            for (auto &o : out) {
                tr.push_back({o.P, (long long)o.nP});
                tr.push_back({o.B, (long long)o.nB});
            }
            const std::vector<long long> nl = trim(tr);
            for (size_t i = 0; i < out.size(); i++) {
                out[i].nP = (size_t)nl[2 * i];
                out[i].nB = (size_t)nl[2 * i + 1];
            }
            nodes.swap(out);
            lev = std::move(next);
            if (prof) {
                sync();
                fprintf(stderr, "binary_split level %d: %zu products, B limbs %zu, %.2f ms\n", t + ++level, 2 * m,
                        nodes[0].nB, sw.lap() * 1e3);
            }
        }
        const Node &r = nodes[0];
        nP = r.nP;
        nB = r.nB;
        P.alloc(std::max<size_t>(nP, 1));
        B.alloc(std::max<size_t>(nB, 1));
        std::vector<ExtractItem> cp{{r.P, P.p, nullptr, (long long)r.nP, (long long)r.nP, 0, 0},
                                    {r.B, B.p, nullptr, (long long)r.nB, (long long)r.nB, 0, 0}};
        extract(cp);
    }

    // ---- reciprocal (reference newton.c) ----
    // Y ~ floor(beta^(2k) / T), within a few units, for T of k limbs with the
    // top bit set; k + 1 limbs. Newton step from h = k/2 + 1 limbs:
    //   U = T Yh, E = |beta^(k+h) - U| (< 6 beta^k), Y = Yh beta^(k-h) +- floor(Yh E / beta^(2h)).
    DBuf recip_approx(const uint32_t *T, size_t k)
    {
        if (k <= kRecipHostLimbs) {   // exact on the host: floor(beta^(2k) / T)
            bn::Num t(k), b(2 * k + 1, 0);
            ECK(cudaMemcpyAsync(t.data(), T, k * sizeof(uint32_t), cudaMemcpyDeviceToHost, g_st));
            sync();
            bn::trim(t);
            if (t.empty()) efail(GBNTT_ERR_ARG, "reciprocal of zero");
            b[2 * k] = 1;
            return upload(bn::div_floor(b, t), k + 1);
        }
        const size_t h = k / 2 + 1;
        DBuf Yh = recip_approx(T + (k - h), h);
        DBuf U(k + h + 1);
        mul(U.p, T, k, Yh.p, h + 1);
        // U >= beta^(k+h) exactly when its top limb is set; the sign picks
        // on the device between E = U - beta^(k+h) = U mod beta^(k+1) and
        // E = beta^(k+h) - U = -U mod beta^(k+1) (both below 6 beta^k)
        const uint32_t *neg = U.p + k + h;
        DBuf E(k + 1);
        {
            std::vector<AddItem> v{{nullptr, U.p, E.p, nullptr, 0, (long long)k + 1, (long long)k + 1, 0, neg, 0}};
            addsub(v, true);
        }
        DBuf M(k + h + 2);
        mul(M.p, Yh.p, h + 1, E.p, k + 1);
        E.release();
        DBuf Y(k + 1);
        extract1(Y.p, k + 1, Yh.p, h + 1, -32LL * (long long)(k - h));   // Yh beta^(k-h)
        {   // Y -+ floor(Yh E / beta^(2h)): subtract when U was above beta^(k+h)
            std::vector<AddItem> v{{Y.p, M.p + 2 * h, Y.p, nullptr, (long long)k + 1, (long long)(k + 2 - h),
                                    (long long)k + 1, 0, neg, 1}};
            addsub(v, false);
        }
        return Y;
    }

    // Exact floor(beta^(2k) / T): start below it, then add T back while the
    // remainder allows (bounded), and check the remainder is below T.
    DBuf recip_exact(const uint32_t *T, size_t k)
    {
        DBuf Y = recip_approx(T, k);
        const bn::Num eight = bn::from_u64(8);
        DBuf c8 = upload(eight, 1);
        add1(Y.p, k + 1, Y.p, k + 1, c8.p, 1, true);                 // Y -= 8
        DBuf R(k + 1), t(k + 1);
        int lw = kMinLog, ll = kMinLog;
        while (((size_t)1 << lw) < k + 2) lw++;
        while (((size_t)1 << ll) < 2 * k) ll++;
        if (wrap_remainders_enabled() && lw < ll) {
            // beta^(2k) - Y T < 16 T < beta^(W-1) from the cyclic product
            // Y T mod (beta^W - 1), with beta^(2k) == beta^(2k - W)
            const size_t W = (size_t)1 << lw;
            DBuf Z(W + 3), X(W);
            batch_mul_wrap({{Z.p, Y.p, T, k + 1, k}}, {lw});
            ECK(cudaMemsetAsync(X.p, 0, W * sizeof(uint32_t), g_st));
            static const uint32_t one = 1;
            ECK(cudaMemcpyAsync(X.p + (2 * k >= W ? 2 * k - W : 2 * k), &one, sizeof one, cudaMemcpyHostToDevice,
                                g_st));
            wrap_remainders({{X.p, W, Z.p, W, R.p, k + 1}});
        } else {
            DBuf Z(2 * k + 1);
            mul(Z.p, Y.p, k + 1, T, k);
            add1(R.p, k + 1, nullptr, 0, Z.p, k + 1, true);           // beta^(2k) - Z < 16 T
        }
        DTab<unsigned> flag(1);
        for (int it = 0; it < 16; it++) {
            add1(t.p, k + 1, R.p, k + 1, T, k, true, flag.p);         // flag: R >= T
            std::vector<ExtractItem> cp{{t.p, R.p, flag.p, (long long)k + 1, (long long)k + 1, 0, 0}};
            extract(cp);
            cond_inc({{Y.p, flag.p, (long long)k + 1}});
        }
        add1(t.p, k + 1, R.p, k + 1, T, k, true, flag.p);
        unsigned f = 0;
        ECK(cudaMemcpyAsync(&f, flag.p, sizeof f, cudaMemcpyDeviceToHost, g_st));
        sync();
        if (f) efail(GBNTT_ERR_DEVICE, "reciprocal correction did not converge (k=%zu)", k);
        return Y;
    }

    // ---- division by a shared divisor (reference bigint_div_newton) ----
    struct Divisor {
        const uint32_t *d = nullptr;   // divisor, nd limbs, top limb nonzero
        size_t nd = 0;
        int s = 0;                     // normalising left shift
        size_t k = 0;                  // reciprocal precision in limbs, k >= nd
        DBuf Y;                        // floor(beta^(k+nd) / (d 2^s)), k + 1 limbs
    };
    // Valid for dividends x with x 2^s < beta^(k+nd).
    void make_divisor(Divisor &D, const uint32_t *d, size_t nd, size_t k)
    {
        D.d = d;
        D.nd = nd;
        D.k = k;
        const uint32_t top = read_limb(d + nd - 1);
        if (!top) efail(GBNTT_ERR_ARG, "divisor not trimmed");
        D.s = __builtin_clz(top);
        DBuf T(k);
        extract1(T.p, k, d, nd, -(long long)D.s - 32LL * (long long)(k - nd));
        D.Y = recip_exact(T.p, k);
    }

    // Divisor for d = 10^(9 2^j) from the one of d^2 = 10^(9 2^(j+1)) (k = nd
    // on both): beta^(2n) / (d 2^s) = [beta^(2n') / (d^2 2^s')] d 2^(s'-s) /
    // beta^(2n'-2n), so Y = floor(Y' d / 2^(32 (2n' - 2n) - s' + s)). With Y'
    // at most two below beta^(2n') / (d^2 2^s'), the dropped part is below
    // 2 beta^(n+1) / beta^(2n-2) < 1 (n' >= 2n - 1, n >= 4): Y is exact or
    // one below, which leaves the quotient estimate of divide() at most two
    // below the quotient, within its two correction rounds.
    void derive_divisor(Divisor &D, const uint32_t *d, size_t nd, const Divisor &up)
    {
        if (nd < 4 || up.k != up.nd || up.nd + 1 < 2 * nd) efail(GBNTT_ERR_ARG, "divisor derivation out of range");
        D.d = d;
        D.nd = nd;
        D.k = nd;
        const uint32_t top = read_limb(d + nd - 1);
        if (!top) efail(GBNTT_ERR_ARG, "divisor not trimmed");
        D.s = __builtin_clz(top);
        const size_t na = up.nd + 1 + nd;
        DBuf A(na);
        mul(A.p, up.Y.p, up.nd + 1, d, nd);
        D.Y.alloc(nd + 1);
        extract1(D.Y.p, nd + 1, A.p, na, 32LL * (long long)(2 * up.nd - 2 * nd) - up.s + D.s);
    }

    // Divisor of the top decimal level d = 10^(9 2^J) = d'^2 for a dividend
    // of nx limbs with the reciprocal precision the quotient needs, k = nx -
    // nd + 2 (x 2^s < beta^(k + nd)), from the exact reciprocal Y' of the
    // level below (made here by Newton, returned in `below` for that level):
    // beta^(k+nd) / (d 2^s) = (beta^(2n') / (d' 2^s'))^2 / 2^(32 (4n' - k -
    // nd) - 2s' + s), so Y = floor(Y'^2 / 2^sh); Y' is below its value by
    // less than 1, which costs less than 2 V' / 2^sh <= 2^64 beta^(k - n')
    // < 1 for k <= n' - 3: Y is exact or one below. False (nothing done)
    // when the quotient needs more precision than that.
    bool short_top_divisor(Divisor &D, const uint32_t *d, size_t nd, size_t nx, const uint32_t *d1, size_t n1,
                           Divisor &below)
    {
        if (nx + 2 <= nd || n1 < 8) return false;
        const size_t k = nx + 2 - nd;
        if (k + 3 > n1 || nd > 2 * n1) return false;
        make_divisor(below, d1, n1, n1);
        D.d = d;
        D.nd = nd;
        D.k = k;
        const uint32_t topl = read_limb(d + nd - 1);
        if (!topl) efail(GBNTT_ERR_ARG, "divisor not trimmed");
        D.s = __builtin_clz(topl);
        DBuf A(2 * n1 + 2);
        mul(A.p, below.Y.p, n1 + 1, below.Y.p, n1 + 1);
        D.Y.alloc(k + 1);
        extract1(D.Y.p, k + 1, A.p, 2 * n1 + 2, 32LL * (long long)(4 * n1 - k - nd) - 2LL * below.s + D.s);
        return true;
    }

    struct DivItem {
        const uint32_t *x;
        size_t nx;
        uint32_t *q;   // nq limbs
        size_t nq;
        uint32_t *r;   // nr limbs, nr >= nd + 1 (remainders before correction are below 2 d)
        size_t nr;
    };
    // q_i = floor(x_i / d), r_i = x_i - q_i d for every item. The estimate
    // q' = floor(floor(x / beta^(nd-1)) Y / 2^(32 (k + 1) - s)) multiplies
    // only the dividend's top limbs (a product of about half the length).
    // With M = 2^(32 (k + nd) - s) and M / d - 2 <= Y <= M / d (an exact or
    // a derived reciprocal), x < M, and the dropped limbs costing less than
    // beta^(nd-1) Y / M <= beta^(nd-1) / d <= 1: x / d - 3 < q' <= x / d.
    // Three rounds of "if r >= d: r -= d, q += 1" finish it; a fourth
    // comparison checks.
    void divide(const std::vector<DivItem> &items, const Divisor &D)
    {
        const size_t n = items.size();
        if (!n) return;
        size_t t1 = 0, t2 = 0, tr = 0;
        for (auto &it : items) {
            t1 += it.nx - std::min(D.nd - 1, it.nx) + D.k + 1;
            t2 += it.nq + D.nd;
            tr += it.nr;
        }
        DBuf T1(t1);
        std::vector<Prod> pr;
        pr.reserve(n);
        std::vector<ExtractItem> ex;
        ex.reserve(n);
        size_t o = 0;
        for (auto &it : items) {   // q' = floor(floor(x / beta^(nd-1)) Y / 2^(32 (k + 1) - s))
            const size_t drop = std::min(D.nd - 1, it.nx), nh = it.nx - drop;
            pr.push_back({T1.p + o, it.x + drop, D.Y.p, nh, D.k + 1});
            ex.push_back({T1.p + o, it.q, nullptr, (long long)(nh + D.k + 1), (long long)it.nq,
                          32LL * (long long)(D.k + D.nd - drop) - D.s, 0});
            o += nh + D.k + 1;
        }
        batch_mul(pr);
        extract(ex);
        T1.release();
        // r = x - q' d: modulo beta^nr from the full product, or modulo
        // beta^W - 1 from a cyclic one (W >= nd + 2, so that the remainder,
        // below 4 d, stays below beta^(W-1)) when that transform is shorter
        int lw = kMinLog;
        while (((size_t)1 << lw) < D.nd + 2) lw++;
        const size_t W = (size_t)1 << lw;
        std::vector<char> wrap(n);
        t2 = 0;
        for (size_t i = 0; i < n; i++) {
            const DivItem &it = items[i];
            int ll = kMinLog;
            while (((size_t)1 << ll) < it.nq + D.nd - 1) ll++;
            wrap[i] = wrap_remainders_enabled() && lw < ll && it.nq <= W && it.nx <= 2 * W && it.nr <= W;
            t2 += wrap[i] ? W + 3 : it.nq + D.nd;
        }
        DBuf T2(t2);
        pr.clear();
        std::vector<Prod> pw;
        std::vector<int> wl;
        std::vector<WrapItem> wr;
        std::vector<AddItem> ad;
        ad.reserve(n);
        o = 0;
        for (size_t i = 0; i < n; i++) {
            const DivItem &it = items[i];
            if (wrap[i]) {
                pw.push_back({T2.p + o, it.q, D.d, it.nq, D.nd});
                wl.push_back(lw);
                wr.push_back({it.x, it.nx, T2.p + o, W, it.r, it.nr});
                o += W + 3;
            } else {
                pr.push_back({T2.p + o, it.q, D.d, it.nq, D.nd});
                ad.push_back({it.x, T2.p + o, it.r, nullptr, (long long)it.nx, (long long)(it.nq + D.nd),
                              (long long)it.nr, 0});
                o += it.nq + D.nd;
            }
        }
        batch_mul(pr);
        batch_mul_wrap(pw, wl);
        addsub(ad, true);
        wrap_remainders(wr);
        T2.release();
        DBuf Tt(tr);
        DTab<unsigned> flags(n);
        std::vector<AddItem> sb;
        std::vector<ExtractItem> cp;
        std::vector<IncItem> inc;
        o = 0;
        for (size_t i = 0; i < n; i++) {   // while r >= d: r -= d, q += 1
            const DivItem &it = items[i];
            sb.push_back({it.r, D.d, Tt.p + o, flags.p + i, (long long)it.nr, (long long)D.nd, (long long)it.nr, 0});
            cp.push_back({Tt.p + o, it.r, flags.p + i, (long long)it.nr, (long long)it.nr, 0, 0});
            inc.push_back({it.q, flags.p + i, (long long)it.nq});
            o += it.nr;
        }
        for (int round = 0; round < 3; round++) {
            addsub(sb, true);
            extract(cp);
            cond_inc(inc);
        }
        addsub(sb, true);   // every remainder must now be below d
        std::vector<unsigned> f(n);
        ECK(cudaMemcpyAsync(f.data(), flags.p, n * sizeof(unsigned), cudaMemcpyDeviceToHost, g_st));
        sync();
        for (size_t i = 0; i < n; i++)
            if (f[i]) efail(GBNTT_ERR_DEVICE, "division correction did not converge (item %zu of %zu)", i, n);
    }

    // ---- powers ----
    // 5^e: leading bits on the host, then GPU squarings and x 5 = (x << 2) + x.
    DBuf pow5(unsigned long long e, size_t &n)
    {
        int i = 63;
        while (i >= 0 && !((e >> i) & 1)) i--;
        unsigned long long v = 0;
        while (i >= 0 && v * 2 + ((e >> i) & 1) <= 27) {
            v = v * 2 + ((e >> i) & 1);
            i--;
        }
        unsigned long long x0 = 1;
        for (unsigned long long j = 0; j < v; j++) x0 *= 5;
        DBuf x = upload(bn::from_u64(x0), 2);
        n = x0 >> 32 ? 2 : 1;
        // 5^k has floor(k log2 5) + 1 bits: below 2^40 the double product is
        // within 1e-6 of k log2 5, so limbs_of(k) holds 5^k and the steps
        // need no length read back from the device (one trim at the end)
        const bool bound = e < (1ull << 40);
        auto limbs_of = [](unsigned long long k) -> size_t {
            return (size_t)((floor((double)k * 2.3219280948873623478703194 + 1e-6) + 1.0) / 32.0) + 1;
        };
        unsigned long long k = v;
        for (; i >= 0; i--) {
            k *= 2;
            const size_t ns = bound ? std::min(2 * n, limbs_of(k)) : 2 * n;
            DBuf y(2 * n);
            mul(y.p, x.p, n, x.p, n);
            n = bound ? ns : trim_top(y.p, 2 * n);
            x = std::move(y);
            if ((e >> i) & 1) {
                k += 1;
                DBuf z(n + 1);
                extract1(z.p, n + 1, x.p, n, -2);
                add1(z.p, n + 1, z.p, n + 1, x.p, n, false);
                n = bound ? std::min(n + 1, limbs_of(k)) : trim_top(z.p, n + 1);
                x = std::move(z);
            }
        }
        n = trim_top(x.p, n);
        return x;
    }

    // 10^e = 5^e 2^e
    DBuf pow10(unsigned long long e, size_t &n)
    {
        size_t n5 = 0;
        DBuf f = pow5(e, n5);
        const size_t cap = n5 + (size_t)(e / 32) + 1;
        DBuf t(cap);
        extract1(t.p, cap, f.p, n5, -(long long)e);
        n = trim_top(t.p, cap);
        return t;
    }

    // ---- decimal conversion (reference base_convert.c) ----
    // Decimal digits of x (no leading zeros; "0" for zero), copied from the
    // device straight to host memory: the leading digit to *first, the
    // others to rest[0 ..]. Returns the digit count; fails with
    // GBNTT_ERR_SIZE before copying when it exceeds max_digits (the count is
    // stored in *count_out first when count_out is given).
    // Levels above `top` are split here, a level at a time, with batched
    // engine products against one reciprocal; dec_block_kernel splits the
    // levels top .. low of each piece and prints the digits.
    size_t to_decimal(const uint32_t *x, size_t nx, char *first, char *rest, size_t max_digits,
                      size_t *count_out = nullptr)
    {
        nx = trim_top(x, nx);
        if (nx == 0) {
            if (count_out) *count_out = 1;
            if (max_digits < 1) efail(GBNTT_ERR_SIZE, "decimal string needs 1 digit");
            *first = '0';
            return 1;
        }
        const uint32_t topl = read_limb(x + nx - 1);
        const double bits = 32.0 * (double)(nx - 1) + (32 - __builtin_clz(topl));
        const long long dub = (long long)floor(bits * 0.30102999566398120) + 2;   // digit count upper bound
        int J = 0;
        while (9LL << (J + 1) < dub) J++;
        const long long TD = 9LL << (J + 1);      // padded digit count
        const long long Z = TD - dub;             // leading digits known to be zero
        const int top = std::min(J, dec_top_level());
        const int low = std::max(0, top - (kDecLeafLog - 1));
        const DecConst &K = dec_constants();
        DTab<char> dig((size_t)TD);
        // d_j = 10^(9 2^j), nd_j limbs; pieces of level j are below d_j^2 and
        // stored at stride 2 nd_j + 1
        std::vector<DBuf> pw(J + 1);
        std::vector<size_t> nd(J + 1, 0);
        nd[top] = K.d[top].size();
        pw[top] = upload(K.d[top], nd[top]);
        for (int j = top + 1; j <= J; j++) {
            pw[j].alloc(2 * nd[j - 1]);
            mul(pw[j].p, pw[j - 1].p, nd[j - 1], pw[j - 1].p, nd[j - 1]);
            nd[j] = trim_top(pw[j].p, 2 * nd[j - 1]);
        }
        auto stride = [&](int j) -> size_t { return 2 * nd[j] + 1; };
        DBuf lev(stride(J));
        extract1(lev.p, stride(J), x, nx, 0);
        const bool prof = getenv("GBNTT_E_PROFILE") != nullptr;
        Divisor up;      // the level above's divisor: its reciprocal seeds this level's
        Divisor below;   // level J - 1's, when the top level's short reciprocal was made from it
        bool have_below = false;
        for (int j = J; j > top; j--) {
            Stopwatch sw;
            Divisor D;
            if (j == J && j - 1 > top && short_top_reciprocal() &&
                short_top_divisor(D, pw[j].p, nd[j], nx, pw[j - 1].p, nd[j - 1], below))
                have_below = true;
            else if (j == J - 1 && have_below) D = std::move(below);
            else if (j < J && nd[j] >= 4 && derive_reciprocals()) derive_divisor(D, pw[j].p, nd[j], up);
            else make_divisor(D, pw[j].p, nd[j], nd[j]);
            double t_recip = 0;
            if (prof) {
                sync();
                t_recip = sw.lap();
            }
            const long long cnt = 1LL << (J - j);
            const size_t W = stride(j), Wc = stride(j - 1);
            DBuf child((size_t)(2 * cnt) * Wc);
            const long long i0 = Z / (9LL << (j + 1));
            std::vector<DivItem> items;
            items.reserve((size_t)(cnt - i0));
            for (long long i = i0; i < cnt; i++)   // (the top piece is x itself: nx limbs, zeros above)
                items.push_back({lev.p + i * W, j == J ? nx : W, child.p + 2 * i * Wc, Wc, child.p + (2 * i + 1) * Wc,
                                 Wc});
            divide(items, D);
            if (prof) {
                sync();
                fprintf(stderr, "to_decimal level %d: divisor %zu limbs, %zu pieces, reciprocal %.2f ms, "
                        "division %.2f ms\n", j, nd[j], items.size(), t_recip * 1e3, sw.lap() * 1e3);
            }
            lev = std::move(child);
            up = std::move(D);
            up.d = nullptr;   // d_j is released; Y, s and nd stay
            pw[j].release();
        }
        up.Y.release();
        {
            Stopwatch sw;
            DBuf ct(K.tab.size());
            ECK(cudaMemcpyAsync(ct.p, K.tab.data(), K.tab.size() * sizeof(uint32_t), cudaMemcpyHostToDevice, g_st));
            DecArgs a{};
            a.pieces = lev.p;
            a.first = Z / (9LL << (top + 1));
            a.top = top;
            a.low = low;
            a.leaf_stride = low > 0 ? K.lv[low - 1].stride : 2;
            a.ctab = ct.p;
            for (int j = 0; j <= kDecMaxTop; j++) a.lv[j] = K.lv[j];
            a.digits = dig.p;
            a.err = d_err;
            long long buf = 0, blk = 0;
            for (int j = low - 1; j <= top; j++)
                buf = std::max(buf, (1LL << (top - j)) * (j >= 0 ? K.lv[j].stride : 2));
            for (int j = low; j <= top; j++) blk = std::max(blk, (1LL << (top - j)) * K.lv[j].nblk);
            a.buf_limbs = (int)buf;
            a.blk_items = (int)blk;
            const size_t smem = (size_t)(2 * buf + blk * (kDecCols + 2)) * sizeof(uint32_t);
            if (smem > 48 * 1024) {
                int dev = 0, cap = 0;
                ECK(cudaGetDevice(&dev));
                ECK(cudaDeviceGetAttribute(&cap, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
                if (smem > (size_t)cap) efail(GBNTT_ERR_SIZE, "decimal block of level %d needs %zu bytes of shared "
                                              "memory (%d available)", top, smem, cap);
                ECK(cudaFuncSetAttribute(dec_block_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
            }
            const long long ncta = (1LL << (J - top)) - a.first;
            dec_block_kernel<<<(unsigned)ncta, kDecThreads, smem, g_st>>>(a);
            ECK(cudaGetLastError());
            if (prof) {
                sync();
                fprintf(stderr, "to_decimal levels %d..%d in one kernel: %lld pieces, %zu bytes shared, %.2f ms\n",
                        top, low, ncta, smem, sw.lap() * 1e3);
            }
        }
        // Z under-counts the leading zeros by at most two (the digit bound
        // from the bit length): read a short head to find the first digit
        const size_t avail = (size_t)(TD - Z);
        char head[64];
        const size_t hn = std::min(avail, sizeof head);
        ECK(cudaMemcpyAsync(head, dig.p + Z, hn, cudaMemcpyDeviceToHost, g_st));
        sync();
        size_t lead = 0;
        while (lead + 1 < hn && head[lead] == '0') lead++;
        if (head[lead] == '0' && hn < avail) efail(GBNTT_ERR_DEVICE, "decimal digits start with %zu zeros", hn);
        const size_t count = avail - lead;
        if (count_out) *count_out = count;
        if (count > max_digits) efail(GBNTT_ERR_SIZE, "decimal string has %zu digits, room for %zu", count, max_digits);
        *first = head[lead];
        if (count > 1) {
            ECK(cudaMemcpyAsync(rest, dig.p + Z + lead + 1, count - 1, cudaMemcpyDeviceToHost, g_st));
            sync();
        }
        return count;
    }
};

// reference split_terms_needed (ntt/app/compute_e/binary_split.c:96-108)
long split_terms(long n_digits)
{
    const double target = (double)n_digits * log(10.0);
    double N = target / log(target);
    for (int i = 0; i < 50; i++) {
        const double logN = log(N);
        if (logN <= 1.0) {
            N = target;
            break;
        }
        N = target / (logN - 1.0);
    }
    return (long)(N * 1.05) + 64;
}

// 32-bit coefficient transform log the e pipeline needs for D digits.
int e_required_log(long digits)
{
    const long K = split_terms(digits + 20);
    const double lnB = lgamma((double)K + 1.0);
    const double nB = lnB / log(2.0) / 32.0 + 4;
    const double nX = nB + (double)(digits - 1) * 3.3219280948873623 / 32.0 + 4;
    const double k = std::max(nB, nX + 1 - nB);
    const double need = nX + k + 2 + 64;
    int L = kMinLog;
    while ((double)(1LL << L) < need) L++;
    return L;
}

// Scoped use of the engine: initialise it when nobody has (torn down at the
// end), refuse when it is initialised but too small.
struct EngineUse {
    bool owned = false;
    explicit EngineUse(int need)
    {
        if (gbntt_is_ready()) {
            if (gbntt_max_log() < need)
                efail(GBNTT_ERR_SIZE, "engine initialised for 2^%d coefficients; this call needs 2^%d", gbntt_max_log(),
                      need);
        } else {
            ERC(gbntt_init(need));
            owned = true;
        }
        g_st = (cudaStream_t)gbntt_stream();
    }
    ~EngineUse()
    {
        if (g_st) cudaStreamSynchronize(g_st);
        // hand the stream-ordered pool's reserved memory back: the pipeline's
        // temporaries reach several GB at 10^8 digits
        int dev = 0;
        cudaMemPool_t pool;
        if (cudaGetDevice(&dev) == cudaSuccess && cudaDeviceGetDefaultMemPool(&pool, dev) == cudaSuccess)
            cudaMemPoolTrimTo(pool, 0);
        if (owned) gbntt_teardown();
        g_st = nullptr;
    }
};

size_t host_trim(const uint32_t *x, size_t n)
{
    while (n > 0 && x[n - 1] == 0) n--;
    return n;
}

int copy_out(uint32_t *out, size_t cap, size_t *n_out, const uint32_t *d, size_t n)
{
    if (n_out) *n_out = n;
    if (n > cap) efail(GBNTT_ERR_SIZE, "output needs %zu limbs, capacity %zu", n, cap);
    if (n) ECK(cudaMemcpyAsync(out, d, n * sizeof(uint32_t), cudaMemcpyDeviceToHost, g_st));
    ECK(cudaStreamSynchronize(g_st));
    return GBNTT_OK;
}

}  // namespace
}  // namespace gbntt

using namespace gbntt;

extern "C" {

long gbntt_split_terms_needed(long n_digits) { return split_terms(n_digits); }

int gbntt_e_required_log(long digits) { return digits < 1 ? -GBNTT_ERR_ARG : e_required_log(digits); }

int gbntt_binary_split(unsigned long long a, unsigned long long b, uint32_t *p, size_t p_cap, size_t *np, uint32_t *q,
                       size_t q_cap, size_t *nq)
{
    try {
        if (!gbntt_is_ready()) efail(GBNTT_ERR_NOT_INIT, "engine not initialised");
        EngineUse eu(gbntt_max_log());
        Pipe pp;
        DBuf P, B;
        size_t nP = 0, nB = 0;
        pp.binary_split(a, b, P, nP, B, nB);
        pp.check_errors();
        copy_out(p, p_cap, np, P.p, nP);
        return copy_out(q, q_cap, nq, B.p, nB);
    } catch (const EFail &f) {
        return f.code;
    }
}

int gbntt_newton_reciprocal_u32(uint32_t *x, size_t x_cap, size_t *nx, const uint32_t *q, size_t nq)
{
    try {
        if (!gbntt_is_ready()) efail(GBNTT_ERR_NOT_INIT, "engine not initialised");
        nq = host_trim(q, nq);
        if (nq == 0) efail(GBNTT_ERR_ARG, "newton_reciprocal: Q is zero");
        EngineUse eu(gbntt_max_log());
        Pipe pp;
        bn::Num hq(q, q + nq);
        DBuf dq = pp.upload(hq, nq);
        const int s = __builtin_clz(q[nq - 1]);
        DBuf T(nq);
        pp.extract1(T.p, nq, dq.p, nq, -(long long)s);
        DBuf Y = pp.recip_exact(T.p, nq);   // floor(2^(64 nq - s) / Q)
        DBuf R(nq + 1);
        pp.extract1(R.p, nq + 1, Y.p, nq + 1, s);   // floor(2^(2 bits(Q)) / Q)
        pp.check_errors();
        return copy_out(x, x_cap, nx, R.p, pp.trim_top(R.p, nq + 1));
    } catch (const EFail &f) {
        return f.code;
    }
}

int gbntt_div_newton_u32(uint32_t *qout, size_t q_cap, size_t *nq, uint32_t *rout, size_t r_cap, size_t *nr,
                         const uint32_t *n, size_t nn, const uint32_t *d, size_t nd)
{
    try {
        if (!gbntt_is_ready()) efail(GBNTT_ERR_NOT_INIT, "engine not initialised");
        nn = host_trim(n, nn);
        nd = host_trim(d, nd);
        if (nd == 0) efail(GBNTT_ERR_ARG, "division by zero");
        EngineUse eu(gbntt_max_log());
        Pipe pp;
        if (nn < nd) {   // quotient 0, remainder n
            if (nq) *nq = 0;
            if (rout || nr) {
                if (nr) *nr = nn;
                if (nn > r_cap) efail(GBNTT_ERR_SIZE, "remainder needs %zu limbs", nn);
                if (rout && nn) memcpy(rout, n, nn * sizeof(uint32_t));
            }
            return GBNTT_OK;
        }
        DBuf dn = pp.upload(bn::Num(n, n + nn), nn);
        DBuf dd = pp.upload(bn::Num(d, d + nd), nd);
        Pipe::Divisor D;
        pp.make_divisor(D, dd.p, nd, std::max(nd, nn + 1 - nd));
        const size_t cq = nn - nd + 1, cr = nd + 1;
        DBuf Q(cq), R(cr);
        pp.divide({{dn.p, nn, Q.p, cq, R.p, cr}}, D);
        pp.check_errors();
        copy_out(qout, q_cap, nq, Q.p, pp.trim_top(Q.p, cq));
        if (rout || nr) {
            const size_t lr = pp.trim_top(R.p, cr);
            if (!rout) { if (nr) *nr = lr; return GBNTT_OK; }
            copy_out(rout, r_cap, nr, R.p, lr);
        }
        return GBNTT_OK;
    } catch (const EFail &f) {
        return f.code;
    }
}

int gbntt_pow10_u32(uint32_t *out, size_t cap, size_t *n_out, unsigned long long e)
{
    try {
        if (!gbntt_is_ready()) efail(GBNTT_ERR_NOT_INIT, "engine not initialised");
        EngineUse eu(gbntt_max_log());
        Pipe pp;
        size_t n = 0;
        DBuf t = pp.pow10(e, n);
        pp.check_errors();
        return copy_out(out, cap, n_out, t.p, n);
    } catch (const EFail &f) {
        return f.code;
    }
}

int gbntt_to_decimal_u32(char *out, size_t cap, size_t *len, const uint32_t *x, size_t nx)
{
    try {
        if (!gbntt_is_ready()) efail(GBNTT_ERR_NOT_INIT, "engine not initialised");
        nx = host_trim(x, nx);
        EngineUse eu(gbntt_max_log());
        Pipe pp;
        DBuf dx = pp.upload(bn::Num(x, x + nx), std::max<size_t>(nx, 1));
        if (!out || cap < 2) efail(GBNTT_ERR_ARG, "output buffer needs at least 2 bytes");
        // *len receives the digit count also when the buffer is too small
        const size_t count = pp.to_decimal(dx.p, nx, out, out + 1, cap - 1, len);
        pp.check_errors();
        out[count] = 0;
        return GBNTT_OK;
    } catch (const EFail &f) {
        return f.code;
    }
}

int gbntt_compute_e(long digits, char *out, size_t cap, double *phase_seconds)
{
    try {
        if (digits < 1) efail(GBNTT_ERR_ARG, "digits must be >= 1");
        if (!out || cap < (size_t)digits + 2) efail(GBNTT_ERR_ARG, "output buffer needs %ld bytes", digits + 2);
        EngineUse eu(e_required_log(digits));
        Pipe pp;
        Stopwatch sw, total;
        double ph[5] = {0, 0, 0, 0, 0};
        const long K = split_terms(digits + 20);
        // P, B of [1, K + 1): B = K!, P / B = sum_{k=1}^{K} 1/k!
        DBuf P, B;
        size_t nP = 0, nB = 0;
        pp.binary_split(1, (unsigned long long)K + 1, P, nP, B, nB);
        pp.sync();
        ph[0] = sw.lap();
        // x = (B + P) 10^(D-1) = ((B + P) 5^(D-1)) << (D-1)
        const size_t cn = std::max(nB, nP) + 1;
        DBuf num(cn);
        pp.add1(num.p, cn, B.p, nB, P.p, nP, false);
        P.release();
        const size_t nn = pp.trim_top(num.p, cn);
        size_t n5 = 0;
        DBuf f5 = pp.pow5((unsigned long long)(digits - 1), n5);
        DBuf X(nn + n5);
        pp.mul(X.p, num.p, nn, f5.p, n5);
        num.release();
        f5.release();
        const size_t nX = pp.trim_top(X.p, nn + n5);
        const size_t cx = nX + (size_t)((digits - 1) / 32) + 1;
        DBuf x(cx);
        pp.extract1(x.p, cx, X.p, nX, -(long long)(digits - 1));
        X.release();
        const size_t nx = pp.trim_top(x.p, cx);
        ph[1] = sw.lap();
        // Q = floor(x / B)
        Pipe::Divisor D;
        pp.make_divisor(D, B.p, nB, std::max(nB, nx + 1 - nB));
        const size_t cq = nx - nB + 1, cr = nB + 1;
        DBuf Q(cq), R(cr);
        pp.divide({{x.p, nx, Q.p, cq, R.p, cr}}, D);
        x.release();
        R.release();
        D.Y.release();
        const size_t nQ = pp.trim_top(Q.p, cq);
        ph[2] = sw.lap();
        // "2.718...": the leading digit, the point, then the others, copied
        // from the device into out
        const size_t count = pp.to_decimal(Q.p, nQ, out, out + 2, cap - 2);   // a wrong count is checked below
        pp.check_errors();
        ph[3] = sw.lap();
        if ((long)count != digits)
            efail(GBNTT_ERR_DEVICE, "quotient has %zu decimal digits, expected %ld", count, digits);
        out[1] = '.';
        out[digits + 1] = 0;
        ph[4] = total.lap();
        if (phase_seconds) memcpy(phase_seconds, ph, sizeof ph);
        return GBNTT_OK;
    } catch (const EFail &f) {
        return f.code;
    }
}

}  // extern "C"
