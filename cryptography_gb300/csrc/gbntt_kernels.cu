// gbntt_kernels.cu — sm_103a kernels of the CRT-NTT multiply.
//
// 1. ntt_pass_kernel: one radix-2^l pass (l = 5..10) of an in-place NTT over
//    all three primes. A CTA owns G adjacent columns of one pass; it stages
//    G x 2^l residues in shared memory with 64-bit coalesced loads, computes
//    each 2^l-point DFT as A x B (A = 2^ceil(l/2), B = 2^floor(l/2)) with
//    fully unrolled register butterflies, and writes back in place.
//    Forward passes are decimation in frequency (natural order in, digit-
//    reversed order out, pass twiddle applied after the sub-DFT); inverse
//    passes are the exact transpose (twiddle before the sub-DFT, natural
//    order out). Fused into the passes: limb -> residue decomposition (first
//    forward pass reads 32-bit limbs), the pointwise product (first inverse
//    pass reads both spectra), and the N^-1 scale (last inverse pass).
//    Reference counterparts: stockham_kernel* and the Bailey 4-step
//    launchers in ntt/lib/ntt_kernel.hip:625-833, :1172-1375, the scatter
//    kernel ntt/lib/arith/ntt_mul.hip:117-160 and hadamard_kernel
//    ntt/lib/ntt_kernel.hip:386-399.
// 2. garner_carry_kernel: CRT reconstruction of every coefficient from its
//    three residues, the limb sums w0(c_j) + w1(c_{j-1}) + w2(c_{j-2}), and
//    the carry propagation over all product limbs as one decoupled look-back
//    scan (bounded waits). Replaces garner_kernel (ntt/lib/garner.hip:
//    187-260) plus the host carry sweep bigint_gather
//    (ntt/lib/arith/bigint.c:333-397); the carry monoid follows the CLA
//    cells of ntt/lib/transfer_core.h:165-251, generalised to carries in
//    {0, 1, 2}.
#include "gbntt_arith.cuh"
#include "gbntt_internal.h"

namespace gbntt {

// Montgomery forms of w_64^i (primitive 64th root, consistent with the
// 2^30-th root of the twiddle tables), per prime and direction.
__constant__ uint64_t c_w64[3][2][64];

cudaError_t upload_root_constants(const uint64_t w64[3][2][64])
{
    return cudaMemcpyToSymbol(c_w64, w64, sizeof(uint64_t) * 3 * 2 * 64);
}

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
// bit-reversed order out (X[k] ends in x[bitrev(k)]).
template <int PI, int DIR, int LOG_R>
__device__ __forceinline__ void dft_reg(uint64_t (&x)[1 << LOG_R])
{
    constexpr int R = 1 << LOG_R;
#pragma unroll
    for (int s = R / 2; s >= 1; s >>= 1) {
#pragma unroll
        for (int blk = 0; blk < R; blk += 2 * s) {
#pragma unroll
            for (int i = 0; i < s; i++) {
                uint64_t u = x[blk + i], v = x[blk + i + s];
                x[blk + i] = add_mod<PI>(u, v);
                uint64_t d = sub_mod<PI>(u, v);
                // w_{2s}^i = w_64^(i * 32 / s)
                x[blk + i + s] = (i == 0) ? d : mont_mul<PI>(d, c_w64[PI][DIR][i * (32 / s)]);
            }
        }
    }
}

// ---------------------------------------------------------------------------
// Element-wise modular operations over device arrays (self-test of the
// arithmetic, as the reference's test_modops.hip pins primes.h / shoup.h).
// op: 0 add_mod, 1 sub_mod, 2 mont_mul, 3..5 the plain C++ forms.
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

constexpr int kPassThreads = 256;

template <int PI, int LOG_L, int DIR, int LD>
__device__ __forceinline__ void pass_body(const PassArgs &a, uint64_t *sm)
{
    constexpr int L = 1 << LOG_L;
    constexpr int LOG_A = (LOG_L + 1) / 2, LOG_B = LOG_L / 2;
    constexpr int A = 1 << LOG_A, B = 1 << LOG_B;
    constexpr int T = kPassThreads;
    constexpr int G = T / A;                 // columns per CTA
    constexpr int LOG_G = 8 - LOG_A;
    constexpr int RS = L + A + 1;            // odd row stride (in 8-byte words)
    const int tid = threadIdx.x;
    const long long col0 = (long long)blockIdx.x * G;
    const int log_s = a.log_s, log_m = a.log_m;
    const long long smask = (1LL << log_s) - 1;
    const int log_gs = LOG_G < log_s ? LOG_G : log_s;
    const long long left = a.ncols - col0;
    const int gvalid = left < G ? (int)left : G;
    uint64_t *data = a.data[PI];
    const uint64_t *twhi = a.tw.hi[PI];
    const uint64_t *twlo = a.tw.lo[PI];
    const int sh = kMaxLog - log_m;

    // ---- cooperative coalesced load: element (g, m) -> sm[g*RS + m + m/B]
#pragma unroll 4
    for (int e = tid; e < G * L; e += T) {
        const int gp = e & ((1 << log_gs) - 1);
        const int rest = e >> log_gs;
        const int m = rest & (L - 1);
        const int g = ((rest >> LOG_L) << log_gs) + gp;
        uint64_t v = 0;
        if (g < gvalid) {
            const long long col = col0 + g;
            const long long addr = ((col >> log_s) << log_m) + (col & smask) + ((long long)m << log_s);
            if (LD == LD_U32) {
                v = addr < a.n_limbs ? (uint64_t)__ldg(a.limbs + addr) : 0ull;
            } else if (LD == LD_PW) {
                v = mont_mul<PI>(data[addr], a.other[PI][addr]);
            } else {
                v = data[addr];
            }
        }
        sm[g * RS + m + (m >> LOG_B)] = v;
    }
    __syncthreads();

    // ---- step 1: A-point DFTs over the high digit, one per (g, b)
    if (tid < G * B) {
        const int g = tid >> LOG_B, b = tid & (B - 1);
        uint64_t x[A];
#pragma unroll
        for (int i = 0; i < A; i++) x[i] = sm[g * RS + i * (B + 1) + b];
        if (DIR == 1 && (a.twiddle || a.use_scale)) {
            // inverse pass: input twiddle w_M^-((iB + b) j), times the scale
            const uint64_t j = (uint64_t)((col0 + g) & smask);
            uint64_t base = tw_exp<PI>(twhi, twlo, (uint32_t)(((uint64_t)b * j) << sh));
            const uint64_t step = tw_exp<PI>(twhi, twlo, (uint32_t)(((uint64_t)B * j) << sh));
            if (a.use_scale) base = mont_mul<PI>(base, a.scale[PI]);
#pragma unroll
            for (int i = 0; i < A; i++) {
                x[i] = mont_mul<PI>(x[i], base);
                if (i + 1 < A) base = mont_mul<PI>(base, step);
            }
        }
        dft_reg<PI, DIR, LOG_A>(x);
#pragma unroll
        for (int ka = 0; ka < A; ka++) {
            uint64_t v = x[bitrev(ka, LOG_A)];
            if (ka > 0 && b > 0)   // in-CTA twiddle w_L^(b ka)
                v = mont_mul<PI>(v, __ldg(twhi + ((b * ka) << (kTwBits - LOG_L))));
            sm[g * RS + ka * (B + 1) + b] = v;
        }
    }
    __syncthreads();

    // ---- step 2: B-point DFTs over the low digit, one per (g, ka)
    const int g2 = tid >> LOG_A, ka = tid & (A - 1);
    uint64_t y[B];
#pragma unroll
    for (int i = 0; i < B; i++) y[i] = sm[g2 * RS + ka * (B + 1) + i];
    dft_reg<PI, DIR, LOG_B>(y);
    if (DIR == 0 && a.twiddle) {
        // forward pass: output twiddle w_M^((ka + A kb) j)
        const uint64_t j = (uint64_t)((col0 + g2) & smask);
        uint64_t base = tw_exp<PI>(twhi, twlo, (uint32_t)(((uint64_t)ka * j) << sh));
        const uint64_t step = tw_exp<PI>(twhi, twlo, (uint32_t)(((uint64_t)A * j) << sh));
#pragma unroll
        for (int kb = 0; kb < B; kb++) {
            const int idx = bitrev(kb, LOG_B);
            y[idx] = mont_mul<PI>(y[idx], base);
            if (kb + 1 < B) base = mont_mul<PI>(base, step);
        }
    }
    __syncthreads();
#pragma unroll
    for (int kb = 0; kb < B; kb++) {
        const int k = ka + A * kb;
        sm[g2 * RS + k + (k >> LOG_B)] = y[bitrev(kb, LOG_B)];
    }
    __syncthreads();

    // ---- cooperative coalesced store
#pragma unroll 4
    for (int e = tid; e < G * L; e += T) {
        const int gp = e & ((1 << log_gs) - 1);
        const int rest = e >> log_gs;
        const int m = rest & (L - 1);
        const int g = ((rest >> LOG_L) << log_gs) + gp;
        if (g < gvalid) {
            const long long col = col0 + g;
            const long long addr = ((col >> log_s) << log_m) + (col & smask) + ((long long)m << log_s);
            data[addr] = sm[g * RS + m + (m >> LOG_B)];
        }
    }
}

template <int LOG_L, int DIR, int LD>
__global__ void __launch_bounds__(kPassThreads, 2) ntt_pass_kernel(PassArgs a)
{
    extern __shared__ uint64_t sm[];
    switch (blockIdx.y + a.prime_base) {
    case 0: pass_body<0, LOG_L, DIR, LD>(a, sm); break;
    case 1: pass_body<1, LOG_L, DIR, LD>(a, sm); break;
    default: pass_body<2, LOG_L, DIR, LD>(a, sm); break;
    }
}

template <int LOG_L>
constexpr size_t pass_smem_bytes()
{
    return (size_t)(kPassThreads >> ((LOG_L + 1) / 2)) * ((1 << LOG_L) + (1 << ((LOG_L + 1) / 2)) + 1) * 8;
}

typedef void (*PassFn)(PassArgs);

template <int LOG_L>
static cudaError_t launch_pass_l(int dir, int load_kind, const PassArgs &args, int nprimes, cudaStream_t stream)
{
    PassFn fn;
    if (dir == 0)
        fn = load_kind == LD_U32 ? ntt_pass_kernel<LOG_L, 0, LD_U32> : ntt_pass_kernel<LOG_L, 0, LD_U64>;
    else
        fn = load_kind == LD_PW ? ntt_pass_kernel<LOG_L, 1, LD_PW> : ntt_pass_kernel<LOG_L, 1, LD_U64>;
    const size_t smem = pass_smem_bytes<LOG_L>();
    static bool attr_done[2][3] = {{false, false, false}, {false, false, false}};
    if (!attr_done[dir][load_kind]) {
        cudaError_t e = cudaFuncSetAttribute((const void *)fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return e;
        attr_done[dir][load_kind] = true;
    }
    constexpr int G = kPassThreads >> ((LOG_L + 1) / 2);
    const long long gx = (args.ncols + G - 1) / G;
    dim3 grid((unsigned)gx, (unsigned)nprimes);
    fn<<<grid, kPassThreads, smem, stream>>>(args);
    return cudaGetLastError();
}

cudaError_t launch_pass(int log_l, int dir, int load_kind, const PassArgs &args, int nprimes, cudaStream_t stream)
{
    switch (log_l) {
    case 5: return launch_pass_l<5>(dir, load_kind, args, nprimes, stream);
    case 6: return launch_pass_l<6>(dir, load_kind, args, nprimes, stream);
    case 7: return launch_pass_l<7>(dir, load_kind, args, nprimes, stream);
    case 8: return launch_pass_l<8>(dir, load_kind, args, nprimes, stream);
    case 9: return launch_pass_l<9>(dir, load_kind, args, nprimes, stream);
    case 10: return launch_pass_l<10>(dir, load_kind, args, nprimes, stream);
    default: return cudaErrorInvalidValue;
    }
}

// ---------------------------------------------------------------------------
// Garner + carry
// ---------------------------------------------------------------------------
constexpr int kCarryThreads = 256;
constexpr int kCarryPerThread = 8;
constexpr int kCarryTile = kCarryThreads * kCarryPerThread;   // limbs per tile
constexpr int kLookbackSpinLimit = 1 << 21;                   // ~0.1 s with backoff

long long carry_tiles(long long n_out) { return (n_out + kCarryTile - 1) / kCarryTile; }

// Carry transfer function over carries {0,1,2}: 2 bits per input value.
__device__ __forceinline__ unsigned fn_apply(unsigned f, unsigned c) { return (f >> (2 * c)) & 3u; }
__device__ __forceinline__ unsigned fn_compose(unsigned g, unsigned f)   // g after f
{
    return fn_apply(g, fn_apply(f, 0)) | (fn_apply(g, fn_apply(f, 1)) << 2) | (fn_apply(g, fn_apply(f, 2)) << 4);
}
constexpr unsigned kFnIdentity = 0u | (1u << 2) | (2u << 4);

__device__ __forceinline__ int spad(int q) { return q + (q >> 5); }

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

__global__ void __launch_bounds__(kCarryThreads) garner_carry_kernel(CarryArgs a)
{
    constexpr int T = kCarryThreads, K = kCarryPerThread, TILE = kCarryTile;
    constexpr int SW = TILE + 2 + (TILE + 2) / 32 + 1;
    __shared__ uint32_t W0[SW], W1[SW], W2[SW];
    __shared__ unsigned s_warp[T / 32];
    __shared__ unsigned s_tile, s_cin;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    if (tid == 0) s_tile = atomicAdd(a.ticket, 1u);
    __syncthreads();
    const long long tile = s_tile;
    const long long base = tile * TILE;
    unsigned err = 0;

    // phase 1: coefficients of positions base-2 .. base+TILE-1 (slot q+2)
#pragma unroll
    for (int r = 0; r < K; r++) {
        const int q = r * T + tid;
        uint32_t w0, w1, w2;
        garner_coef(a, base + q, w0, w1, w2, err);
        W0[spad(q + 2)] = w0; W1[spad(q + 2)] = w1; W2[spad(q + 2)] = w2;
    }
    if (tid < 2) {
        uint32_t w0, w1, w2;
        garner_coef(a, base - 2 + tid, w0, w1, w2, err);
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
    if (tid == 0) {
        unsigned cin = 0;
        if (tile == 0) {
            atomicExch(&a.status[0], (2u << 8) | fn_apply(block_agg, 0));
        } else {
            atomicExch(&a.status[tile], (1u << 8) | block_agg);
            unsigned acc = kFnIdentity;
            long long j = tile - 1;
            for (;;) {
                unsigned w = 0;
                int spins = 0;
                for (;;) {
                    w = atomicAdd(&a.status[j], 0u);
                    if (w >> 8) break;
                    if (++spins > kLookbackSpinLimit) { err |= ERR_LOOKBACK_TIMEOUT; w = 2u << 8; break; }
                    __nanosleep(32);
                }
                const unsigned flag = w >> 8, val = w & 63u;
                if (flag == 2) { cin = fn_apply(acc, val); break; }
                acc = fn_compose(acc, val);
                const unsigned c0 = fn_apply(acc, 0);
                if (c0 == fn_apply(acc, 1) && c0 == fn_apply(acc, 2)) { cin = c0; break; }
                --j;
            }
            atomicExch(&a.status[tile], (2u << 8) | fn_apply(block_agg, cin));
        }
        s_cin = cin;
    }
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

cudaError_t launch_garner_carry(const CarryArgs &args, cudaStream_t stream, long long *ntiles_out)
{
    const long long nt = carry_tiles(args.n_out);
    if (ntiles_out) *ntiles_out = nt;
    if (nt == 0) return cudaSuccess;
    garner_carry_kernel<<<(unsigned)nt, kCarryThreads, 0, stream>>>(args);
    return cudaGetLastError();
}

}  // namespace gbntt
