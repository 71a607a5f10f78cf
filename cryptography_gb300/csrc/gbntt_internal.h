// gbntt_internal.h — declarations shared by the kernel and engine
// translation units (not part of the public C ABI).
#pragma once
#include <stdint.h>
#include <cuda_runtime.h>
#include <mutex>

#include "gbntt.h"

namespace gbntt {

constexpr int kMaxLog = 30;        // largest transform: 2^30 coefficients
constexpr int kTwBits = 15;        // two-level twiddle split: e = hi*2^15 + lo
constexpr int kTwSize = 1 << kTwBits;
constexpr int kMinLog = 5;         // smallest transform length used (32)
constexpr int kMaxPassLog = 10;    // largest sub-DFT staged in one CTA
constexpr int kMaxPasses = 4;      // passes per transform plan

enum LoadKind { LD_U64 = 0, LD_U32 = 1, LD_PW = 2, LD_U64LIMB = 3 };

// Twiddle tables of one direction for the three primes: Montgomery forms of
// w^e, w the primitive 2^30-th root g^((p-1)/2^30) (or its inverse), with
// hi[i] = w^(i*2^15) and lo[i] = w^i for i < 2^15.
//
// st1[k] points at the compact step-1 tables of the same prime and
// direction: for each pass size 2^l (l = 5..10, A = 2^ceil(l/2),
// B = 2^floor(l/2)) the A x B block at offset 2^l - 32 holds
// w_L^(ka b) at [ka B + b]. The pass kernel's step-1 twiddles are
// then one coalesced, L1-resident row per ka instead of a 32-line gather
// from hi[] (whose w_L powers lie 2^(15 - l) entries apart).
struct TwTables {
    const uint64_t *hi[3];
    const uint64_t *lo[3];
    const uint64_t *st1[3];
};

constexpr int kStep1Words = 2048;   // sum of 2^l for l = 5..10 (2016), rounded up

// Host: fill one (prime, direction) block of step-1 tables from that
// prime's hi[] table (hi[i] = w^(i 2^15), so w_L^e = hi[e 2^(15 - l)]).
template <typename W>
inline void build_step1_tables(const W *hi, W *dst)
{
    for (int l = kMinLog; l <= kMaxPassLog; l++) {
        const int L = 1 << l, A = 1 << ((l + 1) / 2), B = 1 << (l / 2);
        W *blk = dst + (L - 32);
        for (int ka = 0; ka < A; ka++)
            for (int b = 0; b < B; b++) blk[ka * B + b] = hi[((ka * b) & (L - 1)) << (kTwBits - l)];
    }
}

struct PassArgs {
    uint64_t *data[3];          // residues per prime, transformed in place
    const uint64_t *other[3];   // second spectrum for the fused pointwise product
    int other_log;              // nonzero: one shared second spectrum of 2^other_log points for every product
    int other_pair_log;         // nonzero: products 2i and 2i + 1 (of 2^other_pair_log points) share second spectrum i
    int other_r3;               // with either: products of 3 2^k points, k = that log, run as sub-transforms
                                // s = 3 p + m of 2^k points; product p's part m reads the second spectrum's
                                // sub-transform m (shared) or 3 (p >> 1) + m (pairs)
    const uint32_t *limbs;      // 32-bit limbs for the fused decomposition
    const uint64_t *limbs64;    // 64-bit limbs (one per coefficient) for the packed mode
    // batched first pass: product b's limbs are limb_tab[b][0 .. len_tab[b]),
    // its coefficients occupy [b 2^log_n_prod, (b+1) 2^log_n_prod)
    const uint32_t *const *limb_tab;
    const long long *len_tab;
    int log_n_prod;
    long long n_limbs;          // limbs beyond this index read as zero
    uint32_t *stage_out;        // first pass: also store each limb read here (a copy in HBM), or null
    TwTables tw;
    // pass twiddle tables (per slot, or null): entry j + m S of the table of
    // a pass over sub-problems of M = 2^log_m points is w_M^(+-j m) (times
    // scale[] in the outermost inverse pass), indexed by the element's offset
    // within its sub-problem; null: the pass builds w_M^(j m) from tw.hi/lo
    const uint64_t *ptw[3];
    uint64_t scale[3];          // Montgomery constant folded into inverse twiddles
    long long ncols;            // N / L columns per prime
    int log_m;                  // log2 of the sub-problem length M
    int log_s;                  // log2 of the column stride S = M / L
    int twiddle;                // apply the pass twiddle w_M^(j k)
    int use_scale;              // fold scale[] into the inverse input twiddles
    int prime_base;             // unused (one launch per prime)
    uint64_t w64[64];           // Montgomery w_64^i of this launch's prime and direction
    // fused innermost passes (forward, pointwise, inverse in one launch):
    // the inverse direction's step-1 tables and w_64 powers
    const uint64_t *st1_inv[3];
    uint64_t w64_inv[64];
};

struct CarryArgs {
    const uint64_t *res[3];     // inverse-transform output, natural order
    uint32_t *out;              // product limbs (32-bit coefficient mode)
    uint64_t *out64;            // product limbs (64-bit coefficient mode)
    long long n_coef;           // length of res[] (the transform length N)
    long long n_out;            // limbs to write
    unsigned int *ticket;       // dynamic tile counter (zeroed per launch)
    unsigned int *status;       // per-tile look-back words (zeroed per launch)
    unsigned int *error;        // sticky error bits
    uint64_t garner[4];         // Montgomery Garner constants (see engine)
    uint64_t q01_lo, q01_hi;    // q0 * q1 as 128 bits (64-bit coefficient mode)
    // batched mode: products of 2^log_n_prod coefficients laid end to end in
    // res[]; global tile t belongs to product b with tile_start[b] <= t <
    // tile_start[b+1]; product b writes out_tab[b][0 .. nout_tab[b])
    const long long *tile_start;
    uint32_t *const *out_tab;
    const long long *nout_tab;
    int nprod;
    int log_n_prod;
    int radix3;                 // batched mode: products of 3 2^log_n_prod coefficients
    int mixed;                  // two-prime set: res[0] q0 (64-bit), res[1] p3 (32-bit words)
};

enum ErrorBits : unsigned int {
    ERR_GARNER_DIGIT = 1u,      // third mixed-radix digit nonzero: corrupted residues
    ERR_LOOKBACK_TIMEOUT = 2u,  // carry look-back wait gave up
};

// Launchers (gbntt_kernels.cu).
template <int PI>
cudaError_t launch_pass_prime(int log_l, int dir, int ld, const PassArgs &a, cudaStream_t st);
// The innermost passes of a product in one launch: the last forward pass of
// data[] and of other[] (other == data: a square), their pointwise product
// and the first inverse pass, in place in data[] (contiguous blocks of
// 2^log_l points; plans of two or more passes).
template <int PI>
cudaError_t launch_inner_fused_prime(int log_l, const PassArgs &a, cudaStream_t st);
// Fill one pass twiddle table (see PassArgs::ptw) of prime PI from the
// two-level tables hi/lo of the wanted direction; use_scale multiplies every
// entry by scale (the outermost inverse pass).
template <int PI>
cudaError_t launch_build_pass_twiddles(uint64_t *table, const uint64_t *hi, const uint64_t *lo, int log_m,
                                       int log_s, int use_scale, uint64_t scale, cudaStream_t st);
cudaError_t launch_garner_carry(const CarryArgs &args, cudaStream_t stream, long long *ntiles_out);
cudaError_t launch_garner_carry64(const CarryArgs &args, cudaStream_t stream, long long *ntiles_out);
cudaError_t launch_garner_carry_batch(const CarryArgs &args, long long grid_tiles, cudaStream_t stream);
long long carry_tiles(long long n_out);
long long carry_tiles64(long long n_out);
cudaError_t launch_fill_splitmix(uint32_t *d, long long n, uint64_t seed, cudaStream_t st);
cudaError_t launch_copy_words(uint32_t *dst, const uint32_t *src, long long n, int grid, cudaStream_t st);

// Negacyclic products (gbntt_negacyclic.cu): the twist writes psi^i-scaled
// residues of coef into spec[0..2]; the finish untwists spec, reconstructs
// each coefficient modulo M = q0 q1 q2 and writes it to out as a signed
// 256-bit integer (4 words, least significant first).
struct NegaArgs {
    uint64_t *spec[3];            // residues per prime
    const uint64_t *coef;         // twist: N input coefficients
    const uint64_t *hi[3], *lo[3];// twiddle tables (forward for the twist, inverse for the finish)
    int shift;                    // psi^i = w^(i << shift)
    long long n;                  // N
    uint64_t *out;                // finish: 4 N words
    uint64_t garner[3];           // Montgomery Garner constants (three-prime set)
    uint64_t q01_lo, q01_hi;      // q0 q1
    uint64_t m[3];                // M = q0 q1 q2
    uint64_t half[3];             // (M - 1) / 2
};
cudaError_t launch_nega_twist(const NegaArgs &a, cudaStream_t st);
cudaError_t launch_nega_finish(const NegaArgs &a, cudaStream_t st);

// Batched products as gbntt_batch_mul_u32, with cyclic items: wrap_log[i] >
// 0 makes item i c = a b mod (beta^(2^L) - 1), L = wrap_log[i], written as
// 2^L + 3 limbs whose top 3 are the carry past limb 2^L - 1, unfolded
// (gbntt_engine.cu).
int batch_mul_wrap(uint32_t *const *d_c, const uint32_t *const *d_a, const size_t *na, const uint32_t *const *d_b,
                   const size_t *nb, const int *wrap_log, int count, cudaStream_t st);

// Batched limb additions out_i = x_i + y_i over n_i limbs (gbntt_e.cu).
int batch_add_limbs(const uint32_t *const *x, const uint32_t *const *y, uint32_t *const *out, const long long *n,
                    int count, cudaStream_t st, unsigned *err);
cudaError_t launch_modops(int prime, int op, const uint64_t *a, const uint64_t *b, uint64_t *out, long long n,
                          cudaStream_t stream);

// Message returned by gbntt_last_error (gbntt_engine.cu).
void set_error_message(const char *msg);

// Sticky error bits of the no-allocation multiply's scratch on the current
// device, cleared on read (gbntt_noalloc.cu); *set_up = 0 when that scratch
// was never set up on this device.
int noalloc_read_errors(unsigned *flags, int *set_up);

// Outer radix-3 stage of length-3 M transforms (gbntt_radix3.cu): W
// products, product w's three M-point sub-spectra at spec + w 3 M + m M.
struct R3Args {
    void *spec;                          // this prime's spectra
    long long M;                         // sub-transform length 2^k
    long long W;                         // products (<= 65535)
    int shift;                           // 30 - k: w_N^j = rho^(j << shift)
    const uint32_t *limbs;               // forward input of a single product ...
    long long n_limbs;
    const uint32_t *const *limb_tab;     // ... or of W products (device tables)
    const long long *len_tab;
    const void *hi, *lo;                 // rho^(i 2^15), i < 3 2^15, and rho^i, i < 2^15 (the field's multiply form)
    uint64_t c;                          // (om - om^2) / 2 in the same form
    uint64_t step;                       // w^G (forward) or w^-G (inverse), G = blocks x 256, same form
    int blocks;                          // grid x (at most 65535)
};
constexpr int kR3Unroll = 4;             // j values a thread's loads cover per step of its loop
cudaError_t launch_radix3(int pi, bool inverse, const R3Args &a, cudaStream_t st);

// Engine state and operations behind the reference-compatible entry points
// (gbntt_refabi.cu, built once for 64-bit and once for 112-bit BigInt
// limbs; gbntt_engine.cu).
std::recursive_mutex &engine_mutex();
bool engine_ready();
int engine_init(int L);            // size the engine for 2^L 32-bit coefficients
int engine_max_log();
const char *engine_error();        // message of the last failure
int ref_log_cap();                 // default cap of ntt_mul_init_impl's max_log_n
int ref_log();                     // max_log_n of the current ntt_mul_init_impl (0: none)
void ref_begin(int max_log_n);     // record it and zero the dispatch count
unsigned long &dispatch_count();
cudaStream_t engine_stream();
// device product of 32-bit limbs (na + nb limbs written to d_c)
int mul_dev_u32(uint32_t *d_c, const uint32_t *d_a, size_t na, const uint32_t *d_b, size_t nb, cudaStream_t st);
// the 64-bit BigInt product behind ntt_bigint_mul (guard and managed-capacity
// failures flagged for the caller's exit / abort)
int bigint_mul_impl(gbntt_bigint *c, const gbntt_bigint *a, const gbntt_bigint *b, bool *guard_fail,
                    bool *managed_fail);

}  // namespace gbntt
