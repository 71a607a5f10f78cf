/*
 * gbntt.h — C ABI of the GB300 CRT-NTT big-integer multiply engine.
 *
 * Two layers:
 *
 * 1. Drop-in entry points with the names, argument meaning and error
 *    behaviour of the reference engine (cecoppola/cryptography, ntt/).
 *    They work on the reference's BigInt layout at LIMB_BITS = 64
 *    (ntt/lib/arith/bigint.h:69-74) and, like the reference, print a
 *    message and exit(1) on misuse or failure.
 *
 * 2. A native API on 32-bit little-endian limbs (a uint64 limb array is the
 *    same bytes as a uint32 array of twice the length) that returns error
 *    codes instead of exiting, with device-pointer, host-pointer and batched
 *    forms.
 *
 * No CUDA or torch types appear in the signatures: streams are passed as
 * `void *` holding a cudaStream_t (NULL = the engine's own stream).
 */
#ifndef GBNTT_H
#define GBNTT_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Layout-identical to the reference BigInt with LIMB_BITS == 64
 * (ntt/lib/arith/bigint.h:69-74): value = sum limbs[i] * 2^(64 i). */
typedef struct {
    uint64_t *limbs;   /* little-endian limbs                      */
    int       n_limbs; /* significant limbs (trimmed)              */
    int       cap;     /* allocated limbs                          */
    int       managed; /* 1: limbs from bigint_alloc_managed       */
} gbntt_bigint;

/* ---- status codes of the native API --------------------------------- */
#define GBNTT_OK              0
#define GBNTT_ERR_NOT_INIT    1  /* engine not initialised                  */
#define GBNTT_ERR_SIZE        2  /* product does not fit the initialised N  */
#define GBNTT_ERR_CUDA        3  /* a CUDA runtime call failed              */
#define GBNTT_ERR_DEVICE      4  /* device-side check failed (Garner digit
                                    or a carry look-back wait gave up)      */
#define GBNTT_ERR_ARG         5  /* invalid argument                        */
#define GBNTT_ERR_MANAGED_CAP 6  /* managed output BigInt too small         */
#define GBNTT_ERR_ALLOC       7  /* device or host allocation failed        */

/* =====================================================================
 * 1. Reference-compatible entry points (libgbntt.so: the reference's
 *    default 64-bit limb build; libgbntt112.so exports the same names for
 *    its LIMB_BITS=112 build, declared in gbntt_limb112.h)
 * ===================================================================== */
#ifndef GBNTT_LIMB112_ABI

/* Replaces ntt_mul_init_impl (ntt/lib/arith/ntt_mul.hip:379), reached from
 * ntt_mul_init (ntt/lib/arith/multiply.c:97). Sizes the engine for products
 * of up to 2^max_log_n 64-bit coefficients, i.e. operands with
 * n_a + n_b - 1 <= 2^max_log_n 64-bit limbs. Valid range [3, cap]; cap is
 * 28 unless NTT_MAX_LOGN (<= 29) raises it. Out of range: message + exit(1).
 * A second call while initialised is a no-op, as in the reference. */
void ntt_mul_init_impl(int max_log_n);

/* Replaces ntt_mul_teardown_impl (ntt/lib/arith/ntt_mul.hip:533). Frees all
 * device state; NTT_PROFILE=1 prints the per-phase summary first. */
void ntt_mul_teardown_impl(void);

/* Replaces ntt_bigint_mul (ntt/lib/arith/ntt_mul.hip:995; prototype
 * ntt/lib/arith/multiply.h:46). c = a * b exactly. c is grown with realloc
 * to n_a + n_b + 4 limbs when needed (a managed c that is too small aborts,
 * as bigint_resize does in ntt/lib/arith/bigint.c:46-60); c->n_limbs is
 * trimmed and limbs above it are zero. c may alias a or b; a == b takes the
 * squaring path (one forward transform). Exits with a message when not
 * initialised or when n_a + n_b - 1 > 2^max_log_n (the reference's cyclic
 * wrap guard, ntt_mul.hip:1013-1022). */
void ntt_bigint_mul(gbntt_bigint *c, const gbntt_bigint *a, const gbntt_bigint *b);

/* Replaces ntt_get_gpu_dispatch_count (ntt/lib/arith/ntt_mul.hip:595). */
unsigned long ntt_get_gpu_dispatch_count(void);

/* Replaces ntt_gpu_emergency_reset (ntt/lib/arith/ntt_mul.hip:1248): drains
 * in-flight work with cudaDeviceSynchronize; never resets the device. */
void ntt_gpu_emergency_reset(void);

/* Strong overrides of the reference's weak allocators
 * (ntt/lib/arith/bigint.c:31-69, ntt/lib/arith/bigint_hip_alloc.hip):
 * cudaMallocManaged limbs, zeroed, managed = 1. */
gbntt_bigint bigint_alloc_managed(int cap);
void hip_free_limbs(uint64_t *p);

/* Additive (no reference equivalent): c = a * a. */
void ntt_bigint_sqr(gbntt_bigint *c, const gbntt_bigint *a);

/* Additive: ntt_bigint_mul returning a GBNTT_* code instead of exiting. */
int ntt_bigint_mul_checked(gbntt_bigint *c, const gbntt_bigint *a, const gbntt_bigint *b);
#endif /* GBNTT_LIMB112_ABI */

/* =====================================================================
 * 2. Native API (32-bit limbs)
 * ===================================================================== */

/* Initialise for transforms up to 2^max_log32 32-bit coefficients
 * (5 <= max_log32 <= 30): products with n_a + n_b - 1 <= 2^max_log32. */
int gbntt_init(int max_log32);
void gbntt_teardown(void);
int gbntt_is_ready(void);
int gbntt_max_log(void);

/* Device memory the engine allocates at gbntt_init(max_log32). */
size_t gbntt_workspace_bytes(int max_log32);

/* Transform length log2 chosen for an n_a x n_b product. */
int gbntt_transform_log(size_t na, size_t nb);

/* Pass plan for a transform of 2^log_n points: writes the pass sizes
 * (log2, outermost first) to passes[0..3] (room for GBNTT_MAX_PASSES ints)
 * and returns the pass count. */
#define GBNTT_MAX_PASSES 4
int gbntt_plan(int log_n, int *passes);

/* Override the pass plan of transforms of 2^log_n points (1 to 4 passes,
 * each of 2^5 .. 2^10 points, sizes summing to log_n, outermost first);
 * npasses = 0 restores the default plan. Used by the autotuner. */
int gbntt_set_plan(int log_n, int npasses, const int *passes);

/* Autotuner (the reference picks its transform factorisation by hand): for
 * each transform length 2^L, log_lo <= L <= log_hi <= the initialised
 * maximum, times every pass plan of 1 to 4 passes of 2^5 .. 2^10 points on a
 * synthetic product (best of `reps` runs after a warm-up, CUDA events) and
 * installs the fastest as that length's plan (as gbntt_set_plan does).
 * plans (may be NULL) receives 1 + GBNTT_MAX_PASSES ints per length: pass
 * count, then the sizes (unused entries 0);
 * ms (may be NULL) the winning time in milliseconds. Synchronous. */
int gbntt_autotune(int log_lo, int log_hi, int reps, int *plans, float *ms);

/* Batched waves run as CUDA graphs: a wave shape (context, table slot,
 * transform length, wave size, prime set) seen a second time is captured
 * and replayed from then on (environment GBNTT_GRAPHS=0 launches every
 * wave directly). Returns the number of instantiated wave graphs held. */
int gbntt_wave_graphs(void);

/* d_c[0 .. na+nb) = d_a * d_b on the device, stream-ordered (returns after
 * enqueueing). d_b == d_a with nb == na squares. d_c must not overlap the
 * inputs. Device-side check failures are recorded and reported by
 * gbntt_device_errors(). */
int gbntt_mul_u32(uint32_t *d_c, const uint32_t *d_a, size_t na, const uint32_t *d_b, size_t nb,
                  void *stream);
int gbntt_sqr_u32(uint32_t *d_c, const uint32_t *d_a, size_t na, void *stream);

/* Negacyclic polynomial product (the reference's crt_ntt negacyclic
 * pipeline, ntt/lib/main.hip:557-684, twist / NTT / pointwise / inverse NTT /
 * untwist / Garner): for N = 2^log_n and f, g of N 64-bit coefficients,
 *   out[k] = sum_{i+j=k} f_i g_j - sum_{i+j=k+N} f_i g_j   (mod X^N + 1),
 * exact, as signed 256-bit two's complement integers (4 uint64 words per
 * coefficient, least significant first; |out[k]| < N 2^128). Device
 * pointers, stream-ordered; d_g == d_f squares. Three 64-bit primes
 * (modulus ~2^192). 5 <= log_n <= min(29, the initialised maximum). The
 * reference writes the unsigned residue modulo its four-prime modulus
 * (U256); here the value itself is written. */
int gbntt_negacyclic_mul_u64(uint64_t *d_out, const uint64_t *d_f, const uint64_t *d_g, int log_n, void *stream);

/* Batched products (no reference counterpart; the reference runs one
 * product at a time): d_c[i][0 .. na[i]+nb[i]) = d_a[i] * d_b[i] for
 * i < count. The arrays are host arrays of device pointers and sizes. The
 * engine groups the products by transform length and runs each group in
 * waves that fit its workspace, one launch per pass and prime per wave.
 * Stream-ordered; results are bit-identical to gbntt_mul_u32 per product.
 * Outputs must not overlap inputs or each other. */
int gbntt_batch_mul_u32(uint32_t *const *d_c, const uint32_t *const *d_a, const size_t *na,
                        const uint32_t *const *d_b, const size_t *nb, int count, void *stream);

/* Serving loop (continuous batching; no reference counterpart). Starts a
 * server thread owning `slots` workspaces of 2^slot_log coefficients (48 x
 * 2^slot_log bytes of device memory each, on their own streams). Requests
 * are device-pointer products queued in arrival order; whenever a slot is
 * free the server admits, in arrival order, the pending requests of the
 * oldest request's transform length that fit the slot and runs them as one
 * wave, so requests arriving while others run are admitted as slots free
 * up and their work overlaps on the device. Results are bit-identical to
 * gbntt_mul_u32. Latency = submit -> completion observed by the server.
 * The engine must be initialised; the ordinary entry points stay usable. */
int gbntt_server_start(int slots, int slot_log);
int gbntt_server_submit(uint32_t *d_c, const uint32_t *d_a, size_t na, const uint32_t *d_b, size_t nb,
                        uint64_t *ticket);
/* state: 0 pending, 1 running, 2 done; latency_us < 0 until done. */
int gbntt_server_query(uint64_t ticket, int *state, double *latency_us);
int gbntt_server_wait(uint64_t ticket, double timeout_s);
/* device_errors: OR of the slots' device check flags (see gbntt_device_errors). */
int gbntt_server_stats(uint64_t *completed, uint64_t *waves, uint64_t *wave_products, unsigned *device_errors);
/* Drains the queue, joins the thread and frees the slots. */
int gbntt_server_stop(void);

/* Packed mode: one 64-bit limb per coefficient (the reference engine's own
 * granularity, ntt/lib/arith/bigint.h:30-43). Operands and product are
 * 64-bit limb arrays (na, nb counted in 64-bit limbs; d_c gets na + nb
 * limbs); the transform length is the smallest power of two >= na + nb - 1,
 * half that of the 32-bit form for the same integers. Stream-ordered. */
int gbntt_mul_u64(uint64_t *d_c, const uint64_t *d_a, size_t na, const uint64_t *d_b, size_t nb, void *stream);
int gbntt_sqr_u64(uint64_t *d_c, const uint64_t *d_a, size_t na, void *stream);
int gbntt_mul_u64_host(uint64_t *c, const uint64_t *a, size_t na, const uint64_t *b, size_t nb);

/* Coefficient width (32 or 64 bits) used by the BigInt entry points
 * (ntt_bigint_mul and friends). Default 32, or 64 when the environment sets
 * GBNTT_COEFF_BITS=64 at initialisation. */
int gbntt_set_coeff_bits(int bits);
int gbntt_coeff_bits(void);

/* Host-pointer form: copies in, multiplies, copies out, synchronises and
 * checks the device error flags. c must hold na + nb limbs. */
int gbntt_mul_u32_host(uint32_t *c, const uint32_t *a, size_t na, const uint32_t *b, size_t nb);

/* Synchronise the engine stream, return and clear the device error bits
 * (1 = Garner digit check, 2 = look-back wait gave up). The bits of
 * gbntt_mul_u32_noalloc on the current device (a separate sticky word in
 * its static scratch) are ORed in and cleared too; without an initialised
 * engine only those are returned (GBNTT_ERR_NOT_INIT when neither the
 * engine nor the no-allocation multiply was set up). */
int gbntt_device_errors(unsigned int *flags);

/* Forward spectra of a limb vector for each prime (3 x 2^log_n uint64, in
 * the engine's digit-reversed order; see gbntt_plan). For known-answer
 * tests. d_out needs 3 * 2^log_n entries. */
int gbntt_debug_forward(uint64_t *d_out, const uint32_t *d_in, size_t n, int log_n, void *stream);

/* Residues of the 3 2^k-point transform path, two-prime set: mode 1, the
 * cyclic convolution of a and b of length 3 2^k (n_a + n_b - 1 <= 3 2^k)
 * before Garner; mode 0, 3 a after the forward and inverse radix-3 stages
 * alone (the 1/3 belongs to the inverse sub-transforms' scale). d_q0 receives 3 2^k q0 residues (uint64), d_p3 3 2^k p3
 * residues (uint32); device pointers. For known-answer tests. */
int gbntt_debug_radix3(uint64_t *d_q0, uint32_t *d_p3, const uint32_t *d_a, size_t na, const uint32_t *d_b,
                       size_t nb, int k, int mode);

/* Self-test of the bounded waits (no reference counterpart): runs the
 * Garner+carry kernel over a few tiles with its tile ticket started past
 * tile 0, so one look-back waits on a status word that nothing writes; the
 * wait gives up after its iteration limit, the kernel finishes and *flags
 * receives the device error bits (bit 1: a look-back wait gave up).
 * *seconds receives the kernel's wall time. Needs an engine of at least
 * 2^13 coefficients. The context stays usable. */
int gbntt_debug_lookback_timeout(unsigned int *flags, double *seconds);

/* Element-wise modular arithmetic on device arrays for self-tests: for
 * prime index 0..2 (2^64 - 2^b + 1, b = 32, 34, 40) and op 0 = (a+b) mod p,
 * 1 = (a-b) mod p, 2 = a*b*2^-64 mod p (Montgomery), 3..5 = the same with
 * the plain C++ forms. a, b canonical (a may be any 64-bit value for op
 * 2 and 5). Prime index 3 is p3 = 3 * 2^30 + 1 on the low 32 bits of each
 * word, op 2 = a*b*2^-32 mod p3 (a may be any 32-bit value for op 2 and 5).
 * Prime index 4 is q0 in lazy normal form: any 64-bit operands, op 2 =
 * a*b mod q0, results in [0, 2^64) congruent mod q0 (canonical for 3..5).
 * Prime index 0 also takes op 6: a * 2^(b mod 96) mod q0, the register
 * DFTs' power-of-two multiply (a canonical). Stream-ordered. */
int gbntt_debug_modops(int prime, int op, const uint64_t *d_a, const uint64_t *d_b, uint64_t *d_out, size_t n,
                       void *stream);

/* Seeded synthetic operand on the device (benchmarks): d[i] = low 32 bits of
 * splitmix64 at seed + (i + 1) * 0x9E3779B97F4A7C15, bit 31 of d[n-1] set.
 * Stream-ordered. */
int gbntt_fill_operand(uint32_t *d, size_t n, uint64_t seed, void *stream);

/* Per-launch timing for roofline reports. gbntt_launch_log(1) makes every
 * following kernel launch record CUDA events (kind: 0 first forward pass,
 * 1 forward pass, 2 first inverse pass with the pointwise product,
 * 3 inverse pass, 4 Garner + carry, 5 the fused innermost passes: both
 * operands' last forward pass, the pointwise product and the first inverse
 * pass in one launch), its pass size log2 and its algorithmic
 * bytes; gbntt_launch_log(0) stops and clears. gbntt_launch_records
 * synchronises and copies up to max_records entries; returns the count or
 * a negative GBNTT_* code. */
int gbntt_launch_log(int enable);
int gbntt_launch_records(int *kind, int *log_l, double *bytes, float *ms, int max_records);

/* No counterpart in the reference. gbntt_mul_u32 without any allocation:
 * for callers that cannot allocate device memory where they need a product
 * (an application whose device allocator is owned by a pool or arena that
 * forbids cudaMalloc/cudaFree, latency-critical loops where cudaMalloc would
 * synchronise the device, or code that has no engine initialised).
 * d_c[0 .. na+nb) = d_a * d_b for na + nb - 1 <= 2^16 (GBNTT_ERR_SIZE above
 * that); needs no gbntt_init. All scratch (6,390,784 bytes, about 6.4 MB)
 * is one static device array that every GPU loading this library keeps
 * until exit. The first call on each device (with that device current)
 * sets the array up with cudaGetSymbolAddress and cudaMemcpy, so make that
 * first call before any stream capture; do not use it across a
 * cudaDeviceReset (the array comes back zeroed, the set-up is not redone).
 * Calls share the array: calls that overlap on the GPU race; serialise them
 * (one stream, one thread at a time). Stream-ordered. Device check failures
 * (Garner bound, look-back wait limit) set a sticky error word in the
 * scratch that gbntt_device_errors reads and clears. */
int gbntt_mul_u32_noalloc(uint32_t *d_c, const uint32_t *d_a, size_t na, const uint32_t *d_b, size_t nb,
                          void *stream);

/* Test hook (no counterpart in the reference): one carry look-back wait in
 * gbntt_mul_u32_noalloc's scratch waits on a status word nothing writes and
 * runs out by itself; the error bit 2 is then reported by
 * gbntt_device_errors. Synchronises the device. */
int gbntt_debug_noalloc_lookback_timeout(double *seconds);

/* ---- e pipeline and the arith layer above the multiply ----
 * Host operands and results, 32-bit limbs little-endian; every product runs
 * on the engine (batched where a level has many). All but gbntt_compute_e
 * need an initialised engine large enough for their products. */

/* Replaces split_terms_needed (ntt/app/compute_e/binary_split.c:96-108):
 * number of series terms for n_digits digits, the same formula. */
long gbntt_split_terms_needed(long n_digits);

/* Transform log (32-bit coefficients) that gbntt_compute_e needs for
 * `digits` digits; negative on bad input. */
int gbntt_e_required_log(long digits);

/* Replaces binary_split (ntt/app/compute_e/binary_split.c:26-86): P and B of
 * [a, b) with B = (b-1)!/(a-1)! and P / B = sum_{k=a}^{b-1} (a-1)!/k!
 * (empty range: P = 0, B = 1). b - 1 < 2^32. p[0 .. *np), q[0 .. *nq). */
int gbntt_binary_split(unsigned long long a, unsigned long long b, uint32_t *p, size_t p_cap, size_t *np,
                       uint32_t *q, size_t q_cap, size_t *nq);

/* Replaces newton_reciprocal (ntt/lib/arith/newton.h:23, newton.c:119):
 * x = floor(2^(2 bits(Q)) / Q), always exact here (the reference's may be
 * one below). */
int gbntt_newton_reciprocal_u32(uint32_t *x, size_t x_cap, size_t *nx, const uint32_t *q, size_t nq);

/* Replaces bigint_div_newton (ntt/lib/arith/newton.h:28, newton.c:128):
 * q = floor(n / d) and, when r or nr is given, r = n mod d. */
int gbntt_div_newton_u32(uint32_t *q, size_t q_cap, size_t *nq, uint32_t *r, size_t r_cap, size_t *nr,
                         const uint32_t *n, size_t nn, const uint32_t *d, size_t nd);

/* Replaces base_convert_pow10_exact (ntt/lib/arith/base_convert.h:32):
 * out = 10^e. */
int gbntt_pow10_u32(uint32_t *out, size_t cap, size_t *n_out, unsigned long long e);

/* Replaces bigint_to_decimal (ntt/lib/arith/base_convert.h:24): decimal
 * digits of x, NUL-terminated, no leading zeros ("0" for zero); *len
 * receives the digit count (cap >= len + 1). */
int gbntt_to_decimal_u32(char *out, size_t cap, size_t *len, const uint32_t *x, size_t nx);

/* Replaces the compute_e application (ntt/app/compute_e/main.c:150-345):
 * writes "2.718..." with `digits` significant digits (the string main.c
 * prints after "e = ", digits + 1 characters) and a NUL into out (cap >=
 * digits + 2). Uses the reference's term count and guard digits, so the
 * digits are the reference's. Initialises the engine for the call when it
 * is not initialised (and tears it down after); fails with GBNTT_ERR_SIZE
 * when it is initialised too small. phase_seconds, when not NULL, receives
 * 5 wall times: product tree, numerator x 10^(D-1), division, decimal
 * conversion, total. */
int gbntt_compute_e(long digits, char *out, size_t cap, double *phase_seconds);

/* No counterpart in the reference (its engine always uses three 64-bit
 * primes). Primes used for products of 32-bit coefficients (gbntt_mul_u32,
 * batches, serving, the e pipeline and ntt_bigint_mul in its default
 * mode): 2 = q0 = 2^64 - 2^32 + 1 (64-bit residues) with p3 = 3 * 2^30 + 1
 * (32-bit residues), CRT modulus ~2^95.6 above every coefficient (< 2^93),
 * the default; 3 = the reference's three 64-bit primes. Products are
 * identical either way. Packed (64-bit coefficient) products always use
 * three 64-bit primes. The default comes from GBNTT_PRIMES (2 or 3) at
 * init. gbntt_prime_set returns 0 when no engine is initialised. Refused
 * (GBNTT_ERR_ARG) while the serving loop runs. */
int gbntt_set_prime_set(int nprimes);
int gbntt_prime_set(void);

/* Last error message of this library. */
const char *gbntt_last_error(void);

/* Engine stream (cudaStream_t) used when NULL is passed. */
void *gbntt_stream(void);

#ifdef __cplusplus
}
#endif

#endif /* GBNTT_H */
