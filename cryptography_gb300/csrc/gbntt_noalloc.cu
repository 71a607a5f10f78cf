// gbntt_noalloc.cu — a multiply entry point that allocates nothing.
//
// Some callers cannot allocate device memory at the point where they need a
// product: code that runs while another component owns the device allocator
// (a pool or arena that forbids cudaMalloc/cudaFree behind its back), code
// in latency-critical loops where cudaMalloc/cudaFree would synchronise the
// device, or callers that have no engine initialised (gbntt_init allocates
// the full-size workspace). gbntt_mul_u32_noalloc serves them for products
// of up to kNoAllocMaxN coefficients: every scratch word it needs (twiddle
// tables, both spectra, the carry scan's ticket and status words) lives in
// the file-scope array below, which every GPU that loads this library holds
// until the process exits. The caller passes device pointers for the
// operands and the product.
//
// Host code must not use `g_noalloc_scratch` as an address: on the host the
// name is only a stand-in for the symbol. The first call on each device
// (with that device current) resolves the real address with
// cudaGetSymbolAddress and uploads the twiddle tables with cudaMemcpy; that
// first call should therefore come before any stream capture. All calls
// share the one array: calls that overlap on the GPU (different streams, or
// different host threads) race and produce wrong results; serialise them.
// The set-up is cached per device for the life of the process: after
// cudaDeviceReset the array comes back zeroed while the cache still says it
// is ready, so this entry point must not be used across a device reset.
//
// Device checks (the Garner bound, the bounded carry look-back waits) set
// bits in an error word inside the array that stays set across calls until
// gbntt_device_errors reads and clears it; each call clears only the carry
// scan's ticket and tile status words.
#include <cuda_runtime.h>
#include <chrono>
#include <mutex>
#include <stdio.h>
#include <string.h>

#include "gbntt_arith.cuh"
#include "gbntt_internal.h"
#include "gbntt.h"

namespace gbntt {

namespace {

constexpr int kNoAllocMaxLog = 16;                       // products of up to 2^16 coefficients
constexpr size_t kNoAllocMaxN = (size_t)1 << kNoAllocMaxLog;
constexpr size_t kHiLoWords = 3 * 2 * 2 * (size_t)kTwSize;            // [prime][dir][hi|lo][2^15]
constexpr size_t kTwWords = kHiLoWords + 3 * 2 * (size_t)kStep1Words;  // then [prime][dir] step-1 tables
constexpr size_t kSpecWords = 6 * kNoAllocMaxN;          // 3 primes x (A, B)
constexpr size_t kCtlWords = 64 + kNoAllocMaxN / 1024;   // ticket, error, tile status (32-bit each, rounded up)
constexpr size_t kScratchWords = kTwWords + kSpecWords + kCtlWords;

}  // namespace

// The scratch array (8-byte words): twiddle tables, spectra, control words;
// 6,390,784 bytes (about 6.4 MB) of static device memory per GPU.
static __device__ __align__(256) uint64_t g_noalloc_scratch[kScratchWords];
static_assert(sizeof(g_noalloc_scratch) == 6390784, "the documented scratch size (include/gbntt.h) is out of date");

namespace {

constexpr int kMaxDevices = 64;
std::mutex g_na_mu;
uint64_t *g_na_ptr[kMaxDevices];      // device address of the scratch per device (nullptr: not set up)
uint64_t g_na_w64[3][2][64];          // Montgomery w_64^i per prime and direction
uint64_t g_na_garner[3];              // Montgomery Garner constants
uint64_t g_na_tw_host[kTwWords];      // host image of the twiddle tables (static: no malloc)
bool g_na_host_ready = false;

typedef unsigned __int128 u128;
uint64_t na_mul(uint64_t a, uint64_t b, uint64_t p) { return (uint64_t)((u128)a * b % p); }
uint64_t na_pow(uint64_t b, uint64_t e, uint64_t p)
{
    uint64_t r = 1;
    b %= p;
    while (e) {
        if (e & 1) r = na_mul(r, b, p);
        b = na_mul(b, b, p);
        e >>= 1;
    }
    return r;
}
uint64_t na_inv(uint64_t a, uint64_t p) { return na_pow(a % p, p - 2, p); }
uint64_t na_mont(uint64_t x, uint64_t p) { return (uint64_t)(((u128)(x % p) << 64) % p); }

void host_tables()
{
    if (g_na_host_ready) return;
    static const uint64_t gen[3] = {7, 10, 19};
    for (int pi = 0; pi < 3; pi++) {
        const uint64_t p = prime_value(pi);
        const uint64_t w = na_pow(gen[pi], (p - 1) >> kMaxLog, p);
        for (int dir = 0; dir < 2; dir++) {
            const uint64_t wd = dir ? na_inv(w, p) : w;
            uint64_t *hi = g_na_tw_host + (((size_t)pi * 2 + dir) * 2 + 0) * kTwSize;
            uint64_t *lo = g_na_tw_host + (((size_t)pi * 2 + dir) * 2 + 1) * kTwSize;
            const uint64_t wbig = na_pow(wd, (uint64_t)kTwSize, p);
            uint64_t x = 1, y = 1;
            for (int i = 0; i < kTwSize; i++) {
                lo[i] = na_mont(x, p);
                hi[i] = na_mont(y, p);
                x = na_mul(x, wd, p);
                y = na_mul(y, wbig, p);
            }
            const uint64_t r64 = na_pow(wd, (uint64_t)1 << (kMaxLog - 6), p);
            uint64_t z = 1;
            for (int i = 0; i < 64; i++) { g_na_w64[pi][dir][i] = na_mont(z, p); z = na_mul(z, r64, p); }
            build_step1_tables(hi, g_na_tw_host + kHiLoWords + ((size_t)pi * 2 + dir) * kStep1Words);
        }
    }
    const uint64_t q0 = prime_value(0), q1 = prime_value(1), q2 = prime_value(2);
    g_na_garner[0] = na_mont(na_inv(q0 % q1, q1), q1);
    g_na_garner[1] = na_mont(q0 % q2, q2);
    g_na_garner[2] = na_mont(na_inv(na_mul(q0 % q2, q1 % q2, q2), q2), q2);
    g_na_host_ready = true;
}

// Once per device, with that device current: resolve the scratch address
// (the host-side name is not a device address) and upload the tables.
int setup_device(int dev, uint64_t **out, char *err, size_t errlen)
{
    if (dev < 0 || dev >= kMaxDevices) { snprintf(err, errlen, "device %d out of range", dev); return GBNTT_ERR_ARG; }
    if (g_na_ptr[dev]) { *out = g_na_ptr[dev]; return GBNTT_OK; }
    host_tables();
    void *ptr = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&ptr, g_noalloc_scratch);
    if (e != cudaSuccess || !ptr) {
        snprintf(err, errlen, "cudaGetSymbolAddress(scratch) failed: %s", cudaGetErrorString(e));
        return GBNTT_ERR_CUDA;
    }
    e = cudaMemcpy(ptr, g_na_tw_host, sizeof g_na_tw_host, cudaMemcpyHostToDevice);
    if (e != cudaSuccess) {
        snprintf(err, errlen, "twiddle upload to scratch failed: %s", cudaGetErrorString(e));
        return GBNTT_ERR_CUDA;
    }
    g_na_ptr[dev] = (uint64_t *)ptr;
    *out = (uint64_t *)ptr;
    return GBNTT_OK;
}

// Fixed pass plan for the lengths this entry point takes (L <= 16): one
// pass up to 2^10 points, otherwise two of ceil(L/2) and floor(L/2). It
// does not read the engine's plan-override table, which gbntt_set_plan and
// gbntt_autotune may rewrite from another thread; every plan gives the same
// product.
int local_plan(int L, int *p)
{
    if (L <= kMaxPassLog) { p[0] = L; return 1; }
    p[0] = (L + 1) / 2;
    p[1] = L / 2;
    return 2;
}

cudaError_t pass_launch(int pi, int log_l, int dir, int ld, PassArgs &a, cudaStream_t st)
{
    memcpy(a.w64, g_na_w64[pi][dir], sizeof a.w64);
    switch (pi) {
    case 0: return launch_pass_prime<0>(log_l, dir, ld, a, st);
    case 1: return launch_pass_prime<1>(log_l, dir, ld, a, st);
    default: return launch_pass_prime<2>(log_l, dir, ld, a, st);
    }
}

}  // namespace
}  // namespace gbntt

using namespace gbntt;

extern "C" int gbntt_mul_u32_noalloc(uint32_t *d_c, const uint32_t *d_a, size_t na, const uint32_t *d_b, size_t nb,
                                     void *stream)
{
    static char err[256];
    if (!d_c || (na && !d_a) || (nb && !d_b)) return GBNTT_ERR_ARG;
    cudaStream_t st = (cudaStream_t)stream;
    const size_t n_out = na + nb;
    if (na == 0 || nb == 0) {
        if (n_out && cudaMemsetAsync(d_c, 0, n_out * sizeof(uint32_t), st) != cudaSuccess) return GBNTT_ERR_CUDA;
        return GBNTT_OK;
    }
    if (na + nb - 1 > kNoAllocMaxN) {
        fprintf(stderr, "gbntt_mul_u32_noalloc: product needs %zu coefficients; this entry point is limited to "
                        "2^%d (use gbntt_mul_u32)\n", na + nb - 1, kNoAllocMaxLog);
        return GBNTT_ERR_SIZE;
    }
    int L = kMinLog;
    while (((size_t)1 << L) < na + nb - 1) L++;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return GBNTT_ERR_CUDA;
    uint64_t *base = nullptr;
    {
        std::lock_guard<std::mutex> lk(g_na_mu);
        const int rc = setup_device(dev, &base, err, sizeof err);
        if (rc) { fprintf(stderr, "gbntt_mul_u32_noalloc: %s\n", err); return rc; }
    }
    uint64_t *tw = base;
    uint64_t *specA = base + kTwWords;
    uint64_t *specB = specA + 3 * kNoAllocMaxN;
    unsigned *ctl = (unsigned *)(specA + kSpecWords);   // [0] ticket, [1] error, [2..] tile status
    const size_t stride = kNoAllocMaxN;

    PassArgs a;
    memset(&a, 0, sizeof a);
    int pl[kMaxPasses];
    const int np = local_plan(L, pl);
    const bool square = (d_a == d_b && na == nb);
    // forward transforms of both operands
    for (int op = 0; op < (square ? 1 : 2); op++) {
        uint64_t *spec = op ? specB : specA;
        for (int pi = 0; pi < 3; pi++) {
            a.data[pi] = spec + pi * stride;
            a.tw.hi[pi] = tw + (((size_t)pi * 2 + 0) * 2 + 0) * kTwSize;
            a.tw.lo[pi] = tw + (((size_t)pi * 2 + 0) * 2 + 1) * kTwSize;
            a.tw.st1[pi] = tw + kHiLoWords + ((size_t)pi * 2 + 0) * kStep1Words;
        }
        a.limbs = op ? d_b : d_a;
        a.n_limbs = (long long)(op ? nb : na);
        int log_m = L;
        for (int i = 0; i < np; i++) {
            a.log_m = log_m;
            a.log_s = log_m - pl[i];
            a.ncols = (long long)1 << (L - pl[i]);
            a.twiddle = a.log_s > 0;
            a.use_scale = 0;
            for (int pi = 0; pi < 3; pi++)
                if (pass_launch(pi, pl[i], 0, i == 0 ? LD_U32 : LD_U64, a, st) != cudaSuccess) return GBNTT_ERR_CUDA;
            log_m -= pl[i];
        }
    }
    // pointwise product and inverse transform in specA
    {
        int log_ms[3];
        int log_m = L;
        for (int i = 0; i < np; i++) { log_ms[i] = log_m; log_m -= pl[i]; }
        for (int pi = 0; pi < 3; pi++) {
            a.data[pi] = specA + pi * stride;
            a.other[pi] = (square ? specA : specB) + pi * stride;
            a.tw.hi[pi] = tw + (((size_t)pi * 2 + 1) * 2 + 0) * kTwSize;
            a.tw.lo[pi] = tw + (((size_t)pi * 2 + 1) * 2 + 1) * kTwSize;
            a.tw.st1[pi] = tw + kHiLoWords + ((size_t)pi * 2 + 1) * kStep1Words;
            const uint64_t p = prime_value(pi);
            a.scale[pi] = na_mont(na_mont(na_inv(((uint64_t)1 << L) % p, p), p), p);
        }
        for (int i = np - 1; i >= 0; i--) {
            a.log_m = log_ms[i];
            a.log_s = log_ms[i] - pl[i];
            a.ncols = (long long)1 << (L - pl[i]);
            a.twiddle = a.log_s > 0;
            a.use_scale = (i == 0);
            for (int pi = 0; pi < 3; pi++)
                if (pass_launch(pi, pl[i], 1, i == np - 1 ? LD_PW : LD_U64, a, st) != cudaSuccess) return GBNTT_ERR_CUDA;
        }
    }
    // Garner + carry; the ticket and the tile status words must start at
    // zero; the error word ctl[1] is left as it is (sticky until read)
    CarryArgs c;
    memset(&c, 0, sizeof c);
    for (int pi = 0; pi < 3; pi++) c.res[pi] = specA + pi * stride;
    c.out = d_c;
    c.n_coef = (long long)1 << L;
    c.n_out = (long long)n_out;
    c.ticket = ctl;
    c.error = ctl + 1;
    c.status = ctl + 2;
    for (int i = 0; i < 3; i++) c.garner[i] = g_na_garner[i];
    const long long nt = carry_tiles((long long)n_out);
    if (cudaMemsetAsync(ctl, 0, sizeof(unsigned), st) != cudaSuccess) return GBNTT_ERR_CUDA;
    if (cudaMemsetAsync(ctl + 2, 0, (size_t)nt * sizeof(unsigned), st) != cudaSuccess) return GBNTT_ERR_CUDA;
    if (launch_garner_carry(c, st, nullptr) != cudaSuccess) return GBNTT_ERR_CUDA;
    return GBNTT_OK;
}

namespace gbntt {

// Error bits the no-allocation multiply's device checks left on the current
// device (0 when it was never set up there; *set_up says which), cleared on
// read. Synchronises the device. Called by gbntt_device_errors.
int noalloc_read_errors(unsigned *flags, int *set_up)
{
    *flags = 0;
    *set_up = 0;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return GBNTT_ERR_CUDA;
    uint64_t *base = nullptr;
    {
        std::lock_guard<std::mutex> lk(g_na_mu);
        if (dev >= 0 && dev < kMaxDevices) base = g_na_ptr[dev];
    }
    if (!base) return GBNTT_OK;
    *set_up = 1;
    unsigned *err = (unsigned *)(base + kTwWords + kSpecWords) + 1;
    if (cudaDeviceSynchronize() != cudaSuccess) return GBNTT_ERR_CUDA;
    if (cudaMemcpy(flags, err, sizeof(unsigned), cudaMemcpyDeviceToHost) != cudaSuccess) return GBNTT_ERR_CUDA;
    if (cudaMemset(err, 0, sizeof(unsigned)) != cudaSuccess) return GBNTT_ERR_CUDA;
    return GBNTT_OK;
}

// Test hook for the bounded waits in this entry point's scratch: the carry
// kernel over three tiles with the ticket started at 1, so no CTA takes
// tile 0 and tile 1's look-back waits on a status word nothing writes. The
// wait runs out by itself and sets ERR_LOOKBACK_TIMEOUT in the scratch's
// error word (read back by gbntt_device_errors). Sets the scratch up first
// if needed. Synchronises.
int noalloc_debug_lookback_timeout(double *seconds)
{
    static char err[256];
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return GBNTT_ERR_CUDA;
    uint64_t *base = nullptr;
    {
        std::lock_guard<std::mutex> lk(g_na_mu);
        const int rc = setup_device(dev, &base, err, sizeof err);
        if (rc) return rc;
    }
    long long n_out = 1;
    while (carry_tiles(n_out) < 3) n_out *= 2;   // smallest power of two spanning three carry tiles
    if ((size_t)n_out > kNoAllocMaxN) return GBNTT_ERR_SIZE;
    uint64_t *specA = base + kTwWords;
    unsigned *ctl = (unsigned *)(specA + kSpecWords);
    CarryArgs c;
    memset(&c, 0, sizeof c);
    for (int pi = 0; pi < 3; pi++) c.res[pi] = specA + pi * kNoAllocMaxN;
    // output into operand B's spectrum area (scratch the check may overwrite)
    c.out = (uint32_t *)(specA + 3 * kNoAllocMaxN);
    c.n_coef = n_out;
    c.n_out = n_out;
    c.ticket = ctl;
    c.error = ctl + 1;
    c.status = ctl + 2;
    for (int i = 0; i < 3; i++) c.garner[i] = g_na_garner[i];
    const unsigned start = 1u;
    if (cudaDeviceSynchronize() != cudaSuccess) return GBNTT_ERR_CUDA;
    if (cudaMemset(ctl + 2, 0, 8 * sizeof(unsigned)) != cudaSuccess) return GBNTT_ERR_CUDA;
    if (cudaMemcpy(ctl, &start, sizeof start, cudaMemcpyHostToDevice) != cudaSuccess) return GBNTT_ERR_CUDA;
    const auto t0 = std::chrono::steady_clock::now();
    if (launch_garner_carry(c, nullptr, nullptr) != cudaSuccess) return GBNTT_ERR_CUDA;
    if (cudaDeviceSynchronize() != cudaSuccess) return GBNTT_ERR_CUDA;
    if (seconds) *seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    return GBNTT_OK;
}

}  // namespace gbntt

// Test hook (no counterpart in the reference): makes one carry look-back wait
// in the no-allocation multiply's scratch run out (see
// noalloc_debug_lookback_timeout) and reports the time it took; the error
// bit is then read with gbntt_device_errors.
extern "C" int gbntt_debug_noalloc_lookback_timeout(double *seconds)
{
    return gbntt::noalloc_debug_lookback_timeout(seconds);
}
