// gbntt_engine.cu — host side of the CRT-NTT multiply engine and its C ABI.
//
// Engine state is one process-wide object (as g_nms in the reference,
// ntt/lib/arith/ntt_mul.hip:312-347) guarded by a mutex, so concurrent host
// callers serialise here instead of relying on the caller's lock
// (ntt/lib/arith/multiply.c:27). Unlike the reference, the transform length
// is chosen per call (the smallest power of two >= n_a + n_b - 1, at least
// 32) instead of always the init-time maximum (ntt_mul.hip:1001-1002), and
// twiddle tables are two-level (2 x 2^15 entries per prime and direction,
// L2-resident) instead of O(N) host-built tables (ntt_mul.hip:189-308).
#include <cuda_runtime.h>
#include <array>
#include <map>
#include <mutex>
#include <tuple>
#include <vector>
#include <algorithm>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <deque>
#include <thread>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <stdarg.h>
#include <time.h>

#include "gbntt_arith.cuh"
#include "gbntt_internal.h"
#include "gbntt.h"

namespace gbntt {

typedef unsigned __int128 u128;

static uint64_t h_mul(uint64_t a, uint64_t b, uint64_t p) { return (uint64_t)((u128)a * b % p); }
static uint64_t h_pow(uint64_t b, uint64_t e, uint64_t p)
{
    uint64_t r = 1;
    b %= p;
    while (e) {
        if (e & 1) r = h_mul(r, b, p);
        b = h_mul(b, b, p);
        e >>= 1;
    }
    return r;
}
static uint64_t h_inv(uint64_t a, uint64_t p) { return h_pow(a % p, p - 2, p); }
static uint64_t h_mont(uint64_t x, uint64_t p) { return (uint64_t)(((u128)(x % p) << 64) % p); }
static const uint64_t kGen[3] = {7, 10, 19};   // reference PRIM_ROOT[0, 2, 3]
static const uint64_t kGen3 = 5;                 // primitive root of p3 = 3 * 2^30 + 1
static uint32_t h_mont3(uint64_t x) { return (uint32_t)(((x % kP3) << 32) % kP3); }   // x 2^32 mod p3

// Prime sets. Two primes (q0 with 64-bit residues, p3 with 32-bit residues)
// carry every product of 32-bit coefficients: q0 p3 ~ 2^95.6 exceeds the
// largest coefficient (< 2^93). The reference's three 64-bit primes stay
// for 64-bit coefficients (packed mode, bound 2^158) and on request.
struct PrimeSet {
    int n;
    int pi[3];
};
static const PrimeSet kSet2 = {2, {4, 3, 0}};       // lazy normal-form q0 + p3
static const PrimeSet kSet2m = {2, {0, 3, 0}};      // Montgomery q0 + p3
static const PrimeSet kSet3 = {3, {0, 1, 2}};

struct Engine {
    bool ready = false;
    int max_log = 0;
    size_t n_max = 0;
    uint64_t *d_spec = nullptr;     // 6 x n_max: spectra of operand A (3) then B (3)
    uint64_t *d_tw = nullptr;       // [prime 0..2, then normal-form q0][dir][hi|lo][2^15]
    uint32_t *d_tw3 = nullptr;      // p3: [dir][hi|lo][2^15]
    uint64_t *d_st1 = nullptr;      // step-1 tables: [table slot 0..3][dir][kStep1Words]
    uint32_t *d_st13 = nullptr;     // p3's: [dir][kStep1Words]
    int prime_set = 2;              // primes used for 32-bit coefficients: 2 or 3
    bool q0_lazy = false;           // two-prime set: q0 as prime 4 (lazy normal form) or 0 (Montgomery)
    bool overlap = true;            // two-prime set: second prime's passes on stream2
    bool zero_copy = true;          // host-pointer calls: kernels read/write pinned host memory directly
    bool stage_inputs = true;       // ... except the operands, copied once to HBM (B's copy overlaps A's transform)
    bool graphs = true;             // batched waves replayed as CUDA graphs
    bool fuse_inner = true;         // innermost forward passes, pointwise product and innermost inverse pass in one launch
    bool pass_tables = true;        // strided passes read their twiddles from pass tables (PassArgs::ptw)
    size_t ptw_budget = 0;          // ... up to this many bytes of tables in all
    bool radix3 = true;             // transforms of length 3 2^k where those are shorter than the next 2^L
    void *d_r3[5] = {};             // per prime: rho^(i 2^15) (3 2^15 words), then rho^i (2^15 words)
    uint64_t r3c[5] = {};           // per prime: c = (om - om^2) / 2 in its multiply form
    uint64_t r3rho[5] = {};         // per prime: rho (order 3 2^30), plain
    int r3_min_log = 20;            // radix-3 for c products of 3 2^k points when c 2^k >= 2^r3_min_log
    bool batch_split = true;        // uneven batch products split into chunk products
    int split_ratio_log = 3;        // ... when the longer operand is >= 2^this x the shorter
    uint64_t garner2[2] = {0, 0};   // two-prime Garner constants (p3 Montgomery multipliers)
    unsigned *d_ctl = nullptr;      // [0] ticket, [1] error, [2..] tile status
    size_t n_status = 0;
    uint32_t *d_io = nullptr;       // staging for host-pointer calls
    size_t io_words = 0;
    cudaStream_t stream = nullptr;
    cudaStream_t stream2 = nullptr;      // second prime's passes run here, overlapping the first's
    cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
    cudaStream_t cstream = nullptr;      // host -> device operand copies overlapping the transforms
    int sms = 152;                       // multiprocessors of the device (copy-kernel grids)
    cudaEvent_t ev_a = nullptr, ev_b = nullptr, ev_stage = nullptr;
    uint64_t garner[4] = {0, 0, 0, 0};
    uint64_t q01_lo = 0, q01_hi = 0;   // q0 * q1
    int bigint_coeff_bits = 32;        // coefficient width used by the BigInt entry points
    // batched calls: two slots of per-wave tables (device + pinned host)
    uint64_t *d_btab = nullptr;
    uint64_t *h_btab = nullptr;
    cudaEvent_t btab_ev[2] = {nullptr, nullptr};
    unsigned long dispatch = 0;
    // profiling (NTT_PROFILE=1): host wall clock per phase
    int prof = 0;
    double prof_ms[3] = {0, 0, 0};   // upload, compute, download
    long prof_calls = 0;
};

static Engine g;
// Montgomery forms of w_64^i per prime and direction (kernel arguments).
static uint64_t g_w64[5][2][64];

static cudaError_t launch_pass_any(int pi, int log_l, int dir, int ld, PassArgs &a, cudaStream_t st)
{
    memcpy(a.w64, g_w64[pi][dir], sizeof a.w64);
    switch (pi) {
    case 0: return launch_pass_prime<0>(log_l, dir, ld, a, st);
    case 1: return launch_pass_prime<1>(log_l, dir, ld, a, st);
    case 2: return launch_pass_prime<2>(log_l, dir, ld, a, st);
    case 3: return launch_pass_prime<3>(log_l, dir, ld, a, st);
    default: return launch_pass_prime<4>(log_l, dir, ld, a, st);
    }
}
static std::recursive_mutex g_mu;
static char g_err[512] = "";

static void set_err(const char *fmt, ...)
{
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_err, sizeof g_err, fmt, ap);
    va_end(ap);
}

void set_error_message(const char *msg) { snprintf(g_err, sizeof g_err, "%s", msg); }

#define CK(expr)                                                                              \
    do {                                                                                      \
        cudaError_t _e = (expr);                                                              \
        if (_e != cudaSuccess) {                                                              \
            set_err("CUDA error %d (%s) at %s:%d: %s", (int)_e, cudaGetErrorString(_e),        \
                    __FILE__, __LINE__, #expr);                                               \
            return GBNTT_ERR_CUDA;                                                            \
        }                                                                                     \
    } while (0)

// Optional per-launch CUDA-event records (kind, pass size, algorithmic bytes)
// for roofline reporting; off by default and never used in timed runs.
struct LaunchRec {
    int kind;       // 0 fwd first pass, 1 fwd pass, 2 inv first pass, 3 inv pass, 4 garner+carry,
                    // 5 fused innermost passes, 6 and 7 forward and inverse radix-3 stages
    int log_l;
    double bytes;   // algorithmic bytes moved by this launch
    cudaEvent_t e0, e1;
};
static bool g_rec_on = false;
static std::vector<LaunchRec> g_recs;

static void rec_begin(cudaStream_t st, int kind, int log_l, double bytes)
{
    if (!g_rec_on) return;
    LaunchRec r;
    r.kind = kind;
    r.log_l = log_l;
    r.bytes = bytes;
    cudaEventCreate(&r.e0);
    cudaEventCreate(&r.e1);
    cudaEventRecord(r.e0, st);
    g_recs.push_back(r);
}
static void rec_end(cudaStream_t st)
{
    if (!g_rec_on || g_recs.empty()) return;
    cudaEventRecord(g_recs.back().e1, st);
}

static double now_ms()
{
    timespec t;
    clock_gettime(CLOCK_MONOTONIC, &t);
    return t.tv_sec * 1e3 + t.tv_nsec * 1e-6;
}

static uint64_t *tw_ptr(int pi, int dir, int hi)
{
    return g.d_tw + (((size_t)pi * 2 + dir) * 2 + hi) * kTwSize;
}

// Pass twiddle tables (PassArgs::ptw), built on first use and kept until
// teardown: one per (prime, direction, sub-problem log, column-stride log,
// scaled). A strided pass then loads each element's twiddle w_M^(j m)
// instead of forming it from the two-level tables with one more Montgomery
// product per element. Tables are shared by every transform length whose
// plan has a pass of the same shape. Guarded by their own mutex: the server
// thread runs passes without the engine lock.
static std::map<std::tuple<int, int, int, int, int>, uint64_t *> g_ptw;
static std::mutex g_ptw_mu;
static size_t g_ptw_bytes = 0;

static cudaError_t launch_build_ptw_any(int pi, uint64_t *t, const uint64_t *hi, const uint64_t *lo, int log_m,
                                        int log_s, int scaled, uint64_t scale, cudaStream_t st)
{
    switch (pi) {
    case 0: return launch_build_pass_twiddles<0>(t, hi, lo, log_m, log_s, scaled, scale, st);
    case 1: return launch_build_pass_twiddles<1>(t, hi, lo, log_m, log_s, scaled, scale, st);
    case 2: return launch_build_pass_twiddles<2>(t, hi, lo, log_m, log_s, scaled, scale, st);
    case 3: return launch_build_pass_twiddles<3>(t, hi, lo, log_m, log_s, scaled, scale, st);
    default: return launch_build_pass_twiddles<4>(t, hi, lo, log_m, log_s, scaled, scale, st);
    }
}

// The table of one strided pass, or nullptr (tables off, over the budget,
// allocation failed, or a stream capture in progress: the pass then forms
// its twiddles itself). A new table is built on st and st is synchronised
// before the table is published, so any stream may use it afterwards.
// scaled: 0 none, 1 the outermost inverse pass's 2^-log_m, 2 that times 1/3
// (transforms of 3 2^k points); the value is `scale`, fixed by the key.
static const uint64_t *pass_table(int pi, int dir, int log_m, int log_s, int scaled, uint64_t scale, cudaStream_t st)
{
    if (!g.pass_tables || log_s <= 0) return nullptr;
    const auto key = std::make_tuple(pi, dir, log_m, log_s, scaled);
    std::lock_guard<std::mutex> lk(g_ptw_mu);
    const auto it = g_ptw.find(key);
    if (it != g_ptw.end()) return it->second;
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    if (cudaStreamIsCapturing(st, &cs) != cudaSuccess || cs != cudaStreamCaptureStatusNone) return nullptr;
    const size_t bytes = ((size_t)1 << log_m) * (pi == 3 ? 4 : 8);
    if (g_ptw_bytes + bytes > g.ptw_budget) return nullptr;
    uint64_t *d = nullptr;
    if (cudaMalloc(&d, bytes) != cudaSuccess) { cudaGetLastError(); return nullptr; }
    const uint64_t *hi, *lo;
    if (pi == 3) {
        hi = (const uint64_t *)(g.d_tw3 + ((size_t)dir * 2 + 0) * kTwSize);
        lo = (const uint64_t *)(g.d_tw3 + ((size_t)dir * 2 + 1) * kTwSize);
    } else {
        const int ts = pi == 4 ? 3 : pi;
        hi = tw_ptr(ts, dir, 0);
        lo = tw_ptr(ts, dir, 1);
    }
    cudaError_t e = launch_build_ptw_any(pi, d, hi, lo, log_m, log_s, scaled ? 1 : 0, scale, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) { cudaFree(d); cudaGetLastError(); return nullptr; }
    g_ptw[key] = d;
    g_ptw_bytes += bytes;
    return d;
}

static void free_pass_tables()
{
    std::lock_guard<std::mutex> lk(g_ptw_mu);
    for (auto &kv : g_ptw) cudaFree(kv.second);
    g_ptw.clear();
    g_ptw_bytes = 0;
}

// Per-length plan overrides (set by gbntt_set_plan, e.g. from an autotuner):
// [log_n][0] = pass count (0: default plan), [1..kMaxPasses] = pass sizes.
static int g_plan_override[kMaxLog + 1][1 + kMaxPasses];

int plan_passes(int log_n, int *p)
{
    if (log_n >= 0 && log_n <= kMaxLog && g_plan_override[log_n][0] > 0) {
        const int np = g_plan_override[log_n][0];
        for (int i = 0; i < np; i++) p[i] = g_plan_override[log_n][1 + i];
        return np;
    }
    if (log_n <= kMaxPassLog) { p[0] = log_n; return 1; }
    // 2^14 .. 2^30: the plans gbntt_autotune measured fastest on GB300 for
    // 2^(L-1) x 2^(L-1)-limb products (two-prime set, innermost passes
    // fused). Passes of 2^6 to 2^8 points beat 2^9 and 2^10 even at the cost
    // of a fourth pass: their register DFTs are shorter (fewer registers, a
    // smaller loop body), and the extra sweep over HBM is cheap next to the
    // integer work. With the innermost passes fused a larger innermost pass
    // pays (2^29: [7, 7, 7, 8] 51.8 ms, [7, 7, 8, 7] 53.3 ms).
    constexpr int kTunedLo = 14;
    static const signed char kTuned[kMaxLog + 1 - kTunedLo][1 + kMaxPasses] = {
        {2, 6, 8},       {2, 7, 8},       {2, 8, 8},       {3, 5, 6, 6},     // 2^14 .. 2^17
        {3, 6, 6, 6},    {3, 5, 6, 8},    {3, 6, 6, 8},    {3, 6, 7, 8},     // 2^18 .. 2^21
        {3, 7, 7, 8},    {3, 7, 8, 8},    {3, 8, 8, 8},    {3, 8, 9, 8},     // 2^22 .. 2^25
        {4, 7, 7, 6, 6}, {4, 7, 7, 7, 6}, {4, 7, 8, 7, 6}, {4, 7, 7, 7, 8},  // 2^26 .. 2^29
        {4, 7, 7, 8, 8},                                                    // 2^30
    };
    if (log_n >= kTunedLo && log_n <= kMaxLog) {
        const signed char *t = kTuned[log_n - kTunedLo];
        for (int i = 0; i < t[0]; i++) p[i] = t[1 + i];
        return t[0];
    }
    p[0] = (log_n + 1) / 2;
    p[1] = log_n / 2;
    return 2;
}

static int choose_log(size_t na, size_t nb)
{
    const size_t need = na + nb - 1;
    int L = kMinLog;
    while (((size_t)1 << L) < need) L++;
    return L;
}

// Products per batched wave and the 8-byte words of one wave's tables:
// limb pointers and lengths of A and B, output pointers and lengths,
// carry tile starts (W + 1).
constexpr int kMaxBatch = 16384;
constexpr size_t kBtabWords = 7 * (size_t)kMaxBatch + 64;   // + one end entry per sub-wave of a serving activation

// Carry tile status words for a workspace of n coefficients per prime: one
// product of n coefficients (64-bit limbs: n / 1024 tiles), or a batched
// wave of W <= kMaxBatch products of 2^L coefficients with W 2^L <= n, whose
// tiles sum to at most sum_b ceil((2^L + 1) / 2048) <= n / 2048 + 2 W.
static size_t status_words(size_t n)
{
    return (size_t)std::max(carry_tiles64((long long)n + 1), carry_tiles((long long)n + 1) + 2 * (long long)kMaxBatch) + 64;
}

static size_t workspace_bytes(int max_log)
{
    const size_t n = (size_t)1 << max_log;
    const size_t spec = 6 * n * sizeof(uint64_t);
    const size_t tw = 4 * 2 * 2 * (size_t)kTwSize * sizeof(uint64_t) + 2 * 2 * (size_t)kTwSize * sizeof(uint32_t) +
                      4 * 2 * (size_t)kStep1Words * sizeof(uint64_t) + 2 * (size_t)kStep1Words * sizeof(uint32_t) +
                      4 * (size_t)kTwSize * (2 * sizeof(uint64_t) + sizeof(uint32_t));   // radix-3 rho tables
    const size_t ctl = (2 + status_words(n)) * sizeof(unsigned);
    const size_t io = (4 * n + 64) * sizeof(uint32_t);
    return spec + tw + ctl + io;
}

static void invalidate_wave_graphs();

static void free_all()
{
    if (g.stream) cudaStreamSynchronize(g.stream);
    cudaFree(g.d_btab);
    if (g.h_btab) cudaFreeHost(g.h_btab);
    for (int i = 0; i < 2; i++) if (g.btab_ev[i]) cudaEventDestroy(g.btab_ev[i]);
    cudaFree(g.d_spec);
    cudaFree(g.d_tw);
    cudaFree(g.d_tw3);
    cudaFree(g.d_st1);
    cudaFree(g.d_st13);
    for (int i = 0; i < 5; i++) cudaFree(g.d_r3[i]);
    cudaFree(g.d_ctl);
    cudaFree(g.d_io);
    if (g.stream2) cudaStreamSynchronize(g.stream2);
    free_pass_tables();
    if (g.ev_fork) cudaEventDestroy(g.ev_fork);
    if (g.ev_join) cudaEventDestroy(g.ev_join);
    if (g.cstream) cudaStreamSynchronize(g.cstream);
    if (g.ev_a) cudaEventDestroy(g.ev_a);
    if (g.ev_b) cudaEventDestroy(g.ev_b);
    if (g.ev_stage) cudaEventDestroy(g.ev_stage);
    if (g.cstream) cudaStreamDestroy(g.cstream);
    if (g.stream2) cudaStreamDestroy(g.stream2);
    if (g.stream) cudaStreamDestroy(g.stream);
    invalidate_wave_graphs();
    g = Engine();
}

static int init_impl(int max_log)
{
    if (g.ready) return GBNTT_OK;
    if (max_log < kMinLog || max_log > kMaxLog) {
        set_err("gbntt_init: max_log32=%d outside [%d, %d]", max_log, kMinLog, kMaxLog);
        return GBNTT_ERR_ARG;
    }
    const char *pe = getenv("NTT_PROFILE");
    g.prof = pe ? atoi(pe) : 0;
    g.max_log = max_log;
    g.n_max = (size_t)1 << max_log;
    CK(cudaStreamCreateWithFlags(&g.stream, cudaStreamNonBlocking));
    CK(cudaStreamCreateWithFlags(&g.stream2, cudaStreamNonBlocking));
    CK(cudaEventCreateWithFlags(&g.ev_fork, cudaEventDisableTiming));
    CK(cudaEventCreateWithFlags(&g.ev_join, cudaEventDisableTiming));
    CK(cudaStreamCreateWithFlags(&g.cstream, cudaStreamNonBlocking));
    {
        int dev = 0, sms = 0;
        if (cudaGetDevice(&dev) == cudaSuccess &&
            cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) == cudaSuccess && sms > 0)
            g.sms = sms;
    }
    CK(cudaEventCreateWithFlags(&g.ev_a, cudaEventDisableTiming));
    CK(cudaEventCreateWithFlags(&g.ev_b, cudaEventDisableTiming));
    CK(cudaEventCreateWithFlags(&g.ev_stage, cudaEventDisableTiming));
    if (cudaMalloc(&g.d_spec, 6 * g.n_max * sizeof(uint64_t)) != cudaSuccess ||
        cudaMalloc(&g.d_tw, 4 * 2 * 2 * (size_t)kTwSize * sizeof(uint64_t)) != cudaSuccess ||
        cudaMalloc(&g.d_tw3, 2 * 2 * (size_t)kTwSize * sizeof(uint32_t)) != cudaSuccess ||
        cudaMalloc(&g.d_st1, 4 * 2 * (size_t)kStep1Words * sizeof(uint64_t)) != cudaSuccess ||
        cudaMalloc(&g.d_st13, 2 * (size_t)kStep1Words * sizeof(uint32_t)) != cudaSuccess) {
        set_err("gbntt_init: device allocation of %zu bytes failed", workspace_bytes(max_log));
        cudaGetLastError();
        free_all();
        return GBNTT_ERR_ALLOC;
    }
    g.n_status = status_words(g.n_max);
    g.io_words = 4 * g.n_max + 64;
    if (cudaMalloc(&g.d_ctl, (2 + g.n_status) * sizeof(unsigned)) != cudaSuccess ||
        cudaMalloc(&g.d_io, g.io_words * sizeof(uint32_t)) != cudaSuccess) {
        set_err("gbntt_init: device allocation of %zu bytes failed", workspace_bytes(max_log));
        cudaGetLastError();
        free_all();
        return GBNTT_ERR_ALLOC;
    }
    CK(cudaMemset(g.d_ctl, 0, (2 + g.n_status) * sizeof(unsigned)));
    if (cudaMalloc(&g.d_btab, 2 * kBtabWords * sizeof(uint64_t)) != cudaSuccess ||
        cudaMallocHost(&g.h_btab, 2 * kBtabWords * sizeof(uint64_t)) != cudaSuccess) {
        set_err("gbntt_init: batch table allocation failed");
        cudaGetLastError();
        free_all();
        return GBNTT_ERR_ALLOC;
    }
    for (int i = 0; i < 2; i++) CK(cudaEventCreateWithFlags(&g.btab_ev[i], cudaEventDisableTiming));

    // Twiddle tables and the w_64 constants.
    const size_t tw_words = 4 * 2 * 2 * (size_t)kTwSize;
    uint64_t *h = (uint64_t *)malloc(tw_words * sizeof(uint64_t));
    if (!h) { set_err("gbntt_init: host allocation failed"); free_all(); return GBNTT_ERR_ALLOC; }
    uint64_t (&w64)[5][2][64] = g_w64;
    // table slot 3 holds q0 in normal form (prime 4); slots 0..2 Montgomery
    for (int ts = 0; ts < 4; ts++) {
        const bool normal = ts == 3;
        const int pi = normal ? 4 : ts;   // prime index of this table slot
        const uint64_t p = prime_value(pi);
        const uint64_t w = h_pow(kGen[normal ? 0 : ts], (p - 1) >> kMaxLog, p);
        for (int dir = 0; dir < 2; dir++) {
            const uint64_t wd = dir ? h_inv(w, p) : w;
            uint64_t *hi = h + (((size_t)ts * 2 + dir) * 2 + 0) * kTwSize;
            uint64_t *lo = h + (((size_t)ts * 2 + dir) * 2 + 1) * kTwSize;
            const uint64_t wbig = h_pow(wd, (uint64_t)kTwSize, p);
            uint64_t x = 1, y = 1;
            for (int i = 0; i < kTwSize; i++) {
                lo[i] = normal ? x : h_mont(x, p);
                hi[i] = normal ? y : h_mont(y, p);
                x = h_mul(x, wd, p);
                y = h_mul(y, wbig, p);
            }
            const uint64_t r64 = h_pow(wd, (uint64_t)1 << (kMaxLog - 6), p);
            uint64_t z = 1;
            for (int i = 0; i < 64; i++) { w64[pi][dir][i] = normal ? z : h_mont(z, p); z = h_mul(z, r64, p); }
        }
    }
    // the q0 pass kernels multiply by w_64^k as the powers of two 2^(39k)
    // (inverse 2^(153k)): the root must be the one those exponents assume
    if (w64[0][0][1] != h_mont(h_pow(2, 39, prime_value(0)), prime_value(0)) ||
        w64[0][1][1] != h_mont(h_pow(2, 153, prime_value(0)), prime_value(0))) {
        free(h);
        set_err("gbntt_init: q0 root of unity does not match the power-of-two DFT constants");
        free_all();
        return GBNTT_ERR_ARG;
    }
    cudaError_t e = cudaMemcpy(g.d_tw, h, tw_words * sizeof(uint64_t), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) {
        std::vector<uint64_t> st(4 * 2 * (size_t)kStep1Words, 0);
        for (int td = 0; td < 8; td++)
            build_step1_tables(h + (size_t)td * 2 * kTwSize, st.data() + (size_t)td * kStep1Words);
        e = cudaMemcpy(g.d_st1, st.data(), st.size() * sizeof(uint64_t), cudaMemcpyHostToDevice);
    }
    free(h);
    if (e != cudaSuccess) { set_err("gbntt_init: twiddle upload failed: %s", cudaGetErrorString(e)); free_all(); return GBNTT_ERR_CUDA; }
    {
        // p3: the same two-level tables in its Montgomery form (R = 2^32)
        std::vector<uint32_t> h3(2 * 2 * (size_t)kTwSize);
        const uint64_t p = kP3;
        const uint64_t w = h_pow(kGen3, (p - 1) >> kMaxLog, p);
        for (int dir = 0; dir < 2; dir++) {
            const uint64_t wd = dir ? h_inv(w, p) : w;
            uint32_t *hi = h3.data() + ((size_t)dir * 2 + 0) * kTwSize;
            uint32_t *lo = h3.data() + ((size_t)dir * 2 + 1) * kTwSize;
            const uint64_t wbig = h_pow(wd, (uint64_t)kTwSize, p);
            uint64_t x = 1, y = 1;
            for (int i = 0; i < kTwSize; i++) {
                lo[i] = h_mont3(x);
                hi[i] = h_mont3(y);
                x = h_mul(x, wd, p);
                y = h_mul(y, wbig, p);
            }
            const uint64_t r64 = h_pow(wd, (uint64_t)1 << (kMaxLog - 6), p);
            uint64_t z = 1;
            for (int i = 0; i < 64; i++) { w64[3][dir][i] = h_mont3(z); z = h_mul(z, r64, p); }
        }
        e = cudaMemcpy(g.d_tw3, h3.data(), h3.size() * sizeof(uint32_t), cudaMemcpyHostToDevice);
        if (e == cudaSuccess) {
            std::vector<uint32_t> st(2 * (size_t)kStep1Words, 0);
            for (int dir = 0; dir < 2; dir++)
                build_step1_tables(h3.data() + (size_t)dir * 2 * kTwSize, st.data() + (size_t)dir * kStep1Words);
            e = cudaMemcpy(g.d_st13, st.data(), st.size() * sizeof(uint32_t), cudaMemcpyHostToDevice);
        }
        if (e != cudaSuccess) { set_err("gbntt_init: twiddle upload failed: %s", cudaGetErrorString(e)); free_all(); return GBNTT_ERR_CUDA; }
        // radix-3 stage: rho of order 3 2^30 for Montgomery q0 (0), normal-form
        // q0 (4) and p3 (3), two-level tables and constants in each form
        for (const int pi : {0, 4, 3}) {
            const uint64_t pp = prime_value(pi), gen = pi == 3 ? kGen3 : kGen[0];
            const uint64_t rho = h_pow(gen, (pp - 1) / (3ull << kMaxLog), pp);
            if (h_pow(rho, 3ull << kMaxLog, pp) != 1 || h_pow(rho, 1ull << kMaxLog, pp) == 1 ||
                h_pow(rho, 3ull << (kMaxLog - 1), pp) == 1) {
                set_err("gbntt_init: no root of order 3 2^30 for prime %d", pi);
                free_all();
                return GBNTT_ERR_ARG;
            }
            auto form = [&](uint64_t x) -> uint64_t { return pi == 3 ? h_mont3(x) : pi == 4 ? x % pp : h_mont(x, pp); };
            const size_t nhi = 3 * (size_t)kTwSize, nw = nhi + (size_t)kTwSize;
            std::vector<uint64_t> t(nw);
            const uint64_t big = h_pow(rho, (uint64_t)kTwSize, pp);
            uint64_t x = 1;
            for (size_t i = 0; i < nhi; i++) { t[i] = form(x); x = h_mul(x, big, pp); }
            x = 1;
            for (size_t i = 0; i < (size_t)kTwSize; i++) { t[nhi + i] = form(x); x = h_mul(x, rho, pp); }
            const size_t wb = pi == 3 ? 4 : 8;
            std::vector<uint32_t> t32;
            if (pi == 3) t32.assign(t.begin(), t.end());
            if (cudaMalloc(&g.d_r3[pi], nw * wb) != cudaSuccess ||
                cudaMemcpy(g.d_r3[pi], pi == 3 ? (const void *)t32.data() : (const void *)t.data(), nw * wb,
                           cudaMemcpyHostToDevice) != cudaSuccess) {
                set_err("gbntt_init: radix-3 table upload failed");
                cudaGetLastError();
                free_all();
                return GBNTT_ERR_CUDA;
            }
            const uint64_t om = h_pow(rho, 1ull << kMaxLog, pp), inv2 = h_inv(2, pp);
            const uint64_t om2 = h_mul(om, om, pp);
            const uint64_t c = h_mul(om >= om2 ? om - om2 : om + (pp - om2), inv2, pp);   // no 64-bit overflow for q0
            g.r3rho[pi] = rho;
            g.r3c[pi] = form(c);
        }
        // two-prime Garner: q0^-1 mod p3 and 2^64 mod p3 as p3 Montgomery multipliers
        const uint64_t q0 = prime_value(0);
        g.garner2[0] = h_mont3(h_inv(q0 % p, p));
        g.garner2[1] = (uint64_t)(((u128)1 << 64) % p);
    }

    // Garner constants (Montgomery forms):
    //   [0] q0^-1 mod q1, [1] q0 mod q2, [2] (q0 q1)^-1 mod q2.
    const uint64_t q0 = prime_value(0), q1 = prime_value(1), q2 = prime_value(2);
    g.garner[0] = h_mont(h_inv(q0 % q1, q1), q1);
    g.garner[1] = h_mont(q0 % q2, q2);
    g.garner[2] = h_mont(h_inv(h_mul(q0 % q2, q1 % q2, q2), q2), q2);
    g.garner[3] = 0;
    {
        const u128 q01 = (u128)q0 * q1;
        g.q01_lo = (uint64_t)q01;
        g.q01_hi = (uint64_t)(q01 >> 64);
    }
    {
        const char *cb = getenv("GBNTT_COEFF_BITS");
        g.bigint_coeff_bits = (cb && atoi(cb) == 64) ? 64 : 32;
        const char *ps = getenv("GBNTT_PRIMES");
        g.prime_set = (ps && atoi(ps) == 3) ? 3 : 2;
        // tuning knobs: q0 form in the two-prime set (Montgomery measured 94 ms
        // against 101 ms lazy at 2^28 limbs) and the two-stream overlap
        const char *qf = getenv("GBNTT_Q0_FORM");
        g.q0_lazy = qf && qf[0] == 'l';
        const char *ov = getenv("GBNTT_OVERLAP");
        g.overlap = !(ov && ov[0] == '0');
        // (measured at 2^28 limbs through ntt_bigint_mul: 105 ms against 110 ms
        // through the staging buffer)
        const char *bs = getenv("GBNTT_BATCH_SPLIT");
        g.batch_split = !(bs && bs[0] == '0');
        const char *sr = getenv("GBNTT_SPLIT_RATIO_LOG");
        g.split_ratio_log = sr ? std::max(1, atoi(sr)) : 3;
        const char *gr = getenv("GBNTT_GRAPHS");
        g.graphs = !(gr && gr[0] == '0');
        const char *si = getenv("GBNTT_STAGE_INPUTS");
        g.stage_inputs = !(si && si[0] == '0');
        const char *zc = getenv("GBNTT_ZERO_COPY");
        g.zero_copy = !(zc && zc[0] == '0');
        // pass twiddle tables: on unless GBNTT_PASS_TABLES=0; budget
        // GBNTT_PASS_TABLES_MB, else a quarter of the memory left after the
        // workspace (a 2^29-point multiply needs about 12 GiB of them)
        const char *fi = getenv("GBNTT_FUSE_INNER");
        g.fuse_inner = !(fi && fi[0] == '0');
        const char *r3 = getenv("GBNTT_RADIX3");
        g.radix3 = !(r3 && r3[0] == '0');
        const char *r3m = getenv("GBNTT_RADIX3_MIN_LOG");
        g.r3_min_log = r3m ? std::max(10, std::min(30, atoi(r3m))) : 20;
        const char *pt = getenv("GBNTT_PASS_TABLES");
        g.pass_tables = !(pt && pt[0] == '0');
        const char *pb = getenv("GBNTT_PASS_TABLES_MB");
        size_t fr = 0, tot = 0;
        if (pb) g.ptw_budget = (size_t)std::max(0L, atol(pb)) << 20;
        else if (cudaMemGetInfo(&fr, &tot) == cudaSuccess) g.ptw_budget = fr / 4;
    }
    g.ready = true;
    return GBNTT_OK;
}

static TwTables tables(const PrimeSet &ps, int dir)
{
    TwTables t;
    memset(&t, 0, sizeof t);
    for (int k = 0; k < ps.n; k++) {
        const int pi = ps.pi[k];
        if (pi != 3) {
            const int ts = pi == 4 ? 3 : pi;   // normal-form q0 tables sit in slot 3
            t.hi[k] = tw_ptr(ts, dir, 0);
            t.lo[k] = tw_ptr(ts, dir, 1);
            t.st1[k] = g.d_st1 + ((size_t)ts * 2 + dir) * kStep1Words;
        } else {
            t.hi[k] = (const uint64_t *)(g.d_tw3 + ((size_t)dir * 2 + 0) * kTwSize);
            t.lo[k] = (const uint64_t *)(g.d_tw3 + ((size_t)dir * 2 + 1) * kTwSize);
            t.st1[k] = (const uint64_t *)(g.d_st13 + (size_t)dir * kStep1Words);
        }
    }
    return t;
}

static const PrimeSet &coef32_set() { return g.prime_set == 3 ? kSet3 : (g.q0_lazy ? kSet2 : kSet2m); }
static double word_bytes(int pi) { return pi == 3 ? 4.0 : 8.0; }

// Overlap of the two-prime set: slot 1's passes go to an auxiliary stream
// forked from st before the first forward pass and joined back before the
// Garner+carry kernel, so the two primes' transforms share the SMs (q0's
// kernels are bound by the integer pipes, p3's by memory latency). forward
// and inverse take the forked stream (nullptr: everything on st).
static bool aux_used(const PrimeSet &ps, cudaStream_t aux)
{
    // per-launch event records (launch_log) need the launches serialised
    return aux && ps.n == 2 && g.overlap && !g_rec_on;
}
static cudaStream_t fork_aux(const PrimeSet &ps, cudaStream_t st, cudaStream_t aux)
{
    if (!aux_used(ps, aux)) return nullptr;
    if (cudaEventRecord(g.ev_fork, st) != cudaSuccess || cudaStreamWaitEvent(aux, g.ev_fork, 0) != cudaSuccess)
        return nullptr;
    return aux;
}
static int join_aux(cudaStream_t st, cudaStream_t aux)
{
    if (!aux) return GBNTT_OK;
    CK(cudaEventRecord(g.ev_join, aux));
    CK(cudaStreamWaitEvent(st, g.ev_join, 0));
    return GBNTT_OK;
}

// Forward transform of one operand: limbs -> one spectrum per prime of the
// set at spec[k * stride] (k = slot; p3's 32-bit words fill half a slot).
// stage (optional, single 32-bit-limb operands): the first prime's first
// pass also copies the limbs it reads into stage[0 .. n), and the other
// primes' first passes read that copy, so limbs in host memory cross
// NVLink-C2C once.
static int forward(const PrimeSet &ps, uint64_t *spec, size_t stride, const void *limbs, size_t n, int L,
                   cudaStream_t st, bool packed = false, long long W = 1, const uint32_t *const *limb_tab = nullptr,
                   const long long *len_tab = nullptr, cudaStream_t aux = nullptr, uint32_t *stage = nullptr,
                   bool preloaded = false, cudaEvent_t after_first = nullptr, bool skip_last = false)
{
    // after_first (optional): recorded on st once the first pass of the
    // first prime is enqueued (the operand's limbs have then been read)
    // preloaded: spec already holds the residues (the first pass reads them)
    // skip_last: leave the innermost pass to the fused kernel (inner_fused)
    int pl[kMaxPasses];
    const int np = plan_passes(L, pl) - (skip_last ? 1 : 0);
    PassArgs a;
    memset(&a, 0, sizeof a);
    for (int k = 0; k < ps.n; k++) a.data[k] = spec + k * stride;
    a.limbs = packed ? nullptr : (const uint32_t *)limbs;
    a.limbs64 = packed ? (const uint64_t *)limbs : nullptr;
    a.n_limbs = (long long)n;
    a.limb_tab = limb_tab;
    a.len_tab = len_tab;
    a.log_n_prod = L;
    a.tw = tables(ps, 0);
    int log_m = L;
    for (int i = 0; i < np; i++) {
        a.log_m = log_m;
        a.log_s = log_m - pl[i];
        a.ncols = W << (L - pl[i]);
        a.twiddle = a.log_s > 0;
        for (int k = 0; k < ps.n; k++) {
            const double nbw = word_bytes(ps.pi[k]) * (double)((size_t)1 << L) * (double)W;
            cudaStream_t sk = (aux && k == 1) ? aux : st;
            const bool staged = stage && i == 0 && !packed && W == 1;
            if (staged && k > 0) {
                a.limbs = stage;
                a.stage_out = nullptr;
                if (sk != st) {   // wait for the first prime's pass to fill the copy
                    CK(cudaEventRecord(g.ev_stage, st));
                    CK(cudaStreamWaitEvent(sk, g.ev_stage, 0));
                }
            } else {
                a.stage_out = staged ? stage : nullptr;
            }
            a.ptw[k] = a.twiddle ? pass_table(ps.pi[k], 0, a.log_m, a.log_s, 0, 0, sk) : nullptr;
            rec_begin(sk, i == 0 ? 0 : 1, pl[i], i == 0 ? (packed ? 8.0 : 4.0) * (double)n + nbw : 2.0 * nbw);
            const int ld0 = preloaded ? LD_U64 : (packed ? LD_U64LIMB : LD_U32);
            CK(launch_pass_any(ps.pi[k], pl[i], 0, i == 0 ? ld0 : LD_U64, a, sk));
            rec_end(sk);
        }
        if (i == 0 && after_first) CK(cudaEventRecord(after_first, st));
        a.stage_out = nullptr;
        log_m -= pl[i];
    }
    return GBNTT_OK;
}

// Pointwise product of the spectra and inverse transform, in place in specA.
// shared_b: specB holds one spectrum (2^L points) that every product of
// the wave multiplies by; pair_b: specB holds W / 2 spectra, spectrum i
// for products 2i and 2i + 1.
static int inverse(const PrimeSet &ps, uint64_t *specA, const uint64_t *specB, size_t stride, int L,
                   cudaStream_t st, bool square, long long W = 1, cudaStream_t aux = nullptr, bool shared_b = false,
                   bool skip_first = false, bool pair_b = false, bool third = false)
{
    // third: scale by (3 2^L)^-1 instead of 2^-L (the sub-transforms of a
    // 3 2^L-point transform; the inverse radix-3 stage then has no 1/3)
    // skip_first: the pointwise product and the innermost inverse pass were
    // done by the fused kernel (inner_fused); start at the next pass
    int pl[kMaxPasses];
    const int np = plan_passes(L, pl);
    PassArgs a;
    memset(&a, 0, sizeof a);
    a.other_log = shared_b ? L : 0;
    a.other_pair_log = !shared_b && pair_b ? L : 0;
    a.other_r3 = third && (shared_b || pair_b) ? 1 : 0;   // the shared spectra are per sub-transform
    for (int k = 0; k < ps.n; k++) {
        const int pi = ps.pi[k];
        a.data[k] = specA + k * stride;
        a.other[k] = specB + k * stride;
        // N^-1 * R^2: with the R^-1 left by the Montgomery pointwise product
        // the inverse output is scaled by exactly N^-1.
        const uint64_t p = prime_value(pi);
        const uint64_t ninv = h_inv(h_mul(((uint64_t)1 << L) % p, third ? 3 : 1, p), p);
        // (normal-form q0: the pointwise product leaves no factor, so N^-1 itself)
        a.scale[k] = pi < 3 ? h_mont(h_mont(ninv, p), p) : pi == 3 ? (uint64_t)h_mont3(h_mont3(ninv)) : ninv;
    }
    a.tw = tables(ps, 1);
    int log_ms[kMaxPasses];
    int log_m = L;
    for (int i = 0; i < np; i++) { log_ms[i] = log_m; log_m -= pl[i]; }
    for (int i = np - 1 - (skip_first ? 1 : 0); i >= 0; i--) {
        a.log_m = log_ms[i];
        a.log_s = log_ms[i] - pl[i];
        a.ncols = W << (L - pl[i]);
        a.twiddle = a.log_s > 0;
        a.use_scale = (i == 0);
        const bool first = (i == np - 1);   // the pointwise pass
        for (int k = 0; k < ps.n; k++) {
            const double nbw = word_bytes(ps.pi[k]) * (double)((size_t)1 << L) * (double)W;
            cudaStream_t sk = (aux && k == 1) ? aux : st;
            a.ptw[k] = a.twiddle ? pass_table(ps.pi[k], 1, a.log_m, a.log_s, a.use_scale ? (third ? 2 : 1) : 0,
                                              a.scale[k], sk)
                                 : nullptr;
            rec_begin(sk, first ? 2 : 3, pl[i], first ? (square ? 2.0 : 3.0) * nbw : 2.0 * nbw);
            CK(launch_pass_any(ps.pi[k], pl[i], 1, first ? LD_PW : LD_U64, a, sk));
            rec_end(sk);
        }
    }
    return GBNTT_OK;
}

// Whether a product of transform length 2^L runs its innermost passes
// fused (plans of two or more passes; off with GBNTT_FUSE_INNER=0).
static bool fuse_inner(int L)
{
    int pl[kMaxPasses];
    return g.fuse_inner && plan_passes(L, pl) >= 2;
}

// The innermost forward pass of specA and specB (specB == specA: a square),
// the pointwise product and the innermost inverse pass in one launch per
// prime, in place in specA (see ntt_inner_fused_kernel). Runs between
// forward(..., skip_last) of both operands and inverse(..., skip_first).
static int inner_fused(const PrimeSet &ps, uint64_t *specA, const uint64_t *specB, size_t stride, int L,
                       cudaStream_t st, bool square, long long W = 1, cudaStream_t aux = nullptr, bool pair_b = false,
                       bool r3 = false)
{
    // r3: W counts sub-transforms of 2^L points of products of 3 2^L (pairs
    // then share per sub-transform)
    int pl[kMaxPasses];
    const int np = plan_passes(L, pl);
    const int l = pl[np - 1];
    PassArgs a;
    memset(&a, 0, sizeof a);
    a.tw = tables(ps, 0);
    const TwTables ti = tables(ps, 1);
    for (int k = 0; k < ps.n; k++) {
        a.data[k] = specA + k * stride;
        a.other[k] = square ? specA + k * stride : specB + k * stride;
        a.st1_inv[k] = ti.st1[k];
    }
    a.log_m = l;
    a.log_s = 0;
    a.ncols = W << (L - l);
    a.other_pair_log = pair_b ? L : 0;   // products 2i and 2i + 1 read specB's spectrum i
    a.other_r3 = pair_b && r3 ? 1 : 0;
    for (int k = 0; k < ps.n; k++) {
        const int pi = ps.pi[k];
        const double nbw = word_bytes(pi) * (double)((size_t)1 << L) * (double)W;
        cudaStream_t sk = (aux && k == 1) ? aux : st;
        memcpy(a.w64, g_w64[pi][0], sizeof a.w64);
        memcpy(a.w64_inv, g_w64[pi][1], sizeof a.w64_inv);
        rec_begin(sk, 5, l, (square ? 2.0 : 3.0) * nbw);
        cudaError_t e;
        switch (pi) {
        case 0: e = launch_inner_fused_prime<0>(l, a, sk); break;
        case 1: e = launch_inner_fused_prime<1>(l, a, sk); break;
        case 2: e = launch_inner_fused_prime<2>(l, a, sk); break;
        case 3: e = launch_inner_fused_prime<3>(l, a, sk); break;
        default: e = launch_inner_fused_prime<4>(l, a, sk); break;
        }
        CK(e);
        rec_end(sk);
    }
    return GBNTT_OK;
}

// Garner constants and residue pointers of a prime set into c.
static void carry_setup(CarryArgs &c, const PrimeSet &ps, const uint64_t *specA, size_t stride)
{
    for (int k = 0; k < ps.n; k++) c.res[k] = specA + k * stride;
    c.mixed = ps.n == 2 ? 1 : 0;
    if (c.mixed) {
        c.garner[0] = g.garner2[0];
        c.garner[1] = g.garner2[1];
    } else {
        for (int i = 0; i < 4; i++) c.garner[i] = g.garner[i];
    }
}

static int carry(const PrimeSet &ps, uint32_t *d_c, size_t n_out, const uint64_t *specA, size_t stride, int L,
                 cudaStream_t st, long long n_coef = 0)
{
    // n_coef: coefficients of the transform (2^L unless given: 3 2^k)
    CarryArgs c;
    memset(&c, 0, sizeof c);
    carry_setup(c, ps, specA, stride);
    c.out = d_c;
    c.n_coef = n_coef ? n_coef : (long long)1 << L;
    c.n_out = (long long)n_out;
    c.ticket = g.d_ctl;
    c.error = g.d_ctl + 1;
    c.status = g.d_ctl + 2;
    const long long nt = carry_tiles((long long)n_out);
    CK(cudaMemsetAsync(g.d_ctl, 0, sizeof(unsigned), st));
    CK(cudaMemsetAsync(g.d_ctl + 2, 0, (size_t)nt * sizeof(unsigned), st));
    double rb = 0;
    for (int k = 0; k < ps.n; k++) rb += word_bytes(ps.pi[k]);
    rec_begin(st, 4, 0, rb * (double)((size_t)1 << L) + 4.0 * (double)n_out);
    CK(launch_garner_carry(c, st, nullptr));
    rec_end(st);
    return GBNTT_OK;
}

// b_ready (optional): an event the second operand's transform waits for
// (its host -> device copy on another stream).
// Host -> device copy of the second operand, issued by mul_dev once the
// first operand's first pass has read its limbs (both share the host link).
struct StageJob {
    uint32_t *dst = nullptr;
    const uint32_t *src = nullptr;   // device-mapped pinned memory, or a host pointer
    size_t n = 0;
    bool mapped = false;
};

// Sub-transform log k of a length-3 2^k transform for an n_a x n_b product
// when that is shorter than the power-of-two one (the product needs at most
// 3/4 of 2^L coefficients), else -1. Two-prime set, 2^k of at least 2^10.
// The radix-3 stage adds six launches and a sweep over the spectrum, which
// the quarter fewer points repay from about 2^20-point sub-transforms on
// (measured per product against the next power of two: 3 2^18 points
// 1.02 x, 3 2^19 0.99 x, 3 2^20 0.84 x, 3 2^22 0.81 x, 3 2^24 0.79 x): a
// product alone takes it from k = r3_min_log, a batch for c products of one
// length when c 2^k >= 2^r3_min_log (batch_mul).
static int r3_log(size_t na, size_t nb)
{
    if (!g.radix3 || g.prime_set != 2 || na == 0 || nb == 0) return -1;
    const int L = choose_log(na, nb);
    const int k = L - 2;
    if (k < 10 || (3ull << k) < na + nb - 1 || (3ull << k) > g.n_max) return -1;
    return k;
}

// The outer radix-3 stage of W products on each prime (gbntt_radix3.cu),
// on the streams the pass chain uses for them.
static int radix3_stage(const PrimeSet &ps, uint64_t *spec, size_t stride, int k, long long W, bool inverse,
                        const uint32_t *limbs, size_t n, const uint32_t *const *limb_tab, const long long *len_tab,
                        cudaStream_t st, cudaStream_t aux)
{
    for (int q = 0; q < ps.n; q++) {
        const int pi = ps.pi[q];
        if (!g.d_r3[pi]) {   // only q0 (both forms) and p3 have radix-3 tables
            set_err("radix-3 transform on prime %d (two-prime set only)", pi);
            return GBNTT_ERR_ARG;
        }
        R3Args a;
        memset(&a, 0, sizeof a);
        a.spec = spec + q * stride;
        a.M = 1LL << k;
        a.W = W;
        a.shift = kMaxLog - k;
        a.limbs = limbs;
        a.n_limbs = (long long)n;
        a.limb_tab = limb_tab;
        a.len_tab = len_tab;
        const size_t wb = pi == 3 ? 4 : 8;
        a.hi = g.d_r3[pi];
        a.lo = (const char *)g.d_r3[pi] + 3 * (size_t)kTwSize * wb;
        a.c = g.r3c[pi];
        // a thread steps through j, j + G, j + 2 G, ... (G = blocks x 256
        // threads): its twiddle is multiplied by w^(+-G) per step
        const long long per_block = 256LL * kR3Unroll;
        a.blocks = (int)std::min<long long>((a.M + per_block - 1) / per_block, 65535LL);
        const uint64_t pp = prime_value(pi), order = 3ull << kMaxLog;
        uint64_t e = (uint64_t)(((u128)(256ull * a.blocks) << a.shift) % order);
        if (inverse && e) e = order - e;
        const uint64_t step = h_pow(g.r3rho[pi], e, pp);
        a.step = pi == 3 ? h_mont3(step) : pi == 4 ? step : h_mont(step, pp);
        cudaStream_t sk = (aux && q == 1) ? aux : st;
        const double nbw = word_bytes(pi) * 3.0 * (double)a.M * (double)W;
        rec_begin(sk, inverse ? 7 : 6, 0, inverse ? 2.0 * nbw : nbw + 4.0 * (double)n);
        CK(launch_radix3(pi, inverse, a, sk));
        rec_end(sk);
    }
    return GBNTT_OK;
}

// c = a b through a transform of length 3 2^k: the radix-3 stage, three
// 2^k-point pass chains per operand (a batch of three for the pass
// kernels), the same fused and inverse passes, the inverse radix-3 stage,
// and Garner + carry over the 3 2^k coefficients.
static int r3_residues(const uint32_t *d_a, size_t na, const uint32_t *d_b, size_t nb, int k, cudaStream_t st,
                       const StageJob *stage_b, uint32_t *stage_a, int debug_mode = -1);

static int mul_dev_r3(uint32_t *d_c, const uint32_t *d_a, size_t na, const uint32_t *d_b, size_t nb, int k,
                      cudaStream_t st, const StageJob *stage_b, uint32_t *stage_a)
{
    const int rc = r3_residues(d_a, na, d_b, nb, k, st, stage_b, stage_a);
    if (rc) return rc;
    return carry(coef32_set(), d_c, na + nb, g.d_spec, g.n_max, k, st, 3LL << k);
}

// The residues of the product of length 3 2^k in the first slots of the
// workspace (q0 at d_spec, p3 at d_spec + n_max). debug_mode 0: only the
// forward and inverse radix-3 stages of A (3 A: the 1/3 is the inverse
// chain's).
static int r3_residues(const uint32_t *d_a, size_t na, const uint32_t *d_b, size_t nb, int k, cudaStream_t st,
                       const StageJob *stage_b, uint32_t *stage_a, int debug_mode)
{
    const bool square = (d_a == d_b && na == nb);
    if (stage_a) {   // A in pinned host memory: one pass over C2C into HBM, read there by both primes
        CK(launch_copy_words(stage_a, d_a, (long long)na, g.sms * 4, st));
        d_a = stage_a;
        if (square) d_b = stage_a;
    }
    uint64_t *specA = g.d_spec;
    uint64_t *specB = g.d_spec + 3 * g.n_max;
    const PrimeSet &ps = coef32_set();
    const bool fused = fuse_inner(k);
    cudaStream_t aux = fork_aux(ps, st, g.stream2);
    int rc = radix3_stage(ps, specA, g.n_max, k, 1, false, d_a, na, nullptr, nullptr, st, aux);
    if (rc) return rc;
    if (debug_mode == 0) {
        rc = radix3_stage(ps, specA, g.n_max, k, 1, true, nullptr, 0, nullptr, nullptr, st, aux);
        if (rc) return rc;
        return join_aux(st, aux);
    }
    if (stage_b && !square) CK(cudaEventRecord(g.ev_a, st));
    rc = forward(ps, specA, g.n_max, nullptr, 0, k, st, false, 3, nullptr, nullptr, aux, nullptr, true, nullptr, fused);
    if (rc) return rc;
    if (!square) {
        if (stage_b) {   // B's copy runs on the copy stream while A is transformed
            CK(cudaStreamWaitEvent(g.cstream, g.ev_a, 0));
            if (stage_b->mapped) CK(launch_copy_words(stage_b->dst, stage_b->src, (long long)stage_b->n, g.sms / 2, g.cstream));
            else CK(cudaMemcpyAsync(stage_b->dst, stage_b->src, stage_b->n * 4, cudaMemcpyHostToDevice, g.cstream));
            CK(cudaEventRecord(g.ev_b, g.cstream));
            CK(cudaStreamWaitEvent(st, g.ev_b, 0));
            if (aux) CK(cudaStreamWaitEvent(aux, g.ev_b, 0));
        }
        rc = radix3_stage(ps, specB, g.n_max, k, 1, false, d_b, nb, nullptr, nullptr, st, aux);
        if (rc) return rc;
        rc = forward(ps, specB, g.n_max, nullptr, 0, k, st, false, 3, nullptr, nullptr, aux, nullptr, true, nullptr,
                     fused);
        if (rc) return rc;
    }
    if (fused) {
        rc = inner_fused(ps, specA, square ? specA : specB, g.n_max, k, st, square, 3, aux);
        if (rc) return rc;
    }
    rc = inverse(ps, specA, square ? specA : specB, g.n_max, k, st, square, 3, aux, false, fused, false, true);
    if (rc) return rc;
    rc = radix3_stage(ps, specA, g.n_max, k, 1, true, nullptr, 0, nullptr, nullptr, st, aux);
    if (rc) return rc;
    return join_aux(st, aux);
}

// stage_a (optional): HBM copy of A made by its first pass (see forward).
// stage_b (optional): copy of B into d_b, run on the copy stream while A is
// transformed.
static int mul_dev(uint32_t *d_c, const uint32_t *d_a, size_t na, const uint32_t *d_b, size_t nb, cudaStream_t st,
                   const StageJob *stage_b = nullptr, uint32_t *stage_a = nullptr)
{
    if (!g.ready) { set_err("engine not initialised"); return GBNTT_ERR_NOT_INIT; }
    if (!st) st = g.stream;
    const size_t n_out = na + nb;
    if (na == 0 || nb == 0) {
        if (n_out) CK(cudaMemsetAsync(d_c, 0, n_out * sizeof(uint32_t), st));
        return GBNTT_OK;
    }
    const int L = choose_log(na, nb);
    if (L > g.max_log) {
        set_err("product needs %zu coefficients but the engine was initialised for 2^%d", na + nb - 1, g.max_log);
        return GBNTT_ERR_SIZE;
    }
    const int k3 = r3_log(na, nb);
    if (k3 >= g.r3_min_log) return mul_dev_r3(d_c, d_a, na, d_b, nb, k3, st, stage_b, stage_a);
    const bool square = (d_a == d_b && na == nb);
    uint64_t *specA = g.d_spec;
    uint64_t *specB = g.d_spec + 3 * g.n_max;
    const PrimeSet &ps = coef32_set();
    const bool fused = fuse_inner(L);
    cudaStream_t aux = fork_aux(ps, st, g.stream2);
    int rc = forward(ps, specA, g.n_max, d_a, na, L, st, false, 1, nullptr, nullptr, aux, stage_a, false,
                     stage_b ? g.ev_a : nullptr, fused);
    if (rc) return rc;
    if (!square) {
        if (stage_b) {
            CK(cudaStreamWaitEvent(g.cstream, g.ev_a, 0));
            if (stage_b->mapped) CK(launch_copy_words(stage_b->dst, stage_b->src, (long long)stage_b->n, g.sms / 2, g.cstream));
            else CK(cudaMemcpyAsync(stage_b->dst, stage_b->src, stage_b->n * 4, cudaMemcpyHostToDevice, g.cstream));
            CK(cudaEventRecord(g.ev_b, g.cstream));
            CK(cudaStreamWaitEvent(st, g.ev_b, 0));
            if (aux) CK(cudaStreamWaitEvent(aux, g.ev_b, 0));
        }
        rc = forward(ps, specB, g.n_max, d_b, nb, L, st, false, 1, nullptr, nullptr, aux, nullptr, false, nullptr,
                     fused);
        if (rc) return rc;
    }
    if (fused) {
        rc = inner_fused(ps, specA, square ? specA : specB, g.n_max, L, st, square, 1, aux);
        if (rc) return rc;
    }
    rc = inverse(ps, specA, square ? specA : specB, g.n_max, L, st, square, 1, aux, false, fused);
    if (rc) return rc;
    rc = join_aux(st, aux);
    if (rc) return rc;
    return carry(ps, d_c, n_out, specA, g.n_max, L, st);
}

static int carry64(uint64_t *d_c, size_t n_out, const uint64_t *specA, size_t stride, int L, cudaStream_t st)
{
    CarryArgs c;
    memset(&c, 0, sizeof c);
    for (int pi = 0; pi < 3; pi++) c.res[pi] = specA + pi * stride;
    c.out64 = d_c;
    c.n_coef = (long long)1 << L;
    c.n_out = (long long)n_out;
    c.ticket = g.d_ctl;
    c.error = g.d_ctl + 1;
    c.status = g.d_ctl + 2;
    for (int i = 0; i < 4; i++) c.garner[i] = g.garner[i];
    c.q01_lo = g.q01_lo;
    c.q01_hi = g.q01_hi;
    const long long nt = carry_tiles64((long long)n_out);
    CK(cudaMemsetAsync(g.d_ctl, 0, sizeof(unsigned), st));
    CK(cudaMemsetAsync(g.d_ctl + 2, 0, (size_t)nt * sizeof(unsigned), st));
    rec_begin(st, 4, 0, 3.0 * 8.0 * (double)((size_t)1 << L) + 8.0 * (double)n_out);
    CK(launch_garner_carry64(c, st, nullptr));
    rec_end(st);
    return GBNTT_OK;
}

// Packed mode: one 64-bit limb per coefficient (the reference's own
// granularity), transform length >= n_a + n_b - 1 in 64-bit limbs.
static int mul_dev64(uint64_t *d_c, const uint64_t *d_a, size_t na, const uint64_t *d_b, size_t nb, cudaStream_t st)
{
    if (!g.ready) { set_err("engine not initialised"); return GBNTT_ERR_NOT_INIT; }
    if (!st) st = g.stream;
    const size_t n_out = na + nb;
    if (na == 0 || nb == 0) {
        if (n_out) CK(cudaMemsetAsync(d_c, 0, n_out * sizeof(uint64_t), st));
        return GBNTT_OK;
    }
    const int L = choose_log(na, nb);
    if (L > g.max_log) {
        set_err("product needs %zu coefficients but the engine was initialised for 2^%d", na + nb - 1, g.max_log);
        return GBNTT_ERR_SIZE;
    }
    const bool square = (d_a == d_b && na == nb);
    uint64_t *specA = g.d_spec;
    uint64_t *specB = g.d_spec + 3 * g.n_max;
    const bool fused = fuse_inner(L);
    int rc = forward(kSet3, specA, g.n_max, d_a, na, L, st, true, 1, nullptr, nullptr, nullptr, nullptr, false, nullptr,
                     fused);
    if (rc) return rc;
    if (!square) {
        rc = forward(kSet3, specB, g.n_max, d_b, nb, L, st, true, 1, nullptr, nullptr, nullptr, nullptr, false, nullptr,
                     fused);
        if (rc) return rc;
    }
    if (fused) {
        rc = inner_fused(kSet3, specA, square ? specA : specB, g.n_max, L, st, square);
        if (rc) return rc;
    }
    rc = inverse(kSet3, specA, square ? specA : specB, g.n_max, L, st, square, 1, nullptr, false, fused);
    if (rc) return rc;
    return carry64(d_c, n_out, specA, g.n_max, L, st);
}

// Batched products: bucket by transform length, then run waves of up to
// W = min(kMaxBatch, cap / N) products through the same pass kernels (a
// wave of W transforms of N points is, for a pass, W N / 2^l columns; a wave
// of W transforms of 3 2^k points is 3 W sub-transforms of 2^k) and the
// batched carry kernel. Per-product pointers and lengths travel in device
// tables, so every launch of a wave has fixed arguments. A context is one
// workspace (the engine's, or a slice of it owned by a serving slot).
struct BatchCtx {
    uint64_t *spec;              // 6 x cap words: A (3 x cap) then B (3 x cap)
    size_t cap;                  // coefficients per prime per operand
    unsigned *ctl;               // [0] ticket, [1] error, [2..] carry tile status
    size_t n_status;             // status words after ctl[2]
    uint64_t *d_btab, *h_btab;   // two table slots (device, pinned host)
    cudaEvent_t *btab_ev;        // two events guarding the host slots
    int *slot;
};

struct BatchItem {
    uint32_t *c;
    const uint32_t *a, *b;
    size_t na, nb;
    size_t nc = 0;   // limbs written to c: na + nb when 0 (a cyclic product writes 2^L + 3)
};

static inline size_t out_limbs(const BatchItem &it) { return it.nc ? it.nc : it.na + it.nb; }

static int wave_launches(BatchCtx &x, uint64_t *dtab, long long W, int L, cudaStream_t st, cudaStream_t aux_stream,
                         long long tiles, bool shared_b, bool pair_b = false, bool r3 = false);
static int wave_graph(BatchCtx &x, uint64_t *dtab, long long W, int L, cudaStream_t st, cudaStream_t aux_stream,
                      long long tiles, bool shared_b, bool pair_b = false, bool r3 = false);

// One wave of W products, all of transform length 2^L (r3: 3 2^L), on
// stream st.
static int batch_wave(BatchCtx &x, const BatchItem *items, long long W, int L, cudaStream_t st,
                      cudaStream_t aux_stream = nullptr, bool r3 = false)
{
    const int slot = *x.slot;
    CK(cudaEventSynchronize(x.btab_ev[slot]));
    uint64_t *h = x.h_btab + slot * kBtabWords;
    uint64_t *dtab = x.d_btab + slot * kBtabWords;
    uint64_t *hA = h, *hLA = h + W, *hB = h + 2 * W, *hLB = h + 3 * W, *hC = h + 4 * W, *hNC = h + 5 * W,
             *hTS = h + 6 * W;
    long long tiles = 0;
    // every product multiplying by the same right operand (a division by a
    // shared divisor or reciprocal): its transform is computed once; products
    // 2i and 2i + 1 multiplying by the same one (a product tree's B_L B_R and
    // P_L B_R): one transform per pair
    bool shared_b = W > 1;
    bool pair_b = W > 1 && W % 2 == 0;
    for (long long k = 0; k < W; k++) {
        const BatchItem &it = items[k];
        const BatchItem &mate = items[k ^ 1];
        if (pair_b && (it.b != mate.b || it.nb != mate.nb || it.a == it.b)) pair_b = false;
        if (it.b != items[0].b || it.nb != items[0].nb || it.a == it.b) shared_b = false;
        hA[k] = (uint64_t)(uintptr_t)it.a;
        hLA[k] = (uint64_t)it.na;
        hB[k] = (uint64_t)(uintptr_t)it.b;
        hLB[k] = (uint64_t)it.nb;
        hC[k] = (uint64_t)(uintptr_t)it.c;
        hNC[k] = (uint64_t)out_limbs(it);
        hTS[k] = (uint64_t)tiles;
        tiles += carry_tiles((long long)out_limbs(it));
    }
    hTS[W] = (uint64_t)tiles;
    if ((size_t)tiles > x.n_status) {
        set_err("batched wave needs %lld carry tiles; workspace holds %zu", tiles, x.n_status);
        return GBNTT_ERR_SIZE;
    }
    if (shared_b) pair_b = false;
    if (pair_b)   // the right operands of the pairs, one table entry each
        for (long long k = 0; k < W / 2; k++) {
            hB[k] = (uint64_t)(uintptr_t)items[2 * k].b;
            hLB[k] = (uint64_t)items[2 * k].nb;
        }
    CK(cudaMemcpyAsync(dtab, h, (7 * (size_t)W + 1) * sizeof(uint64_t), cudaMemcpyHostToDevice, st));
    CK(cudaEventRecord(x.btab_ev[slot], st));
    *x.slot = slot ^ 1;
    if (g.graphs && !g_rec_on) return wave_graph(x, dtab, W, L, st, aux_stream, tiles, shared_b, pair_b, r3);
    return wave_launches(x, dtab, W, L, st, aux_stream, tiles, shared_b, pair_b, r3);
}

// The launches of one wave after its table upload: both operands' forward
// transforms, the fused pointwise product and inverse, the batched carry
// kernel over `tiles` carry tiles.
static int wave_launches(BatchCtx &x, uint64_t *dtab, long long W, int L, cudaStream_t st, cudaStream_t aux_stream,
                         long long tiles, bool shared_b, bool pair_b, bool r3)
{
    uint64_t *specA = x.spec, *specB = x.spec + 3 * x.cap;
    const PrimeSet &ps = coef32_set();
    cudaStream_t aux = fork_aux(ps, st, aux_stream);
    int rc = GBNTT_OK;
    if (r3) {
        // products of length 3 2^L: each operand's radix-3 stage, then its
        // three sub-transforms as a batch of 3 W for the pass chain (a
        // shared right operand: one product's three; pairs: W / 2 products')
        const bool fused = !shared_b && fuse_inner(L);
        for (int o = 0; o < 2; o++) {
            uint64_t *spec = o ? specB : specA;
            const long long Wo = o == 0 ? W : shared_b ? 1 : pair_b ? W / 2 : W;
            rc = radix3_stage(ps, spec, x.cap, L, Wo, false, nullptr, 0, (const uint32_t *const *)(dtab + 2 * o * W),
                              (const long long *)(dtab + (2 * o + 1) * W), st, aux);
            if (rc) return rc;
            rc = forward(ps, spec, x.cap, nullptr, 0, L, st, false, 3 * Wo, nullptr, nullptr, aux, nullptr, true,
                         nullptr, fused);
            if (rc) return rc;
        }
        if (fused && (rc = inner_fused(ps, specA, specB, x.cap, L, st, false, 3 * W, aux, pair_b, true)) != GBNTT_OK)
            return rc;
        if ((rc = inverse(ps, specA, specB, x.cap, L, st, false, 3 * W, aux, shared_b, fused, pair_b, true)) !=
            GBNTT_OK)
            return rc;
        if ((rc = radix3_stage(ps, specA, x.cap, L, W, true, nullptr, 0, nullptr, nullptr, st, aux)) != GBNTT_OK)
            return rc;
    } else {
        // a shared right operand is transformed once and read by every
        // product's pointwise pass, so it keeps the unfused innermost passes
        const bool fused = !shared_b && fuse_inner(L);
        rc = forward(ps, specA, x.cap, nullptr, 0, L, st, false, W, (const uint32_t *const *)(dtab),
                     (const long long *)(dtab + W), aux, nullptr, false, nullptr, fused);
        if (rc) return rc;
        // shared right operand: one transform (table entry 0), read by every
        // product's pointwise pass; pairs: W / 2 transforms (entries 0 .. W/2 - 1)
        rc = forward(ps, specB, x.cap, nullptr, 0, L, st, false, shared_b ? 1 : pair_b ? W / 2 : W,
                     (const uint32_t *const *)(dtab + 2 * W), (const long long *)(dtab + 3 * W), aux, nullptr, false,
                     nullptr, fused);
        if (rc) return rc;
        if (fused) {
            rc = inner_fused(ps, specA, specB, x.cap, L, st, false, W, aux, pair_b);
            if (rc) return rc;
        }
        rc = inverse(ps, specA, specB, x.cap, L, st, false, W, aux, shared_b, fused, pair_b);
        if (rc) return rc;
    }
    rc = join_aux(st, aux);
    if (rc) return rc;
    CarryArgs c;
    memset(&c, 0, sizeof c);
    carry_setup(c, ps, specA, x.cap);
    c.ticket = x.ctl;
    c.error = x.ctl + 1;
    c.status = x.ctl + 2;
    c.tile_start = (const long long *)(dtab + 6 * W);
    c.out_tab = (uint32_t *const *)(dtab + 4 * W);
    c.nout_tab = (const long long *)(dtab + 5 * W);
    c.nprod = (int)W;
    c.log_n_prod = L;
    c.radix3 = r3 ? 1 : 0;
    CK(cudaMemsetAsync(x.ctl, 0, sizeof(unsigned), st));
    CK(cudaMemsetAsync(x.ctl + 2, 0, (size_t)tiles * sizeof(unsigned), st));
    double rb = 0;
    for (int k = 0; k < ps.n; k++) rb += word_bytes(ps.pi[k]);
    const double npt = (double)((r3 ? 3LL : 1LL) << L);
    rec_begin(st, 4, 0, (rb * npt + 4.0 * npt) * (double)W);
    CK(launch_garner_carry_batch(c, tiles, st));
    rec_end(st);
    return GBNTT_OK;
}

// CUDA-graph form of a wave: the launch sequence is captured the second time
// a (context, table slot, transform length, wave size, prime set) key comes
// up (the first run is launched directly, which also performs any one-time
// kernel attribute setup outside a capture) and is replayed with one
// cudaGraphLaunch from then on. Every argument of the captured launches is
// fixed for the key: the tables live at the slot's device address and are
// refreshed by the upload that precedes each replay, and the carry grid is
// the key's upper bound on carry tiles, W ceil((2^L + 1) / 2048) (3 2^L for
// a radix-3 wave), whose surplus CTAs take the highest tickets and exit at
// once. Anything that
// changes the captured launches (plans, prime set, freed contexts) drops the
// cache through invalidate_wave_graphs().
struct WaveKey {
    const uint64_t *spec;
    const uint64_t *dtab;
    const unsigned *ctl;
    size_t cap;
    int L;
    long long W;
    int primes;
    bool operator<(const WaveKey &o) const
    {
        return std::tie(spec, dtab, ctl, cap, L, W, primes) < std::tie(o.spec, o.dtab, o.ctl, o.cap, o.L, o.W, o.primes);
    }
};
struct WaveGraph {
    cudaGraphExec_t exec = nullptr;
    int runs = 0;
};
static std::map<WaveKey, WaveGraph> g_wave_graphs;
static std::mutex g_wave_graphs_mu;
constexpr size_t kMaxWaveGraphs = 512;

static void invalidate_wave_graphs()
{
    std::lock_guard<std::mutex> lk(g_wave_graphs_mu);
    for (auto &kv : g_wave_graphs)
        if (kv.second.exec) cudaGraphExecDestroy(kv.second.exec);   // in-flight replays finish first
    g_wave_graphs.clear();
}

static int wave_graph(BatchCtx &x, uint64_t *dtab, long long W, int L, cudaStream_t st, cudaStream_t aux_stream,
                      long long tiles, bool shared_b, bool pair_b, bool r3)
{
    const PrimeSet &ps = coef32_set();
    const long long ub = W * carry_tiles(((r3 ? 3LL : 1LL) << L) + 1);
    if ((size_t)ub > x.n_status) return wave_launches(x, dtab, W, L, st, aux_stream, tiles, shared_b, pair_b, r3);
    const bool aux = aux_used(ps, aux_stream);
    const WaveKey key{x.spec, dtab, x.ctl, x.cap, L, W,
                      ps.n * 16 + ps.pi[0] * 4 + ps.pi[1] + (aux ? 256 : 0) + (shared_b ? 512 : 0) +
                          (pair_b ? 1024 : 0) + (r3 ? 2048 : 0)};
    cudaGraphExec_t exec = nullptr;
    {
        std::lock_guard<std::mutex> lk(g_wave_graphs_mu);
        WaveGraph &wg = g_wave_graphs[key];
        exec = wg.exec;
        if (!exec && wg.runs++ == 0) exec = (cudaGraphExec_t)-1;
    }
    if (exec == (cudaGraphExec_t)-1) return wave_launches(x, dtab, W, L, st, aux_stream, tiles, shared_b, pair_b, r3);
    if (!exec) {
        CK(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
        const int rc = wave_launches(x, dtab, W, L, st, aux_stream, ub, shared_b, pair_b, r3);
        cudaGraph_t graph = nullptr;
        const cudaError_t e = cudaStreamEndCapture(st, &graph);
        if (rc != GBNTT_OK || e != cudaSuccess) {
            if (graph) cudaGraphDestroy(graph);
            (void)cudaGetLastError();
            if (rc != GBNTT_OK) return rc;
            CK(e);
        }
        const cudaError_t ei = cudaGraphInstantiate(&exec, graph, 0);
        cudaGraphDestroy(graph);
        CK(ei);
        std::lock_guard<std::mutex> lk(g_wave_graphs_mu);
        if (g_wave_graphs.size() >= kMaxWaveGraphs) {
            for (auto &kv : g_wave_graphs)
                if (kv.second.exec) cudaGraphExecDestroy(kv.second.exec);
            g_wave_graphs.clear();
        }
        g_wave_graphs[key].exec = exec;
        g_wave_graphs[key].runs = 2;
    }
    CK(cudaGraphLaunch(exec, st));
    return GBNTT_OK;
}

static int g_batch_slot = 0;

// Uneven products in a batch: a product whose longer operand (nB limbs) is
// at least 2^split_ratio_log times its shorter one (nS limbs, at least
// kSplitMinShort) and whose transform would be longer than the chunks' is
// split into chunk products: the longer operand in
// chunks of 2^ls - nS + 1 limbs (2^ls = 4 x the power of two >= nS), each
// multiplied by the shorter operand at transform length 2^ls, so a
// 2^21 x 2^13 product becomes 86 products of 2^15 points (the shorter
// operand, common to all chunks of a wave, is transformed once) instead of
// three transforms of 2^22 points. Even-numbered chunk products land
// side by side in one buffer E and odd-numbered ones in O (consecutive
// chunk products overlap by nS limbs, every second one does not), and the
// product is E + O by one batched carry-propagating addition.
constexpr size_t kSplitMinShort = 64;

// wrap_log (optional): items with wrap_log[i] > 0 are cyclic products,
// c = a b mod (beta^(2^L) - 1) at transform length 2^L = 2^wrap_log[i] (na,
// nb <= 2^L): the transform's cyclic convolution carried into 2^L + 3
// limbs, the top 3 limbs being the carry past limb 2^L - 1 (not folded).
static int batch_mul(uint32_t *const *d_c, const uint32_t *const *d_a, const size_t *na,
                     const uint32_t *const *d_b, const size_t *nb, int count, cudaStream_t st,
                     const int *wrap_log = nullptr)
{
    if (!g.ready) { set_err("engine not initialised"); return GBNTT_ERR_NOT_INIT; }
    if (count < 0 || (count > 0 && (!d_c || !d_a || !na || !d_b || !nb))) { set_err("bad batch arguments"); return GBNTT_ERR_ARG; }
    if (!st) st = g.stream;
    struct Keyed {
        int L;
        long long group;   // items of one split stay together (shared operand per wave)
        BatchItem item;
        int paired = 0;    // with its neighbour in the batch: the same right operand, one transform
        int chunk = 0;     // a chunk product of a split
        int r3 = 0;        // transform length 3 2^L
    };
    struct Split {
        uint32_t *E, *O, *c;
        long long n;
    };
    std::vector<Keyed> all;
    std::vector<Split> splits;
    all.reserve(count);
    int rc = GBNTT_OK;
    for (int i = 0; i < count && rc == GBNTT_OK; i++) {
        const int wl = wrap_log ? wrap_log[i] : 0;
        if (wl) {
            if (wl < kMinLog || wl > g.max_log || na[i] > ((size_t)1 << wl) || nb[i] > ((size_t)1 << wl)) {
                set_err("cyclic batch product %d: operands of %zu and %zu limbs at 2^%d (engine 2^%d..2^%d)", i,
                        na[i], nb[i], wl, kMinLog, g.max_log);
                rc = GBNTT_ERR_SIZE;
                break;
            }
            const size_t nc = ((size_t)1 << wl) + 3;
            if (na[i] == 0 || nb[i] == 0) {
                CK(cudaMemsetAsync(d_c[i], 0, nc * sizeof(uint32_t), st));
                continue;
            }
            BatchItem it{d_c[i], d_a[i], d_b[i], na[i], nb[i]};
            it.nc = nc;
            all.push_back({wl, (long long)i, it});
            continue;
        }
        if (na[i] == 0 || nb[i] == 0) {
            if (na[i] + nb[i]) CK(cudaMemsetAsync(d_c[i], 0, (na[i] + nb[i]) * sizeof(uint32_t), st));
            continue;
        }
        const int L = choose_log(na[i], nb[i]);
        if (L > g.max_log) {
            set_err("batch product %d needs 2^%d coefficients; engine initialised for 2^%d", i, L, g.max_log);
            rc = GBNTT_ERR_SIZE;
            break;
        }
        const bool a_short = na[i] <= nb[i];
        const size_t nS = a_short ? na[i] : nb[i], nB = a_short ? nb[i] : na[i];
        const uint32_t *S = a_short ? d_a[i] : d_b[i], *Bp = a_short ? d_b[i] : d_a[i];
        int ls = kMinLog;
        while (((size_t)1 << ls) < 4 * nS) ls++;
        if (g.batch_split && nS >= kSplitMinShort && L > ls && nB >= (nS << g.split_ratio_log)) {
            const size_t chunk = ((size_t)1 << ls) - nS + 1;
            const size_t n_out = nB + nS;
            void *E = nullptr, *O = nullptr;
            if (cudaMallocAsync(&E, n_out * sizeof(uint32_t), st) != cudaSuccess ||
                cudaMallocAsync(&O, n_out * sizeof(uint32_t), st) != cudaSuccess) {
                if (E) cudaFreeAsync(E, st);
                (void)cudaGetLastError();
                set_err("batch split: stream-ordered allocation of %zu limbs failed", 2 * n_out);
                rc = GBNTT_ERR_ALLOC;
                break;
            }
            splits.push_back({(uint32_t *)E, (uint32_t *)O, d_c[i], (long long)n_out});
            CK(cudaMemsetAsync(E, 0, n_out * sizeof(uint32_t), st));
            CK(cudaMemsetAsync(O, 0, n_out * sizeof(uint32_t), st));
            for (size_t j = 0, off = 0; off < nB; j++, off += chunk) {
                const size_t len = std::min(chunk, nB - off);
                uint32_t *dst = ((j & 1) ? (uint32_t *)O : (uint32_t *)E) + off;
                all.push_back({choose_log(len, nS), (long long)i, {dst, Bp + off, S, len, nS}, 0, 1});
            }
            continue;
        }
        all.push_back({L, (long long)i, {d_c[i], d_a[i], d_b[i], na[i], nb[i]}});
    }
    if (rc == GBNTT_OK) {
        // consecutive products of the batch with the same right operand and
        // transform length (a product tree's B_L B_R, P_L B_R) run as pairs
        // in waves of pairs only, where each pair's right operand is
        // transformed once
        // (runs of three or more: a batch sharing one right operand, which
        // its wave transforms once)
        for (size_t i = 0; i + 1 < all.size(); i++) {
            const Keyed &u = all[i], &v = all[i + 1];
            const bool run3 = (i > 0 && all[i - 1].item.b == u.item.b) ||
                              (i + 2 < all.size() && all[i + 2].item.b == u.item.b);
            if (!run3 && u.group != v.group && u.L == v.L && u.item.b == v.item.b && u.item.nb == v.item.nb &&
                u.item.a != u.item.b && v.item.a != v.item.b && !u.item.nc && !v.item.nc) {
                all[i].paired = all[i + 1].paired = 1;
                i++;
            }
        }
        // products (not cyclic, not a split's chunk) take a transform of
        // 3 2^k points where it is shorter than the power of two and there
        // is enough of them: c products of 3 2^k points with
        // c 2^k >= 2^r3_min_log. A pair takes it for both or neither (its
        // right operand's transform is shared); a run sharing one right
        // operand is split by length as before, each length's wave sharing it.
        std::vector<int> k3s(all.size(), -1);
        long long count3[kMaxLog + 1] = {};
        auto eligible = [](const Keyed &u) { return u.chunk || u.item.nc ? -1 : r3_log(u.item.na, u.item.nb); };
        for (size_t i = 0; i < all.size(); i++) {
            const int k3 = eligible(all[i]);
            if (all[i].paired) {   // pairs were marked as neighbours (i, i + 1), first to last
                const int k3v = i + 1 < all.size() ? eligible(all[i + 1]) : -1;
                if (k3 >= 0 && k3 == k3v) {
                    k3s[i] = k3s[i + 1] = k3;
                    count3[k3] += 2;
                }
                i++;
                continue;
            }
            if (k3 >= 0) {
                k3s[i] = k3;
                count3[k3]++;
            }
        }
        for (size_t i = 0; i < all.size(); i++) {
            const int k3 = k3s[i];
            if (k3 >= 0 && (k3 >= g.r3_min_log || count3[k3] >= (1LL << (g.r3_min_log - k3)))) {
                all[i].L = k3;
                all[i].r3 = 1;
            }
        }
        std::stable_sort(all.begin(), all.end(), [](const Keyed &x, const Keyed &y) {
            if (x.L != y.L) return x.L < y.L;
            if (x.r3 != y.r3) return x.r3 < y.r3;
            if (x.paired != y.paired) return x.paired < y.paired;
            return x.group < y.group;
        });
        BatchCtx x{g.d_spec, g.n_max, g.d_ctl, g.n_status, g.d_btab, g.h_btab, g.btab_ev, &g_batch_slot};
        std::vector<BatchItem> items;
        size_t pos = 0;
        while (pos < all.size() && rc == GBNTT_OK) {
            const int L = all[pos].L, paired = all[pos].paired, r3 = all[pos].r3;
            size_t end = pos;
            while (end < all.size() && all[end].L == L && all[end].paired == paired && all[end].r3 == r3) end++;
            long long wmax = std::min<long long>(kMaxBatch, (long long)(g.n_max / ((r3 ? 3ull : 1ull) << L)));
            if (paired && wmax > 1) wmax &= ~1LL;   // waves split between pairs
            for (size_t w0 = pos; w0 < end && rc == GBNTT_OK; w0 += (size_t)wmax) {
                const long long W = std::min<long long>(wmax, (long long)(end - w0));
                items.clear();
                for (long long k = 0; k < W; k++) items.push_back(all[w0 + k].item);
                rc = batch_wave(x, items.data(), W, L, st, g.stream2, r3 != 0);
            }
            pos = end;
        }
    }
    if (!splits.empty()) {
        if (rc == GBNTT_OK) {
            std::vector<const uint32_t *> ex(splits.size()), ey(splits.size());
            std::vector<uint32_t *> eo(splits.size());
            std::vector<long long> en(splits.size());
            for (size_t k = 0; k < splits.size(); k++) {
                ex[k] = splits[k].E;
                ey[k] = splits[k].O;
                eo[k] = splits[k].c;
                en[k] = splits[k].n;
            }
            rc = batch_add_limbs(ex.data(), ey.data(), eo.data(), en.data(), (int)splits.size(), st, g.d_ctl + 1);
            if (rc) set_err("batch split: the chunk-product addition failed");
        }
        for (auto &sp : splits) {
            cudaFreeAsync(sp.E, st);
            cudaFreeAsync(sp.O, st);
        }
    }
    return rc;
}

int batch_mul_wrap(uint32_t *const *d_c, const uint32_t *const *d_a, const size_t *na, const uint32_t *const *d_b,
                   const size_t *nb, const int *wrap_log, int count, cudaStream_t st)
{
    std::lock_guard<std::recursive_mutex> lk(g_mu);
    return batch_mul(d_c, d_a, na, d_b, nb, count, st, wrap_log);
}

// ---------------------------------------------------------------------------
// Serving loop (continuous batching). A server thread owns K workspace
// slots, each with its own stream, carry control words and batch tables.
// Requests (device pointers) queue in arrival order; whenever a slot is
// free, the server admits pending requests in arrival order, of any
// transform length, while the sum of their transform lengths fits the slot
// (the HBM-footprint admission: 48 N bytes per product against the slot's
// 48 cap bytes, N = 2^L or, for a product over the radix-3 threshold,
// 3 2^k; at most kMaxBatch), and runs them as one sub-wave per length,
// shortest first, back to back on the slot's stream
// (srv_activation). Waves in different slots overlap on the device. The
// server thread sleeps on a condition variable: a host callback enqueued
// after each sub-wave (srv_done_cb) marks its requests done, the one after
// the last sub-wave also frees the slot, and a submit wakes it. Latency is
// submit -> that callback. Results are bit-identical to gbntt_mul_u32.
// ---------------------------------------------------------------------------
namespace {

struct SrvRequest {
    BatchItem item;
    int L = 0;
    int r3 = 0;      // transform of 3 2^L points (a product alone over the radix-3 threshold)
    int state = 0;   // 0 pending, 1 running, 2 done
    std::chrono::steady_clock::time_point t_submit, t_done;
};

struct SrvSlot {
    BatchCtx ctx;
    uint64_t *spec = nullptr;
    unsigned *ctl = nullptr;
    uint64_t *d_btab = nullptr, *h_btab = nullptr;
    cudaEvent_t btab_ev[2] = {nullptr, nullptr};
    int tab_slot = 0;
    cudaStream_t stream = nullptr;
    cudaEvent_t done = nullptr;
    bool busy = false;   // an activation is in flight (guarded by Server::mu)
};

struct Server {
    std::thread th;
    std::mutex mu;
    std::condition_variable cv;
    std::deque<uint64_t> pending;
    std::deque<SrvRequest> reqs;       // indexed by ticket (stable references)
    std::vector<SrvSlot> slots;
    size_t cap = 0;
    int slot_log = 0;
    bool stop = false;
    std::atomic<uint64_t> completed{0}, waves{0}, wave_products{0}, activations{0};
    int error = 0;
};

Server *g_srv = nullptr;

// Completion of one sub-wave, reported by a host function enqueued after it
// on the slot's stream (no CUDA calls in here): its requests are done; the
// last sub-wave of an activation frees the slot.
struct SrvDone {
    Server *S;
    SrvSlot *sl;
    std::vector<uint64_t> ids;
    bool last;
};

void CUDART_CB srv_done_cb(void *p)
{
    SrvDone *d = (SrvDone *)p;
    Server *S = d->S;
    {
        std::lock_guard<std::mutex> lk(S->mu);
        const auto now = std::chrono::steady_clock::now();
        for (uint64_t id : d->ids) { S->reqs[id].state = 2; S->reqs[id].t_done = now; }
        S->completed += d->ids.size();
        if (d->last) d->sl->busy = false;
    }
    S->cv.notify_all();
    delete d;
}

// One activation of a slot: the admitted requests grouped by transform
// length (ascending), each group one sub-wave through the batched pass
// chain, back to back on the slot's stream (each sub-wave may use the whole
// slot workspace: they run one after the other). The tables of all
// sub-waves are filled into one host table slot and go up in one copy.
// Launches directly (no wave graphs: group layouts rarely repeat).
int srv_activation(Server *S, SrvSlot &sl, const std::vector<int> &gL, const std::vector<int> &g3,
                   const std::vector<std::vector<BatchItem>> &gitems, std::vector<std::vector<uint64_t>> &gids)
{
    BatchCtx &x = sl.ctx;
    const int slot = *x.slot;
    CK(cudaEventSynchronize(x.btab_ev[slot]));   // the previous upload from this table slot has been read
    uint64_t *h = x.h_btab + slot * kBtabWords;
    uint64_t *dtab = x.d_btab + slot * kBtabWords;
    const size_t ng = gL.size();
    std::vector<size_t> off(ng);
    std::vector<long long> tiles(ng);
    std::vector<char> shared(ng);
    size_t pos = 0;
    for (size_t gi = 0; gi < ng; gi++) {
        const std::vector<BatchItem> &items = gitems[gi];
        const long long W = (long long)items.size();
        if (pos + 7 * (size_t)W + 1 > kBtabWords) { set_err("server activation tables overflow"); return GBNTT_ERR_SIZE; }
        uint64_t *hg = h + pos;
        uint64_t *hA = hg, *hLA = hg + W, *hB = hg + 2 * W, *hLB = hg + 3 * W, *hC = hg + 4 * W, *hNC = hg + 5 * W,
                 *hTS = hg + 6 * W;
        long long t = 0;
        bool sb = W > 1 && !g3[gi];
        for (long long k = 0; k < W; k++) {
            const BatchItem &it = items[k];
            if (it.b != items[0].b || it.nb != items[0].nb || it.a == it.b) sb = false;
            hA[k] = (uint64_t)(uintptr_t)it.a;
            hLA[k] = (uint64_t)it.na;
            hB[k] = (uint64_t)(uintptr_t)it.b;
            hLB[k] = (uint64_t)it.nb;
            hC[k] = (uint64_t)(uintptr_t)it.c;
            hNC[k] = (uint64_t)out_limbs(it);
            hTS[k] = (uint64_t)t;
            t += carry_tiles((long long)out_limbs(it));
        }
        hTS[W] = (uint64_t)t;
        if ((size_t)t > x.n_status) { set_err("server sub-wave needs %lld carry tiles", t); return GBNTT_ERR_SIZE; }
        off[gi] = pos;
        tiles[gi] = t;
        shared[gi] = sb ? 1 : 0;
        pos += 7 * (size_t)W + 1;
    }
    CK(cudaMemcpyAsync(dtab, h, pos * sizeof(uint64_t), cudaMemcpyHostToDevice, sl.stream));
    CK(cudaEventRecord(x.btab_ev[slot], sl.stream));
    *x.slot = slot ^ 1;
    for (size_t gi = 0; gi < ng; gi++) {
        const int rc = wave_launches(x, dtab + off[gi], (long long)gitems[gi].size(), gL[gi], sl.stream, nullptr,
                                     tiles[gi], shared[gi] != 0, false, g3[gi] != 0);
        if (rc) return rc;
        SrvDone *d = new SrvDone{S, &sl, std::move(gids[gi]), gi + 1 == ng};
        const cudaError_t e = cudaLaunchHostFunc(sl.stream, srv_done_cb, d);
        if (e != cudaSuccess) { delete d; CK(e); }
    }
    S->waves += ng;
    return GBNTT_OK;
}

// The server thread: sleeps on the condition variable until a request is
// pending and a slot is free (submissions and sub-wave completions notify
// it), then admits pending requests in arrival order while their transform
// lengths fit one slot workspace (the sum of 2^L, or 3 2^L, over the
// admitted requests, HBM-footprint admission; at least the oldest request;
// at most kMaxBatch requests) and starts them as one activation of that
// slot, one sub-wave per transform length.
void server_loop(Server *S)
{
    std::vector<int> gL, g3;
    std::vector<std::vector<BatchItem>> gitems;
    std::vector<std::vector<uint64_t>> gids;
    for (;;) {
        SrvSlot *sl = nullptr;
        size_t count = 0;
        {
            std::unique_lock<std::mutex> lk(S->mu);
            auto free_slot = [&]() -> SrvSlot * {
                for (auto &x : S->slots)
                    if (!x.busy) return &x;
                return nullptr;
            };
            auto any_busy = [&]() {
                for (auto &x : S->slots)
                    if (x.busy) return true;
                return false;
            };
            S->cv.wait(lk, [&] {
                return S->error || (!S->pending.empty() && free_slot()) || (S->stop && S->pending.empty() && !any_busy());
            });
            if (S->error) return;
            if (S->pending.empty()) return;   // stop requested and everything has completed
            sl = free_slot();
            std::map<int, size_t> group_of;
            gL.clear();
            g3.clear();
            gitems.clear();
            gids.clear();
            size_t used = 0;
            while (!S->pending.empty() && count < (size_t)kMaxBatch) {
                const uint64_t id = S->pending.front();
                SrvRequest &r = S->reqs[id];
                const size_t need = (size_t)(r.r3 ? 3 : 1) << r.L;
                if (count > 0 && used + need > S->cap) break;
                used += need;
                count++;
                r.state = 1;
                const int key = 2 * r.L + r.r3;
                auto it = group_of.find(key);
                size_t gi;
                if (it == group_of.end()) {
                    gi = gL.size();
                    group_of[key] = gi;
                    gL.push_back(r.L);
                    g3.push_back(r.r3);
                    gitems.emplace_back();
                    gids.emplace_back();
                } else {
                    gi = it->second;
                }
                gitems[gi].push_back(r.item);
                gids[gi].push_back(id);
                S->pending.pop_front();
            }
            sl->busy = true;
        }
        // shortest transforms first: their requests complete earliest
        std::vector<size_t> order(gL.size());
        for (size_t i = 0; i < order.size(); i++) order[i] = i;
        std::sort(order.begin(), order.end(), [&](size_t a, size_t b) {
            return ((g3[a] ? 3ull : 1ull) << gL[a]) < ((g3[b] ? 3ull : 1ull) << gL[b]);
        });
        std::vector<int> sL, s3;
        std::vector<std::vector<BatchItem>> sitems;
        std::vector<std::vector<uint64_t>> sids;
        for (size_t i : order) {
            sL.push_back(gL[i]);
            s3.push_back(g3[i]);
            sitems.push_back(std::move(gitems[i]));
            sids.push_back(std::move(gids[i]));
        }
        const int rc = srv_activation(S, *sl, sL, s3, sitems, sids);
        S->activations++;
        S->wave_products += count;
        if (rc) {
            std::lock_guard<std::mutex> lk(S->mu);
            S->error = rc;
            S->cv.notify_all();
            return;
        }
    }
}

void server_free(Server *S)
{
    invalidate_wave_graphs();
    for (auto &sl : S->slots) {
        if (sl.stream) cudaStreamSynchronize(sl.stream);
        cudaFree(sl.spec);
        cudaFree(sl.ctl);
        cudaFree(sl.d_btab);
        if (sl.h_btab) cudaFreeHost(sl.h_btab);
        for (int i = 0; i < 2; i++) if (sl.btab_ev[i]) cudaEventDestroy(sl.btab_ev[i]);
        if (sl.done) cudaEventDestroy(sl.done);
        if (sl.stream) cudaStreamDestroy(sl.stream);
    }
    delete S;
}

}  // namespace

static int read_errors(unsigned *flags)
{
    unsigned v = 0;
    CK(cudaStreamSynchronize(g.stream));
    CK(cudaMemcpy(&v, g.d_ctl + 1, sizeof v, cudaMemcpyDeviceToHost));
    CK(cudaMemset(g.d_ctl + 1, 0, sizeof(unsigned)));
    if (flags) *flags = v;
    return GBNTT_OK;
}

// Host-pointer product through the staging buffer (a, b, c contiguous).
// Device address of page-locked host memory (NVLink-C2C makes it directly
// readable and writable by kernels), or nullptr for other memory.
// Negacyclic product modulo X^N + 1 (N = 2^L) of two N-coefficient
// polynomials with 64-bit coefficients, over the three 64-bit primes:
// twist, the cyclic pass chain, the fused pointwise product and inverse,
// then untwist + Garner to signed 256-bit coefficients (reference
// pipeline_negacyclic, ntt/lib/main.hip:557-684).
static int negacyclic_dev(uint64_t *d_out, const uint64_t *d_f, const uint64_t *d_g, int L, cudaStream_t st)
{
    if (!g.ready) { set_err("engine not initialised"); return GBNTT_ERR_NOT_INIT; }
    if (!st) st = g.stream;
    if (L < kMinLog || L > kMaxLog - 1 || L > g.max_log) {
        set_err("gbntt_negacyclic_mul_u64: log_n %d outside [%d, %d]", L, kMinLog, std::min(kMaxLog - 1, g.max_log));
        return GBNTT_ERR_ARG;
    }
    if (!d_out || !d_f || !d_g) { set_err("gbntt_negacyclic_mul_u64: null pointer"); return GBNTT_ERR_ARG; }
    const PrimeSet &ps = kSet3;
    const long long N = 1LL << L;
    uint64_t *specA = g.d_spec, *specB = g.d_spec + 3 * g.n_max;
    const bool square = d_f == d_g;
    NegaArgs na;
    memset(&na, 0, sizeof na);
    na.n = N;
    na.shift = (kMaxLog - 1) - L;   // psi = w^(2^(29 - L)): a primitive 2^(L+1)-th root
    const TwTables tf = tables(ps, 0), ti = tables(ps, 1);
    for (int k = 0; k < 3; k++) { na.hi[k] = tf.hi[k]; na.lo[k] = tf.lo[k]; }
    for (int op = 0; op < (square ? 1 : 2); op++) {
        uint64_t *spec = op ? specB : specA;
        for (int k = 0; k < 3; k++) na.spec[k] = spec + k * g.n_max;
        na.coef = op ? d_g : d_f;
        CK(launch_nega_twist(na, st));
        const int rc = forward(ps, spec, g.n_max, nullptr, (size_t)N, L, st, false, 1, nullptr, nullptr, nullptr,
                               nullptr, true);
        if (rc) return rc;
    }
    int rc = inverse(ps, specA, square ? specA : specB, g.n_max, L, st, square);
    if (rc) return rc;
    for (int k = 0; k < 3; k++) {
        na.spec[k] = specA + k * g.n_max;
        na.hi[k] = ti.hi[k];
        na.lo[k] = ti.lo[k];
        na.garner[k] = g.garner[k];
    }
    na.out = d_out;
    na.q01_lo = g.q01_lo;
    na.q01_hi = g.q01_hi;
    {
        typedef unsigned __int128 u128;
        const u128 q01 = ((u128)g.q01_hi << 64) | g.q01_lo;
        const uint64_t q2 = prime_value(2);
        const u128 lo = (u128)(uint64_t)q01 * q2, hi = (u128)(uint64_t)(q01 >> 64) * q2;
        const u128 mid = (lo >> 64) + (uint64_t)hi;
        na.m[0] = (uint64_t)lo;
        na.m[1] = (uint64_t)mid;
        na.m[2] = (uint64_t)(hi >> 64) + (uint64_t)(mid >> 64);
        // (M - 1) / 2: M is odd
        na.half[0] = (na.m[0] >> 1) | (na.m[1] << 63);
        na.half[1] = (na.m[1] >> 1) | (na.m[2] << 63);
        na.half[2] = na.m[2] >> 1;
    }
    CK(launch_nega_finish(na, st));
    return GBNTT_OK;
}

static void *pinned_device_ptr(const void *p)
{
    cudaPointerAttributes at;
    if (cudaPointerGetAttributes(&at, p) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    return at.type == cudaMemoryTypeHost ? at.devicePointer : nullptr;
}

// Device address under which kernels may read the limbs of a BigInt flagged
// managed: managed or device memory in place, page-locked host memory through
// its mapped address; nullptr for anything else (the caller stages it). A
// reference build linked against this library dynamically keeps its own weak
// bigint_alloc_managed (ntt/lib/arith/bigint.c:61-68: calloc with managed = 1),
// so the flag alone does not mean the GPU can reach the memory.
static const void *managed_device_ptr(const void *p)
{
    cudaPointerAttributes at;
    if (cudaPointerGetAttributes(&at, p) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    if (at.type == cudaMemoryTypeManaged || at.type == cudaMemoryTypeDevice || at.type == cudaMemoryTypeHost)
        return at.devicePointer;
    return nullptr;
}

static int mul_host(uint32_t *c, const uint32_t *a, size_t na, const uint32_t *b, size_t nb,
                    const uint32_t *dev_a, const uint32_t *dev_b)
{
    if (!g.ready) { set_err("engine not initialised"); return GBNTT_ERR_NOT_INIT; }
    const size_t n_out = na + nb;
    if (na == 0 || nb == 0) { if (n_out) memset(c, 0, n_out * 4); return GBNTT_OK; }
    if (choose_log(na, nb) > g.max_log) {
        set_err("product needs %zu coefficients but the engine was initialised for 2^%d", na + nb - 1, g.max_log);
        return GBNTT_ERR_SIZE;
    }
    const bool square = (a == b && na == nb);
    uint32_t *da = g.d_io, *db = g.d_io + na, *dc = g.d_io + na + (square ? 0 : nb);
    double t0 = g.prof ? now_ms() : 0;
    const uint32_t *ua = dev_a, *ub = dev_b;
    // Zero copy: a pinned result is written by the carry kernel over
    // NVLink-C2C. Pinned operands: without stage_inputs the first forward
    // passes of both primes read them in place (twice over C2C). With it
    // (default) A's first q0 pass reads A over C2C once and leaves a copy in
    // HBM for p3's first pass, and B is pulled into HBM by a copy kernel on
    // the copy stream while A is being transformed. Pageable operands go
    // through cudaMemcpyAsync.
    if (!ua && g.zero_copy && !g.stage_inputs) ua = (const uint32_t *)pinned_device_ptr(a);
    if (!ub && !square && g.zero_copy && !g.stage_inputs) ub = (const uint32_t *)pinned_device_ptr(b);
    uint32_t *uc = g.zero_copy ? (uint32_t *)pinned_device_ptr(c) : nullptr;
    auto stage = [&](uint32_t *dst, const uint32_t *src, size_t n, int grid, cudaStream_t s) -> int {
        const uint32_t *mapped = g.zero_copy ? (const uint32_t *)pinned_device_ptr(src) : nullptr;
        if (mapped) CK(launch_copy_words(dst, mapped, (long long)n, grid, s));
        else CK(cudaMemcpyAsync(dst, src, n * 4, cudaMemcpyHostToDevice, s));
        return GBNTT_OK;
    };
    int rs;
    uint32_t *stage_a = nullptr;
    if (!ua && g.zero_copy && g.stage_inputs && (ua = (const uint32_t *)pinned_device_ptr(a)) != nullptr) {
        stage_a = da;   // A's first pass reads it over C2C once and leaves a copy in HBM for the other prime
    } else if (!ua) {
        if ((rs = stage(da, a, na, g.sms * 4, g.stream)) != GBNTT_OK) return rs;
        ua = da;
    }
    StageJob jb;
    const StageJob *stage_b = nullptr;
    if (square) ub = ua;
    else if (!ub) {
        // B is copied by mul_dev on the copy stream (a small-grid copy
        // kernel for pinned memory) after A's first pass: it then overlaps
        // A's remaining passes instead of sharing the host link with them
        const uint32_t *mapped = g.zero_copy ? (const uint32_t *)pinned_device_ptr(b) : nullptr;
        jb.dst = db;
        jb.src = mapped ? mapped : b;
        jb.n = nb;
        jb.mapped = mapped != nullptr;
        stage_b = &jb;
        ub = db;
    }
    if (g.prof) {
        CK(cudaStreamSynchronize(g.stream));
        CK(cudaStreamSynchronize(g.cstream));
        double t = now_ms(); g.prof_ms[0] += t - t0; t0 = t;
    }
    int rc = mul_dev(uc ? uc : dc, ua, na, ub, nb, g.stream, stage_b, stage_a);
    if (rc) return rc;
    if (g.prof) { CK(cudaStreamSynchronize(g.stream)); double t = now_ms(); g.prof_ms[1] += t - t0; t0 = t; }
    if (!uc) CK(cudaMemcpyAsync(c, dc, n_out * 4, cudaMemcpyDeviceToHost, g.stream));
    unsigned flags = 0;
    rc = read_errors(&flags);
    if (rc) return rc;
    if (g.prof) { double t = now_ms(); g.prof_ms[2] += t - t0; g.prof_calls++; }
    if (flags) {
        set_err("device check failed (flags 0x%x): %s", flags,
                (flags & ERR_GARNER_DIGIT) ? "CRT digit out of range" : "carry look-back wait gave up");
        return GBNTT_ERR_DEVICE;
    }
    return GBNTT_OK;
}

// Host-pointer packed product through the staging buffer.
static int mul_host64(uint64_t *c, const uint64_t *a, size_t na, const uint64_t *b, size_t nb, const uint64_t *dev_a,
                      const uint64_t *dev_b)
{
    if (!g.ready) { set_err("engine not initialised"); return GBNTT_ERR_NOT_INIT; }
    const size_t n_out = na + nb;
    if (na == 0 || nb == 0) { if (n_out) memset(c, 0, n_out * 8); return GBNTT_OK; }
    if (choose_log(na, nb) > g.max_log) {
        set_err("product needs %zu coefficients but the engine was initialised for 2^%d", na + nb - 1, g.max_log);
        return GBNTT_ERR_SIZE;
    }
    const bool square = (a == b && na == nb);
    uint64_t *io = (uint64_t *)g.d_io;
    uint64_t *da = io, *db = io + na, *dc = io + na + (square ? 0 : nb);
    double t0 = g.prof ? now_ms() : 0;
    const uint64_t *ua = dev_a, *ub = dev_b;
    if (!ua && g.zero_copy) ua = (const uint64_t *)pinned_device_ptr(a);
    if (!ub && !square && g.zero_copy) ub = (const uint64_t *)pinned_device_ptr(b);
    uint64_t *uc = g.zero_copy ? (uint64_t *)pinned_device_ptr(c) : nullptr;
    if (!ua) { CK(cudaMemcpyAsync(da, a, na * 8, cudaMemcpyHostToDevice, g.stream)); ua = da; }
    if (square) ub = ua;
    else if (!ub) { CK(cudaMemcpyAsync(db, b, nb * 8, cudaMemcpyHostToDevice, g.stream)); ub = db; }
    if (g.prof) { CK(cudaStreamSynchronize(g.stream)); double t = now_ms(); g.prof_ms[0] += t - t0; t0 = t; }
    int rc = mul_dev64(uc ? uc : dc, ua, na, ub, nb, g.stream);
    if (rc) return rc;
    if (g.prof) { CK(cudaStreamSynchronize(g.stream)); double t = now_ms(); g.prof_ms[1] += t - t0; t0 = t; }
    if (!uc) CK(cudaMemcpyAsync(c, dc, n_out * 8, cudaMemcpyDeviceToHost, g.stream));
    unsigned flags = 0;
    rc = read_errors(&flags);
    if (rc) return rc;
    if (g.prof) { double t = now_ms(); g.prof_ms[2] += t - t0; g.prof_calls++; }
    if (flags) {
        set_err("device check failed (flags 0x%x): %s", flags,
                (flags & ERR_GARNER_DIGIT) ? "CRT digit out of range" : "carry look-back wait gave up");
        return GBNTT_ERR_DEVICE;
    }
    return GBNTT_OK;
}

// ---- reference BigInt path -------------------------------------------------
static int g_ref_cap = 28;   // default cap of max_log_n for ntt_mul_init_impl
static int g_ref_log = 0;    // max_log_n given to ntt_mul_init_impl

static size_t limbs32(const gbntt_bigint *x)
{
    if (x->n_limbs <= 0) return 0;
    size_t n = 2 * (size_t)x->n_limbs;
    if ((x->limbs[x->n_limbs - 1] >> 32) == 0) n--;
    return n;
}

int bigint_mul_impl(gbntt_bigint *c, const gbntt_bigint *a, const gbntt_bigint *b, bool *guard_fail,
                    bool *managed_fail)
{
    *guard_fail = false;
    *managed_fail = false;
    if (!g.ready) { set_err("call ntt_mul_init first"); return GBNTT_ERR_NOT_INIT; }
    g.dispatch++;
    const long na64 = a->n_limbs, nb64 = b->n_limbs;
    const long need = na64 + nb64 - 1;
    const long nref = g_ref_log > 0 ? (1L << g_ref_log) : (1L << (g.max_log - 1));
    if (need > nref) {
        *guard_fail = true;
        set_err("operands exceed the fixed NTT size — product needs %ld coeffs but N=%ld (log_n=%d). "
                "Re-init ntt_mul with a larger max_log_n; the size-N cyclic convolution would otherwise "
                "wrap silently and corrupt the result.", need, nref, g_ref_log);
        return GBNTT_ERR_SIZE;
    }
    const size_t na = limbs32(a), nb = limbs32(b);
    const bool square = (a == b) || (a->limbs == b->limbs && a->n_limbs == b->n_limbs);
    const long n_coeffs = na64 + nb64;
    const int newcap = (int)(n_coeffs + 4);
    uint32_t *tmp = nullptr;
    uint32_t *outp;
    // The output lands in a host buffer that cannot alias the inputs.
    const bool alias = (c == a) || (c == b) || c->limbs == a->limbs || c->limbs == b->limbs;
    if (c->cap < newcap && c->managed) {
        *managed_fail = true;
        set_err("bigint_resize: managed BigInt cap=%d insufficient for new_cap=%d — pre-allocate larger", c->cap,
                newcap);
        return GBNTT_ERR_MANAGED_CAP;
    }
    const bool packed = g.bigint_coeff_bits == 64;
    // 32-bit words written: the packed path writes whole 64-bit limbs
    const size_t n_out = packed ? 2 * (size_t)(na64 + nb64) : na + nb;
    if (alias || c->cap < newcap) {
        tmp = (uint32_t *)malloc((n_out + 2) * sizeof(uint32_t));
        if (!tmp) { set_err("host allocation failed"); return GBNTT_ERR_ALLOC; }
        outp = tmp;
    } else {
        outp = (uint32_t *)c->limbs;
    }
    int rc = GBNTT_OK;
    if (na == 0 || nb == 0) {
        memset(outp, 0, n_out * 4);
    } else if (packed) {
        // one 64-bit limb per coefficient
        const uint64_t *pa = a->limbs, *pb = b->limbs;
        rc = mul_host64((uint64_t *)outp, pa, (size_t)na64, square ? pa : pb, square ? (size_t)na64 : (size_t)nb64,
                        a->managed ? (const uint64_t *)managed_device_ptr(pa) : nullptr,
                        (!square && b->managed) ? (const uint64_t *)managed_device_ptr(pb) : nullptr);
    } else {
        const uint32_t *pa = (const uint32_t *)a->limbs, *pb = (const uint32_t *)b->limbs;
        rc = mul_host(outp, pa, na, square ? pa : pb, square ? na : nb,
                      a->managed ? (const uint32_t *)managed_device_ptr(pa) : nullptr,
                      (!square && b->managed) ? (const uint32_t *)managed_device_ptr(pb) : nullptr);
    }
    if (rc) { free(tmp); return rc; }
    if (c->cap < newcap) {
        uint64_t *nl = (uint64_t *)realloc(c->limbs, (size_t)newcap * sizeof(uint64_t));
        if (!nl) { free(tmp); set_err("bigint_resize: OOM"); return GBNTT_ERR_ALLOC; }
        c->limbs = nl;
        c->cap = newcap;
    }
    uint32_t *dst = (uint32_t *)c->limbs;
    if (tmp) memcpy(dst, tmp, n_out * 4);
    memset(dst + n_out, 0, ((size_t)c->cap * 2 - n_out) * 4);
    free(tmp);
    long n = (long)((n_out + 1) / 2);
    while (n > 0 && c->limbs[n - 1] == 0) n--;
    c->n_limbs = (int)n;
    return GBNTT_OK;
}

// ---- engine state for the reference entry points (gbntt_refabi.cu) ----
std::recursive_mutex &engine_mutex() { return g_mu; }
bool engine_ready() { return g.ready; }
int engine_init(int L) { return init_impl(L); }
int engine_max_log() { return g.max_log; }
const char *engine_error() { return g_err; }
int ref_log_cap() { return g_ref_cap; }
int ref_log() { return g_ref_log; }
void ref_begin(int max_log_n)
{
    g_ref_log = max_log_n;
    g.dispatch = 0;
}
unsigned long &dispatch_count() { return g.dispatch; }
cudaStream_t engine_stream() { return g.stream; }
int mul_dev_u32(uint32_t *d_c, const uint32_t *d_a, size_t na, const uint32_t *d_b, size_t nb, cudaStream_t st)
{
    return mul_dev(d_c, d_a, na, d_b, nb, st);
}

}  // namespace gbntt

using namespace gbntt;

extern "C" {

int gbntt_init(int max_log32)
{
    std::lock_guard<std::recursive_mutex> lk(g_mu);
    return init_impl(max_log32);
}

void gbntt_teardown(void)
{
    std::lock_guard<std::recursive_mutex> lk(g_mu);
    if (!g.ready) return;
    if (g.prof > 0 && g.prof_calls > 0) {
        const double tot = g.prof_ms[0] + g.prof_ms[1] + g.prof_ms[2];
        fprintf(stderr, "[ntt_prof] calls=%ld  upload=%.1fms  compute=%.1fms  download=%.1fms  total=%.1fms\n",
                g.prof_calls, g.prof_ms[0], g.prof_ms[1], g.prof_ms[2], tot);
    }
    free_all();
    g_ref_log = 0;
}

int gbntt_is_ready(void) { return g.ready ? 1 : 0; }
int gbntt_max_log(void) { return g.max_log; }
size_t gbntt_workspace_bytes(int max_log32) { return workspace_bytes(max_log32); }
int gbntt_transform_log(size_t na, size_t nb) { return (na == 0 || nb == 0) ? 0 : choose_log(na, nb); }
int gbntt_plan(int log_n, int *passes)
{
    if (log_n < kMinLog || log_n > kMaxLog || !passes) return 0;
    return plan_passes(log_n, passes);
}
const char *gbntt_last_error(void) { return g_err; }

int gbntt_set_plan(int log_n, int npasses, const int *passes)
{
    std::lock_guard<std::recursive_mutex> lk(g_mu);
    if (log_n < kMinLog || log_n > kMaxLog) { set_err("gbntt_set_plan: log_n %d out of range", log_n); return GBNTT_ERR_ARG; }
    if (npasses == 0) { g_plan_override[log_n][0] = 0; invalidate_wave_graphs(); return GBNTT_OK; }
    if (npasses < 1 || npasses > kMaxPasses || !passes) {
        set_err("gbntt_set_plan: 1 to %d passes", kMaxPasses);
        return GBNTT_ERR_ARG;
    }
    int sum = 0;
    for (int i = 0; i < npasses; i++) {
        if (passes[i] < kMinLog || passes[i] > kMaxPassLog) {
            set_err("gbntt_set_plan: pass size 2^%d outside [2^%d, 2^%d]", passes[i], kMinLog, kMaxPassLog);
            return GBNTT_ERR_ARG;
        }
        sum += passes[i];
    }
    if (sum != log_n) { set_err("gbntt_set_plan: pass sizes sum to %d, not %d", sum, log_n); return GBNTT_ERR_ARG; }
    g_plan_override[log_n][0] = npasses;
    for (int i = 0; i < npasses; i++) g_plan_override[log_n][1 + i] = passes[i];
    invalidate_wave_graphs();
    return GBNTT_OK;
}

// Autotuner: for each transform length 2^L in [log_lo, log_hi], time every
// pass plan of 1 to kMaxPasses passes (each 2^5 .. 2^10 points) on a
// synthetic 2^(L-1) x 2^(L-1)-limb product through the normal multiply path
// (CUDA events on the engine stream, best of `reps` after a warm-up), and
// install the fastest through the plan-override table.
// plans[(1 + kMaxPasses) i ...] receives (pass count, sizes...) and ms[i]
// its time for L = log_lo + i.
int gbntt_autotune(int log_lo, int log_hi, int reps, int *plans, float *ms)
{
    std::lock_guard<std::recursive_mutex> lk(g_mu);
    if (!g.ready) { set_err("engine not initialised"); return GBNTT_ERR_NOT_INIT; }
    if (log_lo < kMinLog || log_hi > g.max_log || log_lo > log_hi || reps < 1) {
        set_err("gbntt_autotune: range [%d, %d] outside [%d, %d] or reps < 1", log_lo, log_hi, kMinLog, g.max_log);
        return GBNTT_ERR_ARG;
    }
    if (g_srv) { set_err("gbntt_autotune: stop the server first"); return GBNTT_ERR_ARG; }
    cudaEvent_t e0, e1;
    CK(cudaEventCreate(&e0));
    CK(cudaEventCreate(&e1));
    int rc = GBNTT_OK;
    for (int L = log_lo; L <= log_hi && rc == GBNTT_OK; L++) {
        const size_t half = (size_t)1 << (L - 1);
        uint32_t *da = g.d_io, *db = da + half, *dc = db + half;
        CK(launch_fill_splitmix(da, (long long)half, 0x5eed0000u + L, g.stream));
        CK(launch_fill_splitmix(db, (long long)half, 0x5eed1000u + L, g.stream));
        // every composition of L into 1..kMaxPasses parts of 5..10
        typedef std::array<int, 1 + kMaxPasses> Plan;
        std::vector<Plan> cands;
        Plan cur{};
        auto extend = [&](auto &&self, int depth, int left) -> void {
            if (left == 0 && depth > 0) {
                Plan c{};
                c[0] = depth;
                for (int i = 0; i < depth; i++) c[1 + i] = cur[1 + i];
                cands.push_back(c);
                return;
            }
            if (depth == kMaxPasses) return;
            for (int p = kMinLog; p <= kMaxPassLog && p <= left; p++) {
                cur[1 + depth] = p;
                self(self, depth + 1, left - p);
            }
        };
        extend(extend, 0, L);
        float best = 1e30f;
        Plan best_plan{};
        for (const auto &c : cands) {
            g_plan_override[L][0] = c[0];
            for (int i = 0; i < kMaxPasses; i++) g_plan_override[L][1 + i] = c[1 + i];
            if ((rc = mul_dev(dc, da, half, db, half, g.stream)) != GBNTT_OK) break;   // warm-up
            float t_min = 1e30f;
            for (int r = 0; r < reps && rc == GBNTT_OK; r++) {
                CK(cudaEventRecord(e0, g.stream));
                rc = mul_dev(dc, da, half, db, half, g.stream);
                CK(cudaEventRecord(e1, g.stream));
                CK(cudaEventSynchronize(e1));
                float t = 0;
                CK(cudaEventElapsedTime(&t, e0, e1));
                t_min = std::min(t_min, t);
            }
            if (rc == GBNTT_OK && t_min < best) { best = t_min; best_plan = c; }
            // every candidate builds tables for its own pass shapes; drop
            // them between candidates so they stay within the budget (the
            // server thread, which reads them without the engine lock, is
            // not running: gbntt_autotune refuses to run beside it)
            CK(cudaDeviceSynchronize());
            free_pass_tables();
        }
        g_plan_override[L][0] = best_plan[0];
        for (int i = 0; i < kMaxPasses; i++) g_plan_override[L][1 + i] = best_plan[1 + i];
        if (plans)
            for (int i = 0; i <= kMaxPasses; i++) plans[(1 + kMaxPasses) * (L - log_lo) + i] = best_plan[i];
        if (ms) ms[L - log_lo] = best;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    invalidate_wave_graphs();
    if (rc == GBNTT_OK) {
        unsigned flags = 0;
        rc = read_errors(&flags);
        if (rc == GBNTT_OK && flags) { set_err("gbntt_autotune: device check failed (flags 0x%x)", flags); rc = GBNTT_ERR_DEVICE; }
    }
    return rc;
}

int gbntt_debug_modops(int prime, int op, const uint64_t *d_a, const uint64_t *d_b, uint64_t *d_out, size_t n,
                       void *stream)
{
    if (prime < 0 || prime > 4 || op < 0 || op > 6 || (op == 6 && prime != 0)) {
        set_err("gbntt_debug_modops: bad prime/op");
        return GBNTT_ERR_ARG;
    }
    cudaStream_t st = stream ? (cudaStream_t)stream : (g.ready ? g.stream : (cudaStream_t)0);
    CK(launch_modops(prime, op, d_a, d_b, d_out, (long long)n, st));
    return GBNTT_OK;
}

int gbntt_fill_operand(uint32_t *d, size_t n, uint64_t seed, void *stream)
{
    cudaStream_t st = stream ? (cudaStream_t)stream : (g.ready ? g.stream : (cudaStream_t)0);
    CK(launch_fill_splitmix(d, (long long)n, seed, st));
    return GBNTT_OK;
}

int gbntt_launch_log(int enable)
{
    std::lock_guard<std::recursive_mutex> lk(g_mu);
    for (auto &r : g_recs) { cudaEventDestroy(r.e0); cudaEventDestroy(r.e1); }
    g_recs.clear();
    g_rec_on = enable != 0;
    return GBNTT_OK;
}

int gbntt_launch_records(int *kind, int *log_l, double *bytes, float *ms, int max_records)
{
    std::lock_guard<std::recursive_mutex> lk(g_mu);
    cudaError_t e = cudaDeviceSynchronize();
    int n = 0;
    for (auto &r : g_recs) {
        if (e != cudaSuccess || n >= max_records) break;
        float t = 0.f;
        e = cudaEventElapsedTime(&t, r.e0, r.e1);
        kind[n] = r.kind;
        log_l[n] = r.log_l;
        bytes[n] = r.bytes;
        ms[n] = t;
        n++;
    }
    if (e != cudaSuccess) {
        set_err("gbntt_launch_records: %s", cudaGetErrorString(e));
        return -GBNTT_ERR_CUDA;
    }
    return n;
}

void *gbntt_stream(void) { return (void *)g.stream; }

int gbntt_mul_u32(uint32_t *d_c, const uint32_t *d_a, size_t na, const uint32_t *d_b, size_t nb, void *stream)
{
    std::lock_guard<std::recursive_mutex> lk(g_mu);
    if (!d_c || (na && !d_a) || (nb && !d_b)) { set_err("null pointer"); return GBNTT_ERR_ARG; }
    return mul_dev(d_c, d_a, na, d_b, nb, (cudaStream_t)stream);
}

int gbntt_mul_u64(uint64_t *d_c, const uint64_t *d_a, size_t na, const uint64_t *d_b, size_t nb, void *stream)
{
    std::lock_guard<std::recursive_mutex> lk(g_mu);
    if (!d_c || (na && !d_a) || (nb && !d_b)) { set_err("null pointer"); return GBNTT_ERR_ARG; }
    return mul_dev64(d_c, d_a, na, d_b, nb, (cudaStream_t)stream);
}

int gbntt_sqr_u64(uint64_t *d_c, const uint64_t *d_a, size_t na, void *stream)
{
    return gbntt_mul_u64(d_c, d_a, na, d_a, na, stream);
}

int gbntt_mul_u64_host(uint64_t *c, const uint64_t *a, size_t na, const uint64_t *b, size_t nb)
{
    std::lock_guard<std::recursive_mutex> lk(g_mu);
    if (!c || (na && !a) || (nb && !b)) { set_err("null pointer"); return GBNTT_ERR_ARG; }
    return mul_host64(c, a, na, b, nb, nullptr, nullptr);
}

int gbntt_set_prime_set(int nprimes)
{
    std::lock_guard<std::recursive_mutex> lk(g_mu);
    if (nprimes != 2 && nprimes != 3) { set_err("gbntt_set_prime_set: 2 or 3 primes"); return GBNTT_ERR_ARG; }
    if (!g.ready) { set_err("engine not initialised"); return GBNTT_ERR_NOT_INIT; }
    if (g_srv) {   // its thread reads the prime set per sub-wave, and its requests were sized for it
        set_err("gbntt_set_prime_set: stop the server first");
        return GBNTT_ERR_ARG;
    }
    cudaStreamSynchronize(g.stream);
    g.prime_set = nprimes;
    invalidate_wave_graphs();
    return GBNTT_OK;
}

int gbntt_prime_set(void) { return g.ready ? g.prime_set : 0; }

int gbntt_wave_graphs(void)
{
    std::lock_guard<std::mutex> lk(g_wave_graphs_mu);
    int n = 0;
    for (auto &kv : g_wave_graphs) n += kv.second.exec != nullptr;
    return n;
}

int gbntt_set_coeff_bits(int bits)
{
    std::lock_guard<std::recursive_mutex> lk(g_mu);
    if (bits != 32 && bits != 64) { set_err("gbntt_set_coeff_bits: 32 or 64"); return GBNTT_ERR_ARG; }
    if (!g.ready) { set_err("engine not initialised"); return GBNTT_ERR_NOT_INIT; }
    g.bigint_coeff_bits = bits;
    return GBNTT_OK;
}

int gbntt_coeff_bits(void) { return g.bigint_coeff_bits; }

int gbntt_negacyclic_mul_u64(uint64_t *d_out, const uint64_t *d_f, const uint64_t *d_g, int log_n, void *stream)
{
    std::lock_guard<std::recursive_mutex> lk(g_mu);
    return negacyclic_dev(d_out, d_f, d_g, log_n, (cudaStream_t)stream);
}

int gbntt_batch_mul_u32(uint32_t *const *d_c, const uint32_t *const *d_a, const size_t *na,
                        const uint32_t *const *d_b, const size_t *nb, int count, void *stream)
{
    std::lock_guard<std::recursive_mutex> lk(g_mu);
    return batch_mul(d_c, d_a, na, d_b, nb, count, (cudaStream_t)stream);
}

int gbntt_server_start(int slots, int slot_log)
{
    std::lock_guard<std::recursive_mutex> lk(g_mu);
    if (!g.ready) { set_err("engine not initialised"); return GBNTT_ERR_NOT_INIT; }
    if (g_srv) { set_err("server already running"); return GBNTT_ERR_ARG; }
    if (slots < 1 || slots > 16 || slot_log < kMinLog || slot_log > g.max_log) {
        set_err("gbntt_server_start: 1..16 slots of 2^%d..2^%d coefficients", kMinLog, g.max_log);
        return GBNTT_ERR_ARG;
    }
    Server *S = new Server();
    S->cap = (size_t)1 << slot_log;
    S->slot_log = slot_log;
    S->slots.resize(slots);
    const size_t nstat = status_words(S->cap);
    for (auto &sl : S->slots) {
        bool ok = cudaMalloc(&sl.spec, 6 * S->cap * sizeof(uint64_t)) == cudaSuccess &&
                  cudaMalloc(&sl.ctl, (2 + nstat) * sizeof(unsigned)) == cudaSuccess &&
                  cudaMalloc(&sl.d_btab, 2 * kBtabWords * sizeof(uint64_t)) == cudaSuccess &&
                  cudaMallocHost(&sl.h_btab, 2 * kBtabWords * sizeof(uint64_t)) == cudaSuccess &&
                  cudaStreamCreateWithFlags(&sl.stream, cudaStreamNonBlocking) == cudaSuccess &&
                  cudaEventCreateWithFlags(&sl.done, cudaEventDisableTiming) == cudaSuccess &&
                  cudaEventCreateWithFlags(&sl.btab_ev[0], cudaEventDisableTiming) == cudaSuccess &&
                  cudaEventCreateWithFlags(&sl.btab_ev[1], cudaEventDisableTiming) == cudaSuccess &&
                  cudaMemset(sl.ctl, 0, (2 + nstat) * sizeof(unsigned)) == cudaSuccess;
        if (!ok) {
            cudaGetLastError();
            set_err("gbntt_server_start: allocation of %d slots of 2^%d coefficients failed", slots, slot_log);
            server_free(S);
            return GBNTT_ERR_ALLOC;
        }
        sl.ctx = BatchCtx{sl.spec, S->cap, sl.ctl, nstat, sl.d_btab, sl.h_btab, sl.btab_ev, &sl.tab_slot};
    }
    g_srv = S;
    S->th = std::thread(server_loop, S);
    return GBNTT_OK;
}

int gbntt_server_submit(uint32_t *d_c, const uint32_t *d_a, size_t na, const uint32_t *d_b, size_t nb,
                        uint64_t *ticket)
{
    Server *S = g_srv;
    if (!S) { set_err("server not running"); return GBNTT_ERR_NOT_INIT; }
    if (!d_c || !d_a || !d_b || !ticket || na == 0 || nb == 0) { set_err("bad request"); return GBNTT_ERR_ARG; }
    const int L = choose_log(na, nb);
    if (L > S->slot_log) { set_err("request needs 2^%d coefficients; slots hold 2^%d", L, S->slot_log); return GBNTT_ERR_SIZE; }
    std::lock_guard<std::mutex> lk(S->mu);
    const uint64_t id = S->reqs.size();
    S->reqs.emplace_back();
    SrvRequest &r = S->reqs.back();
    r.item = BatchItem{d_c, d_a, d_b, na, nb};
    r.L = L;
    const int k3 = r3_log(na, nb);   // the single-product rule: the server cannot count future requests
    if (k3 >= g.r3_min_log) {
        r.L = k3;
        r.r3 = 1;
    }
    r.t_submit = std::chrono::steady_clock::now();
    S->pending.push_back(id);
    *ticket = id;
    S->cv.notify_all();
    return GBNTT_OK;
}

int gbntt_server_query(uint64_t ticket, int *state, double *latency_us)
{
    Server *S = g_srv;
    if (!S) { set_err("server not running"); return GBNTT_ERR_NOT_INIT; }
    std::lock_guard<std::mutex> lk(S->mu);
    if (ticket >= S->reqs.size()) { set_err("unknown ticket"); return GBNTT_ERR_ARG; }
    const SrvRequest &r = S->reqs[ticket];
    if (state) *state = r.state;
    if (latency_us)
        *latency_us = r.state == 2 ? std::chrono::duration<double, std::micro>(r.t_done - r.t_submit).count() : -1.0;
    return S->error ? S->error : GBNTT_OK;
}

int gbntt_server_wait(uint64_t ticket, double timeout_s)
{
    Server *S = g_srv;
    if (!S) { set_err("server not running"); return GBNTT_ERR_NOT_INIT; }
    std::unique_lock<std::mutex> lk(S->mu);
    if (ticket >= S->reqs.size()) { set_err("unknown ticket"); return GBNTT_ERR_ARG; }
    const bool ok = S->cv.wait_for(lk, std::chrono::duration<double>(timeout_s),
                                   [&] { return S->reqs[ticket].state == 2 || S->error; });
    if (S->error) return S->error;
    if (!ok) { set_err("gbntt_server_wait: timeout"); return GBNTT_ERR_ARG; }
    return GBNTT_OK;
}

int gbntt_server_stats(uint64_t *completed, uint64_t *waves, uint64_t *wave_products, unsigned *device_errors)
{
    Server *S = g_srv;
    if (!S) { set_err("server not running"); return GBNTT_ERR_NOT_INIT; }
    if (completed) *completed = S->completed;
    if (waves) *waves = S->waves;
    if (wave_products) *wave_products = S->wave_products;
    if (device_errors) {
        unsigned acc = 0;
        for (auto &sl : S->slots) {
            unsigned v = 0;
            CK(cudaMemcpy(&v, sl.ctl + 1, sizeof v, cudaMemcpyDeviceToHost));   // synchronous: finished waves only
            acc |= v;
        }
        *device_errors = acc;
    }
    return GBNTT_OK;
}

int gbntt_server_stop(void)
{
    std::lock_guard<std::recursive_mutex> lk(g_mu);
    Server *S = g_srv;
    if (!S) return GBNTT_OK;
    {
        std::lock_guard<std::mutex> l2(S->mu);
        S->stop = true;
        S->cv.notify_all();
    }
    S->th.join();
    const int err = S->error;
    g_srv = nullptr;
    server_free(S);
    return err;
}

int gbntt_sqr_u32(uint32_t *d_c, const uint32_t *d_a, size_t na, void *stream)
{
    return gbntt_mul_u32(d_c, d_a, na, d_a, na, stream);
}

int gbntt_mul_u32_host(uint32_t *c, const uint32_t *a, size_t na, const uint32_t *b, size_t nb)
{
    std::lock_guard<std::recursive_mutex> lk(g_mu);
    if (!c || (na && !a) || (nb && !b)) { set_err("null pointer"); return GBNTT_ERR_ARG; }
    return mul_host(c, a, na, b, nb, nullptr, nullptr);
}

int gbntt_device_errors(unsigned int *flags)
{
    // the engine's sticky error word, OR the no-allocation multiply's (its
    // own word in its static scratch) on the current device
    std::lock_guard<std::recursive_mutex> lk(g_mu);
    unsigned na = 0;
    int na_set_up = 0;
    const int rc = noalloc_read_errors(&na, &na_set_up);
    if (rc) { set_err("reading the no-allocation multiply's error word failed"); return rc; }
    if (!g.ready) {
        if (!na_set_up) { set_err("engine not initialised"); return GBNTT_ERR_NOT_INIT; }
        if (flags) *flags = na;
        return GBNTT_OK;
    }
    unsigned v = 0;
    const int rc2 = read_errors(&v);
    if (flags) *flags = v | na;
    return rc2;
}

int gbntt_debug_lookback_timeout(unsigned int *flags, double *seconds)
{
    // The carry kernel over 3 tiles with its ticket counter started at 1: no
    // CTA takes tile 0, so tile 1's look-back waits on a status word nothing
    // writes. The wait is bounded; it must end, set ERR_LOOKBACK_TIMEOUT and
    // leave the context usable. Output goes to the staging buffer.
    std::lock_guard<std::recursive_mutex> lk(g_mu);
    if (!g.ready) { set_err("engine not initialised"); return GBNTT_ERR_NOT_INIT; }
    long long n_out = 1;
    while (carry_tiles(n_out) < 3) n_out *= 2;   // smallest power of two spanning three carry tiles
    if ((size_t)n_out > g.io_words || (long long)g.n_max < n_out) {
        set_err("engine too small for the check");
        return GBNTT_ERR_SIZE;
    }
    CK(cudaStreamSynchronize(g.stream));
    CarryArgs c;
    memset(&c, 0, sizeof c);
    carry_setup(c, kSet3, g.d_spec, g.n_max);
    c.out = g.d_io;
    c.n_coef = n_out;
    c.n_out = n_out;
    c.ticket = g.d_ctl;
    c.error = g.d_ctl + 1;
    c.status = g.d_ctl + 2;
    const unsigned start[2] = {1u, 0u};
    CK(cudaMemsetAsync(g.d_ctl + 2, 0, 8 * sizeof(unsigned), g.stream));
    CK(cudaMemcpyAsync(g.d_ctl, start, sizeof start, cudaMemcpyHostToDevice, g.stream));
    CK(cudaStreamSynchronize(g.stream));
    const double t0 = now_ms();
    CK(launch_garner_carry(c, g.stream, nullptr));
    CK(cudaStreamSynchronize(g.stream));
    if (seconds) *seconds = (now_ms() - t0) * 1e-3;
    return read_errors(flags);
}

// Residues of a radix-3 product before Garner (mode 1) or of 3 A after the
// forward and inverse radix-3 stages alone (mode 0): q0 words to d_q0, p3
// words to d_p3, 3 2^k of each (device pointers).
int gbntt_debug_radix3(uint64_t *d_q0, uint32_t *d_p3, const uint32_t *d_a, size_t na, const uint32_t *d_b,
                       size_t nb, int k, int mode)
{
    std::lock_guard<std::recursive_mutex> lk(g_mu);
    if (!g.ready) { set_err("engine not initialised"); return GBNTT_ERR_NOT_INIT; }
    if (g.prime_set != 2 || k < kMinLog || (3ull << k) > g.n_max || na > (3ull << k) || nb > (3ull << k) ||
        (mode == 1 && na + nb - 1 > (3ull << k)) || na == 0 || nb == 0) {
        set_err("bad size");
        return GBNTT_ERR_ARG;
    }
    const int rc = r3_residues(d_a, na, d_b, nb, k, g.stream, nullptr, nullptr, mode);
    if (rc) return rc;
    const size_t M3 = (size_t)3 << k;
    CK(cudaMemcpyAsync(d_q0, g.d_spec, M3 * 8, cudaMemcpyDeviceToDevice, g.stream));
    CK(cudaMemcpyAsync(d_p3, g.d_spec + g.n_max, M3 * 4, cudaMemcpyDeviceToDevice, g.stream));
    CK(cudaStreamSynchronize(g.stream));
    return GBNTT_OK;
}

int gbntt_debug_forward(uint64_t *d_out, const uint32_t *d_in, size_t n, int log_n, void *stream)
{
    std::lock_guard<std::recursive_mutex> lk(g_mu);
    if (!g.ready) { set_err("engine not initialised"); return GBNTT_ERR_NOT_INIT; }
    if (log_n < kMinLog || log_n > g.max_log || n > ((size_t)1 << log_n)) { set_err("bad size"); return GBNTT_ERR_ARG; }
    cudaStream_t st = stream ? (cudaStream_t)stream : g.stream;
    return forward(kSet3, d_out, (size_t)1 << log_n, d_in, n, log_n, st);
}

}  // extern "C"
