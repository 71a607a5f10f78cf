// gbntt_refabi.cu — the reference-compatible entry points (ntt_mul_init_impl,
// ntt_bigint_mul, ...; ntt/lib/arith/multiply.h, ntt/lib/arith/ntt_mul.hip)
// on top of the engine. Built twice: for the reference's default BigInt
// layout with 64-bit limbs (libgbntt.so) and, with GBNTT_LIMB_BITS=112, for
// its LIMB_BITS=112 build (ntt/lib/arith/bigint.h:30-43), whose limbs are
// 16-byte words holding 112 bits (libgbntt112.so). Both export the same
// symbol names; the engine below them is the same.
#ifndef GBNTT_LIMB_BITS
#define GBNTT_LIMB_BITS 64
#endif
#if GBNTT_LIMB_BITS == 112
#define GBNTT_LIMB112_ABI 1
#endif

#include <cuda_runtime.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "gbntt_internal.h"
#if GBNTT_LIMB_BITS == 112
#include "gbntt_limb112.h"
#endif

using namespace gbntt;

#if GBNTT_LIMB_BITS == 64

extern "C" {

void ntt_mul_init_impl(int max_log_n)
{
    std::lock_guard<std::recursive_mutex> lk(engine_mutex());
    if (engine_ready()) return;
    int cap = ref_log_cap();
    const char *e = getenv("NTT_MAX_LOGN");
    if (e) { int v = atoi(e); if (v >= 3 && v <= kMaxLog - 1) cap = v; }
    if (max_log_n < 3 || max_log_n > cap) {
        fprintf(stderr, "ntt_mul_init: log_n=%d out of safe range [3,%d] (set NTT_MAX_LOGN to raise)\n", max_log_n,
                cap);
        exit(1);
    }
    // 64-bit coefficients of the reference = pairs of 32-bit coefficients.
    int L = max_log_n + 1;
    if (L < kMinLog) L = kMinLog;
    int rc = engine_init(L);
    if (rc) {
        fprintf(stderr, "ntt_mul_init: %s\n", engine_error());
        exit(1);
    }
    ref_begin(max_log_n);
}

void ntt_mul_teardown_impl(void) { gbntt_teardown(); }

unsigned long ntt_get_gpu_dispatch_count(void) { return dispatch_count(); }

void ntt_gpu_emergency_reset(void) { (void)cudaDeviceSynchronize(); }

int ntt_bigint_mul_checked(gbntt_bigint *c, const gbntt_bigint *a, const gbntt_bigint *b)
{
    std::lock_guard<std::recursive_mutex> lk(engine_mutex());
    if (!c || !a || !b) {
        set_error_message("null BigInt");
        return GBNTT_ERR_ARG;
    }
    bool gf, mf;
    return bigint_mul_impl(c, a, b, &gf, &mf);
}

void ntt_bigint_mul(gbntt_bigint *c, const gbntt_bigint *a, const gbntt_bigint *b)
{
    std::lock_guard<std::recursive_mutex> lk(engine_mutex());
    if (!engine_ready()) {
        fprintf(stderr, "ntt_bigint_mul: call ntt_mul_init first\n");
        exit(1);
    }
    bool gf = false, mf = false;
    int rc = bigint_mul_impl(c, a, b, &gf, &mf);
    if (rc == GBNTT_OK) return;
    if (mf) {
        fprintf(stderr, "%s\n", engine_error());
        abort();
    }
    fprintf(stderr, "ntt_bigint_mul: %s\n", engine_error());
    fflush(stderr);
    exit(1);
}

void ntt_bigint_sqr(gbntt_bigint *c, const gbntt_bigint *a) { ntt_bigint_mul(c, a, a); }

gbntt_bigint bigint_alloc_managed(int cap)
{
    gbntt_bigint r;
    memset(&r, 0, sizeof r);
    void *p = nullptr;
    if (cap <= 0 || cudaMallocManaged(&p, (size_t)cap * sizeof(uint64_t)) != cudaSuccess) {
        fprintf(stderr, "bigint_alloc_managed: cudaMallocManaged(%d limbs) failed\n", cap);
        exit(1);
    }
    memset(p, 0, (size_t)cap * sizeof(uint64_t));
    r.limbs = (uint64_t *)p;
    r.cap = cap;
    r.managed = 1;
    return r;
}

void hip_free_limbs(uint64_t *p) { cudaFree(p); }


}  // extern "C"

#elif GBNTT_LIMB_BITS == 112

namespace {

// A number in 112-bit limbs is a bit string: bit b is bit b mod 112 of limb
// b / 112, a limb being four 32-bit words w0..w3 with bits 112..127 zero.

// nbits (<= 32) bits of x from bit `bit` on, zero beyond n112 limbs
__device__ __forceinline__ uint32_t bits112(const uint32_t *x, long long n112, long long bit, int nbits)
{
    uint32_t v = 0;
    int got = 0;
    while (got < nbits) {
        const long long l = bit / 112;
        if (l >= n112) break;
        const int o = (int)(bit - l * 112), take = min(nbits - got, 112 - o);
        const uint32_t *w = x + 4 * l;
        const int wi = o >> 5, sh = o & 31;
        uint64_t u = w[wi];
        if (wi < 3) u |= (uint64_t)w[wi + 1] << 32;
        uint32_t part = (uint32_t)(u >> sh);
        if (take < 32) part &= (1u << take) - 1;
        v |= part << got;
        got += take;
        bit += take;
    }
    return v;
}

// 32-bit limbs dst[0 .. n32) of a number held in n112 limbs of 112 bits
__global__ void limbs112_to_u32_kernel(const uint32_t *x, long long n112, uint32_t *dst, long long n32)
{
    for (long long j = blockIdx.x * (long long)blockDim.x + threadIdx.x; j < n32; j += (long long)gridDim.x * blockDim.x)
        dst[j] = bits112(x, n112, 32 * j, 32);
}

// 112-bit limbs dst[0 .. n112) (four words each) of a number held in n32
// 32-bit limbs
__global__ void u32_to_limbs112_kernel(const uint32_t *u, long long n32, uint32_t *dst, long long n112)
{
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n112;
         i += (long long)gridDim.x * blockDim.x) {
        for (int k = 0; k < 4; k++) {
            const long long bit = 112 * i + 32 * k;   // bits [bit, bit + 32) of the 32-bit limbs
            const long long q = bit >> 5;
            const int sh = (int)(bit & 31);
            uint64_t v = q < n32 ? u[q] : 0u;
            if (q + 1 < n32) v |= (uint64_t)u[q + 1] << 32;
            uint32_t w = (uint32_t)(v >> sh);
            if (k == 3) w &= 0xffffu;
            dst[4 * i + k] = w;
        }
    }
}

unsigned blocks_for(long long n) { return (unsigned)std::max<long long>(1, std::min<long long>((n + 255) / 256, 4096)); }

struct DevBuf {
    void *p = nullptr;
    cudaStream_t st = nullptr;
    ~DevBuf()
    {
        if (p) cudaFreeAsync(p, st);
    }
};

#define CKR(expr)                                                                                            \
    do {                                                                                                     \
        const cudaError_t _e = (expr);                                                                       \
        if (_e != cudaSuccess) {                                                                             \
            char _m[256];                                                                                    \
            snprintf(_m, sizeof _m, "CUDA error %d (%s): %s", (int)_e, cudaGetErrorString(_e), #expr);          \
            set_error_message(_m);                                                                           \
            return GBNTT_ERR_CUDA;                                                                           \
        }                                                                                                    \
    } while (0)

long long limbs32_of(const gbntt_bigint112 *x) { return ((long long)x->n_limbs * 112 + 31) / 32; }

// c = a b for 112-bit limbs: the operands go to the device as they are,
// a kernel repacks them into 32-bit limbs, the engine multiplies, a kernel
// repacks the product and it comes back into c (grown to n_a + n_b + 4
// limbs as the 64-bit flavour does). Guards as bigint_mul_impl.
int bigint112_mul_impl(gbntt_bigint112 *c, const gbntt_bigint112 *a, const gbntt_bigint112 *b, bool *guard_fail,
                       bool *managed_fail)
{
    *guard_fail = false;
    *managed_fail = false;
    if (!engine_ready()) {
        set_error_message("call ntt_mul_init first");
        return GBNTT_ERR_NOT_INIT;
    }
    dispatch_count()++;
    const long na = a->n_limbs, nb = b->n_limbs;
    const long need = na + nb - 1;
    const long nref = ref_log() > 0 ? (1L << ref_log()) : (1L << (engine_max_log() - 2));
    if (need > nref) {
        *guard_fail = true;
        char m[400];
        snprintf(m, sizeof m,
                 "operands exceed the fixed NTT size — product needs %ld coeffs but N=%ld (log_n=%d). "
                 "Re-init ntt_mul with a larger max_log_n; the size-N cyclic convolution would otherwise "
                 "wrap silently and corrupt the result.", need, nref, ref_log());
        set_error_message(m);
        return GBNTT_ERR_SIZE;
    }
    const int newcap = (int)(na + nb + 4);
    if (c->cap < newcap && c->managed) {
        *managed_fail = true;
        char m[200];
        snprintf(m, sizeof m, "bigint_resize: managed BigInt cap=%d insufficient for new_cap=%d — pre-allocate larger",
                 c->cap, newcap);
        set_error_message(m);
        return GBNTT_ERR_MANAGED_CAP;
    }
    const long n_out = na + nb;   // 112-bit limbs of the product
    const bool square = (a == b) || (a->limbs == b->limbs && a->n_limbs == b->n_limbs);
    cudaStream_t st = engine_stream();
    DevBuf dA, dB, uA, uB, uC, dC;
    dA.st = dB.st = uA.st = uB.st = uC.st = dC.st = st;
    if (na > 0 && nb > 0) {
        const long long a32 = limbs32_of(a), b32 = limbs32_of(b);
        CKR(cudaMallocAsync(&dA.p, (size_t)na * 16, st));
        CKR(cudaMallocAsync(&uA.p, (size_t)a32 * 4, st));
        CKR(cudaMemcpyAsync(dA.p, a->limbs, (size_t)na * 16, cudaMemcpyDefault, st));
        limbs112_to_u32_kernel<<<blocks_for(a32), 256, 0, st>>>((const uint32_t *)dA.p, na, (uint32_t *)uA.p, a32);
        CKR(cudaGetLastError());
        if (!square) {
            CKR(cudaMallocAsync(&dB.p, (size_t)nb * 16, st));
            CKR(cudaMallocAsync(&uB.p, (size_t)b32 * 4, st));
            CKR(cudaMemcpyAsync(dB.p, b->limbs, (size_t)nb * 16, cudaMemcpyDefault, st));
            limbs112_to_u32_kernel<<<blocks_for(b32), 256, 0, st>>>((const uint32_t *)dB.p, nb, (uint32_t *)uB.p,
                                                                      b32);
            CKR(cudaGetLastError());
        }
        CKR(cudaMallocAsync(&uC.p, (size_t)(a32 + b32) * 4, st));
        CKR(cudaMallocAsync(&dC.p, (size_t)n_out * 16, st));
        const int rc = mul_dev_u32((uint32_t *)uC.p, (const uint32_t *)uA.p, (size_t)a32,
                                   square ? (const uint32_t *)uA.p : (const uint32_t *)uB.p, (size_t)b32, st);
        if (rc) return rc;
        u32_to_limbs112_kernel<<<blocks_for(n_out), 256, 0, st>>>((const uint32_t *)uC.p, a32 + b32,
                                                                   (uint32_t *)dC.p, n_out);
        CKR(cudaGetLastError());
        CKR(cudaStreamSynchronize(st));   // the operands have been read (c may alias them)
    }
    if (c->cap < newcap) {
        gbntt_limb112 *nl = (gbntt_limb112 *)realloc(c->limbs, (size_t)newcap * 16);
        if (!nl) {
            set_error_message("bigint_resize: OOM");
            return GBNTT_ERR_ALLOC;
        }
        c->limbs = nl;
        c->cap = newcap;
    }
    if (na > 0 && nb > 0) {
        CKR(cudaMemcpyAsync(c->limbs, dC.p, (size_t)n_out * 16, cudaMemcpyDefault, st));
        CKR(cudaStreamSynchronize(st));
        memset(c->limbs + n_out, 0, (size_t)(c->cap - n_out) * 16);
    } else {
        memset(c->limbs, 0, (size_t)c->cap * 16);
    }
    long n = (na > 0 && nb > 0) ? n_out : 0;
    while (n > 0 && c->limbs[n - 1] == 0) n--;
    c->n_limbs = (int)n;
    return GBNTT_OK;
}

}  // namespace

extern "C" {

void ntt_mul_init_impl(int max_log_n)
{
    std::lock_guard<std::recursive_mutex> lk(engine_mutex());
    if (engine_ready()) return;
    int cap = ref_log_cap();
    const char *e = getenv("NTT_MAX_LOGN");
    if (e) { int v = atoi(e); if (v >= 3 && v <= kMaxLog - 2) cap = v; }
    if (max_log_n < 3 || max_log_n > cap) {
        fprintf(stderr, "ntt_mul_init: log_n=%d out of safe range [3,%d] (set NTT_MAX_LOGN to raise)\n", max_log_n,
                cap);
        exit(1);
    }
    // 2^max_log_n 112-bit coefficients: a product of up to 2^max_log_n + 1
    // limbs, 3.5 32-bit limbs each, fits 2^(max_log_n + 2) coefficients
    int L = max_log_n + 2;
    if (L < kMinLog) L = kMinLog;
    int rc = engine_init(L);
    if (rc) {
        fprintf(stderr, "ntt_mul_init: %s\n", engine_error());
        exit(1);
    }
    ref_begin(max_log_n);
}

void ntt_mul_teardown_impl(void) { gbntt_teardown(); }

unsigned long ntt_get_gpu_dispatch_count(void) { return dispatch_count(); }

void ntt_gpu_emergency_reset(void) { (void)cudaDeviceSynchronize(); }

int ntt_bigint_mul_checked(gbntt_bigint112 *c, const gbntt_bigint112 *a, const gbntt_bigint112 *b)
{
    std::lock_guard<std::recursive_mutex> lk(engine_mutex());
    if (!c || !a || !b) {
        set_error_message("null BigInt");
        return GBNTT_ERR_ARG;
    }
    bool gf, mf;
    return bigint112_mul_impl(c, a, b, &gf, &mf);
}

void ntt_bigint_mul(gbntt_bigint112 *c, const gbntt_bigint112 *a, const gbntt_bigint112 *b)
{
    std::lock_guard<std::recursive_mutex> lk(engine_mutex());
    if (!engine_ready()) {
        fprintf(stderr, "ntt_bigint_mul: call ntt_mul_init first\n");
        exit(1);
    }
    bool gf = false, mf = false;
    int rc = bigint112_mul_impl(c, a, b, &gf, &mf);
    if (rc == GBNTT_OK) return;
    if (mf) {
        fprintf(stderr, "%s\n", engine_error());
        abort();
    }
    fprintf(stderr, "ntt_bigint_mul: %s\n", engine_error());
    fflush(stderr);
    exit(1);
}

void ntt_bigint_sqr(gbntt_bigint112 *c, const gbntt_bigint112 *a) { ntt_bigint_mul(c, a, a); }

gbntt_bigint112 bigint_alloc_managed(int cap)
{
    gbntt_bigint112 r;
    memset(&r, 0, sizeof r);
    void *p = nullptr;
    if (cap <= 0 || cudaMallocManaged(&p, (size_t)cap * 16) != cudaSuccess) {
        fprintf(stderr, "bigint_alloc_managed: cudaMallocManaged(%d limbs) failed\n", cap);
        exit(1);
    }
    memset(p, 0, (size_t)cap * 16);
    r.limbs = (gbntt_limb112 *)p;
    r.cap = cap;
    r.managed = 1;
    return r;
}

void hip_free_limbs(gbntt_limb112 *p) { cudaFree(p); }

}  // extern "C"

#else
#error "GBNTT_LIMB_BITS must be 64 or 112"
#endif
