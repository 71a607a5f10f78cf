// gbntt_carry.cuh — the carry-propagation monoid and the decoupled look-back
// shared by the Garner+carry kernels (gbntt_kernels.cu) and the big-integer
// add/subtract kernel of the e pipeline (gbntt_e.cu).
//
// A run of limb sums s_k (each below 3 * 2^32) maps an incoming carry
// c in {0, 1, 2} to an outgoing carry in {0, 1, 2}; the map is packed as
// three 2-bit values (f(0), f(1), f(2)). Maps compose associatively, so the
// carries of a whole tile follow from a block scan and the carry into a tile
// from a look-back over its predecessors' published maps. The cells follow
// the carry-lookahead transfer cells of ntt/lib/transfer_core.h:165-251,
// generalised from {0, 1} to {0, 1, 2}.
#pragma once
#include <stdint.h>
#include "gbntt_internal.h"

namespace gbntt {

constexpr int kLookbackSpinLimit = 1 << 21;   // ~0.1 s with backoff

static __device__ __forceinline__ unsigned fn_apply(unsigned f, unsigned c) { return (f >> (2 * c)) & 3u; }
static __device__ __forceinline__ unsigned fn_compose(unsigned g, unsigned f)   // g after f
{
    return fn_apply(g, fn_apply(f, 0)) | (fn_apply(g, fn_apply(f, 1)) << 2) | (fn_apply(g, fn_apply(f, 2)) << 4);
}
constexpr unsigned kFnIdentity = 0u | (1u << 2) | (2u << 4);

// shared-memory index padded by one word per 32 (bank-conflict free)
static __device__ __forceinline__ int spad(int q) { return q + (q >> 5); }

// Decoupled look-back (one thread per tile): publishes this tile's carry
// transfer function, walks predecessors until an inclusive carry (or a
// constant composed function) is known, publishes its own inclusive carry
// and returns the carry into the tile. Status word: bits 8-9 flag (1 =
// aggregate function, 2 = inclusive carry), bits 0-5 value. Every wait is
// bounded; on timeout the error bit is set and carry 0 is assumed.
static __device__ unsigned lookback_carry(unsigned *status, long long tile, unsigned block_agg, unsigned &err)
{
    unsigned cin = 0;
    if (tile == 0) {
        atomicExch(&status[0], (2u << 8) | fn_apply(block_agg, 0));
        return 0;
    }
    atomicExch(&status[tile], (1u << 8) | block_agg);
    unsigned acc = kFnIdentity;
    long long j = tile - 1;
    for (;;) {
        unsigned w = 0;
        int spins = 0;
        for (;;) {
            w = atomicAdd(&status[j], 0u);
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
    atomicExch(&status[tile], (2u << 8) | fn_apply(block_agg, cin));
    return cin;
}

// Transfer function of K consecutive limb sums s[0..K) (each < 3 * 2^32):
// f(c) = carry out of the run when c enters its lowest limb. f(1) and f(2)
// exceed f(0) by one exactly when the low limbs computed with carry 0 are
// all ones (resp. all ones above a lowest limb >= 2^32 - 2).
template <int K>
static __device__ __forceinline__ unsigned run_transfer(const uint64_t (&s)[K])
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
    return f0 | (f1 << 2) | (f2 << 4);
}

// Exclusive block scan of per-thread transfer functions in thread order.
// Returns the composed map of all lower threads; *block_agg receives the
// map of the whole block. s_warp holds T / 32 words of shared memory.
template <int T>
static __device__ __forceinline__ unsigned block_scan_transfer(unsigned fn, unsigned *s_warp, unsigned *block_agg)
{
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    unsigned inc = fn;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        const unsigned o = __shfl_up_sync(0xFFFFFFFFu, inc, d);
        if (lane >= d) inc = fn_compose(inc, o);
    }
    if (lane == 31) s_warp[warp] = inc;
    __syncthreads();
    unsigned warp_prefix = kFnIdentity, agg = kFnIdentity;
#pragma unroll
    for (int w = 0; w < T / 32; w++) {
        if (w == warp) warp_prefix = agg;
        agg = fn_compose(s_warp[w], agg);
    }
    unsigned lane_excl = __shfl_up_sync(0xFFFFFFFFu, inc, 1);
    if (lane == 0) lane_excl = kFnIdentity;
    *block_agg = agg;
    return fn_compose(lane_excl, warp_prefix);
}

}  // namespace gbntt
