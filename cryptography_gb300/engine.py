"""ctypes bindings of ``libgbntt.so`` (see ``include/gbntt.h``)."""
import ctypes
import os

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))

GBNTT_OK = 0
GBNTT_ERR_NOT_INIT = 1
GBNTT_ERR_SIZE = 2
GBNTT_ERR_CUDA = 3
GBNTT_ERR_DEVICE = 4
GBNTT_ERR_ARG = 5
GBNTT_ERR_MANAGED_CAP = 6
GBNTT_ERR_ALLOC = 7

_u32p = ctypes.POINTER(ctypes.c_uint32)
_u64p = ctypes.POINTER(ctypes.c_uint64)
_vp = ctypes.c_void_p
_sz = ctypes.c_size_t


class EngineError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__("gbntt error %d: %s" % (code, msg))
        self.code = code


class BigInt(ctypes.Structure):
    """The reference BigInt at LIMB_BITS == 64 (ntt/lib/arith/bigint.h:69-74)."""
    _fields_ = [("limbs", _u64p), ("n_limbs", ctypes.c_int), ("cap", ctypes.c_int), ("managed", ctypes.c_int)]


# Every symbol declared in include/gbntt.h.
EXPORTS = (
    "ntt_mul_init_impl", "ntt_mul_teardown_impl", "ntt_bigint_mul", "ntt_get_gpu_dispatch_count",
    "ntt_gpu_emergency_reset", "bigint_alloc_managed", "hip_free_limbs", "ntt_bigint_sqr",
    "ntt_bigint_mul_checked", "gbntt_init", "gbntt_teardown", "gbntt_is_ready", "gbntt_max_log",
    "gbntt_workspace_bytes", "gbntt_transform_log", "gbntt_plan", "gbntt_mul_u32", "gbntt_sqr_u32",
    "gbntt_mul_u32_host", "gbntt_device_errors", "gbntt_debug_forward", "gbntt_debug_radix3", "gbntt_last_error", "gbntt_stream",
    "gbntt_launch_log", "gbntt_launch_records", "gbntt_set_plan", "gbntt_debug_modops",
    "gbntt_mul_u64", "gbntt_sqr_u64", "gbntt_mul_u64_host", "gbntt_set_coeff_bits", "gbntt_coeff_bits",
    "gbntt_mul_u32_noalloc", "gbntt_batch_mul_u32", "gbntt_fill_operand",
    "gbntt_server_start", "gbntt_server_submit", "gbntt_server_query", "gbntt_server_wait", "gbntt_server_stats",
    "gbntt_server_stop",
    "gbntt_split_terms_needed", "gbntt_e_required_log", "gbntt_binary_split", "gbntt_newton_reciprocal_u32",
    "gbntt_div_newton_u32", "gbntt_pow10_u32", "gbntt_to_decimal_u32", "gbntt_compute_e",
    "gbntt_set_prime_set", "gbntt_prime_set", "gbntt_debug_lookback_timeout", "gbntt_autotune",
    "gbntt_wave_graphs", "gbntt_negacyclic_mul_u64", "gbntt_debug_noalloc_lookback_timeout",
)

_lib = None


def lib_path():
    return os.path.join(_HERE, "libgbntt.so")


def lib():
    """Load the CUDA library. Raises if it has not been built."""
    global _lib
    if _lib is not None:
        return _lib
    path = lib_path()
    if not os.path.exists(path):
        raise ImportError("libgbntt.so not built: run `python -c \"import __graft_entry__ as g; g.build()\"` "
                          "(no CPU fallback exists)")
    L = ctypes.CDLL(path)
    L.ntt_mul_init_impl.argtypes = [ctypes.c_int]
    L.ntt_mul_init_impl.restype = None
    L.ntt_mul_teardown_impl.restype = None
    L.ntt_bigint_mul.argtypes = [ctypes.POINTER(BigInt)] * 3
    L.ntt_bigint_mul.restype = None
    L.ntt_bigint_sqr.argtypes = [ctypes.POINTER(BigInt)] * 2
    L.ntt_bigint_sqr.restype = None
    L.ntt_bigint_mul_checked.argtypes = [ctypes.POINTER(BigInt)] * 3
    L.ntt_bigint_mul_checked.restype = ctypes.c_int
    L.ntt_get_gpu_dispatch_count.restype = ctypes.c_ulong
    L.ntt_gpu_emergency_reset.restype = None
    L.bigint_alloc_managed.argtypes = [ctypes.c_int]
    L.bigint_alloc_managed.restype = BigInt
    L.hip_free_limbs.argtypes = [_u64p]
    L.hip_free_limbs.restype = None
    L.gbntt_init.argtypes = [ctypes.c_int]
    L.gbntt_init.restype = ctypes.c_int
    L.gbntt_teardown.restype = None
    L.gbntt_is_ready.restype = ctypes.c_int
    L.gbntt_max_log.restype = ctypes.c_int
    L.gbntt_workspace_bytes.argtypes = [ctypes.c_int]
    L.gbntt_workspace_bytes.restype = _sz
    L.gbntt_transform_log.argtypes = [_sz, _sz]
    L.gbntt_transform_log.restype = ctypes.c_int
    L.gbntt_plan.argtypes = [ctypes.c_int, ctypes.POINTER(ctypes.c_int)]
    L.gbntt_plan.restype = ctypes.c_int
    L.gbntt_mul_u32.argtypes = [_vp, _vp, _sz, _vp, _sz, _vp]
    L.gbntt_mul_u32.restype = ctypes.c_int
    L.gbntt_sqr_u32.argtypes = [_vp, _vp, _sz, _vp]
    L.gbntt_sqr_u32.restype = ctypes.c_int
    L.gbntt_mul_u32_host.argtypes = [_u32p, _u32p, _sz, _u32p, _sz]
    L.gbntt_mul_u32_host.restype = ctypes.c_int
    L.gbntt_device_errors.argtypes = [ctypes.POINTER(ctypes.c_uint)]
    L.gbntt_device_errors.restype = ctypes.c_int
    L.gbntt_debug_forward.argtypes = [_vp, _vp, _sz, ctypes.c_int, _vp]
    L.gbntt_debug_forward.restype = ctypes.c_int
    L.gbntt_debug_radix3.argtypes = [_vp, _vp, _vp, _sz, _vp, _sz, ctypes.c_int, ctypes.c_int]
    L.gbntt_debug_radix3.restype = ctypes.c_int
    L.gbntt_debug_modops.argtypes = [ctypes.c_int, ctypes.c_int, _vp, _vp, _vp, _sz, _vp]
    L.gbntt_debug_modops.restype = ctypes.c_int
    L.gbntt_mul_u64.argtypes = [_vp, _vp, _sz, _vp, _sz, _vp]
    L.gbntt_mul_u64.restype = ctypes.c_int
    L.gbntt_sqr_u64.argtypes = [_vp, _vp, _sz, _vp]
    L.gbntt_sqr_u64.restype = ctypes.c_int
    L.gbntt_mul_u64_host.argtypes = [_u64p, _u64p, _sz, _u64p, _sz]
    L.gbntt_mul_u64_host.restype = ctypes.c_int
    L.gbntt_set_coeff_bits.argtypes = [ctypes.c_int]
    L.gbntt_set_coeff_bits.restype = ctypes.c_int
    L.gbntt_coeff_bits.restype = ctypes.c_int
    L.gbntt_server_start.argtypes = [ctypes.c_int, ctypes.c_int]
    L.gbntt_server_start.restype = ctypes.c_int
    L.gbntt_server_submit.argtypes = [_vp, _vp, _sz, _vp, _sz, ctypes.POINTER(ctypes.c_uint64)]
    L.gbntt_server_submit.restype = ctypes.c_int
    L.gbntt_server_query.argtypes = [ctypes.c_uint64, ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_double)]
    L.gbntt_server_query.restype = ctypes.c_int
    L.gbntt_server_wait.argtypes = [ctypes.c_uint64, ctypes.c_double]
    L.gbntt_server_wait.restype = ctypes.c_int
    L.gbntt_server_stats.argtypes = [ctypes.POINTER(ctypes.c_uint64)] * 3 + [ctypes.POINTER(ctypes.c_uint)]
    L.gbntt_server_stats.restype = ctypes.c_int
    L.gbntt_server_stop.restype = ctypes.c_int
    L.gbntt_fill_operand.argtypes = [_vp, _sz, ctypes.c_uint64, _vp]
    L.gbntt_fill_operand.restype = ctypes.c_int
    L.gbntt_batch_mul_u32.argtypes = [_vp, _vp, _vp, _vp, _vp, ctypes.c_int, _vp]
    L.gbntt_batch_mul_u32.restype = ctypes.c_int
    L.gbntt_mul_u32_noalloc.argtypes = [_vp, _vp, _sz, _vp, _sz, _vp]
    L.gbntt_mul_u32_noalloc.restype = ctypes.c_int
    L.gbntt_debug_noalloc_lookback_timeout.argtypes = [ctypes.POINTER(ctypes.c_double)]
    L.gbntt_debug_noalloc_lookback_timeout.restype = ctypes.c_int
    L.gbntt_set_plan.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.POINTER(ctypes.c_int)]
    L.gbntt_set_plan.restype = ctypes.c_int
    L.gbntt_launch_log.argtypes = [ctypes.c_int]
    L.gbntt_launch_log.restype = ctypes.c_int
    L.gbntt_launch_records.argtypes = [ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_int),
                                       ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_float), ctypes.c_int]
    L.gbntt_launch_records.restype = ctypes.c_int
    _szp = ctypes.POINTER(_sz)
    L.gbntt_split_terms_needed.argtypes = [ctypes.c_long]
    L.gbntt_split_terms_needed.restype = ctypes.c_long
    L.gbntt_e_required_log.argtypes = [ctypes.c_long]
    L.gbntt_e_required_log.restype = ctypes.c_int
    L.gbntt_binary_split.argtypes = [ctypes.c_ulonglong, ctypes.c_ulonglong, _u32p, _sz, _szp, _u32p, _sz, _szp]
    L.gbntt_binary_split.restype = ctypes.c_int
    L.gbntt_newton_reciprocal_u32.argtypes = [_u32p, _sz, _szp, _u32p, _sz]
    L.gbntt_newton_reciprocal_u32.restype = ctypes.c_int
    L.gbntt_div_newton_u32.argtypes = [_u32p, _sz, _szp, _u32p, _sz, _szp, _u32p, _sz, _u32p, _sz]
    L.gbntt_div_newton_u32.restype = ctypes.c_int
    L.gbntt_pow10_u32.argtypes = [_u32p, _sz, _szp, ctypes.c_ulonglong]
    L.gbntt_pow10_u32.restype = ctypes.c_int
    L.gbntt_to_decimal_u32.argtypes = [ctypes.c_char_p, _sz, _szp, _u32p, _sz]
    L.gbntt_to_decimal_u32.restype = ctypes.c_int
    L.gbntt_compute_e.argtypes = [ctypes.c_long, ctypes.c_char_p, _sz, ctypes.POINTER(ctypes.c_double)]
    L.gbntt_compute_e.restype = ctypes.c_int
    L.gbntt_set_prime_set.argtypes = [ctypes.c_int]
    L.gbntt_set_prime_set.restype = ctypes.c_int
    L.gbntt_prime_set.restype = ctypes.c_int
    L.gbntt_debug_lookback_timeout.argtypes = [ctypes.POINTER(ctypes.c_uint), ctypes.POINTER(ctypes.c_double)]
    L.gbntt_debug_lookback_timeout.restype = ctypes.c_int
    L.gbntt_autotune.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.POINTER(ctypes.c_int),
                                 ctypes.POINTER(ctypes.c_float)]
    L.gbntt_autotune.restype = ctypes.c_int
    L.gbntt_wave_graphs.restype = ctypes.c_int
    L.gbntt_negacyclic_mul_u64.argtypes = [_vp, _vp, _vp, ctypes.c_int, _vp]
    L.gbntt_negacyclic_mul_u64.restype = ctypes.c_int
    L.gbntt_last_error.restype = ctypes.c_char_p
    L.gbntt_stream.restype = _vp
    _lib = L
    return L


def _check(rc):
    if rc != GBNTT_OK:
        raise EngineError(rc, lib().gbntt_last_error().decode(errors="replace"))


def init(max_log32):
    _check(lib().gbntt_init(int(max_log32)))


def teardown():
    lib().gbntt_teardown()


def is_ready():
    return bool(lib().gbntt_is_ready())


def workspace_bytes(max_log32):
    return int(lib().gbntt_workspace_bytes(int(max_log32)))


def transform_log(na, nb):
    return int(lib().gbntt_transform_log(na, nb))


MAX_PASSES = 4


def plan(log_n):
    p = (ctypes.c_int * MAX_PASSES)()
    n = lib().gbntt_plan(int(log_n), p)
    return [p[i] for i in range(n)]


LAUNCH_KINDS = ("fwd_pass_first", "fwd_pass", "inv_pass_first", "inv_pass", "garner_carry", "fused_inner_pass",
                "radix3_fwd", "radix3_inv")


def launch_log(enable):
    lib().gbntt_launch_log(1 if enable else 0)


def launch_records(max_records=4096):
    """[(kind name, pass log2, algorithmic bytes, ms)] of the logged launches."""
    k = (ctypes.c_int * max_records)()
    l_ = (ctypes.c_int * max_records)()
    b = (ctypes.c_double * max_records)()
    m = (ctypes.c_float * max_records)()
    n = lib().gbntt_launch_records(k, l_, b, m, max_records)
    if n < 0:
        _check(-n)
    return [(LAUNCH_KINDS[k[i]], l_[i], b[i], m[i]) for i in range(n)]


def wave_graphs():
    """Number of batched-wave CUDA graphs currently instantiated."""
    return int(lib().gbntt_wave_graphs())


def autotune(log_lo, log_hi, reps=3):
    """Time every pass plan for transform lengths 2^log_lo .. 2^log_hi and
    install the fastest; returns {L: (plan, ms)}."""
    k = log_hi - log_lo + 1
    w = 1 + MAX_PASSES
    plans = (ctypes.c_int * (w * k))()
    ms = (ctypes.c_float * k)()
    _check(lib().gbntt_autotune(int(log_lo), int(log_hi), int(reps), plans, ms))
    return {log_lo + i: ([plans[w * i + 1 + j] for j in range(plans[w * i])], float(ms[i])) for i in range(k)}


def set_plan(log_n, passes):
    """Override the pass plan for 2^log_n-point transforms ([] restores)."""
    arr = (ctypes.c_int * MAX_PASSES)(*(list(passes) + [0] * MAX_PASSES)[:MAX_PASSES])
    _check(lib().gbntt_set_plan(int(log_n), len(passes), arr))


def device_errors():
    f = ctypes.c_uint(0)
    _check(lib().gbntt_device_errors(ctypes.byref(f)))
    return int(f.value)


def _u32(a):
    return np.ascontiguousarray(a, dtype=np.uint32)


def mul(a, b):
    """Host-pointer product of two uint32 limb vectors; returns na+nb limbs."""
    a = _u32(a)
    b = a if b is a else _u32(b)
    c = np.zeros(len(a) + len(b), dtype=np.uint32)
    _check(lib().gbntt_mul_u32_host(c.ctypes.data_as(_u32p), a.ctypes.data_as(_u32p), len(a),
                                    b.ctypes.data_as(_u32p), len(b)))
    return c


def _u64(a):
    return np.ascontiguousarray(a, dtype=np.uint64)


def mul64(a, b):
    """Packed-mode product of two uint64 limb vectors; returns na+nb limbs."""
    a = _u64(a)
    b = a if b is a else _u64(b)
    c = np.zeros(len(a) + len(b), dtype=np.uint64)
    _check(lib().gbntt_mul_u64_host(c.ctypes.data_as(_u64p), a.ctypes.data_as(_u64p), len(a),
                                    b.ctypes.data_as(_u64p), len(b)))
    return c


def negacyclic_mul_device(out_ptr, f_ptr, g_ptr, log_n, stream=None):
    """Negacyclic product mod X^N + 1 (N = 2^log_n) of device uint64
    coefficient arrays; out receives 4 N words (signed 256-bit values)."""
    _check(lib().gbntt_negacyclic_mul_u64(out_ptr, f_ptr, g_ptr, int(log_n), stream))


def negacyclic_mul(f, g):
    """Host convenience around negacyclic_mul_device: f, g uint64 arrays of
    the same power-of-two length N; returns N Python ints (signed)."""
    from . import cudart
    f = _u64(f)
    same = g is f
    g = f if same else _u64(g)
    n = len(f)
    if n == 0 or n & (n - 1) or len(g) != n:
        raise ValueError("f and g need the same power-of-two length")
    log_n = n.bit_length() - 1
    df = cudart.DeviceBuffer(8 * n)
    dg = df if same else cudart.DeviceBuffer(8 * n)
    do = cudart.DeviceBuffer(32 * n)
    try:
        df.upload(f)
        if not same:
            dg.upload(g)
        negacyclic_mul_device(do.ptr, df.ptr, dg.ptr, log_n, lib().gbntt_stream())
        cudart.stream_sync(lib().gbntt_stream())
        words = do.download(np.uint64, 4 * n).reshape(n, 4)
    finally:
        for b in {id(df): df, id(dg): dg, id(do): do}.values():
            b.free()
    out = []
    for w in words:
        v = int(w[0]) | (int(w[1]) << 64) | (int(w[2]) << 128) | (int(w[3]) << 192)
        out.append(v - (1 << 256) if v >> 255 else v)
    return out


def batch_mul_device(c_ptrs, a_ptrs, na, b_ptrs, nb, stream=None):
    """Batched device products: lists of raw device addresses and sizes."""
    n = len(a_ptrs)
    P = ctypes.c_uint64 * n
    S = ctypes.c_size_t * n
    _check(lib().gbntt_batch_mul_u32(P(*c_ptrs), P(*a_ptrs), S(*na), P(*b_ptrs), S(*nb), n, stream))


class Server:
    """Continuous-batching request loop of the engine (see gbntt.h)."""

    def __init__(self, slots=4, slot_log=26):
        _check(lib().gbntt_server_start(int(slots), int(slot_log)))

    def submit(self, c_ptr, a_ptr, na, b_ptr, nb):
        t = ctypes.c_uint64(0)
        _check(lib().gbntt_server_submit(c_ptr, a_ptr, na, b_ptr, nb, ctypes.byref(t)))
        return t.value

    def query(self, ticket):
        st, lat = ctypes.c_int(0), ctypes.c_double(0)
        _check(lib().gbntt_server_query(ticket, ctypes.byref(st), ctypes.byref(lat)))
        return st.value, lat.value

    def wait(self, ticket, timeout_s=60.0):
        _check(lib().gbntt_server_wait(ticket, timeout_s))

    def stats(self):
        v = [ctypes.c_uint64(0) for _ in range(3)]
        e = ctypes.c_uint(0)
        _check(lib().gbntt_server_stats(*[ctypes.byref(x) for x in v], ctypes.byref(e)))
        return {"completed": v[0].value, "waves": v[1].value, "wave_products": v[2].value, "device_errors": e.value}

    def stop(self):
        _check(lib().gbntt_server_stop())


def set_prime_set(nprimes):
    """2: q0 + the 32-bit p3 (default); 3: the reference's three 64-bit primes."""
    _check(lib().gbntt_set_prime_set(int(nprimes)))


def prime_set():
    return int(lib().gbntt_prime_set())


def set_coeff_bits(bits):
    _check(lib().gbntt_set_coeff_bits(int(bits)))


def sqr(a):
    a = _u32(a)
    return mul(a, a)


def mul_device(c_ptr, a_ptr, na, b_ptr, nb, stream=None):
    """Device-pointer product (raw addresses), stream-ordered."""
    _check(lib().gbntt_mul_u32(c_ptr, a_ptr, na, b_ptr, nb, stream))


_libc = ctypes.CDLL(None)
_libc.calloc.restype = ctypes.c_void_p
_libc.calloc.argtypes = [_sz, _sz]
_libc.free.restype = None
_libc.free.argtypes = [ctypes.c_void_p]


def bigint_alloc(cap):
    """A BigInt whose limbs come from libc calloc, as bigint_alloc does
    (ntt/lib/arith/bigint.c:19-29), so the engine may realloc it."""
    p = _libc.calloc(max(1, int(cap)), 8)
    if not p:
        raise MemoryError("calloc failed")
    return BigInt(ctypes.cast(p, _u64p), 0, max(1, int(cap)), 0)


def bigint_free(b):
    if b.managed:
        lib().hip_free_limbs(b.limbs)
    else:
        _libc.free(ctypes.cast(b.limbs, ctypes.c_void_p))
    b.limbs = ctypes.cast(None, _u64p)
    b.n_limbs = b.cap = b.managed = 0


def bigint_set_int(b, v):
    """Store v in b (must fit b.cap); sets the trimmed n_limbs."""
    n = max(0, (v.bit_length() + 63) // 64)
    if n > b.cap:
        raise ValueError("value needs %d limbs, cap is %d" % (n, b.cap))
    ctypes.memset(b.limbs, 0, 8 * b.cap)
    if n:
        ctypes.memmove(b.limbs, v.to_bytes(8 * n, "little"), 8 * n)
    b.n_limbs = n
    return b


def bigint_from_int(v, cap=None):
    n = max(1, (v.bit_length() + 63) // 64)
    return bigint_set_int(bigint_alloc(max(cap or 0, n)), v)


def bigint_to_int(b):
    if b.n_limbs <= 0:
        return 0
    buf = ctypes.string_at(b.limbs, 8 * b.n_limbs)
    return int.from_bytes(buf, "little")
