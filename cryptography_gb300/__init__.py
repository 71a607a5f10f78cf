"""GB300 CRT-NTT big-integer multiply engine — Python host mirror.

The product is the C-ABI library ``libgbntt.so`` (sources in ``csrc/``,
declarations in ``include/gbntt.h``). This module loads it with ctypes and
mirrors the reference engine's interface (cecoppola/cryptography,
``ntt/lib/arith/multiply.h``): ``ntt_mul_init`` / ``ntt_bigint_mul`` /
``ntt_mul_teardown`` on the reference BigInt layout, plus the native 32-bit
limb API. There is no CPU fallback: if the library is missing or no CUDA
device is present, calls fail with an exception.
"""
from .engine import (  # noqa: F401
    Server,
    BigInt,
    EngineError,
    GBNTT_ERR_ALLOC,
    GBNTT_ERR_ARG,
    GBNTT_ERR_CUDA,
    GBNTT_ERR_DEVICE,
    GBNTT_ERR_MANAGED_CAP,
    GBNTT_ERR_NOT_INIT,
    GBNTT_ERR_SIZE,
    GBNTT_OK,
    autotune,
    batch_mul_device,
    bigint_alloc,
    bigint_free,
    bigint_from_int,
    bigint_set_int,
    bigint_to_int,
    device_errors,
    init,
    is_ready,
    launch_log,
    launch_records,
    lib,
    lib_path,
    mul,
    mul_device,
    mul64,
    negacyclic_mul,
    negacyclic_mul_device,
    set_coeff_bits,
    set_prime_set,
    prime_set,
    plan,
    set_plan,
    sqr,
    teardown,
    transform_log,
    wave_graphs,
    workspace_bytes,
)
