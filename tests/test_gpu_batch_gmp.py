"""The batched-products workload at its own scale, checked pair by pair
against GMP mpz_mul (the ground truth of the reference's oracle test,
ntt/app/compute_e/test_gmp_oracle.c:30-38, :70-76).

4096 independent pairs with operand sizes log-uniform in 2^10 .. 2^22
32-bit limbs (independently per operand, seed 4242), operands generated on
the device from splitmix64 seeds 1000 + 2 i and 1001 + 2 i, one batched
call; then every product is compared limb for limb with GMP on the host
operands that the same generator produces on the CPU. The GMP products run
in a thread pool (the ctypes calls release the interpreter lock)."""
import concurrent.futures
import os

import numpy as np
import pytest

import oracle
from cryptography_gb300 import cudart, synth

pytestmark = [pytest.mark.gpu, pytest.mark.slow]

PAIRS = 4096


def test_batched_workload_every_pair_vs_gmp(engine):
    if not oracle.gmp_available():
        pytest.skip("libgmp.so.10 not available")
    na, nb = synth.batched_sizes(PAIRS, 4242)
    lib = engine.lib()
    da, db, dc = [], [], []
    for i in range(PAIRS):
        a, b = cudart.DeviceBuffer(4 * int(na[i])), cudart.DeviceBuffer(4 * int(nb[i]))
        c = cudart.DeviceBuffer(4 * int(na[i] + nb[i]))
        assert lib.gbntt_fill_operand(a.ptr, int(na[i]), 1000 + 2 * i, None) == 0
        assert lib.gbntt_fill_operand(b.ptr, int(nb[i]), 1001 + 2 * i, None) == 0
        da.append(a)
        db.append(b)
        dc.append(c)
    engine.batch_mul_device([c.ptr for c in dc], [x.ptr for x in da], [int(x) for x in na],
                            [x.ptr for x in db], [int(x) for x in nb])
    cudart.synchronize()
    assert engine.device_errors() == 0
    for buf in da + db:
        buf.free()

    def check(i):
        a = synth.operand(int(na[i]), 1000 + 2 * i)
        b = synth.operand(int(nb[i]), 1001 + 2 * i)
        got = dc[i].download(np.uint32, int(na[i] + nb[i]))
        want = oracle.gmp_mul(a, b)
        ok = np.array_equal(got[:len(want)], want) and not got[len(want):].any()
        return i, ok

    # largest products first so the pool stays busy to the end
    order = sorted(range(PAIRS), key=lambda i: -(int(na[i]) * int(nb[i])))
    bad = []
    with concurrent.futures.ThreadPoolExecutor(max(1, os.cpu_count() or 1)) as ex:
        for i, ok in ex.map(check, order):
            if not ok:
                bad.append(i)
    for buf in dc:
        buf.free()
    assert not bad, "pairs differing from GMP: %s" % bad[:20]
