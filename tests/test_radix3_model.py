"""CPU model of the transforms of 3 2^k points (csrc/gbntt_radix3.cu and the
engine's radix-3 path), step for step as the kernels compute them: the
forward radix-3 stage, three 2^k-point cyclic transforms with an arbitrary
primitive 2^k-th root (the pass chain's root is not w^3), the pointwise
products, the inverse sub-transforms scaled by 1/(3 2^k), the inverse
radix-3 stage without a 1/3, halving as shift plus (p + 1) / 2. The result
must be the cyclic convolution of length 3 2^k, in both CRT primes. Also
pins the host constants: rho of order 3 2^30 from the primes' generators,
c = (om - om^2) / 2 computed without a 64-bit overflow for q0, and the
stepped twiddles w^(j + u G)."""
import random

import pytest

Q0 = (1 << 64) - (1 << 32) + 1
P3 = 3 * (1 << 30) + 1
GEN = {Q0: 7, P3: 5}          # the generators the engine uses for q0 and p3
ORDER = 3 << 30


def rho(p):
    return pow(GEN[p], (p - 1) // ORDER, p)


def half(x, p):
    return (x >> 1) + ((p + 1) // 2 if x & 1 else 0)


def c_const(p):
    om = pow(rho(p), 1 << 30, p)
    om2 = om * om % p
    d = om - om2 if om >= om2 else om + (p - om2)     # the engine's overflow-free difference
    assert 0 <= d < p
    return d * pow(2, p - 2, p) % p


def dft(x, w, p):
    n = len(x)
    return [sum(x[j] * pow(w, j * t, p) for j in range(n)) % p for t in range(n)]


def fwd_stage(x, k, p):
    M = 1 << k
    w = pow(rho(p), 1 << (30 - k), p)
    c = c_const(p)
    y = [0] * (3 * M)
    for j in range(M):
        x0, x1, x2 = x[j], x[j + M], x[j + 2 * M]
        s, d = (x1 + x2) % p, (x1 - x2) % p
        t, e = (x0 - half(s, p)) % p, d * c % p
        w1 = pow(w, j, p)
        y[j] = (x0 + s) % p
        y[M + j] = (t + e) * w1 % p
        y[2 * M + j] = (t - e) * w1 * w1 % p
    return y


def inv_stage(z, k, p):
    M = 1 << k
    wi = pow(pow(rho(p), 1 << (30 - k), p), p - 2, p)
    c = c_const(p)
    x = [0] * (3 * M)
    for j in range(M):
        w1 = pow(wi, j, p)
        t0, t1, t2 = z[j], z[M + j] * w1 % p, z[2 * M + j] * w1 * w1 % p
        s, d = (t1 + t2) % p, (t1 - t2) % p
        q, e = (t0 - half(s, p)) % p, d * c % p
        x[j], x[M + j], x[2 * M + j] = (t0 + s) % p, (q - e) % p, (q + e) % p
    return x


def radix3_convolution(a, b, k, p, root_exp):
    M = 1 << k
    N = 3 * M
    a = a + [0] * (N - len(a))
    b = b + [0] * (N - len(b))
    ya, yb = fwd_stage(a, k, p), fwd_stage(b, k, p)
    # the chain's root: any primitive 2^k-th root (root_exp odd)
    wm = pow(pow(GEN[p], (p - 1) >> k, p), root_exp, p)
    wmi = pow(wm, p - 2, p)
    scale = pow(3 * M, p - 2, p)        # 1 / (3 2^k): the 1/3 rides on the sub-transforms' scale
    z = []
    for m in range(3):
        A, B = dft(ya[m * M:(m + 1) * M], wm, p), dft(yb[m * M:(m + 1) * M], wm, p)
        z += [v * scale % p for v in dft([x * y % p for x, y in zip(A, B)], wmi, p)]
    return inv_stage(z, k, p)


@pytest.mark.parametrize("p", [Q0, P3])
def test_constants(p):
    r = rho(p)
    assert pow(r, ORDER, p) == 1 and pow(r, 1 << 30, p) != 1 and pow(r, 3 << 29, p) != 1
    om = pow(r, 1 << 30, p)
    assert om != 1 and pow(om, 3, p) == 1
    c = c_const(p)
    assert 2 * c % p == (om - om * om) % p
    if p == Q0:
        # in q0 the cube roots of unity are 2^64 and 2^128 (2 has order 192);
        # om + p overflows 64 bits, which the difference above avoids
        assert om in (pow(2, 64, p), pow(2, 128, p)) and om + p >= 1 << 64
    for x in (0, 1, 2, 3, p - 1, p - 2, p // 2, (1 << 32) + 5):
        x %= p
        assert half(x, p) < p and 2 * half(x, p) % p == x


@pytest.mark.parametrize("p", [Q0, P3])
@pytest.mark.parametrize("k", [1, 2, 3, 4])
def test_radix3_gives_cyclic_convolution(p, k):
    rng = random.Random(31 * k + (p & 0xFFFF))
    M = 1 << k
    N = 3 * M
    for trial in range(4):
        na, nb = rng.randint(1, N), rng.randint(1, N)
        a = [rng.randrange(1 << 32) for _ in range(na)]
        b = [rng.randrange(1 << 32) for _ in range(nb)]
        want = [0] * N
        for i, x in enumerate(a):
            for j, y in enumerate(b):
                want[(i + j) % N] = (want[(i + j) % N] + x * y) % p
        root_exp = 1 + 2 * rng.randrange(M // 2) if M > 1 else 1
        assert radix3_convolution(a, b, k, p, root_exp) == want, (p, k, trial)


@pytest.mark.parametrize("p", [Q0, P3])
def test_stages_alone_give_three_x(p):
    # the stages without the sub-transforms multiply by 3 (the 1/3 is the
    # inverse sub-transforms'), as gbntt_debug_radix3 mode 0 reports
    rng = random.Random(5)
    for k in (1, 3, 5):
        x = [rng.randrange(1 << 32) % p for _ in range(3 << k)]
        assert inv_stage(fwd_stage(x, k, p), k, p) == [3 * v % p for v in x]


@pytest.mark.parametrize("p", [Q0, P3])
def test_stepped_twiddles(p):
    # a thread's twiddles: w^j from the two-level tables (rho^(i 2^15) and
    # rho^i), then times w^G per step; forward and inverse
    for k, G in ((10, 256 * 3), (20, 256 * 4096), (28, 256 * 65535)):
        w = pow(rho(p), 1 << (30 - k), p)
        e_step = (G << (30 - k)) % ORDER
        step_f, step_i = pow(rho(p), e_step, p), pow(rho(p), (ORDER - e_step) % ORDER, p)
        for j in (0, 1, 12345 % (1 << k)):
            e = j << (30 - k)
            hi, lo = pow(rho(p), (e >> 15) << 15, p), pow(rho(p), e & 32767, p)
            assert hi * lo % p == pow(w, j, p)
            assert pow(w, j, p) * pow(step_f, 3, p) % p == pow(w, j + 3 * G, p)
            assert pow(w, -j % ORDER, p) * step_i % p == pow(w, (-(j + G)) % ORDER, p)
