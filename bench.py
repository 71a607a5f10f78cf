#!/usr/bin/env python
"""Benchmark of the CRT-NTT big-integer multiply on one GB300.

Workload (default): one multiply of two seeded uniform-random operands of
2^28 32-bit limbs (1 GiB each), transform length N = 2^29 per prime over two
primes: q0 = 2^64 - 2^32 + 1 (uint64 residues) and p3 = 3 * 2^30 + 1
(uint32 residues), whose product exceeds every coefficient of the product
(the reference's three 64-bit primes 2^64 - 2^b + 1, b = 32, 34, 40, are
timed beside it). A step is one full multiply (decomposition, 2 x 2 forward
transforms, pointwise product, 2 inverse transforms, Garner + carry).
Inputs (2 x 1 GiB) and the 12 GiB of spectra are far larger than the 129 MB
L2, so no L2 flush is needed between steps.

Prints one JSON line. ``value`` is milliseconds per multiply with the
operands already resident in HBM (CUDA events on the engine stream); ``e2e``
is the same metric through the reference-facing C-ABI call ntt_bigint_mul on
pinned host BigInts (2 GiB in, 2 GiB out per step, host wall clock).
``--impl reference`` times the reference CPU path (the oracle restatement of
the reference's scatter / NTT / Garner / gather, all host threads) on a
bounded sample and scales it to the same metric.

Under torchrun (--gpus N > 1) every rank runs an independent replica on its
own GPU (the multiply does not shard across GPUs); ``value`` is then the
max-over-ranks step time divided by the number of multiplies all ranks did.
"""
import argparse
import ctypes
import json
import os
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "ms per 2^28-limb multiply (% HBM roofline)"
UNIT = "ms"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--log-limbs", type=int, default=28, help="operand size 2^k limbs (28 = headline)")
    ap.add_argument("--e2e-steps", type=int, default=5)
    ap.add_argument("--cpu-log-limbs", type=int, default=22, help="CPU baseline sample size 2^k limbs")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--cpu-full", type=int, default=1,
                    help="also time one full-size product by the CPU port (all cores but one) and GMP (one core)")
    ap.add_argument("--plan", default="", help="comma-separated pass sizes overriding the default plan")
    ap.add_argument("--no-packed", action="store_true", help="skip the packed (64-bit coefficient) measurement")
    ap.add_argument("--batch-pairs", type=int, default=4096)
    ap.add_argument("--batch-reps", type=int, default=2)
    ap.add_argument("--no-batched", action="store_true", help="skip the batched-products leg")
    ap.add_argument("--no-serving", action="store_true", help="skip the serving leg")
    ap.add_argument("--no-negacyclic", action="store_true", help="skip the negacyclic polynomial-product leg")
    ap.add_argument("--nega-log", type=int, default=24, help="negacyclic leg: N = 2^k coefficients")
    ap.add_argument("--serve-requests", type=int, default=10000)
    ap.add_argument("--serve-saturation", type=int, default=3000)
    ap.add_argument("--serve-slots", type=int, default=4)
    ap.add_argument("--no-three-prime", action="store_true",
                    help="skip timing the same multiply with the reference's three 64-bit primes")
    ap.add_argument("--three-prime-steps", type=int, default=5)
    ap.add_argument("--no-square", action="store_true", help="skip the squaring and 2^20-limb legs")
    ap.add_argument("--no-radix3", action="store_true",
                    help="skip the leg timing products of 3 2^k points against the next power of two")
    ap.add_argument("--radix3-logs", default="20,22,24", help="radix-3 leg: the k of its 3 2^k-point products")
    ap.add_argument("--no-e", action="store_true", help="skip the e-digits leg")
    ap.add_argument("--e-digits", type=int, default=10 ** 8)
    ap.add_argument("--e-reps", type=int, default=3)
    ap.add_argument("--e-cpu-digits", type=int, default=10 ** 7, help="CPU baseline sample of the e leg")
    return ap.parse_args()


def dist_env():
    return int(os.environ.get("RANK", 0)), int(os.environ.get("WORLD_SIZE", 1)), int(os.environ.get("LOCAL_RANK", 0))


class Dist:
    """Barrier and max-reduction across ranks (gloo over torch.distributed)
    for N > 1; no-ops for a single process."""

    def __init__(self):
        self.rank, self.world, self.local = dist_env()
        self.torch = None
        if self.world > 1:
            import torch
            import torch.distributed as td
            td.init_process_group("gloo")
            self.torch, self.td = torch, td

    def barrier(self):
        if self.torch:
            self.td.barrier()

    def max(self, v):
        if not self.torch:
            return v
        t = self.torch.tensor([float(v)], dtype=self.torch.float64)
        self.td.all_reduce(t, op=self.td.ReduceOp.MAX)
        return float(t.item())

    def close(self):
        if self.torch:
            self.td.destroy_process_group()


def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def bytes_model(log_limbs):
    """Whole-multiply algorithmic bytes: 10 k N 8 + 8 (n_a + n_b), k = 3."""
    n = 1 << log_limbs
    N = 1 << (log_limbs + 1)
    return 10 * 3 * N * 8 + 8 * (2 * n)


class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
        self.gpu = gpu_index
        try:
            self.p = subprocess.Popen(["nvidia-smi", "-i", str(gpu_index), "--query-gpu=" + self.FIELDS,
                                       "--format=csv,noheader,nounits", "-lms", "100"], stdout=self.f,
                                      stderr=subprocess.DEVNULL)
        except OSError:
            self.p = None

    def stop(self):
        if self.p is None:
            return None
        self.p.terminate()
        try:
            self.p.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.p.kill()
        self.f.flush()
        rows = []
        for line in open(self.f.name):
            parts = [x.strip() for x in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                rows.append((float(parts[1]), float(parts[2]), parts[5:9], float(parts[3])))
            except ValueError:
                continue
        os.unlink(self.f.name)
        if not rows:
            return None
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if r[2][i].lower() == "active"})
        sm = sorted(r[0] for r in rows)
        return {"sm_mhz": sm[len(sm) // 2], "sm_max_mhz": max(r[1] for r in rows), "reasons": reasons,
                "samples": len(rows), "power_w_max": max(r[3] for r in rows)}


def host_info():
    model = ""
    try:
        for line in open("/proc/cpuinfo"):
            if line.lower().startswith(("model name", "cpu part", "hardware")):
                model = line.split(":", 1)[1].strip()
                break
    except OSError:
        pass
    return {"nproc": os.cpu_count(), "arch": os.uname().machine, "cpu": model,
            "omp_num_threads": os.environ.get("OMP_NUM_THREADS")}


def cpu_baseline(log_limbs_sample, log_limbs_target, reps=1, with_gmp=True):
    """Oracle CRT-NTT (restatement of the reference CPU path) on one bounded
    sample, all host threads, scaled to the target size by N log N."""
    import oracle
    from cryptography_gb300 import synth
    n = 1 << log_limbs_sample
    a = synth.operand(n, 101)
    b = synth.operand(n, 202)
    times = []
    for _ in range(reps):
        t0 = time.perf_counter()
        oracle.mul(a, b)
        times.append(time.perf_counter() - t0)
    t = min(times)
    Ns, Nt = 2 * n, 1 << (log_limbs_target + 1)
    scale = (Nt * (log_limbs_target + 1)) / (Ns * (log_limbs_sample + 1))
    out = {"value": t * 1e3 * scale, "unit": UNIT, "cores": oracle.num_threads(), "kind": "port",
           "sample": "one 2^%d x 2^%d-limb multiply by the oracle CRT-NTT (scatter, radix-2 NTT per prime, "
                     "Garner, gather; OpenMP) took %.2f s; scaled by N log N (x%.1f) to 2^%d limbs"
                     % (log_limbs_sample, log_limbs_sample, t, scale, log_limbs_target),
           "host": host_info()}
    if with_gmp and oracle.gmp_available():
        t0 = time.perf_counter()
        oracle.gmp_mul(a, b)
        tg = time.perf_counter() - t0
        out["gmp_mpz_mul_1thread_sample_s"] = tg
    return out


def _host_mem_available():
    try:
        for line in open("/proc/meminfo"):
            if line.startswith("MemAvailable:"):
                return int(line.split()[1]) * 1024
    except OSError:
        pass
    return os.sysconf("SC_AVPHYS_PAGES") * os.sysconf("SC_PAGE_SIZE")


def cpu_full_size(log_limbs):
    """One full-size multiply (2^k x 2^k limbs, the headline workload's own
    operands) by the oracle CRT-NTT port on all host cores but one, timed
    while GMP mpz_mul multiplies the same operands on the remaining core;
    both products are compared. Skipped (with the reason) when the host has
    too little free memory for both (about 30 GiB for the port at 2^28
    limbs plus GMP's working space)."""
    import threading
    import oracle
    from cryptography_gb300 import synth
    n = 1 << log_limbs
    need = 160 * n
    avail = _host_mem_available()
    if avail < need:
        return {"skipped": "host has %.1f GiB free, the two full-size CPU products need about %.1f GiB"
                           % (avail / 2 ** 30, need / 2 ** 30)}
    a = synth.operand(n, 1)
    b = synth.operand(n, 2)
    threads = max(1, (os.cpu_count() or 2) - 1)
    res = {}

    def run_gmp():
        t0 = time.perf_counter()
        res["gmp"] = oracle.gmp_mul(a, b)
        res["gmp_s"] = time.perf_counter() - t0

    out = {"operands": "2^%d x 2^%d limbs, seeds 1 and 2 (the headline operands)" % (log_limbs, log_limbs)}
    th = None
    if oracle.gmp_available():
        th = threading.Thread(target=run_gmp)
        th.start()
    prev = oracle.num_threads()
    oracle.set_threads(threads)
    try:
        t0 = time.perf_counter()
        c = oracle.mul(a, b)
        out["port_s"] = time.perf_counter() - t0
        out["port_threads"] = threads
    finally:
        oracle.set_threads(prev)
    if th is not None:
        th.join()
        out["gmp_s"] = res["gmp_s"]
        out["gmp_threads"] = 1
        out["port_equals_gmp"] = bool(np.array_equal(c, res["gmp"]))
    return out


def batched_sizes(pairs, seed, lo=10, hi=22):
    """Operand sizes log-uniform in 2^lo .. 2^hi limbs (independent per
    operand), seeded."""
    from cryptography_gb300 import synth
    return synth.batched_sizes(pairs, seed, lo, hi)


# transform-length buckets (log2 N ranges, lower bound exclusive) of the
# batched and serving breakdowns
BUCKETS = (("N<=2^16", 0, 16), ("2^16<N<=2^20", 16, 20), ("N>2^20", 20, 64))


def run_batched_leg(g, cudart, args, stream):
    """4096 independent pairs, batched engine against looping the plain
    single-product path on the same device-resident operands."""
    pairs = args.batch_pairs
    na, nb = batched_sizes(pairs, 4242)
    L = g.lib()
    bufs = []
    a_ptr, b_ptr, c_ptr, p_ptr = [], [], [], []
    for i in range(pairs):
        da, db = cudart.DeviceBuffer(4 * int(na[i])), cudart.DeviceBuffer(4 * int(nb[i]))
        dc, dp = cudart.DeviceBuffer(4 * int(na[i] + nb[i])), cudart.DeviceBuffer(4 * int(na[i] + nb[i]))
        L.gbntt_fill_operand(da.ptr, int(na[i]), 1000 + 2 * i, None)
        L.gbntt_fill_operand(db.ptr, int(nb[i]), 1001 + 2 * i, None)
        bufs += [da, db, dc, dp]
        a_ptr.append(da.ptr); b_ptr.append(db.ptr); c_ptr.append(dc.ptr); p_ptr.append(dp.ptr)
    cudart.synchronize()
    na_l, nb_l = [int(x) for x in na], [int(x) for x in nb]

    def batched():
        g.batch_mul_device(c_ptr, a_ptr, na_l, b_ptr, nb_l, None)

    def plain():
        for i in range(pairs):
            g.mul_device(p_ptr[i], a_ptr[i], na_l[i], b_ptr[i], nb_l[i], None)

    res = {}
    for name, fn in (("batched", batched), ("plain", plain)):
        fn()
        cudart.stream_sync(stream)
        e0, e1 = cudart.Event(), cudart.Event()
        reps = args.batch_reps
        e0.record(stream)
        t0 = time.perf_counter()
        for _ in range(reps):
            fn()
        e1.record(stream)
        e1.synchronize()
        res[name] = {"ms": e0.elapsed_ms(e1) / reps, "host_ms": (time.perf_counter() - t0) * 1e3 / reps}
    flags = g.device_errors()
    # consistency: batched and plain outputs of a sample of pairs are identical
    rng = np.random.default_rng(7)
    sample = sorted(set(int(x) for x in rng.integers(0, pairs, 48)) | {int(np.argmax(na + nb)), int(np.argmin(na + nb))})
    same = True
    for i in sample:
        n = na_l[i] + nb_l[i]
        x = bufs[4 * i + 2].download(np.uint32, n)
        y = bufs[4 * i + 3].download(np.uint32, n)
        same &= bool(np.array_equal(x, y))
    bm = 0
    for i in range(pairs):
        N = 1 << max(5, int(np.ceil(np.log2(na_l[i] + nb_l[i] - 1))))
        bm += 10 * 3 * N * 8 + 8 * (na_l[i] + nb_l[i])
    # where batching pays: the same comparison over the pairs of each
    # transform-length bucket alone
    by_size = {}
    logN = [max(5, int(np.ceil(np.log2(na_l[i] + nb_l[i] - 1)))) for i in range(pairs)]
    for name, lo, hi in BUCKETS:
        sel = [i for i in range(pairs) if lo < logN[i] <= hi]
        if not sel:
            continue

        def bb():
            g.batch_mul_device([c_ptr[i] for i in sel], [a_ptr[i] for i in sel], [na_l[i] for i in sel],
                               [b_ptr[i] for i in sel], [nb_l[i] for i in sel], None)

        def pp():
            for i in sel:
                g.mul_device(p_ptr[i], a_ptr[i], na_l[i], b_ptr[i], nb_l[i], None)

        t = {}
        for nm, fn in (("batched", bb), ("plain", pp)):
            fn()
            cudart.stream_sync(stream)
            e0, e1 = cudart.Event(), cudart.Event()
            e0.record(stream)
            for _ in range(args.batch_reps):
                fn()
            e1.record(stream)
            e1.synchronize()
            t[nm] = e0.elapsed_ms(e1) / args.batch_reps
        by_size[name] = {"pairs": len(sel), "batched_ms": t["batched"], "plain_ms": t["plain"],
                         "batched_products_per_s": len(sel) / (t["batched"] * 1e-3),
                         "plain_products_per_s": len(sel) / (t["plain"] * 1e-3),
                         "speedup": t["plain"] / t["batched"]}
    for b in bufs:
        b.free()
    out = {"pairs": pairs, "sizes": "log2(n) uniform in [10, 22] per operand, seed 4242",
           "batched_ms": res["batched"]["ms"], "plain_ms": res["plain"]["ms"],
           "batched_products_per_s": pairs / (res["batched"]["ms"] * 1e-3),
           "plain_products_per_s": pairs / (res["plain"]["ms"] * 1e-3),
           "speedup": res["plain"]["ms"] / res["batched"]["ms"],
           "plain_host_ms": res["plain"]["host_ms"],
           "bytes_model": bm, "batched_GBps_model": bm / (res["batched"]["ms"] * 1e-3) / 1e9,
           "batched_equals_plain_on_sample": same, "sample_pairs": len(sample), "device_error_flags": flags,
           "by_size": by_size,
           "plain_path": "gbntt_mul_u32 per pair, device pointers, one stream, no host sync per pair"}
    return out


def run_serving_leg(g, cudart, args, stream):
    """Poisson arrivals of multiply requests (sizes log-uniform 2^8..2^24
    limbs per operand, seeded) against the continuous-batching server, at
    0.7 x the serial capacity of the plain path; then a saturation run."""
    L = g.lib()
    rng = np.random.default_rng(5150)
    nreq = args.serve_requests
    warm = 200
    na = np.floor(2.0 ** rng.uniform(8, 24, nreq + warm + 300)).astype(np.int64)
    nb = np.floor(2.0 ** rng.uniform(8, 24, nreq + warm + 300)).astype(np.int64)
    pool = cudart.DeviceBuffer(4 << 25)
    L.gbntt_fill_operand(pool.ptr, 1 << 25, 99, None)
    arena_limbs = 1 << 32
    arena = cudart.DeviceBuffer(4 * arena_limbs)
    cudart.synchronize()
    a_ptr = pool.ptr
    b_ptr = pool.ptr + 4 * (1 << 24)

    # serial capacity of the plain path on the same size mix
    t_plain = []
    for i in range(nreq + warm, nreq + warm + 300):
        t0 = time.perf_counter()
        g.mul_device(arena.ptr, a_ptr, int(na[i]), b_ptr, int(nb[i]), None)
        cudart.stream_sync(stream)
        t_plain.append(time.perf_counter() - t0)
    t_plain = float(np.mean(t_plain[20:]))
    cap_plain = 1.0 / t_plain

    srv = g.Server(slots=args.serve_slots, slot_log=26)
    try:
        def run(indices, rate):
            arrivals = np.cumsum(rng.exponential(1.0 / rate, len(indices))) if rate else np.zeros(len(indices))
            head, inflight, tickets = 0, [], []
            start = time.perf_counter()
            for k, i in enumerate(indices):
                n_out = int(na[i] + nb[i])
                if head + n_out > arena_limbs:
                    head = 0
                # wait for in-flight requests whose output overlaps [head, head + n_out)
                while inflight and inflight[0][1] < head + n_out and inflight[0][1] + inflight[0][2] > head:
                    srv.wait(inflight.pop(0)[0], 120.0)
                now = time.perf_counter() - start
                if arrivals[k] > now:
                    while time.perf_counter() - start < arrivals[k]:
                        pass
                t = srv.submit(arena.ptr + 4 * head, a_ptr, int(na[i]), b_ptr, int(nb[i]))
                tickets.append(t)
                inflight.append((t, head, n_out))
                head += n_out
            for t in tickets:
                srv.wait(t, 300.0)
            wall = time.perf_counter() - start
            lat = np.array([srv.query(t)[1] for t in tickets]) / 1e3
            return wall, lat

        run(list(range(nreq, nreq + warm)), 0.7 * cap_plain)
        rate = 0.7 * cap_plain
        wall, lat = run(list(range(nreq)), rate)
        st = srv.stats()
        sat_n = min(nreq, args.serve_saturation)
        sat_wall, sat_lat = run(list(range(sat_n)), None)
        st2 = srv.stats()
        # saturation and serial plain capacity per transform-length bucket:
        # requests of the same size distribution restricted to the bucket
        by_size = {}
        logN = np.maximum(5, np.ceil(np.log2(na + nb - 1))).astype(int)
        for name, lo, hi in BUCKETS:
            idx = [int(i) for i in np.flatnonzero((logN > lo) & (logN <= hi))]
            if not idx:
                continue
            sub = idx[:{"N<=2^16": 3000, "2^16<N<=2^20": 1500}.get(name, 400)]
            tp = []
            for i in sub[:200]:
                t0 = time.perf_counter()
                g.mul_device(arena.ptr, a_ptr, int(na[i]), b_ptr, int(nb[i]), None)
                cudart.stream_sync(stream)
                tp.append(time.perf_counter() - t0)
            cap_b = 1.0 / float(np.mean(tp[10:] if len(tp) > 20 else tp))
            w0 = srv.stats()
            bw, blat = run(sub, None)
            w1 = srv.stats()
            by_size[name] = {"requests": len(sub), "served_products_per_s": len(sub) / bw,
                             "serial_plain_products_per_s": cap_b, "vs_serial_plain": (len(sub) / bw) / cap_b,
                             "latency_ms_p50": float(np.percentile(blat, 50)),
                             "latency_ms_p99": float(np.percentile(blat, 99)),
                             "products_per_wave": (w1["wave_products"] - w0["wave_products"])
                             / max(1, w1["waves"] - w0["waves"])}
    finally:
        srv.stop()
    pool.free()
    arena.free()
    return {"requests": nreq, "sizes": "log2(n) uniform in [8, 24] per operand, seed 5150", "warmup_requests": warm,
            "offered_rate_per_s": rate, "served_products_per_s": nreq / wall,
            "latency_ms_p50": float(np.percentile(lat, 50)), "latency_ms_p99": float(np.percentile(lat, 99)),
            "latency_ms_mean": float(lat.mean()),
            "serial_plain_products_per_s": cap_plain, "serial_plain_ms_per_product": t_plain * 1e3,
            "saturation": {"requests": sat_n, "products_per_s": sat_n / sat_wall,
                           "vs_serial_plain": (sat_n / sat_wall) / cap_plain,
                           "latency_ms_p50": float(np.percentile(sat_lat, 50)),
                           "latency_ms_p99": float(np.percentile(sat_lat, 99))},
            "slots": args.serve_slots, "slot_coefficients": 1 << 26,
            "waves": st2["waves"], "products_per_wave": st2["wave_products"] / max(1, st2["waves"]),
            "by_size": by_size,
            "admission": "a free slot takes pending requests in arrival order while the sum of their transform "
                         "lengths fits the slot workspace; they run as one sub-wave per transform length, "
                         "shortest first, back to back on the slot stream",
            "device_error_flags": st2["device_errors"],
            "latency": "submit -> completion observed by the server thread (host clock)",
            "load": "0.7 x serial capacity of the plain path (gbntt_mul_u32 + sync per request)"}


def run_e_leg(args):
    """e to args.e_digits digits through gbntt_compute_e (the whole pipeline:
    product tree, numerator x 10^(D-1), Newton division, decimal conversion;
    the digit string lands in host memory), checked against the reference's
    own digits (sha256 in tests/golden/e_digits.json); CPU baseline: the same
    algorithm on GMP (oracle/e_gmp_oracle.c, one thread) at a bounded
    sample."""
    import hashlib
    from cryptography_gb300 import arith
    D = args.e_digits
    gold = {}
    gp = os.path.join(ROOT, "tests", "golden", "e_digits.json")
    if os.path.exists(gp):
        gold = json.load(open(gp)).get(str(D), {})
    arith.compute_e(min(D, 10 ** 6))   # warm-up
    buf = arith.e_buffer(D)            # host output buffer, allocated before the timed calls
    runs = []
    for _ in range(max(1, args.e_reps)):
        t0 = time.perf_counter()
        ph = arith.compute_e_raw(D, buf)
        runs.append((time.perf_counter() - t0, ph))
    best = min(runs, key=lambda r: r[0])
    digest = hashlib.sha256(memoryview(buf)[:D + 1]).hexdigest()
    out = {"digits": D, "seconds": best[0], "seconds_all": [r[0] for r in runs],
           "phases_s": dict(zip(("product_tree", "numerator_x_10pow", "division", "decimal", "total"), best[1])),
           "sha256": digest, "matches_reference_digits": (digest == gold["sha256"]) if gold else None,
           "api": "gbntt_compute_e (C ABI) wall time, \"2.718...\" written to a host buffer",
           "engine_transform_log_needed": arith.e_required_log(D)}
    if gold:
        out["reference_cpu_recorded"] = {"seconds": gold.get("reference_seconds"), "cores": gold.get("cores"),
                                         "note": "reference host compute_e (GMP multiply shim) when the digits "
                                                 "were recorded; other host"}
    if not args.no_cpu and args.e_cpu_digits > 0:
        try:
            from oracle import e_oracle
            cs, ct = e_oracle.gmp_e_string(args.e_cpu_digits)
            cg = json.load(open(gp)).get(str(args.e_cpu_digits), {}) if os.path.exists(gp) else {}
            out["cpu_baseline"] = {"value": ct, "unit": "s", "cores": 1, "kind": "port",
                                   "sample": "e to %d digits, reference algorithm on GMP (e_gmp_oracle.c)"
                                             % args.e_cpu_digits,
                                   "matches_reference_digits": (hashlib.sha256(cs.encode()).hexdigest()
                                                                == cg.get("sha256")) if cg else None}
        except Exception as ex:   # the baseline is reported, never required
            out["cpu_baseline"] = {"error": str(ex)}
    return out


def run_reference(args, dist):
    if dist.rank != 0:
        return 0
    times = []
    res = None
    for i in range(args.warmup + args.steps):
        r = cpu_baseline(args.cpu_log_limbs, args.log_limbs, with_gmp=(i == args.warmup + args.steps - 1))
        if i >= args.warmup:
            times.append(r["value"])
            res = r
    v = float(np.median(times))
    res["value"] = v
    res["value_kind"] = "sample scaled by N log N"
    if args.cpu_full and not args.no_cpu:
        # one full-size product measured on the same cores: the scaled
        # samples are reported next to it, with their error
        full = cpu_full_size(args.log_limbs)
        res["measured_full"] = full
        if "port_s" in full:
            res["measured_full_s"] = {"port": full["port_s"], "gmp_1thread": full.get("gmp_s")}
            res["extrapolation_error"] = v / (full["port_s"] * 1e3) - 1.0
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": v, "higher_is_better": False,
            "scaling": "weak", "vs_baseline": None, "dtype": "u64", "data": "synthetic (seeded splitmix64 limbs)",
            "config": {"workload": "2^%d x 2^%d 32-bit limbs, N=2^%d, 3 primes" % (args.log_limbs, args.log_limbs,
                                                                                    args.log_limbs + 1),
                       "sample_log_limbs": args.cpu_log_limbs},
            "cpu_baseline": res, "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    return 0


def run_gpu(args, dist):
    import cryptography_gb300 as g
    from cryptography_gb300 import cudart, synth

    cudart.set_device(dist.local)
    lg = args.log_limbs
    n = 1 << lg
    g.init(lg + 1)
    if args.plan:
        g.set_plan(lg + 1, [int(x) for x in args.plan.split(",")])
    stream = g.lib().gbntt_stream()
    a = synth.operand(n, 1 + 2 * dist.rank)
    b = synth.operand(n, 2 + 2 * dist.rank)
    da, db, dc = cudart.DeviceBuffer(4 * n), cudart.DeviceBuffer(4 * n), cudart.DeviceBuffer(8 * n)
    da.upload(a)
    db.upload(b)

    def step():
        g.mul_device(dc.ptr, da.ptr, n, db.ptr, n, None)

    for _ in range(args.warmup):
        step()
    cudart.stream_sync(stream)
    flags = g.device_errors()

    clocks = ClockSampler(dist.local)
    dist.barrier()
    cudart.synchronize()
    e0, e1 = cudart.Event(), cudart.Event()
    e0.record(stream)
    for _ in range(args.steps):
        step()
    e1.record(stream)
    e1.synchronize()
    cudart.synchronize()
    dist.barrier()
    total_ms = e0.elapsed_ms(e1)
    clk = clocks.stop()
    flags |= g.device_errors()
    total_ms = dist.max(total_ms)
    ms = total_ms / (args.steps * dist.world)

    # the same multiply with the reference's prime set (three 64-bit primes)
    three = None
    if not args.no_three_prime and args.three_prime_steps > 0:
        g.set_prime_set(3)
        try:
            for _ in range(2):
                step()
            t0, t1 = cudart.Event(), cudart.Event()
            dist.barrier()
            t0.record(stream)
            for _ in range(args.three_prime_steps):
                step()
            t1.record(stream)
            t1.synchronize()
            dist.barrier()
            tms = dist.max(t0.elapsed_ms(t1)) / (args.three_prime_steps * dist.world)
        finally:
            g.set_prime_set(2)
        flags |= g.device_errors()
        three = {"ms": tms, "steps": args.three_prime_steps,
                 "primes": "2^64-2^b+1, b = 32, 34, 40 (the reference's set; 64-bit residues)",
                 "note": "same product, same transform length; the headline uses two primes"}

    # squaring of the same operand (one forward transform), reported apart
    square = small = None
    if not args.no_square:
        def sq_step():
            g.mul_device(dc.ptr, da.ptr, n, da.ptr, n, None)
        for _ in range(2):
            sq_step()
        s0, s1 = cudart.Event(), cudart.Event()
        dist.barrier()
        s0.record(stream)
        for _ in range(args.steps):
            sq_step()
        s1.record(stream)
        s1.synchronize()
        dist.barrier()
        sq_ms = dist.max(s0.elapsed_ms(s1)) / (args.steps * dist.world)
        bm_sq = 6 * 3 * (1 << (lg + 1)) * 8 + 12 * n
        square = {"ms": sq_ms, "bytes_model": bm_sq, "model": "6*k*N*8 + 12*n, k=3",
                  "frac": bm_sq / (sq_ms * 1e-3) / 1e9 / peaks()[0]}
        # the 2^20 x 2^20-limb product (N = 2^21), checked against GMP
        ns = 1 << 20
        xa, xb = synth.operand(ns, 11), synth.operand(ns, 12)
        sa, sb, sc = cudart.DeviceBuffer(4 * ns), cudart.DeviceBuffer(4 * ns), cudart.DeviceBuffer(8 * ns)
        sa.upload(xa)
        sb.upload(xb)
        for _ in range(3):
            g.mul_device(sc.ptr, sa.ptr, ns, sb.ptr, ns, None)
        k0, k1 = cudart.Event(), cudart.Event()
        reps = 50
        k0.record(stream)
        for _ in range(reps):
            g.mul_device(sc.ptr, sa.ptr, ns, sb.ptr, ns, None)
        k1.record(stream)
        k1.synchronize()
        sm_ms = k0.elapsed_ms(k1) / reps
        bm_small = 10 * 3 * (1 << 21) * 8 + 8 * (2 * ns)
        small = {"ms": sm_ms, "operand_limbs": ns, "transform_log": 21, "steps": reps,
                 "bytes_model": bm_small, "frac": bm_small / (sm_ms * 1e-3) / 1e9 / peaks()[0],
                 "parity": "tests/test_gpu_parity.py checks this size against GMP"}
        for buf in (sa, sb, sc):
            buf.free()
        flags |= g.device_errors()

    radix3 = None if args.no_radix3 else run_radix3_leg(g, cudart, synth, lg, stream,
                                                        [int(x) for x in args.radix3_logs.split(",") if x])
    if radix3:
        flags |= radix3["device_error_flags"]

    # packed mode (one 64-bit limb per coefficient, transform length 2^lg)
    packed = None
    if not args.no_packed:
        def step64():
            g.lib().gbntt_mul_u64(dc.ptr, da.ptr, n // 2, db.ptr, n // 2, None)
        for _ in range(args.warmup):
            step64()
        cudart.stream_sync(stream)
        p0, p1 = cudart.Event(), cudart.Event()
        dist.barrier()
        p0.record(stream)
        for _ in range(args.steps):
            step64()
        p1.record(stream)
        p1.synchronize()
        dist.barrier()
        pms = dist.max(p0.elapsed_ms(p1)) / (args.steps * dist.world)
        flags |= g.device_errors()
        bmp = 10 * 3 * (1 << lg) * 8 + 8 * (2 * n)
        packed = {"ms": pms, "transform_log": lg, "bytes_model": bmp,
                  "multiply_roofline_frac": bmp / (pms * 1e-3) / 1e9 / peaks()[0],
                  "note": "same integers as 2^%d 64-bit limbs, one coefficient per limb (reference granularity); "
                          "not the headline configuration" % (lg - 1)}

    negacyclic = None
    if not args.no_negacyclic and dist.rank == 0:
        negacyclic = run_negacyclic_leg(g, cudart, args, stream)
        flags |= g.device_errors()

    batched = None
    if not args.no_batched and dist.rank == 0:
        batched = run_batched_leg(g, cudart, args, stream)
        flags |= batched["device_error_flags"]

    serving = None
    if not args.no_serving and dist.rank == 0:
        serving = run_serving_leg(g, cudart, args, stream)
        flags |= serving["device_error_flags"]

    e_leg = None
    if not args.no_e and dist.rank == 0:
        e_leg = run_e_leg(args)
        flags |= g.device_errors()

    # per-launch breakdown of one multiply (separate, instrumented run)
    g.launch_log(True)
    step()
    recs = g.launch_records()
    g.launch_log(False)
    launches_per_step = len(recs)
    by_kind = {}
    for kind, log_l, nbytes, t in recs:
        d = by_kind.setdefault(kind, {"launches": 0, "ms": 0.0, "bytes": 0.0})
        d["launches"] += 1
        d["ms"] += t
        d["bytes"] += nbytes
    tot = sum(d["ms"] for d in by_kind.values()) or 1.0
    for d in by_kind.values():
        d["share"] = d["ms"] / tot
        d["GBps"] = d["bytes"] / (d["ms"] * 1e-3) / 1e9 if d["ms"] > 0 else None
    pass_kinds = [k for k in by_kind if "pass" in k]
    pass_ms = sum(by_kind[k]["ms"] for k in pass_kinds)
    pass_bytes = sum(by_kind[k]["bytes"] for k in pass_kinds)
    pass_launches = sum(by_kind[k]["launches"] for k in pass_kinds)
    peak, peak_kind = peaks()
    achieved = pass_bytes / (pass_ms * 1e-3) / 1e9
    traffic = None
    tp = os.path.join(ROOT, "profiles", "ncu_traffic.json")
    if os.path.exists(tp):
        try:
            tj = json.load(open(tp))
            traffic = tj.get("ntt_pass_kernel_bytes_per_launch" if g.prime_set() == 2 else
                             "three_prime_64bit_bytes_per_launch")
        except (ValueError, OSError):
            traffic = None
    issue = None
    ip = os.path.join(ROOT, "profiles", "ncu_issue.json")
    if os.path.exists(ip) and g.prime_set() == 2:
        try:
            ij = json.load(open(ip))
            scale = float(1 << (lg + 1)) / float(1 << 27)   # the capture's transform length is 2^27
            inst = ij["multiply_2pow27_warp_instructions"] * scale
            alu = ij["multiply_2pow27_alu_warp_instructions"] * scale
            sms = cudart.sm_count()
            sm_hz = float((clk or {}).get("sm_mhz") or 2070.0) * 1e6   # SM clock sampled in the timed region
            cap = sms * 4 * sm_hz * ms * 1e-3          # warp-instruction issue slots in one multiply
            issue = {"bound": "integer issue", "instructions_per_multiply": inst,
                     "achieved": inst / (ms * 1e-3), "peak": sms * 4 * sm_hz, "unit": "warp instructions/s",
                     "frac": inst / cap, "alu_pipe_frac": 2.0 * alu / cap,
                     "sm_mhz": sm_hz / 1e6, "source": "profiles/ncu_issue.json (ncu instruction counts of one "
                                                    "2^27-point multiply, scaled to this transform length)"}
        except (ValueError, OSError, KeyError):
            issue = None
    bm = bytes_model(lg)
    res_bytes = 12 if g.prime_set() == 2 else 24
    bm_own = 10 * (1 << (lg + 1)) * res_bytes + 8 * (2 * n)

    # e2e through the reference-facing C ABI with pinned host BigInts
    e2e = None
    if args.e2e_steps > 0:
        n64 = n // 2
        pa, pb = cudart.PinnedBuffer(n64, np.uint64), cudart.PinnedBuffer(n64, np.uint64)
        pc = cudart.PinnedBuffer(2 * n64 + 8, np.uint64)
        pa.array[:] = a.view(np.uint64)
        pb.array[:] = b.view(np.uint64)
        u64p = ctypes.POINTER(ctypes.c_uint64)
        A = g.BigInt(ctypes.cast(pa.ptr, u64p), n64, n64, 0)
        B = g.BigInt(ctypes.cast(pb.ptr, u64p), n64, n64, 0)
        C = g.BigInt(ctypes.cast(pc.ptr, u64p), 0, 2 * n64 + 8, 0)
        L = g.lib()
        L.ntt_bigint_mul(ctypes.byref(C), ctypes.byref(A), ctypes.byref(B))
        dist.barrier()
        per = []
        for _ in range(args.e2e_steps):
            t0 = time.perf_counter()
            L.ntt_bigint_mul(ctypes.byref(C), ctypes.byref(A), ctypes.byref(B))
            per.append((time.perf_counter() - t0) * 1e3)
        t_e2e = sum(per)
        dist.barrier()
        t_e2e = dist.max(t_e2e)
        e2e = {"value": t_e2e / (args.e2e_steps * dist.world), "unit": UNIT, "h2d_bytes_per_step": 8 * n,
               "d2h_bytes_per_step": 8 * n, "api": "ntt_bigint_mul (pinned host BigInts)",
               "steps": args.e2e_steps, "per_step_ms": [round(x, 2) for x in per],
               "transfer": _transfer_mode()}
        if C.cap != 2 * n64 + 8 or C.n_limbs != 2 * n64:
            e2e["warning"] = "unexpected output size"
        for p_ in (pa, pb, pc):
            p_.free()

    cpu = None
    if dist.rank == 0 and not args.no_cpu:
        try:
            cpu = cpu_baseline(args.cpu_log_limbs, lg)
            if args.cpu_full:
                full = cpu_full_size(lg)
                cpu["measured_full"] = full
                if "port_s" in full:
                    cpu["measured_full_s"] = {"port": full["port_s"], "gmp_1thread": full.get("gmp_s")}
                    cpu["extrapolation_error"] = cpu["value"] / (full["port_s"] * 1e3) - 1.0
        except Exception as ex:   # the baseline is reported, never required
            cpu = {"error": str(ex)}

    line = {
        "metric": METRIC, "value": ms, "unit": UNIT, "n_gpus": dist.world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": False, "scaling": "weak",
        "vs_baseline": None, "dtype": "u64",
        "data": "synthetic (seeded splitmix64 limbs; inputs resident in HBM)",
        "config": {"workload": "multiply 2^%d x 2^%d 32-bit limbs, NTT length 2^%d per prime, bit-exact"
                               % (lg, lg, lg + 1),
                   "primes": "q0 = 2^64-2^32+1 (uint64 residues) and p3 = 3*2^30+1 (uint32 residues); CRT "
                             "modulus 2^95.6 > largest coefficient 2^92; the reference's three 64-bit primes "
                             "are timed in three_prime_64bit" if g.prime_set() == 2 else
                             "2^64-2^b+1, b = 32, 34, 40 (uint64 residues)",
                   "operand_limbs": n, "transform_log": lg + 1, "passes": g.plan(lg + 1),
                   "l2_policy": "inputs and 24 GiB spectra >> 129 MB L2; no flush", "parallelism": "replicas"},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "traffic": traffic, "peak_source": peak_kind,
                     "kernel": "ntt_pass_kernel (%d launches per multiply)" % pass_launches,
                     "algorithmic_bytes_per_launch": pass_bytes / max(1, pass_launches)},
        "issue_roofline": issue,
        "multiply_roofline": {"bytes_model": bm, "achieved_GBps": bm / (ms * 1e-3) / 1e9,
                              "frac": bm / (ms * 1e-3) / 1e9 / peak,
                              "model": "10*k*N*8 + 8*(n_a+n_b), k=3 (2-pass four-step with fused decomposition, "
                                       "pointwise product and Garner+carry)",
                              "bytes_model_own_primes": bm_own,
                              "frac_own_primes": bm_own / (ms * 1e-3) / 1e9 / peak,
                              "model_own_primes": "the same model with this run's residue words "
                                                  "(%d bytes per coefficient over all primes)" % res_bytes},
        "three_prime_64bit": three,
        "square": square,
        "multiply_2pow20": small,
        "radix3": radix3,
        "packed_64bit_coefficients": packed,
        "negacyclic": negacyclic,
        "batched": batched,
        "serving": serving,
        "e_digits": e_leg,
        "launch_breakdown": by_kind,
        "gpu_launches": launches_per_step * args.steps,
        "device_error_flags": flags,
        "clocks": clk,
        "e2e": e2e,
        "cpu_baseline": cpu,
    }
    if dist.rank == 0:
        print(json.dumps(line), flush=True)
    for buf in (da, db, dc):
        buf.free()
    g.teardown()
    return 0 if flags == 0 else 3


def run_radix3_leg(g, cudart, synth, lg, stream, logs):
    """Products whose coefficient count fits 3 2^k but not 2^(k+1): n x n
    limbs with 2 n - 1 = 3 2^k - 1 run a transform of 3 2^k points, timed
    against n + 1 x n + 1 limbs (3 2^k + 1 coefficients), which take the
    power of two 2^(k+2): nearly the same product, a third more points."""
    out = {"sizes": [], "rule": "a product alone takes 3 2^k points from k = %s (GBNTT_RADIX3_MIN_LOG)"
                                % os.environ.get("GBNTT_RADIX3_MIN_LOG", "20")}
    flags = 0
    for k in logs:
        if k < 10 or (3 << k) + 1 > (1 << (lg + 1)):
            continue
        n3 = 3 << (k - 1)
        xa, xb = synth.operand(n3 + 1, 31), synth.operand(n3 + 1, 32)
        ra, rb = cudart.DeviceBuffer(4 * (n3 + 1)), cudart.DeviceBuffer(4 * (n3 + 1))
        rc = cudart.DeviceBuffer(8 * (n3 + 1))
        ra.upload(xa)
        rb.upload(xb)
        reps = min(200, 40 << (20 - k)) if k < 20 else max(5, 40 >> (k - 20))

        def timed(nn):
            for _ in range(2):
                g.mul_device(rc.ptr, ra.ptr, nn, rb.ptr, nn, None)
            e0, e1 = cudart.Event(), cudart.Event()
            e0.record(stream)
            for _ in range(reps):
                g.mul_device(rc.ptr, ra.ptr, nn, rb.ptr, nn, None)
            e1.record(stream)
            e1.synchronize()
            return e0.elapsed_ms(e1) / reps

        if not out["sizes"]:   # the clocks ramp on the first sizeable work of the leg
            for _ in range(30):
                g.mul_device(rc.ptr, ra.ptr, n3 + 1, rb.ptr, n3 + 1, None)
        m3, m2 = timed(n3), timed(n3 + 1)
        g.launch_log(True)
        g.mul_device(rc.ptr, ra.ptr, n3, rb.ptr, n3, None)
        cudart.stream_sync(stream)
        recs = g.launch_records(256)
        g.launch_log(False)
        flags |= g.device_errors()
        by = {}
        for kind, _, nbytes, kms in recs:
            e = by.setdefault(kind, {"launches": 0, "ms": 0.0, "bytes": 0.0})
            e["launches"] += 1
            e["ms"] += kms
            e["bytes"] += nbytes
        for e in by.values():
            e["GBps"] = e["bytes"] / (e["ms"] * 1e-3) / 1e9 if e["ms"] > 0 else None
        out["sizes"].append({"operand_limbs": n3, "points": 3 << k, "ms": m3, "pow2_operand_limbs": n3 + 1,
                             "pow2_points": 1 << (k + 2), "pow2_ms": m2, "ratio": m3 / m2, "steps": reps,
                             "radix3_launches": sum(by[x]["launches"] for x in by if x.startswith("radix3")),
                             "launch_breakdown": by,
                             "launch_breakdown_note": "one product with per-launch CUDA events (launches "
                                                      "serialised, both primes on one stream)"})
        for buf in (ra, rb, rc):
            buf.free()
    out["device_error_flags"] = flags
    return out


def run_negacyclic_leg(g, cudart, args, stream):
    """Negacyclic polynomial product mod X^N + 1 (the reference's crt_ntt
    negacyclic pipeline): N seeded 64-bit coefficients per operand, device
    resident, three 64-bit primes, signed 256-bit outputs."""
    L = args.nega_log
    n = 1 << L
    df, dgb, do = cudart.DeviceBuffer(8 * n), cudart.DeviceBuffer(8 * n), cudart.DeviceBuffer(32 * n)
    # 64-bit coefficients from two 32-bit splitmix streams each
    g.lib().gbntt_fill_operand(ctypes.c_void_p(df.ptr), 2 * n, 0x6E6100 + L, ctypes.c_void_p(stream))
    g.lib().gbntt_fill_operand(ctypes.c_void_p(dgb.ptr), 2 * n, 0x6E6200 + L, ctypes.c_void_p(stream))

    def step():
        g.negacyclic_mul_device(do.ptr, df.ptr, dgb.ptr, L, stream)
    for _ in range(max(1, args.warmup)):
        step()
    cudart.stream_sync(stream)
    e0, e1 = cudart.Event(), cudart.Event()
    steps = max(1, min(args.steps, 10))
    e0.record(stream)
    for _ in range(steps):
        step()
    e1.record(stream)
    e1.synchronize()
    ms = e0.elapsed_ms(e1) / steps
    for b in (df, dgb, do):
        b.free()
    # bytes: coefficients in (16 N), three primes x (twist write, 2-pass
    # forward per operand, pointwise + inverse, finish read) and 32 N out
    bm = 16 * n + 3 * 8 * n * (2 + 2 * 2 * 2 + 3 + 2 + 1) + 32 * n
    return {"ms": ms, "log_n": L, "coefficients": n, "primes": 3,
            "bytes_model": bm, "bytes_model_GBps": bm / (ms * 1e-3) / 1e9,
            "output": "signed 256-bit coefficients (4 uint64 words each)",
            "api": "gbntt_negacyclic_mul_u64 (device pointers)"}


def _transfer_mode():
    if os.environ.get("GBNTT_ZERO_COPY", "1") == "0":
        return "cudaMemcpyAsync through the engine's staging buffer"
    if os.environ.get("GBNTT_STAGE_INPUTS", "1") == "0":
        return ("zero copy: the first forward passes of both primes read the pinned operands and the carry "
                "kernel writes the pinned result over NVLink-C2C")
    return ("operand A read over NVLink-C2C once by its first q0 pass (which leaves a copy in HBM for p3), "
            "operand B pulled into HBM by a copy kernel on a second stream while A is transformed, product "
            "written to pinned memory by the carry kernel (zero copy)")


def main():
    args = parse()
    dist = Dist()
    try:
        if args.impl == "reference":
            return run_reference(args, dist)
        return run_gpu(args, dist)
    finally:
        dist.close()


if __name__ == "__main__":
    sys.exit(main())
