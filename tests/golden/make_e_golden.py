"""Generate tests/golden/e_digits.json from the REFERENCE's own host
compute_e (ntt/app/compute_e/main.c and the arith layer, compiled by path by
oracle/build.py::build_ref_compute_e, multiplies served by GMP through
oracle/ref_e_gmp_shim.c). Run here, where the reference checkout exists:

    python tests/golden/make_e_golden.py 1000 10000 100000 1000000 10000000 100000000

Stores, per digit count D, the sha256 of the printed string "2.71828..."
(D digits after the "e = " of main.c:340-345), its first and last 40
characters and the reference's wall time.
"""
import hashlib
import json
import os
import subprocess
import sys
import time

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from oracle import build  # noqa: E402

OUT = os.path.join(os.path.dirname(os.path.abspath(__file__)), "e_digits.json")


def reference_digits(D):
    exe = build.build_ref_compute_e()
    if exe is None:
        sys.exit("reference checkout not found")
    env = dict(os.environ, NTT_MAX_LOGN="26")
    t0 = time.time()
    out = subprocess.run([exe, "-d", str(D), "-f"], capture_output=True, text=True, env=env, check=True).stdout
    dt = time.time() - t0
    line = next(x for x in out.splitlines() if x.startswith("e = "))
    return line[4:], dt


def main(ds):
    gold = json.load(open(OUT)) if os.path.exists(OUT) else {}
    for D in ds:
        s, dt = reference_digits(D)
        assert len(s) == D + 1, (len(s), D)
        gold[str(D)] = {"sha256": hashlib.sha256(s.encode()).hexdigest(), "head": s[:40], "tail": s[-40:],
                        "reference_seconds": round(dt, 2), "cores": os.cpu_count()}
        with open(OUT, "w") as f:
            json.dump(gold, f, indent=1, sort_keys=True)
        print(D, gold[str(D)], flush=True)


if __name__ == "__main__":
    main([int(x) for x in sys.argv[1:]] or [1000, 10000, 100000, 1000000])
