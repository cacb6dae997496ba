"""Records the reference algorithm's CG iterations per step on the benchmark's
cavity workload (1024^2, Re 1000, van Leer, FP64 CG to 1e-8 with mean
removal) by running the oracle restatement in full, step by step.

    python oracle/record_cg_iters.py [--n 1024] [--steps 14] [--threads 4]

Writes oracle/cavity_cg_iters_<n>.json, which bench.py uses to scale its
bounded CPU samples (a capped-CG step) to full steps. TEST/BENCH
INFRASTRUCTURE: the product never reads it.
"""
import argparse
import json
import os
import sys
import time

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(HERE))

from oracle import restate as R  # noqa: E402


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--n", type=int, default=1024)
    ap.add_argument("--steps", type=int, default=14)
    ap.add_argument("--threads", type=int, default=4)
    a = ap.parse_args()
    g = R.Grid(a.n, a.n, 2)
    st = R.new_state(g, 0.5 / a.n)
    rows = []
    out = os.path.join(HERE, f"cavity_cg_iters_{a.n}.json")
    for s in range(a.steps):
        t0 = time.perf_counter()
        code, sdt, sit, sres = R.ns_run(g, st, 1, scheme="vanleer", cg_tol=1e-8,
                                        cg_max_iter=200000, threads=a.threads)
        rows.append({"step": s + 1, "cg_iters": int(sit[0]), "dt": float(sdt[0]),
                     "resid": float(sres[0]), "code": int(code),
                     "sec": time.perf_counter() - t0})
        print(rows[-1], flush=True)
        with open(out, "w") as f:
            json.dump({"n": a.n, "threads": a.threads, "tol": 1e-8,
                       "workload": "lid-driven cavity from rest, Re 1000, van Leer",
                       "rows": rows}, f, indent=1)


if __name__ == "__main__":
    main()
