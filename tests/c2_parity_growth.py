"""Growth of the GPU/reference difference over the 2000-step cavity (config C2).

The lid-driven cavity (Re 1000, van Leer, dt0 = 0.5 h, all-Neumann pressure
by CG to 1e-10 with mean removal) runs side by side on the GPU (FP64
projection, the library's public API) and in the oracle (the reference's
algorithm restated, bit for bit equal to the reference's own runs) from
rest; every EVERY steps the relative L2 differences of u, v and p (normal
cells) are printed as one JSON line. The last line compares the GPU with the
reference's own 2000-step fixture when there is one.

    python tests/c2_parity_growth.py [N] [STEPS] [EVERY]     (defaults 256 2000 100)

Test infrastructure: it needs a GPU and runs for minutes; the pytest suite
asserts the resulting bound (tests/test_gpu_ns.py::test_cavity_2000_steps).
"""
import json
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(HERE))
sys.path.insert(0, HERE)


def main():
    n = int(sys.argv[1]) if len(sys.argv) > 1 else 256
    steps = int(sys.argv[2]) if len(sys.argv) > 2 else 2000
    every = int(sys.argv[3]) if len(sys.argv) > 3 else 100
    from conftest import golden, golden_names, rel_l2
    from oracle import restate as R
    from test_gpu_ns import make_cavity
    g, ns = make_cavity(n, "VanLeer", 0.5 / n)
    og = R.Grid(n, n, 2)
    so = R.new_state(og, 0.5 / n)
    threads = os.cpu_count() or 1
    t0 = time.time()
    done = 0
    while done < steps:
        k = min(every, steps - done)
        assert ns.run(k) == 0
        code, _, _, _ = R.ns_run(og, so, k, scheme="vanleer", cg_tol=1e-10,
                                 cg_max_iter=100000, threads=threads)
        assert code == 0
        done += k
        st = ns.state()
        row = {"n": n, "step": done, "wall_s": round(time.time() - t0, 1)}
        for f in ("u", "v", "p"):
            row[f] = rel_l2(g.interior(st[f]), og.interior(so[f]))
        print(json.dumps(row), flush=True)
    name = f"cavity_{n}_vanleer_{steps}"
    if name in golden_names("cavity_"):
        d = golden(name)
        st = ns.state()
        row = {"n": n, "step": steps, "against": name}
        for f in ("u", "v", "p"):
            row[f] = rel_l2(g.interior(st[f]), d[f + "_interior"])
            row["oracle_" + f] = rel_l2(og.interior(so[f]), d[f + "_interior"])
        print(json.dumps(row), flush=True)


if __name__ == "__main__":
    main()
