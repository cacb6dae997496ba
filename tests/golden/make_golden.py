"""Regenerates the golden fixtures in this directory by running the
reference's own code (oracle/_ref/ref_harness, compiled from the reference's
headers by `make -C oracle ref`).

    python tests/golden/make_golden.py --ref /path/to/reference [--long]
        [--only NAME_PREFIX]

Each fixture is a compressed .npz of the harness's inputs and outputs.
Residual histories longer than 64 entries keep their first and last 32
entries plus the full length. --long also runs the 128^2 and 256^2 cavity
(2000 steps each; the 256^2 run takes about 45 minutes on one core) or picks
up an earlier run of them from --long-dir.
"""
import argparse
import os
import shutil
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
HARNESS = os.path.join(ROOT, "oracle", "_ref", "ref_harness")


def load_dir(d):
    out = {}
    with open(os.path.join(d, "meta.txt")) as f:
        for line in f:
            p = line.split()
            if not p:
                continue
            if p[0] == "scalar":
                out[p[1]] = np.float64(float(p[2]))
            else:
                dt = {"f64": np.float64, "u32": np.uint32}[p[2]]
                shape = tuple(int(s) for s in p[3:])
                out[p[1]] = np.fromfile(os.path.join(d, p[1] + ".bin"),
                                        dtype=dt).reshape(shape)
    return out


def trim_hist(d, key="lresid"):
    if key in d:
        h = d[key]
        d[key + "_len"] = np.int64(h.size)
        if h.size > 64:
            d[key + "_head"] = h[:32].copy()
            d[key + "_tail"] = h[-32:].copy()
            del d[key]
    return d


def run(args, ref):
    d = _run(args, ref)
    # the harness arguments, minus host paths, for the tests to rebuild inputs
    d["case_args"] = np.array([os.path.basename(str(x)) for x in args])
    return d


def _run(args, ref):
    tmp = tempfile.mkdtemp(prefix="golden_")
    out = os.path.join(tmp, "o")
    cmd = [HARNESS] + [str(a) for a in args] + [out]
    env = dict(os.environ)
    if args and args[0] == "kim":
        # NS_kim_ builds plot objects through lib/io/plotly.h; the stand-in
        # package lets it import `plotly` (not installed here)
        env["PYTHONPATH"] = os.path.join(ROOT, "oracle", "ref", "pystub")
    r = subprocess.run(cmd, capture_output=True, text=True, env=env)
    try:
        if not os.path.exists(os.path.join(out, "meta.txt")) or \
                "failure" in r.stdout + r.stderr:
            return {"aborted": np.bool_(True),
                    "message": np.array((r.stdout + r.stderr).strip()),
                    "exit_code": np.int64(r.returncode)}
        if r.returncode != 0:
            raise RuntimeError(" ".join(cmd) + "\n" + r.stderr)
        d = load_dir(out)
        dump = os.path.join(out, "dump.txt")
        if os.path.exists(dump):
            # Output_Scalar's text file, byte for byte
            with open(dump, "rb") as f:
                d["dump_text"] = np.frombuffer(f.read(), dtype=np.uint8).copy()
        return d
    finally:
        shutil.rmtree(tmp, ignore_errors=True)


def save(name, d):
    path = os.path.join(HERE, name + ".npz")
    np.savez_compressed(path, **d)
    print(f"{name}: {os.path.getsize(path) // 1024} KiB")


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", required=True, help="the reference checkout")
    ap.add_argument("--long", action="store_true")
    ap.add_argument("--long-dir", default=None)
    ap.add_argument("--only-long", action="store_true",
                    help="write only the 2000-step cavity fixtures")
    ap.add_argument("--only", default="",
                    help="write only the fixtures whose name starts with this")
    a = ap.parse_args()

    def want(name):
        return name.startswith(a.only)
    subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "ref",
                    f"REF={a.ref}"], check=True)
    if a.only_long:
        a.long = True
    mtx = os.path.join(a.ref, "test", "input_files")
    csr_cases = [] if a.only_long else [
        ("csr_bus685_cg", ["685_bus.mtx", "ones", "zeros", "cg", 10000, 1e-10]),
        ("csr_bus685_jacobi_class",
         ["685_bus.mtx", "ones", "ones", "jacobi_class", 100000, 1e-6]),
        ("csr_bus685_dia_bicgstab",
         ["685_bus.mtx", "ones", "zeros", "dia_bicgstab", 10000, 1e-10]),
        ("csr_pde225_bicgstab", ["pde225.mtx", "ones", "zeros", "bicgstab", 1000, 1e-10]),
        ("csr_pde225_dia_bicgstab",
         ["pde225.mtx", "ones", "zeros", "dia_bicgstab", 1000, 1e-10]),
        ("csr_pde225_jacobi", ["pde225.mtx", "ones", "zeros", "jacobi", 5000, 1e-8]),
        ("csr_e05r0100_dia_bicgstab",
         ["e05r0100.mtx", "e05r0100_rhs1.mtx", "zeros", "dia_bicgstab", 1000, 1e-8]),
        ("csr_bus685_ic_cg", ["685_bus.mtx", "ones", "zeros", "ic_cg", 10000, 1e-10]),
        ("csr_bus685_ic_cgs", ["685_bus.mtx", "ones", "zeros", "ic_cgs", 10000, 1e-10]),
        ("csr_pde225_ic_cgs", ["pde225.mtx", "ones", "zeros", "ic_cgs", 1000, 1e-10]),
    ]
    for name, c in csr_cases:
        if not want(name):
            continue
        args = ["csr", os.path.join(mtx, c[0])]
        args.append(c[1] if c[1] == "ones" else os.path.join(mtx, c[1]))
        args += c[2:]
        save(name, trim_hist(run(args, a.ref)))
    poisson_cases = [] if a.only_long else [
        ("poisson_c1_64_cg", ["c1", 64, "cg", 1000, 1e-10, 0]),
        ("poisson_c1_64_jacobi", ["c1", 64, "jacobi", 100000, 1e-10, 0]),
        ("poisson_c1_64_dia_bicgstab", ["c1", 64, "dia_bicgstab", 1000, 1e-10, 0]),
        ("poisson_c1_64_bicgstab", ["c1", 64, "bicgstab", 1000, 1e-10, 0]),
        ("poisson_c1_128_cg", ["c1", 128, "cg", 1000, 1e-10, 0]),
        ("poisson_neumann_32_cg", ["neumann", 32, "cg", 5000, 1e-10, 7]),
        ("poisson_neumann_48_cg", ["neumann", 48, "cg", 5000, 1e-12, 11]),
        ("poisson_mixed_24_cg", ["mixed", 24, "cg", 5000, 1e-10, 0]),
        ("poisson_mixed_24_dia_bicgstab", ["mixed", 24, "dia_bicgstab", 5000, 1e-10, 0]),
        ("poisson_mixed_24_bicgstab", ["mixed", 24, "bicgstab", 5000, 1e-10, 0]),
        ("poisson_mixed_16_jacobi", ["mixed", 16, "jacobi", 20000, 1e-8, 0]),
        ("poisson_mixed_24_cg_stretch", ["mixed", 24, "cg", 5000, 1e-10, 0, "stretch"]),
        ("poisson_vbeta_24_bicgstab", ["vbeta", 24, "bicgstab", 20000, 1e-10, 0]),
        ("poisson_c1_48_ic_cg", ["c1", 48, "ic_cg", 1000, 1e-10, 0]),
        ("poisson_mixed_24_ic_cgs", ["mixed", 24, "ic_cgs", 1000, 1e-10, 0]),
        ("poisson_vbeta_20_jacobi", ["vbeta", 20, "jacobi", 20000, 1e-10, 0, "stretch"]),
        ("poisson_neumann_32_cg_stretch", ["neumann", 32, "cg", 5000, 1e-10, 7, "stretch"]),
    ]
    csr_kept = {"poisson_c1_64_cg", "poisson_neumann_32_cg", "poisson_mixed_24_cg"}
    for name, c in poisson_cases:
        if not want(name):
            continue
        d = trim_hist(run(["poisson"] + c, a.ref))
        if name not in csr_kept:
            for k in ("rowptr", "colind", "val"):
                d.pop(k, None)
        save(name, d)
    # cavity: n steps scheme tol max_iter dt0 Re dump_every
    cav = [] if a.only_long else [
        ("cavity_32_vanleer_20", [32, 20, "VanLeer", 1e-10, 100000, 0.015625, 1000, 0]),
        ("cavity_16_superbee_10", [16, 10, "superbee", 1e-10, 100000, 0.03125, 1000, 0]),
        ("cavity_16_minmod_10", [16, 10, "minmod", 1e-10, 100000, 0.03125, 1000, 0]),
        ("cavity_16_upwind1_10", [16, 10, "upwind1", 1e-10, 100000, 0.03125, 1000, 0]),
        ("cavity_20_quick_8", [20, 8, "QUICK", 1e-10, 100000, 0.025, 100, 0]),
        ("cavity_64_vanleer_200", [64, 200, "VanLeer", 1e-10, 100000, 0.0078125, 1000, 0]),
        ("cavity_24_vanleer_10_stretch", [24, 10, "VanLeer", 1e-10, 100000, 0.01, 1000, 0,
                                          "stretch"]),
        # the shipped projection solver (Solver_IC_CGS_: no mean removal):
        # converges at 64^2; at 256^2 it stops at the example's max_iter 100
        # far from tol, and with 1000 iterations it diverges
        ("cavity_24_vanleer_10_mu", [24, 10, "VanLeer", 1e-10, 100000, 0.01, 1000, 0,
                                     "mu=field"]),
        ("cavity_64_vanleer_3_ic_cgs", [64, 3, "VanLeer", 1e-10, 1000, 0.0078125, 1000, 0,
                                        "proj=ic_cgs_nomean"]),
        ("cavity_256_vanleer_1_ic_cgs_fail", [256, 1, "VanLeer", 1e-6, 100, 0.001953125,
                                              1000, 0, "proj=ic_cgs_nomean"]),
        ("cavity_256_vanleer_1_ic_cgs_diverge", [256, 1, "VanLeer", 1e-6, 1000,
                                                 0.001953125, 1000, 0, "proj=ic_cgs_nomean"]),
    ]
    for name, c in cav:
        if not want(name):
            continue
        d = run(["cavity"] + c, a.ref)
        if not name.startswith("cavity_32"):
            d = {k: v for k, v in d.items() if not k.startswith("s1_")}
        if name.startswith("cavity_256"):
            # the solver's outcome only: the GPU test steps the cavity itself
            d = {k: d[k] for k in ("cg_ret", "cg_iters", "cg_resid", "dt", "case_args")}
        save(name, d)
    # NS_kim_: n steps scheme tol max_iter dt0 Re
    kim = [] if a.only_long else [
        ("kim_24_vanleer_10", [24, 10, "VanLeer", 1e-10, 100000, 0.005, 100]),
        ("kim_16_superbee_6", [16, 6, "superbee", 1e-10, 100000, 0.01, 400]),
    ]
    for name, c in kim:
        if not want(name):
            continue
        save(name, run(["kim"] + c, a.ref))
    # stand-alone Advection_: n steps scheme dt case [stretch]; the first is
    # the shipped 2-D TVD example (50^2, dt 0.002, set_time(1000) = 1001 steps)
    adv = [] if a.only_long else [
        ("advect_50_vanleer_band", [50, 1001, "VanLeer", 0.002, "band"]),
        ("advect_40_quick_rotate", [40, 60, "QUICK", 0.004, "rotate"]),
        ("advect_40_superbee_rotate", [40, 60, "superbee", 0.004, "rotate"]),
        ("advect_30_upwind1_band", [30, 50, "upwind1", 0.003, "band"]),
        ("advect_30_center4_band", [30, 50, "center4", 0.001, "band"]),
        ("advect_24_center_rotate", [24, 40, "center", 0.002, "rotate"]),
        ("advect_24_upwind2_band", [24, 40, "upwind2", 0.002, "band"]),
        ("advect_32_cui_rotate_stretch", [32, 40, "CUI", 0.003, "rotate", "stretch"]),
        ("advect_32_wahyd_band_stretch", [32, 40, "WAHYD", 0.002, "band", "stretch"]),
    ]
    for name, c in adv:
        if not want(name):
            continue
        d = run(["advect"] + c, a.ref)
        d.update(n=np.int64(c[0]), steps=np.int64(c[1]), scheme=np.array(c[2]),
                 dt=np.float64(c[3]), case=np.array(c[4]),
                 stretch=np.float64(1.0 if len(c) > 5 else 0.0))
        save(name, d)
    ops = [] if a.only_long else [("ops_13_gl2", [13, 5, 2]), ("ops_9_gl1", [9, 3, 1]),
                                  ("ops_12_gl2_stretch", [12, 7, 2, "stretch"])]
    for name, c in ops:
        if not want(name):
            continue
        save(name, run(["ops"] + c, a.ref))
    if a.long:
        for n, dt0 in [(128, 0.5 / 128), (256, 0.5 / 256)]:
            src = os.path.join(a.long_dir, f"ref_c2_{n}") if a.long_dir else None
            if src and os.path.exists(os.path.join(src, "meta.txt")):
                d = load_dir(src)
            else:
                d = run(["cavity", n, 2000, "VanLeer", 1e-10, 100000, dt0, 1000, 0], a.ref)
            g = 2
            keep = {k: d[k] for k in ("dt", "cg_iters", "cg_resid", "Re", "dt0", "tol")}
            for k in ("u", "v", "p"):
                keep[k + "_interior"] = d[k][g:-g, g:-g].copy()
            keep["cg_ms"] = d["cg_ms"]
            save(f"cavity_{n}_vanleer_2000", keep)


if __name__ == "__main__":
    sys.exit(main())
