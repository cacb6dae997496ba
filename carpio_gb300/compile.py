"""Compiles libcarpio_gpu.so in place from carpio_gb300/csrc with nvcc for
sm_103a only. Translation units compile in parallel; the .so lands next to
this file (git-ignored)."""
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libcarpio_gpu.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# host code must not contract a*b+c (aarch64 gcc would) so the host-built
# stencil coefficients carry the reference's bits on every machine
COMMON = ["-O3", "-lineinfo", "-std=c++17", "--expt-relaxed-constexpr",
          "-Xcompiler", "-fPIC,-ffp-contract=off", "-Xptxas", "-v"]
# per-file extra flags: the projection operators must round like the
# reference's C++ (no FMA contraction)
EXTRA = {"ns.cu": ["--fmad=false"]}
SOURCES = ["runtime.cu", "csr.cu", "csr_noalloc.cu", "poisson.cu", "ns.cu", "batch.cu", "batch_k256.cu", "batch_k512.cu", "batch_mg.cu", "nn_conv.cu", "nn.cu", "learned.cu"]


def nvcc():
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _headers():
    out = []
    for d in (CSRC, os.path.join(HERE, "..", "include")):
        for f in os.listdir(d):
            if f.endswith((".cuh", ".hpp", ".h")):
                out.append(os.path.join(d, f))
    return out


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build(verbose=False, force=False):
    os.makedirs(BUILD, exist_ok=True)
    cc = nvcc()
    hdrs = _headers()
    objs, jobs = [], []
    for src in SOURCES:
        path = os.path.join(CSRC, src)
        obj = os.path.join(BUILD, src.replace(".cu", ".o"))
        objs.append(obj)
        if force or _stale(obj, [path] + hdrs):
            cmd = [cc] + ARCH + COMMON + EXTRA.get(src, []) + [
                "-c", path, "-o", obj]
            jobs.append((src, cmd))

    def run(job):
        src, cmd = job
        r = subprocess.run(cmd, capture_output=True, text=True)
        return src, cmd, r

    if jobs:
        with cf.ThreadPoolExecutor(max_workers=min(8, len(jobs))) as ex:
            for src, cmd, r in ex.map(run, jobs):
                if r.returncode != 0:
                    sys.stderr.write(r.stdout + r.stderr)
                    raise RuntimeError(f"nvcc failed on {src}")
                if verbose:
                    sys.stderr.write(r.stderr)
                with open(os.path.join(BUILD, src + ".ptxas.txt"), "w") as f:
                    f.write(r.stderr)
    if force or jobs or _stale(LIB, objs):
        cmd = [cc] + ARCH + ["-shared", "-o", LIB] + objs + ["-lcudart"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            sys.stderr.write(r.stdout + r.stderr)
            raise RuntimeError("link of libcarpio_gpu.so failed")
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv, force="-f" in sys.argv))
