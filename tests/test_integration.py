"""The reference-side integration: tests/integration/ref_drop_in.cpp (a
Solver_<2> calling carpio_gpu::CG) and ref_ns_drop_in.cpp (NS_explicit_GPU_,
tests/integration/ns_explicit_gpu.hpp) compile against the reference's own
headers and link against libcarpio_gpu.so where the reference sources are
present (they are not on the machine with the GPU, so there they stop at
"no CUDA device" here). binding_gpu.cpp runs the same C++ binding
(include/carpio_gpu.hpp) and the NS binding's call sequence on the GPU,
with stand-ins for the reference's matrix and vector types, against the
reference's own results."""
import os
import subprocess

import numpy as np
import pytest

from conftest import ROOT, golden, rel_l2

def reference_dir():
    """CARPIO_REFERENCE, else the location the oracle's build recipe uses"""
    ref = os.environ.get("CARPIO_REFERENCE")
    if ref:
        return ref
    r = subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "print-ref"],
                       capture_output=True, text=True)
    return r.stdout.strip()


REF = reference_dir()


@pytest.mark.skipif(not os.path.isdir(os.path.join(REF, "lib", "structure")),
                    reason="reference sources not present on this machine")
@pytest.mark.parametrize("src", ["ref_drop_in.cpp", "ref_ns_drop_in.cpp"])
def test_reference_drop_in_compiles_links_and_runs(tmp_path, src):
    shims = os.path.join(ROOT, "oracle", "ref", "shims")
    exe = str(tmp_path / "drop_in")
    py_inc = subprocess.run(["python3-config", "--includes"], capture_output=True,
                            text=True).stdout.split()
    py_ld = subprocess.run(["python3-config", "--ldflags", "--embed"],
                           capture_output=True, text=True).stdout.split()
    cmd = (["g++", "-std=c++11", "-O1", "-w", "-include",
            os.path.join(shims, "preinclude.h"), "-I" + shims,
            "-I" + os.path.join(REF, "lib"), "-I" + os.path.join(ROOT, "include"),
            "-I" + os.path.join(ROOT, "tests", "integration")]
           + py_inc + ["-o", exe,
                       os.path.join(ROOT, "tests", "integration", src),
                       os.path.join(REF, "lib", "utility", "format.cpp"),
                       "-L" + os.path.join(ROOT, "carpio_gb300"), "-lcarpio_gpu",
                       "-Wl,-rpath," + os.path.join(ROOT, "carpio_gb300")] + py_ld)
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
    r = subprocess.run([exe], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "linked" in r.stdout or "code 0" in r.stdout


def build_binding(tmp_path):
    exe = str(tmp_path / "binding_gpu")
    cmd = ["g++", "-std=c++11", "-O1", "-I" + os.path.join(ROOT, "include"), "-o", exe,
           os.path.join(ROOT, "tests", "integration", "binding_gpu.cpp"),
           "-L" + os.path.join(ROOT, "carpio_gb300"), "-lcarpio_gpu",
           "-Wl,-rpath," + os.path.join(ROOT, "carpio_gb300")]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
    return exe


def test_cpp_binding_compiles_without_the_reference(tmp_path):
    """the C++ binding needs only include/ and the library"""
    exe = build_binding(tmp_path)
    assert os.path.exists(exe)


@pytest.mark.gpu
def test_cpp_binding_solves_on_the_gpu(gpu_lib, tmp_path):
    """carpio_gpu::CG / BiCGSTAB through the C++ templates on the
    reference's MatrixMarket systems (685_bus, pde225), and the NS binding's
    calls on the 32 x 32 cavity, 20 steps, against the reference's own run"""
    exe = build_binding(tmp_path)
    for name, kinds in (("csr_bus685_cg", ("cg",)), ("csr_pde225_bicgstab", ("bicgstab",))):
        d = golden(name)
        case = tmp_path / name
        case.mkdir()
        d["rowptr"].astype(np.uint32).tofile(case / "rowptr")
        d["colind"].astype(np.uint32).tofile(case / "colind")
        d["val"].astype(np.float64).tofile(case / "val")
        d["b"].astype(np.float64).tofile(case / "b")
        for k in kinds:
            r = subprocess.run([exe, "csr", str(case), k], capture_output=True, text=True,
                               timeout=300)
            assert r.returncode == 0, r.stdout + r.stderr
            x = np.fromfile(case / ("x_" + k), dtype=np.float64)
            # both solved to 1e-13 against the reference's run at its own
            # tolerance (1e-10): agreement to the larger of the two
            assert rel_l2(x, d["x"]) <= 1e-7, (name, k, rel_l2(x, d["x"]), r.stdout)
    out = tmp_path / "ns.bin"
    r = subprocess.run([exe, "ns", str(out)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    f = np.fromfile(out, dtype=np.float64).reshape(3, 36, 36)
    d = golden("cavity_32_vanleer_20")
    for k, field in zip(("u", "v", "p"), f):
        assert rel_l2(field, d[k]) <= 1e-10, (k, rel_l2(field, d[k]))
