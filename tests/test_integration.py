"""The reference-side integration (tests/integration/ref_drop_in.cpp) compiles
against the reference's own headers and links against libcarpio_gpu.so. Runs
where the reference sources are present; the GPU solve inside it runs only
where a device is visible."""
import os
import subprocess

import pytest

from conftest import ROOT

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
def test_reference_drop_in_compiles_links_and_runs(tmp_path):
    shims = os.path.join(ROOT, "oracle", "ref", "shims")
    exe = str(tmp_path / "drop_in")
    py_inc = subprocess.run(["python3-config", "--includes"], capture_output=True,
                            text=True).stdout.split()
    py_ld = subprocess.run(["python3-config", "--ldflags", "--embed"],
                           capture_output=True, text=True).stdout.split()
    cmd = (["g++", "-std=c++11", "-O1", "-w", "-include",
            os.path.join(shims, "preinclude.h"), "-I" + shims,
            "-I" + os.path.join(REF, "lib"), "-I" + os.path.join(ROOT, "include")]
           + py_inc + ["-o", exe,
                       os.path.join(ROOT, "tests", "integration", "ref_drop_in.cpp"),
                       os.path.join(REF, "lib", "utility", "format.cpp"),
                       "-L" + os.path.join(ROOT, "carpio_gb300"), "-lcarpio_gpu",
                       "-Wl,-rpath," + os.path.join(ROOT, "carpio_gb300")] + py_ld)
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
    r = subprocess.run([exe], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "linked" in r.stdout or "code 0" in r.stdout
