"""The header-only C++ front end (include/einsums_gb300/TensorAlgebra.hpp):
compiles with g++ against the C-ABI library (its static_asserts pin the
compile-time pattern analysis) on CPU; the binary runs the reference's
known-answer tests on the GPU."""
import os
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "tests", "cpp", "frontend_test.cpp")


def build_frontend():
    from einsums_gb300 import build
    lib = build.build()
    out = os.path.join(ROOT, "einsums_gb300", "_build", "frontend_test")
    libdir = os.path.dirname(lib)
    cmd = ["g++", "-std=c++20", "-O1", "-Wall", "-I", os.path.join(ROOT, "include"), SRC, "-L", libdir,
           "-leinsums_gb300", f"-Wl,-rpath,{libdir}", "-o", out]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-4000:]
    return out


def test_frontend_compiles():
    assert os.path.exists(build_frontend())


@pytest.mark.gpu
def test_frontend_runs_on_gpu():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    exe = build_frontend()
    r = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "all checks passed" in r.stdout
