"""Builds tests/cpp/functionality.cu against the drop-in headers and runs it on the GPU."""

import os
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
LIBDIR = os.path.join(ROOT, "cudaexactknn_gb300")


def _build():
    out = os.path.join(ROOT, "cudaexactknn_gb300", "_build", "functionality_test")
    os.makedirs(os.path.dirname(out), exist_ok=True)
    cmd = ["nvcc", "-std=c++17", "-O2", "-gencode", "arch=compute_103a,code=sm_103a",
           f"-I{os.path.join(ROOT, 'include')}", os.path.join(ROOT, "tests", "cpp", "functionality.cu"),
           "-o", out, f"-L{LIBDIR}", "-lcudaexactknn", f"-Xlinker=-rpath,{LIBDIR}"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-4000:]
    return out


def test_cpp_functionality_builds():
    _build()


@pytest.mark.gpu
def test_cpp_functionality_runs():
    exe = _build()
    r = subprocess.run([exe], capture_output=True, text=True, timeout=600)
    print(r.stdout)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "All tests passed" in r.stdout
