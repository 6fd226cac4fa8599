"""The reference's own test programs compile unchanged against the drop-in headers.

Each of the reference's tests/*.cu (the functionality test and the four speed tests:
construction, 3-d, D-sweep with the range-limited workload, speedup) includes
"../src/{BruteForce,KdTree,BallTree}.cuh" (CPU classes, kept as the reference's own code) and
"../src/{KnnTrees,BruteForceGpu,KdTreeGpu,BallTreeGpu}.cuh", and instantiates the GPU classes with
the template arguments its callers use.
Here a temporary tree puts the drop-in headers at those paths (symbolic links, nothing copied)
and nvcc builds and links the program against libcudaexactknn.so.  It needs the reference
sources, so it is skipped where they are not mounted; running the binary needs a GPU, and the
same assertions run on the GPU through tests/cpp/functionality.cu."""

import os
import subprocess
import tempfile

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
# The reference checkout (KNN_REF_DIR, as for oracle/Makefile); skipped where it is absent.
REF = os.environ.get("KNN_REF_DIR", "/root/reference")
DROPIN = os.path.join(ROOT, "include", "KnnTrees")
LIBDIR = os.path.join(ROOT, "cudaexactknn_gb300")


PROGRAMS = ["FunctionalityTests", "ConstructionSpeedTests", "Dim3SpeedTests", "DimXSpeedTests", "SpeedupSpeedTests"]


@pytest.mark.skipif(not os.path.isdir(os.path.join(REF, "tests")), reason="reference sources not mounted")
@pytest.mark.parametrize("program", PROGRAMS)
def test_reference_test_program_builds_against_dropin(program):
    with tempfile.TemporaryDirectory() as tmp:
        os.makedirs(os.path.join(tmp, "src"))
        os.makedirs(os.path.join(tmp, "tests"))
        for name in ("BruteForce.cuh", "KdTree.cuh", "BallTree.cuh"):
            os.symlink(os.path.join(REF, "src", name), os.path.join(tmp, "src", name))
        for name in ("KnnTrees.cuh", "BruteForceGpu.cuh", "KdTreeGpu.cuh", "BallTreeGpu.cuh"):
            os.symlink(os.path.join(DROPIN, name), os.path.join(tmp, "src", name))
        for name in (program + ".cu", "Tests.cuh"):
            os.symlink(os.path.join(REF, "tests", name), os.path.join(tmp, "tests", name))
        out = os.path.join(tmp, program)
        cmd = ["nvcc", "-std=c++17", "-O2", "-gencode", "arch=compute_103a,code=sm_103a",
               f"-I{os.path.join(ROOT, 'include')}", os.path.join(tmp, "tests", program + ".cu"),
               "-o", out, f"-L{LIBDIR}", "-lcudaexactknn", f"-Xlinker=-rpath,{LIBDIR}"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        assert r.returncode == 0, r.stderr[-4000:]
        assert os.path.exists(out)
