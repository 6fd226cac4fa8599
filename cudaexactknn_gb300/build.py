"""Build recipe of the engine's shared library (libcudaexactknn.so), sm_103a only.

Every translation unit is compiled by nvcc in parallel; the query-kernel files are compiled
once per padded dimension count (-DKNN_DP=...).  Objects go to cudaexactknn_gb300/_build/,
the library to cudaexactknn_gb300/libcudaexactknn.so.  Up-to-date objects are reused.
"""

from __future__ import annotations

import concurrent.futures as cf
import glob
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
BUILD = os.path.join(PKG, "_build")
LIB = os.path.join(PKG, "libcudaexactknn.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
PADDED_DIMS = [1, 2, 3, 4, 8, 16, 32, 64, 128]
PER_DIM = ["bf_kernels.cu", "kd_kernels.cu", "ball_kernels.cu"]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _flags() -> list[str]:
    return ["-std=c++17", "-O3", "-lineinfo", *ARCH, "-Xcompiler", "-fPIC", "-Xcompiler", "-fvisibility=hidden",
            f"-I{os.path.join(ROOT, 'include')}", "--expt-relaxed-constexpr"]


def _units():
    units = []
    for src in sorted(glob.glob(os.path.join(CSRC, "*.cu"))):
        name = os.path.basename(src)
        if name in PER_DIM:
            for dp in PADDED_DIMS:
                units.append((src, os.path.join(BUILD, f"{name[:-3]}_d{dp}.o"), [f"-DKNN_DP={dp}"]))
        else:
            units.append((src, os.path.join(BUILD, name[:-3] + ".o"), []))
    return units


def _deps_mtime() -> float:
    files = glob.glob(os.path.join(CSRC, "*")) + glob.glob(os.path.join(ROOT, "include", "*.h"))
    return max(os.path.getmtime(f) for f in files)


def build(jobs: int | None = None, verbose: bool = False) -> str:
    os.makedirs(BUILD, exist_ok=True)
    newest = _deps_mtime()
    todo = [(s, o, x) for (s, o, x) in _units() if not os.path.exists(o) or os.path.getmtime(o) < newest]
    cc = nvcc()

    def compile_one(unit):
        src, obj, extra = unit
        cmd = [cc, *_flags(), *extra, "-c", src, "-o", obj + ".tmp"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed for {os.path.basename(src)} {extra}:\n{r.stderr[-4000:]}")
        os.replace(obj + ".tmp", obj)
        return obj

    jobs = jobs or max(1, min(len(todo), os.cpu_count() or 4))
    if todo:
        with cf.ThreadPoolExecutor(jobs) as ex:
            for obj in ex.map(compile_one, todo):
                if verbose:
                    print("compiled", os.path.basename(obj), flush=True)
    objs = [o for (_, o, _) in _units()]
    if todo or not os.path.exists(LIB) or os.path.getmtime(LIB) < max(os.path.getmtime(o) for o in objs):
        cmd = [cc, *ARCH, "-shared", "-o", LIB + ".tmp", *objs, "-lcudart_static", "-lpthread", "-ldl", "-lrt"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("link failed:\n" + r.stderr[-4000:])
        os.replace(LIB + ".tmp", LIB)
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv))
