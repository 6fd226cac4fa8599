"""C-ABI checks that need no GPU: the library loads, exports what the header declares, and
rejects bad arguments before touching the device."""

import ctypes
import os
import subprocess

import pytest

from cudaexactknn_gb300 import _lib

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_library_loads_and_exports_every_declared_symbol():
    lib = _lib.load()
    declared = _lib.header_symbols()
    assert len(declared) >= 12
    for name in declared:
        assert hasattr(lib, name), name
    out = subprocess.run(["nm", "-D", "--defined-only", _lib.LIB_PATH], capture_output=True, text=True,
                         check=True).stdout
    exported = {line.split()[-1] for line in out.splitlines() if " T " in line}
    assert set(declared) <= exported


def test_library_is_built_for_sm_103a():
    out = subprocess.run(["cuobjdump", "--list-elf", _lib.LIB_PATH], capture_output=True, text=True)
    if out.returncode != 0:
        pytest.skip("cuobjdump unavailable")
    assert "sm_103a" in out.stdout


def test_status_strings_and_version():
    lib = _lib.load()
    assert lib.knn_status_string(0) == b"ok"
    assert lib.knn_status_string(_lib.ERR_INVALID_ARGUMENT) == b"invalid argument"
    assert lib.knn_version() >= 10000


@pytest.mark.parametrize("dims,expect", [(0, _lib.ERR_INVALID_ARGUMENT), (129, _lib.ERR_UNSUPPORTED)])
def test_create_rejects_bad_dims_without_a_device(dims, expect):
    lib = _lib.load()
    h = ctypes.c_void_p()
    st = lib.knn_bf_create(None, 10, dims, None, ctypes.byref(h))
    assert st == expect
    assert not h
    assert lib.knn_last_error()


def test_create_rejects_null_points_and_bad_aux_dims():
    lib = _lib.load()
    h = ctypes.c_void_p()
    assert lib.knn_kd_create(None, 10, 3, 3, 0, 256, None, ctypes.byref(h)) == _lib.ERR_INVALID_ARGUMENT
    assert lib.knn_kd_create(ctypes.c_void_p(16), 10, 3, 4, 0, 256, None, ctypes.byref(h)) == _lib.ERR_INVALID_ARGUMENT
    assert lib.knn_kd_create(ctypes.c_void_p(16), 10, 3, 0, 0, 256, None, ctypes.byref(h)) == _lib.ERR_INVALID_ARGUMENT
    assert lib.knn_ball_create(None, 10, 3, 1, 256, None, None) == _lib.ERR_INVALID_ARGUMENT


def test_query_rejects_null_index_and_bad_k():
    lib = _lib.load()
    o = _lib.opts()
    assert lib.knn_query(None, None, 1, 1.0, 4, None, None, ctypes.byref(o), None) == _lib.ERR_INVALID_ARGUMENT


def test_cpp_shim_headers_compile():
    """The C++ KnnTrees drop-in headers compile (host code, no GPU needed)."""
    src = os.path.join(ROOT, "tests", "cpp", "shim_compile_check.cu")
    if not os.path.exists(src):
        pytest.skip("shim check source missing")
    out = os.path.join(ROOT, "cudaexactknn_gb300", "_build", "shim_compile_check.o")
    os.makedirs(os.path.dirname(out), exist_ok=True)
    r = subprocess.run(["nvcc", "-std=c++17", "-gencode", "arch=compute_103a,code=sm_103a",
                        f"-I{os.path.join(ROOT, 'include')}", "-c", src, "-o", out],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]


def _blob(structure=1, n=1000, dims=3, aux=3, skips=0, has_model=0, model_k=0, sizes=(0, 0, 0, 0, 0),
          payload=b"", magic=b"CEKNNIX1", version=1, checksum=None):
    import struct

    def fnv(data):
        h = 0xcbf29ce484222325
        for b in data:
            h ^= b
            h = (h * 0x100000001b3) & 0xFFFFFFFFFFFFFFFF
        return h
    head = struct.pack("<8sI5I2I5QQ", magic, version, structure, n, dims, aux, skips, has_model, model_k, *sizes,
                       fnv(payload) if checksum is None else checksum)
    assert len(head) == 88
    return head + payload


@pytest.mark.parametrize("case", ["short", "magic", "version", "sizes", "total", "checksum", "skips", "aux", "model",
                                  "n"])
def test_deserialize_rejects_malformed_blobs_without_a_device(case):
    """knn_index_deserialize validates the header, the array sizes the shape implies, the total
    size and the checksum before it touches the device (a kd tree of n=1000, dims 3, skips 0:
    1023 splits, 1024 leaf slots of 4 floats)."""
    lib = _lib.load()
    good = dict(structure=_lib.KD_TREE, n=1000, dims=3, aux=3, skips=0, sizes=(0, 4 * 1023, 4 * 1024 * 4, 0, 0))
    payload = bytes(4 * 1023 + 16 * 1024)
    kw = dict(good, payload=payload)
    if case == "short":
        blob = b"CEKNNIX1"
    elif case == "magic":
        blob = _blob(**dict(kw, magic=b"NOTANIDX"))
    elif case == "version":
        blob = _blob(**dict(kw, version=2))
    elif case == "sizes":
        blob = _blob(**dict(kw, sizes=(0, 4 * 1023, 4 * 1024 * 4 - 16, 0, 16)))
    elif case == "total":
        blob = _blob(**kw)[:-4]
    elif case == "checksum":
        blob = bytearray(_blob(**kw))
        blob[100] ^= 1
        blob = bytes(blob)
    elif case == "skips":
        blob = _blob(**dict(kw, skips=12))
    elif case == "aux":
        blob = _blob(**dict(kw, aux=4))
    elif case == "model":
        blob = _blob(**dict(kw, has_model=1, model_k=16))
    else:
        # n beyond construction's limit (2^31 - 1), sizes as a kd tree of 2^32 leaves would have.
        blob = _blob(**dict(kw, n=0xFFFFFFFF, sizes=(0, 4 * (2 ** 32 - 1), 16 * 2 ** 32, 0, 0)))
    h = ctypes.c_void_p()
    buf = ctypes.create_string_buffer(blob, len(blob))
    assert lib.knn_index_deserialize(buf, len(blob), None, ctypes.byref(h)) == _lib.ERR_INVALID_ARGUMENT
    assert not h.value
    assert b"serialised index" in lib.knn_last_error()
    if case == "n":
        assert b"2^31" in lib.knn_last_error()
    # A missing blob is refused too, and the handle is cleared.
    h = ctypes.c_void_p(0x1234)
    assert lib.knn_index_deserialize(None, len(blob), None, ctypes.byref(h)) == _lib.ERR_INVALID_ARGUMENT
    assert not h.value


def _header_prototypes():
    import re
    text = open(_lib.HEADER).read()
    text = re.sub(r"/\*.*?\*/", " ", text, flags=re.S)
    protos = {}
    for name, params in re.findall(r"KNN_API\s+[\w\s\*]+?\b(knn_\w+)\s*\(([^)]*)\)", text, flags=re.S):
        params = params.strip()
        protos[name] = 0 if params in ("", "void") else len(params.split(","))
    return protos


def test_ctypes_signatures_match_the_header():
    """Every declared function has a ctypes signature with the header's parameter count, so a
    Python caller can never pass a misaligned argument list."""
    protos = _header_prototypes()
    assert set(protos) == set(_lib.header_symbols())
    assert set(protos) == set(_lib._SIGNATURES), set(protos) ^ set(_lib._SIGNATURES)
    for name, count in protos.items():
        assert len(_lib._SIGNATURES[name]) == count, name


def test_query_flags_match_the_header():
    """Every KNN_QF_* flag of the header has the same value in the Python mirror (QF_*), and the
    flags are distinct bits."""
    import re
    text = open(os.path.join(ROOT, "include", "cudaexactknn.h")).read()
    flags = {m.group(1): int(m.group(2), 0) for m in re.finditer(r"#define KNN_(QF_\w+)\s+(0x[0-9a-fA-F]+|\d+)u", text)}
    assert len(flags) >= 8, flags
    for name, value in flags.items():
        assert getattr(_lib, name) == value, name
    values = list(flags.values())
    assert all(v & (v - 1) == 0 for v in values) and len(set(values)) == len(values)


def test_ctypes_structs_match_the_c_layout(tmp_path):
    """The Python mirrors of the header's structs have the C compiler's size and field offsets."""
    structs = {"knn_query_opts": _lib.QueryOpts, "knn_query_counters": _lib.QueryCounters,
               "knn_index_info": _lib.IndexInfo, "knn_train_opts": _lib.TrainOpts,
               "knn_train_report": _lib.TrainReport, "knn_batch_item": _lib.BatchItem}
    lines = ['#include <stdio.h>', '#include <stddef.h>', '#include "cudaexactknn.h"', "int main(void) {"]
    for cname, py in structs.items():
        lines.append(f'printf("{cname} size %zu\\n", sizeof({cname}));')
        for field, _ in py._fields_:
            lines.append(f'printf("{cname} {field} %zu\\n", offsetof({cname}, {field}));')
    lines += ["return 0;", "}"]
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines))
    exe = tmp_path / "layout"
    subprocess.run(["gcc", "-std=c11", f"-I{os.path.join(ROOT, 'include')}", str(src), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout
    got = {tuple(line.split()[:2]): int(line.split()[2]) for line in out.splitlines()}
    for cname, py in structs.items():
        assert got[(cname, "size")] == ctypes.sizeof(py), cname
        for field, _ in py._fields_:
            assert got[(cname, field)] == getattr(py, field).offset, (cname, field)


def _cuda_device_usable():
    import torch
    return torch.cuda.is_available()


def test_entry_points_report_a_failing_cuda_runtime():
    """Where the CUDA runtime fails (here: no device), every entry point that needs it returns
    KNN_ERR_CUDA with the runtime's message and leaves no handle; nothing throws or crashes, and
    the stand-in device pointer is never dereferenced."""
    if _cuda_device_usable():
        pytest.skip("a CUDA device is present")
    lib = _lib.load()
    fake = ctypes.c_void_p(0x1000)
    calls = {
        "knn_bf_create": lambda h: lib.knn_bf_create(fake, 100, 3, None, ctypes.byref(h)),
        "knn_kd_create": lambda h: lib.knn_kd_create(fake, 100, 3, 3, 0, 256, None, ctypes.byref(h)),
        "knn_ball_create": lambda h: lib.knn_ball_create(fake, 100, 3, 1, 256, None, ctypes.byref(h)),
        "knn_bf_query_noalloc": lambda h: lib.knn_bf_query_noalloc(fake, 100, 3, fake, 10, 1.0, 4, fake, fake, None),
        "knn_tc_selftest": lambda h: lib.knn_tc_selftest(16, ctypes.byref(ctypes.c_float()),
                                                        ctypes.byref(ctypes.c_uint32())),
    }
    for name, call in calls.items():
        h = ctypes.c_void_p(0x1234)
        assert call(h) == _lib.ERR_CUDA, name
        assert lib.knn_last_error(), name
        if name.endswith("_create"):
            assert not h.value, name


def test_dropin_classes_throw_cuda_exception_on_runtime_failure(tmp_path):
    """The C++ drop-in maps a failing status to KnnTrees::CudaException, as the reference's
    classes throw it (src/KnnTrees.cuh:20-23)."""
    if _cuda_device_usable():
        pytest.skip("a CUDA device is present")
    exe = tmp_path / "no_device_errors"
    libdir = os.path.dirname(_lib.LIB_PATH)
    r = subprocess.run(["nvcc", "-std=c++17", "-gencode", "arch=compute_103a,code=sm_103a",
                        f"-I{os.path.join(ROOT, 'include')}", os.path.join(ROOT, "tests", "cpp", "no_device_errors.cu"),
                        "-o", str(exe), f"-L{libdir}", "-lcudaexactknn", f"-Xlinker=-rpath,{libdir}"],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
    out = subprocess.run([str(exe)], capture_output=True, text=True, timeout=60)
    assert out.returncode == 0, out.stdout + out.stderr
    lines = out.stdout.splitlines()
    assert [s.split(" ")[0] for s in lines] == ["BruteForceGpu", "KdTreeGpu", "BallTreeGpu"]
    assert all(" threw: " in s for s in lines)


def test_empty_batch_needs_no_device():
    """A batch with no items plans, runs, reports and frees without touching the device."""
    lib = _lib.load()
    b = ctypes.c_void_p()
    assert lib.knn_batch_create(None, 0, 0, None, ctypes.byref(b)) == _lib.OK and b.value
    classes, kernels = ctypes.c_uint32(7), ctypes.c_uint32(7)
    assert lib.knn_batch_info(b, ctypes.byref(classes), ctypes.byref(kernels)) == _lib.OK
    assert (classes.value, kernels.value) == (0, 0)
    assert lib.knn_batch_run(b, None) == _lib.OK
    assert lib.knn_batch_destroy(b) == _lib.OK
    assert lib.knn_batch_create(None, 2, 0, None, ctypes.byref(b)) == _lib.ERR_INVALID_ARGUMENT
    assert not b.value


def test_library_is_not_older_than_its_sources():
    """The tests run the library as built: a source edited after the last build (or a build that
    failed and left the previous library in place) would make them test stale code."""
    from cudaexactknn_gb300 import build
    assert os.path.getmtime(_lib.LIB_PATH) >= build._deps_mtime(), "rebuild: python -c 'import __graft_entry__ as g; g.build()'"
