"""CPU: the C-ABI libraries load without a GPU and export every function that
include/*.h declares; the headers compile as C and C++."""
import ctypes
import os
import re
import shutil
import subprocess

import numpy as np
import pytest

from conftest import ROOT
from oracle import loader

INCLUDE = os.path.join(ROOT, "include")


def declared_functions():
    names = set()
    for h in ("mat.h", "matgb.h"):
        src = open(os.path.join(INCLUDE, h)).read()
        src = re.sub(r"/\*.*?\*/", " ", src, flags=re.S)
        src = re.sub(r"//[^\n]*", " ", src)
        # drop preprocessor lines (with continuations)
        src = re.sub(r"^\s*#(?:[^\n]*\\\n)*[^\n]*", " ", src, flags=re.M)
        src = re.sub(r"typedef[^;]*;", " ", src)
        for m in re.finditer(r"([A-Za-z_][\w\s\*]*?)\b([A-Za-z_]\w*)\s*\(([^;{}]*)\)\s*;",
                             src):
            names.add(m.group(2))
    names.discard("if")
    return sorted(names)


def test_headers_declare_the_hot_path():
    names = declared_functions()
    for f in ("mat_mul", "mat_rmul", "mat_gemm", "mat_syrk", "mat_syrk_t",
              "mat_gemv", "mat_gemv_t", "mat_axpy",
              "mat_plu", "mat_lu", "mat_chol", "mat_solve", "mat_solve_spd",
              "mat_solve_tril", "mat_solve_tril_unit", "mat_solve_triu",
              "mat_solve_trilt", "matgb_getrf_dev", "matgb_getrf_full_dev",
              "matgb_potrf_dev"):
        assert f in names, f


@pytest.fixture(scope="module")
def libs():
    import libmat_gb300 as mg
    out = {}
    for prec in ("f32", "f64"):
        path = mg.lib_path(prec)
        if not os.path.exists(path):
            mg_build = __import__("libmat_gb300.build", fromlist=["build"])
            mg_build.build()
        out[prec] = ctypes.CDLL(path, mode=ctypes.RTLD_LOCAL)
    return out


@pytest.mark.parametrize("prec", ["f32", "f64"])
def test_library_exports_every_declared_symbol(libs, prec):
    missing = [f for f in declared_functions() if not hasattr(libs[prec], f)]
    assert not missing, missing


@pytest.mark.parametrize("prec,size", [("f32", 4), ("f64", 8)])
def test_element_size(libs, prec, size):
    assert libs[prec].matgb_elem_size() == size


def test_host_helpers_without_gpu():
    """Construction helpers are plain host code (no device needed)."""
    import libmat_gb300 as mg
    L = mg.load("f32")
    c = L.c
    c.mat_from.restype = ctypes.POINTER(mg.MatStruct)
    c.mat_from.argtypes = [ctypes.c_size_t, ctypes.c_size_t, ctypes.c_void_p]
    c.mat_rt.restype = ctypes.POINTER(mg.MatStruct)
    c.mat_rt.argtypes = [ctypes.POINTER(mg.MatStruct)]
    c.mat_at.restype = ctypes.c_float
    c.mat_at.argtypes = [ctypes.POINTER(mg.MatStruct), ctypes.c_size_t,
                         ctypes.c_size_t]
    vals = np.array([1, 2, 3, 4, 5, 6], np.float32)  # row-major 2x3
    m = c.mat_from(2, 3, vals.ctypes.data)
    assert c.mat_at(m, 0, 2) == 3 and c.mat_at(m, 1, 0) == 4
    t = c.mat_rt(m)
    assert t.contents.rows == 3 and c.mat_at(t, 2, 1) == 6
    c.mat_free_mat(m)
    c.mat_free_mat(t)


@pytest.mark.skipif(shutil.which("gcc") is None, reason="no C compiler")
def test_headers_compile_as_c_and_cpp(tmp_path):
    src = tmp_path / "t.c"
    src.write_text('#include "matgb.h"\nint main(void){Mat m={0,0,0};(void)m;'
                   'return mat_solve_spd==0;}\n')
    for cc, flags in (("gcc", ["-std=c99"]), ("g++", ["-x", "c++"])):
        if shutil.which(cc) is None:
            continue
        r = subprocess.run([cc] + flags + ["-I", INCLUDE, "-fsyntax-only",
                                           str(src)], capture_output=True,
                           text=True)
        assert r.returncode == 0, r.stderr
    src2 = tmp_path / "t2.c"
    src2.write_text('#define MAT_DOUBLE_PRECISION\n#include "mat.h"\n'
                    'int main(void){mat_elem_t x=0;return sizeof(x)!=8;}\n')
    r = subprocess.run(["gcc", "-I", INCLUDE, "-fsyntax-only", str(src2)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr


REF_TESTS = ["test_mat_solve.c", "test_mat_chol.c", "test_mat_solve_spd.c",
             "test_mat_solve_tri.c", "test_mat_mul.c", "test_mat_plu.c"]
_REF = loader.ref_dir()
_REF_TESTS_DIR = os.path.join(_REF, "tests") if _REF else None


@pytest.mark.skipif(not (_REF_TESTS_DIR and os.path.isdir(_REF_TESTS_DIR)),
                    reason="reference source tree not present on this host")
@pytest.mark.parametrize("name", REF_TESTS)
def test_reference_unit_tests_link_against_libmatgb(libs, tmp_path, name):
    """Drop-in at the source level: the reference's own unit tests for the hot
    path (they #define MATDEF static inline + MAT_IMPLEMENTATION) compile
    against include/mat.h and link against libmatgb_f32 unchanged."""
    import libmat_gb300 as mg
    out = tmp_path / name.replace(".c", "")
    r = subprocess.run(
        ["gcc", "-std=gnu99", "-I", INCLUDE, "-I", _REF_TESTS_DIR,
         os.path.join(_REF_TESTS_DIR, name), "-o", str(out),
         os.path.join(mg.LIBDIR, "libmatgb_f32.so"), "-lm",
         "-Wl,-rpath," + mg.LIBDIR], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr


def test_report_struct_layout_matches_ctypes(tmp_path):
    """MatIROpts / MatIRReport: the ctypes mirror has the C header's size and
    field offsets (a mismatch would corrupt memory on every refinement
    call)."""
    import ctypes as C
    import libmat_gb300 as mg
    if shutil.which("gcc") is None:
        pytest.skip("no C compiler")
    lines = []
    for st in (mg.MatIROpts, mg.MatIRReport):
        name = st.__name__
        lines.append(f'printf("{name} %zu\\n", sizeof({name}));')
        for f, _ in st._fields_:
            lines.append(f'printf("{name}.{f} %zu\\n", offsetof({name}, {f}));')
    src = tmp_path / "layout.c"
    src.write_text('#include <stdio.h>\n#include <stddef.h>\n#include "matgb.h"\n'
                   "int main(void){" + "".join(lines) + "return 0;}\n")
    exe = tmp_path / "layout"
    r = subprocess.run(["gcc", "-I", INCLUDE, str(src), "-o", str(exe)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    got = dict(l.split() for l in subprocess.run(
        [str(exe)], capture_output=True, text=True, check=True).stdout.split("\n") if l)
    for st in (mg.MatIROpts, mg.MatIRReport):
        name = st.__name__
        assert int(got[name]) == C.sizeof(st), name
        for f, _ in st._fields_:
            assert int(got[f"{name}.{f}"]) == getattr(st, f).offset, (name, f)


def test_batched_schedule_file_is_read(tmp_path):
    """The batched solver's schedule table comes from the tuner's JSON file
    (read at the first batched call; no device needed): entries for this
    build override the defaults, entries for the other precision and
    malformed ones are skipped; the committed table parses."""
    import json
    import sys
    doc = {"fused": 1, "fused_ctas_per_sm": 2, "entries": [
        {"prec": "f32", "nb": 96, "kind": 1, "algo": 1, "ctas_per_sm": 3},
        {"prec": "f64", "nb": 96, "kind": 1, "algo": 0, "ctas_per_sm": 5},
        {"prec": "f32", "nb": 16, "kind": 0, "algo": 1, "ctas_per_sm": 2},
        {"nb": 32, "kind": 0}]}
    f = tmp_path / "tune.json"
    f.write_text(json.dumps(doc))
    code = (
        "import ctypes as C, sys; sys.path.insert(0, %r)\n"
        "import libmat_gb300 as mg\n"
        "L = mg.load('f32'); a, c = C.c_int(), C.c_int()\n"
        "assert L.c.matgb_batched_tune_get(96, 1, C.byref(a), C.byref(c)) == 0\n"
        "print(a.value, c.value)\n"
        "assert L.c.matgb_batched_tune_get(16, 0, C.byref(a), C.byref(c)) == 0\n"
        "print(a.value, c.value)\n"
        "print(L.c.matgb_batched_schedule(-1, -1, -1))\n"
        "print(L.c.matgb_batched_tune_source().decode())\n") % ROOT
    env = dict(os.environ, LIBMATGB_BATCHED_TUNE=str(f))
    r = subprocess.run([sys.executable, "-c", code], capture_output=True,
                       text=True, env=env)
    assert r.returncode == 0, r.stderr
    out = r.stdout.split("\n")
    assert out[0] == "1 3"   # the f32 entry for (96, SPD)
    assert out[1] == "0 0"   # blocked form refused below order 64
    assert out[2] == "1"     # fused schedule chosen by the file
    assert "tune.json (1 entries)" in out[3]
    # the committed table
    env = dict(os.environ)
    env.pop("LIBMATGB_BATCHED_TUNE", None)
    r = subprocess.run([sys.executable, "-c", code.replace(
        "assert L.c.matgb_batched_tune_get(96, 1, C.byref(a), C.byref(c)) == 0\n", "").replace(
        "assert L.c.matgb_batched_tune_get(16, 0, C.byref(a), C.byref(c)) == 0\n", "")],
        capture_output=True, text=True, env=env)
    assert r.returncode == 0, r.stderr
    # every entry of the committed file is used: the per-queue schedule and,
    # for the mixed-precision mode, the per-queue routing ("mixed_tc")
    import json
    with open(os.path.join(ROOT, "libmat_gb300", "batched_tune.json")) as fh:
        entries = json.load(fh)["entries"]
    assert f"batched_tune.json ({len(entries)} entries)" in r.stdout
