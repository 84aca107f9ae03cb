"""GPU: the reference's own unit tests for the hot path (and the rows beside
it: det, inv, full-pivoting LU, QR), compiled unchanged against
include/mat.h, linked against libmatgb_f32 and RUN on the GPU -- the drop-in
at the source level, checked by the reference's own assertions (its test.h
harness: "N passed, 0 failed", exit status 0).

The test sources are read from the reference tree, or from the copy that
oracle/Makefile keeps in oracle/_ref/src (never committed) on a host without
the tree; the test skips when neither is present.
"""
import os
import shutil
import subprocess

import pytest

from oracle import loader

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
INCLUDE = os.path.join(ROOT, "include")
TESTS = ["test_mat_solve.c", "test_mat_chol.c", "test_mat_solve_spd.c",
         "test_mat_solve_tri.c", "test_mat_mul.c", "test_mat_plu.c",
         "test_mat_det.c", "test_mat_inv.c", "test_mat_lu.c", "test_mat_qr.c"]
_REF = loader.ref_dir()
_DIR = os.path.join(_REF, "tests") if _REF else None


@pytest.mark.skipif(not (_DIR and os.path.isdir(_DIR)) or shutil.which("gcc") is None,
                    reason="reference unit tests or a C compiler not present on this host")
@pytest.mark.parametrize("name", TESTS)
def test_reference_unit_test_passes_on_gpu(gpu, tmp_path, name):
    import libmat_gb300 as mg
    src = os.path.join(_DIR, name)
    if not os.path.exists(src):
        pytest.skip(f"{name} not in the reference tree")
    exe = tmp_path / name.replace(".c", "")
    r = subprocess.run(
        ["gcc", "-std=gnu99", "-I", INCLUDE, "-I", _DIR, src, "-o", str(exe),
         os.path.join(mg.LIBDIR, "libmatgb_f32.so"), "-lm",
         "-Wl,-rpath," + mg.LIBDIR], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    run = subprocess.run([str(exe)], capture_output=True, text=True, timeout=300)
    assert run.returncode == 0, run.stdout[-3000:] + run.stderr[-2000:]
    assert " 0 failed" in run.stdout, run.stdout[-3000:]
