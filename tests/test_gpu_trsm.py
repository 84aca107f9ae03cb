"""Triangular solves with many right-hand sides through matgb_trsm_dev.

matgb_trsm_dev generalises mat_solve_tril / _tril_unit / _triu / _trilt
(mat.h:4580-4803) to a block of right-hand sides, in place.  These cases
drive every uplo / trans / diag variant over ragged orders (one row, one
short of a 64-row tile, exactly one tile, one past it, many tiles) and over
right-hand-side counts on both sides of the 64-column chunk the solver
launches per pass.  The triangle the solve must not read (and the diagonal
of a unit solve) holds NaN, so any read of it shows in the result, as the
reference's substitution loops never touch those entries.  Leading
dimensions larger than the order check the strided addressing.
"""
import itertools

import numpy as np
import pytest
import scipy.linalg

from libmat_gb300 import rng

pytestmark = pytest.mark.gpu

TOL = {"f32": 2e-4, "f64": 1e-11}
VARIANTS = list(itertools.product("LU", "NT", "NU"))


def tri_case(seed, n, uplo, diag, ldt, dt):
    """Column-major ldt x n buffer holding a well-conditioned triangle of
    order n, NaN elsewhere; plus the clean n x n triangle for the check."""
    off = rng.uniform(seed, (n, n), -1, 1, np.float64) * (2.0 / max(n, 1))
    d = rng.uniform(seed + 1, (n,), 1, 2, np.float64)
    d *= np.where(rng.uniform(seed + 2, (n,), -1, 1, np.float64) < 0, -1, 1)
    tri = np.tril(off, -1) if uplo == "L" else np.triu(off, 1)
    clean = tri + np.diag(np.ones(n) if diag == "U" else d)
    clean = clean.astype(dt)
    buf = np.full((ldt, n), np.nan, dt, order="F")
    mask = np.tril(np.ones((n, n), bool), -1 if diag == "U" else 0)
    if uplo == "U":
        mask = mask.T
    view = buf[:n, :]
    view[mask] = clean[mask]
    return buf, clean


def run_trsm(L, uplo, trans, diag, buf, n, B, ldb):
    nrhs = B.shape[1]
    Bbuf = np.zeros((ldb, nrhs), B.dtype, order="F")
    Bbuf[:n, :] = B
    dT = L.dalloc(max(buf.nbytes, 8))
    dB = L.dalloc(max(Bbuf.nbytes, 8))
    try:
        L.h2d(dT, buf)
        L.h2d(dB, Bbuf)
        rc = L.c.matgb_trsm_dev(uplo.encode(), trans.encode(), diag.encode(),
                                n, nrhs, dT, buf.shape[0], dB, ldb)
        L.check(rc, "trsm_dev")
        out = np.empty_like(Bbuf)
        L.d2h(out, dB)
    finally:
        L.dfree(dT)
        L.dfree(dB)
    # rows past n belong to the caller and must come back untouched
    assert not np.any(out[n:, :]), "trsm wrote past row n"
    return out[:n, :]


@pytest.mark.parametrize("prec", ["f32", "f64"])
@pytest.mark.parametrize("n", [1, 63, 64, 65, 200, 1000])
@pytest.mark.parametrize("nrhs", [1, 2, 64, 65, 130])
def test_trsm_variants_vs_scipy(gpu, prec, n, nrhs):
    L = gpu[prec]
    dt = L.dtype
    pad = (n * 7 + nrhs) % 5  # ragged leading dimensions on some cases
    ldt, ldb = n + pad, n + (pad * 3) % 7
    for v, (uplo, trans, diag) in enumerate(VARIANTS):
        seed = 1000 * n + 10 * nrhs + v
        buf, clean = tri_case(seed, n, uplo, diag, ldt, dt)
        B = rng.normal(seed + 7, (n, nrhs), dt)
        got = run_trsm(L, uplo, trans, diag, buf, n, B, ldb)
        want = scipy.linalg.solve_triangular(
            clean.astype(np.float64), B.astype(np.float64),
            lower=(uplo == "L"), trans=(1 if trans == "T" else 0),
            unit_diagonal=(diag == "U"))
        assert np.all(np.isfinite(got)), f"{uplo}{trans}{diag}: non-finite"
        scale = max(np.abs(want).max(), 1e-300)
        err = np.abs(got.astype(np.float64) - want).max() / scale
        assert err <= TOL[prec], (f"{uplo}{trans}{diag} n={n} nrhs={nrhs}: "
                                  f"rel err {err:.3e}")


@pytest.mark.parametrize("prec", ["f32", "f64"])
def test_trsm_zero_sizes_are_noops(gpu, prec):
    L = gpu[prec]
    dB = L.dalloc(64)
    try:
        L.check(L.c.matgb_memset_dev(dB, 0x5a, 64), "memset")
        for n, nrhs in ((0, 5), (5, 0)):
            rc = L.c.matgb_trsm_dev(b"L", b"N", b"N", n, nrhs, None, max(n, 1),
                                    dB, max(n, 1))
            L.check(rc, "trsm_dev")
        out = np.empty(64, np.uint8)
        L.d2h(out, dB)
        assert np.all(out == 0x5A)
    finally:
        L.dfree(dB)
