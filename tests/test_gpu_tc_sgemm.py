"""GPU: the float build's tensor-core products behind mat_gemm / mat_mul /
mat_syrk and the plain Cholesky's SYRK updates (FP16 hi + remainder split
under power-of-two row / column scales, three products, FP32 accumulation)
and behind the plain LU's trailing updates (hi + mid + remainder, six
products, about 33 bits of each operand), through the C ABI.

Each case is checked against an FP64 product of the same float inputs (the
exact answer to ~1e-16) and against the oracle where it is quick, within the
parity suite's product bound, 2e-5 * max(1, K/256) of max |C| (relative,
max-norm), and against the FP32 SIMT kernel (matgb_plain_tensor_core(0)) on
the same call.  Factorisations: pivots identical to the oracle's (the
reference's scalar path) on tie-free inputs, factors within 2e-4 of max
|ref|, as in the parity suite.
"""
import ctypes as C

import numpy as np
import pytest

from libmat_gb300 import rng
from oracle.loader import Oracle

pytestmark = pytest.mark.gpu

TOL = 2e-5


def rel(got, ref):
    ref = np.asarray(ref, np.float64)
    return np.abs(np.asarray(got, np.float64) - ref).max() / max(np.abs(ref).max(), 1e-300)


def dev_gemm(L, ta, tb, A, B, C0, alpha, beta):
    m = A.shape[1] if ta else A.shape[0]
    k = A.shape[0] if ta else A.shape[1]
    n = B.shape[0] if tb else B.shape[1]
    dA, dB, dC = L.dalloc(A.nbytes), L.dalloc(B.nbytes), L.dalloc(C0.nbytes)
    try:
        L.h2d(dA, np.asfortranarray(A))
        L.h2d(dB, np.asfortranarray(B))
        L.h2d(dC, np.asfortranarray(C0))
        L.check(L.c.matgb_gemm_dev(b"T" if ta else b"N", b"T" if tb else b"N",
                                   m, n, k, alpha, dA, A.shape[0], dB,
                                   B.shape[0], beta, dC, m), "gemm")
        out = np.empty((m, n), np.float32, order="F")
        L.d2h(out, dC)
    finally:
        for p in (dA, dB, dC):
            L.dfree(p)
    return out


@pytest.fixture
def tc_mode(gpu):
    L = gpu["f32"]
    prev = L.c.matgb_plain_tensor_core(-1)
    yield L
    L.c.matgb_plain_tensor_core(prev)


@pytest.mark.parametrize("ta,tb", [(False, False), (True, False), (False, True),
                                   (True, True)])
@pytest.mark.parametrize("mkn", [(256, 16, 256), (300, 77, 513), (1000, 1000, 257),
                                 (777, 2500, 390)])
def test_tc_gemm_matches_fp64_and_simt(tc_mode, ta, tb, mkn):
    L = tc_mode
    m, k, n = mkn
    A = rng.normal(21, (k, m) if ta else (m, k), np.float32)
    B = rng.normal(22, (n, k) if tb else (k, n), np.float32)
    C0 = rng.normal(23, (m, n), np.float32)
    opA = A.T if ta else A
    opB = B.T if tb else B
    exact = 1.5 * opA.astype(np.float64) @ opB.astype(np.float64) - 0.5 * C0
    tol = TOL * max(1.0, k / 256)
    L.c.matgb_plain_tensor_core(1)
    got = dev_gemm(L, ta, tb, A, B, C0, 1.5, -0.5)
    L.c.matgb_plain_tensor_core(0)
    simt = dev_gemm(L, ta, tb, A, B, C0, 1.5, -0.5)
    assert rel(got, exact) <= tol
    assert rel(got, simt) <= tol


def test_tc_gemm_row_and_column_scales(tc_mode):
    """Rows of A and columns of B spanning 60 binades: per-row / per-column
    scales keep every entry of C accurate relative to its own row/column."""
    L = tc_mode
    L.c.matgb_plain_tensor_core(1)
    m = k = n = 384
    A = rng.normal(31, (m, k), np.float32)
    B = rng.normal(32, (k, n), np.float32)
    rs = (2.0 ** np.linspace(-30, 30, m)).astype(np.float32)
    cs = (2.0 ** np.linspace(30, -30, n)).astype(np.float32)
    A *= rs[:, None]
    B *= cs[None, :]
    got = dev_gemm(L, False, False, A, B, np.zeros((m, n), np.float32), 1.0, 0.0)
    exact = A.astype(np.float64) @ B.astype(np.float64)
    # entry-wise relative to |A||B| (the product's natural scale)
    scale = np.abs(A).astype(np.float64) @ np.abs(B).astype(np.float64)
    assert (np.abs(got - exact) / scale).max() <= TOL * 2


def test_tc_gemm_special_values(tc_mode):
    """beta = 0 never reads C (NaN there is ignored); NaN and infinity in the
    operands reach exactly the entries they touch; a zero row gives zeros."""
    L = tc_mode
    L.c.matgb_plain_tensor_core(1)
    m = k = n = 300
    A = rng.normal(41, (m, k), np.float32)
    B = rng.normal(42, (k, n), np.float32)
    A[5, 7] = np.nan
    A[9, :] = 0.0
    B[3, 11] = np.inf
    C0 = np.full((m, n), np.nan, np.float32)
    got = dev_gemm(L, False, False, A, B, C0, 1.0, 0.0)
    exp = A.astype(np.float64) @ B.astype(np.float64)
    assert np.isnan(got[5]).all()
    assert np.array_equal(np.isfinite(got), np.isfinite(exp))
    ok = np.isfinite(exp)
    assert np.abs(got[ok] - exp[ok]).max() / np.abs(exp[ok]).max() <= TOL * 2
    # a zero row gives zeros except where it meets the infinite column
    # (0 * inf = NaN, as in FP32)
    assert np.all(got[9][np.arange(n) != 11] == 0.0) and np.isnan(got[9, 11])


@pytest.mark.parametrize("uplo", ["L", "U"])
@pytest.mark.parametrize("trans", [False, True])
def test_tc_syrk(tc_mode, uplo, trans):
    L = tc_mode
    L.c.matgb_plain_tensor_core(1)
    n, k = 520, 200
    A = rng.normal(51, (k, n) if trans else (n, k), np.float32)
    C0 = rng.normal(52, (n, n), np.float32)
    got = L.mat_syrk(C0, A, 0.75, 0.5, uplo=uplo, trans=trans)
    opA = (A.T if trans else A).astype(np.float64)
    full = 0.75 * opA @ opA.T + 0.5 * C0
    tri = np.tril if uplo == "L" else np.triu
    tol = TOL * max(1.0, k / 256)
    assert rel(tri(got), tri(full)) <= tol
    O = Oracle("f32")
    ref = O.syrk_t(C0, A, 0.75, 0.5, uplo) if trans else O.syrk(C0, A, 0.75, 0.5, uplo)
    assert rel(got, ref) <= tol


@pytest.mark.parametrize("n", [1024, 1500])
def test_tc_plain_lu_and_chol_vs_oracle(tc_mode, n):
    """The plain float LU and Cholesky with the tensor cores switched on (the
    Cholesky takes tensor-core SYRK updates at these orders): the oracle's
    pivots exactly; the LU factors reproduce P A to n u of |A| (at these
    orders the last multipliers of two float eliminations differ by ~1e-3,
    rounding noise, so they are not compared entry by entry); the Cholesky
    factor of a well-conditioned matrix within 2e-4 of the oracle's."""
    L = tc_mode
    L.c.matgb_plain_tensor_core(1)
    O = Oracle("f32")
    A = rng.uniform(61 + n, (n, n), -1.0, 1.0, np.float32)
    Lg, Ug, pg, sg = L.mat_plu(A)
    _, _, pr, sr = O.plu(A)
    assert np.array_equal(pg, pr) and sg == sr
    A64 = A.astype(np.float64)
    res = np.abs(A64[pg] - Lg.astype(np.float64) @ Ug.astype(np.float64)).max()
    assert res <= n * 2.0 ** -24 * np.abs(A64).max()
    Bm = rng.normal(62 + n, (n, n), np.float32)
    S = (Bm.T @ Bm / n + np.eye(n, dtype=np.float32)).astype(np.float32)
    Lc, rc = L.mat_chol(S)
    Lo, ro = O.chol(S)
    assert rc == ro == 0
    assert rel(Lc, Lo) <= 2e-4


@pytest.mark.parametrize("n", [2048, 3000])
def test_tc_plain_lu_matches_simt_lu(tc_mode, n):
    """The plain float LU with its trailing updates on the tensor cores (the
    six-product split) against the same LU with FP32 SIMT updates, through
    matgb_getrf_dev: the same pivots on the data-determined steps (all but
    the last 5%, where the float Schur complement is rounding noise -- as
    at the 8192 config, where the reference's own float and double pivots
    part at step 8116); the leading half of the factors' columns within the
    parity suite's factor bound (2e-4 of max |ref|; the last multipliers of
    two float eliminations at these orders differ by ~3e-4, rounding noise
    amplified by the late Schur complements); both factorisations reproduce
    P A to n u of |A|."""
    L = tc_mode
    A = rng.uniform(71 + n, (n, n), -1.0, 1.0, np.float32)
    out = {}
    for on in (1, 0):
        L.c.matgb_plain_tensor_core(on)
        dA, dp = L.dalloc(A.nbytes), L.dalloc(8 * n)
        try:
            L.h2d(dA, np.asfortranarray(A))
            L.check(L.c.matgb_getrf_dev(n, dA, n, dp, dp + 4 * n), "getrf")
            LU = np.empty((n, n), np.float32, order="F")
            L.d2h(LU, dA)
            piv = np.empty(2 * n, np.int32)
            L.d2h(piv, dp)
        finally:
            L.dfree(dA)
            L.dfree(dp)
        out[on] = (LU, piv)
    p1, p0 = out[1][1][n:], out[0][1][n:]
    diff = np.nonzero(p1 != p0)[0]
    k = int(diff[0]) if len(diff) else n
    assert k >= int(0.95 * n), k
    assert rel(out[1][0][:, :n // 2], out[0][0][:, :n // 2]) <= 2e-4
    A64 = A.astype(np.float64)
    for LU, piv in out.values():
        LU = LU.astype(np.float64)
        Lf = np.tril(LU, -1) + np.eye(n)
        Uf = np.triu(LU)
        res = np.abs(A64[piv[n:]] - Lf @ Uf).max()
        assert res <= n * 2.0 ** -24 * np.abs(A64).max(), res
