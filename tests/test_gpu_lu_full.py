"""mat_lu (full pivoting, mat.h:4476-4574) on the GPU, bit-identical to the
reference.

Integer results (p, q, the swap count) and the factors themselves must be
identical: the reference's elimination rounds every product before it is
subtracted and picks the first entry (row-major) of the largest magnitude,
and the GPU kernel does the same operations in the same order per entry.

Cases:
  - the reference's own test matrices (tests/golden/lu_<prec>.npz, made
    by the reference compiled in place);
  - the scalar oracle on seeded inputs: values in steps of 0.1 (many ties,
    test_mat_lu.c's generator), Gaussian values, orders around the 64-entry
    tile, a zero matrix (every step skipped), NaN, infinity and sub-epsilon
    entries;
  - the vectorised restatement (tests/lu_full_np.py, pinned to the scalar
    oracle on the CPU) at orders the scalar oracle cannot reach in seconds,
    n = 2304 (f32) and 1100 (f64), whose early steps have more 64 x 32
    tiles than resident CTAs, so that each CTA covers several;
  - matgb_getrf_full_dev with a leading dimension above n.
"""
import numpy as np
import pytest

from conftest import golden
from lu_full_np import lu_full_np, perms
from oracle.loader import Oracle

pytestmark = pytest.mark.gpu

PRECS = ["f32", "f64"]
DT = {"f32": np.float32, "f64": np.float64}
EPS = {"f32": np.float32(1e-6), "f64": 1e-9}


def same(a, b):
    return np.array_equal(a, b, equal_nan=True)


@pytest.mark.parametrize("prec", PRECS)
def test_lu_full_golden(gpu, prec):
    L_ = gpu[prec]
    g = golden(f"lu_{prec}.npz")
    names = sorted({k[:-2] for k in g if k.endswith("_A")})
    assert len(names) == 6
    for name in names:
        L, U, p, q, s = L_.mat_lu(g[name + "_A"])
        assert same(L, g[name + "_L"]), name
        assert same(U, g[name + "_U"]), name
        assert np.array_equal(p, g[name + "_p"]), name
        assert np.array_equal(q, g[name + "_q"]), name
        assert s == int(g[name + "_s"]), name


@pytest.mark.parametrize("prec", PRECS)
def test_lu_full_oracle(gpu, prec):
    L_, dt = gpu[prec], DT[prec]
    O = Oracle(prec, "port")
    rs = np.random.default_rng(2024)
    cases = [np.zeros((6, 6), dt), np.ones((1, 1), dt),
             np.array([[0, 1], [1, 0]], dt)]
    for n in (2, 3, 31, 63, 64, 65, 128, 129, 300):
        cases.append((rs.integers(0, 200, (n, n)) - 100).astype(dt) / dt(10))
        cases.append(rs.standard_normal((n, n)).astype(dt))
    odd = rs.standard_normal((70, 70)).astype(dt)
    odd[0, 0], odd[40, 7], odd[3, 66], odd[69, 69] = np.nan, np.inf, -np.inf, 0
    odd[10:20, 10:20] = dt(1e-12)
    cases.append(odd)
    small = rs.standard_normal((40, 40)).astype(dt) * dt(1e-7)  # steps skipped
    small[:8, :8] = rs.standard_normal((8, 8)).astype(dt)
    cases.append(small)
    for A in cases:
        got, ref = L_.mat_lu(A), O.lu(A)
        for a, b in zip(got[:4], ref[:4]):
            assert same(a, b), A.shape
        assert got[4] == ref[4], A.shape


@pytest.mark.parametrize("prec,n", [("f32", 2304), ("f64", 1100)])
def test_lu_full_large(gpu, prec, n):
    L_, dt = gpu[prec], DT[prec]
    A = np.random.default_rng(n).standard_normal((n, n)).astype(dt)
    L, U, p, q, s = L_.mat_lu(A)
    M, rp, cp, s2 = lu_full_np(A, EPS[prec])
    p2, q2 = perms(rp, cp)
    assert np.array_equal(p, p2) and np.array_equal(q, q2) and s == s2
    assert np.array_equal(L, np.tril(M, -1) + np.eye(n, dtype=dt))
    assert np.array_equal(U, np.triu(M))
    # full pivoting: multipliers at most 1, each pivot the largest in its row
    assert np.abs(L).max() <= 1
    d = np.abs(np.diag(U))
    assert np.all(d[:, None] >= np.abs(np.triu(U)))
    r = A.astype(np.float64)[p][:, q] - L.astype(np.float64) @ U.astype(np.float64)
    u = np.finfo(dt).eps
    assert np.abs(r).max() <= 4 * n * u * np.abs(A).max() * max(1.0, np.abs(U).max())


@pytest.mark.parametrize("prec", PRECS)
def test_getrf_full_dev_strided(gpu, prec):
    """The device entry on a buffer with lda > n: the padding rows are not
    touched, the packed factor and the recorded swaps are the oracle's."""
    L_, dt = gpu[prec], DT[prec]
    n, lda = 97, 101
    A = (np.random.default_rng(7).integers(0, 200, (n, n)) - 100).astype(dt) / dt(10)
    buf = np.full((lda, n), 12345.0, dt, order="F")
    buf[:n] = A
    dA = L_.dalloc(buf.nbytes)
    dp = L_.dalloc(8 * n)
    try:
        L_.h2d(dA, buf)
        L_.check(L_.c.matgb_getrf_full_dev(n, dA, lda, dp, dp + 4 * n), "getrf_full")
        out = np.empty((lda, n), dt, order="F")
        L_.d2h(out, dA)
        pv = np.empty(2 * n, np.int32)
        L_.d2h(pv, dp)
    finally:
        L_.dfree(dA)
        L_.dfree(dp)
    assert np.all(out[n:] == dt(12345.0))
    M, rp, cp, _ = lu_full_np(A, EPS[prec])
    assert np.array_equal(out[:n], M)
    assert np.array_equal(pv[:n], rp) and np.array_equal(pv[n:], cp)
    assert L_.c.matgb_getrf_full_dev(n, None, n - 1, None, None) != 0  # lda < n
    L_.c.matgb_clear_error()
