"""mat_gemv_t (mat.h:2224-2248) and mat_axpy (mat.h:2009-2015) on the GPU.

mat_axpy rounds alpha * x[i] before the addition, as the reference's scalar
loop does, so its results must be identical to the oracle's, NaN and
infinity included.  mat_gemv_t sums each column's dot product in a
different order from the reference's index-order loop.  It is checked
entrywise against the oracle within
    |y - y_ref| <= 2 * m * u * (|alpha| * |A|^T |x| + |beta * y0|) + tiny,
the standard bound for two summation orders of the same dot product.
Shapes cover one row and one column, ragged sizes around the 32-lane and
8-column granules, and tall, skinny products whose rows are split into
chunks, which a second launch adds in a fixed order.  At 700000 x 64 the
chunk count is capped by the column count, so each chunk spans more than
the 8192-row minimum.
"""
import numpy as np
import pytest

from oracle.loader import Oracle

pytestmark = pytest.mark.gpu

PRECS = ["f32", "f64"]
DT = {"f32": np.float32, "f64": np.float64}


def gemv_t_bound(A, x, y0, alpha, beta, dt):
    u = np.finfo(dt).eps
    m = A.shape[0]
    mag = abs(alpha) * (np.abs(A.astype(np.float64)).T @ np.abs(x.astype(np.float64)))
    return 2 * max(m, 1) * u * (mag + np.abs(beta * y0.astype(np.float64))) \
        + np.finfo(dt).tiny


@pytest.mark.parametrize("prec", PRECS)
def test_gemv_t_against_oracle(gpu, prec):
    L_, dt = gpu[prec], DT[prec]
    O = Oracle(prec, "port")
    rs = np.random.default_rng(31)
    shapes = [(1, 1), (1, 9), (33, 1), (31, 8), (257, 65), (1000, 300),
              (40000, 3), (20000, 17), (700000, 64)]
    for m, n in shapes:
        A = rs.standard_normal((m, n)).astype(dt)
        x = rs.standard_normal(m).astype(dt)
        y0 = rs.standard_normal(n).astype(dt)
        for alpha, beta in ((1.0, 0.0), (-0.75, 1.0), (2.5, -0.5)):
            got = L_.mat_gemv_t(y0, alpha, A, x, beta)
            ref = O.gemv_t(alpha, A, x, beta, y0)
            err = np.abs(got.astype(np.float64) - ref.astype(np.float64))
            assert np.all(err <= gemv_t_bound(A, x, y0, alpha, beta, dt)), (m, n)


@pytest.mark.parametrize("prec", PRECS)
def test_gemv_t_propagates_nan_like_reference(gpu, prec):
    """beta * y is always formed (mat.h:2235): a NaN in y survives beta = 0,
    and an infinity in A reaches its column only."""
    L_, dt = gpu[prec], DT[prec]
    O = Oracle(prec, "port")
    A = np.arange(12, dtype=dt).reshape(4, 3) / dt(7)
    A[1, 2] = np.inf
    x = np.array([1, -2, 0.5, 3], dt)
    y0 = np.array([np.nan, 1, 2], dt)
    got = L_.mat_gemv_t(y0, 1.0, A, x, 0.0)
    ref = O.gemv_t(1.0, A, x, 0.0, y0)
    assert np.isnan(got[0]) and np.isnan(ref[0])
    assert np.isinf(got[2]) and got[2] == ref[2]
    assert abs(float(got[1]) - float(ref[1])) <= 8 * np.finfo(dt).eps * 10


@pytest.mark.parametrize("prec", PRECS)
def test_axpy_bit_identical(gpu, prec):
    L_, dt = gpu[prec], DT[prec]
    O = Oracle(prec, "port")
    rs = np.random.default_rng(41)
    for n in (1, 31, 32, 1000, 1 << 20):
        x = rs.standard_normal(n).astype(dt)
        y = rs.standard_normal(n).astype(dt)
        if n > 2:
            x[1], y[2] = np.inf, np.nan
        for alpha in (0.0, 1.0, -3.25, 1e-3):
            got = L_.mat_axpy(y, alpha, x)
            assert np.array_equal(got, O.axpy(y, alpha, x), equal_nan=True), n


@pytest.mark.parametrize("prec", PRECS)
def test_gemv_t_dev_strided(gpu, prec):
    """The device entry with lda > m; padding rows hold NaN, which any read
    of them would carry into y."""
    L_, dt = gpu[prec], DT[prec]
    O = Oracle(prec, "port")
    m, n, lda = 300, 40, 307
    rs = np.random.default_rng(5)
    A = rs.standard_normal((m, n)).astype(dt)
    buf = np.full((lda, n), np.nan, dt, order="F")
    buf[:m] = A
    x = rs.standard_normal(m).astype(dt)
    y0 = rs.standard_normal(n).astype(dt)
    dA, dx, dy = L_.dalloc(buf.nbytes), L_.dalloc(x.nbytes), L_.dalloc(y0.nbytes)
    try:
        L_.h2d(dA, buf)
        L_.h2d(dx, x)
        L_.h2d(dy, y0)
        L_.check(L_.c.matgb_gemv_t_dev(m, n, L_.ct(0.5), dA, lda, dx,
                                       L_.ct(2.0), dy), "gemv_t")
        got = np.empty(n, dt)
        L_.d2h(got, dy)
    finally:
        for d in (dA, dx, dy):
            L_.dfree(d)
    ref = O.gemv_t(0.5, A, x, 2.0, y0)
    err = np.abs(got.astype(np.float64) - ref.astype(np.float64))
    assert np.all(err <= gemv_t_bound(A, x, y0, 0.5, 2.0, dt))
