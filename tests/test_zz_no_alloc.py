"""GPU: matgb_gemv_noalloc_dev, the GEMV for callers that must not allocate
device memory (its partial sums use a static device array instead of the
library workspace), called through the C ABI and checked against
matgb_gemv_dev on two calls in a row.  Tolerance: the GEMV bound of the
parity suite, f32 2e-5 / f64 1e-13 relative to max|y|, scaled by K/256 (the
two entry points may split the columns differently, so sums may round
differently).  Collected last so a failure here never hides another test."""
import numpy as np
import pytest

from libmat_gb300 import rng

pytestmark = pytest.mark.gpu

TOL = {"f32": 2e-5, "f64": 1e-13}
SCRATCH_ELEMS = 1 << 20


def run(L, fn, m, n, alpha, dA, dx, beta, y0, dy, stream):
    L.h2d(dy, y0)
    if fn == "noalloc":
        rc = L.c.matgb_gemv_noalloc_dev(m, n, alpha, dA, m, dx, beta, dy, stream)
    else:
        rc = L.c.matgb_gemv_dev(m, n, alpha, dA, m, dx, beta, dy)
    L.check(rc, fn)
    out = np.empty(m, L.dtype)
    L.d2h(out, dy)
    return out


@pytest.mark.parametrize("prec", ["f32", "f64"])
def test_noalloc_gemv_matches_workspace_gemv_twice(gpu, prec):
    L = gpu[prec]
    dt = L.dtype
    stream = L.c.matgb_stream()
    for call, (m, n) in enumerate([(3000, 2000), (777, 4097)]):
        A = rng.normal(900 + call, (m, n), dt)
        x = rng.normal(910 + call, (n,), dt)
        y0 = rng.normal(920 + call, (m,), dt)
        dA, dx, dy = L.dalloc(A.nbytes), L.dalloc(x.nbytes), L.dalloc(y0.nbytes)
        try:
            L.h2d(dA, A)
            L.h2d(dx, x)
            ref = run(L, "ws", m, n, 1.5, dA, dx, -0.5, y0, dy, stream)
            got = run(L, "noalloc", m, n, 1.5, dA, dx, -0.5, y0, dy, stream)
        finally:
            for p in (dA, dx, dy):
                L.dfree(p)
        err = np.abs(got.astype(np.float64) - ref).max() / np.abs(ref).max()
        assert err <= TOL[prec] * max(1.0, n / 256), (call, err)
        exact = A.astype(np.float64) @ x.astype(np.float64) * 1.5 - 0.5 * y0
        assert np.abs(got - exact).max() / np.abs(exact).max() <= \
            TOL[prec] * max(1.0, n / 256) * 4


@pytest.mark.parametrize("prec", ["f32", "f64"])
def test_noalloc_gemv_rejects_rows_beyond_scratch(gpu, prec):
    L = gpu[prec]
    m = SCRATCH_ELEMS + 1
    rc = L.c.matgb_gemv_noalloc_dev(m, 1, 1.0, None, m, None, 0.0, None, None)
    assert rc == -2  # MATGB_ERR_ARG
    msg = L.c.matgb_last_error().decode()
    L.c.matgb_clear_error()
    assert "static scratch" in msg


@pytest.mark.parametrize("prec", ["f32", "f64"])
@pytest.mark.parametrize("which", ["caller", "null"])
def test_noalloc_gemv_on_callers_stream(gpu, prec, which):
    """The allocation-free GEMV runs on the stream the caller passes -- one it
    created, or NULL (the legacy default stream) -- and leaves the library
    stream alone: the caller synchronises its own stream before reading y."""
    torch = pytest.importorskip("torch")
    L = gpu[prec]
    dt = L.dtype
    m, n = 2500, 1500
    A = rng.normal(930, (m, n), dt)
    x = rng.normal(931, (n,), dt)
    y0 = rng.normal(932, (m,), dt)
    dA, dx, dy = L.dalloc(A.nbytes), L.dalloc(x.nbytes), L.dalloc(y0.nbytes)
    s = torch.cuda.Stream() if which == "caller" else None
    try:
        L.h2d(dA, A)
        L.h2d(dx, x)
        ref = run(L, "ws", m, n, 0.75, dA, dx, 2.0, y0, dy, L.c.matgb_stream())
        for _ in range(2):
            L.h2d(dy, y0)
            L.sync()
            rc = L.c.matgb_gemv_noalloc_dev(m, n, 0.75, dA, m, dx, 2.0, dy,
                                            s.cuda_stream if s else None)
            L.check(rc, "noalloc")
            if s is not None:
                s.synchronize()
            else:
                torch.cuda.synchronize()
            got = np.empty(m, dt)
            L.d2h(got, dy)
            err = np.abs(got.astype(np.float64) - ref).max() / np.abs(ref).max()
            assert err <= TOL[prec] * max(1.0, n / 256), err
    finally:
        for p in (dA, dx, dy):
            L.dfree(p)
