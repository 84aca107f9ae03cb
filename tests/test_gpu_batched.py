"""GPU: the batched small-system solver (one pass over many uneven systems),
each system checked against the oracle's mat_solve / mat_solve_spd.

Systems are well conditioned by construction (U[-1,1] + n*I for LU,
B^T B + n*I for Cholesky), so the tolerance is the parity suite's factor
bound: max|x - x_ref| <= 2e-4 * max|x_ref| (f32) / 1e-11 (f64).  Systems
that pivot (U[-1,1], no shift) are held to the parity suite's conditioning
bound: |x - x_ref| <= 10 * cond(A) * u * |x_ref| (the oracle solves with the
same pivots; two backward-stable float solves differ by ~cond * u).  Both
schedules of the large buckets -- the blocked LU and the register
Gauss-Jordan kernel -- are run (matgb_batched_tune)."""
import ctypes as C

import numpy as np
import pytest

from oracle.loader import Oracle

pytestmark = pytest.mark.gpu
TOL = {"f32": 2e-4, "f64": 1e-11}
U = {"f32": 2.0 ** -24, "f64": 2.0 ** -53}


@pytest.fixture(params=[1, 0], ids=["blocked", "gauss_jordan"])
def algo(request, gpu):
    """Every large bucket on one algorithm for the test, defaults restored."""
    saved = {}
    for prec in ("f32", "f64"):
        L = gpu[prec]
        for nb in (64, 96, 128):
            for kind in (0, 1):
                a, c = C.c_int(), C.c_int()
                L.check(L.c.matgb_batched_tune_get(nb, kind, C.byref(a), C.byref(c)))
                saved[prec, nb, kind] = (a.value, c.value)
                # the double build's 96 and 128 buckets have one form only
                L.check(L.c.matgb_batched_tune(nb, kind, request.param, c.value))
    yield request.param
    for (prec, nb, kind), (a, c) in saved.items():
        gpu[prec].c.matgb_batched_tune(nb, kind, a, c)


def make_batch(count, nmax, dt, seed):
    rs = np.random.default_rng(seed)
    mats, rhs, kinds = [], [], []
    for s in range(count):
        n = int(rs.integers(1, nmax + 1))
        kind = s % 2
        if kind == 0:
            A = rs.uniform(-1, 1, (n, n)) + n * np.eye(n)
        else:
            B = rs.standard_normal((n, n))
            A = B.T @ B + n * np.eye(n)
        mats.append(np.asfortranarray(A.astype(dt)))
        rhs.append(rs.standard_normal(n).astype(dt))
        kinds.append(kind)
    return mats, rhs, kinds


@pytest.mark.parametrize("prec,nmax,count", [("f32", 128, 600), ("f32", 20, 300),
                                             ("f64", 128, 300)])
def test_batched_matches_oracle(gpu, algo, prec, nmax, count):
    L = gpu[prec]
    O = Oracle(prec)
    mats, rhs, kinds = make_batch(count, nmax, L.dtype, 11 + nmax)
    xs, status = L.solve_batched(mats, rhs, kinds)
    assert np.all(status == 0)
    for A, b, k, x in zip(mats, rhs, kinds, xs):
        xr = O.solve(A, b) if k == 0 else O.solve_spd(A, b)[0]
        err = np.abs(x.astype(np.float64) - xr).max() / np.abs(xr).max()
        assert err <= TOL[prec], (A.shape[0], k, err)


@pytest.mark.parametrize("prec", ["f32", "f64"])
def test_batched_pivoting_and_not_spd(gpu, algo, prec):
    """Row exchanges on every step (U[-1,1], no diagonal shift) in every
    bucket: x within 10 * cond * u of the oracle's mat_solve; a non-SPD
    system (a negative Schur diagonal at step 3, and one at the last step)
    reports -1 and leaves its x untouched while its neighbours solve."""
    L = gpu[prec]
    O = Oracle(prec)
    dt = L.dtype
    rs = np.random.default_rng(5)
    mats, rhs, kinds = [], [], []
    sizes = (1, 2, 3, 8, 9, 16, 17, 31, 33, 40, 64, 65, 77, 96, 97, 120, 128)
    for n in sizes:
        mats.append(np.asfortranarray(rs.uniform(-1, 1, (n, n)).astype(dt)))
        rhs.append(rs.standard_normal(n).astype(dt))
        kinds.append(0)
    for n, where in ((5, 3), (100, 99)):
        bad = np.eye(n, dtype=dt) * 2
        bad[where, where] = -2.0
        mats.append(bad)
        rhs.append(np.ones(n, dt))
        kinds.append(1)
    xs, status = L.solve_batched(mats, rhs, kinds)
    assert list(status) == [0] * len(sizes) + [-1, -1]
    # untouched: the solution buffer still holds the input copy
    assert np.array_equal(xs[-1], rhs[-1]) and np.array_equal(xs[-2], rhs[-2])
    for A, b, x in zip(mats[:len(sizes)], rhs, xs):
        xr = O.solve(A, b).astype(np.float64)
        cond = np.linalg.cond(A.astype(np.float64), np.inf)
        err = np.abs(x.astype(np.float64) - xr).max() / np.abs(xr).max()
        assert err <= 10 * cond * U[prec], (A.shape[0], err, cond)


def test_batched_marks_unsupported_order(gpu):
    """Orders above 128 (and below 1) get status -2; their neighbours are
    still solved, in both builds (the double build's 65..128 orders keep
    their rows in shared memory)."""
    for prec in ("f32", "f64"):
        L = gpu[prec]
        dt = L.dtype
        mats = [np.eye(130, dtype=dt) * 2, np.eye(3, dtype=dt) * 4,
                np.eye(100, dtype=dt) * 8]
        xs, status = L.solve_batched(mats, [np.ones(130, dt), np.ones(3, dt),
                                            np.ones(100, dt)], [0, 1, 0])
        assert list(status) == [-2, 0, 0]
        assert np.allclose(xs[1], 0.25) and np.allclose(xs[2], 0.125)
