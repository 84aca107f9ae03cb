"""GPU: the batched small-system solver (one pass over many uneven systems),
each system checked against the oracle's mat_solve / mat_solve_spd.

Systems are well conditioned by construction (U[-1,1] + n*I for LU,
B^T B + n*I for Cholesky), so the tolerance is the parity suite's factor
bound: max|x - x_ref| <= 2e-4 * max|x_ref| (f32) / 1e-11 (f64)."""
import numpy as np
import pytest

from oracle.loader import Oracle

pytestmark = pytest.mark.gpu
TOL = {"f32": 2e-4, "f64": 1e-11}


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
                                             ("f64", 64, 300)])
def test_batched_matches_oracle(gpu, prec, nmax, count):
    L = gpu[prec]
    O = Oracle(prec)
    mats, rhs, kinds = make_batch(count, nmax, L.dtype, 11 + nmax)
    xs, status = L.solve_batched(mats, rhs, kinds)
    assert np.all(status == 0)
    for A, b, k, x in zip(mats, rhs, kinds, xs):
        xr = O.solve(A, b) if k == 0 else O.solve_spd(A, b)[0]
        err = np.abs(x.astype(np.float64) - xr).max() / np.abs(xr).max()
        assert err <= TOL[prec], (A.shape[0], k, err)


def test_batched_pivoting_and_not_spd(gpu):
    """Row exchanges are exercised (no diagonal shift), and a non-SPD system
    reports -1 and leaves its x untouched while its neighbours solve."""
    L = gpu["f32"]
    O = Oracle("f32")
    rs = np.random.default_rng(5)
    mats, rhs, kinds = [], [], []
    for n in (3, 17, 40, 77, 128):
        mats.append(np.asfortranarray(rs.uniform(-1, 1, (n, n)).astype(np.float32)))
        rhs.append(rs.standard_normal(n).astype(np.float32))
        kinds.append(0)
    bad = np.eye(5, dtype=np.float32)
    bad[3, 3] = -2.0
    mats.append(bad)
    rhs.append(np.ones(5, np.float32))
    kinds.append(1)
    xs, status = L.solve_batched(mats, rhs, kinds)
    assert list(status) == [0, 0, 0, 0, 0, -1]
    assert np.array_equal(xs[-1], rhs[-1])  # untouched: still the input copy
    for A, b, x in zip(mats[:-1], rhs[:-1], xs[:-1]):
        xr = O.solve(A, b)
        # random U[-1,1] matrices: compare through the backward error
        r = np.abs(A.astype(np.float64) @ x - b).max()
        eta = r / (np.abs(A).sum(1).max() * np.abs(x).max() + np.abs(b).max())
        assert eta <= 1e-5, (A.shape[0], eta)
        assert np.abs(x - xr).max() / np.abs(xr).max() <= 0.05


def test_batched_f64_marks_unsupported_order(gpu):
    """The double build solves orders up to 64; larger systems get status -2
    and their neighbours are still solved."""
    L = gpu["f64"]
    mats = [np.eye(100) * 2, np.eye(3) * 4]
    xs, status = L.solve_batched(mats, [np.ones(100), np.ones(3)], [0, 1])
    assert list(status) == [-2, 0]
    assert np.allclose(xs[1], 0.25)
