"""GPU parity: every hot-path entry point of libmatgb, called through its C ABI
(include/mat.h), against the reference's outputs (golden fixtures made by the
reference itself) and against the oracle (C restatement of the reference's
scalar path) on the same seeded inputs.

Tolerances (stated once, used everywhere; max-norm, relative to max|ref|):
  factors / solutions: f32 2e-4, f64 1e-11
  products (GEMM/SYRK/GEMV): f32 2e-5 * max(1, K/256), f64 1e-13 * max(1, K/256)
The reference's own f32-vs-f64 spread on the 256x256 config is 1.1e-5 for
the LU factors, so the f32 bound leaves a 15x margin for the GPU's different
summation order.  Solutions of ill-conditioned inputs are bounded in terms of
the conditioning (forward error <= 10 * cond(A) * u against the reference's,
normwise backward error <= n * u): two backward-stable solves in f32 of the
256x256 config (cond 1.3e4) may differ by ~cond*u.  Pivot permutations and
swap counts must be identical (integer results: exact).
"""
import numpy as np
import pytest

from conftest import golden
from libmat_gb300 import rng
from oracle.loader import Oracle

pytestmark = pytest.mark.gpu

PRECS = ["f32", "f64"]
TOL_FACT = {"f32": 2e-4, "f64": 1e-11}
TOL_PROD = {"f32": 2e-5, "f64": 1e-13}


def rel(got, ref):
    got = np.asarray(got, np.float64)
    ref = np.asarray(ref, np.float64)
    s = max(np.abs(ref).max(initial=0.0), 1e-300)
    return np.abs(got - ref).max(initial=0.0) / s


def close(got, ref, tol):
    e = rel(got, ref)
    assert e <= tol, f"max rel err {e:.3e} > {tol:.1e}"


# ---------------------------------------------------------------- KATs ----
@pytest.mark.parametrize("prec", PRECS)
def test_kat_plu(gpu, prec):
    L_ = gpu[prec]
    g = golden(f"kat_{prec}.npz")
    for name in ("plu_2x2", "plu_3x3"):
        L, U, p, s = L_.mat_plu(g[name + "_A"])
        assert np.array_equal(p, g[name + "_p"]) and s == g[name + "_s"]
        close(L, g[name + "_L"], TOL_FACT[prec])
        close(U, g[name + "_U"], TOL_FACT[prec])
        A = g[name + "_A"]
        assert np.allclose(A[p], L @ U, atol=1e-5)  # tests/test_mat_plu.c:37


@pytest.mark.parametrize("prec", PRECS)
def test_kat_solve(gpu, prec):
    L_ = gpu[prec]
    g = golden(f"kat_{prec}.npz")
    for name in ("solve_1x1", "solve_identity", "solve_2x2", "solve_3x3"):
        x = L_.mat_solve(g[name + "_A"], g[name + "_b"])
        close(x, g[name + "_x"], TOL_FACT[prec])
    # the reference tests' own expectations (tests/test_mat_solve.c:30-31 ...)
    assert np.allclose(L_.mat_solve(g["solve_2x2_A"], g["solve_2x2_b"]), [1, 2],
                       atol=1e-5)
    assert np.allclose(L_.mat_solve(g["solve_3x3_A"], g["solve_3x3_b"]),
                       [1, 2, 3], atol=1e-4)


@pytest.mark.parametrize("prec", PRECS)
def test_kat_chol_and_spd(gpu, prec):
    L_ = gpu[prec]
    g = golden(f"kat_{prec}.npz")
    for name in ("chol_2x2_identity", "chol_2x2_known", "chol_3x3_known",
                 "chol_not_spd"):
        L, r = L_.mat_chol(g[name + "_A"])
        assert r == g[name + "_r"], name
        if r == 0:
            close(L, g[name + "_L"], TOL_FACT[prec])
            assert np.all(np.triu(L, 1) == 0)
    for name in ("spd_1x1", "spd_identity", "spd_2x2", "spd_3x3", "spd_not_spd"):
        x, r = L_.mat_solve_spd(g[name + "_A"], g[name + "_b"])
        assert r == g[name + "_r"], name
        if r == 0:
            close(x, g[name + "_x"], TOL_FACT[prec])


@pytest.mark.parametrize("prec", PRECS)
def test_kat_tri_and_mul(gpu, prec):
    L_ = gpu[prec]
    g = golden(f"kat_{prec}.npz")
    fns = {"tril_2x2": "mat_solve_tril", "tril_unit_2x2": "mat_solve_tril_unit",
           "triu_2x2": "mat_solve_triu", "trilt_2x2": "mat_solve_trilt",
           "tril_3x3": "mat_solve_tril"}
    for name, fn in fns.items():
        close(getattr(L_, fn)(g[name + "_T"], g[name + "_b"]), g[name + "_x"],
              TOL_FACT[prec])
    for name in ("mul_basic", "mul_identity", "mul_rect", "mul_vector"):
        c = L_.mat_mul(g[name + "_a"], g[name + "_b"])
        assert np.array_equal(c, g[name + "_c"])  # small integers: exact
        assert np.array_equal(L_.mat_rmul(g[name + "_a"], g[name + "_b"]),
                              g[name + "_c"])


# ------------------------------------------- reference random fixtures ----
@pytest.mark.parametrize("prec", PRECS)
def test_reference_random_fixtures(gpu, prec):
    L_ = gpu[prec]
    g = golden(f"rand_{prec}.npz")
    for n in (10, 50, 100):
        L, U, p, s = L_.mat_plu(g[f"plu{n}_A"])
        assert np.array_equal(p, g[f"plu{n}_p"]) and s == g[f"plu{n}_s"]
        close(L, g[f"plu{n}_L"], TOL_FACT[prec])
        close(U, g[f"plu{n}_U"], TOL_FACT[prec])
        close(L_.mat_solve(g[f"solve{n}_A"], g[f"solve{n}_b"]), g[f"solve{n}_x"],
              TOL_FACT[prec])
        x, r = L_.mat_solve_spd(g[f"spd{n}_A"], g[f"spd{n}_b"])
        assert r == 0
        # M M^T + 0.1 I is ill-conditioned; compare through the residual the
        # reference test uses (tests/test_mat_solve_spd.c:140-146).
        A = g[f"spd{n}_A"].astype(np.float64)
        res = np.abs(A @ x - g[f"spd{n}_b"]).max()
        res_ref = np.abs(A @ g[f"spd{n}_x"] - g[f"spd{n}_b"]).max()
        assert res <= max(10 * res_ref, 1e-3 if prec == "f32" else 1e-9)
        close(L_.mat_solve_trilt(g[f"trilt{n}_L"], g[f"trilt{n}_b"]),
              g[f"trilt{n}_x"], TOL_FACT[prec])
    for n in (10, 50, 100, 128, 200):
        L, r = L_.mat_chol(g[f"chol{n}_A"])
        assert r == 0
        close(L, g[f"chol{n}_L"], TOL_FACT[prec])


@pytest.mark.parametrize("prec", PRECS)
def test_c1_plain_256(gpu, prec):
    """Plain small config: mat_mul(A,A), mat_plu(A), mat_solve(A,b) against
    the reference's output; same permutation exactly."""
    L_ = gpu[prec]
    g = golden(f"c1_{prec}.npz")
    L, U, p, s = L_.mat_plu(g["A"])
    assert np.array_equal(p, g["p"]) and s == g["s"]
    close(np.tril(L, -1) + U, g["LU"], TOL_FACT[prec])
    assert np.all(np.diag(L) == 1) and np.all(np.triu(L, 1) == 0)
    assert np.all(np.tril(U, -1) == 0)
    # The solution: kappa(A) ~ 1.3e4 here, so in f32 any backward-stable solve
    # may land up to ~kappa*u from the reference's; the bound is stated in
    # those terms (forward: 10*kappa*u against the reference's x; backward:
    # the normwise backward error at most n*u).
    x = L_.mat_solve(g["A"], g["b"]).astype(np.float64).reshape(-1)
    A64 = g["A"].astype(np.float64)
    b64 = g["b"].astype(np.float64).reshape(-1)
    u = 2.0 ** -24 if prec == "f32" else 2.0 ** -53
    kappa = np.linalg.cond(A64)
    xr = g["x"].astype(np.float64).reshape(-1)
    assert np.abs(x - xr).max() / np.abs(xr).max() <= 10 * kappa * u
    eta = np.abs(b64 - A64 @ x).max() / (np.abs(A64).sum(1).max() * np.abs(x).max()
                                         + np.abs(b64).max())
    assert eta <= A64.shape[0] * u, eta
    close(L_.mat_mul(g["A"], g["A"]), g["AA"], TOL_PROD[prec])


# ------------------------------------------------- against the oracle ----
@pytest.mark.parametrize("prec", PRECS)
@pytest.mark.parametrize("n", [1, 2, 23, 24, 25, 95, 96, 97, 191, 300, 777])
def test_plu_solve_ragged_vs_oracle(gpu, prec, n):
    L_ = gpu[prec]
    O = Oracle(prec)
    A = rng.uniform(3000 + n, (n, n), -1.0, 1.0, O.dtype)
    b = rng.normal(4000 + n, (n,), O.dtype)
    L, U, p, s = L_.mat_plu(A)
    Lr, Ur, pr, sr = O.plu(A)
    assert np.array_equal(p, pr) and s == sr
    tol = TOL_FACT[prec] * max(1.0, n / 256)
    close(L, Lr, tol)
    close(U, Ur, tol)
    x = L_.mat_solve(A, b)
    xr = O.solve(A, b)
    # x's sensitivity grows with cond(A); bound its deviation through the
    # oracle's own f32/f64 spread where that is larger.
    close(x, xr, max(tol, 20 * rel(Oracle("f64").solve(A, b), xr)))


@pytest.mark.parametrize("prec", PRECS)
@pytest.mark.parametrize("n", [1, 5, 31, 32, 33, 96, 97, 250, 513])
def test_chol_spd_ragged_vs_oracle(gpu, prec, n):
    L_ = gpu[prec]
    O = Oracle(prec)
    B = rng.normal(5000 + n, (n, n), np.float64)
    A = (B @ B.T + n * np.eye(n)).astype(O.dtype)
    b = rng.normal(6000 + n, (n,), O.dtype)
    L, r = L_.mat_chol(A)
    Lr, rr = O.chol(A)
    assert r == rr == 0
    close(L, Lr, TOL_FACT[prec] * max(1.0, n / 256))
    x, r = L_.mat_solve_spd(A, b)
    xr, rr = O.solve_spd(A, b)
    assert r == rr == 0
    close(x, xr, TOL_FACT[prec] * max(1.0, n / 256))


@pytest.mark.parametrize("prec", PRECS)
def test_not_spd_returns_minus_one_at_any_block(gpu, prec):
    """mat_chol/mat_solve_spd return -1 (mat.h:5973-5975, 4855-4859) wherever
    the first non-positive pivot sits: first block, later block, last row."""
    L_ = gpu[prec]
    dt = np.float32 if prec == "f32" else np.float64
    for n, bad in ((5, 0), (200, 150), (300, 299)):
        A = np.eye(n, dtype=dt) * 4
        A[bad, bad] = -1.0
        L, r = L_.mat_chol(A)
        assert r == -1
        x, r = L_.mat_solve_spd(A, np.ones(n, dt))
        assert r == -1
    A = np.eye(4, dtype=dt)
    A[2, 2] = np.nan  # NaN passes the "<= 0" test, as in the reference
    _, r = L_.mat_chol(A)
    assert r == Oracle(prec).chol(A)[1] == 0


@pytest.mark.parametrize("prec", PRECS)
@pytest.mark.parametrize("n", [1, 3, 64, 65, 95, 96, 97, 200, 500, 1000, 2049])
def test_tri_solves_vs_oracle(gpu, prec, n):
    L_ = gpu[prec]
    O = Oracle(prec)
    T = rng.uniform(7000 + n, (n, n), -0.5, 0.5, O.dtype)
    T += (np.abs(T).sum(1) + 1).astype(O.dtype)[:, None] * np.eye(n, dtype=O.dtype)
    b = rng.normal(8000 + n, (n,), O.dtype)
    Lo, Up = np.tril(T), np.triu(T)
    tol = TOL_FACT[prec]
    close(L_.mat_solve_tril(Lo, b), O.solve_tril(Lo, b), tol)
    close(L_.mat_solve_tril_unit(Lo, b), O.solve_tril_unit(Lo, b),
          tol * max(1, n / 32))
    close(L_.mat_solve_triu(Up, b), O.solve_triu(Up, b), tol)
    close(L_.mat_solve_trilt(Lo, b), O.solve_trilt(Lo, b), tol)


@pytest.mark.parametrize("prec", PRECS)
@pytest.mark.parametrize("mkn", [(1, 1, 1), (7, 5, 3), (33, 129, 17),
                                 (128, 128, 128), (257, 130, 300), (600, 64, 1000)])
def test_gemm_vs_oracle(gpu, prec, mkn):
    L_ = gpu[prec]
    O = Oracle(prec)
    m, k, n = mkn
    A = rng.normal(11, (m, k), O.dtype)
    B = rng.normal(12, (k, n), O.dtype)
    C0 = rng.normal(13, (m, n), O.dtype)
    tol = TOL_PROD[prec] * max(1.0, k / 256)
    close(L_.mat_gemm(C0, 1.5, A, B, -0.5), O.gemm(1.5, A, B, -0.5, C0), tol)
    close(L_.mat_mul(A, B), O.mul(A, B), tol)
    x = rng.normal(14, (k,), O.dtype)
    y0 = rng.normal(15, (m,), O.dtype)
    close(L_.mat_gemv(y0, 2.0, A, x, 0.5), O.gemv(2.0, A, x, 0.5, y0), tol)


@pytest.mark.parametrize("prec", PRECS)
@pytest.mark.parametrize("nk", [(1, 1), (5, 3), (100, 24), (200, 96), (301, 33)])
def test_syrk_vs_oracle(gpu, prec, nk):
    L_ = gpu[prec]
    O = Oracle(prec)
    n, k = nk
    A = rng.normal(21, (n, k), O.dtype)
    At = np.asfortranarray(A.T)
    C0 = rng.normal(22, (n, n), O.dtype)
    tol = TOL_PROD[prec] * max(1.0, k / 256) * 4
    for up in "LU":
        close(L_.mat_syrk(C0, A, -1.0, 1.0, up), O.syrk(C0, A, -1.0, 1.0, up), tol)
        close(L_.mat_syrk(C0, At, 0.5, 2.0, up, trans=True),
              O.syrk_t(C0, At, 0.5, 2.0, up), tol)


@pytest.mark.parametrize("prec", PRECS)
def test_pivot_rules_match_oracle(gpu, prec):
    """Ties take the first index, a NaN at the top wins, NaN below is ignored,
    tiny pivots are swapped in but not divided by (mat.h:1247-1262, 4235).
    The cases are exact in floating point, so the pivots cannot depend on
    rounding order."""
    L_ = gpu[prec]
    O = Oracle(prec)
    dt = O.dtype
    cases = [np.array([[1, 1], [-1, 2]], dt),
             np.array([[np.nan, 1], [5, 2]], dt),
             np.array([[1, 1], [np.nan, 2]], dt),
             np.array([[1, 2, 3], [2, 4, 6], [4, 8, 13]], dt),
             np.array([[1e-12, 1, 2], [0, 1e-13, 3], [0, 0, 1]], dt),
             np.zeros((4, 4), dt),
             np.array([[2, 1, 1], [-2, 3, 1], [2, -1, 5]], dt)]
    for A in cases:
        L, U, p, s = L_.mat_plu(A)
        Lr, Ur, pr, sr = O.plu(A)
        assert np.array_equal(p, pr) and s == sr, A
        if np.isfinite(A).all():
            assert np.array_equal(L, Lr) and np.array_equal(U, Ur), A


@pytest.mark.parametrize("prec", PRECS)
def test_det_inv(gpu, prec):
    L_ = gpu[prec]
    dt = np.float32 if prec == "f32" else np.float64
    A = np.array([[6, 1, 1], [4, -2, 5], [2, 8, 7]], dt)  # det = -306
    assert abs(L_.mat_det(A) + 306) < 1e-3
    B = np.array([[1, 2, 3, 4], [2, 1, 7, 1], [9, 3, 1, 2], [1, 8, 2, 3]], dt)
    X = L_.mat_inv(B)
    assert np.allclose(B.astype(np.float64) @ X, np.eye(4), atol=1e-4)


@pytest.mark.parametrize("prec", PRECS)
def test_multi_rhs_superset(gpu, prec):
    L_ = gpu[prec]
    O = Oracle(prec)
    n, r = 200, 16
    A = rng.uniform(31, (n, n), -1, 1, O.dtype)
    B = rng.normal(32, (n, r), O.dtype)
    X = L_.solve_multi(A, B)
    for c in range(r):
        close(X[:, c], O.solve(A, B[:, c]), TOL_FACT[prec] * 20)
    S = (A @ A.T + n * np.eye(n)).astype(O.dtype)
    X, ret = L_.solve_multi(S, B, spd=True)
    assert ret == 0
    for c in range(r):
        close(X[:, c], O.solve_spd(S, B[:, c])[0], TOL_FACT[prec])


def test_launch_counter_moves(gpu):
    L_ = gpu["f32"]
    before = L_.launches()
    L_.mat_solve(np.eye(3, dtype=np.float32), np.ones(3, np.float32))
    assert L_.launches() > before
