"""CPU: pin the oracle (C restatement of the reference's scalar path) against
the reference's own outputs -- the committed golden fixtures everywhere, and
the reference compiled in place (oracle/_ref) where its source tree exists."""
import numpy as np
import pytest

from conftest import golden
from oracle.loader import Oracle, available

PRECS = [("f32", np.float32), ("f64", np.float64)]


@pytest.mark.parametrize("prec,dt", PRECS)
def test_port_matches_golden_kat(prec, dt):
    O = Oracle(prec, "port")
    g = golden(f"kat_{prec}.npz")
    for name in ("plu_2x2", "plu_3x3"):
        L, U, p, s = O.plu(g[name + "_A"])
        assert np.array_equal(L, g[name + "_L"]) and np.array_equal(U, g[name + "_U"])
        assert np.array_equal(p, g[name + "_p"]) and s == g[name + "_s"]
    for name in ("solve_1x1", "solve_identity", "solve_2x2", "solve_3x3"):
        assert np.array_equal(O.solve(g[name + "_A"], g[name + "_b"]), g[name + "_x"])
    for name in ("chol_2x2_identity", "chol_2x2_known", "chol_3x3_known",
                 "chol_not_spd"):
        L, r = O.chol(g[name + "_A"])
        assert r == g[name + "_r"] and np.array_equal(L, g[name + "_L"])
    for name in ("spd_1x1", "spd_identity", "spd_2x2", "spd_3x3", "spd_not_spd"):
        x, r = O.solve_spd(g[name + "_A"], g[name + "_b"])
        assert r == g[name + "_r"]
        if r == 0:
            assert np.array_equal(x, g[name + "_x"])
    fns = {"tril_2x2": "solve_tril", "tril_unit_2x2": "solve_tril_unit",
           "triu_2x2": "solve_triu", "trilt_2x2": "solve_trilt",
           "tril_3x3": "solve_tril"}
    for name, fn in fns.items():
        assert np.array_equal(getattr(O, fn)(g[name + "_T"], g[name + "_b"]),
                              g[name + "_x"])
    for name in ("mul_basic", "mul_identity", "mul_rect", "mul_vector"):
        assert np.array_equal(O.mul(g[name + "_a"], g[name + "_b"]), g[name + "_c"])


@pytest.mark.parametrize("prec,dt", PRECS)
def test_golden_kat_meets_reference_test_expectations(prec, dt):
    """The fixtures satisfy the reference tests' own asserts (e.g.
    tests/test_mat_solve.c:30-31 expects x = [1, 2] within 1e-5)."""
    g = golden(f"kat_{prec}.npz")
    assert np.allclose(g["solve_2x2_x"], [1, 2], atol=1e-5)
    assert np.allclose(g["solve_3x3_x"], [1, 2, 3], atol=1e-4)
    assert np.allclose(g["solve_1x1_x"], [3], atol=1e-6)
    assert np.allclose(g["chol_2x2_known_L"], [[2, 0], [1, 2]], atol=1e-5)
    assert g["chol_not_spd_r"] == -1 and g["spd_not_spd_r"] == -1
    assert np.allclose(g["tril_3x3_x"], [1, 2, 3], atol=1e-5)
    assert np.array_equal(g["mul_rect_c"], [[58, 64], [139, 154]])
    for name in ("plu_2x2", "plu_3x3"):
        A, L, U, p = (g[name + s] for s in ("_A", "_L", "_U", "_p"))
        assert np.allclose(A[p], L @ U, atol=1e-5)


@pytest.mark.parametrize("prec,dt", PRECS)
def test_port_matches_golden_random(prec, dt):
    O = Oracle(prec, "port")
    g = golden(f"rand_{prec}.npz")
    for n in (10, 50, 100):
        L, U, p, s = O.plu(g[f"plu{n}_A"])
        assert np.array_equal(L, g[f"plu{n}_L"]) and np.array_equal(U, g[f"plu{n}_U"])
        assert np.array_equal(p, g[f"plu{n}_p"]) and s == g[f"plu{n}_s"]
        assert np.array_equal(O.solve(g[f"solve{n}_A"], g[f"solve{n}_b"]),
                              g[f"solve{n}_x"])
        x, r = O.solve_spd(g[f"spd{n}_A"], g[f"spd{n}_b"])
        assert r == 0 and np.array_equal(x, g[f"spd{n}_x"])
        assert np.array_equal(O.solve_trilt(g[f"trilt{n}_L"], g[f"trilt{n}_b"]),
                              g[f"trilt{n}_x"])
    for n in (10, 50, 100, 128, 200):
        L, r = O.chol(g[f"chol{n}_A"])
        assert r == 0 and np.array_equal(L, g[f"chol{n}_L"])


@pytest.mark.parametrize("prec,dt", PRECS)
def test_port_matches_golden_c1(prec, dt):
    """256x256 plain config (U[-1,1] A, N(0,1) b): bit-exact."""
    O = Oracle(prec, "port")
    g = golden(f"c1_{prec}.npz")
    L, U, p, s = O.plu(g["A"])
    assert np.array_equal(np.tril(L, -1) + U, g["LU"])
    assert np.array_equal(p, g["p"]) and s == g["s"]
    assert np.array_equal(O.solve(g["A"], g["b"]), g["x"])
    assert np.array_equal(O.mul(g["A"], g["A"]), g["AA"])


@pytest.mark.skipif(not available("f32", "ref"),
                    reason="reference source tree not present on this host")
@pytest.mark.parametrize("prec,dt", PRECS)
def test_port_matches_reference_live(prec, dt):
    """Bit-exact against the reference compiled from its own header, on
    ragged sizes that straddle its 24-column LU blocks."""
    P, R = Oracle(prec, "port"), Oracle(prec, "ref")
    rs = np.random.default_rng(7)
    for n in (1, 2, 5, 23, 24, 25, 47, 49, 97):
        A = rs.uniform(-1, 1, (n, n)).astype(dt)
        b = rs.standard_normal(n).astype(dt)
        a1, a2 = P.plu(A), R.plu(A)
        for u, v in zip(a1, a2):
            assert np.array_equal(u, v)
        assert np.array_equal(P.solve(A, b), R.solve(A, b))
        S = (A @ A.T + n * np.eye(n)).astype(dt)
        assert np.array_equal(P.chol(S)[0], R.chol(S)[0])
        assert np.array_equal(P.solve_spd(S, b)[0], R.solve_spd(S, b)[0])
        C = rs.standard_normal((n, n)).astype(dt)
        for up in "LU":
            assert np.array_equal(P.syrk(C, A, -1.0, 1.0, up), R.syrk(C, A, -1.0, 1.0, up))
            assert np.array_equal(P.syrk_t(C, A, 2.0, 0.5, up),
                                  R.syrk_t(C, A, 2.0, 0.5, up))
        assert np.array_equal(P.gemm(1.5, A, C, 0.5, C), R.gemm(1.5, A, C, 0.5, C))
        assert np.array_equal(P.gemv(1.0, A, b, 0.0, b), R.gemv(1.0, A, b, 0.0, b))


@pytest.mark.parametrize("prec,dt", PRECS)
def test_port_pivot_rules(prec, dt):
    """Edge cases of the reference's pivot rule (mat.h:1247-1262, 4235): first
    index on ties, NaN at the top wins, NaN below is ignored, tiny pivots are
    swapped in but not divided by."""
    O = Oracle(prec, "port")
    A = np.array([[1, 1], [-1, 2]], dt)        # |1| == |-1|: keep row 0
    _, _, p, s = O.plu(A)
    assert list(p) == [0, 1] and s == 0
    A = np.array([[np.nan, 1], [5, 2]], dt)    # NaN at the top: pivot 0
    _, _, p, _ = O.plu(A)
    assert list(p) == [0, 1]
    A = np.array([[1, 1], [np.nan, 2]], dt)    # NaN below: ignored
    _, _, p, _ = O.plu(A)
    assert list(p) == [0, 1]
    A = np.array([[1, 2, 3], [2, 4, 6], [3, 6, 10]], dt)  # singular minor
    M, p, ipiv, s = O.plu_inplace(A)
    assert list(ipiv) == [2, 2, 2] or ipiv[0] == 2


@pytest.mark.parametrize("prec,dt", PRECS)
def test_port_full_pivot_lu_matches_reference_live(prec, dt):
    """mat_lu (full pivoting, mat.h:4476-4574) bit-exact against the reference
    compiled in place: the reference tests' matrices, tie-heavy inputs in
    steps of 0.1 (test_mat_lu.c's generator), Gaussian inputs, a zero matrix
    (every step below eps) and a NaN entry."""
    if not available(prec, "ref"):
        pytest.skip("reference source tree not present")
    P, R = Oracle(prec, "port"), Oracle(prec, "ref")
    rs = np.random.default_rng(11)
    cases = [np.array([[2, -1, -2], [-4, 6, 3], [-4, -2, 8]], dt),
             np.array([[4, 3, 2, 1], [3, 4, 3, 2], [2, 3, 4, 3], [1, 2, 3, 4]], dt),
             np.zeros((5, 5), dt), np.ones((1, 1), dt)]
    for n in (2, 10, 37, 50, 100):
        cases.append((rs.integers(0, 200, (n, n)) - 100).astype(dt) / dt(10))
        cases.append(rs.standard_normal((n, n)).astype(dt))
    nan = rs.standard_normal((6, 6)).astype(dt)
    nan[3, 2] = np.nan
    cases.append(nan)
    for A in cases:
        a1, a2 = P.lu(A), R.lu(A)
        for u, v in zip(a1[:4], a2[:4]):
            assert np.array_equal(u, v, equal_nan=True), A.shape
        assert a1[4] == a2[4]


@pytest.mark.parametrize("prec,dt", PRECS)
def test_port_full_pivot_lu_matches_golden(prec, dt):
    """The port against the committed mat_lu fixtures (made from the reference
    compiled in place): test_mat_lu.c's known-answer and random matrices and
    test_mat_plu.c's determinant matrix.  Also the reference tests' own
    checks: P A Q = L U within their tolerance and unit-diagonal L."""
    g = golden(f"lu_{prec}.npz")
    P = Oracle(prec, "port")
    names = sorted({k[:-2] for k in g if k.endswith("_A")})
    assert len(names) == 6
    for name in names:
        A = g[name + "_A"]
        L, U, p, q, s = P.lu(A)
        assert np.array_equal(L, g[name + "_L"]), name
        assert np.array_equal(U, g[name + "_U"]), name
        assert np.array_equal(p, g[name + "_p"]), name
        assert np.array_equal(q, g[name + "_q"]), name
        assert s == int(g[name + "_s"]), name
        n = A.shape[0]
        PAQ = A.astype(np.float64)[p][:, q]
        LU = L.astype(np.float64) @ U.astype(np.float64)
        tol = 1e-3 if prec == "f32" else 1e-9
        assert np.max(np.abs(PAQ - LU)) <= tol * max(1.0, np.abs(A).max()) * n
        assert np.all(np.diag(L) == 1)


@pytest.mark.parametrize("prec,dt", PRECS)
def test_vectorised_full_pivot_lu_matches_port(prec, dt):
    """The vectorised restatement used at large sizes by the GPU tests
    (tests/lu_full_np.py) is bit-identical to the scalar port: tie-heavy,
    Gaussian, zero (every step skipped), NaN and infinity inputs."""
    from lu_full_np import lu_full_np, perms
    P = Oracle(prec, "port")
    eps = dt(1e-6) if prec == "f32" else 1e-9
    rs = np.random.default_rng(5)
    cases = [np.zeros((4, 4), dt), np.ones((1, 1), dt)]
    for n in (2, 3, 17, 64, 65, 130):
        cases.append((rs.integers(0, 200, (n, n)) - 100).astype(dt) / dt(10))
        cases.append(rs.standard_normal((n, n)).astype(dt))
    odd = rs.standard_normal((9, 9)).astype(dt)
    odd[0, 0], odd[4, 7], odd[2, 2] = np.nan, np.inf, dt(1e-7)
    cases.append(odd)
    odd2 = odd.copy()
    odd2[0, 0] = 0
    cases.append(odd2)
    for A in cases:
        n = A.shape[0]
        L, U, p, q, s = P.lu(A)
        M, rp, cp, s2 = lu_full_np(A, eps)
        p2, q2 = perms(rp, cp)
        assert np.array_equal(L, np.tril(M, -1) + np.eye(n, dtype=dt),
                              equal_nan=True), n
        assert np.array_equal(U, np.triu(M), equal_nan=True), n
        assert np.array_equal(p, p2) and np.array_equal(q, q2) and s == s2


@pytest.mark.parametrize("prec,dt", PRECS)
def test_port_gemv_t_axpy_match_reference_live(prec, dt):
    """mat_gemv_t (mat.h:2224-2248) and mat_axpy (2009-2015) bit-exact
    against the reference compiled in place, on ragged shapes, with beta 0,
    1 and other values, and NaN / infinity entries."""
    if not available(prec, "ref"):
        pytest.skip("reference source tree not present")
    P, R = Oracle(prec, "port"), Oracle(prec, "ref")
    rs = np.random.default_rng(17)
    for m, n in ((1, 1), (7, 3), (64, 65), (257, 31), (1000, 9)):
        A = rs.standard_normal((m, n)).astype(dt)
        x = rs.standard_normal(m).astype(dt)
        y = rs.standard_normal(n).astype(dt)
        for alpha, beta in ((1.0, 0.0), (-0.75, 1.0), (2.5, -0.5)):
            assert np.array_equal(P.gemv_t(alpha, A, x, beta, y),
                                  R.gemv_t(alpha, A, x, beta, y))
        v = rs.standard_normal(m).astype(dt)
        v[0] = np.nan if m > 1 else v[0]
        for alpha in (0.0, 1.0, -3.25):
            assert np.array_equal(P.axpy(v, alpha, x), R.axpy(v, alpha, x),
                                  equal_nan=True)
    A = rs.standard_normal((5, 4)).astype(dt)
    A[2, 1] = np.inf
    x = rs.standard_normal(5).astype(dt)
    assert np.array_equal(P.gemv_t(1.0, A, x, 0.0, np.zeros(4, dt)),
                          R.gemv_t(1.0, A, x, 0.0, np.zeros(4, dt)), equal_nan=True)


@pytest.mark.parametrize("prec,dt", PRECS)
def test_port_qr_matches_reference_live(prec, dt):
    """mat_qr (mat.h:3907-4064): the port restates the reference's unblocked
    path, which the reference itself takes below 64 columns -- identical
    there; from 64 columns the reference applies 16-column WY blocks, and the
    two agree within 64 * n * u of max|.| (summation order only).  Also
    test_mat_qr.c's checks on its matrices: Q orthogonal, R upper
    triangular within m * eps, Q R = A."""
    if not available(prec, "ref"):
        pytest.skip("reference source tree not present")
    P, R_ = Oracle(prec, "port"), Oracle(prec, "ref")
    rs = np.random.default_rng(23)
    u = np.finfo(dt).eps
    kats = [np.array([[12, -51, 4], [6, 167, -68], [-4, 24, -41]], dt),
            np.arange(1, 13, dtype=dt).reshape(4, 3), np.eye(3, dtype=dt),
            np.zeros((4, 2), dt)]
    for A in kats + [rs.standard_normal(s).astype(dt)
                     for s in ((1, 1), (5, 3), (10, 10), (63, 40), (100, 63))]:
        q1, r1 = P.qr(A)
        q2, r2 = R_.qr(A)
        assert np.array_equal(q1, q2) and np.array_equal(r1, r2), A.shape
    for s in ((64, 64), (130, 100)):
        A = rs.standard_normal(s).astype(dt)
        (q1, r1), (q2, r2) = P.qr(A), R_.qr(A)
        tol = 64 * s[1] * u
        assert np.abs(q1 - q2).max() <= tol * np.abs(q2).max(), s
        assert np.abs(r1 - r2).max() <= tol * np.abs(r2).max(), s
    eps = 1e-6 if prec == "f32" else 1e-9
    for A in kats[:3]:
        Q, R = P.qr(A)
        m = A.shape[0]
        assert np.abs(Q.T.astype(np.float64) @ Q - np.eye(m)).max() <= 1e-5
        assert np.abs(np.tril(R, -1)).max(initial=0) <= m * eps
        assert np.abs(Q.astype(np.float64) @ R - A).max() <= 1e-4
