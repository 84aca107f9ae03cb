"""GPU parity at the 8192 plain config (float PLU + 16-right-hand-side solve,
and the float GEMM at 2048^3), through the C ABI.

The oracle here is the reference itself: tests/golden/c2_8192.npz holds the
reference's float mat_plu permutation and swap count on A ~ N(0,1) 8192 x 8192
(seed 1002, regenerated from libmat_gb300.rng), its float solutions (PLU once,
then the public mat_solve_tril_unit / mat_solve_triu per column on B[p]) and
its double solutions of the same system (the FP64 oracle of the forward
error), with kappa_inf(A) from LAPACK's dgecon.

Criteria (max-norm, per column, stated here once):
  * float permutation: identical to the reference's float permutation on
    every step where the reference's pivots are set by the data rather than
    by its rounding -- the steps before the first one where the reference's
    own float and double factorisations pick different rows (step 8116 of
    8192 on this matrix: there the float Schur complement is rounding noise,
    its two candidates 15% apart in magnitude but both below the noise
    level).  A complete match is reported, and then the swap count must
    match too;
  * double permutation: identical to the reference's double permutation
    (which LAPACK's dgetrf reproduces exactly);
  * normwise backward error eta <= n * u32 (u32 = 2^-24);
  * forward error against the reference's double solution:
      fe <= 2 * kappa_inf * eta           (the first-order bound), and
      fe <= 10 * fe_ref                   (no worse than 10x the reference's
                                           own float solve on the same system);
  * the double build: the same, with u64 and the reference's double
    permutation.
GEMM 2048^3 (float): rows 0..63 of C against the oracle (the reference's
scalar product) and all of C against an FP64 product, both within the parity
suite's product bound 2e-5 * K/256 relative to max |C|.
"""
import os

import numpy as np
import pytest

from conftest import GOLDEN
from libmat_gb300 import rng
from oracle.loader import Oracle

pytestmark = pytest.mark.gpu

N, NRHS, SEED_A, SEED_B = 8192, 16, 1002, 2002
U = {"f32": 2.0 ** -24, "f64": 2.0 ** -53}


@pytest.fixture(scope="module")
def c2():
    with np.load(os.path.join(GOLDEN, "c2_8192.npz")) as z:
        g = {k: z[k] for k in z.files}
    assert int(g["seed_A"]) == SEED_A and int(g["seed_B"]) == SEED_B
    A = rng.normal(SEED_A, (N, N), np.float32)
    B = rng.normal(SEED_B, (N, NRHS), np.float32)
    return g, A, B


def gpu_plu_solve(L, A, B):
    """matgb_getrf_dev + matgb_getrs_dev on the device: (perm, swaps, LU, X)."""
    dt = L.dtype
    A = np.asfortranarray(A, dtype=dt)
    B = np.asfortranarray(B, dtype=dt)
    n, nrhs = B.shape
    dA, dB, dX = L.dalloc(A.nbytes), L.dalloc(B.nbytes), L.dalloc(B.nbytes)
    dp = L.dalloc(8 * n)
    try:
        L.h2d(dA, A)
        L.h2d(dB, B)
        L.check(L.c.matgb_getrf_dev(n, dA, n, dp, dp + 4 * n), "getrf")
        L.check(L.c.matgb_getrs_dev(n, nrhs, dA, n, dp + 4 * n, dB, n, dX, n),
                "getrs")
        piv = np.empty(2 * n, np.int32)
        L.d2h(piv, dp)
        LU = np.empty((n, n), dt, order="F")
        L.d2h(LU, dA)
        X = np.empty((n, nrhs), dt, order="F")
        L.d2h(X, dX)
    finally:
        for p in (dA, dB, dX, dp):
            L.dfree(p)
    ipiv, perm = piv[:n], piv[n:]
    swaps = int(np.sum(ipiv != np.arange(n)))
    return perm, swaps, LU, X


def bwd_err(A64, X, B):
    R = B - A64 @ X
    return np.abs(R).max(0) / (np.abs(A64).sum(1).max() * np.abs(X).max(0)
                               + np.abs(B).max(0))


def fwd_err(X, Xt):
    return np.abs(np.asarray(X, np.float64) - Xt).max(0) / np.abs(Xt).max(0)


def first_step_tie(A64, LU, perm, ref_perm):
    """At the first step k where the permutations differ: the relative gap
    between the magnitudes of the GPU's pivot and the reference's, both taken
    from the GPU's own Schur complement column k (rows of A in original
    numbering)."""
    k = int(np.nonzero(perm != ref_perm)[0][0])
    r_gpu, r_ref = int(perm[k]), int(ref_perm[k])
    Lk = np.tril(LU[:, :k].astype(np.float64), -1)  # rows in pivoted order
    uk = np.triu(LU[:k, k:k + 1].astype(np.float64))[:, 0]
    pos = np.empty(len(perm), np.int64)
    pos[perm] = np.arange(len(perm))  # original row -> position
    s = lambda r: A64[r, k] - Lk[pos[r]] @ uk if k else A64[r, k]  # noqa: E731
    a, b = abs(s(r_gpu)), abs(s(r_ref))
    return k, abs(a - b) / max(a, b, 1e-300)


@pytest.mark.parametrize("prec", ["f32", "f64"])
def test_c2_plu_solve_8192_vs_reference(gpu, c2, prec):
    g, A, B = c2
    L = gpu[prec]
    perm, swaps, LU, X = gpu_plu_solve(L, A, B)
    ref_perm = g[f"p_{prec}"].astype(np.int64)
    A64 = A.astype(np.float64)
    B64 = B.astype(np.float64)
    if prec == "f32":
        # steps whose pivots the data determines (see the module docstring)
        det = int(np.nonzero(g["p_f32"] != g["p_f64"])[0][0])
        assert det > N * 0.9, det
        assert np.array_equal(perm[:det], ref_perm[:det]), \
            f"first difference at step {int(np.nonzero(perm != ref_perm)[0][0])}"
        if np.array_equal(perm, ref_perm):
            assert swaps == int(g["s_f32"])
            print("f32: permutation identical to the reference's on all steps")
        else:
            k, gap = first_step_tie(A64, LU, perm, ref_perm)
            print(f"f32: permutation identical on the {det} data-determined "
                  f"steps; differs first at step {k} (relative gap {gap:.1e})")
    else:
        assert np.array_equal(perm, ref_perm)
        assert swaps == int(g["s_f64"])
    kappa = float(g["kappa_inf_est"])
    eta = bwd_err(A64, X.astype(np.float64), B64)
    assert eta.max() <= N * U[prec], eta.max()
    xt = g["x_f64"]
    fe = fwd_err(X, xt)
    assert np.all(fe <= 2 * kappa * np.maximum(eta, U[prec])), (fe.max(), kappa)
    if prec == "f32":
        fe_ref = fwd_err(g["x_f32"], xt)
        assert np.all(fe <= 10 * fe_ref), (fe / fe_ref).max()
    print(f"{prec}: kappa_inf~{kappa:.2e} eta<={eta.max():.2e} "
          f"fe<={fe.max():.2e}")


def test_c2_gemm_2048_vs_oracle(gpu):
    L = gpu["f32"]
    O = Oracle("f32")
    n = 2048
    A = rng.normal(1012, (n, n), np.float32)
    Bm = rng.normal(1013, (n, n), np.float32)
    Cg = L.mat_mul(A, Bm)
    exact = A.astype(np.float64) @ Bm.astype(np.float64)
    tol = 2e-5 * max(1.0, n / 256)
    scale = np.abs(exact).max()
    assert np.abs(Cg - exact).max() / scale <= tol
    rows = 64
    Co = O.mul(A[:rows], Bm)
    assert np.abs(Cg[:rows] - Co).max() / np.abs(Co).max() <= tol
