"""GPU parity of mat_qr / mat_qr_r / matgb_qr_dev (Householder QR, blocked WY)
against the oracle (the reference's Householder path restated, pinned to the
reference in tests/test_oracle.py), through the C ABI.

Criteria (max-norm, relative to max|ref|):
  * tall matrices (m >= 2n, condition number below ~6): Q and R's upper
    triangle within the parity suite's factor bound (f32 2e-4, f64 1e-11);
    R's entries below the diagonal (rounding residue in both) below that
    bound times max|R|;
  * square matrices (condition ~n, where two Householder QRs in different
    summation orders differ by ~cond * u): the backward-stable properties
    |QR - A| <= 30 n u |A| and |Q^T Q - I| <= 30 n u, and diag(R) with the
    reference's signs (beta = -sign(a_jj) |x|);
  * mat_qr_r's R identical to mat_qr's (the same reflections);
  * a column below MAT_DEFAULT_EPSILON takes no reflection, as there.
"""
import numpy as np
import pytest

from libmat_gb300 import rng
from oracle.loader import Oracle

pytestmark = pytest.mark.gpu

PRECS = ["f32", "f64"]
TOL = {"f32": 2e-4, "f64": 1e-11}
U = {"f32": 2.0 ** -24, "f64": 2.0 ** -53}


def rel(got, ref):
    ref = np.asarray(ref, np.float64)
    return np.abs(np.asarray(got, np.float64) - ref).max() / max(np.abs(ref).max(), 1e-300)


@pytest.mark.parametrize("prec", PRECS)
@pytest.mark.parametrize("mn", [(1, 1), (5, 3), (64, 32), (100, 33), (300, 100),
                                (513, 200), (1100, 300)])
def test_qr_tall_vs_oracle(gpu, prec, mn):
    L = gpu[prec]
    O = Oracle(prec)
    m, n = mn
    A = rng.normal(71 + m + n, (m, n), O.dtype)
    Q, R = L.mat_qr(A)
    Qo, Ro = O.qr(A)
    tol = TOL[prec]
    assert rel(Q, Qo) <= tol
    assert rel(np.triu(R), np.triu(Ro)) <= tol
    below = np.tril(R, -1)
    assert np.abs(below).max(initial=0.0) <= tol * np.abs(Ro).max()
    R2 = L.mat_qr(A, want_q=False)
    assert np.array_equal(R2, R)


@pytest.mark.parametrize("prec", PRECS)
@pytest.mark.parametrize("n", [256, 600])
def test_qr_square_properties(gpu, prec, n):
    L = gpu[prec]
    A = rng.uniform(81 + n, (n, n), -1.0, 1.0, np.float32 if prec == "f32" else np.float64)
    Q, R = L.mat_qr(A)
    A64, Q64, R64 = (x.astype(np.float64) for x in (A, Q, np.triu(R)))
    bound = 30 * n * U[prec]
    assert np.abs(Q64 @ R64 - A64).max() / np.abs(A64).max() <= bound
    assert np.abs(Q64.T @ Q64 - np.eye(n)).max() <= bound
    # the reference's sign convention: R_jj = beta_j = -sign(x0) |x|
    O = Oracle(prec)
    _, Ro = O.qr(A[:, :8])
    assert np.array_equal(np.sign(np.diag(R)[:8]), np.sign(np.diag(Ro)))


@pytest.mark.parametrize("prec", PRECS)
def test_qr_small_column_and_device_entry(gpu, prec):
    """A column that is zero below the processed rows takes no reflection
    (|x| < MAT_DEFAULT_EPSILON); the device entry with ldr, ldq > m."""
    L = gpu[prec]
    O = Oracle(prec)
    dt = O.dtype
    m, n = 70, 40
    A = rng.normal(91, (m, n), dt)
    A[:, 5] = 0
    A[:, 17] = 1e-12
    Q, R = L.mat_qr(A)
    Qo, Ro = O.qr(A)
    assert rel(Q, Qo) <= TOL[prec]
    assert rel(np.triu(R), np.triu(Ro)) <= TOL[prec]
    ld = m + 9
    Rp = np.zeros((ld, n), dt, order="F")
    Rp[:m] = A
    Qp = np.zeros((ld, m), dt, order="F")
    dR, dQ = L.dalloc(Rp.nbytes), L.dalloc(Qp.nbytes)
    try:
        L.h2d(dR, Rp)
        L.h2d(dQ, Qp)
        L.check(L.c.matgb_qr_dev(m, n, dR, ld, dQ, ld), "qr_dev")
        L.d2h(Rp, dR)
        L.d2h(Qp, dQ)
    finally:
        L.dfree(dR)
        L.dfree(dQ)
    assert np.array_equal(Rp[:m], R) and np.array_equal(Qp[:m], Q)
    assert L.c.matgb_qr_dev(3, 5, None, 3, None, 3) == -2  # m < n
    L.c.matgb_clear_error()
