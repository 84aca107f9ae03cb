"""CPU experiment: can the mixed SPD solve take its SYRK trailing updates in
FP8 (E4M3) with per-tile scaling, for A = Q diag(lambda) Q^T with lambda
log-uniform in [1, 1e3]?  (The Cholesky of mat.h:5988-6027, SYRK update at
6021-6023, in the blocked right-looking form the GPU uses: 128-column
blocks, FP32 panels and trailing matrix, only the update operand L21 in low
precision.)

E4M3 is emulated exactly in numpy (3 mantissa bits, exponent bias 7,
subnormal quantum 2^-9, round to nearest even, saturation at 448); each
128 x 128 tile of L21 is scaled by a power of two bringing its largest
magnitude just under 448 before rounding.  The products accumulate in FP32,
as the tensor cores do; refinement runs in FP64.

Findings (n = 2048 and 1024, asserted below):
  * one FP8 product per update (the "FP8 with per-tile scaling" form): the
    FP32 Schur complement loses definiteness -- the factorisation stops
    with a pivot <= 0 three quarters of the way through.  Quantising only
    the tiles at least four tiles away from the diagonal fails the same way
    (A is dense: its far tiles are as large as its near ones).  With
    u(E4M3) = 2^-4, the update error ~ u * lambda_max ~ 60 exceeds
    lambda_min = 1;
  * FP8 with a diagonal shift (factor A + 6.25 I): definite, but classic
    refinement stagnates (kappa * u ~ 60) and GMRES-IR needs ~46 Krylov
    steps, against 3 with the FP16 split factors;
  * the FP8 split (hi + remainder, three FP8 products): definite and
    refinable, but 9-10 classic refinement steps against 2 for the FP16
    split (the library's form).
The update is bound by HBM (the FP32 trailing matrix is read and written
once per block; the 16-bit operands are a few percent of those bytes), so
FP8 operands would shorten the factorisation by at most a few percent while
every extra refinement step of the 64-right-hand-side solve costs a full
residual and two triangular solves.  The library therefore keeps the FP16
split for both SPD workloads.
"""
import numpy as np
import pytest

sl = pytest.importorskip("scipy.linalg")
spla = pytest.importorskip("scipy.sparse.linalg")

NB = 128


def e4m3(x):
    """Round to the nearest FP8 E4M3 value (ties to even, saturating)."""
    a = np.abs(x)
    e = np.maximum(np.floor(np.log2(np.maximum(a, 2.0 ** -9))), -6)
    q = 2.0 ** (e - 3)
    return np.sign(x) * np.minimum(np.round(a / q) * q, 448.0)


def quant_tiles(L21, far_from=None):
    """E4M3 per 128 x 128 tile under a power-of-two scale; far_from: leave
    tiles whose row offset from the block is below far_from tiles in FP32."""
    out = L21.astype(np.float64).copy()
    for i in range(0, L21.shape[0], NB):
        if far_from is not None and i < far_from * NB:
            continue
        T = out[i:i + NB]
        mx = np.abs(T).max()
        if mx > 0:
            s = 2.0 ** np.floor(np.log2(448.0 / mx))
            out[i:i + NB] = e4m3(T * s) / s
    return out


def fp16(x):
    return x.astype(np.float16).astype(np.float64)


def cholesky_lp(A, form, shift=0.0):
    """Blocked Cholesky with FP32 panels and trailing matrix; returns (L,
    None) or (None, first failing block column)."""
    n = A.shape[0]
    W = (A + shift * np.eye(n)).astype(np.float32)
    for kb in range(0, n, NB):
        ke = min(kb + NB, n)
        try:
            L11 = np.linalg.cholesky(W[kb:ke, kb:ke].astype(np.float64))
        except np.linalg.LinAlgError:
            return None, kb
        W[kb:ke, kb:ke] = L11
        if ke == n:
            break
        L21 = sl.solve_triangular(L11, W[ke:, kb:ke].T.astype(np.float64),
                                  lower=True).T.astype(np.float32)
        W[ke:, kb:ke] = L21
        if form == "fp16_split":
            s = 2.0 ** np.floor(np.log2(32768.0 / np.abs(L21).max()))
            h = fp16(L21 * s)
            lo = fp16(L21 * s - h)
            upd = (h @ h.T + h @ lo.T + lo @ h.T) / (s * s)
        elif form == "fp8":
            q = quant_tiles(L21)
            upd = q @ q.T
        elif form == "fp8_far":
            q = quant_tiles(L21, far_from=4)
            upd = q @ q.T
        elif form == "fp8_split":
            h = quant_tiles(L21)
            lo = quant_tiles((L21 - h).astype(np.float32))
            upd = h @ h.T + h @ lo.T + lo @ h.T
        else:
            raise ValueError(form)
        W[ke:, ke:] -= upd.astype(np.float32)
    return np.tril(W), None


def classic_ir(A, b, L, maxit=30):
    n = A.shape[0]
    L64 = L.astype(np.float64)
    an, bn, tol = np.abs(A).sum(1).max(), np.abs(b).max(), n * 2.0 ** -53
    x = np.zeros(n)
    for it in range(maxit):
        r = b - A @ x
        if np.abs(r).max() / (an * np.abs(x).max() + bn) <= tol:
            return it
        x += sl.solve_triangular(L64, sl.solve_triangular(L64, r, lower=True),
                                 lower=True, trans="T")
    return None


def gmres_steps(A, b, L):
    """Krylov steps of one GMRES(50) cycle preconditioned by L L^T, to a
    relative residual of 1e-14."""
    n = A.shape[0]
    L64 = L.astype(np.float64)
    M = spla.LinearOperator((n, n), matvec=lambda r: sl.solve_triangular(
        L64, sl.solve_triangular(L64, r, lower=True), lower=True, trans="T"))
    its = [0]
    spla.gmres(A, b, M=M, rtol=1e-14, restart=50, maxiter=1,
               callback=lambda _: its.__setitem__(0, its[0] + 1),
               callback_type="pr_norm")
    return its[0]


@pytest.fixture(scope="module")
def spd_1e3():
    n = 2048
    rs = np.random.default_rng(2048)
    Q, _ = np.linalg.qr(rs.standard_normal((n, n)))
    lam = np.exp(rs.uniform(0, np.log(1e3), n))
    A = (Q * lam) @ Q.T
    return (A + A.T) / 2, rs.standard_normal(n)


def test_fp8_per_tile_update_loses_definiteness(spd_1e3):
    A, _ = spd_1e3
    for form in ("fp8", "fp8_far"):
        L, fail = cholesky_lp(A, form)
        assert L is None, form
        assert A.shape[0] // 2 <= fail < A.shape[0], (form, fail)


def test_fp16_split_refines_in_two_steps(spd_1e3):
    A, b = spd_1e3
    L, fail = cholesky_lp(A, "fp16_split")
    assert fail is None
    assert classic_ir(A, b, L) <= 2
    assert gmres_steps(A, b, L) <= 4


def test_fp8_alternatives_cost_many_more_refinement_steps(spd_1e3):
    A, b = spd_1e3
    L, fail = cholesky_lp(A, "fp8_split")
    assert fail is None
    assert classic_ir(A, b, L) >= 6
    L, fail = cholesky_lp(A, "fp8", shift=6.25)
    assert fail is None
    assert classic_ir(A, b, L) is None  # stagnates
    assert gmres_steps(A, b, L) >= 30
