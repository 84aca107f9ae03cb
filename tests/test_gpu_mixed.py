"""GPU: the tensor-core rank-K update (tcgen05/TMEM/TMA) and the
mixed-precision LU + iterative refinement, through the C ABI.

Tolerances:
  tc_gemm: FP32 accumulation of exactly representable 16-bit products;
           max |err| <= 2e-6 * K * max|ref| against an FP64 product of the
           same rounded inputs.
  LU factors with 16-bit trailing updates: within 3x of a numpy model of the
           same rounding (BF16, FP16) or of FP32 (the FP16 split, FP32).
  tc_gemm split: the three products exact to the FP32 accumulation bound,
           and within 1e-5 + 2e-7 K of the unsplit FP32 product.
  Refined solutions: normwise backward error <= n * 2^-53 (libmatgb_f64) or
           n * 2^-24 (libmatgb_f32), the refinement target.
"""
import ctypes as C

import numpy as np
import pytest

from libmat_gb300 import MatIRReport, rng

pytestmark = pytest.mark.gpu


def to_bf16_bits(x):
    b = np.ascontiguousarray(x, np.float32).view(np.uint32).astype(np.uint64)
    b = (b + 0x7FFF + ((b >> 16) & 1)) >> 16
    return b.astype(np.uint16)


def bf16_bits_to_f64(b):
    return (b.astype(np.uint32) << 16).view(np.float32).astype(np.float64)


def lp_pack(x, bf16):
    """Row-major (K contiguous) 16-bit operand and its exact float64 value."""
    x = np.ascontiguousarray(x, np.float32)
    if bf16:
        bits = to_bf16_bits(x)
        return bits, bf16_bits_to_f64(bits)
    h = x.astype(np.float16)
    return h.view(np.uint16), h.astype(np.float64)


@pytest.mark.parametrize("bf16", [1, 0])
@pytest.mark.parametrize("mnk", [(128, 256, 64), (200, 300, 128), (1000, 700, 128),
                                 (1, 1, 64), (129, 257, 64), (4096, 512, 128)])
def test_tc_gemm_vs_fp64(gpu, bf16, mnk):
    L = gpu["f32"]
    M, N, K = mnk
    A = rng.normal(101, (M, K), np.float32)
    B = rng.normal(102, (N, K), np.float32)
    C0 = rng.normal(103, (M, N), np.float32)
    Ab, Ad = lp_pack(A, bf16)
    Bb, Bd = lp_pack(B, bf16)
    ref = C0.astype(np.float64) - 0.75 * (Ad @ Bd.T)
    dA, dB = L.dalloc(Ab.nbytes), L.dalloc(Bb.nbytes)
    dC = L.dalloc(C0.nbytes)
    try:
        L.h2d(dA, Ab)
        L.h2d(dB, Bb)
        L.h2d(dC, C0)
        rc = L.c.matgb_tc_gemm_dev(bf16, M, N, K, dA, K, dB, K, -0.75, 1.0,
                                   dC, M)
        L.check(rc, "tc_gemm")
        out = np.empty((M, N), np.float32, order="F")
        L.d2h(out, dC)
        L.check(L.c.matgb_tc_status(), "tc_status")
    finally:
        for p in (dA, dB, dC):
            L.dfree(p)
    err = np.abs(out - ref).max() / np.abs(ref).max()
    assert err <= 2e-6 * K, err


@pytest.mark.parametrize("mnk", [(128, 256, 64), (1000, 700, 128), (129, 257, 64),
                                 (2048, 1024, 128), (300, 500, 256)])
def test_tc_gemm_split_vs_fp64(gpu, mnk):
    """Three-product FP16 split: exact for the split operands (FP32
    accumulation bound) and FP32-level against the unsplit FP32 product."""
    L = gpu["f32"]
    M, N, K = mnk
    A = rng.normal(111, (M, K), np.float32)
    B = rng.normal(112, (N, K), np.float32)
    C0 = rng.normal(113, (M, N), np.float32)
    Ah = A.astype(np.float16)
    Al = (A - Ah.astype(np.float32)).astype(np.float16)
    Bh = B.astype(np.float16)
    Bl = (B - Bh.astype(np.float32)).astype(np.float16)
    f = lambda x: x.astype(np.float64)
    ref = C0.astype(np.float64) - 0.75 * (f(Ah) @ f(Bh).T + f(Ah) @ f(Bl).T +
                                          f(Al) @ f(Bh).T)
    true = C0.astype(np.float64) - 0.75 * (f(A) @ f(B).T)
    bufs = [L.dalloc(x.nbytes) for x in (Ah, Al, Bh, Bl, C0)]
    try:
        for d, x in zip(bufs, (Ah, Al, Bh, Bl)):
            L.h2d(d, np.ascontiguousarray(x).view(np.uint16))
        L.h2d(bufs[4], C0)
        rc = L.c.matgb_tc_gemm_split_dev(M, N, K, bufs[0], bufs[1], K, bufs[2],
                                         bufs[3], K, -0.75, 1.0, bufs[4], M)
        L.check(rc, "tc_gemm_split")
        out = np.empty((M, N), np.float32, order="F")
        L.d2h(out, bufs[4])
        L.check(L.c.matgb_tc_status(), "tc_status")
    finally:
        for d in bufs:
            L.dfree(d)
    scale = np.abs(ref).max()
    assert np.abs(out - ref).max() / scale <= 2e-6 * K
    assert np.abs(out - true).max() / scale <= 1e-5 + 2e-7 * K


def factor_lp(L, A, lp):
    n = A.shape[0]
    dA = L.dalloc(A.nbytes)
    dp = L.dalloc(8 * n)
    try:
        L.h2d(dA, np.asfortranarray(A, np.float32))
        L.check(L.c.matgb_getrf_lp_dev(n, dA, n, dp, dp + 4 * n, lp), "getrf_lp")
        LU = np.empty((n, n), np.float32, order="F")
        L.d2h(LU, dA)
        pv = np.empty(2 * n, np.int32)
        L.d2h(pv, dp)
        L.check(L.c.matgb_tc_status(), "tc_status")
    finally:
        L.dfree(dA)
        L.dfree(dp)
    return LU, pv[n:]


def round_lp(x, lp):
    """16-bit rounding of an update operand (lp -1: exact FP32; the split
    form lp 2 is modelled by split16)."""
    if lp == 1:
        return bf16_bits_to_f64(to_bf16_bits(x))
    if lp == 0:
        return x.astype(np.float16).astype(np.float64)
    return x.astype(np.float64)


def split16(x):
    """The split operand: power-of-two scale s (max |x| s at most 2^14), FP16
    hi part of x s and the FP16 rounding of the FP32 remainder."""
    x = np.asarray(x, np.float32)
    am = np.abs(x).max()
    s = 2.0 ** (14 - np.frexp(am)[1]) if am > 0 else 1.0
    xs = (x * np.float32(s)).astype(np.float32)
    h = xs.astype(np.float16)
    lo = (xs - h.astype(np.float32)).astype(np.float16)
    return h.astype(np.float64), lo.astype(np.float64), s


def emulate_lp_lu(A, lp, nb=128):
    """numpy model of the mixed LU: FP32 panels and FP32 trailing matrix, the
    trailing products of each nb-column block formed from 16-bit-rounded
    L21/U12 (FP16 with the per-block power-of-two scale of U12; the split form
    with hi + remainder parts of both, three products).  Returns the
    normwise factorisation error |PA - LU|_max / |A|_max it reaches."""
    M = np.array(A, np.float32)
    n = M.shape[0]
    perm = np.arange(n)
    for kb in range(0, n, nb):
        ke = min(kb + nb, n)
        for k in range(kb, ke):
            p = k + int(np.argmax(np.abs(M[k:, k])))
            if p != k:
                M[[k, p]] = M[[p, k]]
                perm[[k, p]] = perm[[p, k]]
            if M[k, k] != 0:
                M[k + 1:, k] *= np.float32(1) / M[k, k]
            M[k + 1:, k + 1:ke] -= np.outer(M[k + 1:, k], M[k, k + 1:ke])
        if ke < n:
            L11 = np.tril(M[kb:ke, kb:ke].astype(np.float64), -1) + np.eye(ke - kb)
            M[kb:ke, ke:] = np.linalg.solve(L11, M[kb:ke, ke:].astype(np.float64))
            U12 = M[kb:ke, ke:].astype(np.float64)
            if lp == 2:
                Lh, Ll, sl = split16(M[ke:, kb:ke])
                Uh, Ul, su = split16(M[kb:ke, ke:])
                upd = (Lh @ Uh + Lh @ Ul + Ll @ Uh) / (sl * su)
                M[ke:, ke:] = (M[ke:, ke:].astype(np.float64) - upd).astype(np.float32)
                continue
            s = 1.0
            if lp == 0 and np.abs(U12).max() > 0:
                s = 2.0 ** (14 - np.frexp(np.abs(U12).max())[1])
            upd = round_lp(M[ke:, kb:ke], lp) @ round_lp((U12 * s).astype(np.float32), lp)
            M[ke:, ke:] = (M[ke:, ke:].astype(np.float64) - upd / s).astype(np.float32)
    Lm = np.tril(M.astype(np.float64), -1) + np.eye(n)
    Um = np.triu(M.astype(np.float64))
    return np.abs(A[perm].astype(np.float64) - Lm @ Um).max() / np.abs(A).max()


@pytest.mark.parametrize("lp", [1, 0, 2, -1])
@pytest.mark.parametrize("n", [300, 1000, 1537])
def test_lp_lu_reconstructs(gpu, lp, n):
    """|PA - LU| of the GPU factorisation stays within 3x of what the numpy
    model of the same precision scheme reaches (plus an FP32 floor)."""
    L = gpu["f32"]
    A = rng.uniform(200 + n, (n, n), -1, 1, np.float32)
    LU, perm = factor_lp(L, A, lp)
    assert np.array_equal(np.sort(perm), np.arange(n))
    Lm = np.tril(LU.astype(np.float64), -1) + np.eye(n)
    Um = np.triu(LU.astype(np.float64))
    err = np.abs(A[perm].astype(np.float64) - Lm @ Um).max() / np.abs(A).max()
    model = emulate_lp_lu(A, lp)
    assert err <= 3 * model + 1e-5, (err, model)
    assert np.abs(Lm).max() <= 1.0 + 1e-6  # partial pivoting bound


def ktime_names(L):
    """Names of the library's timed scopes since timing was enabled."""
    out, i = set(), 0
    nm = C.create_string_buffer(64)
    cnt, ms, fl, by = C.c_longlong(), C.c_double(), C.c_double(), C.c_double()
    while L.c.matgb_ktime_get(i, nm, 64, C.byref(cnt), C.byref(ms), C.byref(fl),
                              C.byref(by)) == 0:
        out.add(nm.value.decode())
        i += 1
    return out


@pytest.mark.parametrize("n", [291, 300, 433, 1000, 1537])
def test_lookahead_prep_in_one_launch(gpu, n):
    """After a fused 144-column block, the split update's look-ahead runs the
    next block's row swaps, its U12 solve and both operands' packing as one
    launch (la_prep; U12 scaled per column).  Its factors reconstruct PA as
    well as the separate launches' do (n = 300: the last look-ahead has 12
    columns; n = 291 and 433: 3 and 1), and it is the form that ran."""
    L = gpu["f32"]
    A = rng.uniform(900 + n, (n, n), -1, 1, np.float32)
    errs = {}
    for on in (0, 1):
        prev = L.c.matgb_la_prep(on)
        try:
            L.check(L.c.matgb_ktime_enable(1), "ktime")
            LU, perm = factor_lp(L, A, 2)
            names = ktime_names(L)
        finally:
            L.c.matgb_ktime_enable(0)
            L.c.matgb_la_prep(prev)
        assert ("la_prep" in names) == bool(on), names
        assert np.array_equal(np.sort(perm), np.arange(n))
        Lm = np.tril(LU.astype(np.float64), -1) + np.eye(n)
        Um = np.triu(LU.astype(np.float64))
        assert np.abs(Lm).max() <= 1.0 + 1e-6
        errs[on] = np.abs(A[perm].astype(np.float64) - Lm @ Um).max() / np.abs(A).max()
    assert errs[1] <= 2 * errs[0] + 1e-6, errs


def conditioned(n, kappa, seed):
    rs = np.random.default_rng(seed)
    U, _ = np.linalg.qr(rs.standard_normal((n, n)))
    V, _ = np.linalg.qr(rs.standard_normal((n, n)))
    s = np.geomspace(1.0, 1.0 / kappa, n)
    return np.asfortranarray((U * s) @ V.T)


# Classic refinement (krylov=0): kappa * u_16 < 1 (BF16 u = 2^-8, FP16
# u = 2^-11) refines the 16-bit factors to FP64 accuracy on their own, beyond
# it the FP32 refactorisation takes over.  FGMRES refinement (krylov=1) keeps
# the 16-bit factors further (FP16 to kappa = 1e4 here) and otherwise gives
# up early and refactors in FP32 (final_lp None: either outcome).
@pytest.mark.parametrize("krylov,lp,n,kappa,final_lp", [
    (0, 1, 512, 1e2, 1), (0, 0, 512, 1e2, 0), (0, 1, 1024, 1e2, 1),
    (0, 0, 1024, 1e2, 0), (0, 0, 1000, 1e3, 0), (0, 1, 1000, 1e4, -1),
    (0, 0, 1000, 1e6, -1), (0, -1, 700, 1e6, -1),
    (1, 1, 512, 1e2, 1), (1, 0, 1024, 1e2, 0), (1, 0, 1000, 1e4, 0),
    (1, 1, 1000, 1e4, None), (1, 0, 1200, 1e6, None), (1, 1, 1000, 1e6, None),
    (1, -1, 700, 1e6, -1), (0, 2, 1000, 1e6, 2), (1, 2, 1200, 1e6, 2),
    (1, 2, 2048, 1e4, 2)])
def test_ir_f64_reaches_fp64_backward_error(gpu, krylov, lp, n, kappa, final_lp):
    L = gpu["f64"]
    A = conditioned(n, kappa, 7 + n)
    b = np.random.default_rng(n).standard_normal(n)
    x, rep = L.mat_solve_ir(A, b, lp_format=lp, krylov=krylov)
    assert rep["converged"] == 1, rep
    if final_lp is None:
        assert rep["lp_format"] in (lp, -1), rep
    else:
        assert rep["lp_format"] == final_lp, rep
    assert (rep["krylov_steps"] > 0) == (krylov == 1), rep
    eta = np.abs(b - A @ x).max() / (np.abs(A).sum(1).max() * np.abs(x).max()
                                     + np.abs(b).max())
    assert eta <= n * 2.0 ** -53, (eta, rep)
    xr = np.linalg.solve(A, b)
    assert np.abs(x - xr).max() / np.abs(xr).max() <= kappa * n * 2.0 ** -50


def test_ir_f32_reaches_fp32_backward_error(gpu):
    L = gpu["f32"]
    n = 800
    A = rng.uniform(55, (n, n), -1, 1, np.float32) + n * np.eye(n, dtype=np.float32) / 8
    b = rng.normal(56, (n,), np.float32)
    x, rep = L.mat_solve_ir(A, b, lp_format=1)
    assert rep["converged"] == 1 and rep["backward_error"] <= n * 2.0 ** -24, rep


@pytest.mark.parametrize("n", [8192, 8292])
def test_ir_host_matrix_in_chunks(gpu, n):
    """mat_solve_ir with a host matrix from order 8192 up: A is copied in
    column chunks while the LU runs (the chunks that arrive later catch up
    with the blocks already factored).  The solution reaches the FP64
    backward-error target and agrees with the device-pointer entry (A copied
    first) to well within kappa * u."""
    L = gpu["f64"]
    rs = np.random.default_rng(n)
    A = np.asfortranarray(rs.standard_normal((n, n)))
    b = rs.standard_normal(n)
    # three solves: the same factors each time (the chunks' catch-ups on
    # their own streams must not race), the split's usual Krylov count
    runs = [L.mat_solve_ir(A, b) for _ in range(3)]
    for x, rep in runs:
        assert rep["converged"] == 1 and rep["lp_format"] == 2, rep
        assert rep["krylov_steps"] <= 12, rep
    assert len({r["krylov_steps"] for _, r in runs}) == 1
    x, rep = runs[0]
    eta = np.abs(b - A @ x).max() / (np.abs(A).sum(1).max() * np.abs(x).max()
                                     + np.abs(b).max())
    assert eta <= n * 2.0 ** -53, (eta, rep)
    dA, db, dx = L.dalloc(A.nbytes), L.dalloc(b.nbytes), L.dalloc(b.nbytes)
    try:
        L.h2d(dA, A)
        L.h2d(db, b)
        o = L.ir_opts()
        rep2 = MatIRReport()
        L.check(L.c.matgb_gesv_ir_dev(n, dA, n, db, dx, C.byref(o), C.byref(rep2)),
                "gesv_ir_dev")
        x2 = np.empty(n)
        L.d2h(x2, dx)
    finally:
        for d in (dA, db, dx):
            L.dfree(d)
    assert np.abs(x - x2).max() / np.abs(x2).max() <= 1e-8


def test_ir_reports_nonconvergence_for_singular(gpu):
    L = gpu["f64"]
    n = 256
    A = np.ones((n, n))
    b = np.arange(n, dtype=np.float64)
    x, rep = L.mat_solve_ir(A, b, lp_format=1, max_iter=5)
    assert rep["converged"] == 0 and rep["iterations"] <= 5
    assert not np.isfinite(rep["backward_error"]) or rep["backward_error"] > 1e-6


def spd_conditioned(n, lam_max, seed):
    """Q diag(lambda) Q^T, lambda log-uniform in [1, lam_max]."""
    rs = np.random.default_rng(seed)
    Q, _ = np.linalg.qr(rs.standard_normal((n, n)))
    lam = np.exp(rs.uniform(0, np.log(lam_max), n))
    A = (Q * lam) @ Q.T
    return np.asfortranarray((A + A.T) / 2)


@pytest.mark.parametrize("lp,n,lam,final_lp", [
    (1, 600, 1e2, 1), (0, 700, 1e3, 0), (1, 500, 1e6, -1), (-1, 400, 1e6, -1),
    (2, 600, 1e6, 2)])
def test_spd_ir_reaches_fp64_backward_error(gpu, lp, n, lam, final_lp):
    L = gpu["f64"]
    A = spd_conditioned(n, lam, 31 + n)
    B = np.random.default_rng(n).standard_normal((n, 8))
    X, ret, rep = L.mat_solve_spd_ir(A, B, lp_format=lp)
    assert ret == 0 and rep["converged"] == 1 and rep["lp_format"] == final_lp, rep
    for c in range(B.shape[1]):
        x, b = X[:, c], B[:, c]
        eta = np.abs(b - A @ x).max() / (np.abs(A).sum(1).max() * np.abs(x).max()
                                         + np.abs(b).max())
        assert eta <= n * 2.0 ** -53, (c, eta)


@pytest.mark.parametrize("lp,lam,keep", [(0, 1e2, True), (1, 1e3, False),
                                         (0, 1e6, False)])
def test_spd_ir_single_rhs_fgmres(gpu, lp, lam, keep):
    """One right-hand side: FGMRES on the Cholesky-preconditioned correction.
    With lambda up to 1e6 the 16-bit Schur complements may lose definiteness,
    and the FP32 refactorisation then takes over (keep False: either)."""
    L = gpu["f64"]
    n = 800
    A = spd_conditioned(n, lam, 91)
    b = np.random.default_rng(3).standard_normal((n, 1))
    X, ret, rep = L.mat_solve_spd_ir(A, b, lp_format=lp)
    assert ret == 0 and rep["converged"] == 1, rep
    assert rep["lp_format"] == lp if keep else rep["lp_format"] in (lp, -1), rep
    assert rep["krylov_steps"] > 0
    x = X[:, 0]
    eta = np.abs(b[:, 0] - A @ x).max() / (np.abs(A).sum(1).max() * np.abs(x).max()
                                           + np.abs(b).max())
    assert eta <= n * 2.0 ** -53, eta


def test_spd_ir_not_spd_returns_minus_one(gpu):
    L = gpu["f64"]
    A = np.eye(300)
    A[150, 150] = -1.0
    X, ret, rep = L.mat_solve_spd_ir(A, np.ones((300, 2)), lp_format=1)
    assert ret == -1


def test_lp_cholesky_reconstructs(gpu):
    """FP32 Cholesky with BF16/FP16 tensor-core SYRK updates: L L^T = A up to
    the 16-bit rounding of the update operands."""
    L = gpu["f32"]
    n = 900
    A = spd_conditioned(n, 1e2, 5).astype(np.float32)
    for lp, tol in ((1, 3e-2), (0, 4e-3), (2, 1e-5), (-1, 1e-5)):
        dA = L.dalloc(A.nbytes)
        di = L.dalloc(4)
        try:
            L.h2d(dA, A)
            L.check(L.c.matgb_potrf_lp_dev(n, dA, n, di, lp), "potrf_lp")
            F = np.empty((n, n), np.float32, order="F")
            L.d2h(F, dA)
            info = np.zeros(1, np.int32)
            L.d2h(info, di)
            L.check(L.c.matgb_tc_status(), "tc_status")
        finally:
            L.dfree(dA)
            L.dfree(di)
        assert info[0] == 0
        Lf = np.tril(F.astype(np.float64))
        err = np.abs(Lf @ Lf.T - A).max() / np.abs(A).max()
        assert err <= tol, (lp, err)


def potrf_lp(L, A, lp):
    n = A.shape[0]
    dA = L.dalloc(A.nbytes)
    di = L.dalloc(4)
    try:
        L.h2d(dA, np.asfortranarray(A, np.float32))
        L.check(L.c.matgb_potrf_lp_dev(n, dA, n, di, lp), "potrf_lp")
        F = np.empty((n, n), np.float32, order="F")
        L.d2h(F, dA)
        info = np.zeros(1, np.int32)
        L.d2h(info, di)
        L.check(L.c.matgb_tc_status(), "tc_status")
    finally:
        L.dfree(dA)
        L.dfree(di)
    return F, int(info[0])


@pytest.mark.parametrize("lp", [2, 1])
@pytest.mark.parametrize("n", [129, 300, 1000, 1537])
def test_cholesky_lookahead_identical(gpu, lp, n):
    """The tensor-core Cholesky's look-ahead (diagonal block, column solve
    and the next block's update on the panel stream, the rest of the
    trailing update beside it) computes every entry with the same operands
    and the same products as the one-stream order: the factors agree bit for
    bit, and so does the not-SPD report (a negative pivot in block 3)."""
    L = gpu["f32"]
    A = spd_conditioned(n, 1e3, 70 + n).astype(np.float32)
    bad = A.copy()
    if n > 400:
        bad[400, 400] = -1.0
    out = {}
    for on in (0, 1):
        prev = L.c.matgb_chol_lookahead(on)
        try:
            out[on] = (potrf_lp(L, A, lp), potrf_lp(L, bad, lp))
        finally:
            L.c.matgb_chol_lookahead(prev)
    (F0, i0), (G0, j0) = out[0]
    (F1, i1), (G1, j1) = out[1]
    assert i0 == i1 == 0
    assert np.array_equal(np.tril(F0), np.tril(F1))
    assert j0 == j1 and (j0 == 401 if n > 400 else j0 == 0), (j0, j1)
    if j0 == 0:
        assert np.array_equal(np.tril(G0), np.tril(G1))


@pytest.mark.parametrize("n", [100, 1030, 2100])
@pytest.mark.parametrize("nrhs", [1, 7, 64, 65])
def test_resid64_matches_fp64(gpu, n, nrhs):
    """R -= A X from FP16 digit slices on the tensor cores agrees with the FP64
    product within the FP64 GEMM's own error bound (n u |A||X|), with rows
    and columns of very different scales, a zero row and a zero column."""
    L = gpu["f64"]
    rs = np.random.default_rng(900 + n + nrhs)
    A = rs.standard_normal((n, n)) * 10.0 ** rs.uniform(-6, 6, (n, 1))
    A[n // 3, :] = 0.0
    X = rs.standard_normal((n, nrhs)) * 10.0 ** rs.uniform(-6, 6, (1, nrhs))
    X[:, nrhs // 2] = 0.0
    B = rs.standard_normal((n, nrhs))
    A, X, B = (np.asfortranarray(v) for v in (A, X, B))
    bufs = [L.dalloc(v.nbytes) for v in (A, X, B)]
    try:
        for d, v in zip(bufs, (A, X, B)):
            L.h2d(d, v)
        L.check(L.c.matgb_resid64_dev(n, nrhs, bufs[0], n, bufs[1], n, bufs[2], n),
                "resid64")
        R = np.empty((n, nrhs), np.float64, order="F")
        L.d2h(R, bufs[2])
        L.check(L.c.matgb_tc_status(), "tc_status")
    finally:
        for d in bufs:
            L.dfree(d)
    ref = B - A @ X
    bound = n * 2.0 ** -53 * (np.abs(A) @ np.abs(X)) + 2.0 ** -52 * np.abs(B)
    assert np.all(np.abs(R - ref) <= 2 * bound + 1e-300)


def test_resid64_propagates_nan(gpu):
    L = gpu["f64"]
    n, nrhs = 300, 3
    rs = np.random.default_rng(7)
    A = np.asfortranarray(rs.standard_normal((n, n)))
    A[5, 7] = np.nan
    X = np.asfortranarray(rs.standard_normal((n, nrhs)))
    B = np.asfortranarray(np.zeros((n, nrhs)))
    bufs = [L.dalloc(v.nbytes) for v in (A, X, B)]
    try:
        for d, v in zip(bufs, (A, X, B)):
            L.h2d(d, v)
        L.check(L.c.matgb_resid64_dev(n, nrhs, bufs[0], n, bufs[1], n, bufs[2], n),
                "resid64")
        R = np.empty((n, nrhs), np.float64, order="F")
        L.d2h(R, bufs[2])
    finally:
        for d in bufs:
            L.dfree(d)
    assert np.all(np.isnan(R[5]))
    assert np.all(np.isfinite(np.delete(R, 5, axis=0)))


@pytest.mark.parametrize("lam,nrhs", [(1e3, 8), (1e6, 70)])
def test_spd_ir_tensor_core_residual(gpu, lam, nrhs):
    """From n = 1024 up the multi-RHS refinement forms its FP64 residuals from
    FP16 digit products on the tensor cores: the solve still reaches the FP64
    backward-error target (checked here in numpy), and agrees with the same
    solve whose residuals come from the FP64 GEMM."""
    L = gpu["f64"]
    n = 1100
    A = spd_conditioned(n, lam, 77)
    B = np.random.default_rng(nrhs).standard_normal((n, nrhs))
    try:
        X1, ret1, rep1 = L.mat_solve_spd_ir(A, B, lp_format=2)
        L.check(L.c.matgb_resid64_mode(0), "resid64_mode")
        X0, ret0, rep0 = L.mat_solve_spd_ir(A, B, lp_format=2)
    finally:
        L.c.matgb_resid64_mode(1)
    assert ret1 == 0 and rep1["converged"] == 1, rep1
    assert ret0 == 0 and rep0["converged"] == 1, rep0
    for c in range(nrhs):
        x, b = X1[:, c], B[:, c]
        eta = np.abs(b - A @ x).max() / (np.abs(A).sum(1).max() * np.abs(x).max()
                                         + np.abs(b).max())
        assert eta <= n * 2.0 ** -53, (c, eta)
    assert np.abs(X1 - X0).max() <= 1e-9 * np.abs(X0).max() * lam
