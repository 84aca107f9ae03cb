"""GPU: the batched solver's mixed-precision mode (matgb_batched_mixed): orders
33..128 factored on the tensor cores (TF32 hi + remainder trailing updates,
matrix in tensor memory), refined in FP32 to a normwise backward error
|b - A x| / (|A| |x| + |b|) <= n 2^-24, through the C ABI.

Criteria (max-norm):
  * every system with status 0 meets the backward-error target, recomputed
    here in FP64 from the returned x (the kernel's own test uses an FP32
    residual; the bound checked here is 2 n 2^-24 to leave room for that
    residual's rounding);
  * its forward error against an FP64 solve is within 10 cond(A) n 2^-24;
  * well-conditioned batches (U[-1,1] + n I, B^T B + n I) all converge;
  * systems that pivot (U[-1,1], no shift) converge too, and their solutions
    meet the same bounds;
  * an SPD-kind system that is not positive definite gives status -1 with x
    untouched, as mat_solve_spd returns -1;
  * orders 1..32 in the same call keep the FP32 kernels' results exactly;
  * switching the mode off restores the plain kernels' results;
  * mode 1 routes only the chosen (bucket, kind) queues.
Mode 2 (every queue of orders 33..128 on the tensor cores) is used unless a
test says otherwise.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
U32 = 2.0 ** -24


@pytest.fixture
def mixed(gpu):
    """Every queue of orders 33..128 on the tensor-core kernels."""
    L = gpu["f32"]
    prev = L.c.matgb_batched_mixed(2)
    yield L
    L.c.matgb_batched_mixed(prev)


def batch(count, nlo, nhi, seed, shift=True):
    rs = np.random.default_rng(seed)
    mats, rhs, kinds = [], [], []
    for s in range(count):
        n = int(rs.integers(nlo, nhi + 1))
        kind = s % 2
        if kind == 0:
            A = rs.uniform(-1, 1, (n, n)) + (n * np.eye(n) if shift else 0)
        else:
            B = rs.standard_normal((n, n))
            A = B.T @ B + n * np.eye(n)
        mats.append(np.asfortranarray(A.astype(np.float32)))
        rhs.append(rs.standard_normal(n).astype(np.float32))
        kinds.append(kind)
    return mats, rhs, kinds


def sym_lower(A, kind):
    """The matrix the solver sees: SPD kinds read the lower triangle."""
    A = A.astype(np.float64)
    if kind == 1:
        A = np.tril(A) + np.tril(A, -1).T
    return A


def check(mats, rhs, kinds, xs, status):
    for A, b, k, x, st in zip(mats, rhs, kinds, xs, status):
        n = A.shape[0]
        A64 = sym_lower(A, k)
        b64 = b.astype(np.float64)
        x64 = x.astype(np.float64)
        assert st == 0, (n, k, st)
        eta = np.abs(b64 - A64 @ x64).max() / (
            np.abs(A64).sum(1).max() * np.abs(x64).max() + np.abs(b64).max())
        assert eta <= 2 * n * U32, (n, k, eta)
        xt = np.linalg.solve(A64, b64)
        cond = np.linalg.cond(A64, np.inf)
        fe = np.abs(x64 - xt).max() / np.abs(xt).max()
        assert fe <= 10 * cond * n * U32, (n, k, fe, cond)


@pytest.mark.parametrize("nlo,nhi,count", [(33, 64, 400), (65, 96, 300), (97, 128, 300),
                                           (1, 128, 600)])
def test_mixed_well_conditioned(mixed, nlo, nhi, count):
    L = mixed
    mats, rhs, kinds = batch(count, nlo, nhi, 500 + nhi + nlo)
    xs, status = L.solve_batched(mats, rhs, kinds)
    check(mats, rhs, kinds, xs, status)
    corr, unconv, tout = C.c_int(), C.c_int(), C.c_int()
    L.check(L.c.matgb_batched_mixed_stats(C.byref(corr), C.byref(unconv), C.byref(tout)))
    assert unconv.value == 0 and tout.value == 0


def test_mixed_pivoting_systems(mixed):
    """U[-1,1] with no diagonal shift: the diagonal-first pass is beaten and
    the system is factored again with the pivot search."""
    L = mixed
    mats, rhs, kinds = batch(200, 33, 128, 77, shift=False)
    kinds = [0] * len(mats)
    xs, status = L.solve_batched(mats, rhs, kinds)
    check(mats, rhs, kinds, xs, status)


def test_mixed_not_spd_and_small_orders(gpu, mixed):
    L = mixed
    rs = np.random.default_rng(5)
    n = 70
    Bm = rs.standard_normal((n, n))
    bad = np.asfortranarray((Bm.T @ Bm - 5 * n * np.eye(n)).astype(np.float32))
    mats, rhs, kinds = batch(40, 1, 32, 6)
    mats.append(bad)
    rhs.append(rs.standard_normal(n).astype(np.float32))
    kinds.append(1)
    xs, status = L.solve_batched(mats, rhs, kinds)
    assert status[-1] == -1
    # orders 1..32 keep the FP32 kernels: identical to the plain mode
    L.c.matgb_batched_mixed(0)
    xs0, status0 = L.solve_batched(mats, rhs, kinds)
    L.c.matgb_batched_mixed(2)
    assert np.array_equal(status0, status)
    for a, b_ in zip(xs[:-1], xs0[:-1]):
        assert np.array_equal(a, b_)


def test_mixed_off_restores_plain(gpu):
    L = gpu["f32"]
    mats, rhs, kinds = batch(60, 33, 128, 9)
    prev = L.c.matgb_batched_mixed(0)
    try:
        xa, sa = L.solve_batched(mats, rhs, kinds)
        L.c.matgb_batched_mixed(2)
        xm, sm = L.solve_batched(mats, rhs, kinds)
        L.c.matgb_batched_mixed(0)
        xb, sb = L.solve_batched(mats, rhs, kinds)
    finally:
        L.c.matgb_batched_mixed(prev)
    assert np.all(sa == 0) and np.all(sm == 0) and np.array_equal(sa, sb)
    for a, b_ in zip(xa, xb):
        assert np.array_equal(a, b_)
    assert gpu["f64"].c.matgb_batched_mixed(1) < 0
    gpu["f64"].c.matgb_clear_error()


def test_mixed_per_queue_routing(gpu):
    """Mode 1 routes only the queues chosen per (bucket, kind); the others
    give the plain kernels' results bit for bit."""
    L = gpu["f32"]
    mats, rhs, kinds = batch(80, 65, 128, 13)
    prev = L.c.matgb_batched_mixed(0)
    try:
        x0, s0 = L.solve_batched(mats, rhs, kinds)
        for nb in (64, 96, 128):
            for kind in (0, 1):
                L.check(L.c.matgb_batched_mixed_tune(nb, kind, 1 if (nb, kind) == (128, 0) else 0))
        L.c.matgb_batched_mixed(1)
        x1, s1 = L.solve_batched(mats, rhs, kinds)
    finally:
        L.c.matgb_batched_mixed(prev)
        L.check(L.c.matgb_batched_mixed_tune(128, 0, 1))
    check(mats, rhs, kinds, x1, s1)
    for A, k, a, b_ in zip(mats, kinds, x0, x1):
        if not (k == 0 and A.shape[0] > 96):  # not routed: the FP32 kernel's result
            assert np.array_equal(a, b_)
