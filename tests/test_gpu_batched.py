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


@pytest.fixture(params=["fused", "queues_gauss_jordan", "queues_blocked"])
def algo(request, gpu):
    """Every schedule: the one persistent launch (replayed as a CUDA graph),
    or one launch per queue with the large buckets on the register
    Gauss-Jordan kernel or the blocked LU; defaults restored after."""
    fused = request.param == "fused"
    algo_ = 1 if request.param == "queues_blocked" else 0
    saved = {}
    for prec in ("f32", "f64"):
        L = gpu[prec]
        saved[prec, "fused"] = L.c.matgb_batched_schedule(1 if fused else 0, -1, 1)
        for nb in (64, 96, 128):
            for kind in (0, 1):
                a, c = C.c_int(), C.c_int()
                L.check(L.c.matgb_batched_tune_get(nb, kind, C.byref(a), C.byref(c)))
                saved[prec, nb, kind] = (a.value, c.value)
                # the double build's 96 and 128 buckets have one form only
                L.check(L.c.matgb_batched_tune(nb, kind, algo_, c.value))
    yield request.param
    for key, v in saved.items():
        if key[1] == "fused":
            gpu[key[0]].c.matgb_batched_schedule(v, -1, -1)
        else:
            prec, nb, kind = key
            gpu[prec].c.matgb_batched_tune(nb, kind, *v)


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


@pytest.mark.parametrize("prec", ["f32", "f64"])
def test_batched_graph_replay_same_buffers(gpu, prec):
    """The one-launch schedule captures its launch sequence in a CUDA graph on
    the first call with a set of buffers and replays it on later calls with
    the same buffers: new data in the same buffers must give the new
    solutions, and other buffers a new capture."""
    L = gpu[prec]
    O = Oracle(prec)
    prev = L.c.matgb_batched_schedule(1, -1, 1)
    try:
        count = 200
        outs = []
        for seed in (3, 4):
            mats, rhs, kinds = make_batch(count, 128, L.dtype, seed)
            ns = np.array([m.shape[0] for m in mats], np.int32)
            offA = np.zeros(count, np.int64)
            offA[1:] = np.cumsum(ns.astype(np.int64) ** 2)[:-1]
            offv = np.zeros(count, np.int64)
            offv[1:] = np.cumsum(ns.astype(np.int64))[:-1]
            outs.append((mats, rhs, kinds, ns, offA, offv))
        # buffers sized for the larger of the two batches, reused by both
        tot_a = max(sum(m.size for m in o[0]) for o in outs)
        tot_v = max(sum(v.size for v in o[1]) for o in outs)
        es = np.dtype(L.dtype).itemsize
        dn, doA, dov = L.dalloc(4 * count), L.dalloc(8 * count), L.dalloc(8 * count)
        dA, db, dx = L.dalloc(es * tot_a), L.dalloc(es * tot_v), L.dalloc(es * tot_v)
        dk, dst = L.dalloc(count), L.dalloc(4 * count)
        try:
            for rep in range(3):  # calls 2 and 3 replay the graph of call 1 or 2
                mats, rhs, kinds, ns, offA, offv = outs[rep % 2]
                Acat = np.concatenate([m.ravel(order="F") for m in mats])
                bcat = np.concatenate(rhs)
                for d, a in ((dn, ns), (doA, offA), (dov, offv), (dA, Acat),
                             (db, bcat), (dk, np.asarray(kinds, np.uint8))):
                    L.h2d(d, a)
                L.check(L.c.matgb_solve_batched_dev(count, dn, doA, dA, dov, db, dx,
                                                    dk, dst), "batched")
                x = np.empty_like(bcat)
                L.d2h(x, dx)
                st = np.empty(count, np.int32)
                L.d2h(st, dst)
                assert np.all(st == 0)
                for s in range(0, count, 7):
                    n = ns[s]
                    xs = x[offv[s]:offv[s] + n]
                    xr = O.solve(mats[s], rhs[s]) if kinds[s] == 0 else \
                        O.solve_spd(mats[s], rhs[s])[0]
                    assert np.abs(xs - xr).max() / np.abs(xr).max() <= TOL[prec]
        finally:
            for d in (dn, doA, dov, dA, db, dx, dk, dst):
                L.dfree(d)
    finally:
        L.c.matgb_batched_schedule(prev, -1, -1)
