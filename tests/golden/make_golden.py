"""Generate the golden fixtures in tests/golden/ from the REFERENCE ITSELF.

Runs only where the reference source tree is present: it builds
oracle/_ref/libref_{f32,f64}.so from the reference's own mat.h (oracle/Makefile)
and records, for each fixture input, the reference's outputs.

Fixtures:
  kat_<prec>.npz  -- the known-answer inputs of the reference's unit tests
                     (tests/test_mat_{plu,solve,chol,solve_spd,solve_tri,mul}.c)
                     with the reference's outputs.
  rand_<prec>.npz -- the reference tests' srand(42) random inputs, regenerated
                     with the same glibc rand() call sequence, plus outputs.
  lu_<prec>.npz   -- mat_lu (full pivoting): the known-answer matrices of
                     tests/test_mat_lu.c and test_mat_plu.c's determinant
                     test, and test_mat_lu.c's random inputs (glibc rand()
                     from its default seed, values in steps of 0.1).
  c1_<prec>.npz   -- the 256x256 plain config: A ~ U[-1,1] (seed 1000),
                     b ~ N(0,1) (seed 2000); mat_mul(A, A), mat_plu(A),
                     mat_solve(A, b).
  c2_8192.npz     -- the 8192 plain config (PLU + 16-RHS solve): A ~ N(0,1)
                     float32 (seed 1002), B ~ N(0,1) float32 8192 x 16
                     (seed 2002), both from libmat_gb300.rng.  Holds the
                     reference's float mat_plu permutation and swap count,
                     its float solutions (mat_plu once, then per column the
                     public mat_solve_tril_unit / mat_solve_triu on B[p]) and
                     its double solutions of the same (exactly widened)
                     system, plus kappa_inf(A) estimated by LAPACK's dgecon
                     (scipy).  A itself is not stored: it is regenerated from
                     the seed.  Takes a few minutes (two scalar
                     factorisations).  Only with --c2.

Usage: python tests/golden/make_golden.py [reference_dir] [--c2]
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import loader  # noqa: E402
from libmat_gb300 import rng  # noqa: E402


def rm(rows, cols, vals, dt):
    """mat_from: row-major C initialiser -> column-major array."""
    return np.array(vals, dtype=dt).reshape(rows, cols)


def kat(R, dt):
    out = {}
    # tests/test_mat_plu.c:17-80
    for name, A in (("plu_2x2", rm(2, 2, [4, 3, 6, 3], dt)),
                    ("plu_3x3", rm(3, 3, [1, 2, 3, 0, 1, 4, 5, 6, 0], dt))):
        L, U, p, s = R.plu(A)
        out.update({name + "_A": A, name + "_L": L, name + "_U": U,
                    name + "_p": p, name + "_s": np.int64(s)})
    # tests/test_mat_solve.c:7-77, 120-136
    solves = {
        "solve_1x1": (rm(1, 1, [5], dt), [15]),
        "solve_identity": (np.eye(3, dtype=dt), [1, 2, 3]),
        "solve_2x2": (rm(2, 2, [2, 3, 4, 5], dt), [8, 14]),
        "solve_3x3": (rm(3, 3, [1, 2, 3, 0, 1, 4, 5, 6, 0], dt), [14, 14, 17]),
    }
    for name, (A, b) in solves.items():
        b = np.array(b, dt)
        out.update({name + "_A": A, name + "_b": b, name + "_x": R.solve(A, b)})
    # tests/test_mat_chol.c:45-151
    chols = {
        "chol_2x2_identity": np.eye(2, dtype=dt),
        "chol_2x2_known": rm(2, 2, [4, 2, 2, 5], dt),
        "chol_3x3_known": rm(3, 3, [4, 12, -16, 12, 37, -43, -16, -43, 98], dt),
        "chol_not_spd": rm(2, 2, [1, 2, 2, 1], dt),
    }
    for name, A in chols.items():
        L, r = R.chol(A)
        out.update({name + "_A": A, name + "_L": L, name + "_r": np.int64(r)})
    # tests/test_mat_solve_spd.c:28-122, 157-174
    spds = {
        "spd_1x1": (rm(1, 1, [4], dt), [12]),
        "spd_identity": (np.eye(3, dtype=dt), [1, 2, 3]),
        "spd_2x2": (rm(2, 2, [4, 2, 2, 3], dt), [8, 8]),
        "spd_3x3": (rm(3, 3, [5, 4, 1, 4, 6, 4, 1, 4, 5], dt), [16, 28, 24]),
        "spd_not_spd": (rm(2, 2, [1, 2, 2, 1], dt), [1, 1]),
    }
    for name, (A, b) in spds.items():
        b = np.array(b, dt)
        x, r = R.solve_spd(A, b)
        out.update({name + "_A": A, name + "_b": b, name + "_x": x,
                    name + "_r": np.int64(r)})
    # tests/test_mat_solve_tri.c:7-123
    tris = {
        "tril_2x2": ("solve_tril", rm(2, 2, [2, 0, 3, 4], dt), [2, 11]),
        "tril_unit_2x2": ("solve_tril_unit", rm(2, 2, [1, 0, 3, 1], dt), [1, 5]),
        "triu_2x2": ("solve_triu", rm(2, 2, [2, 3, 0, 4], dt), [8, 8]),
        "trilt_2x2": ("solve_trilt", rm(2, 2, [2, 0, 3, 4], dt), [8, 8]),
        "tril_3x3": ("solve_tril", rm(3, 3, [2, 0, 0, 1, 3, 0, 4, 2, 5], dt),
                     [2, 7, 23]),
    }
    for name, (fn, T, b) in tris.items():
        b = np.array(b, dt)
        out.update({name + "_T": T, name + "_b": b,
                    name + "_x": getattr(R, fn)(T, b)})
    # tests/test_mat_mul.c:6-90
    muls = {
        "mul_basic": (rm(2, 2, [1, 2, 3, 4], dt), rm(2, 2, [5, 6, 7, 8], dt)),
        "mul_identity": (rm(2, 2, [1, 2, 3, 4], dt), np.eye(2, dtype=dt)),
        "mul_rect": (rm(2, 3, [1, 2, 3, 4, 5, 6], dt),
                     rm(3, 2, [7, 8, 9, 10, 11, 12], dt)),
        "mul_vector": (rm(2, 2, [1, 2, 3, 4], dt), rm(2, 1, [5, 6], dt)),
    }
    for name, (a, b) in muls.items():
        out.update({name + "_a": a, name + "_b": b, name + "_c": R.mul(a, b)})
    return out


def crand(R, dt, div, sub):
    return dt(dt(R.rand() % 100) / dt(div) - dt(sub))


def diag_dominant(R, n, dt):
    """tests/test_mat_plu.c:85-94 and tests/test_mat_solve.c:82-91"""
    A = np.zeros((n, n), dt, order="F")
    for i in range(n):
        s = dt(0)
        for j in range(n):
            v = crand(R, dt, 10.0, 5.0)
            A[i, j] = v
            if i != j:
                s = dt(s + abs(v))
        A[i, i] = dt(s + dt(1.0))
    return A


def rand_fixtures(R, dt):
    out = {}
    # tests/test_mat_plu.c:157-167 (srand(42); sizes 10, 50, 100)
    R.srand(42)
    for n in (10, 50, 100):
        A = diag_dominant(R, n, dt)
        L, U, p, s = R.plu(A)
        out.update({f"plu{n}_A": A, f"plu{n}_L": L, f"plu{n}_U": U,
                    f"plu{n}_p": p, f"plu{n}_s": np.int64(s)})
    # tests/test_mat_solve.c:151-163
    R.srand(42)
    for n in (10, 50, 100):
        A = diag_dominant(R, n, dt)
        b = np.array([crand(R, dt, 10.0, 0.0) for _ in range(n)], dt)
        out.update({f"solve{n}_A": A, f"solve{n}_b": b,
                    f"solve{n}_x": R.solve(A, b)})
    # tests/test_mat_chol.c:8-29, 203-217: A = B B^T + n I, B filled linearly
    R.srand(42)
    for n in (10, 50, 100, 128, 200):
        B = np.zeros(n * n, dt)
        for i in range(n * n):
            B[i] = crand(R, dt, 10.0, 5.0)
        B = B.reshape(n, n, order="F")
        A = R.mul(B, np.asfortranarray(B.T))
        A[np.arange(n), np.arange(n)] += dt(n)
        L, r = R.chol(A)
        out.update({f"chol{n}_A": A, f"chol{n}_L": L, f"chol{n}_r": np.int64(r)})
    # tests/test_mat_solve_spd.c:8-26, 176-186: A = M M^T + 0.1 I
    R.srand(42)
    for n in (10, 50, 100):
        M = np.zeros((n, n), dt, order="F")
        for i in range(n):
            for j in range(n):
                M[i, j] = crand(R, dt, 10.0, 5.0)
        A = R.mul(M, np.asfortranarray(M.T))
        A[np.arange(n), np.arange(n)] += dt(0.1)
        b = np.array([crand(R, dt, 10.0, 0.0) for _ in range(n)], dt)
        x, r = R.solve_spd(A, b)
        out.update({f"spd{n}_A": A, f"spd{n}_b": b, f"spd{n}_x": x,
                    f"spd{n}_r": np.int64(r)})
    # tests/test_mat_solve_tri.c:125-148, 172-181
    R.srand(42)
    for n in (10, 50, 100):
        L = np.zeros((n, n), dt, order="F")
        for i in range(n):
            s = dt(0)
            for j in range(i):
                v = crand(R, dt, 100.0, 0.5)
                L[i, j] = v
                s = dt(s + abs(v))
            L[i, i] = dt(s + dt(1.0))
        b = np.array([crand(R, dt, 10.0, 0.0) for _ in range(n)], dt)
        out.update({f"trilt{n}_L": L, f"trilt{n}_b": b,
                    f"trilt{n}_x": R.solve_trilt(L, b)})
    return out


def lu_fixtures(R, dt):
    out = {}
    # tests/test_mat_lu.c:7-80 and tests/test_mat_plu.c:125-130
    kats = {
        "lu_3x3": rm(3, 3, [2, -1, -2, -4, 6, 3, -4, -2, 8], dt),
        "lu_4x4": rm(4, 4, [4, 3, 2, 1, 3, 4, 3, 2, 2, 3, 4, 3, 1, 2, 3, 4], dt),
        "lu_det3": rm(3, 3, [6, 1, 1, 4, -2, 5, 2, 8, 7], dt),
    }
    # tests/test_mat_lu.c:82-90, 115-117: no srand, (rand() % 200 - 100) / 10.0f
    R.srand(1)
    for n in (10, 50, 100):
        A = np.zeros((n, n), dt, order="F")
        for i in range(n):
            for j in range(n):
                A[i, j] = dt(dt(R.rand() % 200 - 100) / dt(10.0))
        kats[f"lu_random{n}"] = A
    for name, A in kats.items():
        L, U, p, q, s = R.lu(A)
        out.update({name + "_A": A, name + "_L": L, name + "_U": U,
                    name + "_p": p, name + "_q": q, name + "_s": np.int64(s)})
    return out


def c1(R, dt):
    n = 256
    A = rng.uniform(1000, (n, n), -1.0, 1.0, dt)
    b = rng.normal(2000, (n,), dt)
    L, U, p, s = R.plu(A)
    LU = np.tril(L, -1) + U
    return {"A": A, "b": b, "AA": R.mul(A, A), "LU": LU, "p": p,
            "s": np.int64(s), "x": R.solve(A, b)}


C2_N, C2_NRHS, C2_SEED_A, C2_SEED_B = 8192, 16, 1002, 2002


def c2_inputs():
    """The 8192 plain config's inputs (regenerated the same way by the GPU
    parity test)."""
    A = rng.normal(C2_SEED_A, (C2_N, C2_N), np.float32)
    B = rng.normal(C2_SEED_B, (C2_N, C2_NRHS), np.float32)
    return A, B


def c2():
    import time
    import scipy.linalg as sl
    A, B = c2_inputs()
    out = {"seed_A": np.int64(C2_SEED_A), "seed_B": np.int64(C2_SEED_B)}
    for prec, dt in (("f32", np.float32), ("f64", np.float64)):
        R = loader.Oracle(prec, "ref")
        Ad = A.astype(dt)
        t0 = time.time()
        L, U, p, s = R.plu(Ad)
        X = np.empty((C2_N, C2_NRHS), dt, order="F")
        for j in range(C2_NRHS):
            X[:, j] = R.solve_triu(U, R.solve_tril_unit(L, B[p, j].astype(dt)))
        print(f"c2 {prec}: plu + {C2_NRHS} solves {time.time() - t0:.0f} s, "
              f"MAT_ARCH {R.arch()}")
        out[f"p_{prec}"] = p.astype(np.int32)
        out[f"s_{prec}"] = np.int64(s)
        out[f"x_{prec}"] = X
        del L, U
    A64 = A.astype(np.float64)
    lu, piv, info = sl.lapack.dgetrf(A64)
    anorm = np.abs(A64).sum(1).max()
    rcond, info2 = sl.lapack.dgecon(lu, anorm, norm="I")
    out["kappa_inf_est"] = np.float64(1.0 / rcond)
    out["lapack_perm_matches_ref_f64"] = np.int64(
        np.array_equal(_perm_from_ipiv(piv), out["p_f64"]))
    return out


def _perm_from_ipiv(ipiv):
    """LAPACK's row interchanges as mat_plu's permutation (p[i] = source row
    of row i)."""
    p = np.arange(len(ipiv))
    for k, r in enumerate(ipiv):
        p[[k, r]] = p[[r, k]]
    return p


def main():
    args = [a for a in sys.argv[1:] if not a.startswith("--")]
    ref = args[0] if args else loader.ref_dir()
    if not ref:
        raise SystemExit("reference source tree not found: pass it as the "
                         f"first argument or set ${loader.REF_ENV}")
    loader.build(ref)
    if "--c2" in sys.argv:  # the 8192 fixture alone (minutes)
        np.savez_compressed(os.path.join(HERE, "c2_8192.npz"), **c2())
        print("c2 ok")
        return
    for prec, dt in (("f32", np.float32), ("f64", np.float64)):
        R = loader.Oracle(prec, "ref")
        np.savez_compressed(os.path.join(HERE, f"kat_{prec}.npz"), **kat(R, dt))
        np.savez_compressed(os.path.join(HERE, f"rand_{prec}.npz"),
                            **rand_fixtures(R, dt))
        np.savez_compressed(os.path.join(HERE, f"c1_{prec}.npz"), **c1(R, dt))
        np.savez_compressed(os.path.join(HERE, f"lu_{prec}.npz"), **lu_fixtures(R, dt))
        print(prec, "ok")


if __name__ == "__main__":
    main()
