"""ctypes loader for the CPU oracle (TEST INFRASTRUCTURE ONLY).

Only tests/, ``__graft_entry__.smoke()`` and bench.py's CPU-baseline leg may
import this module.  The shipped library never touches it.

``Oracle(prec, kind)`` wraps either the C restatement (kind="port",
oracle/build/liboracle_*.so, builds anywhere) or the reference's own mat.h
compiled in place (kind="ref", oracle/_ref/libref_*.so, only where the
reference source tree exists).  Every routine takes and returns numpy arrays in
column-major (Fortran) order, mirroring the reference's Mat layout
(mat.h:389, MAT_IDX = j*rows + i).
"""
import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))

# Where the reference source tree (mat.h and its tests/) is read from when it
# exists on this host: $LIBMAT_REF_DIR, else the checker's default location.
# On hosts without it (the GPU machines) every reference-backed check skips.
REF_ENV = "LIBMAT_REF_DIR"
_REF_DEFAULT = "/root/reference"


def ref_dir():
    """The reference source tree, or None when it is not present here.  On a
    host without it, the copy of its header and unit tests that
    oracle/Makefile made on a host that has it (oracle/_ref/src, never
    committed) stands in."""
    d = os.environ.get(REF_ENV) or _REF_DEFAULT
    if os.path.isfile(os.path.join(d, "mat.h")):
        return d
    d = os.path.join(HERE, "_ref", "src")
    return d if os.path.isfile(os.path.join(d, "mat.h")) else None


def build(ref=None):
    """Run oracle/Makefile: the port always, the reference shim when a
    reference tree is given (or found by ref_dir())."""
    ref = ref or ref_dir()
    subprocess.run(["make", "-s", "-C", HERE, "oracle"], check=True,
                   stdout=subprocess.DEVNULL)
    # the reference's own builds: a checker and a baseline, never required (a
    # host where its header does not compile keeps the restatements)
    cmd = ["make", "-s", "-k", "-C", HERE, "ref"]
    # the copy in _ref/src is the Makefile's own default source
    if ref and os.path.abspath(ref) != os.path.join(HERE, "_ref", "src"):
        cmd.append("REF_DIR=" + ref)
    subprocess.run(cmd, check=False, stdout=subprocess.DEVNULL,
                   stderr=subprocess.DEVNULL)


def _path(prec, kind):
    if kind == "port":
        return os.path.join(HERE, "build", f"liboracle_{prec}.so")
    if kind == "neon":
        return os.path.join(HERE, "build", f"libneon_{prec}.so")
    if kind == "time":
        return os.path.join(HERE, "_ref", f"libreftime_{prec}.so")
    return os.path.join(HERE, "_ref", f"libref_{prec}.so")


class NeonPort:
    """The reference's NEON-path mat_solve restated (oracle/neon_port.c),
    double only: the CPU baseline on hosts without the reference source.
    On aarch64 it runs the NEON micro-kernel (arch() == "NEON")."""

    def __init__(self):
        path = _path("f64", "neon")
        if not os.path.exists(path):
            build()
        self.lib = C.CDLL(path, mode=C.RTLD_LOCAL)
        self.lib.np_arch.restype = C.c_char_p
        self.lib.np_plu_inplace.restype = C.c_int

    def arch(self):
        return self.lib.np_arch().decode()

    def solve(self, A, b):
        A = np.asfortranarray(A, dtype=np.float64)
        b = np.ascontiguousarray(np.asarray(b, np.float64).reshape(-1))
        x = np.zeros(A.shape[0])
        self.lib.np_solve(x.ctypes.data_as(C.c_void_p), A.ctypes.data_as(C.c_void_p),
                          b.ctypes.data_as(C.c_void_p), C.c_size_t(A.shape[0]))
        return x

    def plu(self, A):
        """(packed LU, perm, swaps)."""
        M = np.array(A, dtype=np.float64, order="F", copy=True)
        n = M.shape[0]
        p = np.zeros(n, np.uint64)
        s = self.lib.np_plu_inplace(M.ctypes.data_as(C.c_void_p), C.c_size_t(n),
                                    p.ctypes.data_as(C.c_void_p))
        return M, p.astype(np.int64), int(s)


def available(prec="f32", kind="port"):
    return os.path.exists(_path(prec, kind))


class Oracle:
    def __init__(self, prec="f32", kind="port"):
        assert prec in ("f32", "f64") and kind in ("port", "ref", "time")
        path = _path(prec, kind)
        if not os.path.exists(path) and kind == "port":
            build()
        if not os.path.exists(path):
            raise FileNotFoundError(path)
        self.lib = C.CDLL(path, mode=C.RTLD_LOCAL)
        self.prec, self.kind = prec, kind
        self.dtype = np.float32 if prec == "f32" else np.float64
        self.ct = C.c_float if prec == "f32" else C.c_double
        self.pre = "orc_" if kind == "port" else "ref_"  # "time": the reference too

    def arch(self):
        """MAT_ARCH of the reference build ("port" for the restatement)."""
        if self.kind == "port":
            return "port"
        self.lib.ref_arch.restype = C.c_char_p
        return self.lib.ref_arch().decode()

    def _fn(self, name):
        return getattr(self.lib, self.pre + name)

    def _arr(self, a):
        a = np.asfortranarray(a, dtype=self.dtype)
        return a, a.ctypes.data_as(C.c_void_p)

    # -- products -----------------------------------------------------------
    def gemm(self, alpha, A, B, beta, Cm):
        A, pa = self._arr(A)
        B, pb = self._arr(B)
        Cm = np.array(Cm, dtype=self.dtype, order="F", copy=True)
        m, k = A.shape
        n = B.shape[1]
        self._fn("gemm")(C.c_size_t(m), C.c_size_t(k), C.c_size_t(n),
                         self.ct(alpha), pa, pb, self.ct(beta),
                         Cm.ctypes.data_as(C.c_void_p))
        return Cm

    def mul(self, A, B):
        return self.gemm(1.0, A, B, 0.0,
                         np.zeros((A.shape[0], B.shape[1]), self.dtype))

    def gemv(self, alpha, A, x, beta, y):
        A, pa = self._arr(A)
        x, px = self._arr(np.asarray(x).reshape(-1))
        y = np.array(y, dtype=self.dtype, copy=True).reshape(-1)
        m, n = A.shape
        self._fn("gemv")(y.ctypes.data_as(C.c_void_p), self.ct(alpha), pa, px,
                         self.ct(beta), C.c_size_t(m), C.c_size_t(n))
        return y

    def gemv_t(self, alpha, A, x, beta, y):
        """y = beta*y + alpha*A^T x (mat_gemv_t)."""
        A, pa = self._arr(A)
        x, px = self._arr(np.asarray(x).reshape(-1))
        y = np.array(y, dtype=self.dtype, copy=True).reshape(-1)
        m, n = A.shape
        self._fn("gemv_t")(y.ctypes.data_as(C.c_void_p), self.ct(alpha), pa,
                           px, self.ct(beta), C.c_size_t(m), C.c_size_t(n))
        return y

    def qr(self, A):
        """(Q, R) exactly as mat_qr fills them (the port: the reference's
        unblocked path, used by the reference for n < 64)."""
        A, pa = self._arr(A)
        m, n = A.shape
        Q = np.zeros((m, m), self.dtype, order="F")
        R = np.zeros((m, n), self.dtype, order="F")
        self._fn("qr")(pa, C.c_size_t(m), C.c_size_t(n),
                       Q.ctypes.data_as(C.c_void_p), R.ctypes.data_as(C.c_void_p))
        return Q, R

    def axpy(self, y, alpha, x):
        """y + alpha*x (mat_axpy)."""
        x, px = self._arr(np.asarray(x).reshape(-1))
        y = np.array(y, dtype=self.dtype, copy=True).reshape(-1)
        self._fn("axpy")(y.ctypes.data_as(C.c_void_p), self.ct(alpha), px,
                         C.c_size_t(y.size))
        return y

    def syrk(self, Cm, A, alpha, beta, uplo="L"):
        A, pa = self._arr(A)
        Cm = np.array(Cm, dtype=self.dtype, order="F", copy=True)
        n, k = A.shape
        self._fn("syrk")(Cm.ctypes.data_as(C.c_void_p), pa, C.c_size_t(n),
                         C.c_size_t(k), self.ct(alpha), self.ct(beta),
                         C.c_char(uplo.encode()))
        return Cm

    def syrk_t(self, Cm, A, alpha, beta, uplo="L"):
        A, pa = self._arr(A)
        Cm = np.array(Cm, dtype=self.dtype, order="F", copy=True)
        k, n = A.shape
        self._fn("syrk_t")(Cm.ctypes.data_as(C.c_void_p), pa, C.c_size_t(n),
                           C.c_size_t(k), self.ct(alpha), self.ct(beta),
                           C.c_char(uplo.encode()))
        return Cm

    # -- factorisations ------------------------------------------------------
    def plu(self, A):
        """Returns (L, U, perm, swaps) exactly as mat_plu fills them."""
        A, pa = self._arr(A)
        n = A.shape[0]
        L = np.zeros((n, n), self.dtype, order="F")
        U = np.zeros((n, n), self.dtype, order="F")
        p = np.zeros(n, np.uint64)
        self._fn("plu").restype = C.c_int
        s = self._fn("plu")(pa, C.c_size_t(n), L.ctypes.data_as(C.c_void_p),
                            U.ctypes.data_as(C.c_void_p),
                            p.ctypes.data_as(C.c_void_p))
        return L, U, p.astype(np.int64), int(s)

    def lu(self, A):
        """Returns (L, U, p, q, swaps) exactly as mat_lu (full pivoting) fills
        them."""
        A, pa = self._arr(A)
        n = A.shape[0]
        L = np.zeros((n, n), self.dtype, order="F")
        U = np.zeros((n, n), self.dtype, order="F")
        p = np.zeros(n, np.uint64)
        q = np.zeros(n, np.uint64)
        self._fn("lu").restype = C.c_int
        s = self._fn("lu")(pa, C.c_size_t(n), L.ctypes.data_as(C.c_void_p),
                           U.ctypes.data_as(C.c_void_p),
                           p.ctypes.data_as(C.c_void_p),
                           q.ctypes.data_as(C.c_void_p))
        return L, U, p.astype(np.int64), q.astype(np.int64), int(s)

    def plu_inplace(self, A):
        """Port only: packed LU, perm, per-step pivot rows and swap count."""
        assert self.kind == "port"
        M = np.array(A, dtype=self.dtype, order="F", copy=True)
        n = M.shape[0]
        p = np.arange(n, dtype=np.uint64)
        ipiv = np.zeros(n, np.uint64)
        self.lib.orc_plu_inplace.restype = C.c_int
        s = self.lib.orc_plu_inplace(M.ctypes.data_as(C.c_void_p),
                                     C.c_size_t(n),
                                     p.ctypes.data_as(C.c_void_p),
                                     ipiv.ctypes.data_as(C.c_void_p))
        return M, p.astype(np.int64), ipiv.astype(np.int64), int(s)

    def chol(self, A):
        """Returns (L, ret) as mat_chol fills them (ret 0 or -1)."""
        A, pa = self._arr(A)
        n = A.shape[0]
        L = np.zeros((n, n), self.dtype, order="F")
        self._fn("chol").restype = C.c_int
        r = self._fn("chol")(pa, C.c_size_t(n), L.ctypes.data_as(C.c_void_p))
        return L, int(r)

    # -- solves --------------------------------------------------------------
    def _tri(self, name, T, b):
        T, pt = self._arr(T)
        b, pb = self._arr(np.asarray(b).reshape(-1))
        n = T.shape[0]
        x = np.zeros(n, self.dtype)
        self._fn(name)(x.ctypes.data_as(C.c_void_p), pt, pb, C.c_size_t(n))
        return x

    def solve_tril(self, L, b):
        return self._tri("solve_tril", L, b)

    def solve_tril_unit(self, L, b):
        return self._tri("solve_tril_unit", L, b)

    def solve_triu(self, U, b):
        return self._tri("solve_triu", U, b)

    def solve_trilt(self, L, b):
        return self._tri("solve_trilt", L, b)

    def solve(self, A, b):
        return self._tri("solve", A, b)

    def solve_spd(self, A, b):
        A, pa = self._arr(A)
        b, pb = self._arr(np.asarray(b).reshape(-1))
        n = A.shape[0]
        x = np.zeros(n, self.dtype)
        self._fn("solve_spd").restype = C.c_int
        r = self._fn("solve_spd")(x.ctypes.data_as(C.c_void_p), pa, pb,
                                  C.c_size_t(n))
        return x, int(r)

    # -- glibc rand stream (reference shim only) -----------------------------
    def srand(self, s):
        self.lib.ref_srand(C.c_uint(s))

    def rand(self):
        return int(self.lib.ref_rand())
