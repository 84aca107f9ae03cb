"""Python view of libmatgb, the GB300 build of libmat's dense-solve hot path.

The product is the C-ABI shared library (libmat_gb300/lib/libmatgb_f32.so and
libmatgb_f64.so, declared by include/mat.h and include/matgb.h).  This module
only loads it with ctypes and mirrors mat.h's functions for numpy arrays, so
tests and benchmarks read like the reference's own C tests.  There is no
fallback: if the library is missing, loading raises.

Arrays are column-major (Fortran order) like the reference's Mat
(mat.h:389, MAT_IDX = j*rows + i).
"""
import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIBDIR = os.path.join(HERE, "lib")


class MatStruct(C.Structure):
    _fields_ = [("rows", C.c_size_t), ("cols", C.c_size_t),
                ("data", C.c_void_p)]


class PermStruct(C.Structure):
    _fields_ = [("data", C.c_void_p), ("size", C.c_size_t)]


class MatIROpts(C.Structure):
    _fields_ = [("lp_format", C.c_int), ("max_iter", C.c_int),
                ("tol", C.c_double), ("fp32_fallback", C.c_int),
                ("krylov", C.c_int), ("krylov_dim", C.c_int)]


class MatIRReport(C.Structure):
    _fields_ = [("iterations", C.c_int), ("converged", C.c_int),
                ("lp_format", C.c_int), ("backward_error", C.c_double),
                ("residual_inf", C.c_double), ("x_inf", C.c_double),
                ("a_inf", C.c_double), ("b_inf", C.c_double),
                ("tol", C.c_double), ("ms_factor", C.c_double),
                ("ms_refine", C.c_double), ("refinements", C.c_int),
                ("krylov_steps", C.c_int), ("forward_error_est", C.c_double)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class MatGBError(RuntimeError):
    pass


def lib_path(prec):
    return os.path.join(LIBDIR, f"libmatgb_{prec}.so")


_P = C.c_void_p
_S = C.c_size_t
_I = C.c_int


class Lib:
    """One precision build ("f32" or "f64") of libmatgb."""

    def __init__(self, prec="f32"):
        assert prec in ("f32", "f64")
        path = lib_path(prec)
        if not os.path.exists(path):
            raise FileNotFoundError(
                f"{path} is missing: build it with `python -m libmat_gb300.build`")
        self.prec = prec
        self.dtype = np.float32 if prec == "f32" else np.float64
        self.ct = C.c_float if prec == "f32" else C.c_double
        self.c = C.CDLL(path, mode=C.RTLD_LOCAL)
        self._sig()
        self.c.matgb_set_abort_on_error(0)

    # ------------------------------------------------------------------ ABI
    def _sig(self):
        c, E = self.c, self.ct
        MP = C.POINTER(MatStruct)
        PP = C.POINTER(PermStruct)
        sigs = {
            "matgb_init": (_I, [_I]),
            "matgb_elem_size": (_I, []),
            "matgb_last_error": (C.c_char_p, []),
            "matgb_clear_error": (None, []),
            "matgb_set_abort_on_error": (None, [_I]),
            "matgb_sync": (_I, []),
            "matgb_stream": (_P, []),
            "matgb_launch_count": (C.c_ulonglong, []),
            "matgb_sm_count": (_I, []),
            "matgb_ktime_enable": (_I, [_I]),
            "matgb_ktime_get": (_I, [_I, C.c_char_p, _I,
                                     C.POINTER(C.c_longlong),
                                     C.POINTER(C.c_double),
                                     C.POINTER(C.c_double),
                                     C.POINTER(C.c_double)]),
            "matgb_ktime_trace": (_I, [_I, C.c_char_p, _I,
                                       C.POINTER(C.c_double),
                                       C.POINTER(C.c_double),
                                       C.POINTER(C.c_int)]),
            "matgb_measure_fma_peak": (C.c_double, [_I]),
            "matgb_plain_tensor_core": (_I, [_I]),
            "matgb_device_alloc": (_P, [_S]),
            "matgb_device_free": (_I, [_P]),
            "matgb_host_alloc": (_P, [_S]),
            "matgb_host_free": (_I, [_P]),
            "matgb_memcpy_h2d": (_I, [_P, _P, _S]),
            "matgb_memcpy_d2h": (_I, [_P, _P, _S]),
            "matgb_memcpy_d2d": (_I, [_P, _P, _S]),
            "matgb_memset_dev": (_I, [_P, _I, _S]),
            "matgb_event_record": (_I, [_I]),
            "matgb_event_elapsed_ms": (C.c_double, [_I, _I]),
            "matgb_fill_uniform_dev": (_I, [_P, _S, C.c_uint64, C.c_double,
                                            C.c_double]),
            "matgb_fill_normal_dev": (_I, [_P, _S, C.c_uint64]),
            "matgb_add_diag_dev": (_I, [_P, _S, _S, C.c_double]),
            "matgb_gemm_dev": (_I, [C.c_char, C.c_char, _S, _S, _S, E, _P, _S,
                                    _P, _S, E, _P, _S]),
            "matgb_syrk_dev": (_I, [C.c_char, C.c_char, _S, _S, E, _P, _S, E,
                                    _P, _S]),
            "matgb_getrf_dev": (_I, [_S, _P, _S, _P, _P]),
            "matgb_getrf_full_dev": (_I, [_S, _P, _S, _P, _P]),
            "matgb_getrs_dev": (_I, [_S, _S, _P, _S, _P, _P, _S, _P, _S]),
            "matgb_potrf_dev": (_I, [_S, _P, _S, _P]),
            "matgb_potrs_dev": (_I, [_S, _S, _P, _S, _P, _S, _P]),
            "matgb_trsm_dev": (_I, [C.c_char, C.c_char, C.c_char, _S, _S, _P,
                                    _S, _P, _S]),
            "matgb_gemv_dev": (_I, [_S, _S, E, _P, _S, _P, E, _P]),
            "matgb_gemv_t_dev": (_I, [_S, _S, E, _P, _S, _P, E, _P]),
            "matgb_axpy_dev": (_I, [_S, E, _P, _P]),
            "matgb_solve_multi": (None, [MP, MP, MP]),
            "matgb_solve_spd_multi": (_I, [MP, MP, MP]),
            "mat_mul": (None, [MP, MP, MP]),
            "mat_rmul": (MP, [MP, MP]),
            "mat_gemm": (None, [MP, E, MP, MP, E]),
            "mat_gemv": (None, [MP, E, MP, MP, E]),
            "mat_gemv_t": (None, [MP, E, MP, MP, E]),
            "mat_axpy": (None, [MP, E, MP]),
            "mat_syrk": (None, [MP, MP, E, E, C.c_char]),
            "mat_syrk_t": (None, [MP, MP, E, E, C.c_char]),
            "mat_plu": (_I, [MP, MP, MP, PP]),
            "mat_lu": (_I, [MP, MP, MP, PP, PP]),
            "mat_chol": (_I, [MP, MP]),
            "mat_det": (E, [MP]),
            "mat_inv": (None, [MP, MP]),
            "mat_qr": (None, [MP, MP, MP]),
            "mat_qr_r": (None, [MP, MP]),
            "matgb_qr_dev": (_I, [_S, _S, _P, _S, _P, _S]),
            "mat_solve": (None, [MP, MP, MP]),
            "mat_solve_spd": (_I, [MP, MP, MP]),
            "mat_solve_tril": (None, [MP, MP, MP]),
            "mat_solve_tril_unit": (None, [MP, MP, MP]),
            "mat_solve_triu": (None, [MP, MP, MP]),
            "mat_solve_trilt": (None, [MP, MP, MP]),
            "mat_free_mat": (None, [MP]),
            "matgb_tc_gemm_dev": (_I, [_I, _S, _S, _S, _P, _S, _P, _S,
                                       C.c_float, C.c_float, _P, _S]),
            "matgb_tc_status": (_I, []),
            "matgb_tc_persistent": (_I, [_I]),
            "matgb_la_prep": (_I, [_I]),
            "matgb_chol_lookahead": (_I, [_I]),
            "matgb_tc_gemm_split_dev": (_I, [_S, _S, _S, _P, _P, _S, _P, _P, _S,
                                             C.c_float, C.c_float, _P, _S]),
            "matgb_getrf_lp_dev": (_I, [_S, _P, _S, _P, _P, _I]),
            "matgb_ir_default_opts": (None, [C.POINTER(MatIROpts)]),
            "matgb_gesv_ir_dev": (_I, [_S, _P, _S, _P, _P,
                                       C.POINTER(MatIROpts),
                                       C.POINTER(MatIRReport)]),
            "mat_solve_ir": (_I, [MP, MP, MP, C.POINTER(MatIROpts),
                                  C.POINTER(MatIRReport)]),
            "matgb_gemv_noalloc_dev": (_I, [_S, _S, E, _P, _S, _P, E, _P,
                                            _P]),
            "matgb_solve_batched_dev": (_I, [C.c_int64, _P, _P, _P, _P, _P,
                                             _P, _P, _P]),
            "matgb_batched_tune": (_I, [_I, _I, _I, _I]),
            "matgb_batched_tune_get": (_I, [_I, _I, C.POINTER(_I), C.POINTER(_I)]),
            "matgb_batched_tune_source": (C.c_char_p, []),
            "matgb_batched_schedule": (_I, [_I, _I, _I]),
            "matgb_batched_mixed": (_I, [_I]),
            "matgb_batched_mixed_tune": (_I, [_I, _I, _I]),
            "matgb_batched_mixed_stats": (_I, [C.POINTER(_I), C.POINTER(_I), C.POINTER(_I)]),
            "matgb_library_dir": (C.c_char_p, []),
            "matgb_gesv_ir_multi_dev": (_I, [_S, _S, _P, _S, _P, _S, _P, _S,
                                             C.POINTER(MatIROpts),
                                             C.POINTER(MatIRReport)]),
            "matgb_posv_ir_dev": (_I, [_S, _S, _P, _S, _P, _S, _P, _S,
                                       C.POINTER(MatIROpts),
                                       C.POINTER(MatIRReport)]),
            "mat_solve_spd_ir": (_I, [MP, MP, MP, C.POINTER(MatIROpts),
                                      C.POINTER(MatIRReport)]),
            "matgb_potrf_lp_dev": (_I, [_S, _P, _S, _P, _I]),
            "matgb_resid64_dev": (_I, [_S, _S, _P, _S, _P, _S, _P, _S]),
            "matgb_resid64_mode": (_I, [_I]),
        }
        for name, (res, args) in sigs.items():
            f = getattr(c, name)
            f.restype = res
            f.argtypes = args

    def check(self, rc=0, where=""):
        msg = self.c.matgb_last_error()
        if rc not in (0, None) or (msg and len(msg) > 0):
            self.c.matgb_clear_error()
            raise MatGBError(f"{where}: rc={rc} {msg.decode() if msg else ''}")

    # ------------------------------------------------------------ helpers
    def arr(self, a, shape=None):
        a = np.asarray(a, dtype=self.dtype)
        if a.ndim == 1:
            a = a.reshape(-1, 1)
        return np.asfortranarray(a)

    def mat(self, a):
        """Mat view over a Fortran-ordered numpy array (kept alive by caller)."""
        assert a.flags.f_contiguous and a.dtype == self.dtype
        return MatStruct(a.shape[0], a.shape[1], a.ctypes.data)

    # ------------------------------------------------------ mat.h mirrors
    def mat_mul(self, a, b):
        a, b = self.arr(a), self.arr(b)
        out = np.zeros((a.shape[0], b.shape[1]), self.dtype, order="F")
        self.c.mat_mul(C.byref(self.mat(out)), C.byref(self.mat(a)),
                       C.byref(self.mat(b)))
        self.check(0, "mat_mul")
        return out

    def mat_rmul(self, a, b):
        a, b = self.arr(a), self.arr(b)
        r = self.c.mat_rmul(C.byref(self.mat(a)), C.byref(self.mat(b)))
        self.check(0, "mat_rmul")
        m = r.contents
        out = np.ctypeslib.as_array(
            C.cast(m.data, C.POINTER(self.ct)), shape=(m.rows * m.cols,))
        out = out.reshape((m.rows, m.cols), order="F").copy(order="F")
        self.c.mat_free_mat(r)
        return out

    def mat_gemm(self, Cm, alpha, A, B, beta):
        A, B = self.arr(A), self.arr(B)
        Cm = np.array(self.arr(Cm), order="F", copy=True)
        self.c.mat_gemm(C.byref(self.mat(Cm)), self.ct(alpha),
                        C.byref(self.mat(A)), C.byref(self.mat(B)),
                        self.ct(beta))
        self.check(0, "mat_gemm")
        return Cm

    def mat_gemv(self, y, alpha, A, x, beta):
        A, x = self.arr(A), self.arr(x)
        y = np.array(self.arr(y), order="F", copy=True)
        self.c.mat_gemv(C.byref(self.mat(y)), self.ct(alpha),
                        C.byref(self.mat(A)), C.byref(self.mat(x)),
                        self.ct(beta))
        self.check(0, "mat_gemv")
        return y.reshape(-1)

    def mat_gemv_t(self, y, alpha, A, x, beta):
        A, x = self.arr(A), self.arr(x)
        y = np.array(self.arr(y), order="F", copy=True)
        self.c.mat_gemv_t(C.byref(self.mat(y)), self.ct(alpha),
                          C.byref(self.mat(A)), C.byref(self.mat(x)),
                          self.ct(beta))
        self.check(0, "mat_gemv_t")
        return y.reshape(-1)

    def mat_axpy(self, y, alpha, x):
        x = self.arr(x)
        y = np.array(self.arr(y), order="F", copy=True)
        self.c.mat_axpy(C.byref(self.mat(y)), self.ct(alpha),
                        C.byref(self.mat(x)))
        self.check(0, "mat_axpy")
        return y.reshape(-1)

    def mat_syrk(self, Cm, A, alpha, beta, uplo="L", trans=False):
        A = self.arr(A)
        Cm = np.array(self.arr(Cm), order="F", copy=True)
        f = self.c.mat_syrk_t if trans else self.c.mat_syrk
        f(C.byref(self.mat(Cm)), C.byref(self.mat(A)), self.ct(alpha),
          self.ct(beta), C.c_char(uplo.encode()))
        self.check(0, "mat_syrk")
        return Cm

    def mat_plu(self, A):
        A = self.arr(A)
        n = A.shape[0]
        L = np.zeros((n, n), self.dtype, order="F")
        U = np.zeros((n, n), self.dtype, order="F")
        pd = np.zeros(n, np.uint64)
        p = PermStruct(pd.ctypes.data, n)
        s = self.c.mat_plu(C.byref(self.mat(A)), C.byref(self.mat(L)),
                           C.byref(self.mat(U)), C.byref(p))
        self.check(0, "mat_plu")
        return L, U, pd.astype(np.int64), int(s)

    def mat_lu(self, A):
        """mat_lu (full pivoting): (L, U, p, q, swaps)."""
        A = self.arr(A)
        n = A.shape[0]
        L = np.zeros((n, n), self.dtype, order="F")
        U = np.zeros((n, n), self.dtype, order="F")
        pd = np.zeros(n, np.uint64)
        qd = np.zeros(n, np.uint64)
        p = PermStruct(pd.ctypes.data, n)
        q = PermStruct(qd.ctypes.data, n)
        s = self.c.mat_lu(C.byref(self.mat(A)), C.byref(self.mat(L)),
                          C.byref(self.mat(U)), C.byref(p), C.byref(q))
        self.check(0, "mat_lu")
        return L, U, pd.astype(np.int64), qd.astype(np.int64), int(s)

    def mat_chol(self, A):
        A = self.arr(A)
        n = A.shape[0]
        L = np.zeros((n, n), self.dtype, order="F")
        r = self.c.mat_chol(C.byref(self.mat(A)), C.byref(self.mat(L)))
        self.check(0, "mat_chol")
        return L, int(r)

    def mat_det(self, A):
        A = self.arr(A)
        d = self.c.mat_det(C.byref(self.mat(A)))
        self.check(0, "mat_det")
        return float(d)

    def mat_inv(self, A):
        A = self.arr(A)
        out = np.zeros_like(A, order="F")
        self.c.mat_inv(C.byref(self.mat(out)), C.byref(self.mat(A)))
        self.check(0, "mat_inv")
        return out

    def mat_qr(self, A, want_q=True):
        """(Q, R) from mat_qr, or R alone from mat_qr_r."""
        A = self.arr(A)
        m, n = A.shape
        R = np.zeros((m, n), self.dtype, order="F")
        if want_q:
            Q = np.zeros((m, m), self.dtype, order="F")
            self.c.mat_qr(C.byref(self.mat(A)), C.byref(self.mat(Q)),
                          C.byref(self.mat(R)))
            self.check(0, "mat_qr")
            return Q, R
        self.c.mat_qr_r(C.byref(self.mat(A)), C.byref(self.mat(R)))
        self.check(0, "mat_qr_r")
        return R

    def _vec_call(self, name, A, b):
        A, b = self.arr(A), self.arr(b)
        x = np.zeros((A.shape[1], 1), self.dtype, order="F")
        r = getattr(self.c, name)(C.byref(self.mat(x)), C.byref(self.mat(A)),
                                  C.byref(self.mat(b)))
        self.check(0, name)
        return x.reshape(-1), r

    def mat_solve(self, A, b):
        return self._vec_call("mat_solve", A, b)[0]

    def mat_solve_spd(self, A, b):
        x, r = self._vec_call("mat_solve_spd", A, b)
        return x, int(r)

    def mat_solve_tril(self, L, b):
        return self._vec_call("mat_solve_tril", L, b)[0]

    def mat_solve_tril_unit(self, L, b):
        return self._vec_call("mat_solve_tril_unit", L, b)[0]

    def mat_solve_triu(self, U, b):
        return self._vec_call("mat_solve_triu", U, b)[0]

    def mat_solve_trilt(self, L, b):
        return self._vec_call("mat_solve_trilt", L, b)[0]

    def solve_multi(self, A, B, spd=False):
        A, B = self.arr(A), self.arr(B)
        X = np.zeros((A.shape[1], B.shape[1]), self.dtype, order="F")
        f = self.c.matgb_solve_spd_multi if spd else self.c.matgb_solve_multi
        r = f(C.byref(self.mat(X)), C.byref(self.mat(A)), C.byref(self.mat(B)))
        self.check(0, "solve_multi")
        return (X, int(r)) if spd else X

    def ir_opts(self, **kw):
        """MatIROpts with the library defaults, fields overridden by kw."""
        o = MatIROpts()
        self.c.matgb_ir_default_opts(C.byref(o))
        for k, v in kw.items():
            if v is not None:
                setattr(o, k, v)
        return o

    def mat_solve_ir(self, A, b, lp_format=None, max_iter=None, tol=0.0,
                     fp32_fallback=1, krylov=None, krylov_dim=None):
        """Mixed-precision LU + refinement; returns (x, report dict)."""
        A, b = self.arr(A), self.arr(b)
        x = np.zeros((A.shape[1], 1), self.dtype, order="F")
        o = self.ir_opts(lp_format=lp_format, max_iter=max_iter, tol=tol,
                         fp32_fallback=fp32_fallback, krylov=krylov,
                         krylov_dim=krylov_dim)
        rep = MatIRReport()
        rc = self.c.mat_solve_ir(C.byref(self.mat(x)), C.byref(self.mat(A)),
                                 C.byref(self.mat(b)), C.byref(o), C.byref(rep))
        self.check(rc, "mat_solve_ir")
        return x.reshape(-1), rep.as_dict()

    def solve_batched(self, mats, rhs, kinds):
        """Solve many small systems in one pass.  mats: list of square arrays,
        rhs: list of vectors, kinds: 0 (LU) / 1 (Cholesky) per system.
        Returns (list of solutions, status array)."""
        count = len(mats)
        ns = np.array([m.shape[0] for m in mats], np.int32)
        offA = np.zeros(count, np.int64)
        offv = np.zeros(count, np.int64)
        offA[1:] = np.cumsum(ns.astype(np.int64) ** 2)[:-1]
        offv[1:] = np.cumsum(ns.astype(np.int64))[:-1]
        Acat = np.concatenate([np.asarray(m, self.dtype).ravel(order="F")
                               for m in mats])
        bcat = np.concatenate([np.asarray(v, self.dtype).ravel() for v in rhs])
        kd = np.asarray(kinds, np.uint8)
        bufs = [self.dalloc(a.nbytes) for a in (ns, offA, offv, Acat, bcat, bcat, kd)]
        st = self.dalloc(4 * count)
        try:
            for d, a in zip(bufs, (ns, offA, offv, Acat, bcat, bcat, kd)):
                self.h2d(d, a)
            rc = self.c.matgb_solve_batched_dev(count, bufs[0], bufs[1], bufs[3],
                                                bufs[2], bufs[4], bufs[5],
                                                bufs[6], st)
            self.check(rc, "solve_batched")
            x = np.empty_like(bcat)
            self.d2h(x, bufs[5])
            status = np.empty(count, np.int32)
            self.d2h(status, st)
        finally:
            for d in bufs + [st]:
                self.dfree(d)
        return [x[o:o + k] for o, k in zip(offv, ns)], status

    def mat_solve_spd_ir(self, A, B, lp_format=None, max_iter=None, tol=0.0,
                         fp32_fallback=1, krylov=None, krylov_dim=None):
        """Mixed-precision Cholesky + refinement, many RHS; (X, ret, report)."""
        A, B = self.arr(A), self.arr(B)
        X = np.zeros((A.shape[1], B.shape[1]), self.dtype, order="F")
        o = self.ir_opts(lp_format=lp_format, max_iter=max_iter, tol=tol,
                         fp32_fallback=fp32_fallback, krylov=krylov,
                         krylov_dim=krylov_dim)
        rep = MatIRReport()
        rc = self.c.mat_solve_spd_ir(C.byref(self.mat(X)), C.byref(self.mat(A)),
                                     C.byref(self.mat(B)), C.byref(o),
                                     C.byref(rep))
        if rc not in (0, -1):
            self.check(rc, "mat_solve_spd_ir")
        return X, int(rc), rep.as_dict()

    # --------------------------------------------------- device helpers
    def dalloc(self, nbytes):
        p = self.c.matgb_device_alloc(nbytes)
        if not p:
            self.check(-3, "device_alloc")
        return p

    def dfree(self, p):
        self.check(self.c.matgb_device_free(p), "device_free")

    def h2d(self, dst, a):
        a = np.ascontiguousarray(a) if not a.flags.f_contiguous else a
        self.check(self.c.matgb_memcpy_h2d(dst, a.ctypes.data, a.nbytes), "h2d")

    def d2h(self, a, src):
        self.check(self.c.matgb_memcpy_d2h(a.ctypes.data, src, a.nbytes), "d2h")
        self.sync()

    def sync(self):
        self.check(self.c.matgb_sync(), "sync")

    def launches(self):
        return int(self.c.matgb_launch_count())


_libs = {}


def load(prec="f32"):
    """Load (once) and return the Lib for a precision."""
    if prec not in _libs:
        _libs[prec] = Lib(prec)
    return _libs[prec]
