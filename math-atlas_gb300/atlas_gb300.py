"""ctypes binding of libatlas_gb300.so (the C ABI declared in include/atlas_gb300.h).

The host-pointer functions mirror the reference's cblas_* / clapack_* calls on
numpy arrays; the ``*_dev`` functions take device pointers (e.g. torch CUDA
tensors' ``data_ptr()``) and a CUDA stream handle.  There is no fallback: if
the shared library is missing or fails to load, every call raises.
"""
import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libatlas_gb300.so")

RowMajor, ColMajor = 101, 102
NoTrans, Trans, ConjTrans = 111, 112, 113
Upper, Lower = 121, 122
NonUnit, Unit = 131, 132
Left, Right = 141, 142

# every exported symbol of include/atlas_gb300.h
EXPORTS = [
    "cblas_errprn", "cblas_xerbla", "cblas_dgemm", "cblas_sgemm", "cblas_dtrsm", "cblas_strsm",
    "clapack_dgetrf", "clapack_sgetrf", "clapack_dgetrs", "clapack_sgetrs", "clapack_dgesv",
    "clapack_sgesv", "atlg_num_sms", "atlg_stream", "atlg_status", "atlg_dgemm_dev",
    "atlg_dgemm_dev_opts", "atlg_sgemm_dev", "atlg_dtrsm_dev", "atlg_dlaswp_dev", "atlg_dgetrf_dev",
    "atlg_sgetrf_dev", "atlg_sgetrf_tc_dev", "atlg_dlag2s_dev", "atlg_dgetrs_dev", "atlg_launch_count", "atlg_prof_enable", "atlg_prof_collect",
    "atlg_probe_peaks", "atlg_probe_fp64_mma", "atlg_prof_panels", "atlg_prof_panels_collect", "dgesv_mixed", "dgesv_adjoint", "atlg_dgesv_mixed_dev", "atlg_dgesv_adjoint_dev",
    "atlg_dlaswp_noalloc", "dgemm_split", "atlg_dgemm_split_dev", "atlg_sgemm_tf32x3_dev",
    "cblas_dsyrk", "cblas_ssyrk", "clapack_dpotrf", "clapack_spotrf", "clapack_dpotrs", "clapack_spotrs",
    "clapack_dposv", "clapack_sposv", "atlg_dsyrk_dev", "atlg_dpotrf_dev", "atlg_dpotrs_dev",
    "cblas_dtrmm", "cblas_strmm", "cblas_dgemv", "cblas_sgemv", "cblas_dtrsv", "cblas_strsv",
    "atlg_dtrmm_dev", "atlg_dgemv_dev", "atlg_dtrsv_dev", "atlg_strsv_chain_ws", "atlg_strsv_chain_prepare_dev",
    "atlg_strsv_chain_dev",
    "clapack_dtrtri", "clapack_strtri", "clapack_dgetri", "clapack_sgetri", "atlg_dtrtri_dev", "atlg_dgetri_dev",
    "atlg_panel_cluster", "atlg_panel_split", "atlg_lu_defer_rows", "atlg_panel_fuse", "atlg_refine_trsv", "dgesv_split", "atlg_dgetrf_split_dev", "atlg_panel_grid", "atlg_split_lu_leaf", "atlg_panel_width",
    "cblas_idamax", "cblas_isamax", "atlg_idamax_dev", "atlg_isamax_dev",
]

_lib = None


def build(jobs=8):
    subprocess.check_call(["make", "-s", "-j%d" % jobs, "-C", HERE, "libatlas_gb300.so"])


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError("libatlas_gb300.so is not built (run __graft_entry__.build())")
        _lib = C.CDLL(LIB_PATH)
        _declare(_lib)
    return _lib


_dp = np.ctypeslib.ndpointer(dtype=np.float64, flags="F_CONTIGUOUS")
_sp = np.ctypeslib.ndpointer(dtype=np.float32, flags="F_CONTIGUOUS")
_ip = np.ctypeslib.ndpointer(dtype=np.int32, flags="C_CONTIGUOUS")
_v1d = np.ctypeslib.ndpointer(dtype=np.float64, ndim=1, flags="C_CONTIGUOUS")
_v1s = np.ctypeslib.ndpointer(dtype=np.float32, ndim=1, flags="C_CONTIGUOUS")
_i, _d, _f, _v, _u = C.c_int, C.c_double, C.c_float, C.c_void_p, C.c_uint


def _declare(L):
    sig = {
        "cblas_dgemm": (None, [_i, _i, _i, _i, _i, _i, _d, _dp, _i, _dp, _i, _d, _dp, _i]),
        "cblas_sgemm": (None, [_i, _i, _i, _i, _i, _i, _f, _sp, _i, _sp, _i, _f, _sp, _i]),
        "cblas_dtrsm": (None, [_i, _i, _i, _i, _i, _i, _i, _d, _dp, _i, _dp, _i]),
        "cblas_strsm": (None, [_i, _i, _i, _i, _i, _i, _i, _f, _sp, _i, _sp, _i]),
        "clapack_dgetrf": (_i, [_i, _i, _i, _dp, _i, _ip]),
        "clapack_sgetrf": (_i, [_i, _i, _i, _sp, _i, _ip]),
        "clapack_dgetrs": (_i, [_i, _i, _i, _i, _dp, _i, _ip, _dp, _i]),
        "clapack_sgetrs": (_i, [_i, _i, _i, _i, _sp, _i, _ip, _sp, _i]),
        "clapack_dgesv": (_i, [_i, _i, _i, _dp, _i, _ip, _dp, _i]),
        "clapack_sgesv": (_i, [_i, _i, _i, _sp, _i, _ip, _sp, _i]),
        "cblas_dsyrk": (None, [_i, _i, _i, _i, _i, _d, _dp, _i, _d, _dp, _i]),
        "cblas_ssyrk": (None, [_i, _i, _i, _i, _i, _f, _sp, _i, _f, _sp, _i]),
        "clapack_dpotrf": (_i, [_i, _i, _i, _dp, _i]),
        "clapack_spotrf": (_i, [_i, _i, _i, _sp, _i]),
        "clapack_dpotrs": (_i, [_i, _i, _i, _i, _dp, _i, _dp, _i]),
        "clapack_spotrs": (_i, [_i, _i, _i, _i, _sp, _i, _sp, _i]),
        "clapack_dposv": (_i, [_i, _i, _i, _i, _dp, _i, _dp, _i]),
        "clapack_sposv": (_i, [_i, _i, _i, _i, _sp, _i, _sp, _i]),
        "atlg_dsyrk_dev": (_i, [_i, _i, _i, _i, _d, _v, _i, _d, _v, _i, _v]),
        "atlg_dpotrf_dev": (_i, [_i, _i, _v, _i, _v]),
        "atlg_dpotrs_dev": (_i, [_i, _i, _i, _i, _v, _i, _v, _i, _v]),
        "cblas_dtrmm": (None, [_i, _i, _i, _i, _i, _i, _i, _d, _dp, _i, _dp, _i]),
        "cblas_strmm": (None, [_i, _i, _i, _i, _i, _i, _i, _f, _sp, _i, _sp, _i]),
        "cblas_dgemv": (None, [_i, _i, _i, _i, _d, _dp, _i, _v1d, _i, _d, _v1d, _i]),
        "cblas_sgemv": (None, [_i, _i, _i, _i, _f, _sp, _i, _v1s, _i, _f, _v1s, _i]),
        "cblas_dtrsv": (None, [_i, _i, _i, _i, _i, _dp, _i, _v1d, _i]),
        "cblas_strsv": (None, [_i, _i, _i, _i, _i, _sp, _i, _v1s, _i]),
        "atlg_dtrmm_dev": (_i, [_i, _i, _i, _i, _i, _i, _d, _v, _i, _v, _i, _v]),
        "atlg_dgemv_dev": (_i, [_i, _i, _i, _d, _v, _i, _v, _i, _d, _v, _v]),
        "atlg_dtrsv_dev": (_i, [_i, _i, _i, _i, _v, _i, _v, _v]),
        "atlg_strsv_chain_ws": (C.c_size_t, [_i]),
        "atlg_strsv_chain_prepare_dev": (_i, [_i, _i, _i, _v, _i, _v, _v]),
        "atlg_strsv_chain_dev": (_i, [_i, _i, _v, _i, _v, _v, _v]),
        "clapack_dtrtri": (_i, [_i, _i, _i, _i, _dp, _i]),
        "clapack_strtri": (_i, [_i, _i, _i, _i, _sp, _i]),
        "clapack_dgetri": (_i, [_i, _i, _dp, _i, _ip]),
        "clapack_sgetri": (_i, [_i, _i, _sp, _i, _ip]),
        "atlg_dtrtri_dev": (_i, [_i, _i, _i, _i, _v, _i, _v]),
        "atlg_dgetri_dev": (_i, [_i, _v, _i, _v, _v]),
        "atlg_panel_cluster": (None, [_i]),
        "atlg_panel_split": (None, [_i]),
        "atlg_lu_defer_rows": (None, [_i]),
        "atlg_panel_fuse": (None, [_i]),
        "atlg_refine_trsv": (None, [_i]),
        "atlg_panel_grid": (None, [_i]),
        "atlg_split_lu_leaf": (None, [_i]),
        "atlg_panel_width": (None, [_i]),
        "dgesv_split": (_i, [_i, _i, _dp, _i, _ip, _dp, _i]),
        "atlg_dgetrf_split_dev": (_i, [_i, _v, _i, _v, _i, _i, _v]),
        "atlg_num_sms": (_i, []),
        "atlg_stream": (_v, []),
        "atlg_status": (_u, []),
        "atlg_dgemm_dev": (_i, [_i, _i, _i, _i, _i, _d, _v, _i, _v, _i, _d, _v, _i, _v]),
        "atlg_dgemm_dev_opts": (_i, [_i, _i, _i, _i, _i, _d, _v, _i, _v, _i, _d, _v, _i, _i, _v]),
        "atlg_sgemm_dev": (_i, [_i, _i, _i, _i, _i, _f, _v, _i, _v, _i, _f, _v, _i, _v]),
        "atlg_dtrsm_dev": (_i, [_i, _i, _i, _i, _i, _i, _d, _v, _i, _v, _i, _v]),
        "atlg_dlaswp_dev": (_i, [_i, _v, _i, _i, _i, _v, _i, _i, _v]),
        "cblas_idamax": (_i, [_i, _v1d, _i]),
        "cblas_isamax": (_i, [_i, _v1s, _i]),
        "atlg_idamax_dev": (_i, [_i, _v, _i, _v, _v]),
        "atlg_isamax_dev": (_i, [_i, _v, _i, _v, _v]),
        "atlg_dlaswp_noalloc": (_i, [_i, _v, _i, _i, _i, _v, _i, _i, _v]),
        "atlg_dgetrf_dev": (_i, [_i, _i, _v, _i, _v, _v, _v]),
        "atlg_sgetrf_dev": (_i, [_i, _i, _v, _i, _v, _v, _v]),
        "atlg_sgetrf_tc_dev": (_i, [_i, _i, _v, _i, _v, _v, _v]),
        "atlg_dlag2s_dev": (_i, [_i, _i, _v, _i, _v, _i, _v]),
        "atlg_dgetrs_dev": (_i, [_i, _i, _i, _i, _v, _i, _v, _v, _i, _v]),
        "dgesv_mixed": (_i, [_i, _i, _dp, _i, _ip, _dp, _i, _dp, _i, np.ctypeslib.ndpointer(np.float64),
                             np.ctypeslib.ndpointer(np.float64), C.POINTER(_i), C.POINTER(_i)]),
        "dgesv_adjoint": (_i, [_i, _i, _dp, _i, _ip, _dp, _i, _dp, _i, _dp, _i, _dp, _i]),
        "atlg_dgesv_mixed_dev": (_i, [_i, _i, _v, _i, _v, _v, _i, _v, _i, C.POINTER(_d), C.POINTER(_d),
                                      C.POINTER(_i), C.POINTER(_i), _v]),
        "atlg_dgesv_adjoint_dev": (_i, [_i, _i, _v, _i, _v, _v, _i, _v, _i, _v, _i, _v, _i, _v]),
        "dgemm_split": (None, [_i, _i, _i, _i, _i, _i, _d, _dp, _i, _dp, _i, _d, _dp, _i, _i]),
        "atlg_dgemm_split_dev": (_i, [_i, _i, _i, _i, _i, _d, _v, _i, _v, _i, _d, _v, _i, _i, _v]),
        "atlg_sgemm_tf32x3_dev": (_i, [_i, _i, _i, _f, _v, _i, _v, _i, _v, _i, _v]),
        "atlg_launch_count": (C.c_ulonglong, []),
        "atlg_prof_enable": (None, [_i]),
        "atlg_prof_collect": (_i, [C.POINTER(_d), C.POINTER(_d), C.POINTER(_i)]),
        "atlg_probe_peaks": (None, [C.POINTER(_d), C.POINTER(_d)]),
        "atlg_probe_fp64_mma": (None, [C.POINTER(_d), C.POINTER(_d), C.POINTER(_d)]),
        "atlg_prof_panels": (None, [_i]),
        "atlg_prof_panels_collect": (_i, [C.POINTER(_d), C.POINTER(_d), C.POINTER(_i)]),
    }
    for name, (res, args) in sig.items():
        fn = getattr(L, name)
        fn.restype = res
        fn.argtypes = args


def _f64(a):
    if not (a.dtype == np.float64 and a.flags.f_contiguous):
        raise TypeError("expected a Fortran-ordered float64 array")
    return a


# ------------------------------------------------------------ host-pointer API
def cblas_dgemm(order, ta, tb, M, N, K, alpha, A, lda, B, ldb, beta, Cm, ldc):
    lib().cblas_dgemm(order, ta, tb, M, N, K, alpha, A, lda, B, ldb, beta, Cm, ldc)


def cblas_sgemm(order, ta, tb, M, N, K, alpha, A, lda, B, ldb, beta, Cm, ldc):
    lib().cblas_sgemm(order, ta, tb, M, N, K, alpha, A, lda, B, ldb, beta, Cm, ldc)


def cblas_dtrsm(order, side, uplo, ta, diag, M, N, alpha, A, lda, B, ldb):
    lib().cblas_dtrsm(order, side, uplo, ta, diag, M, N, alpha, A, lda, B, ldb)


def cblas_strsm(order, side, uplo, ta, diag, M, N, alpha, A, lda, B, ldb):
    lib().cblas_strsm(order, side, uplo, ta, diag, M, N, alpha, A, lda, B, ldb)


def clapack_dgetrf(order, M, N, A, lda, ipiv):
    return lib().clapack_dgetrf(order, M, N, A, lda, ipiv)


def clapack_sgetrf(order, M, N, A, lda, ipiv):
    return lib().clapack_sgetrf(order, M, N, A, lda, ipiv)


def clapack_dgetrs(order, trans, N, NRHS, A, lda, ipiv, B, ldb):
    return lib().clapack_dgetrs(order, trans, N, NRHS, A, lda, ipiv, B, ldb)


def clapack_dgesv(order, N, NRHS, A, lda, ipiv, B, ldb):
    return lib().clapack_dgesv(order, N, NRHS, A, lda, ipiv, B, ldb)


def clapack_sgesv(order, N, NRHS, A, lda, ipiv, B, ldb):
    return lib().clapack_sgesv(order, N, NRHS, A, lda, ipiv, B, ldb)


def cblas_dtrmm(order, side, uplo, ta, diag, M, N, alpha, A, lda, B, ldb):
    lib().cblas_dtrmm(order, side, uplo, ta, diag, M, N, alpha, A, lda, B, ldb)


def cblas_strmm(order, side, uplo, ta, diag, M, N, alpha, A, lda, B, ldb):
    lib().cblas_strmm(order, side, uplo, ta, diag, M, N, alpha, A, lda, B, ldb)


def cblas_idamax(N, X, incx):
    return int(lib().cblas_idamax(N, np.ascontiguousarray(X, dtype=np.float64), incx))


def cblas_isamax(N, X, incx):
    return int(lib().cblas_isamax(N, np.ascontiguousarray(X, dtype=np.float32), incx))


def cblas_dgemv(order, ta, M, N, alpha, A, lda, X, incx, beta, Y, incy):
    lib().cblas_dgemv(order, ta, M, N, alpha, A, lda, X, incx, beta, Y, incy)


def cblas_sgemv(order, ta, M, N, alpha, A, lda, X, incx, beta, Y, incy):
    lib().cblas_sgemv(order, ta, M, N, alpha, A, lda, X, incx, beta, Y, incy)


def cblas_dtrsv(order, uplo, ta, diag, N, A, lda, X, incx):
    lib().cblas_dtrsv(order, uplo, ta, diag, N, A, lda, X, incx)


def cblas_strsv(order, uplo, ta, diag, N, A, lda, X, incx):
    lib().cblas_strsv(order, uplo, ta, diag, N, A, lda, X, incx)


def cblas_dsyrk(order, uplo, trans, N, K, alpha, A, lda, beta, Cm, ldc):
    lib().cblas_dsyrk(order, uplo, trans, N, K, alpha, A, lda, beta, Cm, ldc)


def cblas_ssyrk(order, uplo, trans, N, K, alpha, A, lda, beta, Cm, ldc):
    lib().cblas_ssyrk(order, uplo, trans, N, K, alpha, A, lda, beta, Cm, ldc)


def clapack_dpotrf(order, uplo, N, A, lda):
    return lib().clapack_dpotrf(order, uplo, N, A, lda)


def clapack_spotrf(order, uplo, N, A, lda):
    return lib().clapack_spotrf(order, uplo, N, A, lda)


def clapack_dpotrs(order, uplo, N, NRHS, A, lda, B, ldb):
    return lib().clapack_dpotrs(order, uplo, N, NRHS, A, lda, B, ldb)


def clapack_spotrs(order, uplo, N, NRHS, A, lda, B, ldb):
    return lib().clapack_spotrs(order, uplo, N, NRHS, A, lda, B, ldb)


def clapack_dposv(order, uplo, N, NRHS, A, lda, B, ldb):
    return lib().clapack_dposv(order, uplo, N, NRHS, A, lda, B, ldb)


def clapack_sposv(order, uplo, N, NRHS, A, lda, B, ldb):
    return lib().clapack_sposv(order, uplo, N, NRHS, A, lda, B, ldb)


def clapack_dtrtri(order, uplo, diag, N, A, lda):
    return lib().clapack_dtrtri(order, uplo, diag, N, A, lda)


def clapack_strtri(order, uplo, diag, N, A, lda):
    return lib().clapack_strtri(order, uplo, diag, N, A, lda)


def clapack_dgetri(order, N, A, lda, ipiv):
    return lib().clapack_dgetri(order, N, A, lda, ipiv)


def clapack_sgetri(order, N, A, lda, ipiv):
    return lib().clapack_sgetri(order, N, A, lda, ipiv)


def dgesv_split(N, NRHS, A, lda, ipiv, B, ldb):
    return lib().dgesv_split(N, NRHS, A, lda, ipiv, B, ldb)


def dgemm_split(ta, tb, alpha, A, B, beta, Cm, nslices=7):
    M, N = Cm.shape
    K = A.shape[1] if ta == NoTrans else A.shape[0]
    lib().dgemm_split(ColMajor, ta, tb, M, N, K, alpha, A, A.shape[0], B, B.shape[0], beta, Cm, Cm.shape[0],
                      nslices)
    return Cm


def dgesv_mixed(A, ipiv, B, X):
    """Mixed-precision solve on Fortran arrays; returns (info, berr, ferr, iters, status)."""
    n, nrhs = B.shape
    berr = np.zeros(max(nrhs, 1))
    ferr = np.zeros(max(nrhs, 1))
    it, stt = _i(), _i()
    info = lib().dgesv_mixed(n, nrhs, A, A.shape[0], ipiv, B, B.shape[0], X, X.shape[0], berr, ferr,
                             C.byref(it), C.byref(stt))
    return info, berr[:nrhs], ferr[:nrhs], it.value, stt.value


def dgesv_adjoint(LU, ipiv, X, gX):
    n, nrhs = X.shape
    gA = np.zeros((n, n), order="F")
    gB = np.zeros((n, nrhs), order="F")
    lib().dgesv_adjoint(n, nrhs, LU, LU.shape[0], ipiv, X, X.shape[0], gX, gX.shape[0], gA, n, gB, n)
    return gA, gB


# convenience wrappers on whole arrays (column-major)
def dgemm(ta, tb, alpha, A, B, beta, Cm):
    M, N = Cm.shape
    K = A.shape[1] if ta == NoTrans else A.shape[0]
    f = cblas_dgemm if Cm.dtype == np.float64 else cblas_sgemm
    f(ColMajor, ta, tb, M, N, K, alpha, A, A.shape[0], B, B.shape[0], beta, Cm, Cm.shape[0])
    return Cm


def getrf(A, order=ColMajor, M=None, N=None):
    M = A.shape[0] if M is None else M
    N = A.shape[1] if N is None else N
    ipiv = np.zeros(max(min(M, N), 1), dtype=np.int32)
    f = clapack_dgetrf if A.dtype == np.float64 else clapack_sgetrf
    info = f(order, M, N, A, A.shape[0], ipiv)
    return info, ipiv[: min(M, N)]


# ---------------------------------------------------------- device-pointer API
def status():
    return lib().atlg_status()


def num_sms():
    return lib().atlg_num_sms()


def launch_count():
    return int(lib().atlg_launch_count())


def prof_enable(on=True):
    lib().atlg_prof_enable(1 if on else 0)


def prof_collect():
    ms, fl, n = _d(), _d(), _i()
    lib().atlg_prof_collect(C.byref(ms), C.byref(fl), C.byref(n))
    return ms.value, fl.value, n.value


def probe_peaks():
    a, b = _d(), _d()
    lib().atlg_probe_peaks(C.byref(a), C.byref(b))
    return a.value, b.value


def probe_fp64_mma():
    """FP64 mma.sync throughput (TFLOP/s) for shapes m8n8k4, m16n8k4, m16n8k16."""
    a, b, c = _d(), _d(), _d()
    lib().atlg_probe_fp64_mma(C.byref(a), C.byref(b), C.byref(c))
    return {"m8n8k4": a.value, "m16n8k4": b.value, "m16n8k16": c.value}
