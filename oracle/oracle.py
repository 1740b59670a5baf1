"""ctypes binding of the CPU oracle (oracle/liboracle.so).

TEST INFRASTRUCTURE ONLY.  The oracle is a CPU restatement of ATLAS 3.11.42's
Level-3 / LU path (see atlas_oracle.h for the routine-by-routine citations).
Only tests/, the smoke test and bench.py's CPU-baseline leg import this module;
the product library in math-atlas_gb300/ never does.

Arrays are numpy arrays in Fortran (column-major) order, as the reference's
ColMajor interfaces expect; ``ipiv`` is int32 and 0-based.
"""
import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "liboracle.so")

RowMajor, ColMajor = 101, 102
NoTrans, Trans, ConjTrans = 111, 112, 113
Upper, Lower = 121, 122
NonUnit, Unit = 131, 132
Left, Right = 141, 142

_lib = None


def build():
    """Compile liboracle.so with its Makefile (gcc, no GPU needed)."""
    subprocess.check_call(["make", "-s", "-C", HERE, "liboracle.so"])


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        _lib = C.CDLL(LIB_PATH)
        _declare(_lib)
    return _lib


_dp = np.ctypeslib.ndpointer(dtype=np.float64, flags="F_CONTIGUOUS")
_sp = np.ctypeslib.ndpointer(dtype=np.float32, flags="F_CONTIGUOUS")
_ip = np.ctypeslib.ndpointer(dtype=np.int32, flags="C_CONTIGUOUS")
_i, _d, _f, _l = C.c_int, C.c_double, C.c_float, C.c_long
_v1d = np.ctypeslib.ndpointer(dtype=np.float64, ndim=1, flags="C_CONTIGUOUS")
_v1s = np.ctypeslib.ndpointer(dtype=np.float32, ndim=1, flags="C_CONTIGUOUS")


def _declare(L):
    sig = {
        "ora_srand": (None, [_i]),
        "ora_rand": (_i, []),
        "ora_dgegen": (None, [_i, _i, _dp, _i, _i]),
        "ora_sgegen": (None, [_i, _i, _sp, _i, _i]),
        "ora_dgechkgap": (_i, [_i, _i, _dp, _i]),
        "ora_depsilon": (_d, []),
        "ora_sepsilon": (_f, []),
        "ora_dgenrm1": (_d, [_i, _i, _dp, _i]),
        "ora_dgediffnrm1": (_d, [_i, _i, _dp, _i, _dp, _i]),
        "ora_dgemm": (None, [_i, _i, _i, _i, _i, _d, _dp, _i, _dp, _i, _d, _dp, _i]),
        "ora_sgemm": (None, [_i, _i, _i, _i, _i, _f, _sp, _i, _sp, _i, _f, _sp, _i]),
        "ora_dcblas_gemm": (None, [_i, _i, _i, _i, _i, _i, _d, _dp, _i, _dp, _i, _d, _dp, _i]),
        "ora_dtrsm": (None, [_i, _i, _i, _i, _i, _i, _d, _dp, _i, _dp, _i]),
        "ora_strsm": (None, [_i, _i, _i, _i, _i, _i, _f, _sp, _i, _sp, _i]),
        "ora_dcblas_trsm": (None, [_i, _i, _i, _i, _i, _i, _i, _d, _dp, _i, _dp, _i]),
        "ora_idamax": (_i, [_i, _dp, _i]),
        "ora_dcblas_iamax": (_i, [_i, _dp, _i]),
        "ora_scblas_iamax": (_i, [_i, _sp, _i]),
        "ora_dlaswp": (None, [_i, _dp, _i, _i, _i, _ip, _i]),
        "ora_slaswp": (None, [_i, _sp, _i, _i, _i, _ip, _i]),
        "ora_set_lu_params": (None, [_l, _i]),
        "ora_dgetrf": (_i, [_i, _i, _i, _dp, _i, _ip]),
        "ora_sgetrf": (_i, [_i, _i, _i, _sp, _i, _ip]),
        "ora_dgetrs": (None, [_i, _i, _i, _i, _dp, _i, _ip, _dp, _i]),
        "ora_sgetrs": (None, [_i, _i, _i, _i, _sp, _i, _ip, _sp, _i]),
        "ora_dgesv": (_i, [_i, _i, _i, _dp, _i, _ip, _dp, _i]),
        "ora_dlu_resid": (_d, [_i, _i, _dp, _i, _ip, _i]),
        "ora_slu_resid": (_f, [_i, _i, _sp, _i, _ip, _i]),
        "ora_dgemm_resid": (_d, [_i, _i, _i, _i, _i, _d, _dp, _i, _dp, _i, _d, _dp, _dp, _dp, _i]),
        "ora_dslv_resid": (_d, [_i, _i, _dp, _i, _dp, _i, _dp, _i]),
        "ora_dgemm_dd_samples": (None, [_i, _i, _i, _i, _i, _dp, _i, _dp, _i, _i, _ip, _ip,
                                        np.ctypeslib.ndpointer(np.float64), np.ctypeslib.ndpointer(np.float64)]),
        "ora_dbackward_error": (_d, [_i, _dp, _i, np.ctypeslib.ndpointer(np.float64),
                                    np.ctypeslib.ndpointer(np.float64)]),
        "ora_dsyrk": (None, [_i, _i, _i, _i, _d, _dp, _i, _d, _dp, _i]),
        "ora_ssyrk": (None, [_i, _i, _i, _i, _f, _sp, _i, _f, _sp, _i]),
        "ora_dcblas_syrk": (None, [_i, _i, _i, _i, _i, _d, _dp, _i, _d, _dp, _i]),
        "ora_scblas_syrk": (None, [_i, _i, _i, _i, _i, _f, _sp, _i, _f, _sp, _i]),
        "ora_dpotrf": (_i, [_i, _i, _i, _dp, _i]),
        "ora_spotrf": (_i, [_i, _i, _i, _sp, _i]),
        "ora_dpotrs": (None, [_i, _i, _i, _i, _dp, _i, _dp, _i]),
        "ora_spotrs": (None, [_i, _i, _i, _i, _sp, _i, _sp, _i]),
        "ora_dposv": (_i, [_i, _i, _i, _i, _dp, _i, _dp, _i]),
        "ora_sposv": (_i, [_i, _i, _i, _i, _sp, _i, _sp, _i]),
        "ora_dtrmm": (None, [_i, _i, _i, _i, _i, _i, _d, _dp, _i, _dp, _i]),
        "ora_strmm": (None, [_i, _i, _i, _i, _i, _i, _f, _sp, _i, _sp, _i]),
        "ora_dcblas_trmm": (None, [_i, _i, _i, _i, _i, _i, _i, _d, _dp, _i, _dp, _i]),
        "ora_scblas_trmm": (None, [_i, _i, _i, _i, _i, _i, _i, _f, _sp, _i, _sp, _i]),
        "ora_dcblas_gemv": (None, [_i, _i, _i, _i, _d, _dp, _i, _v1d, _i, _d, _v1d, _i]),
        "ora_scblas_gemv": (None, [_i, _i, _i, _i, _f, _sp, _i, _v1s, _i, _f, _v1s, _i]),
        "ora_dcblas_trsv": (None, [_i, _i, _i, _i, _i, _dp, _i, _v1d, _i]),
        "ora_scblas_trsv": (None, [_i, _i, _i, _i, _i, _sp, _i, _v1s, _i]),
        "ora_dtrtri": (_i, [_i, _i, _i, _i, _dp, _i]),
        "ora_strtri": (_i, [_i, _i, _i, _i, _sp, _i]),
        "ora_dgetri": (_i, [_i, _i, _dp, _i, _ip]),
        "ora_sgetri": (_i, [_i, _i, _sp, _i, _ip]),
        "ora_set_threads": (_i, [_i]),
        "ora_get_threads": (_i, []),
    }
    for name, (res, args) in sig.items():
        fn = getattr(L, name)
        fn.restype = res
        fn.argtypes = args


# ---------------------------------------------------------------- helpers
def gegen(M, N, seed, lda=None, dtype=np.float64):
    """ATL_gegen: uniform (-0.5, 0.5] column by column from the test LCG; the
    lda gap holds the fill constant -2.56e9."""
    lda = max(M, 1) if lda is None else lda
    A = np.empty((lda, N), dtype=dtype, order="F")
    if dtype == np.float64:
        lib().ora_dgegen(M, N, A, lda, seed)
    else:
        lib().ora_sgegen(M, N, A, lda, seed)
    return A


def rand_stream(seed, n):
    lib().ora_srand(seed)
    return np.array([lib().ora_rand() for _ in range(n)], dtype=np.int64)


def eps(dtype=np.float64):
    return lib().ora_depsilon() if dtype == np.float64 else lib().ora_sepsilon()


def gemm(TA, TB, M, N, K, alpha, A, B, beta, C):
    """C <- alpha*op(A)*op(B) + beta*C in place (column-major arrays)."""
    f = lib().ora_dgemm if C.dtype == np.float64 else lib().ora_sgemm
    f(TA, TB, M, N, K, alpha, A, A.shape[0], B, B.shape[0], beta, C, C.shape[0])
    return C


def trsm(Side, Uplo, TA, Diag, M, N, alpha, A, B):
    f = lib().ora_dtrsm if B.dtype == np.float64 else lib().ora_strsm
    f(Side, Uplo, TA, Diag, M, N, alpha, A, A.shape[0], B, B.shape[0])
    return B


def syrk(Uplo, Trans, N, K, alpha, A, beta, C, order=ColMajor):
    """C <- alpha*op(A)*op(A)^T + beta*C on the Uplo triangle, in place."""
    f = lib().ora_dcblas_syrk if C.dtype == np.float64 else lib().ora_scblas_syrk
    f(order, Uplo, Trans, N, K, alpha, A, A.shape[0], beta, C, C.shape[0])
    return C


def trmm(Side, Uplo, TA, Diag, M, N, alpha, A, B, order=ColMajor):
    f = lib().ora_dcblas_trmm if B.dtype == np.float64 else lib().ora_scblas_trmm
    f(order, Side, Uplo, TA, Diag, M, N, alpha, A, A.shape[0], B, B.shape[0])
    return B


def gemv(TA, M, N, alpha, A, x, incx, beta, y, incy, order=ColMajor):
    """y <- alpha*op(A)*x + beta*y on 1-D strided storage (cblas_gemv)."""
    f = lib().ora_dcblas_gemv if A.dtype == np.float64 else lib().ora_scblas_gemv
    f(order, TA, M, N, alpha, A, A.shape[0], x, incx, beta, y, incy)
    return y


def trsv(Uplo, TA, Diag, N, A, x, incx, order=ColMajor):
    f = lib().ora_dcblas_trsv if A.dtype == np.float64 else lib().ora_scblas_trsv
    f(order, Uplo, TA, Diag, N, A, A.shape[0], x, incx)
    return x


def trtri(A, uplo, diag=NonUnit, N=None, order=ColMajor):
    N = A.shape[1] if N is None else N
    f = lib().ora_dtrtri if A.dtype == np.float64 else lib().ora_strtri
    return f(order, uplo, diag, N, A, A.shape[0])


def getri(A, ipiv, N=None, order=ColMajor):
    N = A.shape[1] if N is None else N
    f = lib().ora_dgetri if A.dtype == np.float64 else lib().ora_sgetri
    return f(order, N, A, A.shape[0], np.ascontiguousarray(ipiv, dtype=np.int32))


def potrf(A, uplo=Lower, N=None, order=ColMajor):
    """In-place Cholesky of the uplo triangle; returns info."""
    N = A.shape[1] if N is None else N
    f = lib().ora_dpotrf if A.dtype == np.float64 else lib().ora_spotrf
    return f(order, uplo, N, A, A.shape[0])


def potrs(A, B, uplo=Lower, N=None, order=ColMajor):
    N = A.shape[1] if N is None else N
    f = lib().ora_dpotrs if A.dtype == np.float64 else lib().ora_spotrs
    nrhs = B.shape[1]
    f(order, uplo, N, nrhs, A, A.shape[0], B, B.shape[0])
    return B


def cblas_iamax(N, X, incX):
    """cblas_i?amax on a 1-D array (ATL_i?amax semantics, NaNs included)."""
    X = np.asfortranarray(X)
    f = lib().ora_dcblas_iamax if X.dtype == np.float64 else lib().ora_scblas_iamax
    return int(f(N, X, incX))


def laswp(N, A, K1, K2, ipiv, inci):
    f = lib().ora_dlaswp if A.dtype == np.float64 else lib().ora_slaswp
    f(N, A, A.shape[0], K1, K2, np.ascontiguousarray(ipiv, dtype=np.int32), inci)
    return A


def getrf(A, M=None, N=None, order=ColMajor):
    """In-place LU; returns (info, ipiv)."""
    M = A.shape[0] if M is None else M
    N = A.shape[1] if N is None else N
    ipiv = np.zeros(max(min(M, N), 1), dtype=np.int32)
    f = lib().ora_dgetrf if A.dtype == np.float64 else lib().ora_sgetrf
    info = f(order, M, N, A, A.shape[0], ipiv)
    return info, ipiv[: min(M, N)]


def getrs(A, ipiv, B, trans=NoTrans, N=None, order=ColMajor):
    N = A.shape[1] if N is None else N
    f = lib().ora_dgetrs if A.dtype == np.float64 else lib().ora_sgetrs
    nrhs = B.shape[1]
    f(order, trans, N, nrhs, A, A.shape[0], np.ascontiguousarray(ipiv, dtype=np.int32), B, B.shape[0])
    return B


def lu_resid(M, N, LU, ipiv, seed):
    f = lib().ora_dlu_resid if LU.dtype == np.float64 else lib().ora_slu_resid
    return f(M, N, LU, LU.shape[0], np.ascontiguousarray(ipiv, dtype=np.int32), seed)


def gemm_resid(TA, TB, M, N, K, alpha, A, B, beta, Cin, Ctest, Ctrust):
    return lib().ora_dgemm_resid(TA, TB, M, N, K, alpha, A, A.shape[0], B, B.shape[0], beta,
                                 Cin, Ctest, Ctrust, Cin.shape[0])


def dd_samples(TA, TB, M, N, K, A, B, ii, jj):
    ii = np.ascontiguousarray(ii, dtype=np.int32)
    jj = np.ascontiguousarray(jj, dtype=np.int32)
    hi = np.zeros(len(ii))
    lo = np.zeros(len(ii))
    lib().ora_dgemm_dd_samples(TA, TB, M, N, K, A, A.shape[0], B, B.shape[0], len(ii), ii, jj, hi, lo)
    return hi, lo


def backward_error(A, x, b):
    n = A.shape[1]
    return lib().ora_dbackward_error(n, A, A.shape[0], np.ascontiguousarray(x, dtype=np.float64),
                                     np.ascontiguousarray(b, dtype=np.float64))


def set_threads(n):
    return lib().ora_set_threads(n)


def get_threads():
    return lib().ora_get_threads()


# ---- the reference's own routines (oracle/_ref/libatlref.so, built by
# oracle/ref_build.sh from the reference's basefiles) ----
REF_LIB_PATH = os.path.join(HERE, "_ref", "libatlref.so")
_ref = None


def ref_lib():
    """The reference's own LU-path routines on its C reference BLAS, or None
    when oracle/_ref was not built (no reference tree or extraction)."""
    global _ref
    if _ref is None and os.path.exists(REF_LIB_PATH):
        R = C.CDLL(REF_LIB_PATH)
        R.atlref_dgetrf.argtypes = [_i, _i, _i, _dp, _i, _ip]
        R.atlref_dgetrf.restype = _i
        R.atlref_dgetrs.argtypes = [_i, _i, _i, _i, _dp, _i, _ip, _dp, _i]
        R.atlref_dgemm.argtypes = [_i, _i, _i, _i, _i, _i, _d, _dp, _i, _dp, _i, _d, _dp, _i]
        _ref = R
    return _ref
