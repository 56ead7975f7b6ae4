"""Python binding of the oracle (oracle.c): the CPU restatement of the
reference's host-side check loops, plus the Dot2 accuracy oracle.

TEST INFRASTRUCTURE.  Only tests/, ``__graft_entry__.smoke()`` and the CPU
legs of bench.py (``cpu_baseline`` and ``--impl reference``) import this
package, and only as the checker or the timed CPU baseline.  The product
library (libgbblas) never calls it.
"""
import ctypes
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB = None

_i64 = ctypes.c_int64
_dp = ctypes.c_void_p


def build(quiet=True):
    """Compile liboracle.so in place (gcc, a few seconds)."""
    out = subprocess.run(["make", "-C", _HERE, "oracle"], capture_output=True, text=True)
    if out.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + out.stdout + out.stderr)
    if not quiet:
        print(out.stdout)


def lib():
    global _LIB
    if _LIB is None:
        path = os.path.join(_HERE, "liboracle.so")
        if not os.path.exists(path):
            build()
        L = ctypes.CDLL(path)
        sigs = {
            "gbo_fill_f64": [_dp, _i64, _i64, _i64, ctypes.c_uint64, ctypes.c_int],
            "gbo_fill_f32": [_dp, _i64, _i64, _i64, ctypes.c_uint64, ctypes.c_int],
            "gbo_dgemm_ref": [ctypes.c_int, ctypes.c_int, _i64, _i64, _i64, _dp, _i64, _dp, _i64, _dp, _i64, _i64],
            "gbo_sgemm_ref": [ctypes.c_int, ctypes.c_int, _i64, _i64, _i64, ctypes.c_float, _dp, _i64, _dp, _i64,
                              ctypes.c_float, _dp, _i64, _i64, ctypes.c_int],
            "gbo_sgemm_irr_ref": [ctypes.c_int, ctypes.c_int, _i64, _i64, _i64, _dp, _i64, _dp, _i64, _dp, _i64, _i64],
            "gbo_thinB_sgemm_ref": [ctypes.c_int, ctypes.c_int, _i64, _i64, _i64, ctypes.c_float, _dp, _i64, _dp, _i64,
                                    ctypes.c_float, _dp, _i64, _i64, _i64, ctypes.c_int],
            "gbo_transpose_f32": [_i64, _i64, _dp, _i64, _dp, _i64],
            "gbo_transpose_f64": [_i64, _i64, _dp, _i64, _dp, _i64],
            "gbo_transpose_add_f32": [_i64, _i64, _dp, _i64, _dp, _i64],
            "gbo_stencil9_f32": [_i64, _i64, _dp, _dp, ctypes.c_int, _dp],
            "gbo_stencil9_f64": [_i64, _i64, _dp, _dp, ctypes.c_int, _dp],
            "gbo_transpose_add_f64": [_i64, _i64, _dp, _i64, _dp, _i64],
            "gbo_stencil_f64": [_i64, _i64, _dp, _dp, ctypes.c_int, ctypes.c_int],
            "gbo_stencil_f32": [_i64, _i64, _dp, _dp, ctypes.c_int, ctypes.c_int],
            "gbo_gemm_dot2_f64": [ctypes.c_int, ctypes.c_int, _i64, _i64, _i64, ctypes.c_double, _dp, _i64, _dp, _i64,
                                  ctypes.c_double, _dp, _i64, _dp, _i64, _dp, _i64, _dp],
            "gbo_gemm_dot2_f32": [ctypes.c_int, ctypes.c_int, _i64, _i64, _i64, ctypes.c_double, _dp, _i64, _dp, _i64,
                                  ctypes.c_double, _dp, _i64, _dp, _i64, _dp, _i64, _dp],
            "gbo_op_norms_f64": [ctypes.c_int, ctypes.c_int, _i64, _i64, _i64, _dp, _i64, _dp, _i64, _dp, _i64, _dp,
                                 _i64, _dp, _dp],
            "gbo_op_norms_f32": [ctypes.c_int, ctypes.c_int, _i64, _i64, _i64, _dp, _i64, _dp, _i64, _dp, _i64, _dp,
                                 _i64, _dp, _dp],
            "gbo_set_threads": [ctypes.c_int],
            "gbo_get_threads": [],
        }
        for name, args in sigs.items():
            f = getattr(L, name)
            f.argtypes = args
            f.restype = ctypes.c_int if name == "gbo_get_threads" else None
        _LIB = L
    return _LIB


def _p(a):
    if a is None:
        return None
    assert a.flags["C_CONTIGUOUS"]
    return a.ctypes.data


def _t(c):
    return 1 if c in ("T", "t", 1, True) else 0


def set_threads(n):
    lib().gbo_set_threads(int(n))


def threads():
    return lib().gbo_get_threads()


def fill(rows, cols, seed, kind=0, dtype=np.float64, ld=None):
    ld = cols if ld is None else ld
    X = np.zeros((rows, ld), dtype=dtype)
    f = lib().gbo_fill_f64 if dtype == np.float64 else lib().gbo_fill_f32
    f(_p(X), rows, cols, ld, seed & 0xFFFFFFFFFFFFFFFF, kind)
    return X


def dgemm_ref(ta, tb, M, N, K, A, lda, B, ldb, C, ldc, kg=512):
    """C += op(A)op(B) in place (dgemm_demo.c:233-252)."""
    lib().gbo_dgemm_ref(_t(ta), _t(tb), M, N, K, _p(A), lda, _p(B), ldb, _p(C), ldc, kg)


def sgemm_ref(ta, tb, M, N, K, alpha, A, lda, B, ldb, beta, C, ldc, kg=512, accumulate=False):
    """C = [C +] alpha*op(A)op(B) + beta (scalar) in place (sgemm_demo.c:214-242)."""
    lib().gbo_sgemm_ref(_t(ta), _t(tb), M, N, K, alpha, _p(A), lda, _p(B), ldb, beta, _p(C), ldc, kg,
                        1 if accumulate else 0)


def sgemm_irr_ref(ta, tb, M, N, K, A, lda, B, ldb, C, ldc, kg=512):
    """C += op(A)op(B) in place (irr_shortA_sgemm_demo.c:206-222)."""
    lib().gbo_sgemm_irr_ref(_t(ta), _t(tb), M, N, K, _p(A), lda, _p(B), ldb, _p(C), ldc, kg)


def thinB_sgemm_ref(ta, tb, M, N, K, alpha, A, lda, B, ldb, beta, C, ldc, kg=3072, ka=512, accumulate=False):
    """C = [C +] (alpha*op(A)op(B) + beta) in place (irr_thinB_sgemm_demo.c:217-239)."""
    lib().gbo_thinB_sgemm_ref(_t(ta), _t(tb), M, N, K, alpha, _p(A), lda, _p(B), ldb, beta, _p(C), ldc, kg, ka,
                              1 if accumulate else 0)


def transpose_into(M, N, A, lda, B, ldb):
    f = lib().gbo_transpose_f64 if A.dtype == np.float64 else lib().gbo_transpose_f32
    f(M, N, _p(A), lda, _p(B), ldb)


def transpose_add_into(M, N, A, lda, B, ldb):
    """B += A^T in place (transpose-accumulate)."""
    f = lib().gbo_transpose_add_f64 if A.dtype == np.float64 else lib().gbo_transpose_add_f32
    f(M, N, _p(A), lda, _p(B), ldb)


def stencil9(M, N, A, B, iters, w):
    """iters 9-point sweeps with the 3x3 weight window w, ping-ponging A and B."""
    dt = A.dtype
    wv = np.ascontiguousarray(np.asarray(w, dtype=dt).reshape(9))
    f = lib().gbo_stencil9_f64 if dt == np.float64 else lib().gbo_stencil9_f32
    f(M, N, _p(A), _p(B), iters, _p(wv))


def stencil(M, N, A, B, iters, order=0):
    """iters Jacobi sweeps ping-ponging A and B (padded (M+2)x(N+2))."""
    f = lib().gbo_stencil_f64 if A.dtype == np.float64 else lib().gbo_stencil_f32
    f(M, N, _p(A), _p(B), iters, order)


def gemm_dot2(ta, tb, M, N, K, alpha, A, lda, B, ldb, beta, C0, ldc, rows, cols):
    rows = np.ascontiguousarray(rows, dtype=np.int64)
    cols = np.ascontiguousarray(cols, dtype=np.int64)
    out = np.zeros((len(rows), len(cols)), dtype=np.float64)
    f = lib().gbo_gemm_dot2_f64 if A.dtype == np.float64 else lib().gbo_gemm_dot2_f32
    f(_t(ta), _t(tb), M, N, K, float(alpha), _p(A), lda, _p(B), ldb, float(beta), _p(C0), ldc,
      _p(rows), len(rows), _p(cols), len(cols), _p(out))
    return out


def op_norms(ta, tb, M, N, K, A, lda, B, ldb, rows, cols):
    rows = np.ascontiguousarray(rows, dtype=np.int64)
    cols = np.ascontiguousarray(cols, dtype=np.int64)
    rn2 = np.zeros(len(rows))
    cn2 = np.zeros(len(cols))
    f = lib().gbo_op_norms_f64 if A.dtype == np.float64 else lib().gbo_op_norms_f32
    f(_t(ta), _t(tb), M, N, K, _p(A), lda, _p(B), ldb, _p(rows), len(rows), _p(cols), len(cols), _p(rn2), _p(cn2))
    return rn2, cn2


def normwise_error(C_hat, ta, tb, M, N, K, alpha, A, lda, B, ldb, beta, C0, ldc, rows=None, cols=None):
    """||C_hat - C*||_F / (|alpha| ||op(A)_I||_F ||op(B)_J||_F + |beta| ||C0_IJ||_F)
    over the row set I and column set J (all rows/cols when None).
    C_hat is the full M x ldc result; C* comes from Dot2."""
    rows = np.arange(M) if rows is None else np.asarray(rows)
    cols = np.arange(N) if cols is None else np.asarray(cols)
    ref = gemm_dot2(ta, tb, M, N, K, alpha, A, lda, B, ldb, beta, C0, ldc, rows, cols)
    got = C_hat[np.ix_(rows, cols)].astype(np.float64)
    rn2, cn2 = op_norms(ta, tb, M, N, K, A, lda, B, ldb, rows, cols)
    den = abs(alpha) * np.sqrt(rn2.sum()) * np.sqrt(cn2.sum())
    if C0 is not None and beta != 0:
        den += abs(beta) * np.linalg.norm(C0[np.ix_(rows, cols)].astype(np.float64))
    num = np.linalg.norm(got - ref)
    maxrel = float(np.max(np.abs(got - ref) / np.maximum(np.abs(ref), 1e-300))) if got.size else 0.0
    return (num / den if den > 0 else num), maxrel
