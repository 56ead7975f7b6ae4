"""gbblas -- Python binding of libgbblas.so, the GB300 (sm_103a) BLAS hot path.

A thin ctypes layer over the C ABI in include/gbblas.h and
include/gbblas_ref.h.  Device buffers are passed as torch CUDA tensors or as
raw device addresses (int).  There is no CPU fallback: if libgbblas.so is
missing or no sm_103 device is present the calls raise.

    import gbblas
    gbblas.sgemm('N', 'T', M, N, K, 1.5, A, lda, B, ldb, -0.5, C, ldc,
                 algo=gbblas.ALGO_BF16X3)
"""
import ctypes
import os
import re

_HERE = os.path.dirname(os.path.abspath(__file__))
_PKG = os.path.dirname(_HERE)
_REPO = os.path.dirname(_PKG)
LIB_PATH = os.path.join(_HERE, "libgbblas.so")
INCLUDE_DIR = os.path.join(_REPO, "include")

# gb_status
OK, ERR_INVALID_ARG, ERR_UNSUPPORTED, ERR_OOM, ERR_DEVICE_TIMEOUT, ERR_CUDA, ERR_NO_DEVICE = range(7)
# gb_algo
ALGO_AUTO, ALGO_ORDERED, ALGO_SIMT, ALGO_DMMA, ALGO_BF16X3, ALGO_OZAKI, ALGO_SKINNY, ALGO_BF16X6, ALGO_FP16X3 = range(9)
ALGO_NAMES = {0: "auto", 1: "ordered", 2: "simt", 3: "dmma", 4: "bf16x3", 5: "ozaki", 6: "skinny", 7: "bf16x6",
              8: "fp16x3"}
# gb_semantics
SEM_BLAS, SEM_SCALAR_BETA, SEM_ACCUM_SCALAR_BETA = range(3)
# gb_stencil_order
STENCIL_HOST, STENCIL_SCALAR, STENCIL_VECTOR = range(3)


class GBError(RuntimeError):
    def __init__(self, status, msg):
        super().__init__("%s: %s" % (_status_name(status), msg))
        self.status = status


def _status_name(st):
    return {0: "GB_OK", 1: "GB_ERR_INVALID_ARG", 2: "GB_ERR_UNSUPPORTED", 3: "GB_ERR_OOM",
            4: "GB_ERR_DEVICE_TIMEOUT", 5: "GB_ERR_CUDA", 6: "GB_ERR_NO_DEVICE"}.get(st, "GB_ERR_%d" % st)


class GemmOpts(ctypes.Structure):
    _fields_ = [("stream", ctypes.c_void_p), ("algo", ctypes.c_int32), ("semantics", ctypes.c_int32),
                ("k_block", ctypes.c_int32), ("k_slab", ctypes.c_int32), ("alpha_on_b", ctypes.c_int32),
                ("ozaki_slices", ctypes.c_int32), ("target_err", ctypes.c_double),
                ("accum_k", ctypes.c_int32), ("split_k", ctypes.c_int32), ("err_out", ctypes.c_void_p)]


class TuneChoice(ctypes.Structure):
    _fields_ = [("algo", ctypes.c_int32), ("accum_k", ctypes.c_int32), ("split_k", ctypes.c_int32),
                ("ozaki_slices", ctypes.c_int32), ("ms", ctypes.c_double)]


class GemmDesc(ctypes.Structure):
    _fields_ = [("dtype_bits", ctypes.c_int32), ("transA", ctypes.c_char), ("transB", ctypes.c_char),
                ("pad", ctypes.c_char * 2), ("semantics", ctypes.c_int32), ("reserved", ctypes.c_int32),
                ("M", ctypes.c_int64), ("N", ctypes.c_int64), ("K", ctypes.c_int64),
                ("alpha", ctypes.c_double), ("beta", ctypes.c_double),
                ("A", ctypes.c_void_p), ("lda", ctypes.c_int64), ("B", ctypes.c_void_p), ("ldb", ctypes.c_int64),
                ("C", ctypes.c_void_p), ("ldc", ctypes.c_int64)]


class Request(ctypes.Structure):
    _fields_ = [("op", ctypes.c_int32), ("dtype_bits", ctypes.c_int32), ("transA", ctypes.c_char),
                ("transB", ctypes.c_char), ("pad", ctypes.c_char * 2), ("algo", ctypes.c_int32),
                ("semantics", ctypes.c_int32), ("iters", ctypes.c_int32), ("order", ctypes.c_int32),
                ("reserved", ctypes.c_int32),
                ("M", ctypes.c_int64), ("N", ctypes.c_int64), ("K", ctypes.c_int64),
                ("alpha", ctypes.c_double), ("beta", ctypes.c_double),
                ("A", ctypes.c_void_p), ("lda", ctypes.c_int64), ("B", ctypes.c_void_p), ("ldb", ctypes.c_int64),
                ("C", ctypes.c_void_p), ("ldc", ctypes.c_int64), ("bytes", ctypes.c_uint64),
                ("tag", ctypes.c_uint64)]


class ServerConfig(ctypes.Structure):
    _fields_ = [("hbm_budget_bytes", ctypes.c_uint64), ("workspace_bytes", ctypes.c_uint64),
                ("group_max_work", ctypes.c_double), ("streams", ctypes.c_int32), ("max_batch", ctypes.c_int32),
                ("max_inflight", ctypes.c_int32), ("use_graphs", ctypes.c_int32), ("use_grouped", ctypes.c_int32),
                ("dry_run", ctypes.c_int32), ("short_us", ctypes.c_double), ("short_streams", ctypes.c_int32),
                ("long_sm_percent", ctypes.c_int32)]


class ServerStats(ctypes.Structure):
    _fields_ = [("submitted", ctypes.c_int64), ("completed", ctypes.c_int64), ("rejected", ctypes.c_int64),
                ("failed", ctypes.c_int64), ("waiting", ctypes.c_int64), ("inflight", ctypes.c_int64),
                ("inflight_bytes", ctypes.c_uint64), ("launches", ctypes.c_int64),
                ("grouped_launches", ctypes.c_int64), ("grouped_requests", ctypes.c_int64),
                ("p50_s", ctypes.c_double), ("p99_s", ctypes.c_double), ("mean_s", ctypes.c_double),
                ("req_per_s", ctypes.c_double), ("graph_launches", ctypes.c_int64),
                ("graph_instantiations", ctypes.c_int64), ("urgent_launches", ctypes.c_int64)]


OP_GEMM, OP_TRANSPOSE, OP_STENCIL = range(3)

_i64, _vp, _int, _dbl, _flt = ctypes.c_int64, ctypes.c_void_p, ctypes.c_int, ctypes.c_double, ctypes.c_float
_ul = ctypes.c_ulong
_SIGS = {
    "gb_status_string": ([_int], ctypes.c_char_p),
    "gb_get_last_status": ([], _int),
    "gb_last_error": ([], ctypes.c_char_p),
    "gb_last_error_string": ([], ctypes.c_char_p),
    "gb_clear_last_status": ([], None),
    "gb_version": ([], _int),
    "gb_launch_count": ([], ctypes.c_uint64),
    "gb_device_arch": ([], _int),
    "gb_sync": ([_vp], _int),
    "gb_malloc": ([ctypes.POINTER(ctypes.c_void_p), ctypes.c_size_t], _int),
    "gb_free": ([_vp], _int),
    "gb_memcpy": ([_vp, _vp, ctypes.c_size_t, _int, _vp], _int),
    "gb_fill_f64": ([_vp, _i64, _i64, _i64, ctypes.c_uint64, _int, _vp], _int),
    "gb_fill_f32": ([_vp, _i64, _i64, _i64, ctypes.c_uint64, _int, _vp], _int),
    "gb_gemm_opts_init": ([ctypes.POINTER(GemmOpts)], None),
    "gb_sgemm": ([ctypes.c_char, ctypes.c_char, _i64, _i64, _i64, _flt, _vp, _i64, _vp, _i64, _flt, _vp, _i64,
                  ctypes.POINTER(GemmOpts)], _int),
    "gb_dgemm": ([ctypes.c_char, ctypes.c_char, _i64, _i64, _i64, _dbl, _vp, _i64, _vp, _i64, _dbl, _vp, _i64,
                  ctypes.POINTER(GemmOpts)], _int),
    "gb_gemm_pick_algo": ([_int, ctypes.c_char, ctypes.c_char, _i64, _i64, _i64], _int),
    "gb_transpose_f32": ([_i64, _i64, _vp, _i64, _vp, _i64, _vp], _int),
    "gb_transpose_add_f32": ([_i64, _i64, _vp, _i64, _vp, _i64, _vp], _int),
    "gb_stencil9_f32": ([_i64, _i64, _vp, _vp, _int, _vp, _vp], _int),
    "gb_stencil9_f64": ([_i64, _i64, _vp, _vp, _int, _vp, _vp], _int),
    "gb_transpose_add_f64": ([_i64, _i64, _vp, _i64, _vp, _i64, _vp], _int),
    "gb_gemm_strided_batched": ([_int, ctypes.c_char, ctypes.c_char, _i64, _i64, _i64, ctypes.c_double, _vp, _i64,
                                 _i64, _vp, _i64, _i64, ctypes.c_double, _vp, _i64, _i64, _i64, _int, _vp], _int),
    "gb_transpose_f64": ([_i64, _i64, _vp, _i64, _vp, _i64, _vp], _int),
    "gb_stencil2d_f64": ([_i64, _i64, _vp, _vp, _int, _int, _vp], _int),
    "gb_stencil2d_f32": ([_i64, _i64, _vp, _vp, _int, _int, _vp], _int),
    "gb_exec": ([ctypes.c_char_p, _int, _int, ctypes.POINTER(_ul)], _int),
    "gb_ref_set_stream": ([_vp], None),
    "gb_workspace_reserve": ([ctypes.c_size_t, _vp], _int),
    "gb_workspace_query": ([_int, ctypes.c_char, ctypes.c_char, _i64, _i64, _i64, _vp, _i64, _vp, _i64,
                            ctypes.POINTER(GemmOpts), ctypes.POINTER(ctypes.c_size_t)], _int),
    "gb_selftest_bounded_wait": ([ctypes.c_uint64, _vp], _int),
    "gb_measure_fma_peak": ([_int, ctypes.POINTER(ctypes.c_double), _vp], _int),
    "gb_gemm_batch": ([ctypes.POINTER(GemmDesc), _int, _vp], _int),
    "gb_server_config_init": ([ctypes.POINTER(ServerConfig)], None),
    "gb_server_create": ([ctypes.POINTER(ServerConfig), ctypes.POINTER(ctypes.c_void_p)], _int),
    "gb_server_submit": ([_vp, ctypes.POINTER(Request)], _int),
    "gb_server_poll": ([_vp, ctypes.POINTER(ctypes.c_uint64), ctypes.POINTER(ctypes.c_double), _int], _int),
    "gb_server_drain": ([_vp, _dbl], _int),
    "gb_server_get_stats": ([_vp, ctypes.POINTER(ServerStats)], _int),
    "gb_server_destroy": ([_vp], None),
    "gb_autotune_gemm": ([_int, ctypes.c_char, ctypes.c_char, _i64, _i64, _i64, ctypes.POINTER(_int),
                          ctypes.POINTER(_dbl)], _int),
    "gb_autotune_set": ([_int, ctypes.c_char, ctypes.c_char, _i64, _i64, _i64, _int], _int),
    "gb_autotune_gemm_ex": ([_int, ctypes.c_char, ctypes.c_char, _i64, _i64, _i64, _dbl, _int, _vp,
                             ctypes.POINTER(TuneChoice)], _int),
    "gb_autotune_lookup": ([_int, ctypes.c_char, ctypes.c_char, _i64, _i64, _i64, ctypes.POINTER(TuneChoice)], _int),
    "gb_autotune_get": ([_int, ctypes.c_char, ctypes.c_char, _i64, _i64, _i64], _int),
    "gb_autotune_save": ([ctypes.c_char_p], _int),
    "gb_autotune_load": ([ctypes.c_char_p], _int),
    "gb_ref_set_algo": ([_int], None),
}

_LIB = None


def lib():
    """Load libgbblas.so (raises if it was not built)."""
    global _LIB
    if _LIB is None:
        if not os.path.exists(LIB_PATH):
            raise GBError(ERR_NO_DEVICE, "libgbblas.so not built: run __graft_entry__.build() or "
                                         "python blas-for-multi-core-dsp_gb300/build.py")
        L = ctypes.CDLL(LIB_PATH)
        for name, (args, res) in _SIGS.items():
            f = getattr(L, name, None)
            if f is None:
                continue
            f.argtypes = args
            f.restype = res
        _LIB = L
    return _LIB


def declared_symbols():
    """Every function name declared in include/*.h."""
    names = set()
    for fn in sorted(os.listdir(INCLUDE_DIR)):
        if not fn.endswith(".h") or fn.startswith("gbblas_noexport"):
            continue
        src = open(os.path.join(INCLUDE_DIR, fn)).read()
        src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
        src = re.sub(r"//[^\n]*", "", src)
        for m in re.finditer(r"\b([A-Za-z_][A-Za-z0-9_]*)\s*\([^;{}]*\)\s*;", src):
            name = m.group(1)
            if name not in ("if", "while", "for", "return", "sizeof"):
                names.add(name)
    return sorted(names)


def _check(st, what=""):
    if st != OK:
        raise GBError(st, (lib().gb_last_error() or b"").decode() or what)


def _ptr(x):
    if x is None:
        return None
    if isinstance(x, int):
        return x
    if hasattr(x, "data_ptr"):
        return x.data_ptr()
    raise TypeError("expected a torch tensor or an int device address, got %r" % type(x))


def _stream(s):
    if s is None:
        return None
    if isinstance(s, int):
        return s
    return s.cuda_stream


def launch_count():
    return lib().gb_launch_count()


def arch():
    return lib().gb_device_arch()


def fma_peak(bits, stream=None):
    """Measured scalar FMA throughput (TFLOP/s) of the device: FFMA (32) or DFMA (64)."""
    v = ctypes.c_double()
    _check(lib().gb_measure_fma_peak(bits, ctypes.byref(v), _stream(stream)), "gb_measure_fma_peak")
    return v.value


def sync(stream=None):
    _check(lib().gb_sync(_stream(stream)))


def opts(algo=ALGO_AUTO, semantics=SEM_BLAS, stream=None, k_block=0, k_slab=0, alpha_on_b=0,
         ozaki_slices=0, target_err=0.0, accum_k=0, split_k=0, err_out=None):
    o = GemmOpts()
    lib().gb_gemm_opts_init(ctypes.byref(o))
    o.stream = _stream(stream)
    o.algo = algo
    o.semantics = semantics
    o.k_block = k_block
    o.k_slab = k_slab
    o.alpha_on_b = alpha_on_b
    o.ozaki_slices = ozaki_slices
    o.target_err = target_err
    o.accum_k = accum_k
    o.split_k = split_k
    o.err_out = _ptr(err_out) if err_out is not None else None
    return o


def sgemm(ta, tb, M, N, K, alpha, A, lda, B, ldb, beta, C, ldc, **kw):
    o = opts(**kw)
    _check(lib().gb_sgemm(ta.encode(), tb.encode(), M, N, K, alpha, _ptr(A), lda, _ptr(B), ldb, beta, _ptr(C),
                          ldc, ctypes.byref(o)), "gb_sgemm")


def dgemm(ta, tb, M, N, K, alpha, A, lda, B, ldb, beta, C, ldc, **kw):
    o = opts(**kw)
    _check(lib().gb_dgemm(ta.encode(), tb.encode(), M, N, K, alpha, _ptr(A), lda, _ptr(B), ldb, beta, _ptr(C),
                          ldc, ctypes.byref(o)), "gb_dgemm")


def gemm(ta, tb, M, N, K, alpha, A, lda, B, ldb, beta, C, ldc, dtype_bits, **kw):
    f = dgemm if dtype_bits == 64 else sgemm
    f(ta, tb, M, N, K, alpha, A, lda, B, ldb, beta, C, ldc, **kw)


def pick_algo(bits, ta, tb, M, N, K):
    return lib().gb_gemm_pick_algo(bits, ta.encode(), tb.encode(), M, N, K)


def workspace_query(bits, ta, tb, M, N, K, lda, ldb, A=None, B=None, **kw):
    """Workspace bytes the gb_sgemm / gb_dgemm call with these arguments and options may use."""
    o = opts(**kw)
    n = ctypes.c_size_t(0)
    _check(lib().gb_workspace_query(bits, ta.encode(), tb.encode(), M, N, K, _ptr(A), lda, _ptr(B), ldb,
                                    ctypes.byref(o), ctypes.byref(n)), "gb_workspace_query")
    return n.value


def workspace_reserve(nbytes, stream=None):
    _check(lib().gb_workspace_reserve(nbytes, _stream(stream)), "gb_workspace_reserve")


def transpose(M, N, A, lda, B, ldb, bits, stream=None):
    f = lib().gb_transpose_f64 if bits == 64 else lib().gb_transpose_f32
    _check(f(M, N, _ptr(A), lda, _ptr(B), ldb, _stream(stream)), "transpose")


def transpose_add(M, N, A, lda, B, ldb, bits, stream=None):
    """B += A^T (bit-exact transpose-accumulate)."""
    f = lib().gb_transpose_add_f64 if bits == 64 else lib().gb_transpose_add_f32
    _check(f(M, N, _ptr(A), lda, _ptr(B), ldb, _stream(stream)), "transpose_add")


def gemm_strided_batched(bits, ta, tb, M, N, K, alpha, A, lda, strideA, B, ldb, strideB, beta, C, ldc, strideC,
                         batch, semantics=SEM_BLAS, stream=None):
    _check(lib().gb_gemm_strided_batched(bits, ta.encode(), tb.encode(), M, N, K, alpha, _ptr(A), lda, strideA,
                                         _ptr(B), ldb, strideB, beta, _ptr(C), ldc, strideC, batch, semantics,
                                         _stream(stream)), "gb_gemm_strided_batched")


def stencil9(M, N, A, B, iters, w, bits=64, stream=None):
    """9-point stencil with the 3x3 weight window w (host sequence of 9)."""
    import numpy as _np
    wv = _np.ascontiguousarray(_np.asarray(w, dtype=_np.float64 if bits == 64 else _np.float32).reshape(9))
    f = lib().gb_stencil9_f64 if bits == 64 else lib().gb_stencil9_f32
    _check(f(M, N, _ptr(A), _ptr(B), iters, wv.ctypes.data, _stream(stream)), "stencil9")


def stencil2d(M, N, A, B, iters, order=STENCIL_HOST, bits=64, stream=None):
    f = lib().gb_stencil2d_f64 if bits == 64 else lib().gb_stencil2d_f32
    _check(f(M, N, _ptr(A), _ptr(B), iters, order, _stream(stream)), "stencil2d")


def fill(X, rows, cols, ld, seed, kind=0, bits=64, stream=None):
    f = lib().gb_fill_f64 if bits == 64 else lib().gb_fill_f32
    _check(f(_ptr(X), rows, cols, ld, seed & 0xFFFFFFFFFFFFFFFF, kind, _stream(stream)), "fill")


def exec_by_name(name, scalars, pointers):
    """The reference's launch-by-name call: scalars first, then pointers."""
    vals = [int(s) for s in scalars] + [_ptr(p) for p in pointers]
    arr = (_ul * len(vals))(*vals)
    _check(lib().gb_exec(name.encode(), len(scalars), len(pointers), arr), "gb_exec " + name)


def ref_call(name, *args):
    """Call a reference-named entry point of gbblas_ref.h with plain ints /
    floats / tensors (pointers by data_ptr).  Returns the recorded status."""
    f = getattr(lib(), name)
    cargs = []
    for a in args:
        if isinstance(a, float):
            cargs.append(ctypes.c_float(a))
        elif isinstance(a, int):
            cargs.append(ctypes.c_ulong(a))
        else:
            cargs.append(ctypes.c_void_p(_ptr(a)))
    lib().gb_clear_last_status()
    f.restype = None
    f(*cargs)
    return lib().gb_get_last_status()


# ------------------------------------------------------------- grouped / serving
def gemm_desc(ta, tb, M, N, K, alpha, A, lda, B, ldb, beta, C, ldc, bits, semantics=SEM_BLAS):
    d = GemmDesc()
    d.dtype_bits, d.transA, d.transB, d.semantics = bits, ta.encode(), tb.encode(), semantics
    d.M, d.N, d.K, d.alpha, d.beta = M, N, K, alpha, beta
    d.A, d.lda, d.B, d.ldb, d.C, d.ldc = _ptr(A), lda, _ptr(B), ldb, _ptr(C), ldc
    return d


def gemm_batch(descs, stream=None):
    arr = (GemmDesc * len(descs))(*descs)
    _check(lib().gb_gemm_batch(arr, len(descs), _stream(stream)), "gb_gemm_batch")


def request(op, bits, M, N, K=0, A=None, lda=0, B=None, ldb=0, C=None, ldc=0, ta="N", tb="N", alpha=1.0,
            beta=0.0, algo=ALGO_AUTO, semantics=SEM_BLAS, iters=0, order=STENCIL_HOST, tag=0, nbytes=0):
    r = Request()
    r.op, r.dtype_bits, r.transA, r.transB = op, bits, ta.encode(), tb.encode()
    r.algo, r.semantics, r.iters, r.order = algo, semantics, iters, order
    r.M, r.N, r.K, r.alpha, r.beta = M, N, K, alpha, beta
    r.A, r.lda, r.B, r.ldb, r.C, r.ldc = _ptr(A), lda, _ptr(B), ldb, _ptr(C), ldc
    r.bytes, r.tag = nbytes, tag
    return r


class Server:
    """Thin wrapper over gb_server_* (include/gbblas.h)."""

    def __init__(self, **cfg):
        c = ServerConfig()
        lib().gb_server_config_init(ctypes.byref(c))
        for k, v in cfg.items():
            setattr(c, k, v)
        h = ctypes.c_void_p()
        _check(lib().gb_server_create(ctypes.byref(c), ctypes.byref(h)), "gb_server_create")
        self.h = h

    def submit(self, req):
        st = lib().gb_server_submit(self.h, ctypes.byref(req))
        if st != OK:
            raise GBError(st, (lib().gb_last_error() or b"").decode())

    def poll(self, max_n=4096):
        tags = (ctypes.c_uint64 * max_n)()
        lat = (ctypes.c_double * max_n)()
        n = lib().gb_server_poll(self.h, tags, lat, max_n)
        return [(tags[i], lat[i]) for i in range(n)]

    def drain(self, timeout_s=0.0):
        _check(lib().gb_server_drain(self.h, timeout_s), "gb_server_drain")

    def stats(self):
        st = ServerStats()
        _check(lib().gb_server_get_stats(self.h, ctypes.byref(st)), "gb_server_get_stats")
        return {name: getattr(st, name) for name, _ in ServerStats._fields_}

    def close(self):
        if self.h:
            lib().gb_server_destroy(self.h)
            self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()


def autotune_gemm(bits, ta, tb, M, N, K):
    best = ctypes.c_int()
    ms = ctypes.c_double()
    _check(lib().gb_autotune_gemm(bits, ta.encode(), tb.encode(), M, N, K, ctypes.byref(best), ctypes.byref(ms)),
           "gb_autotune_gemm")
    return best.value, ms.value


def autotune_gemm_ex(bits, ta, tb, M, N, K, target_err=0.0, reps=5, stream=None):
    """Search the candidates for the shape; returns the chosen TuneChoice as a dict."""
    c = TuneChoice()
    _check(lib().gb_autotune_gemm_ex(bits, ta.encode(), tb.encode(), M, N, K, target_err, reps, _stream(stream),
                                     ctypes.byref(c)), "gb_autotune_gemm_ex")
    return {name: getattr(c, name) for name, _ in TuneChoice._fields_}


def autotune_lookup(bits, ta, tb, M, N, K):
    """The bucket's TuneChoice as a dict, or None."""
    c = TuneChoice()
    if lib().gb_autotune_lookup(bits, ta.encode(), tb.encode(), M, N, K, ctypes.byref(c)) != OK:
        return None
    return {name: getattr(c, name) for name, _ in TuneChoice._fields_}
