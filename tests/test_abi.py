"""The C-ABI library without a GPU: it loads, exports every symbol declared
in include/*.h, and rejects bad arguments on the host before any device
work (status codes + messages)."""
import ctypes
import os
import subprocess

import pytest

import gbblas


@pytest.fixture(scope="module")
def L():
    if not os.path.exists(gbblas.LIB_PATH):
        import __graft_entry__
        __graft_entry__.build()
    return gbblas.lib()


def test_exports_every_declared_symbol(L):
    names = gbblas.declared_symbols()
    assert "gb_sgemm" in names and "dgemm_NN" in names and "stencil_vector" in names
    missing = [n for n in names if not hasattr(L, n)]
    assert not missing, missing
    out = subprocess.run(["nm", "-D", "--defined-only", gbblas.LIB_PATH], capture_output=True, text=True).stdout
    exported = {l.split()[-1] for l in out.splitlines() if l.strip()}
    assert set(names) <= exported, sorted(set(names) - exported)


def test_status_strings(L):
    assert L.gb_status_string(0) == b"GB_OK"
    assert L.gb_status_string(1) == b"GB_ERR_INVALID_ARG"
    assert L.gb_version() >= 100


def _sgemm(L, ta="N", tb="N", M=4, N=4, K=4, lda=4, ldb=4, ldc=4, A=8, B=8, C=8, **kw):
    o = gbblas.opts(**kw)
    return L.gb_sgemm(ta.encode(), tb.encode(), M, N, K, 1.0, A, lda, B, ldb, 0.0, C, ldc, ctypes.byref(o))


@pytest.mark.parametrize("kw,frag", [
    (dict(ta="X"), "transA"),
    (dict(M=-1), "negative"),
    (dict(lda=3), "lda"),
    (dict(ta="T", M=8, lda=4), "lda"),
    (dict(ldb=3), "ldb"),
    (dict(tb="T", K=8, lda=8, ldb=4), "ldb"),
    (dict(ldc=3), "ldc"),
    (dict(C=None), "C is null"),
    (dict(A=None), "A or B is null"),
    (dict(semantics=7), "semantics"),
    (dict(algo=42), "algo"),
])
def test_gemm_rejects_bad_arguments(L, kw, frag):
    st = _sgemm(L, **kw)
    assert st == gbblas.ERR_INVALID_ARG
    assert frag in L.gb_last_error().decode()


def test_gemm_empty_is_ok_without_device(L):
    assert _sgemm(L, M=0) == gbblas.OK
    assert _sgemm(L, N=0, A=None, B=None, C=None) == gbblas.OK


def test_dgemm_rejects_bad_arguments(L):
    o = gbblas.opts()
    st = L.gb_dgemm(b"N", b"N", 4, 4, 4, 1.0, 8, 2, 8, 4, 0.0, 8, 4, ctypes.byref(o))
    assert st == gbblas.ERR_INVALID_ARG and b"lda" in L.gb_last_error()
    o = gbblas.opts(algo=gbblas.ALGO_OZAKI, ozaki_slices=10)
    st = L.gb_dgemm(b"N", b"N", 4, 4, 4, 1.0, 8, 4, 8, 4, 0.0, 8, 4, ctypes.byref(o))
    assert st == gbblas.ERR_INVALID_ARG and b"ozaki_slices" in L.gb_last_error()


def test_transpose_and_stencil_reject_bad_arguments(L):
    assert L.gb_transpose_f32(4, 5, 8, 4, 16, 4, None) == gbblas.ERR_INVALID_ARG   # lda < N
    assert L.gb_transpose_f64(4, 5, 8, 5, 16, 3, None) == gbblas.ERR_INVALID_ARG   # ldb < M
    assert L.gb_transpose_f32(4, 5, 8, 5, 8, 4, None) == gbblas.ERR_INVALID_ARG    # in place
    assert L.gb_transpose_f32(0, 5, None, 5, None, 0, None) == gbblas.OK
    assert L.gb_stencil2d_f64(4, 4, 8, 16, 1, 5, None) == gbblas.ERR_INVALID_ARG   # order
    assert L.gb_stencil2d_f64(4, 4, 8, 8, 1, 0, None) == gbblas.ERR_INVALID_ARG    # A == B
    assert L.gb_stencil2d_f64(4, 4, 8, 16, -1, 0, None) == gbblas.ERR_INVALID_ARG
    assert L.gb_stencil2d_f32(4, 4, 8, 16, 0, 0, None) == gbblas.OK                # no sweeps
    assert L.gb_fill_f32(8, 2, 2, 2, 1, 3, None) == gbblas.ERR_INVALID_ARG         # kind


def test_exec_rejects_unknown_names_and_bad_packing(L):
    arr = (ctypes.c_ulong * 10)(*range(10))
    assert L.gb_exec(b"launch_nothing_NN", 7, 3, arr) == gbblas.ERR_INVALID_ARG
    assert L.gb_exec(b"launch_dgemm_NN", 6, 3, arr) == gbblas.ERR_INVALID_ARG      # needs 7 scalars
    assert L.gb_exec(b"launch_dgemm_TN", 7, 3, arr) == gbblas.ERR_INVALID_ARG      # TN needs 8
    assert L.gb_exec(b"launch_sgemm_NX", 4, 3, arr) == gbblas.ERR_INVALID_ARG
    assert L.gb_exec(b"launch_dgemm_null", 7, 3, arr) == gbblas.OK                 # no-op kernels
    assert L.gb_exec(b"stencil_vector", 1, 2, arr) == gbblas.ERR_INVALID_ARG


def test_null_kernels_are_noops(L):
    assert gbblas.ref_call("sgemm_null", 4, 4, 4, 0, 0, 0, 0, 1.0, 1.0) == gbblas.OK
    assert gbblas.ref_call("stencil_null", 4, 4, 0, 0) == gbblas.OK


def test_auto_algorithm_choice(L):
    assert gbblas.pick_algo(32, "N", "N", 262144, 8, 4096) == gbblas.ALGO_SKINNY
    assert gbblas.pick_algo(32, "N", "N", 262144, 64, 4096) == gbblas.ALGO_SKINNY
    assert gbblas.pick_algo(64, "T", "T", 16, 262144, 4096) == gbblas.ALGO_SKINNY
    assert gbblas.pick_algo(64, "T", "T", 48, 262144, 4096) == gbblas.ALGO_SKINNY
    assert gbblas.pick_algo(64, "T", "T", 16, 2000, 1000) == gbblas.ALGO_SKINNY
    assert gbblas.pick_algo(64, "N", "N", 512, 512, 512) == gbblas.ALGO_ORDERED
    assert gbblas.pick_algo(64, "N", "N", 1024, 1024, 1024) == gbblas.ALGO_OZAKI
    assert gbblas.pick_algo(32, "N", "N", 4096, 4096, 4096) == gbblas.ALGO_BF16X3
    assert gbblas.pick_algo(32, "N", "N", 256, 256, 256) == gbblas.ALGO_SIMT


@pytest.mark.parametrize("lang", ["c99", "c++17"])
def test_headers_compile_and_link(lang, tmp_path):
    """The public headers as a reference-side host program uses them: valid
    C99 and C++ with all warnings as errors, every call family links."""
    import shutil
    import subprocess
    import gbblas
    if not os.path.exists(gbblas.LIB_PATH):
        pytest.skip("libgbblas.so not built")
    cc = "gcc" if lang == "c99" else "g++"
    if not shutil.which(cc):
        pytest.skip(cc + " not found")
    repo = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    src = os.path.join(repo, "tests", "c", "abi_compile.c")
    flags = ["-std=c99", "-x", "c"] if lang == "c99" else ["-std=c++17", "-x", "c++"]
    out = str(tmp_path / "abi")
    libdir = os.path.dirname(gbblas.LIB_PATH)
    r = subprocess.run([cc] + flags + ["-Wall", "-Wextra", "-Werror", "-pedantic", "-I", os.path.join(repo, "include"),
                        src, "-x", "none", "-L" + libdir, "-lgbblas", "-Wl,-rpath," + libdir, "-o", out],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
    assert subprocess.run([out], capture_output=True).returncode == 0


def test_workspace_query_two_pass_forms_and_validation(L):
    """The workspace bound of the split-operand forms is the two halves of
    up to three 16-bit pieces per operand value (K padded to 64); forms that
    keep no scratch report 0; bad arguments are refused like a call's."""
    M, N, K = 1000, 700, 900
    kp = (K + 63) // 64 * 64
    want = 2 * (3 * (M + N) * kp * 2 + (M + N) * 4 + 1024) + 4096
    for algo in (gbblas.ALGO_BF16X3, gbblas.ALGO_BF16X6, gbblas.ALGO_FP16X3):
        assert gbblas.workspace_query(32, "N", "T", M, N, K, K, K, algo=algo) == want
    assert gbblas.workspace_query(32, "N", "N", M, N, K, K, N, algo=gbblas.ALGO_SIMT) == 0
    assert gbblas.workspace_query(64, "T", "N", M, N, K, M, N, algo=gbblas.ALGO_ORDERED) == 0
    assert gbblas.workspace_query(32, "N", "N", 0, N, K, K, N, algo=gbblas.ALGO_BF16X3) == 0
    n = ctypes.c_size_t(7)
    o = gbblas.opts()
    assert L.gb_workspace_query(16, b"N", b"N", 4, 4, 4, None, 4, None, 4, ctypes.byref(o),
                                ctypes.byref(n)) == gbblas.ERR_INVALID_ARG
    assert b"dtype_bits" in L.gb_last_error() and n.value == 0
    assert L.gb_workspace_query(32, b"X", b"N", 4, 4, 4, None, 4, None, 4, ctypes.byref(o),
                                ctypes.byref(n)) == gbblas.ERR_INVALID_ARG
    assert L.gb_last_error_string() == L.gb_last_error()
    o = gbblas.opts(algo=gbblas.ALGO_OZAKI, ozaki_slices=1)
    assert L.gb_workspace_query(64, b"N", b"N", 4, 4, 4, None, 4, None, 4, ctypes.byref(o),
                                ctypes.byref(n)) == gbblas.ERR_INVALID_ARG
    assert L.gb_workspace_query(32, b"N", b"N", 4, 4, 4, None, 4, None, 4, ctypes.byref(o),
                                None) == gbblas.ERR_INVALID_ARG


@pytest.mark.parametrize("lang", ["c99", "c++17"])
def test_serving_loop_from_c_dry_run(lang, tmp_path):
    """The serving calls and the workspace query from a C (and C++) program,
    on a dry-run server: struct layouts, defaults, routing to the urgent
    streams and the statistics as the header declares them."""
    import shutil
    import subprocess
    import gbblas
    if not os.path.exists(gbblas.LIB_PATH):
        pytest.skip("libgbblas.so not built")
    cc = "gcc" if lang == "c99" else "g++"
    if not shutil.which(cc):
        pytest.skip(cc + " not found")
    repo = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    src = os.path.join(repo, "tests", "c", "server_dryrun.c")
    flags = ["-std=c99", "-x", "c"] if lang == "c99" else ["-std=c++17", "-x", "c++"]
    out = str(tmp_path / "server_dryrun")
    libdir = os.path.dirname(gbblas.LIB_PATH)
    r = subprocess.run([cc] + flags + ["-Wall", "-Wextra", "-Werror", "-pedantic", "-I", os.path.join(repo, "include"),
                        src, "-x", "none", "-L" + libdir, "-lgbblas", "-Wl,-rpath," + libdir, "-o", out],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
    run = subprocess.run([out], capture_output=True, text=True, timeout=60)
    assert run.returncode == 0, (run.returncode, run.stdout, run.stderr)
    assert "server dry run ok" in run.stdout
