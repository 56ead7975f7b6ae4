"""GEMM on the GPU against the oracle.

* ORDERED: bit-exact with the reference's host check loops -- the golden
  fixtures (results of the reference demos' own CPU loops) through the
  launch-by-name boundary and the reference-named entry points, and the
  oracle on seeded U[-1,1] inputs (512^3 DGEMM, all four modes).
* Fast algorithms: normwise error against the Dot2 oracle <= 2*K*u
  (u = 2^-24 FP32, 2^-53 FP64), the GEMM tolerance.
"""
import numpy as np
import pytest

import golden_cases as gc
import oracle
from gpu_util import dev, host, op_shape, torch_cuda, u_bound

pytestmark = pytest.mark.gpu
MODES = ["NN", "NT", "TN", "TT"]


@pytest.fixture(scope="module")
def torch():
    return torch_cuda()


# ----------------------------------------------------------- golden fixtures
def _launch_name(demo, mode):
    return {"dgemm_v11": "launch_dgemm_", "sgemm_v132": "launch_sgemm_",
            "shortA_dgemm_v00": "launch_irr_shortA_dgemm_", "shortA_sgemm_v00": "launch_irr_shortA_sgemm_",
            "thinB_dgemm_v00": "launch_irr_thinB_dgemm_", "thinB_sgemm_v12": "launch_irr_thinB_sgemm_"}[demo] + mode


@pytest.mark.parametrize("name", [n for n in gc.gemm_names()
                                  if gc.index()[n]["demo"] not in ("sgemm_v131", "thinB_sgemm_v00")])
def test_golden_via_exec_bit_exact(torch, name):
    import gbblas
    meta, ops, ldc, crows = gc.gemm_case(name)
    M, K, N = meta["M"], meta["K"], meta["N"]
    dt = np.float64 if meta["dtype"] == "float64" else np.float32
    want = gc.expected(meta)
    for mode in MODES:
        A, lda, B, ldb = ops[mode]
        dA, dB = dev(A), dev(B)
        dC = dev(np.zeros((crows, ldc), dtype=dt))
        for _ in range(meta.get("repeats", 1)):
            if meta["demo"] == "dgemm_v11":
                bid = [0, 0] if mode == "TN" else [0]
                gbblas.exec_by_name(_launch_name(meta["demo"], mode), [lda, ldb, ldc, M, N, K] + bid, [dA, dB, dC])
            else:
                two_bids = {"sgemm_v132": ("TN",), "shortA_dgemm_v00": ("TN", "TT"), "shortA_sgemm_v00": ("TN", "TT"),
                            "thinB_dgemm_v00": ("TN", "NN"), "thinB_sgemm_v12": ("TN", "NN")}[meta["demo"]]
                bid = [0, 0] if mode in two_bids else [0]
                gbblas.exec_by_name(_launch_name(meta["demo"], mode), [M, N, K] + bid, [dA, dB, dC])
        got = host(dC)[:M, :N]
        assert got.tobytes() == want.tobytes(), (name, mode, np.abs(got - want).max())


@pytest.mark.parametrize("name", ["sgemm_v131_16x600x24", "thinB_sgemm_v00_96x1100x16"])
def test_golden_other_versions_bit_exact(torch, name):
    """sgemm V1.3.1 (accumulate) and irr_thinB_sgemm V0.0 (C += AB) through gb_sgemm."""
    import gbblas
    meta, ops, ldc, crows = gc.gemm_case(name)
    M, K, N = meta["M"], meta["K"], meta["N"]
    want = gc.expected(meta)
    for mode in MODES:
        A, lda, B, ldb = ops[mode]
        dA, dB, dC = dev(A), dev(B), dev(np.zeros((M, N), np.float32))
        if meta["demo"] == "sgemm_v131":
            gbblas.sgemm(mode[0], mode[1], M, N, K, 5.0, dA, lda, dB, ldb, 3.0, dC, N,
                         algo=gbblas.ALGO_ORDERED, semantics=gbblas.SEM_ACCUM_SCALAR_BETA)
        else:
            gbblas.sgemm(mode[0], mode[1], M, N, K, 1.0, dA, lda, dB, ldb, 1.0, dC, N, algo=gbblas.ALGO_ORDERED)
        assert host(dC).tobytes() == want.tobytes(), (name, mode)


def test_golden_via_reference_named_entry_points(torch):
    import gbblas
    meta, ops, ldc, crows = gc.gemm_case("dgemm_v11_20x1030x36")
    M, K, N = meta["M"], meta["K"], meta["N"]
    want = gc.expected(meta)
    for mode in MODES:
        A, lda, B, ldb = ops[mode]
        dA, dB, dC = dev(A), dev(B), dev(np.zeros((crows, ldc)))
        args = [lda, ldb, ldc, M, N, K, 0] + ([0] if mode == "TN" else []) + [dA, dB, dC]
        assert gbblas.ref_call("dgemm_" + mode, *args) == gbblas.OK
        gbblas.sync()
        assert host(dC)[:M, :N].tobytes() == want.tobytes(), mode
    meta, ops, ldc, crows = gc.gemm_case("sgemm_v132_24x1100x40")
    M, K, N = meta["M"], meta["K"], meta["N"]
    want = gc.expected(meta)
    for mode in MODES:
        A, lda, B, ldb = ops[mode]
        dA, dB, dC = dev(A), dev(B), dev(np.full((M, N), 999.0, np.float32))
        args = [M, N, K, 0] + ([0] if mode == "TN" else []) + [dA, dB, dC, 5.0, 3.0]
        assert gbblas.ref_call("sgemm_%s_qxx" % mode, *args) == gbblas.OK
        gbblas.sync()
        assert host(dC).tobytes() == want.tobytes(), mode


# ------------------------------------------------- seeded inputs vs oracle
def _inputs(ta, tb, M, N, K, dtype, seed, pad=0, kind=0):
    ar, ac = op_shape(ta, M, K)
    br, bc = op_shape(tb, K, N)
    A = oracle.fill(ar, ac, seed * 10 + 1, kind=kind, dtype=dtype, ld=ac + pad)
    B = oracle.fill(br, bc, seed * 10 + 2, kind=kind, dtype=dtype, ld=bc + pad)
    C = oracle.fill(M, N, seed * 10 + 3, kind=kind, dtype=dtype, ld=N + pad)
    return A, ac + pad, B, bc + pad, C, N + pad


@pytest.mark.parametrize("mode", MODES)
def test_dgemm_512_config_ordered_bit_exact(torch, mode):
    """DGEMM C = A x B + C, FP64, M=N=K=512, ld=512, U[-1,1] seed 0."""
    import gbblas
    ta, tb = mode
    M = N = K = 512
    A, lda, B, ldb, C0, ldc = _inputs(ta, tb, M, N, K, np.float64, 0)
    want = C0.copy()
    oracle.dgemm_ref(ta, tb, M, N, K, A, lda, B, ldb, want, ldc)
    for algo in (gbblas.ALGO_ORDERED, gbblas.ALGO_AUTO):
        dC = dev(C0)
        gbblas.dgemm(ta, tb, M, N, K, 1.0, dev(A), lda, dev(B), ldb, 1.0, dC, ldc, algo=algo)
        assert host(dC).tobytes() == want.tobytes()


@pytest.mark.parametrize("mode", MODES)
@pytest.mark.parametrize("algo_name", ["DMMA", "SIMT"])
def test_dgemm_fast_normwise(torch, mode, algo_name):
    import gbblas
    algo = getattr(gbblas, "ALGO_" + algo_name)
    ta, tb = mode
    M, N, K = 200, 136, 515
    A, lda, B, ldb, C0, ldc = _inputs(ta, tb, M, N, K, np.float64, 1, pad=3)
    dC = dev(C0)
    gbblas.dgemm(ta, tb, M, N, K, 0.75, dev(A), lda, dev(B), ldb, -1.25, dC, ldc, algo=algo)
    err, _ = oracle.normwise_error(host(dC), ta, tb, M, N, K, 0.75, A, lda, B, ldb, -1.25, C0, ldc)
    assert err <= 2 * K * u_bound(np.float64), err


@pytest.mark.parametrize("mode", MODES)
def test_sgemm_ordered_scalar_beta_bit_exact(torch, mode):
    """sgemm V1.3.2 semantics (C = alpha op(A)op(B) + beta) in the reference order."""
    import gbblas
    ta, tb = mode
    M, N, K = 70, 90, 1100
    A, lda, B, ldb, C0, ldc = _inputs(ta, tb, M, N, K, np.float32, 2, pad=5)
    want = C0.copy()
    oracle.sgemm_ref(ta, tb, M, N, K, 1.5, A, lda, B, ldb, -0.5, want, ldc)
    dC = dev(C0)
    gbblas.sgemm(ta, tb, M, N, K, 1.5, dev(A), lda, dev(B), ldb, -0.5, dC, ldc,
                 algo=gbblas.ALGO_ORDERED, semantics=gbblas.SEM_SCALAR_BETA)
    assert host(dC).tobytes() == want.tobytes()


@pytest.mark.parametrize("mode", MODES)
def test_sgemm_simt_384x320x1040_padded_ld_normwise(torch, mode):
    """SGEMM BLAS semantics, alpha=1.5 beta=-0.5, leading dimensions padded by
    16 (the 4096^3 ld-4112 configuration itself: test_gpu_configs_full.py)."""
    import gbblas
    ta, tb = mode
    M, N, K = 384, 320, 1040
    A, lda, B, ldb, C0, ldc = _inputs(ta, tb, M, N, K, np.float32, 3, pad=16)
    dC = dev(C0)
    gbblas.sgemm(ta, tb, M, N, K, 1.5, dev(A), lda, dev(B), ldb, -0.5, dC, ldc, algo=gbblas.ALGO_SIMT)
    err, _ = oracle.normwise_error(host(dC), ta, tb, M, N, K, 1.5, A, lda, B, ldb, -0.5, C0, ldc)
    assert err <= 2 * K * u_bound(np.float32), err


@pytest.mark.parametrize("dtype", [np.float32, np.float64])
@pytest.mark.parametrize("M,N,K", [(1, 1, 1), (3, 5, 0), (129, 1, 7), (1, 129, 513), (67, 65, 33)])
def test_gemm_edge_shapes(torch, dtype, M, N, K):
    import gbblas
    bits = 64 if dtype == np.float64 else 32
    for mode in MODES:
        ta, tb = mode
        A, lda, B, ldb, C0, ldc = _inputs(ta, tb, M, N, K, dtype, 4)
        algos = [gbblas.ALGO_ORDERED, gbblas.ALGO_AUTO, gbblas.ALGO_SIMT]
        if min(M, N) <= 64:
            algos.append(gbblas.ALGO_SKINNY)
        for algo in algos:
            dC = dev(C0)
            gbblas.gemm(ta, tb, M, N, K, 1.0, dev(A), max(lda, 1), dev(B), max(ldb, 1), 1.0, dC, ldc, bits, algo=algo)
            got = host(dC)
            if algo == gbblas.ALGO_ORDERED:
                want = C0.copy()
                if dtype == np.float64:
                    oracle.dgemm_ref(ta, tb, M, N, K, A, lda, B, ldb, want, ldc)
                else:
                    oracle.sgemm_irr_ref(ta, tb, M, N, K, A, lda, B, ldb, want, ldc)
                assert got.tobytes() == want.tobytes(), (mode, algo)
            elif K > 0:
                err, _ = oracle.normwise_error(got, ta, tb, M, N, K, 1.0, A, lda, B, ldb, 1.0, C0, ldc)
                assert err <= 2 * K * u_bound(dtype), (mode, algo, err)
            else:
                assert np.array_equal(got, C0)


def test_skinny_rejects_wide_shapes(torch):
    import gbblas
    z = dev(np.zeros((70, 70), np.float32))
    with pytest.raises(gbblas.GBError) as e:
        gbblas.sgemm("N", "N", 70, 70, 70, 1.0, z, 70, z, 70, 0.0, dev(np.zeros((70, 70), np.float32)), 70,
                     algo=gbblas.ALGO_SKINNY)
    assert e.value.status == gbblas.ERR_UNSUPPORTED


@pytest.mark.parametrize("dtype", [np.float32, np.float64])
@pytest.mark.parametrize("kind", ["thinB", "shortA"])
@pytest.mark.parametrize("small", [8, 16, 33, 64])
def test_skinny_normwise(torch, dtype, kind, small):
    import gbblas
    bits = 64 if dtype == np.float64 else 32
    big, K = 3000, 1100
    M, N = (big, small) if kind == "thinB" else (small, big)
    for mode in MODES:
        ta, tb = mode
        A, lda, B, ldb, C0, ldc = _inputs(ta, tb, M, N, K, dtype, 5)
        dC = dev(C0)
        gbblas.gemm(ta, tb, M, N, K, 0.5, dev(A), lda, dev(B), ldb, 2.0, dC, ldc, bits, algo=gbblas.ALGO_SKINNY)
        rows = np.arange(0, M, max(1, M // 64))
        cols = np.arange(0, N, max(1, N // 64))
        err, _ = oracle.normwise_error(host(dC), ta, tb, M, N, K, 0.5, A, lda, B, ldb, 2.0, C0, ldc, rows, cols)
        assert err <= 2 * K * u_bound(dtype), (mode, err)


def test_skinny_split_k_and_scalar_beta(torch):
    """small row count forces split-K through the workspace; scalar-beta epilogue."""
    import gbblas
    M, N, K = 300, 8, 20000
    A, lda, B, ldb, C0, ldc = _inputs("N", "N", M, N, K, np.float32, 6)
    dC = dev(C0)
    gbblas.sgemm("N", "N", M, N, K, 1.0, dev(A), lda, dev(B), ldb, 0.25, dC, ldc, algo=gbblas.ALGO_SKINNY,
                 semantics=gbblas.SEM_SCALAR_BETA)
    ref = oracle.gemm_dot2("N", "N", M, N, K, 1.0, A, lda, B, ldb, 0.0, None, ldc, np.arange(M), np.arange(N)) + 0.25
    got = host(dC).astype(np.float64)
    rn2, cn2 = oracle.op_norms("N", "N", M, N, K, A, lda, B, ldb, np.arange(M), np.arange(N))
    assert np.linalg.norm(got - ref) / (np.sqrt(rn2.sum() * cn2.sum())) <= 2 * K * 2.0 ** -24
