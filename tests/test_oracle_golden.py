"""The oracle against the golden fixtures made from the reference's own
host check loops (bit-exact), and the oracle's generators against numpy."""
import hashlib

import numpy as np
import pytest

import gbgen
import golden_cases as gc
import oracle


def run_oracle_gemm(meta, mode, A, lda, B, ldb, ldc, crows):
    M, K, N = meta["M"], meta["K"], meta["N"]
    dt = np.float64 if meta["dtype"] == "float64" else np.float32
    C = np.zeros((crows, ldc), dtype=dt)
    ta, tb = mode[0], mode[1]
    demo = meta["demo"]
    for _ in range(meta.get("repeats", 1)):
        if dt == np.float64:
            oracle.dgemm_ref(ta, tb, M, N, K, A, lda, B, ldb, C, ldc)
        elif demo.startswith("sgemm"):
            oracle.sgemm_ref(ta, tb, M, N, K, 5.0, A, lda, B, ldb, 3.0, C, ldc,
                             accumulate=(demo == "sgemm_v131"))
        elif demo == "thinB_sgemm_v12":
            oracle.thinB_sgemm_ref(ta, tb, M, N, K, 5.0, A, lda, B, ldb, 3.0, C, ldc)
        else:
            oracle.sgemm_irr_ref(ta, tb, M, N, K, A, lda, B, ldb, C, ldc)
    return C[:M, :N]


@pytest.mark.parametrize("name", gc.gemm_names())
def test_gemm_fixture_bit_exact(name):
    meta, ops, ldc, crows = gc.gemm_case(name)
    assert all(v == "Success!" for v in meta["verdicts"]), meta["verdicts"]
    want = gc.expected(meta)
    for mode in gc.MODES:
        A, lda, B, ldb = ops[mode]
        got = run_oracle_gemm(meta, mode, A, lda, B, ldb, ldc, crows)
        assert got.tobytes() == want.tobytes(), (name, mode)


@pytest.mark.parametrize("M,N", [(312, 228), (1512, 1536)])
def test_transpose_fixture(M, N):
    meta = gc.index()["transpose_f32_%dx%d" % (M, N)]
    A = gbgen.demo_transpose(M, N)
    B = np.zeros((N, M), dtype=np.float32)
    oracle.transpose_into(M, N, A, N, B, M)
    assert hashlib.sha256(B.tobytes()).hexdigest() == meta["sha256"]


@pytest.mark.parametrize("M,N", [(55, 111), (256, 300)])
def test_stencil_fixture(M, N):
    meta = gc.index()["stencil_f64_%dx%d" % (M, N)]
    A = gbgen.demo_stencil(M, N)
    B = np.zeros_like(A)
    oracle.stencil(M, N, A, B, 1, order=0)
    got = np.ascontiguousarray(B[1:M + 1, 1:N + 1])
    assert hashlib.sha256(got.tobytes()).hexdigest() == meta["sha256"]
    if "file" in meta:
        assert got.tobytes() == gc.expected(meta).tobytes()


@pytest.mark.parametrize("kind", [0, 1, 2])
@pytest.mark.parametrize("dtype", [np.float64, np.float32])
def test_generator_matches_numpy(kind, dtype):
    X = oracle.fill(37, 53, 1234567, kind=kind, dtype=dtype, ld=61)
    Y = gbgen.fill(37, 53, 1234567, kind=kind, dtype=dtype, ld=61)
    assert X.tobytes() == Y.tobytes()
    if kind == 0:
        assert X[:, :53].min() >= -1 and X[:, :53].max() <= 1


def test_stencil_orders_differ_but_close():
    M, N = 40, 70
    A = gbgen.fill(M + 2, N + 2, 5, kind=1)
    outs = []
    for order in (0, 1, 2):
        a, b = A.copy(), np.zeros_like(A)
        oracle.stencil(M, N, a, b, 3, order)
        outs.append(b)
    for o in outs[1:]:
        d = np.abs(o - outs[0]).max()
        assert d < 1e-15 and d >= 0


def test_dot2_exact_on_small_integers():
    rng = np.random.default_rng(0)
    A = rng.integers(-50, 50, size=(9, 13)).astype(np.float64)
    B = rng.integers(-50, 50, size=(13, 7)).astype(np.float64)
    C0 = rng.integers(-50, 50, size=(9, 7)).astype(np.float64)
    ref = oracle.gemm_dot2("N", "N", 9, 7, 13, 2.0, A, 13, B, 7, -3.0, C0, 7, np.arange(9), np.arange(7))
    assert np.array_equal(ref, 2.0 * (A @ B) - 3.0 * C0)


def test_dot2_beats_naive_on_ill_conditioned():
    # x . y with massive cancellation: exact answer 1.0
    x = np.array([1e16, 1.0, -1e16], dtype=np.float64).reshape(1, 3)
    y = np.array([1.0, 1.0, 1.0]).reshape(3, 1)
    ref = oracle.gemm_dot2("N", "N", 1, 1, 3, 1.0, x, 3, y, 1, 0.0, None, 1, [0], [0])
    assert ref[0, 0] == 1.0


def test_stencil9_reduces_to_weighted_sum():
    """The 9-point oracle on a tiny grid against a direct numpy evaluation in
    the same fused order (numpy has no fma, so compare with a tolerance and
    check the halo is untouched)."""
    import numpy as np
    M, N = 5, 6
    rng = np.random.default_rng(3)
    w = rng.uniform(-1, 1, size=9)
    A = rng.uniform(0, 1, size=(M + 2, N + 2))
    B = A.copy()
    a, b = A.copy(), B.copy()
    oracle.stencil9(M, N, a, b, 1, w)
    ref = np.zeros((M, N))
    for di in range(3):
        for dj in range(3):
            ref += w[di * 3 + dj] * A[di:di + M, dj:dj + N]
    assert np.allclose(b[1:M + 1, 1:N + 1], ref, rtol=0, atol=1e-14)
    assert np.array_equal(b[0], B[0]) and np.array_equal(b[:, 0], B[:, 0])


@pytest.mark.parametrize("spread,seed", [(0, 1), (20, 2), (60, 3)])
def test_dot2_within_its_published_bound_against_exact_rationals(spread, seed):
    """The accuracy oracle itself: Dot2 (Ogita, Rump & Oishi 2005, Prop. 5.5) satisfies
    |dot2 - x.y| <= u |x.y| + gamma_{n-1}^2 sum |x_i y_i| (u = 2^-53, gamma_k = k u / (1 - k u));
    checked against the exact dot product in rational arithmetic, on entries u * 2^e with e
    spread over [-spread, spread] as in the DGEMM precision study."""
    from fractions import Fraction
    rng = np.random.default_rng(seed)
    K, rows, cols = 400, 3, 4
    A = rng.uniform(-1, 1, size=(rows, K)) * np.exp2(rng.integers(-spread, spread + 1, size=(rows, K)))
    B = rng.uniform(-1, 1, size=(K, cols)) * np.exp2(rng.integers(-spread, spread + 1, size=(K, cols)))
    ref = oracle.gemm_dot2("N", "N", rows, cols, K, 1.0, A, K, B, cols, 0.0, None, cols, np.arange(rows),
                           np.arange(cols))
    u = Fraction(1, 2 ** 53)
    g = (K - 1) * u / (1 - (K - 1) * u)
    for i in range(rows):
        for j in range(cols):
            exact = sum(Fraction(float(A[i, k])) * Fraction(float(B[k, j])) for k in range(K))
            absum = sum(abs(Fraction(float(A[i, k])) * Fraction(float(B[k, j]))) for k in range(K))
            err = abs(Fraction(float(ref[i, j])) - exact)
            assert err <= u * abs(exact) + g * g * absum, (i, j, float(err), float(exact))


def test_normwise_metric_matches_its_definition():
    """normwise_error = ||C - C*||_F / (|alpha| ||op(A)||_F ||op(B)||_F + |beta| ||C0||_F) on the
    sampled rows / columns, recomputed here from numpy norms."""
    rng = np.random.default_rng(5)
    M, N, K = 20, 15, 30
    A = rng.uniform(-1, 1, size=(M, K))
    B = rng.uniform(-1, 1, size=(K, N))
    C0 = rng.uniform(-1, 1, size=(M, N))
    alpha, beta = 1.5, -0.5
    rows, cols = np.array([0, 3, 7, 19]), np.array([1, 2, 14])
    ref = oracle.gemm_dot2("N", "N", M, N, K, alpha, A, K, B, N, beta, C0, N, rows, cols)
    got = ref + 1e-6 * rng.standard_normal(ref.shape)
    C_hat = np.zeros((M, N))
    C_hat[np.ix_(rows, cols)] = got
    e, _ = oracle.normwise_error(C_hat, "N", "N", M, N, K, alpha, A, K, B, N, beta, C0, N, rows, cols)
    den = abs(alpha) * np.linalg.norm(A[rows]) * np.linalg.norm(B[:, cols]) + abs(beta) * np.linalg.norm(
        C0[np.ix_(rows, cols)])
    assert e == pytest.approx(np.linalg.norm(got - ref) / den, rel=1e-12)
