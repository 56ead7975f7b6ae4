"""Seeded input generators for the tests (numpy restatement).

TEST INFRASTRUCTURE.  Two families:

* ``fill`` -- the project's counter-based generator, bit-identical to
  ``gbo_fill_*`` in oracle/oracle.c and to ``gb_fill_*`` in the CUDA library:
  element (r, c) of a rows x cols matrix is a SplitMix64 finaliser of
  ``mix(seed) + (r*cols + c + 1) * 0x9E3779B97F4A7C15``.
* ``demo_*`` -- the inputs the reference's own host demos generate, replayed
  exactly, for the golden fixtures made by tests/golden/make_golden.py (the
  demos were compiled with ``rand()`` replaced by the same counter stream,
  seed 0xC0FFEE, drawn sequentially).
"""
import numpy as np

_M1 = np.uint64(0xBF58476D1CE4E5B9)
_M2 = np.uint64(0x94D049BB133111EB)
_G = np.uint64(0x9E3779B97F4A7C15)
RAND_MAX = 2147483647
DEMO_RAND_SEED = 0xC0FFEE


def mix64(z):
    z = np.asarray(z, dtype=np.uint64)
    with np.errstate(over="ignore"):
        z = (z ^ (z >> np.uint64(30))) * _M1
        z = (z ^ (z >> np.uint64(27))) * _M2
    return z ^ (z >> np.uint64(31))


def bits(seed, idx):
    s = mix64(np.uint64(seed & 0xFFFFFFFFFFFFFFFF))
    with np.errstate(over="ignore"):
        return mix64(s + (np.asarray(idx, dtype=np.uint64) + np.uint64(1)) * _G)


def unit(seed, idx):
    return (bits(seed, idx) >> np.uint64(11)).astype(np.float64) * 2.0 ** -53


def values(seed, idx, kind=0):
    u = unit(seed, idx)
    if kind == 1:
        return u
    v = 2.0 * u - 1.0
    if kind == 2:
        e = (bits(seed ^ 0x5851F42D4C957F2D, idx) % np.uint64(41)).astype(np.int64) - 20
        v = np.ldexp(v, e)
    return v


def fill(rows, cols, seed, kind=0, dtype=np.float64, ld=None):
    """rows x cols matrix (optionally embedded in a rows x ld buffer)."""
    idx = np.arange(rows * cols, dtype=np.uint64)
    v = values(seed, idx, kind).reshape(rows, cols)
    if dtype == np.float32:
        v = v.astype(np.float32)
    if ld is None or ld == cols:
        return np.ascontiguousarray(v)
    out = np.zeros((rows, ld), dtype=dtype)
    out[:, :cols] = v
    return out


# --------------------------------------------------------- reference demos
def demo_rand(n, start=0):
    """n draws of the counter-based rand() the demos were compiled with."""
    idx = np.arange(start, start + n, dtype=np.uint64)
    return (bits(DEMO_RAND_SEED, idx) >> np.uint64(33)).astype(np.int64)


def demo_dgemm_v11(M, K, N):
    """dgemm_release_V1.1/host_code/dgemm_demo.c:44-85 (padded buffers)."""
    M0, K0, N0 = M + 64, K + 128, N + 256
    r = demo_rand(M0 * K0 + K0 * N0)
    vals = r.astype(np.float64) / RAND_MAX * 2.0 + 2.0
    A = vals[: M0 * K0].reshape(M0, K0).copy()
    B = vals[M0 * K0:].reshape(K0, N0).copy()
    return dict(A=A, AT=np.ascontiguousarray(A.T), B=B, BT=np.ascontiguousarray(B.T),
                lda=K0, ldaT=M0, ldb=N0, ldbT=K0, ldc=N0, M0=M0, N0=N0)


def demo_sgemm(M, K, N):
    """sgemm_release_V1.3.x/host_code/sgemm_demo.c:66-79:
    (float)rand() / RAND_MAX (float division, RAND_MAX -> 2^31 as float),
    * 2.0 + 2.0 in double, stored as float."""
    r = demo_rand(M * K + K * N)
    f = r.astype(np.float32) / np.float32(RAND_MAX)
    vals = (f.astype(np.float64) * 2.0 + 2.0).astype(np.float32)
    A = vals[: M * K].reshape(M, K).copy()
    B = vals[M * K:].reshape(K, N).copy()
    return dict(A=A, AT=np.ascontiguousarray(A.T), B=B, BT=np.ascontiguousarray(B.T))


def demo_irr(M, K, N, dtype):
    """irr_*_demo.c:63-78: A = OFFSET(i,j,K) % 11, B = OFFSET(i,j,N) % 7."""
    A = (np.arange(M * K, dtype=np.int64) % 11).astype(dtype).reshape(M, K)
    B = (np.arange(K * N, dtype=np.int64) % 7).astype(dtype).reshape(K, N)
    return dict(A=A, AT=np.ascontiguousarray(A.T), B=B, BT=np.ascontiguousarray(B.T))


def demo_transpose(M, N):
    """transpose/host_code/transpose.c:49-56: A[i] = i % 7 (float)."""
    return (np.arange(M * N, dtype=np.int64) % 7).astype(np.float32).reshape(M, N)


def demo_stencil(M, N):
    """stencil_2d_V1.2/host_code/matrix_stencil.c:72-83: zero halo, interior
    1.0 * rand() / RAND_MAX drawn row by row."""
    A = np.zeros((M + 2, N + 2), dtype=np.float64)
    r = demo_rand(M * N)
    A[1:M + 1, 1:N + 1] = (1.0 * r.astype(np.float64) / RAND_MAX).reshape(M, N)
    return A
