"""The configurations the GEMM path is quoted on, at their full sizes.

Inputs come from the library's seeded generator on the device (bit-identical
to the oracle's) with the seeds bench.py uses; the Dot2 accuracy oracle
checks a seeded subgrid of rows and columns, read back as compact host
copies (the sampled rows of op(A) and columns of op(B), both K-contiguous)
so that the compensated dot products stream through memory.

* SGEMM 4096^3, leading dimensions 4112, alpha 1.5, beta -0.5, all four
  modes: plain FFMA, BF16X3, BF16X6 and FP16X3 within 2*K*u32; the forms
  that claim FP32-level error (BF16X6, FP16X3) no worse than FFMA.
* thinB / shortA with 262144 rows (columns), K = 4096, FP32 and FP64: within
  2*K*u on a row (column) sample.
* DGEMM 8192^3 NN and TT, entries u * 2^e (e in [-20, 20]): the Ozaki form at
  the slice count the library picks for FP64-level error is no worse than
  native FP64 (DMMA and DFMA) on a seeded 1024 x 1024 subgrid.
* The Ozaki slice selector: a normwise target is met.
"""
import numpy as np
import pytest

import oracle
from gpu_util import torch_cuda

pytestmark = pytest.mark.gpu
MODES = ["NN", "NT", "TN", "TT"]


@pytest.fixture(scope="module")
def torch():
    t = torch_cuda()
    yield t
    t.cuda.empty_cache()


def _fill(torch, rows, cols, ld, seed, kind, bits):
    import gbblas
    # the padding columns keep a finite sentinel (never recycled memory, which may hold NaNs)
    t = torch.full((rows, ld), 7.25, dtype=torch.float64 if bits == 64 else torch.float32, device="cuda:0")
    gbblas.fill(t, rows, cols, ld, seed, kind, bits)
    return t


def _op_rows(X, t, idx, K):
    """Rows idx of op(X) (op(X) = X^T when t == 'T'), K-contiguous, on the host."""
    import torch
    ix = torch.as_tensor(idx, device=X.device)
    sub = X[ix, :K] if t == "N" else X[:K, ix].t()
    return np.ascontiguousarray(sub.cpu().numpy())


def _op_cols(X, t, idx, K):
    """Columns idx of op(X) as rows (op(X)^T rows), K-contiguous, on the host."""
    import torch
    ix = torch.as_tensor(idx, device=X.device)
    sub = X[:K, ix].t() if t == "N" else X[ix, :K]
    return np.ascontiguousarray(sub.cpu().numpy())


def _sub_error(C, rows, cols, ref, rn2, cn2, alpha, beta, c0sub):
    """The oracle's normwise metric on the subgrid, from the device result C."""
    import torch
    got = C[torch.as_tensor(rows, device=C.device)][:, torch.as_tensor(cols, device=C.device)]
    got = got.cpu().numpy().astype(np.float64)
    den = abs(alpha) * np.sqrt(rn2.sum()) * np.sqrt(cn2.sum())
    if beta != 0:
        den += abs(beta) * np.linalg.norm(c0sub.astype(np.float64))
    return float(np.linalg.norm(got - ref) / den)


def _reference(ta, tb, Adev, Bdev, C0dev, K, alpha, beta, rows, cols):
    """Dot2 reference and op norms on the subgrid (compact N x T problem)."""
    import torch
    a = _op_rows(Adev, ta, rows, K)
    b = _op_cols(Bdev, tb, cols, K)
    c0 = C0dev[torch.as_tensor(rows, device=C0dev.device)][:, torch.as_tensor(cols, device=C0dev.device)]
    c0 = np.ascontiguousarray(c0.cpu().numpy())
    nr, nc = len(rows), len(cols)
    ref = oracle.gemm_dot2("N", "T", nr, nc, K, alpha, a, K, b, K, beta, c0, nc, np.arange(nr), np.arange(nc))
    rn2, cn2 = oracle.op_norms("N", "T", nr, nc, K, a, K, b, K, np.arange(nr), np.arange(nc))
    return ref, rn2, cn2, c0


# ------------------------------------------------------------- SGEMM 4096^3
@pytest.mark.parametrize("mode", MODES)
def test_sgemm_4096_ld4112_alpha1p5_beta_m0p5_all_forms(torch, mode):
    import gbblas
    M = N = K = 4096
    LD = 4112
    ALPHA, BETA = 1.5, -0.5
    ta, tb = mode
    seeds = {"A_N": 11, "A_T": 12, "B_N": 13, "B_T": 14, "C": 15}   # bench.py's
    A = _fill(torch, M, K, LD, seeds["A_T" if ta == "T" else "A_N"], 0, 32)
    B = _fill(torch, M, K, LD, seeds["B_T" if tb == "T" else "B_N"], 0, 32)
    C0 = _fill(torch, M, N, LD, seeds["C"], 0, 32)
    rng = np.random.default_rng(1)
    rows = np.sort(rng.choice(M, 256, replace=False))
    cols = np.sort(rng.choice(N, 256, replace=False))
    ref, rn2, cn2, c0 = _reference(ta, tb, A, B, C0, K, ALPHA, BETA, rows, cols)
    errs = {}
    for name in ("SIMT", "BF16X3", "BF16X6", "FP16X3"):
        C = C0.clone()
        gbblas.sgemm(ta, tb, M, N, K, ALPHA, A, LD, B, LD, BETA, C, LD, algo=getattr(gbblas, "ALGO_" + name))
        torch.cuda.synchronize()
        errs[name] = _sub_error(C, rows, cols, ref, rn2, cn2, ALPHA, BETA, c0)
        # the padding columns of C are never written
        assert torch.equal(C[:, N:], C0[:, N:]), name
    bound = 2 * K * 2.0 ** -24
    assert all(e <= bound for e in errs.values()), errs
    assert errs["BF16X6"] <= errs["SIMT"], errs
    assert errs["FP16X3"] <= errs["SIMT"], errs


# ---------------------------------------------------- thinB / shortA, full size
CASES3 = [(32, "thinB", 64, "NN"), (32, "thinB", 8, "TN"), (32, "shortA", 16, "NT"), (32, "shortA", 8, "TT"),
          (64, "thinB", 16, "NN"), (64, "thinB", 64, "TT"), (64, "shortA", 32, "NT"), (64, "shortA", 8, "TN")]


@pytest.mark.parametrize("bits,kind,small,mode", CASES3)
def test_skinny_262144_rows_full_size(torch, bits, kind, small, mode):
    import gbblas
    big, K = 262144, 4096
    M, N = (big, small) if kind == "thinB" else (small, big)
    ta, tb = mode
    ar, ac = (K, M) if ta == "T" else (M, K)
    br, bc = (N, K) if tb == "T" else (K, N)
    A = _fill(torch, ar, ac, ac, 21 + (ta == "T"), 0, bits)      # bench.py's seeds
    B = _fill(torch, br, bc, bc, 23 + (tb == "T"), 0, bits)
    C0 = _fill(torch, M, N, N, 25, 0, bits)
    C = C0.clone()
    gbblas.gemm(ta, tb, M, N, K, 1.0, A, ac, B, bc, 1.0, C, N, bits, algo=gbblas.ALGO_AUTO)
    torch.cuda.synchronize()
    rng = np.random.default_rng(2)
    rows = np.sort(rng.choice(M, 512, replace=False)) if M == big else np.arange(M)
    cols = np.sort(rng.choice(N, 512, replace=False)) if N == big else np.arange(N)
    ref, rn2, cn2, c0 = _reference(ta, tb, A, B, C0, K, 1.0, 1.0, rows, cols)
    err = _sub_error(C, rows, cols, ref, rn2, cn2, 1.0, 1.0, c0)
    u = 2.0 ** -53 if bits == 64 else 2.0 ** -24
    assert err <= 2 * K * u, err
    del A, B, C0, C
    torch.cuda.empty_cache()


# ------------------------------------------------------------- DGEMM 8192^3
@pytest.mark.parametrize("mode", ["NN", "TT"])
def test_dgemm_8192_ozaki_no_worse_than_native(torch, mode):
    import gbblas
    n = 8192
    ta, tb = mode
    seeds = {"A": 31, "AT": 33, "B": 32, "BT": 34, "C": 35}   # bench.py's
    A = _fill(torch, n, n, n, seeds["AT" if ta == "T" else "A"], 2, 64)
    B = _fill(torch, n, n, n, seeds["BT" if tb == "T" else "B"], 2, 64)
    C0 = _fill(torch, n, n, n, seeds["C"], 2, 64)
    rng = np.random.default_rng(3)
    rows = np.sort(rng.choice(n, 1024, replace=False))
    cols = np.sort(rng.choice(n, 1024, replace=False))
    ref, rn2, cn2, c0 = _reference(ta, tb, A, B, C0, n, 1.0, 1.0, rows, cols)
    errs = {}
    for name in ("OZAKI", "DMMA", "ORDERED"):
        C = C0.clone()
        gbblas.dgemm(ta, tb, n, n, n, 1.0, A, n, B, n, 1.0, C, n, algo=getattr(gbblas, "ALGO_" + name))
        torch.cuda.synchronize()
        errs[name] = _sub_error(C, rows, cols, ref, rn2, cn2, 1.0, 1.0, c0)
        del C
    assert errs["OZAKI"] <= errs["DMMA"] and errs["OZAKI"] <= errs["ORDERED"], errs
    assert errs["OZAKI"] <= 2 * n * 2.0 ** -53, errs
    del A, B, C0
    torch.cuda.empty_cache()


@pytest.mark.parametrize("kind", [0, 2])
@pytest.mark.parametrize("target", [1e-5, 1e-8, 1e-11, 1e-14])
def test_ozaki_slice_selector_meets_target(torch, kind, target):
    """ozaki_slices = 0 with a normwise target: the slice count the library
    picks for this K meets the target (U[-1,1] and u * 2^e inputs)."""
    import gbblas
    M, N, K = 1024, 768, 4096
    A = _fill(torch, M, K, K, 41, kind, 64)
    B = _fill(torch, K, N, N, 42, kind, 64)
    C0 = _fill(torch, M, N, N, 43, kind, 64)
    C = C0.clone()
    gbblas.dgemm("N", "N", M, N, K, 1.0, A, K, B, N, 1.0, C, N, algo=gbblas.ALGO_OZAKI, target_err=target)
    torch.cuda.synchronize()
    rows = np.arange(0, M, 4)
    cols = np.arange(0, N, 4)
    ref, rn2, cn2, c0 = _reference("N", "N", A, B, C0, K, 1.0, 1.0, rows, cols)
    err = _sub_error(C, rows, cols, ref, rn2, cn2, 1.0, 1.0, c0)
    assert err <= target, (target, err)
