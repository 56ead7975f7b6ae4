"""Helpers for the GPU parity tests (test infrastructure)."""
import numpy as np
import pytest


def torch_cuda():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import gbblas
    gbblas.lib()
    assert gbblas.arch() == 103, "these kernels are built for sm_103a only"
    return torch


def dev(x):
    import torch
    return torch.from_numpy(np.ascontiguousarray(x)).to("cuda:0")


def host(t):
    import torch
    torch.cuda.synchronize()
    return t.cpu().numpy()


def u_bound(dtype):
    return 2.0 ** -24 if dtype == np.float32 else 2.0 ** -53


def op_shape(t, rows, cols):
    """storage shape of op(X) = rows x cols"""
    return (cols, rows) if t == "T" else (rows, cols)
