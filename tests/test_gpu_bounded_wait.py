"""Bounded device waits: every mbarrier wait of the TMA / tensor-core kernels
gives up after a time limit, records a code in the per-device error word and
lets the kernel wind down; gb_sync() reports GB_ERR_DEVICE_TIMEOUT once and
clears the word.  gb_selftest_bounded_wait runs that wait on a barrier that
nothing arrives at, with a 1 ms limit, so it gives up on purpose -- no fault,
no hang -- and the device must stay usable."""
import numpy as np
import pytest

from gpu_util import dev, host, torch_cuda

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def torch():
    return torch_cuda()


def test_bounded_wait_gives_up_and_the_device_stays_usable(torch):
    import gbblas
    L = gbblas.lib()
    assert L.gb_sync(None) == gbblas.OK
    assert L.gb_selftest_bounded_wait(1000000, None) == gbblas.OK
    assert L.gb_sync(None) == gbblas.ERR_DEVICE_TIMEOUT
    assert b"code 99" in L.gb_last_error()
    assert L.gb_sync(None) == gbblas.OK          # reported once, then cleared
    # the tensor-core kernels run normally afterwards: small integers, exact
    rng = np.random.default_rng(5)
    M, N, K = 512, 384, 256
    A = rng.integers(-8, 9, size=(M, K)).astype(np.float32)
    B = rng.integers(-8, 9, size=(K, N)).astype(np.float32)
    for algo in (gbblas.ALGO_BF16X3, gbblas.ALGO_BF16X6, gbblas.ALGO_FP16X3):
        dC = dev(np.zeros((M, N), np.float32))
        gbblas.sgemm("N", "N", M, N, K, 1.0, dev(A), K, dev(B), N, 0.0, dC, N, algo=algo)
        assert L.gb_sync(None) == gbblas.OK
        assert np.array_equal(host(dC), (A.astype(np.float64) @ B.astype(np.float64)).astype(np.float32))


def test_bounded_wait_selftest_checks_its_limit(torch):
    import gbblas
    L = gbblas.lib()
    assert L.gb_selftest_bounded_wait(10, None) == gbblas.ERR_INVALID_ARG
    assert L.gb_selftest_bounded_wait(10 ** 9, None) == gbblas.ERR_INVALID_ARG
    assert L.gb_sync(None) == gbblas.OK
