"""Serving loop bookkeeping on the host (dry-run server: admission, budget,
validation, completion and statistics run; no device work), the autotune
table, and grouped-batch argument checks -- no GPU needed."""
import ctypes
import os

import pytest

import gbblas


@pytest.fixture(scope="module")
def L():
    if not os.path.exists(gbblas.LIB_PATH):
        import __graft_entry__
        __graft_entry__.build()
    return gbblas.lib()


def gemm_req(M, N, K, bits=32, tag=0, nbytes=0):
    # dummy non-null pointers: dry-run never touches them
    return gbblas.request(gbblas.OP_GEMM, bits, M, N, K, A=16, lda=K, B=32, ldb=N, C=48, ldc=N, tag=tag,
                          nbytes=nbytes)


def test_dry_run_server_completes_everything(L):
    with gbblas.Server(dry_run=1, hbm_budget_bytes=1 << 30) as s:
        for i in range(100):
            s.submit(gemm_req(64 + i, 64, 64, tag=i))
        s.drain(10.0)
        st = s.stats()
        assert st["submitted"] == 100 and st["completed"] == 100 and st["inflight"] == 0
        assert st["inflight_bytes"] == 0
        tags = sorted(t for t, _ in s.poll())
        assert tags == list(range(100))
        assert st["p99_s"] >= st["p50_s"] >= 0.0


def test_requests_over_budget_are_rejected(L):
    with gbblas.Server(dry_run=1, hbm_budget_bytes=1 << 20) as s:
        with pytest.raises(gbblas.GBError) as e:
            s.submit(gemm_req(1024, 1024, 1024))          # 12 MB of operands > 1 MB
        assert e.value.status == gbblas.ERR_OOM
        s.submit(gemm_req(64, 64, 64, nbytes=1 << 19))     # explicit charge, fits
        s.drain(10.0)
        st = s.stats()
        assert st["rejected"] == 1 and st["completed"] == 1


@pytest.mark.parametrize("bad", [
    dict(op=7), dict(bits=16), dict(M=-1), dict(lda=1), dict(C=None),
])
def test_malformed_requests_are_rejected(L, bad):
    r = gbblas.request(bad.get("op", gbblas.OP_GEMM), bad.get("bits", 32), bad.get("M", 8), 8, 8, A=16,
                       lda=bad.get("lda", 8), B=32, ldb=8, C=bad.get("C", 48), ldc=8)
    with gbblas.Server(dry_run=1) as s:
        with pytest.raises(gbblas.GBError) as e:
            s.submit(r)
        assert e.value.status == gbblas.ERR_INVALID_ARG
        assert s.stats()["rejected"] == 1


def test_server_config_validation(L):
    for field, val in (("streams", 0), ("max_batch", 0), ("hbm_budget_bytes", 0), ("max_inflight", 0),
                       ("short_streams", 0), ("long_sm_percent", 0), ("long_sm_percent", 101)):
        c = gbblas.ServerConfig()
        L.gb_server_config_init(ctypes.byref(c))
        c.dry_run = 1
        setattr(c, field, val)
        h = ctypes.c_void_p()
        assert L.gb_server_create(ctypes.byref(c), ctypes.byref(h)) == gbblas.ERR_INVALID_ARG


def test_drain_times_out_while_requests_wait(L):
    # max_inflight = 1 and a request that never completes cannot happen in
    # dry-run; instead a drain with nothing submitted returns at once
    with gbblas.Server(dry_run=1) as s:
        s.drain(0.5)
        assert s.stats()["completed"] == 0


def test_autotune_table_roundtrip(L, tmp_path):
    assert L.gb_autotune_set(32, b"N", b"T", 1000, 2000, 3000, gbblas.ALGO_BF16X3) == gbblas.OK
    assert L.gb_autotune_get(32, b"N", b"T", 1024, 2048, 2900) == gbblas.ALGO_BF16X3   # same log2 bucket
    assert L.gb_autotune_get(32, b"N", b"N", 1024, 2048, 2900) == -1
    path = str(tmp_path / "tune.txt").encode()
    assert L.gb_autotune_save(path) == gbblas.OK
    assert L.gb_autotune_set(32, b"N", b"T", 1000, 2000, 3000, gbblas.ALGO_SIMT) == gbblas.OK
    assert L.gb_autotune_load(path) == gbblas.OK
    assert L.gb_autotune_get(32, b"N", b"T", 1000, 2000, 3000) == gbblas.ALGO_BF16X3
    assert L.gb_autotune_set(32, b"N", b"T", 1, 1, 1, 99) == gbblas.ERR_INVALID_ARG


def test_autotune_choice_file_keeps_knobs(L, tmp_path):
    """A saved choice carries its knobs (accumulator chunk, split-K, slices);
    a file with only the seven legacy columns still loads."""
    path = tmp_path / "tune.txt"
    path.write_text("# bits ta tb log2M log2N log2K algo accum_k split_k slices ms\n"
                    "32 0 1 12 12 12 8 256 0 0 0.41\n"
                    "64 0 0 10 10 12 5 0 0 7 1.5\n"
                    "32 1 0 4 18 12 6 0 16 0 0.2\n"
                    "64 1 1 11 11 11 3\n")
    assert L.gb_autotune_load(str(path).encode()) == gbblas.OK
    c = gbblas.autotune_lookup(32, "N", "T", 4096, 4096, 4096)
    assert c["algo"] == gbblas.ALGO_FP16X3 and c["accum_k"] == 256 and abs(c["ms"] - 0.41) < 1e-9
    c = gbblas.autotune_lookup(64, "N", "N", 1024, 1024, 4096)
    assert c["algo"] == gbblas.ALGO_OZAKI and c["ozaki_slices"] == 7
    c = gbblas.autotune_lookup(32, "T", "N", 16, 262144, 4096)
    assert c["algo"] == gbblas.ALGO_SKINNY and c["split_k"] == 16
    assert gbblas.autotune_lookup(64, "T", "T", 2048, 2048, 2048)["algo"] == gbblas.ALGO_DMMA
    assert gbblas.autotune_lookup(64, "T", "T", 7, 7, 7) is None
    out = tmp_path / "again.txt"
    assert L.gb_autotune_save(str(out).encode()) == gbblas.OK
    assert "32 1 0 4 18 12 6 0 16 0" in out.read_text()


def test_gemm_rejects_bad_split_k(L):
    o = gbblas.opts(algo=gbblas.ALGO_SKINNY, split_k=65)
    st = L.gb_sgemm(b"N", b"N", 100, 8, 100, 1.0, 16, 100, 32, 8, 0.0, 48, 8, ctypes.byref(o))
    assert st == gbblas.ERR_INVALID_ARG


def test_gemm_batch_rejects_bad_descriptors(L):
    d = gbblas.gemm_desc("N", "N", 8, 8, 8, 1.0, 16, 4, 32, 8, 0.0, 48, 8, 32)   # lda < K
    arr = (gbblas.GemmDesc * 1)(d)
    assert L.gb_gemm_batch(arr, 1, None) == gbblas.ERR_INVALID_ARG
    d = gbblas.gemm_desc("N", "N", 8, 8, 8, 1.0, 16, 8, 32, 8, 0.0, 48, 8, 16)   # dtype 16
    arr = (gbblas.GemmDesc * 1)(d)
    assert L.gb_gemm_batch(arr, 1, None) == gbblas.ERR_INVALID_ARG
    assert L.gb_gemm_batch(None, 0, None) == gbblas.OK


@pytest.mark.parametrize("streams,short_streams,short_us,urgent", [(6, 2, 200.0, 10), (6, 2, 0.0, 0), (1, 2, 200.0, 0)])
def test_short_requests_go_to_the_urgent_streams(L, streams, short_streams, short_us, urgent):
    """Requests estimated below short_us (small transposes) are routed to the high-priority
    streams and long ones (a 2048^3 FP64 product) to the others; with priorities off (short_us 0)
    or a single stream nothing is urgent."""
    with gbblas.Server(dry_run=1, streams=streams, short_streams=short_streams, short_us=short_us,
                       use_grouped=0) as s:
        for i in range(10):
            s.submit(gbblas.request(gbblas.OP_TRANSPOSE, 32, 256, 256, A=16, lda=256, B=32, ldb=256, tag=i))
        for i in range(7):
            s.submit(gbblas.request(gbblas.OP_GEMM, 64, 2048, 2048, 2048, A=16, lda=2048, B=32, ldb=2048, C=48,
                                    ldc=2048, algo=gbblas.ALGO_OZAKI, tag=100 + i))
        s.drain(10.0)
        st = s.stats()
        assert st["completed"] == 17 and st["launches"] == 17
        assert st["urgent_launches"] == urgent
