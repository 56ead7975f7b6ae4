"""bench.py's replica logic on CPU: two ranks over gloo (127.0.0.1).

The path has no exchange step (one process per GPU runs its own replica), so
what has to hold across ranks is the measurement: every rank passes the
barriers, the reported time is the slowest rank's, the throughput counts the
units of all ranks, and rank 0 alone prints the JSON line; the reference arm
runs on rank 0 only and the other ranks exit 0 without output."""
import json
import os
import socket
import subprocess
import sys

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out_dir):
    os.environ.update({"RANK": str(rank), "WORLD_SIZE": str(world), "LOCAL_RANK": str(rank),
                       "MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port)})
    sys.path.insert(0, REPO)
    import bench
    r = bench.Ranks("gloo", "cpu")
    r.barrier()
    ms = 10.0 * (rank + 1)                    # the ranks' own elapsed times differ
    slowest = r.max(ms)
    value = bench.aggregate(r.world, 3, 1e9, slowest)   # 3 steps of 1e9 units per rank
    with open(os.path.join(out_dir, "rank%d.out" % rank), "w") as f:
        r.finish({"value": value, "ms": slowest, "n_gpus": r.world}, out=f)
    with open(os.path.join(out_dir, "rank%d.max" % rank), "w") as f:
        f.write(repr(slowest))


def test_two_ranks_gloo(tmp_path):
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp
    port = _free_port()
    ctx = mp.get_context("spawn")
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, str(tmp_path))) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    # both ranks agree on the slowest time
    assert float((tmp_path / "rank0.max").read_text()) == 20.0
    assert float((tmp_path / "rank1.max").read_text()) == 20.0
    # rank 0 alone prints; throughput = units of both ranks / the slowest time
    line = json.loads((tmp_path / "rank0.out").read_text())
    assert (tmp_path / "rank1.out").read_text() == ""
    assert line["n_gpus"] == 2 and line["ms"] == 20.0
    assert line["value"] == pytest.approx(2 * 3 * 1e9 / 20e-3)


def test_aggregate_single_rank():
    sys.path.insert(0, REPO)
    import bench
    assert bench.aggregate(1, 4, 2.5e12, 1000.0) == pytest.approx(1e13)


def test_reference_arm_other_ranks_exit_quietly():
    env = dict(os.environ, RANK="1", WORLD_SIZE="2", LOCAL_RANK="1")
    r = subprocess.run([sys.executable, os.path.join(REPO, "bench.py"), "--impl", "reference", "--steps", "1",
                        "--warmup", "3"], env=env, capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stderr
    assert r.stdout.strip() == ""


def test_parse_cpulist():
    sys.path.insert(0, REPO)
    import bench
    assert bench.parse_cpulist("0-3,8,10-11\n") == {0, 1, 2, 3, 8, 10, 11}
    assert bench.parse_cpulist("5") == {5}
    assert bench.parse_cpulist("") == set()


def test_near_gpu_leaves_affinity_alone_when_local_cores_unknown():
    sys.path.insert(0, REPO)
    import bench

    class NoProps:   # a torch whose device properties carry no PCI ids
        class cuda:
            @staticmethod
            def get_device_properties(dev):
                raise AttributeError("no PCI ids")

    before = os.sched_getaffinity(0)
    with bench.near_gpu(NoProps, 0) as placed:
        assert os.sched_getaffinity(0) == before
    assert os.sched_getaffinity(0) == before
    assert "unknown" in placed.note


def test_e2e_measure_reports_the_median_run():
    """e2e_measure: one untimed step, then `runs` timed runs of `steps` steps each; the rate of
    the median run (a fake context whose events read a simulated clock)."""
    sys.path.insert(0, REPO)
    import bench

    clock = [0.0]

    class Ev:
        def record(self, stream):
            self.t = clock[0]

        def elapsed_time(self, other):
            return other.t - self.t

    class FakeTorch:
        class cuda:
            @staticmethod
            def synchronize():
                pass

    class FakeCtx:
        torch, stream, world = FakeTorch, None, 1

        def event(self):
            return Ev()

        def barrier(self):
            pass

        def max_over_ranks(self, ms):
            return ms

    # ms per step: the untimed one, then three runs of two steps (20, 60 and 40 ms per run)
    per_step = iter([1.0, 10.0, 10.0, 30.0, 30.0, 20.0, 20.0])

    def step_host():
        clock[0] += next(per_step)
        return 100, 200

    rate, h2d, d2h = bench.e2e_measure(FakeCtx(), step_host, 2, 1e9, 1e9)
    assert rate == pytest.approx(2 * 1e9 / 40e-3 / 1e9)   # the 40 ms run
    assert (h2d, d2h) == (100, 200)
    assert bench.E2E_RUNS == 3 and "median" in bench.E2E_TIMING
