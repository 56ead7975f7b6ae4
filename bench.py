"""Benchmarks of the GB300 BLAS hot path.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]
                    [--workload sgemm|dgemm|thinb|shorta|transpose|jacobi] [options]

With no flags it runs the headline workload (the default line):

sgemm   SGEMM C = alpha*op(A)op(B) + beta*C, FP32, row-major, M = N = K = 4096,
        leading dimensions 4112, alpha 1.5, beta -0.5, all four transpose modes,
        entries U[-1,1] from seed 1 (generated on the device by gb_fill_f32).
        One step = the four GEMMs with the headline form: the fastest emulated
        form (BF16X3, BF16X6, FP16X3 on tcgen05) whose normwise error against
        the Dot2 oracle is no worse than plain FFMA's on the same subgrid
        (matched error); every form's rate and error are reported beside it.

Other workloads (one JSON line each, same contract):
dgemm     M = N = K = 8192 FP64, NN and TT, alpha = beta = 1, entries u*2^e
          (u ~ U[-1,1], e ~ U{-20..20}, seed 3): Ozaki slices vs native FP64,
          TFLOP/s and normwise error on a seeded 1024 x 1024 subgrid.
thinb     M = 262144, K = 4096, N in {8,16,32,64} (--n), FP32 or FP64 (--bits),
          all four modes, U[-1,1] seed 2: HBM GB/s, bytes = s(MK + KN + 2MN).
shorta    the mirror: M in {8..64}, K = 4096, N = 262144.
transpose 30000 x 17000, FP32 or FP64: HBM GB/s, bytes = 2*M*N*s.
jacobi    8192 x 8192 interior, boundary 1.0, interior U[0,1] seed 2, 200 sweeps,
          FP32 or FP64: algorithmic GB/s = 2*M*N*s per sweep.

value is the whole-job figure over all ranks (replicas: each rank runs the same
workload, no collective on the data path; "scaling": "weak"), timed with CUDA
events on the launching stream between a barrier + synchronize on both sides,
max over ranks.  e2e repeats the metric through the C ABI with host (pinned)
buffers, host<->device copies inside the timed region.  Inputs of every
workload exceed the 129 MB L2.  cpu_baseline times the oracle's port of the
reference host loop on a bounded sample with every host core.
"""
import argparse
import ctypes
import json
import math
import os
import statistics
import subprocess
import sys
import threading
import time

REPO = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.join(REPO, "blas-for-multi-core-dsp_gb300")
for _p in (REPO, PKG):
    if _p not in sys.path:
        sys.path.insert(0, _p)

METRIC = "TFLOP/s (emulated vs plain FP64/FP32) at matched error; serve p50/p99, req/s"
MODES = ("NN", "NT", "TN", "TT")


def log(*a):
    print(*a, file=sys.stderr, flush=True)


def measured_peaks():
    try:
        with open(os.path.join(REPO, "MEASURED_PEAKS.json")) as f:
            return json.load(f), "measured"
    except (OSError, ValueError):
        return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "bf16_tflops_sustained": 1700.0}, "fallback"


def _gpu_local_cpus(torch, dev):
    """The host cores attached to GPU `dev` (the sysfs local_cpulist of its PCI function) that
    this process may run on; empty when that is unknown."""
    try:
        p = torch.cuda.get_device_properties(dev)
        path = "/sys/bus/pci/devices/%04x:%02x:%02x.0/local_cpulist" % (p.pci_domain_id, p.pci_bus_id,
                                                                          p.pci_device_id)
        with open(path) as f:
            return parse_cpulist(f.read()) & os.sched_getaffinity(0)
    except (AttributeError, OSError, ValueError):
        return set()


def parse_cpulist(spec):
    """A sysfs CPU list ("0-3,8,10-11") as a set of core numbers."""
    cpus = set()
    for part in spec.strip().split(","):
        if "-" in part:
            a, b = part.split("-")
            cpus.update(range(int(a), int(b) + 1))
        elif part:
            cpus.add(int(part))
    return cpus


class near_gpu:
    """Context: the enclosed host allocations run on the GPU's local cores, so that pinned
    buffers are first touched, and placed, on the memory node next to the GPU (a far node puts
    every host<->device copy across the socket link).  The process's own core set comes back
    on exit; where the local cores are unknown or not ours, nothing changes."""

    def __init__(self, torch, dev):
        self.torch, self.dev, self.saved, self.note = torch, dev, None, "pinned"

    def __enter__(self):
        local = _gpu_local_cpus(self.torch, self.dev)
        allowed = os.sched_getaffinity(0)
        if not local:
            self.note = "pinned (the GPU's local cores unknown or outside this process's set)"
        elif local == allowed:
            self.note = "pinned, allocated on the GPU-local cores (all %d of this process's)" % len(local)
        else:
            try:
                os.sched_setaffinity(0, local)
                self.saved = allowed
                self.note = "pinned, allocated on the %d GPU-local cores of this process's %d" % (len(local),
                                                                                                  len(allowed))
            except OSError:
                self.note = "pinned (could not bind to the GPU's local cores)"
        return self

    def __exit__(self, *exc):
        if self.saved is not None:
            os.sched_setaffinity(0, self.saved)
        return False


def profile_traffic(name):
    """DRAM bytes per launch from profiles/<name>.txt ('traffic_bytes_per_launch: N'), else None."""
    try:
        for line in open(os.path.join(REPO, "profiles", name + ".txt")):
            if line.startswith("traffic_bytes_per_launch:"):
                return int(float(line.split(":", 1)[1].strip()))
    except OSError:
        pass
    return None




class Cublas:
    """cuBLAS through ctypes, for yardsticks printed beside the library's own
    numbers (context only: never the measured product).  Row-major GEMMs are
    issued as the column-major C^T = op(B)^T op(A)^T."""
    R32, R64 = 0, 1                                   # cudaDataType
    COMPUTE = {"32F": 68, "32F_EMULATED_16BFX9": 78, "64F": 70, "64F_EMULATED_FIXEDPOINT": 79}
    EAGER = 2                                         # cublasEmulationStrategy_t

    def __init__(self, stream):
        import glob
        paths = sorted(glob.glob("/usr/local/cuda/lib64/libcublas.so*"))
        if not paths:
            raise OSError("no libcublas.so")
        self.L = ctypes.CDLL(paths[0])
        self.h = ctypes.c_void_p()
        if self.L.cublasCreate_v2(ctypes.byref(self.h)) != 0:
            raise OSError("cublasCreate failed")
        self.L.cublasSetStream_v2(self.h, ctypes.c_void_p(stream))
        f = self.L.cublasGemmEx
        f.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                      ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_void_p, ctypes.c_int,
                      ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                      ctypes.c_int]

    def gemm(self, ta, tb, M, N, K, alpha, A, lda, B, ldb, beta, C, ldc, bits, compute):
        emulated = "EMULATED" in compute
        if hasattr(self.L, "cublasSetEmulationStrategy"):
            self.L.cublasSetEmulationStrategy(self.h, self.EAGER if emulated else 0)
        ct = ctypes.c_double if bits == 64 else ctypes.c_float
        al, be = ct(alpha), ct(beta)
        dt = self.R64 if bits == 64 else self.R32
        rc = self.L.cublasGemmEx(self.h, 1 if tb == "T" else 0, 1 if ta == "T" else 0, N, M, K,
                                 ctypes.addressof(al), B.data_ptr(), dt, ldb, A.data_ptr(), dt, lda,
                                 ctypes.addressof(be), C.data_ptr(), dt, ldc, self.COMPUTE[compute], -1)
        if rc != 0:
            raise RuntimeError("cublasGemmEx(%s) status %d" % (compute, rc))


class ClockSampler:
    """nvidia-smi samples of SM clock and throttle reasons during a timed region."""
    Q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index, self.proc, self.lines = index, None, []

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.Q,
                                          "--format=csv,noheader,nounits", "-lms", "100"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            threading.Thread(target=self._read, daemon=True).start()
        except OSError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for l in self.lines:
            f = [x.strip() for x in l.split(",")]
            if len(f) < 7:
                continue
            try:
                sm.append(float(f[0]))
                mx.append(float(f[1]))
            except ValueError:
                continue
            for n, v in zip(names, f[3:7]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


# ================================================================== ranks
class Ranks:
    """One process per GPU (replicas): rank / world from the launcher's
    environment, a barrier, the maximum of a per-rank time, and rank 0 alone
    printing the result line.  `backend` nccl with a CUDA device on the GPU
    box; gloo with the CPU in the CPU tests."""

    def __init__(self, backend="nccl", device=None):
        import torch
        self.torch = torch
        self.rank = int(os.environ.get("RANK", "0"))
        self.world = int(os.environ.get("WORLD_SIZE", "1"))
        self.local = int(os.environ.get("LOCAL_RANK", "0"))
        self.device = device
        self.dist = None
        if self.world > 1:
            import torch.distributed as dist
            dist.init_process_group(backend)
            self.dist = dist

    def barrier(self):
        if self.dist:
            self.dist.barrier()

    def max(self, v):
        if not self.dist:
            return v
        t = self.torch.tensor([float(v)], dtype=self.torch.float64, device=self.device)
        self.dist.all_reduce(t, op=self.dist.ReduceOp.MAX)
        return float(t.item())

    def finish(self, line, out=None):
        if self.dist:
            self.dist.barrier()
            self.dist.destroy_process_group()
        if self.rank == 0:
            print(json.dumps(line), file=out or sys.stdout, flush=True)


def aggregate(world, steps, units_per_step, ms):
    """Whole-job throughput: the units all ranks processed / the slowest rank's time (s)."""
    return world * steps * units_per_step / (ms * 1e-3)


# ================================================================== context
class Ctx:
    def __init__(self, args):
        import torch
        import gbblas
        self.args = args
        self.torch, self.gb = torch, gbblas
        self.local = int(os.environ.get("LOCAL_RANK", "0"))
        torch.cuda.set_device(self.local)
        self.ranks = Ranks("nccl", torch.device("cuda", self.local))
        self.rank, self.world, self.dist = self.ranks.rank, self.ranks.world, self.ranks.dist
        gbblas.lib()
        arch = gbblas.arch()
        if arch != 103:
            raise SystemExit("bench.py: needs an sm_103 GPU (found sm_%d)" % arch)
        self.dev = torch.device("cuda", self.local)
        self.stream = torch.cuda.current_stream(self.dev)
        self.peaks, self.peak_src = measured_peaks()
        # scalar FMA rooflines, measured on this GPU (FFMA and DFMA chains on every SM)
        self.fma_peak = {32: gbblas.fma_peak(32, self.stream.cuda_stream),
                         64: gbblas.fma_peak(64, self.stream.cuda_stream)}

    def event(self):
        return self.torch.cuda.Event(enable_timing=True)

    def barrier(self):
        self.ranks.barrier()
        self.torch.cuda.synchronize()

    def max_over_ranks(self, ms):
        return self.ranks.max(ms)

    def timed(self, step, steps, per_launch=None):
        """Run `steps` steps between barriers; returns (elapsed ms max over ranks,
        mean ms of the launches recorded by per_launch, clocks, launch count)."""
        sampler = ClockSampler(self.local)
        self.barrier()
        sampler.start()
        time.sleep(0.25)
        l0 = self.gb.launch_count()
        t0, t1 = self.event(), self.event()
        evs = []
        t0.record(self.stream)
        for _ in range(steps):
            step(evs)
        t1.record(self.stream)
        self.torch.cuda.synchronize()
        launches = self.gb.launch_count() - l0
        clocks = sampler.stop()
        ms = self.max_over_ranks(t0.elapsed_time(t1))
        kms = statistics.mean(a.elapsed_time(b) for a, b in evs) if evs else None
        self.last_evs = evs
        return ms, kms, clocks, int(launches)

    def per_mode_ms(self, modes):
        """Mean launch time per mode when each step records one event pair per mode."""
        evs = getattr(self, "last_evs", [])
        return {m: statistics.mean(a.elapsed_time(b) for a, b in evs[i::len(modes)])
                for i, m in enumerate(modes)} if evs else {}

    def finish(self, line):
        self.ranks.finish(line)


def base_line(ctx, metric, value, unit, ms, steps, dtype, config, hib=True):
    return {"metric": metric, "value": value, "unit": unit, "n_gpus": ctx.world, "steps": steps,
            "warmup": ctx.args.warmup, "ms_per_step": ms / steps, "higher_is_better": hib, "scaling": "weak",
            "vs_baseline": None, "dtype": dtype, "data": "synthetic", "config": config,
            "fma_peak_tflops": {"ffma": ctx.fma_peak[32], "dfma": ctx.fma_peak[64],
                                "note": "scalar FMA throughput measured on this GPU (gb_measure_fma_peak)"}}


def memcpy(ctx, dst, src, nbytes, kind, stream=None):
    st = ctx.gb.lib().gb_memcpy(ctypes.c_void_p(dst.data_ptr()), ctypes.c_void_p(src.data_ptr()), nbytes, kind,
                                ctypes.c_void_p((stream or ctx.stream).cuda_stream))
    assert st == 0, ctx.gb.lib().gb_last_error()


E2E_RUNS = 3
E2E_TIMING = "median of %d timed runs of the steps (slowest rank each), after one untimed step" % E2E_RUNS


def e2e_measure(ctx, step_host, steps, flops_or_bytes, unit_div, runs=E2E_RUNS):
    """Time step_host() (copies + compute through the C ABI) `steps` times, `runs` times over;
    the median run's rate (one run of a few steps is short enough for a burst of other traffic
    on the host side to decide it)."""
    step_host()
    ctx.torch.cuda.synchronize()
    ctx.barrier()
    rates = []
    for _ in range(runs):
        t0, t1 = ctx.event(), ctx.event()
        t0.record(ctx.stream)
        for _ in range(steps):
            h2d, d2h = step_host()
        t1.record(ctx.stream)
        ctx.torch.cuda.synchronize()
        ms = ctx.max_over_ranks(t0.elapsed_time(t1))
        rates.append(aggregate(ctx.world, steps, flops_or_bytes, ms) / unit_div)
    return statistics.median(rates), h2d, d2h


# ================================================================== CPU legs
def cpu_sgemm_sample(max_seconds=10.0):
    import numpy as np
    import oracle
    M = N = K = 4096
    LD = 4112
    nt = os.cpu_count() or 1
    oracle.set_threads(nt)
    A = oracle.fill(M, K, 11, dtype=np.float32, ld=LD)
    B = oracle.fill(K, N, 12, dtype=np.float32, ld=LD)
    rows = 8
    while True:
        flops = secs = 0.0
        for mode in MODES:
            Cs = np.zeros((rows, LD), dtype=np.float32)
            t0 = time.perf_counter()
            oracle.sgemm_ref(mode[0], mode[1], rows, N, K, 1.5, A, LD, B, LD, -0.5, Cs, LD)
            secs += time.perf_counter() - t0
            flops += 2.0 * rows * N * K
        if secs * 3 > max_seconds or rows >= 256:
            break
        rows *= 2
    return (flops / secs / 1e12, nt, "sampled rate (not the full problem): %d of %d rows of C per mode, 4 modes, "
            "K=%d: oracle port of the reference host loop sgemm_demo.c:214-242, gcc -O2 -fopenmp, %d threads"
            % (rows, M, K, nt))


def cpu_dgemm_sample(max_seconds=10.0):
    import numpy as np
    import oracle
    n = 8192
    nt = os.cpu_count() or 1
    oracle.set_threads(nt)
    A = oracle.fill(64, n, 31, kind=2)
    B = oracle.fill(n, n, 32, kind=2)
    rows = 4
    while True:
        C = np.zeros((rows, n))
        t0 = time.perf_counter()
        oracle.dgemm_ref("N", "N", rows, n, n, A, n, B, n, C, n)
        secs = time.perf_counter() - t0
        if secs * 3 > max_seconds or rows >= 64:
            break
        rows *= 2
    return (2.0 * rows * n * n / secs / 1e12, nt, "sampled rate (not the full problem): %d of 8192 rows of C, NN, "
            "K=8192: oracle port of dgemm_demo.c:233-252, %d threads (rate extrapolated to the full problem)"
            % (rows, nt))


def cpu_bw_sample(kind, bits, max_seconds=8.0):
    """Reference host loops for the bandwidth workloads on a bounded sample; returns GB/s."""
    import numpy as np
    import oracle
    nt = os.cpu_count() or 1
    oracle.set_threads(nt)
    dt = np.float64 if bits == 64 else np.float32
    s = 8 if bits == 64 else 4
    if kind == "transpose":
        M, N = 30000, 4000
        A = oracle.fill(M, N, 2, dtype=dt)
        B = np.zeros((N, M), dtype=dt)
        t0 = time.perf_counter()
        oracle.transpose_into(M, N, A, N, B, M)
        secs = time.perf_counter() - t0
        return 2.0 * M * N * s / secs / 1e9, nt, "30000 x 4000 slice, transpose.c:113-119 loop, %d threads" % nt
    if kind == "jacobi":
        M = N = 8192
        A = np.ones((M + 2, N + 2), dtype=dt)
        A[1:-1, 1:-1] = oracle.fill(M, N, 2, kind=1, dtype=dt)
        B = A.copy()
        t0 = time.perf_counter()
        oracle.stencil(M, N, A, B, 2, 0)
        secs = time.perf_counter() - t0
        return 2 * 2.0 * M * N * s / secs / 1e9, nt, "2 sweeps of 8192^2, matrix_stencil.c:35-48 loop, %d threads" % nt
    # skinny: thinB rows sample
    n, K = 8, 4096
    rows = 2048
    A = oracle.fill(rows, K, 2, dtype=dt)
    B = oracle.fill(K, n, 3, dtype=dt)
    C = np.zeros((rows, n), dtype=dt)
    t0 = time.perf_counter()
    if bits == 64:
        oracle.dgemm_ref("N", "N", rows, n, K, A, K, B, n, C, n)
    else:
        oracle.sgemm_irr_ref("N", "N", rows, n, K, A, K, B, n, C, n)
    secs = time.perf_counter() - t0
    return (s * (rows * K + K * n + 2 * rows * n) / secs / 1e9, nt,
            "%d rows of thinB N=8 K=4096, irr demo loop, %d threads" % (rows, nt))


# ================================================================== workloads
def run_sgemm(ctx):
    torch, gb, args = ctx.torch, ctx.gb, ctx.args
    import numpy as np
    M = N = K = 4096
    LD = 4112
    ALPHA, BETA = 1.5, -0.5
    flops = 2.0 * M * N * K
    bufs = {}
    for name, seed in {"A_N": 11, "A_T": 12, "B_N": 13, "B_T": 14, "C": 15}.items():
        t = torch.empty((M, LD), dtype=torch.float32, device=ctx.dev)
        gb.fill(t, M, K, LD, seed, 0, 32, stream=ctx.stream)
        bufs[name] = t
    C0 = bufs["C"].clone()

    def ops(mode):
        return bufs["A_T" if mode[0] == "T" else "A_N"], bufs["B_T" if mode[1] == "T" else "B_N"]

    def gemm(mode, algo, C=None):
        A, B = ops(mode)
        gb.sgemm(mode[0], mode[1], M, N, K, ALPHA, A, LD, B, LD, BETA, bufs["C"] if C is None else C, LD,
                 algo=algo, stream=ctx.stream)

    ids = {"bf16x3": gb.ALGO_BF16X3, "bf16x6": gb.ALGO_BF16X6, "fp16x3": gb.ALGO_FP16X3, "simt": gb.ALGO_SIMT}
    products = {"bf16x3": 3, "bf16x6": 6, "fp16x3": 3}

    # normwise error of every form against Dot2 on a seeded subgrid (worst of the four modes)
    errors = {}
    try:
        import oracle
        rng = np.random.default_rng(1)
        rows = np.sort(rng.choice(M, 128, replace=False))
        cols = np.sort(rng.choice(N, 128, replace=False))
        hb = {k: v.cpu().numpy() for k, v in bufs.items() if k != "C"}
        c0 = C0.cpu().numpy()
        for an in ("simt", "bf16x3", "bf16x6", "fp16x3"):
            worst = 0.0
            for mode in MODES:
                Cw = C0.clone()
                gemm(mode, ids[an], Cw)
                A = hb["A_T" if mode[0] == "T" else "A_N"]
                B = hb["B_T" if mode[1] == "T" else "B_N"]
                e, _ = oracle.normwise_error(Cw.cpu().numpy(), mode[0], mode[1], M, N, K, ALPHA, A, LD, B, LD, BETA,
                                             c0, LD, rows, cols)
                worst = max(worst, e)
            errors[an] = worst
        errors["bound_2Ku"] = 2 * K * 2.0 ** -24
        errors["subgrid"] = "seeded 128 x 128 rows/cols, Dot2 oracle, worst of 4 modes"
    except Exception as e:
        errors["error"] = repr(e)

    # every form timed on the same inputs: warm-up, then four rounds of the four modes back to back
    def rate(aid):
        for _ in range(2):
            for mode in MODES:
                gemm(mode, aid)
        s0, s1 = ctx.event(), ctx.event()
        s0.record(ctx.stream)
        for _ in range(4):
            for mode in MODES:
                gemm(mode, aid)
        s1.record(ctx.stream)
        torch.cuda.synchronize()
        return 4 * len(MODES) * flops / (s0.elapsed_time(s1) * 1e-3) / 1e12

    compare = {an + "_tflops": rate(ids[an]) for an in ("simt", "bf16x3", "bf16x6", "fp16x3")}
    # cuBLAS on the same inputs (yardsticks, not the product): native FP32 and its emulated
    # BF16x9 form, rate and error on the same subgrid
    try:
        cb = Cublas(ctx.stream.cuda_stream)
        for name, compute in (("cublas_sgemm", "32F"), ("cublas_bf16x9", "32F_EMULATED_16BFX9")):
            def cgemm(mode, Cx, compute=compute):
                A, B = ops(mode)
                cb.gemm(mode[0], mode[1], M, N, K, ALPHA, A, LD, B, LD, BETA, Cx, LD, 32, compute)
            if "simt" in errors:
                worst = 0.0
                for mode in MODES:
                    Cw = C0.clone()
                    cgemm(mode, Cw)
                    A = hb["A_T" if mode[0] == "T" else "A_N"]
                    B = hb["B_T" if mode[1] == "T" else "B_N"]
                    e, _ = oracle.normwise_error(Cw.cpu().numpy(), mode[0], mode[1], M, N, K, ALPHA, A, LD, B, LD,
                                                 BETA, c0, LD, rows, cols)
                    worst = max(worst, e)
                errors[name] = worst
            Cw = C0.clone()
            for mode in MODES:
                cgemm(mode, Cw)
            s0, s1 = ctx.event(), ctx.event()
            s0.record(ctx.stream)
            for _ in range(4):
                for mode in MODES:
                    cgemm(mode, Cw)
            s1.record(ctx.stream)
            torch.cuda.synchronize()
            compare[name + "_tflops"] = 4 * len(MODES) * flops / (s0.elapsed_time(s1) * 1e-3) / 1e12
        compare["cublas_note"] = ("cuBLAS yardsticks on the same inputs: CUBLAS_COMPUTE_32F and "
                                  "CUBLAS_COMPUTE_32F_EMULATED_16BFX9 (emulation strategy eager)")
    except Exception as e:
        compare["cublas_error"] = repr(e)
    # the headline form: the fastest emulated form whose measured error is no worse than plain
    # FFMA's on the same subgrid (matched error); --algo names one instead
    if args.algo != "best":
        algo_name = args.algo
    elif "simt" in errors:
        ok = [an for an in products if errors.get(an, 1.0) <= errors["simt"]]
        algo_name = max(ok, key=lambda an: compare[an + "_tflops"]) if ok else "simt"
    else:
        algo_name = "simt"
    algo = ids[algo_name]
    compare["matched_error_rule"] = ("headline form = fastest emulated form with normwise error <= plain FFMA's "
                                     "on the same subgrid")
    compare["notes"] = {"bf16x3": "hi/lo BF16 pieces, 3 products, one accumulator over K",
                        "bf16x6": "hi/mid/lo BF16 pieces, 6 products, folded accumulation (256 k)",
                        "fp16x3": "hi/lo FP16 pieces of power-of-two scaled rows/columns, 3 products, "
                                  "folded accumulation (128 k)",
                        "simt": "plain FP32 FFMA register tiles"}

    for _ in range(args.warmup):
        for mode in MODES:
            gemm(mode, algo)
    torch.cuda.synchronize()

    # the timed steps issue the calls back to back (nothing between them on the stream, so a
    # call's split pass may run beside the previous call's GEMM); the duration of one call is
    # measured afterwards with events around each call
    def step(evs):
        for mode in MODES:
            gemm(mode, algo)

    ms, _, clocks, launches = ctx.timed(step, args.steps)
    value = aggregate(ctx.world, args.steps, len(MODES) * flops, ms) / 1e12

    def step_events(evs):
        for mode in MODES:
            a, b = ctx.event(), ctx.event()
            a.record(ctx.stream)
            gemm(mode, algo)
            b.record(ctx.stream)
            evs.append((a, b))

    _, kms, _, _ = ctx.timed(step_events, args.steps)
    by_mode = ctx.per_mode_ms(MODES)
    compare["speedup_vs_simt"] = value / ctx.world / compare["simt_tflops"]

    with near_gpu(torch, torch.cuda.current_device()) as placed:
        pin = {k: v.cpu().pin_memory() for k, v in bufs.items()}
        hostC = [torch.empty((M, LD), dtype=torch.float32).pin_memory() for _ in range(2)]
    nbytes = M * LD * 4
    # End to end, pipelined over the four modes as a caller would: mode i+1's operands go up on
    # one stream while mode i computes and mode i-1's C comes down on another (the host link
    # carries both directions at once); device operands are double-buffered by mode parity.
    slots = [{k: torch.empty_like(bufs["C"]) for k in ("A", "B", "C")} for _ in range(2)]
    s_in, s_out = torch.cuda.Stream(), torch.cuda.Stream()

    def step_host():
        h2d = d2h = 0
        e0 = torch.cuda.Event()
        e0.record(ctx.stream)
        s_in.wait_event(e0)
        used = [None, None]   # per slot: D2H of the C of the last mode that used it
        for i, mode in enumerate(MODES):
            sl = slots[i % 2]
            an, bn = ("A_T" if mode[0] == "T" else "A_N"), ("B_T" if mode[1] == "T" else "B_N")
            if used[i % 2] is not None:
                s_in.wait_event(used[i % 2])
            for dst, src in ((sl["A"], pin[an]), (sl["B"], pin[bn]), (sl["C"], pin["C"])):
                memcpy(ctx, dst, src, nbytes, 0, s_in)
                h2d += nbytes
            e_in = torch.cuda.Event()
            e_in.record(s_in)
            ctx.stream.wait_event(e_in)
            gb.sgemm(mode[0], mode[1], M, N, K, ALPHA, sl["A"], LD, sl["B"], LD, BETA, sl["C"], LD,
                     algo=algo, stream=ctx.stream)
            e_c = torch.cuda.Event()
            e_c.record(ctx.stream)
            s_out.wait_event(e_c)
            memcpy(ctx, hostC[i % 2], sl["C"], nbytes, 1, s_out)
            d2h += nbytes
            used[i % 2] = torch.cuda.Event()
            used[i % 2].record(s_out)
        ctx.stream.wait_stream(s_out)
        return h2d, d2h

    e2e, h2d, d2h = e2e_measure(ctx, step_host, max(1, min(args.steps, 5)), len(MODES) * flops, 1e12)

    # the library's own per-call error report (gb_gemm_opts.err_out) of the headline form, after
    # the timed region: 16 x 16 sample, Dot2 on the device
    report = {}
    rep = torch.zeros(1, dtype=torch.float64, device=ctx.dev)
    for mode in MODES:
        Cw = C0.clone()
        A, B = ops(mode)
        gb.sgemm(mode[0], mode[1], M, N, K, ALPHA, A, LD, B, LD, BETA, Cw, LD, algo=algo, stream=ctx.stream,
                 err_out=rep)
        torch.cuda.synchronize()
        report[mode] = float(rep.item())
    report["note"] = "gb_gemm_opts.err_out: 16 rows x 16 columns spread evenly, Dot2 on the device"

    # achieved: algorithmic flops of one call over the calls' average duration in the timed region
    # (the calls back to back, as a caller issues them); the duration of a call timed alone
    # (events around it, which also keep its scan / split from overlapping the previous GEMM)
    # is kept beside it
    call_ms = ms / (args.steps * len(MODES))
    kernel_tflops = flops / (call_ms * 1e-3) / 1e12
    if algo_name in products:
        npr = products[algo_name]
        roof = {"bound": "tensor", "achieved": kernel_tflops, "peak": ctx.peaks["bf16_tflops"] / npr,
                "unit": "TFLOP/s", "peak_note": "BF16 dense %s burst peak / %d (%d 16-bit products per FP32 "
                "product; FP16 and BF16 run at one rate); achieved = 2MNK / average duration of one gb_sgemm call "
                "in the timed region (%s)" % (ctx.peak_src, npr, npr, "scan + split + MMA kernels" if algo_name == "fp16x3"
                                               else "split + MMA kernels")}
        kname = "sgemm_%s_4096" % algo_name
    else:
        roof = {"bound": "fp32-simt", "achieved": kernel_tflops, "peak": ctx.fma_peak[32], "unit": "TFLOP/s",
                "peak_note": "FFMA peak measured on this GPU (gb_measure_fma_peak)"}
        kname = "sgemm_simt_4096"
    roof["frac"] = roof["achieved"] / roof["peak"]
    roof["traffic"] = profile_traffic(kname)
    roof["call_ms"] = call_ms
    roof["call_ms_alone"] = kms
    roof["call_ms_alone_by_mode"] = by_mode

    config = {"workload": "SGEMM 4096^3, ld 4112, alpha 1.5, beta -0.5, NN/NT/TN/TT, U[-1,1] seed 1",
              "M": M, "N": N, "K": K, "ld": LD, "alpha": ALPHA, "beta": BETA, "modes": list(MODES),
              "algo": algo_name, "parallelism": "replicas x%d" % ctx.world,
              "l2": "inputs larger than L2 (8 operand buffers of 67 MB + C per step)"}
    line = base_line(ctx, METRIC, value, "TFLOP/s", ms, args.steps, "f32", config)
    line.update({"roofline": roof, "e2e": {"value": e2e, "unit": "TFLOP/s", "h2d_bytes_per_step": h2d,
                                           "d2h_bytes_per_step": d2h, "host_buffers": placed.note,
                                           "timing": E2E_TIMING},
                 "gpu_launches": launches, "clocks": clocks, "errors_normwise": errors, "err_report": report,
                 "compare": compare})
    if ctx.rank == 0 and not args.no_cpu_baseline:
        v, nt, desc = cpu_sgemm_sample()
        line["cpu_baseline"] = {"value": v, "unit": "TFLOP/s", "cores": nt, "kind": "port", "sample": desc}
    ctx.finish(line)


def run_dgemm(ctx):
    torch, gb, args = ctx.torch, ctx.gb, ctx.args
    import numpy as np
    n = args.size or 8192
    flops = 2.0 * n ** 3
    bufs = {}
    for name, seed in {"A": 31, "AT": 33, "B": 32, "BT": 34, "C": 35}.items():
        t = torch.empty((n, n), dtype=torch.float64, device=ctx.dev)
        gb.fill(t, n, n, n, seed, 2, 64, stream=ctx.stream)
        bufs[name] = t
    C0 = bufs["C"].clone()
    modes = ("NN", "TT")

    def gemm(mode, algo, C, s=0):
        A = bufs["AT" if mode[0] == "T" else "A"]
        B = bufs["BT" if mode[1] == "T" else "B"]
        gb.dgemm(mode[0], mode[1], n, n, n, 1.0, A, n, B, n, 1.0, C, n, algo=algo, ozaki_slices=s, stream=ctx.stream)

    slices = args.slices
    study = {}
    try:
        import oracle
        rng = np.random.default_rng(3)
        sub = args.subgrid
        rows = np.sort(rng.choice(n, sub, replace=False))
        cols = np.sort(rng.choice(n, sub, replace=False))
        hb = {k: v.cpu().numpy() for k, v in bufs.items() if k != "C"}
        c0 = C0.cpu().numpy()
        refs = {}
        for mode in modes:
            A = hb["AT" if mode[0] == "T" else "A"]
            B = hb["BT" if mode[1] == "T" else "B"]
            refs[mode] = (A, B, oracle.gemm_dot2(mode[0], mode[1], n, n, n, 1.0, A, n, B, n, 1.0, c0, n, rows, cols))
        rn2 = {m: oracle.op_norms(m[0], m[1], n, n, n, refs[m][0], n, refs[m][1], n, rows, cols) for m in modes}

        def err_of(mode, C):
            A, B, ref = refs[mode]
            got = C.cpu().numpy()[np.ix_(rows, cols)]
            r2, c2 = rn2[mode]
            den = math.sqrt(r2.sum() * c2.sum()) + np.linalg.norm(c0[np.ix_(rows, cols)])
            maxrel = float(np.max(np.abs(got - ref) / np.maximum(np.abs(ref), 1e-300)))
            return float(np.linalg.norm(got - ref) / den), maxrel

        for s in (4, 5, 6, 7, 8, 9):
            res = {}
            for mode in modes:
                Cw = C0.clone()
                gemm(mode, gb.ALGO_OZAKI, Cw, s)
                a, b = ctx.event(), ctx.event()
                Cw2 = C0.clone()
                a.record(ctx.stream)
                gemm(mode, gb.ALGO_OZAKI, Cw2, s)
                b.record(ctx.stream)
                torch.cuda.synchronize()
                e, mr = err_of(mode, Cw2)
                res[mode] = {"tflops": flops / (a.elapsed_time(b) * 1e-3) / 1e12, "normwise": e, "max_rel": mr}
            study["ozaki_s%d" % s] = res
        res = {}
        for mode in modes:
            Cw = C0.clone()
            a, b = ctx.event(), ctx.event()
            a.record(ctx.stream)
            gemm(mode, gb.ALGO_ORDERED, Cw)
            b.record(ctx.stream)
            torch.cuda.synchronize()
            e, mr = err_of(mode, Cw)
            res[mode] = {"tflops": flops / (a.elapsed_time(b) * 1e-3) / 1e12, "normwise": e, "max_rel": mr}
        study["native_fp64"] = res
        try:   # cuBLAS yardsticks (not the product): native DGEMM and its fixed-point emulation
            cb = Cublas(ctx.stream.cuda_stream)
            for name, compute in (("cublas_dgemm", "64F"), ("cublas_fixedpoint", "64F_EMULATED_FIXEDPOINT")):
                res = {}
                for mode in modes:
                    A = bufs["AT" if mode[0] == "T" else "A"]
                    B = bufs["BT" if mode[1] == "T" else "B"]
                    Cw = C0.clone()
                    cb.gemm(mode[0], mode[1], n, n, n, 1.0, A, n, B, n, 1.0, Cw, n, 64, compute)
                    Cw2 = C0.clone()
                    a, b = ctx.event(), ctx.event()
                    a.record(ctx.stream)
                    cb.gemm(mode[0], mode[1], n, n, n, 1.0, A, n, B, n, 1.0, Cw2, n, 64, compute)
                    b.record(ctx.stream)
                    torch.cuda.synchronize()
                    e, mr = err_of(mode, Cw2)
                    res[mode] = {"tflops": flops / (a.elapsed_time(b) * 1e-3) / 1e12, "normwise": e, "max_rel": mr}
                study[name] = res
        except Exception as e:
            study["cublas_error"] = repr(e)
        study["subgrid"] = "seeded %d x %d rows/cols, Dot2 oracle" % (sub, sub)
        if slices == 0:   # fewest slices whose error is no worse than native FP64's in both modes
            for s in (4, 5, 6, 7, 8, 9):
                if all(study["ozaki_s%d" % s][m]["normwise"] <= study["native_fp64"][m]["normwise"]
                       for m in modes):
                    slices = s
                    break
            else:
                slices = 9
    except Exception as e:
        study["error"] = repr(e)
        slices = slices or 8

    for _ in range(args.warmup):
        for mode in modes:
            gemm(mode, gb.ALGO_OZAKI, bufs["C"], slices)
    torch.cuda.synchronize()

    def step(evs):
        for mode in modes:
            a, b = ctx.event(), ctx.event()
            a.record(ctx.stream)
            gemm(mode, gb.ALGO_OZAKI, bufs["C"], slices)
            b.record(ctx.stream)
            evs.append((a, b))

    ms, kms, clocks, launches = ctx.timed(step, args.steps)
    value = aggregate(ctx.world, args.steps, len(modes) * flops, ms) / 1e12
    npairs = slices * (slices + 1) // 2
    roof = {"bound": "tensor", "achieved": flops * npairs / (kms * 1e-3) / 1e12, "peak": ctx.peaks["bf16_tflops"],
            "unit": "TFLOP/s", "peak_note": "BF16 slice-product flops (%d pairs x 2MNK) / mean gb_dgemm duration "
            "(exponents + slicing + MMA) against the %s BF16 burst peak" % (npairs, ctx.peak_src)}
    roof["frac"] = roof["achieved"] / roof["peak"]
    roof["traffic"] = profile_traffic("dgemm_ozaki_8192")
    roof["kernel_ms"] = kms
    nbytes = n * n * 8
    with near_gpu(torch, torch.cuda.current_device()) as placed:
        pin = {k: v.cpu().pin_memory() for k, v in bufs.items()}
        hostC = torch.empty((n, n), dtype=torch.float64).pin_memory()

    def step_host():
        h2d = d2h = 0
        for mode in modes:
            for name in (("AT" if mode[0] == "T" else "A"), ("BT" if mode[1] == "T" else "B"), "C"):
                memcpy(ctx, bufs[name], pin[name], nbytes, 0)
                h2d += nbytes
            gemm(mode, gb.ALGO_OZAKI, bufs["C"], slices)
            memcpy(ctx, hostC, bufs["C"], nbytes, 1)
            d2h += nbytes
        return h2d, d2h

    e2e, h2d, d2h = e2e_measure(ctx, step_host, max(1, min(args.steps, 3)), len(modes) * flops, 1e12)
    config = {"workload": "DGEMM 8192^3 NN+TT, alpha=beta=1, entries u*2^e (e in [-20,20]) seed 3",
              "M": n, "N": n, "K": n, "modes": list(modes), "algo": "ozaki", "slices": slices,
              "slices_rule": "fewest slices (4-9) whose normwise error is no worse than native FP64's in both modes",
              "parallelism": "replicas x%d" % ctx.world, "l2": "inputs larger than L2 (5 x 512 MB)"}
    line = base_line(ctx, METRIC, value, "TFLOP/s", ms, args.steps, "f64", config)
    line.update({"roofline": roof, "e2e": {"value": e2e, "unit": "TFLOP/s", "h2d_bytes_per_step": h2d,
                                           "d2h_bytes_per_step": d2h, "host_buffers": placed.note,
                                           "timing": E2E_TIMING},
                 "gpu_launches": launches, "clocks": clocks, "precision_study": study})
    if ctx.rank == 0 and not args.no_cpu_baseline:
        v, nt, desc = cpu_dgemm_sample()
        line["cpu_baseline"] = {"value": v, "unit": "TFLOP/s", "cores": nt, "kind": "port", "sample": desc}
    ctx.finish(line)


def bw_roof(ctx, gbs, kms_bytes_per_launch, kname, extra=None):
    roof = {"bound": "hbm", "achieved": gbs, "peak": ctx.peaks["hbm_gbs"], "unit": "GB/s",
            "peak_note": "%s copy bandwidth (MEASURED_PEAKS.json hbm_gbs)" % ctx.peak_src}
    roof["frac"] = roof["achieved"] / roof["peak"]
    roof["traffic"] = profile_traffic(kname)
    if extra:
        roof.update(extra)
    return roof


def run_skinny(ctx):
    torch, gb, args = ctx.torch, ctx.gb, ctx.args
    bits = args.bits
    dt = torch.float64 if bits == 64 else torch.float32
    s = bits // 8
    small, big, K = args.n, args.rows, 4096
    thin = args.workload == "thinb"
    M, N = (big, small) if thin else (small, big)
    nbytes_alg = s * (M * K + K * N + 2 * M * N)
    flops = 2.0 * M * N * K
    ops = {}
    pad = args.ld_pad   # extra elements per stored row (an unaligned leading dimension when not 0 mod 4)
    for mode in MODES:
        ar, ac = (K, M) if mode[0] == "T" else (M, K)
        br, bc = (N, K) if mode[1] == "T" else (K, N)
        A = torch.empty((ar, ac + pad), dtype=dt, device=ctx.dev)
        B = torch.empty((br, bc + pad), dtype=dt, device=ctx.dev)
        gb.fill(A, ar, ac, ac + pad, 21 + (mode[0] == "T"), 0, bits, stream=ctx.stream)
        gb.fill(B, br, bc, bc + pad, 23 + (mode[1] == "T"), 0, bits, stream=ctx.stream)
        ops[mode] = (A, ac + pad, B, bc + pad)
    C = torch.empty((M, N), dtype=dt, device=ctx.dev)
    gb.fill(C, M, N, N, 25, 0, bits, stream=ctx.stream)

    skinny_algo = {"skinny": gb.ALGO_SKINNY, "auto": gb.ALGO_AUTO, "bf16x3": gb.ALGO_BF16X3,
                   "ozaki": gb.ALGO_OZAKI}[args.skinny_algo]

    def gemm(mode):
        A, lda, B, ldb = ops[mode]
        gb.gemm(mode[0], mode[1], M, N, K, 1.0, A, lda, B, ldb, 1.0, C, N, bits, algo=skinny_algo,
                stream=ctx.stream)

    for _ in range(args.warmup):
        for mode in MODES:
            gemm(mode)
    torch.cuda.synchronize()

    def step(evs):
        for mode in MODES:
            a, b = ctx.event(), ctx.event()
            a.record(ctx.stream)
            gemm(mode)
            b.record(ctx.stream)
            evs.append((a, b))

    ms, kms, clocks, launches = ctx.timed(step, args.steps)
    value = aggregate(ctx.world, args.steps, len(MODES) * nbytes_alg, ms) / 1e9
    tflops = flops / (kms * 1e-3) / 1e12
    cpeak = ctx.fma_peak[bits]
    roof = bw_roof(ctx, nbytes_alg / (kms * 1e-3) / 1e9, None, "%s_%s_n%d" % (args.workload, "f%d" % bits, small),
                   {"compute_tflops": tflops, "compute_peak_tflops": cpeak,
                    "compute_frac": tflops / cpeak, "kernel_ms": kms, "kernel_ms_by_mode": ctx.per_mode_ms(MODES),
                    "peak_note_compute": "%s peak measured on this GPU (gb_measure_fma_peak)"
                                         % ("DFMA" if bits == 64 else "FFMA")})
    with near_gpu(torch, torch.cuda.current_device()) as placed:
        hostbufs = {m: (ops[m][0].cpu().pin_memory(), ops[m][2].cpu().pin_memory()) for m in MODES}
        hostC = C.cpu().pin_memory()

    def step_host():
        h2d = d2h = 0
        for mode in MODES:
            A, _, B, _ = ops[mode]
            hA, hB = hostbufs[mode]
            for d, h in ((A, hA), (B, hB), (C, hostC)):
                memcpy(ctx, d, h, d.numel() * s, 0)
                h2d += d.numel() * s
            gemm(mode)
            memcpy(ctx, hostC, C, C.numel() * s, 1)
            d2h += C.numel() * s
        return h2d, d2h

    e2e, h2d, d2h = e2e_measure(ctx, step_host, max(1, min(args.steps, 3)), len(MODES) * nbytes_alg, 1e9)
    config = {"workload": "%s FP%d M=%d N=%d K=%d, NN/NT/TN/TT, U[-1,1] seed 2" % (args.workload, bits, M, N, K),
              "M": M, "N": N, "K": K, "modes": list(MODES), "algo": args.skinny_algo, "ld_pad": pad,
              "bytes_per_gemm": nbytes_alg, "parallelism": "replicas x%d" % ctx.world,
              "l2": "inputs larger than L2 (large operand %d MB)" % (s * big * K // 10 ** 6)}
    line = base_line(ctx, "HBM GB/s (%s)" % args.workload, value, "GB/s", ms, args.steps, "f%d" % bits, config)
    line.update({"roofline": roof, "e2e": {"value": e2e, "unit": "GB/s", "h2d_bytes_per_step": h2d,
                                           "d2h_bytes_per_step": d2h, "host_buffers": placed.note,
                                           "timing": E2E_TIMING},
                 "gpu_launches": launches, "clocks": clocks})
    if ctx.rank == 0 and not args.no_cpu_baseline:
        v, nt, desc = cpu_bw_sample("skinny", bits)
        line["cpu_baseline"] = {"value": v, "unit": "GB/s", "cores": nt, "kind": "port", "sample": desc}
    ctx.finish(line)


def run_transpose(ctx):
    torch, gb, args = ctx.torch, ctx.gb, ctx.args
    bits = args.bits
    dt = torch.float64 if bits == 64 else torch.float32
    s = bits // 8
    M, N = (int(x) for x in args.shape.split("x"))
    A = torch.empty((M, N), dtype=dt, device=ctx.dev)
    gb.fill(A, M, N, N, 2, 0, bits, stream=ctx.stream)
    B = torch.empty((N, M), dtype=dt, device=ctx.dev)
    nbytes = 2.0 * M * N * s

    def op():
        gb.transpose(M, N, A, N, B, M, bits, stream=ctx.stream)

    for _ in range(args.warmup):
        op()
    torch.cuda.synchronize()

    def step(evs):
        a, b = ctx.event(), ctx.event()
        a.record(ctx.stream)
        op()
        b.record(ctx.stream)
        evs.append((a, b))

    ms, kms, clocks, launches = ctx.timed(step, args.steps)
    value = aggregate(ctx.world, args.steps, nbytes, ms) / 1e9
    roof = bw_roof(ctx, nbytes / (kms * 1e-3) / 1e9, None, "transpose_f%d_%s" % (bits, args.shape), {"kernel_ms": kms})
    with near_gpu(torch, torch.cuda.current_device()) as placed:
        hA = A.cpu().pin_memory()
        hB = torch.empty_like(B, device="cpu").pin_memory()

    def step_host():
        memcpy(ctx, A, hA, A.numel() * s, 0)
        op()
        memcpy(ctx, hB, B, B.numel() * s, 1)
        return A.numel() * s, B.numel() * s

    e2e, h2d, d2h = e2e_measure(ctx, step_host, max(1, min(args.steps, 3)), nbytes, 1e9)
    config = {"workload": "transpose %d x %d FP%d, bit-exact" % (M, N, bits), "M": M, "N": N,
              "parallelism": "replicas x%d" % ctx.world, "l2": "inputs larger than L2"}
    line = base_line(ctx, "HBM GB/s (transpose)", value, "GB/s", ms, args.steps, "f%d" % bits, config)
    line.update({"roofline": roof, "e2e": {"value": e2e, "unit": "GB/s", "h2d_bytes_per_step": h2d,
                                           "d2h_bytes_per_step": d2h, "host_buffers": placed.note,
                                           "timing": E2E_TIMING},
                 "gpu_launches": launches, "clocks": clocks})
    if ctx.rank == 0 and not args.no_cpu_baseline:
        v, nt, desc = cpu_bw_sample("transpose", bits)
        line["cpu_baseline"] = {"value": v, "unit": "GB/s", "cores": nt, "kind": "port", "sample": desc}
    ctx.finish(line)


def run_jacobi(ctx):
    torch, gb, args = ctx.torch, ctx.gb, ctx.args
    bits = args.bits
    dt = torch.float64 if bits == 64 else torch.float32
    s = bits // 8
    M = N = 8192
    iters = args.iters
    A = torch.ones((M + 2, N + 2), dtype=dt, device=ctx.dev)
    inner = torch.empty((M, N), dtype=dt, device=ctx.dev)
    gb.fill(inner, M, N, N, 2, 1, bits, stream=ctx.stream)
    A[1:-1, 1:-1] = inner
    del inner
    A0 = A.clone()
    B = A.clone()
    nbytes = 2.0 * M * N * s * iters
    nine = args.points == 9
    w9 = [0.05, 0.1, 0.05, 0.1, 0.4, 0.1, 0.05, 0.1, 0.05]   # a smoothing window

    def op():
        if nine:
            gb.stencil9(M, N, A, B, iters, w9, bits, stream=ctx.stream)
        else:
            gb.stencil2d(M, N, A, B, iters, gb.STENCIL_HOST, bits, stream=ctx.stream)

    for _ in range(max(1, args.warmup)):
        op()
    torch.cuda.synchronize()

    def step(evs):
        a, b = ctx.event(), ctx.event()
        a.record(ctx.stream)
        op()
        b.record(ctx.stream)
        evs.append((a, b))

    ms, kms, clocks, launches = ctx.timed(step, args.steps)
    value = aggregate(ctx.world, args.steps, nbytes, ms) / 1e9
    gflops = (17.0 if nine else 5.0) * M * N * iters / (kms * 1e-3) / 1e12
    extra = {"kernel_ms": kms, "points_per_s": M * N * iters / (kms * 1e-3),
             "fp_tflops": gflops, "note": "achieved = algorithmic bytes (2*M*N*s per sweep) / time; temporal "
             "blocking lets it exceed the HBM peak (DRAM bytes in profiles/)"}
    if bits == 64:
        extra.update({"compute_bound": "fp64", "compute_peak_tflops": ctx.fma_peak[64],
                      "compute_frac": gflops / ctx.fma_peak[64], "compute_peak_note": "DFMA peak measured on this GPU"})
    roof = bw_roof(ctx, nbytes / (kms * 1e-3) / 1e9, None, "%s_f%d_8192" % ("stencil9" if nine else "jacobi", bits),
                   extra)
    with near_gpu(torch, torch.cuda.current_device()) as placed:
        hA = A0.cpu().pin_memory()
        hR = torch.empty_like(A, device="cpu").pin_memory()

    def step_host():
        memcpy(ctx, A, hA, A.numel() * s, 0)
        memcpy(ctx, B, hA, A.numel() * s, 0)
        op()
        memcpy(ctx, hR, B if iters % 2 else A, A.numel() * s, 1)
        return 2 * A.numel() * s, A.numel() * s

    e2e, h2d, d2h = e2e_measure(ctx, step_host, max(1, min(args.steps, 3)), nbytes, 1e9)
    config = {"workload": "%s 8192^2 FP%d, %d sweeps, boundary 1.0, interior U[0,1] seed 2"
                          % ("9-point stencil (3x3 smoothing window)" if nine else "Jacobi", bits, iters),
              "M": M, "N": N, "iters": iters, "order": "window, product + 8 fma" if nine else "host",
              "parallelism": "replicas x%d" % ctx.world,
              "l2": "grid larger than L2"}
    line = base_line(ctx, "HBM GB/s (%s)" % ("stencil9" if nine else "jacobi"), value, "GB/s", ms, args.steps,
                     "f%d" % bits, config)
    line.update({"roofline": roof, "e2e": {"value": e2e, "unit": "GB/s", "h2d_bytes_per_step": h2d,
                                           "d2h_bytes_per_step": d2h, "host_buffers": placed.note,
                                           "timing": E2E_TIMING},
                 "gpu_launches": launches, "clocks": clocks})
    if ctx.rank == 0 and not args.no_cpu_baseline and not nine:
        v, nt, desc = cpu_bw_sample("jacobi", bits)
        line["cpu_baseline"] = {"value": v, "unit": "GB/s", "cores": nt, "kind": "port", "sample": desc}
    ctx.finish(line)


def _serve_stream(rate, duration, seed, max_dim):
    """The mixed request stream (arrival time, class, dtype, shape, modes, alpha, beta)."""
    import numpy as np
    rng = np.random.default_rng(seed)
    n = int(rate * duration)
    t = np.cumsum(rng.exponential(1.0 / rate, size=n))
    cls = rng.choice(5, size=n, p=[0.40, 0.25, 0.25, 0.05, 0.05])
    bits = np.where(rng.random(n) < 0.70, 32, 64)
    modes = rng.integers(0, 4, size=n)
    ab = rng.uniform(-2, 2, size=(n, 2))

    def logu(lo, hi, size=None):
        return np.exp(rng.uniform(np.log(lo), np.log(min(hi, max_dim)), size=size)).astype(np.int64)

    reqs = []
    for i in range(n):
        c = int(cls[i])
        if c == 0:
            m = int(logu(256, 4096))
            shape = (m, m, m)
        elif c == 1:
            shape = (int(logu(1024, 65536)), int(rng.integers(4, 65)), int(logu(1024, 65536)))
        elif c == 2:
            shape = (int(rng.integers(4, 65)), int(logu(1024, 65536)), int(logu(1024, 65536)))
        elif c == 3:
            shape = (int(logu(1024, 8192)), int(logu(1024, 8192)), 0)
        else:
            g = int(logu(512, 4096))
            shape = (g, g, int(rng.integers(10, 101)))
        reqs.append((float(t[i]), c, int(bits[i]), shape, "NN NT TN TT".split()[int(modes[i])],
                     float(ab[i, 0]), float(ab[i, 1])))
    return reqs


def run_serve(ctx):
    """Serving workload: Poisson arrivals (seed 4) of a mixed stream
    (40% GEMM M=N=K log-uniform 256-4096, 25% thinB N 4-64 / M,K log-uniform
    1024-65536, 25% shortA mirror, 5% transpose, 5% Jacobi 10-100 sweeps on
    512-4096 grids; 70/30 FP32/FP64; uniform modes; alpha, beta ~ U[-2,2];
    entries U[-1,1]) served under a 48 GB HBM budget, against the plain path
    (one launch per request, one stream, no grouping or graphs).  Operands
    are read from resident pools filled once; outputs go to per-request
    ring slots.  Transpose shapes (unspecified in the config) are
    log-uniform 1024-8192 per side."""
    torch, gb, args = ctx.torch, ctx.gb, ctx.args
    import numpy as np
    reqs = _serve_stream(args.rate, args.duration, 4, args.max_dim)
    max_in = max(r[3][0] * r[3][2] if r[1] == 1 else (r[3][1] * r[3][2] if r[1] == 2 else 0) for r in reqs)
    max_in = max(max_in, 4096 * 4096, 8192 * 8192)
    pools = {}
    for bits, dt in ((32, torch.float32), (64, torch.float64)):
        t = torch.empty(max_in, dtype=dt, device=ctx.dev)
        gb.fill(t, 1, max_in, max_in, 40 + bits, 0, bits, stream=ctx.stream)
        pools[bits] = t
    slots = args.slots
    slot_elems = 8192 * 8192
    outs = [torch.empty(slot_elems, dtype=torch.float64, device=ctx.dev) for _ in range(slots)]
    grid_bytes = 4098 * 4098
    torch.cuda.synchronize()

    # warm the tuner on the bucket grid the stream uses most (regular GEMMs)
    tuned = {}
    if not args.no_tune:
        for bits in (32, 64):
            for lg in range(8, 13):
                m = 1 << lg
                a, ms = gb.autotune_gemm(bits, "N", "N", m, m, m)
                for mode in ("NT", "TN", "TT"):
                    gb.lib().gb_autotune_set(bits, mode[0].encode(), mode[1].encode(), m, m, m, a)
                tuned["%d_%d" % (bits, m)] = gb.ALGO_NAMES[a]

    def make_request(i, r, slot):
        t, c, bits, shape, mode, alpha, beta = r
        pool = pools[bits]
        out = outs[slot]
        es = bits // 8
        optr = out.data_ptr()
        if c in (0, 1, 2):
            M, N, K = shape
            lda = M if mode[0] == "T" else K
            ldb = K if mode[1] == "T" else N
            return gb.request(gb.OP_GEMM, bits, M, N, K, A=pool.data_ptr(), lda=lda, B=pool.data_ptr(), ldb=ldb,
                              C=optr, ldc=N, ta=mode[0], tb=mode[1], alpha=alpha, beta=beta, tag=i)
        if c == 3:
            M, N, _ = shape
            return gb.request(gb.OP_TRANSPOSE, bits, M, N, A=pool.data_ptr(), lda=N, B=optr, ldb=M, tag=i)
        g, _, iters = shape
        # two padded grids inside the slot (halo keeps whatever the slot holds)
        return gb.request(gb.OP_STENCIL, bits, g, g, A=optr, C=optr + grid_bytes * es, iters=iters, tag=i)

    def serve(label, **cfg):
        # each stream's workspace reserved up front (a workspace that grows mid-run frees its old
        # buffer, and cudaFree waits for the whole device: every stream stalls)
        srv = gb.Server(hbm_budget_bytes=int(args.budget_gb * (1 << 30)),
                        workspace_bytes=int(args.workspace_gb * (1 << 30)), **cfg)
        lats = {}
        free = list(range(slots))
        slot_of = {}
        t0 = time.perf_counter()
        lag = 0.0
        for i, r in enumerate(reqs):
            wait = r[0] - (time.perf_counter() - t0)
            if wait > 0:
                time.sleep(wait)
            else:
                lag = max(lag, -wait)
            while not free:   # every output slot is held by an unfinished request
                for tag, lat in srv.poll():
                    free.append(slot_of.pop(tag))
                    lats[tag] = lat
                if not free:
                    time.sleep(50e-6)
            for tag, lat in srv.poll():
                free.append(slot_of.pop(tag))
                lats[tag] = lat
            slot = free.pop()
            slot_of[i] = slot
            srv.submit(make_request(i, r, slot))
        submit_end = time.perf_counter() - t0
        try:
            srv.drain(args.drain_timeout)
            drained = True
        except gb.GBError:
            drained = False
        for tag, lat in srv.poll(1 << 20):
            lats[tag] = lat
        st = srv.stats()
        srv.close()
        # latency by request class (the 1 % slowest of each)
        per = {}
        for tag, lat in lats.items():
            r = reqs[tag]
            per.setdefault("%s_f%d" % (("gemm", "thinB", "shortA", "transpose", "jacobi")[r[1]], r[2]), []).append(lat)
        by_class = {k: {"n": len(v), "p50_ms": 1e3 * float(np.percentile(v, 50)),
                        "p99_ms": 1e3 * float(np.percentile(v, 99))} for k, v in sorted(per.items())}
        return {"label": label, "p50_ms": st["p50_s"] * 1e3, "p99_ms": st["p99_s"] * 1e3,
                "mean_ms": st["mean_s"] * 1e3, "req_per_s": st["req_per_s"], "completed": st["completed"],
                "submitted": st["submitted"], "failed": st["failed"], "launches": st["launches"],
                "grouped_launches": st["grouped_launches"], "grouped_requests": st["grouped_requests"],
                "graph_launches": st["graph_launches"], "graph_instantiations": st["graph_instantiations"],
                "graph_fraction": st["graph_launches"] / st["launches"] if st["launches"] else 0.0,
                "urgent_launches": st["urgent_launches"],
                "drained": drained, "submit_lag_s": lag, "submit_span_s": submit_end, "by_class": by_class}

    l0 = gb.launch_count()
    sampler = ClockSampler(ctx.local)
    sampler.start()
    main = serve("streams=%d grouped=%d graphs=%d short_us=%g short_streams=%d long_sm=%d%%"
                 % (args.serve_streams, args.serve_grouped, args.serve_graphs, args.serve_short_us,
                    args.serve_short_streams, args.serve_long_sm),
                 streams=args.serve_streams, use_grouped=args.serve_grouped, use_graphs=args.serve_graphs,
                 short_us=args.serve_short_us, short_streams=args.serve_short_streams,
                 long_sm_percent=args.serve_long_sm)
    clocks = sampler.stop()
    launches = gb.launch_count() - l0
    plain = serve("plain", streams=1, use_grouped=0, use_graphs=0) if not args.no_plain else None
    # isolated solves: a sample of the stream, one request at a time
    iso = []
    by_class = {}
    rng = np.random.default_rng(44)
    srv = gb.Server(streams=1)
    for i in rng.choice(len(reqs), size=min(args.iso_sample, len(reqs)), replace=False):
        srv.submit(make_request(int(i), reqs[int(i)], 0))
        srv.drain(60.0)
        lats = [lat for _, lat in srv.poll()]
        iso += lats
        r = reqs[int(i)]
        by_class.setdefault("%s_f%d" % (("gemm", "thinB", "shortA", "transpose", "jacobi")[r[1]], r[2]), []).extend(lats)
    srv.close()
    iso_p50, iso_p99 = float(np.percentile(iso, 50)) * 1e3, float(np.percentile(iso, 99)) * 1e3
    # offered load: the stream's share of each class x its mean isolated solve time
    share = {}
    for r in reqs:
        k = "%s_f%d" % (("gemm", "thinB", "shortA", "transpose", "jacobi")[r[1]], r[2])
        share[k] = share.get(k, 0) + 1
    iso_classes = {k: {"n": len(v), "mean_ms": 1e3 * float(np.mean(v)), "p99_ms": 1e3 * float(np.percentile(v, 99))}
                   for k, v in sorted(by_class.items())}
    offered = sum(share[k] / len(reqs) * args.rate * float(np.mean(v)) for k, v in by_class.items())
    config = {"workload": "serving stream: Poisson %g req/s for %g s (seed 4), mixed GEMM/thinB/shortA/transpose/"
                          "Jacobi, 70/30 FP32/FP64, 48 GB HBM budget" % (args.rate, args.duration),
              "requests": len(reqs), "budget_gb": args.budget_gb, "workspace_gb_per_stream": args.workspace_gb,
              "streams": args.serve_streams,
              "grouped": args.serve_grouped, "graphs": args.serve_graphs, "short_us": args.serve_short_us,
              "short_streams": args.serve_short_streams, "long_sm_percent": args.serve_long_sm,
              "ring_slots": slots,
              "max_dim": args.max_dim, "tuned": tuned}
    line = base_line(ctx, "serve p50/p99, req/s", main["req_per_s"], "req/s", main["submit_span_s"] * 1e3, 1,
                     "f32+f64", config)
    line.update({"serve": main, "plain": plain,
                 "isolated": {"p50_ms": iso_p50, "p99_ms": iso_p99, "sample": len(iso), "by_class": iso_classes},
                 "offered_load_gpu_s_per_s": offered,
                 "p99_over_isolated_p99": main["p99_ms"] / iso_p99 if iso_p99 > 0 else None,
                 "gpu_launches": launches, "clocks": clocks,
                 "e2e": {"value": main["req_per_s"], "unit": "req/s", "h2d_bytes_per_step": 0,
                         "d2h_bytes_per_step": 0, "note": "operands resident by design (device-resident serving)"}})
    ctx.finish(line)


# ================================================================== reference arm
def run_reference_arm(args):
    """The reference's own CPU implementation of the path (the oracle's port of
    its host loop: the reference's device code needs the MT-3000 toolchain and
    its package does not install), timed on the host cores, rank 0 only."""
    if int(os.environ.get("RANK", "0")) != 0:
        return
    world = int(os.environ.get("WORLD_SIZE", "1"))
    vals, desc, nt = [], "", 1
    fn = {"sgemm": cpu_sgemm_sample, "dgemm": cpu_dgemm_sample}.get(args.workload)
    for _ in range(max(1, args.steps)):
        if fn:
            v, nt, desc = fn(max_seconds=6.0)
        else:
            v, nt, desc = cpu_bw_sample("skinny" if args.workload in ("thinb", "shorta") else args.workload, args.bits)
        vals.append(v)
    value = statistics.median(vals)
    unit = "TFLOP/s" if fn else "GB/s"
    metric = METRIC if fn else "HBM GB/s (%s)" % args.workload
    line = {"impl": "reference", "metric": metric, "value": value, "unit": unit, "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32" if args.workload == "sgemm" else "f%d" % args.bits,
            "data": "synthetic",
            "config": {"workload": args.workload, "algo": "reference host loop (CPU)"},
            "cpu_baseline": {"value": value, "unit": unit, "cores": nt, "kind": "port", "sample": desc},
            "e2e": {"value": value, "unit": unit, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    if args.workload == "sgemm":
        line["config"].update({"workload": "SGEMM 4096^3, ld 4112, alpha 1.5, beta -0.5, NN/NT/TN/TT, U[-1,1] seed 1",
                               "M": 4096, "N": 4096, "K": 4096})
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--workload", default="sgemm",
                    choices=["sgemm", "dgemm", "thinb", "shorta", "transpose", "jacobi", "serve"])
    ap.add_argument("--algo", default="best", choices=["best", "bf16x3", "bf16x6", "fp16x3", "simt"])
    ap.add_argument("--bits", type=int, default=32, choices=[32, 64])
    ap.add_argument("--n", type=int, default=8, help="small dimension of thinb/shorta")
    ap.add_argument("--skinny-algo", default="auto", choices=["auto", "skinny", "bf16x3", "ozaki"])
    ap.add_argument("--rows", type=int, default=262144, help="thinb/shorta: the large dimension")
    ap.add_argument("--ld-pad", type=int, default=0, help="thinb/shorta: leading-dimension padding in elements")
    ap.add_argument("--shape", default="30000x17000", help="transpose: MxN")
    ap.add_argument("--iters", type=int, default=200, help="jacobi sweeps")
    ap.add_argument("--points", type=int, default=5, choices=[5, 9], help="jacobi: 5-point or 9-point stencil")
    ap.add_argument("--slices", type=int, default=0, help="dgemm: Ozaki slices (0: fewest matching native error)")
    ap.add_argument("--size", type=int, default=0, help="dgemm: M=N=K (default 8192)")
    ap.add_argument("--subgrid", type=int, default=1024, help="dgemm: error subgrid size")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--rate", type=float, default=2000.0, help="serve: arrivals per second")
    ap.add_argument("--duration", type=float, default=60.0, help="serve: seconds of arrivals")
    ap.add_argument("--budget-gb", type=float, default=48.0, help="serve: HBM admission budget")
    ap.add_argument("--workspace-gb", type=float, default=1.0, help="serve: workspace reserved per stream")
    ap.add_argument("--max-dim", type=int, default=65536, help="serve: cap on log-uniform sizes")
    ap.add_argument("--slots", type=int, default=64, help="serve: output ring slots (max in flight)")
    ap.add_argument("--drain-timeout", type=float, default=120.0)
    ap.add_argument("--iso-sample", type=int, default=200)
    ap.add_argument("--no-plain", action="store_true")
    ap.add_argument("--serve-streams", type=int, default=6, help="serve: stream pool of the measured server")
    ap.add_argument("--serve-grouped", type=int, default=1, help="serve: group small GEMMs (1) or not (0)")
    ap.add_argument("--serve-graphs", type=int, default=1, help="serve: replay CUDA graphs (1) or not (0)")
    ap.add_argument("--serve-short-us", type=float, default=200.0,
                    help="serve: requests estimated below this go to the high-priority streams (0: off)")
    ap.add_argument("--serve-short-streams", type=int, default=2, help="serve: high-priority streams")
    ap.add_argument("--serve-long-sm", type=int, default=100, help="serve: percent of SMs a long request plans for")
    ap.add_argument("--no-tune", action="store_true")
    args = ap.parse_args()
    if args.impl == "reference":
        return run_reference_arm(args)
    args.warmup = max(args.warmup, 3)
    ctx = Ctx(args)
    {"sgemm": run_sgemm, "dgemm": run_dgemm, "thinb": run_skinny, "shorta": run_skinny,
     "transpose": run_transpose, "jacobi": run_jacobi, "serve": run_serve}[args.workload](ctx)


if __name__ == "__main__":
    main()
