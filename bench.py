"""Benchmark of the GB300 BLAS hot path on the SGEMM headline workload.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference] [--algo best|bf16x3|simt]

Workload (one "step"): SGEMM C = alpha*op(A)op(B) + beta*C, FP32, row-major,
M = N = K = 4096, leading dimensions padded to 4112, alpha = 1.5,
beta = -0.5, in all four transpose modes (NN, NT, TN, TT), entries uniform in
[-1,1] from seed 1 (the project's counter-based generator, on the device).
Each step runs the four GEMMs; the operands of a step (8 x 67 MB + C) exceed
the 129 MB L2, so no explicit flush is needed between iterations.

value   = whole-job TFLOP/s = n_gpus * 4 * 2*M*N*K / (max over ranks of the
          timed region), inputs resident in HBM;
e2e     = the same metric through the C ABI with host buffers: each GEMM's
          A, B, C are copied host->device (pinned memory, gb_memcpy), computed,
          and C is copied back, all inside the timed region;
roofline: the GEMM kernel's achieved TFLOP/s (2*M*N*K per launch / the mean
          CUDA-event duration of its launches in the timed region) against
          the measured peak of its pipe (MEASURED_PEAKS.json);
cpu_baseline: the reference's host SGEMM loop (the oracle's restatement of
          sgemm_release_V1.3.2/host_code/sgemm_demo.c:214-242) on a bounded
          sample of rows, with every host core.
Multi-GPU: replicas (each rank runs the same workload; no collective on the
data path), "scaling": "weak".
"""
import argparse
import ctypes
import json
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
M = N = K = 4096
LD = 4112
ALPHA, BETA = 1.5, -0.5
MODES = ("NN", "NT", "TN", "TT")
FLOPS_PER_GEMM = 2.0 * M * N * K


def log(*a):
    print(*a, file=sys.stderr, flush=True)


def measured_peaks():
    try:
        with open(os.path.join(REPO, "MEASURED_PEAKS.json")) as f:
            p = json.load(f)
        return p, "measured"
    except (OSError, ValueError):
        return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "bf16_tflops_sustained": 1700.0}, "fallback"


def profile_traffic(name):
    """DRAM bytes per launch recorded from an ncu capture in profiles/<name>.txt
    (a line 'traffic_bytes_per_launch: <int>'), else None."""
    path = os.path.join(REPO, "profiles", name + ".txt")
    try:
        for line in open(path):
            if line.startswith("traffic_bytes_per_launch:"):
                return int(float(line.split(":", 1)[1].strip()))
    except OSError:
        pass
    return None


class ClockSampler:
    """nvidia-smi samples of SM clock and throttle reasons during the timed region."""
    Q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.Q,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
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


# ------------------------------------------------------------- CPU legs
def cpu_reference_sample(max_seconds=12.0):
    """The reference's host SGEMM loop (oracle restatement) on a bounded sample
    of C rows, all four modes; returns (TFLOP/s, threads, description)."""
    import numpy as np
    import oracle

    nt = os.cpu_count() or 1
    oracle.set_threads(nt)
    A = oracle.fill(M, K, 11, dtype=np.float32, ld=LD)
    B = oracle.fill(K, N, 12, dtype=np.float32, ld=LD)
    rows = 8
    while True:
        flops, secs = 0.0, 0.0
        for mode in MODES:
            ta, tb = mode
            Cs = np.zeros((rows, LD), dtype=np.float32)
            t0 = time.perf_counter()
            # rows of C: op(A) restricted to `rows` rows (TN/TT read A^T storage: same bytes pattern)
            oracle.sgemm_ref(ta, tb, rows, N, K, ALPHA, A, LD, B, LD, BETA, Cs, LD)
            secs += time.perf_counter() - t0
            flops += 2.0 * rows * N * K
        if secs * 3 > max_seconds or rows >= 256:
            break
        rows *= 2
    return flops / secs / 1e12, nt, "%d of %d rows of C per mode, 4 modes, K=%d (oracle port of the reference " \
        "host loop, gcc -O2 -fopenmp, %d threads)" % (rows, M, K, nt)


def run_reference_arm(args, rank, world):
    if rank != 0:
        return
    import numpy as np  # noqa: F401
    nt = os.cpu_count() or 1
    for _ in range(args.warmup):
        pass
    vals = []
    desc = ""
    for _ in range(max(1, args.steps)):
        v, nt, desc = cpu_reference_sample(max_seconds=6.0)
        vals.append(v)
    value = statistics.median(vals)
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": "TFLOP/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": config_dict(world, "reference host loop (CPU)"),
            "cpu_baseline": {"value": value, "unit": "TFLOP/s", "cores": nt, "kind": "port", "sample": desc},
            "e2e": {"value": value, "unit": "TFLOP/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def config_dict(world, algo):
    return {"workload": "SGEMM 4096^3, ld 4112, alpha 1.5, beta -0.5, NN/NT/TN/TT, U[-1,1] seed 1",
            "M": M, "N": N, "K": K, "ld": LD, "alpha": ALPHA, "beta": BETA, "modes": list(MODES),
            "algo": algo, "parallelism": "replicas x%d" % world,
            "l2": "inputs larger than L2 (8 operand buffers of 67 MB + C per step)"}


# ------------------------------------------------------------- GPU leg
def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--algo", default="best", choices=["best", "bf16x3", "simt"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3) if args.impl == "gb300" else args.warmup

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))

    if args.impl == "reference":
        return run_reference_arm(args, rank, world)

    import numpy as np
    import torch

    import gbblas

    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    gbblas.lib()
    arch = gbblas.arch()
    if arch != 103:
        raise SystemExit("bench.py: needs an sm_103 GPU (found sm_%d)" % arch)

    dev = torch.device("cuda", local)
    stream = torch.cuda.current_stream(dev)
    bufs = {}
    seeds = {"A_N": 11, "A_T": 12, "B_N": 13, "B_T": 14, "C": 15}
    for name, seed in seeds.items():
        t = torch.empty((M, LD), dtype=torch.float32, device=dev)
        gbblas.fill(t, M, K, LD, seed, 0, 32, stream=stream)
        bufs[name] = t
    C0 = bufs["C"].clone()

    def operands(mode):
        return bufs["A_T" if mode[0] == "T" else "A_N"], bufs["B_T" if mode[1] == "T" else "B_N"]

    def algo_id(name):
        return {"bf16x3": gbblas.ALGO_BF16X3, "simt": gbblas.ALGO_SIMT}[name]

    def gemm(mode, algo, C=None):
        A, B = operands(mode)
        gbblas.sgemm(mode[0], mode[1], M, N, K, ALPHA, A, LD, B, LD, BETA, bufs["C"] if C is None else C, LD,
                     algo=algo, stream=stream)

    # choose the headline algorithm
    algo_name = args.algo
    if algo_name == "best":
        algo_name = "bf16x3"
        try:
            gemm("NN", gbblas.ALGO_BF16X3)
            torch.cuda.synchronize()
        except gbblas.GBError as e:
            if e.status != gbblas.ERR_UNSUPPORTED:
                raise
            algo_name = "simt"
    algo = algo_id(algo_name)

    # ---- accuracy (checker): normwise error on a seeded 128x128 subgrid
    errors = {}
    try:
        import oracle
        rng = np.random.default_rng(1)
        rows = np.sort(rng.choice(M, 128, replace=False))
        cols = np.sort(rng.choice(N, 128, replace=False))
        hostbuf = {k: v.cpu().numpy() for k, v in bufs.items() if k != "C"}
        c0 = C0.cpu().numpy()
        for an in (["simt", "bf16x3"] if algo_name == "bf16x3" else ["simt"]):
            worst = 0.0
            for mode in MODES:
                Cw = C0.clone()
                gemm(mode, algo_id(an), Cw)
                got = Cw.cpu().numpy()
                A = hostbuf["A_T" if mode[0] == "T" else "A_N"]
                B = hostbuf["B_T" if mode[1] == "T" else "B_N"]
                e, _ = oracle.normwise_error(got, mode[0], mode[1], M, N, K, ALPHA, A, LD, B, LD, BETA, c0, LD,
                                             rows, cols)
                worst = max(worst, e)
            errors[an] = worst
        errors["bound_2Ku"] = 2 * K * 2.0 ** -24
    except Exception as e:  # the error report must not hide the timing
        errors["error"] = repr(e)

    # ---- warmup
    for _ in range(args.warmup):
        for mode in MODES:
            gemm(mode, algo)
    torch.cuda.synchronize()

    # ---- timed region (device-resident inputs)
    nev = args.steps * len(MODES)
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(nev)]
    t_start, t_end = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    sampler = ClockSampler(local)
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    sampler.start()
    time.sleep(0.3)
    launches0 = gbblas.launch_count()
    t_start.record(stream)
    i = 0
    for _ in range(args.steps):
        for mode in MODES:
            ev[i][0].record(stream)
            gemm(mode, algo)
            ev[i][1].record(stream)
            i += 1
    t_end.record(stream)
    torch.cuda.synchronize()
    launches = gbblas.launch_count() - launches0
    clocks = sampler.stop()
    elapsed_ms = t_start.elapsed_time(t_end)
    if dist:
        t = torch.tensor([elapsed_ms], device=dev)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        elapsed_ms = float(t.item())
    per_launch_ms = statistics.mean(a.elapsed_time(b) for a, b in ev)
    value = world * args.steps * len(MODES) * FLOPS_PER_GEMM / (elapsed_ms * 1e-3) / 1e12

    # ---- plain SIMT comparison (one step, same workload), when the headline is bf16x3
    compare = {}
    if algo_name != "simt":
        s0, s1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        for mode in MODES:
            gemm(mode, gbblas.ALGO_SIMT)
        s0.record(stream)
        for _ in range(2):
            for mode in MODES:
                gemm(mode, gbblas.ALGO_SIMT)
        s1.record(stream)
        torch.cuda.synchronize()
        compare["simt_tflops"] = 2 * len(MODES) * FLOPS_PER_GEMM / (s0.elapsed_time(s1) * 1e-3) / 1e12

    # ---- e2e through the C ABI with host buffers
    pin = {k: v.cpu().pin_memory() for k, v in bufs.items()}
    hostC = torch.empty((M, LD), dtype=torch.float32).pin_memory()
    nbytes = M * LD * 4
    L = gbblas.lib()

    def e2e_step():
        h2d = d2h = 0
        for mode in MODES:
            an, bn = ("A_T" if mode[0] == "T" else "A_N"), ("B_T" if mode[1] == "T" else "B_N")
            for src, dst in ((pin[an], bufs[an]), (pin[bn], bufs[bn]), (pin["C"], bufs["C"])):
                st = L.gb_memcpy(ctypes.c_void_p(dst.data_ptr()), ctypes.c_void_p(src.data_ptr()), nbytes, 0,
                                 ctypes.c_void_p(stream.cuda_stream))
                assert st == 0
                h2d += nbytes
            gemm(mode, algo)
            st = L.gb_memcpy(ctypes.c_void_p(hostC.data_ptr()), ctypes.c_void_p(bufs["C"].data_ptr()), nbytes, 1,
                             ctypes.c_void_p(stream.cuda_stream))
            assert st == 0
            d2h += nbytes
        return h2d, d2h

    e2e_step()
    torch.cuda.synchronize()
    e_steps = max(1, min(args.steps, 5))
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    if dist:
        dist.barrier()
    e0.record(stream)
    for _ in range(e_steps):
        h2d, d2h = e2e_step()
    e1.record(stream)
    torch.cuda.synchronize()
    e_ms = e0.elapsed_time(e1)
    if dist:
        t = torch.tensor([e_ms], device=dev)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        e_ms = float(t.item())
    e2e_value = world * e_steps * len(MODES) * FLOPS_PER_GEMM / (e_ms * 1e-3) / 1e12

    # ---- roofline of the GEMM kernel
    peaks, peak_src = measured_peaks()
    kernel_tflops = FLOPS_PER_GEMM / (per_launch_ms * 1e-3) / 1e12
    if algo_name == "bf16x3":
        # three BF16 products per FP32 product on the tensor pipe
        roof = {"bound": "tensor", "achieved": kernel_tflops, "peak": peaks["bf16_tflops"] / 3.0,
                "unit": "TFLOP/s", "peak_note": "bf16 dense %s peak / 3 (3 products per FP32 FMA)" % peak_src}
        kname = "sgemm_bf16x3_4096"
    else:
        fp32_peak = 152 * 128 * 2 * 2.07e9 / 1e12
        roof = {"bound": "fp32-simt", "achieved": kernel_tflops, "peak": fp32_peak, "unit": "TFLOP/s",
                "peak_note": "nominal FFMA peak 152 SMs x 128 lanes x 2 x 2.07 GHz (no measured FP32 peak)"}
        kname = "sgemm_simt_4096"
    roof["frac"] = roof["achieved"] / roof["peak"]
    roof["traffic"] = profile_traffic(kname)
    roof["kernel_ms"] = per_launch_ms

    line = {"metric": METRIC, "value": value, "unit": "TFLOP/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": elapsed_ms / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": config_dict(world, algo_name), "roofline": roof,
            "e2e": {"value": e2e_value, "unit": "TFLOP/s", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h},
            "gpu_launches": int(launches), "clocks": clocks, "errors_normwise": errors, "compare": compare}

    if rank == 0 and not args.no_cpu_baseline:
        try:
            v, nt, desc = cpu_reference_sample()
            line["cpu_baseline"] = {"value": v, "unit": "TFLOP/s", "cores": nt, "kind": "port", "sample": desc}
        except Exception as e:
            line["cpu_baseline"] = {"value": None, "unit": "TFLOP/s", "cores": 0, "kind": "port",
                                    "sample": "failed: %r" % e}
    if dist:
        dist.barrier()
        dist.destroy_process_group()
    if rank == 0:
        print(json.dumps(line), flush=True)


if __name__ == "__main__":
    main()
