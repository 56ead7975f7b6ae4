"""Generate the golden fixtures from the reference's own host demo programs.

Run here (where the reference tree exists):  python tests/golden/make_golden.py

What it does, per case:
1. ``make -C oracle`` compiles each reference demo (``*/host_code/*_demo.c``,
   ``transpose.c``, ``matrix_stencil.c``, unmodified, read from the reference
   tree) against oracle/ref_harness/, a fake MT-3000 host runtime whose
   ``hthread_group_exec`` runs the oracle and whose ``rand()`` is a counter
   stream the tests can replay (tests/gbgen.py ``demo_*``).
2. Runs the demo; its own CHECK_DATA loop compares the oracle's result with
   the reference loop element by element and prints Success!/Result Error!.
3. Reads the buffer dump (``$GBREF_DUMP``) and stores the reference loop's
   result array (``C_cpu`` / ``B_ref`` / ``B_cpu``) -- small ones in full,
   large ones as a SHA-256 plus a few sample values -- with the demo's
   verdict lines.

The fixtures need nothing from the reference at test time: the inputs are
replayed by tests/gbgen.py.
"""
import hashlib
import json
import os
import struct
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
ORACLE = os.path.join(REPO, "oracle")
REF = os.path.join(ORACLE, "_ref")

# (fixture name, demo binary, argv, kind, (M, K, N) or (M, N))
GEMM_CASES = [
    ("dgemm_v11_20x1030x36", "dgemm_v11", (20, 1030, 36)),
    ("dgemm_v11_33x512x17", "dgemm_v11", (33, 512, 17)),
    ("dgemm_v11_5x7x3", "dgemm_v11", (5, 7, 3)),
    ("sgemm_v132_24x1100x40", "sgemm_v132", (24, 1100, 40)),
    ("sgemm_v132_9x513x7", "sgemm_v132", (9, 513, 7)),
    ("sgemm_v131_16x600x24", "sgemm_v131", (16, 600, 24)),
    ("shortA_dgemm_v00_16x1100x64", "shortA_dgemm_v00", (16, 1100, 64)),
    ("shortA_sgemm_v00_8x1100x96", "shortA_sgemm_v00", (8, 1100, 96)),
    ("thinB_dgemm_v00_96x1100x8", "thinB_dgemm_v00", (96, 1100, 8)),
    ("thinB_sgemm_v00_96x1100x16", "thinB_sgemm_v00", (96, 1100, 16)),
    ("thinB_sgemm_v12_96x4000x8", "thinB_sgemm_v12", (96, 4000, 8)),
    ("thinB_sgemm_v12_64x3100x16", "thinB_sgemm_v12", (64, 3100, 16)),
]
TRANSPOSE_CASES = [(312, 228), (1512, 1536), (8210, 8190)]   # transpose/bin/run.sh:3-9
STENCIL_CASES = [(55, 111), (256, 300)]                      # stencil_2d_V1.2/bin/run.sh:1


def read_dump(path):
    with open(path, "rb") as f:
        data = f.read()
    assert data[:8] == b"GBREFDMP"
    (cnt,) = struct.unpack_from("<I", data, 8)
    off = 12
    bufs = []
    for _ in range(cnt):
        host, n = struct.unpack_from("<IQ", data, off)
        off += 12
        bufs.append((host, data[off:off + n]))
        off += n
    return bufs


def run(binary, args):
    dump = os.path.join(HERE, "_dump.bin")
    env = dict(os.environ, GBREF_DUMP=dump)
    out = subprocess.run([os.path.join(REF, binary)] + [str(a) for a in args], env=env,
                         capture_output=True, text=True, check=True)
    bufs = read_dump(dump)
    os.remove(dump)
    verdicts = [l.strip() for l in out.stdout.splitlines()
                if l.startswith("Success") or l.startswith("Result Error") or l.startswith("error_num")]
    return bufs, verdicts


def sha(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def main():
    subprocess.run(["make", "-C", ORACLE], check=True)
    index = {}
    for name, binary, (M, K, N) in GEMM_CASES:
        bufs, verdicts = run(binary, [1, M, K, N, 1])
        dt = np.float64 if "dgemm" in binary else np.float32
        c_cpu = np.frombuffer(bufs[8][1], dtype=dt)
        ldc = N + 256 if binary == "dgemm_v11" else N
        C = c_cpu.reshape(-1, ldc)[:M, :N].copy()
        np.save(os.path.join(HERE, name + ".npy"), C)
        # the V0.0 irregular DGEMM demos run the kernel and the check NUM_TESTS=50
        # times, accumulating into C (irr_shortA_dgemm_demo.c:11, :205)
        repeats = 50 if binary in ("shortA_dgemm_v00", "thinB_dgemm_v00") else 1
        index[name] = dict(demo=binary, M=M, K=K, N=N, dtype=str(np.dtype(dt)), verdicts=verdicts,
                           file=name + ".npy", sha256=sha(C), repeats=repeats)
        print(name, verdicts)
    for (M, N) in TRANSPOSE_CASES:
        name = "transpose_f32_%dx%d" % (M, N)
        bufs, verdicts = run("transpose", [1, M, N, 1])
        Bref = np.frombuffer(bufs[2][1], dtype=np.float32).reshape(N, M)
        picks = [0, 1, M * N // 2, M * N - 2, M * N - 1]
        index[name] = dict(demo="transpose", M=M, N=N, dtype="float32", verdicts=verdicts, sha256=sha(Bref),
                           samples={str(p): float(Bref.reshape(-1)[p]) for p in picks})
        print(name, verdicts)
    for (M, N) in STENCIL_CASES:
        name = "stencil_f64_%dx%d" % (M, N)
        bufs, verdicts = run("stencil", [M, N, 1, 1])
        # host buffers: A_cpu, B_cpu; reference_stencil writes B_cpu densely (M x N)
        Bcpu = np.frombuffer(bufs[3][1], dtype=np.float64)[: M * N].reshape(M, N).copy()
        index[name] = dict(demo="stencil", M=M, N=N, dtype="float64", verdicts=verdicts, sha256=sha(Bcpu),
                           samples={str(p): float(Bcpu.reshape(-1)[p]) for p in [0, M * N // 3, M * N - 1]})
        if M * N <= 10000:
            np.save(os.path.join(HERE, name + ".npy"), Bcpu)
            index[name]["file"] = name + ".npy"
        print(name, verdicts)
    with open(os.path.join(HERE, "golden.json"), "w") as f:
        json.dump(index, f, indent=1, sort_keys=True)


if __name__ == "__main__":
    sys.exit(main())
