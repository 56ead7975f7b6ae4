"""Build libgbblas.so in place: every .cu file for sm_103a with nvcc, the C
shim with gcc, compiled in parallel, linked into gbblas/libgbblas.so.

    python blas-for-multi-core-dsp_gb300/build.py [--force] [-j N]

Objects go to blas-for-multi-core-dsp_gb300/_build/.  A source is recompiled
when it (or any header) is newer than its object.
"""
import argparse
import concurrent.futures as cf
import glob
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
OUT = os.path.join(HERE, "gbblas", "libgbblas.so")
INCLUDE = os.path.join(REPO, "include")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-Wall",
                     "--expt-relaxed-constexpr", "-I" + INCLUDE, "-I" + CSRC]
CC_FLAGS = ["-O2", "-std=c99", "-fPIC", "-Wall", "-Wextra", "-I" + INCLUDE]


def nvcc():
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _newest_header():
    hs = glob.glob(os.path.join(CSRC, "*.cuh")) + glob.glob(os.path.join(CSRC, "*.h")) + \
        glob.glob(os.path.join(INCLUDE, "*.h"))
    return max((os.path.getmtime(h) for h in hs), default=0.0)


def _compile(src, force, hdr_time):
    base = os.path.basename(src)
    obj = os.path.join(BUILD, base + ".o")
    if not force and os.path.exists(obj):
        t = os.path.getmtime(obj)
        if t >= os.path.getmtime(src) and t >= hdr_time:
            return obj, None
    if src.endswith(".cu"):
        cmd = [nvcc()] + NVCC_FLAGS + ["-c", src, "-o", obj]
    else:
        cmd = [os.environ.get("CC", "gcc")] + CC_FLAGS + ["-c", src, "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        return obj, "FAILED: " + " ".join(cmd) + "\n" + r.stdout + r.stderr
    return obj, (r.stderr.strip() or None) if "warning" in r.stderr else None


def build(force=False, jobs=None, verbose=False):
    os.makedirs(BUILD, exist_ok=True)
    srcs = sorted(glob.glob(os.path.join(CSRC, "*.cu")) + glob.glob(os.path.join(CSRC, "*.c")))
    hdr_time = _newest_header()
    jobs = jobs or min(len(srcs), os.cpu_count() or 4)
    objs, errors = [], []
    with cf.ThreadPoolExecutor(jobs) as ex:
        for obj, msg in ex.map(lambda s: _compile(s, force, hdr_time), srcs):
            objs.append(obj)
            if msg and msg.startswith("FAILED"):
                errors.append(msg)
            elif msg and verbose:
                print(msg)
    if errors:
        raise RuntimeError("\n".join(errors))
    newest_obj = max(os.path.getmtime(o) for o in objs)
    if force or not os.path.exists(OUT) or os.path.getmtime(OUT) < newest_obj:
        cmd = [nvcc()] + ARCH + ["-shared", "-o", OUT] + objs + ["-lcuda"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("link failed: " + " ".join(cmd) + "\n" + r.stdout + r.stderr)
    return OUT


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--force", action="store_true")
    ap.add_argument("-j", type=int, default=None)
    ap.add_argument("-v", action="store_true")
    a = ap.parse_args()
    print(build(a.force, a.j, a.v))


if __name__ == "__main__":
    sys.exit(main())
