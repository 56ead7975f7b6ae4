"""The hthread_host.h shim: the reference's host programs build unmodified
against libgbblas (here, where the reference tree exists), and a host
program written against that interface runs on the GPU bit-exactly."""
import os
import subprocess

import pytest

import gbblas

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
INCLUDE = os.path.join(REPO, "include")
LIBDIR = os.path.dirname(gbblas.LIB_PATH)
REF = os.environ.get("REF_ROOT", "/root/reference")
DEMOS = ["dgemm_release_V1.1/host_code/dgemm_demo.c", "sgemm_release_V1.3.2/host_code/sgemm_demo.c",
         "irr_shortA_sgemm_release_V0.0/host_code/irr_shortA_sgemm_demo.c",
         "irr_thinB_sgemm_release_V1.2/host_code/irr_thinB_sgemm_demo.c",
         "transpose/host_code/transpose.c", "stencil_2d_V1.2/host_code/matrix_stencil.c"]


def _link_args():
    return ["-I" + INCLUDE, "-L" + LIBDIR, "-lgbblas", "-Wl,-rpath," + LIBDIR, "-lm"]


@pytest.mark.skipif(not os.path.isdir(REF), reason="reference tree not present")
@pytest.mark.parametrize("demo", DEMOS)
def test_reference_demo_builds_against_shim(demo, tmp_path):
    if not os.path.exists(gbblas.LIB_PATH):
        pytest.skip("libgbblas.so not built")
    out = str(tmp_path / "demo")
    r = subprocess.run(["gcc", "-O2", "-std=gnu99", "-fopenmp", "-w", os.path.join(REF, demo), "-o", out]
                       + _link_args(), capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-2000:]


def test_shim_demo_builds(tmp_path):
    if not os.path.exists(gbblas.LIB_PATH):
        pytest.skip("libgbblas.so not built")
    out = str(tmp_path / "hthread_demo")
    r = subprocess.run(["gcc", "-O2", "-std=gnu99", "-ffp-contract=off", os.path.join(REPO, "tests", "c",
                        "hthread_demo.c"), "-o", out] + _link_args(), capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-2000:]


@pytest.mark.gpu
def test_shim_demo_runs_bit_exact(tmp_path):
    from gpu_util import torch_cuda
    torch_cuda()
    out = str(tmp_path / "hthread_demo")
    r = subprocess.run(["gcc", "-O2", "-std=gnu99", "-ffp-contract=off", os.path.join(REPO, "tests", "c",
                        "hthread_demo.c"), "-o", out] + _link_args(), capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-2000:]
    run = subprocess.run([out], capture_output=True, text=True, timeout=300)
    assert run.returncode == 0, run.stdout + run.stderr
    assert run.stdout.count("Success!") == 6, run.stdout
