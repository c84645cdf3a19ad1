"""The integer-arithmetic IEEE double operations of gfm_xfp64.cuh (xmul,
xadd, xdiv, xsqrt) return exactly the double that the FP64 operation
returns: on the host against the host's own IEEE arithmetic (g++), on the
GPU against its division and square root (nvcc; the device's seeds are the
hardware's approximate reciprocal and reciprocal square root)."""
import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))


def test_integer_path_matches_host_ieee(tmp_path):
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("g++ not available")
    exe = str(tmp_path / "xfp64_check")
    subprocess.run([gxx, "-O2", "-std=c++17", "-ffp-contract=off", os.path.join(HERE, "xfp64_check.cpp"), "-o", exe],
                   check=True)
    out = subprocess.run([exe, "2000000"], capture_output=True, text=True, timeout=600)
    assert out.returncode == 0 and out.stdout.startswith("ok"), out.stdout + out.stderr


@pytest.mark.gpu
def test_integer_division_and_root_match_the_gpu(tmp_path):
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    exe = str(tmp_path / "xfp64_gpu_check")
    subprocess.run([nvcc, "-gencode", "arch=compute_103a,code=sm_103a", "-O3", "--fmad=false",
                    os.path.join(HERE, "xfp64_gpu_check.cu"), "-o", exe], check=True)
    out = subprocess.run([exe], capture_output=True, text=True, timeout=600)
    assert out.returncode == 0 and out.stdout.startswith("ok"), out.stdout + out.stderr
