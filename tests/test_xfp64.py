"""The integer-arithmetic IEEE double operations of gfm_xfp64.cuh (xmul,
xadd, xdiv, xsqrt) return exactly the double that the FP64 operation
returns: on the host against the host's own IEEE arithmetic (g++), on the
GPU against its division and square root (nvcc; the device's seeds are the
hardware's approximate reciprocal and reciprocal square root).  The
fixed-point gfm_pow gives the same bits on the device as on the host, is
within 0.51 ulp of x^y (mpmath), and equals the oracle's restatement."""
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


def _pow_check(tmp_path):
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("g++ not available")
    exe = str(tmp_path / "pow_check")
    subprocess.run([gxx, "-O2", "-std=c++17", "-ffp-contract=off", os.path.join(HERE, "pow_check.cpp"), "-o", exe],
                   check=True)
    return exe


def test_fixed_point_pow_matches_the_oracle(tmp_path):
    out = subprocess.run([_pow_check(tmp_path), "3000000"], capture_output=True, text=True, timeout=600)
    assert out.returncode == 0 and out.stdout.startswith("ok"), out.stdout + out.stderr


def test_fixed_point_pow_accuracy(tmp_path):
    """Within 0.51 ulp of x^y evaluated at 40 digits, over the same argument
    families (bases over the whole range, near 1, pressure ratios)."""
    mpmath = pytest.importorskip("mpmath")
    import math
    mpmath.mp.dps = 40
    out = subprocess.run([_pow_check(tmp_path), "12000", "dump"], capture_output=True, text=True, timeout=600)
    assert out.returncode == 0, out.stdout + out.stderr
    worst = 0.0
    n = 0
    for line in out.stdout.split("\n"):
        if not line:
            continue
        x, y, got = (float.fromhex(t) for t in line.split())
        ref = mpmath.power(mpmath.mpf(x), mpmath.mpf(y))
        r = float(ref)
        if r == 0.0 or math.isinf(r) or abs(r) < 2.2250738585072014e-308:
            continue
        worst = max(worst, float(abs(mpmath.mpf(got) - ref) / math.ulp(r)))
        n += 1
    assert n > 11000
    assert worst < 0.51, worst


def test_learned_gate_comparisons_match_the_logarithm(tmp_path):
    """The learned proposal's gate, two comparisons against thresholds, decides
    as |log(ratio)| > 1e-2 did for every ratio checked."""
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("g++ not available")
    exe = str(tmp_path / "gate_check")
    subprocess.run([gxx, "-O2", "-std=c++17", "-ffp-contract=off", os.path.join(HERE, "gate_check.cpp"), "-o", exe],
                   check=True)
    out = subprocess.run([exe], capture_output=True, text=True, timeout=600)
    assert out.returncode == 0 and out.stdout.startswith("ok"), out.stdout + out.stderr


@pytest.mark.gpu
def test_integer_division_and_root_match_the_gpu(tmp_path):
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    exe = str(tmp_path / "xfp64_gpu_check")
    subprocess.run([nvcc, "-gencode", "arch=compute_103a,code=sm_103a", "-O3", "--fmad=false", "-std=c++17",
                    "-Xcompiler", "-ffp-contract=off", os.path.join(HERE, "xfp64_gpu_check.cu"), "-o", exe],
                   check=True)
    out = subprocess.run([exe], capture_output=True, text=True, timeout=600)
    assert out.returncode == 0 and out.stdout.startswith("ok"), out.stdout + out.stderr
