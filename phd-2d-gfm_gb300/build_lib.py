"""Build recipe of the native libraries (no cmake, no torch extension).

    libgfm_gb300.so   CUDA kernels + C ABI + host test-case set-up, sm_103a only
    liboracle.so      the CPU oracle (test infrastructure), built beside it
    oracle/_ref/gfm_ref  the reference checker (test infrastructure): the
                      reference's own sources compiled by oracle/build_ref.py,
                      only where those sources are present

Translation units compile in parallel.  The FP64 arithmetic of kernels and
oracle must agree bit for bit, so every compile disables contraction of
multiply-add pairs: --fmad=false for device code, -ffp-contract=off for host
code (gcc contracts by default on aarch64).
"""
import concurrent.futures as cf
import os
import platform
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
MACHINE = platform.machine()   # x86_64 here, aarch64 on the GB300 hosts: separate outputs
LIBDIR = os.path.join(HERE, "lib", MACHINE)
ORACLE = os.path.join(ROOT, "oracle")
ORACLE_LIBDIR = os.path.join(ORACLE, "lib", MACHINE)

CU_SOURCES = ["gfm_flux.cu", "gfm_step.cu", "gfm_api.cu", "gfm_noalloc.cu", "gfm_batch.cu", "gfm_mlp.cu",
              "gfm_output.cu", "gfm_cases_dev.cu"]
CPP_SOURCES = ["gfm_cases.cpp", "gfm_classes.cpp"]
HEADERS = ["gfm_math.cuh", "gfm_xfp64.cuh", "gfm_internal.cuh", "gfm_tables.h", "gfm_mlp.cuh", "gfm_cases.cuh"]

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-std=c++17", "--fmad=false", "-lineinfo", "-Xcompiler", "-fPIC,-ffp-contract=off"]
CXX_FLAGS = ["-O2", "-std=c++17", "-fPIC", "-ffp-contract=off"]


def _nvcc():
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _newer(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps if os.path.exists(d))


def _run(cmd):
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        raise RuntimeError("build step failed: %s\n%s" % (" ".join(cmd), r.stdout))
    return r.stdout


def build_library(verbose=False):
    """Compile libgfm_gb300.so; returns its path."""
    os.makedirs(os.path.join(LIBDIR, "obj"), exist_ok=True)
    out = os.path.join(LIBDIR, "libgfm_gb300.so")
    hdrs = [os.path.join(CSRC, h) for h in HEADERS] + [os.path.join(ROOT, "include", "gfm_gb300.h"),
                                                       os.path.join(ROOT, "include", "gfm_gb300.hpp")]
    nvcc = _nvcc()
    cuda_inc = os.path.join(os.path.dirname(os.path.dirname(os.path.realpath(nvcc))), "include")
    jobs, objs = [], []
    for src in CU_SOURCES + CPP_SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(LIBDIR, "obj", src + ".o")
        objs.append(o)
        if not _newer(o, [s] + hdrs):
            continue
        if src.endswith(".cu"):
            jobs.append([nvcc] + ARCH + NVCC_FLAGS + ["-c", s, "-o", o])
        else:
            jobs.append(["g++"] + CXX_FLAGS + ["-I", cuda_inc, "-c", s, "-o", o])
    with cf.ThreadPoolExecutor(max_workers=max(1, len(jobs))) as ex:
        for log in ex.map(_run, jobs):
            if verbose and log:
                sys.stdout.write(log)
    if _newer(out, objs):
        _run([nvcc] + ARCH + ["-shared", "-o", out] + objs)
    return out


def build_oracle(verbose=False):
    """Compile the CPU oracle (test infrastructure) into oracle/lib/liboracle.so."""
    os.makedirs(ORACLE_LIBDIR, exist_ok=True)
    out = os.path.join(ORACLE_LIBDIR, "liboracle.so")
    srcs = [os.path.join(ORACLE, "gfm_oracle.cpp")]
    deps = srcs + [os.path.join(ORACLE, "oracle_math.hpp"), os.path.join(ORACLE, "oracle_itm.hpp"),
                   os.path.join(CSRC, "gfm_tables.h"),
                   os.path.join(ROOT, "include", "gfm_gb300.h")]
    if _newer(out, deps):
        _run(["g++", "-O3", "-std=c++17", "-fPIC", "-shared", "-ffp-contract=off"] + srcs + ["-o", out])
    return out


def build_reference_checker(verbose=False):
    """oracle/_ref/gfm_ref when the reference's sources are present, else None."""
    if ORACLE not in sys.path:
        sys.path.insert(0, ORACLE)
    import build_ref
    return build_ref.build(verbose)


def build_all(verbose=False):
    lib = build_library(verbose)
    orc = build_oracle(verbose)
    build_reference_checker(verbose)
    return lib, orc


if __name__ == "__main__":
    print(build_all(verbose=True))
