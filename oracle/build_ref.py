"""TEST INFRASTRUCTURE: build recipe of the reference checker, oracle/_ref/gfm_ref.

Compiles murraycutforth/PhD-2D-GFM's own sources, unchanged, from where they
lie (REFERENCE_ROOT: sourcecode/*.cpp with headers/ on the include path),
together with this directory's stand-in headers (ref_shim/) for the libraries
the reference takes from outside its repository (Eigen, blitz++, PhD-Common,
PhD-Interface-tracking-methods, exact_riemann_solver_stiffenedgas), and the
driver ref_driver.cpp.  Outputs go only to oracle/_ref/ (git-ignored).

The stand-ins for the absent libraries are the oracle's own definitions
(oracle_math.hpp, oracle_itm.hpp), so the checker compares the oracle's
restatement of the reference's in-repository code (flux solvers, ghost-fluid
methods, extrapolation, boundary conditions, state algebra, time step and
initial conditions) with that code itself.

Flags follow the reference's Makefile (asserts live: no -DNDEBUG) except
-ffp-contract=off, which keeps a*b+c unfused as on the x86-64 host the
reference was written for (gcc contracts by default on aarch64).
"""
import concurrent.futures as cf
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
REFERENCE_ROOT = os.environ.get("GFM_REFERENCE_ROOT", "/root/reference")
OUT = os.path.join(HERE, "_ref")
BINARY = os.path.join(OUT, "gfm_ref")

# the reference's translation units on the checked path
REF_SOURCES = ["FS_MUSCL", "FS_godunov", "pure_RS_exact", "mixed_RS_exact", "GFM_base", "GFM_original",
               "GFM_riemann", "GFM_real", "GFM_modified", "GFM_VOF", "OGFM_VOF", "extrapolate_vector",
               "extrapolate_extension_vfield", "sim_twofluid", "sim_onefluid"]
FLAGS = ["-O2", "-std=c++17", "-ffp-contract=off", "-g0"]


def available():
    return os.path.isdir(os.path.join(REFERENCE_ROOT, "sourcecode"))


def _run(cmd):
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        raise RuntimeError("build step failed: %s\n%s" % (" ".join(cmd), r.stdout))


def _deps():
    shim = os.path.join(HERE, "ref_shim")
    deps = [os.path.join(HERE, f) for f in ("ref_driver.cpp", "oracle_math.hpp", "oracle_itm.hpp", "build_ref.py")]
    for d, _, files in os.walk(shim):
        deps += [os.path.join(d, f) for f in files]
    deps += [os.path.join(HERE, "..", "phd-2d-gfm_gb300", "csrc", "gfm_tables.h")]
    return deps


def build(verbose=False):
    """Build oracle/_ref/gfm_ref; returns its path, or None without the reference's sources."""
    if not available():
        return None
    os.makedirs(os.path.join(OUT, "obj"), exist_ok=True)
    inc = ["-I", os.path.join(HERE, "ref_shim"), "-I", os.path.join(REFERENCE_ROOT, "headers")]
    deps = _deps()
    newest_dep = max(os.path.getmtime(d) for d in deps if os.path.exists(d))
    jobs, objs = [], []
    for name in REF_SOURCES:
        src = os.path.join(REFERENCE_ROOT, "sourcecode", name + ".cpp")
        obj = os.path.join(OUT, "obj", name + ".o")
        objs.append(obj)
        if not os.path.exists(obj) or os.path.getmtime(obj) < max(newest_dep, os.path.getmtime(src)):
            jobs.append(["g++"] + FLAGS + inc + ["-c", src, "-o", obj])
    drv = os.path.join(OUT, "obj", "ref_driver.o")
    objs.append(drv)
    if not os.path.exists(drv) or os.path.getmtime(drv) < newest_dep:
        jobs.append(["g++"] + FLAGS + inc + ["-c", os.path.join(HERE, "ref_driver.cpp"), "-o", drv])
    with cf.ThreadPoolExecutor(max_workers=max(1, min(8, len(jobs)))) as ex:
        list(ex.map(_run, jobs))
    if jobs or not os.path.exists(BINARY):
        _run(["g++"] + FLAGS + objs + ["-o", BINARY])
    if verbose:
        print(BINARY)
    return BINARY


if __name__ == "__main__":
    p = build(verbose=True)
    if p is None:
        sys.exit("the reference's sources are not at %s" % REFERENCE_ROOT)
