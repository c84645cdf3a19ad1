"""TEST INFRASTRUCTURE: ctypes binding of the CPU oracle (liboracle.so).

Only tests/, __graft_entry__.smoke() and bench.py's cpu_baseline leg may use
this module, and only as the test reference or the timed CPU baseline.

PARITY UNPINNED: the reference cannot be built in this environment and ships
no golden vectors; the oracle restates its code (see gfm_oracle.cpp).
"""
import ctypes
import os
import platform
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
LIB_PATH = os.path.join(HERE, "lib", platform.machine(), "liboracle.so")

sys.path.insert(0, os.path.join(ROOT, "phd-2d-gfm_gb300"))
from gfm_gb300 import GridDesc, MethodDesc  # noqa: E402  (struct layouts of the C ABI)

_lib = None


def lib():
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        sys.path.insert(0, os.path.join(ROOT, "phd-2d-gfm_gb300"))
        import build_lib
        build_lib.build_oracle()
    L = ctypes.CDLL(LIB_PATH)
    pd = ctypes.POINTER(ctypes.c_double)
    D, I = ctypes.c_double, ctypes.c_int
    for name in ("oracle_exp", "oracle_log", "oracle_acos"):
        getattr(L, name).argtypes = [D]
        getattr(L, name).restype = D
    L.oracle_pow.argtypes = [D, D]
    L.oracle_pow.restype = D
    L.oracle_status.restype = ctypes.c_uint32
    L.oracle_newton_iters.restype = ctypes.c_int64
    L.oracle_rs_pure_batch.argtypes = [I, I, D, D, pd, pd, pd]
    L.oracle_rs_mixed_batch.argtypes = [I, D, D, D, D, pd, pd, pd]
    L.oracle_onefluid_run.argtypes = [ctypes.POINTER(GridDesc), ctypes.POINTER(MethodDesc), pd, I, pd,
                                      ctypes.POINTER(I)]
    L.oracle_onefluid_run.restype = I
    L.oracle_twofluid_run.argtypes = [ctypes.POINTER(GridDesc), ctypes.POINTER(MethodDesc), pd, pd, pd, I, pd,
                                      ctypes.POINTER(I), pd, ctypes.POINTER(ctypes.c_int64)]
    L.oracle_twofluid_run.restype = I
    L.oracle_interfacial_mask.argtypes = [ctypes.POINTER(GridDesc), pd, ctypes.POINTER(ctypes.c_uint8)]
    L.oracle_fluid_mass.argtypes = [ctypes.POINTER(GridDesc), D, pd, pd]
    L.oracle_fluid_mass.restype = D
    L.oracle_case_params.argtypes = [ctypes.c_char_p, ctypes.c_char_p, I, I, ctypes.POINTER(GridDesc), pd]
    L.oracle_case_init.argtypes = [ctypes.c_char_p, ctypes.c_char_p, ctypes.POINTER(GridDesc), pd, pd, pd]
    L.oracle_bubble_case.argtypes = [D, D, D, D, I, I, ctypes.POINTER(GridDesc), pd]
    L.oracle_bubble_init.argtypes = [D, D, D, D, ctypes.POINTER(GridDesc), pd, pd, pd]
    _lib = L
    return L


def _p(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def rs_pure(paralleltox, gamma, pinf, UL, UR):
    UL = np.ascontiguousarray(UL, dtype=np.float64)
    UR = np.ascontiguousarray(UR, dtype=np.float64)
    out = np.zeros_like(UL)
    lib().oracle_rs_pure_batch(len(UL), int(paralleltox), gamma, pinf, _p(UL), _p(UR), _p(out))
    return out


def rs_mixed(gL, pinfL, gR, pinfR, UL, UR):
    UL = np.ascontiguousarray(UL, dtype=np.float64)
    UR = np.ascontiguousarray(UR, dtype=np.float64)
    out = np.zeros_like(UL)
    lib().oracle_rs_mixed_batch(len(UL), gL, pinfL, gR, pinfR, _p(UL), _p(UR), _p(out))
    return out


def onefluid_run(desc, m, U, nsteps, t=0.0, numsteps=0):
    U = np.ascontiguousarray(U, dtype=np.float64).copy()
    tt = ctypes.c_double(t)
    ns = ctypes.c_int(numsteps)
    taken = lib().oracle_onefluid_run(ctypes.byref(desc), ctypes.byref(m), _p(U), nsteps, ctypes.byref(tt),
                                      ctypes.byref(ns))
    return U, tt.value, ns.value, taken


def twofluid_run(desc, m, U1, U2, phi, nsteps, t=0.0, numsteps=0):
    U1 = np.ascontiguousarray(U1, dtype=np.float64).copy()
    U2 = np.ascontiguousarray(U2, dtype=np.float64).copy()
    phi = np.ascontiguousarray(phi, dtype=np.float64).copy()
    vel = np.zeros((2,) + phi.shape)
    tt = ctypes.c_double(t)
    ns = ctypes.c_int(numsteps)
    nifc = ctypes.c_int64(0)
    taken = lib().oracle_twofluid_run(ctypes.byref(desc), ctypes.byref(m), _p(U1), _p(U2), _p(phi), nsteps,
                                      ctypes.byref(tt), ctypes.byref(ns), _p(vel), ctypes.byref(nifc))
    return {"U1": U1, "U2": U2, "phi": phi, "vel": vel, "t": tt.value, "numsteps": ns.value, "taken": taken,
            "n_interfacial": nifc.value}


def case_setup(sim_type, test_case, Nx, Ny):
    """(desc, T, U1, U2, phi) of a timed workload from the oracle's own
    restatement of its initial conditions (U2, phi None for one fluid)."""
    desc = GridDesc()
    T = ctypes.c_double()
    if lib().oracle_case_params(sim_type.encode(), test_case.encode(), Nx, Ny, ctypes.byref(desc), ctypes.byref(T)):
        raise ValueError("no oracle initial condition for %s %s" % (sim_type, test_case))
    nr, nc = desc.Ny + 2 * desc.numGC, desc.Nx + 2 * desc.numGC
    U1 = np.zeros((4, nr, nc))
    if sim_type == "onefluid":
        lib().oracle_case_init(sim_type.encode(), test_case.encode(), ctypes.byref(desc), _p(U1), None, None)
        return desc, T.value, U1, None, None
    U2 = np.zeros((4, nr, nc))
    phi = np.zeros((nr, nc))
    lib().oracle_case_init(sim_type.encode(), test_case.encode(), ctypes.byref(desc), _p(U1), _p(U2), _p(phi))
    return desc, T.value, U1, U2, phi


def bubble_setup(Nx, Ny, mach, gamma_bubble, rho_ratio, radius_frac):
    """(desc, T, U1, U2, phi) of a member of the batched shock-bubble family."""
    desc = GridDesc()
    T = ctypes.c_double()
    lib().oracle_bubble_case(mach, gamma_bubble, rho_ratio, radius_frac, Nx, Ny, ctypes.byref(desc), ctypes.byref(T))
    nr, nc = desc.Ny + 2 * desc.numGC, desc.Nx + 2 * desc.numGC
    U1, U2, phi = np.zeros((4, nr, nc)), np.zeros((4, nr, nc)), np.zeros((nr, nc))
    lib().oracle_bubble_init(mach, gamma_bubble, rho_ratio, radius_frac, ctypes.byref(desc), _p(U1), _p(U2), _p(phi))
    return desc, T.value, U1, U2, phi


def fluid_mass(desc, interiorsign, U, phi):
    """sim_twofluid::fluid_mass: sum of rho dx dy over real cells with interiorsign * phi > 0."""
    U = np.ascontiguousarray(U, dtype=np.float64)
    phi = np.ascontiguousarray(phi, dtype=np.float64)
    return lib().oracle_fluid_mass(ctypes.byref(desc), interiorsign, _p(U), _p(phi))


def interfacial_mask(desc, phi):
    phi = np.ascontiguousarray(phi, dtype=np.float64)
    mask = np.zeros(phi.shape, dtype=np.uint8)
    lib().oracle_interfacial_mask(ctypes.byref(desc), _p(phi), mask.ctypes.data_as(ctypes.POINTER(ctypes.c_uint8)))
    return mask


def last_realcells():
    """realcells1 and realcells2 of the last two-fluid step, each (imin, imax, jmin, jmax)."""
    rc = (ctypes.c_int * 8)()
    lib().oracle_last_realcells(rc)
    return tuple(rc[:4]), tuple(rc[4:])


def status():
    return lib().oracle_status()


def clear_status():
    lib().oracle_clear_status()


def newton_iters():
    return lib().oracle_newton_iters()


def mixed_stats():
    """(calls, Newton iterations) of the mixed Riemann solves since the last clear."""
    a, b = ctypes.c_int64(), ctypes.c_int64()
    lib().oracle_mixed_stats(ctypes.byref(a), ctypes.byref(b))
    return a.value, b.value


def iter_histogram():
    """Riemann solves (pure and mixed) by Newton iteration count since the last
    clear; entry 15 counts 15 or more."""
    h = np.zeros(16, dtype=np.int64)
    lib().oracle_iter_histogram(h.ctypes.data_as(ctypes.POINTER(ctypes.c_int64)))
    return h
