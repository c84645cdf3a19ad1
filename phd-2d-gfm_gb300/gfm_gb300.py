"""Python host side of the GB300 two-fluid ghost-fluid Euler step.

A thin ctypes layer over the C ABI in include/gfm_gb300.h (libgfm_gb300.so),
mirroring the reference's host objects:

    GFM_settingsfile   headers/GFM_settingsfile.hpp:9-60 (same keys, plus
                       nsteps / reinit_every / reinit_iters / ls_order)
    sim_onefluid       sourcecode/sim_onefluid.cpp:12-64  (run_sim)
    sim_twofluid       sourcecode/sim_twofluid.cpp:27-103 (run_sim)
    Context            the device-resident grids behind both

The library is the only compute path: if libgfm_gb300.so cannot be loaded,
every entry point raises.  There is no CPU fallback.
"""
import ctypes
import os
import platform

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "lib", platform.machine(), "libgfm_gb300.so")

BC = {"transmissive": 0, "reflective": 1, "periodic": 2}
FS = {"Godunov": 0, "MUSCL": 1}
GFM = {"OGFM": 0, "riemannGFM": 1, "realGFM": 2, "MGFM": 3, "VOFGFM": 4, "OGFMVOF": 5}
# interface trackers: (advection order, reinitialise every k steps, tracker kind)
ITM = {"LS1": (1, 1, 0), "LS5": (5, 1, 0), "PYVOF": (0, 0, 1)}
ITM_LEVELSET, ITM_VOF = 0, 1

ST_BITS = {
    1 << 0: "UNPHYSICAL_STATE",
    1 << 1: "NEWTON_NO_CONVERGE",
    1 << 2: "VACUUM",
    1 << 3: "NAN_DETECTED",
    1 << 4: "DT_NONPOSITIVE",
    1 << 5: "SCHEDULE_LIMIT",
}


class GridDesc(ctypes.Structure):
    """sim_info + binarySGparams (gfm_grid_desc)."""
    _fields_ = [("Nx", ctypes.c_int), ("Ny", ctypes.c_int), ("numGC", ctypes.c_int),
                ("x0", ctypes.c_double), ("y0", ctypes.c_double), ("dx", ctypes.c_double), ("dy", ctypes.c_double),
                ("BC_L", ctypes.c_int), ("BC_R", ctypes.c_int), ("BC_B", ctypes.c_int), ("BC_T", ctypes.c_int),
                ("gamma1", ctypes.c_double), ("pinf1", ctypes.c_double),
                ("gamma2", ctypes.c_double), ("pinf2", ctypes.c_double)]

    @property
    def shape(self):
        return (self.Ny + 2 * self.numGC, self.Nx + 2 * self.numGC)


class MethodDesc(ctypes.Structure):
    """Strategy choices of set_sim_methods (gfm_method_desc)."""
    _fields_ = [("fs", ctypes.c_int), ("gfm", ctypes.c_int), ("ls_order", ctypes.c_int),
                ("reinit_every", ctypes.c_int), ("reinit_iters", ctypes.c_int),
                ("use_extension_vfield", ctypes.c_int), ("use_slip_BCs", ctypes.c_int),
                ("CFL", ctypes.c_double), ("T", ctypes.c_double), ("itm", ctypes.c_int)]


class GFMError(RuntimeError):
    pass


_lib = None


def lib():
    """Load libgfm_gb300.so once (raises if it is missing: no fallback)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise GFMError("libgfm_gb300.so is not built (run __graft_entry__.build())")
    L = ctypes.CDLL(LIB_PATH)
    P, I, D, V = ctypes.c_void_p, ctypes.c_int, ctypes.c_double, ctypes.c_void_p
    pd = ctypes.POINTER(ctypes.c_double)
    sig = {
        "gfm_ctx_create": [ctypes.POINTER(GridDesc), I, ctypes.POINTER(P)],
        "gfm_ctx_destroy": [P],
        "gfm_set_stream": [P, V],
        "gfm_upload": [P, I, pd], "gfm_download": [P, I, pd],
        "gfm_upload_phi": [P, pd], "gfm_download_phi": [P, pd], "gfm_download_velocity": [P, pd],
        "gfm_upload_state": [P, pd, pd, pd], "gfm_download_state": [P, pd, pd, pd],
        "gfm_upload_state_async": [P, pd, pd, pd],
        "gfm_set_time": [P, D, I],
        "gfm_download_mask": [P, ctypes.POINTER(ctypes.c_uint8)],
        "gfm_get_time": [P, pd, ctypes.POINTER(I), pd],
        "gfm_get_realcells": [P, ctypes.POINTER(I)],
        "gfm_compute_dt": [P, D, D],
        "gfm_set_ghost_states": [P, ctypes.POINTER(MethodDesc)],
        "gfm_fs_update": [P, I, I],
        "gfm_ls_update": [P, ctypes.POINTER(MethodDesc)],
        "gfm_apply_bcs": [P, I], "gfm_set_interface_tracker": [P, I],
        "gfm_step": [P, ctypes.POINTER(MethodDesc), I],
        "gfm_step_timed": [P, ctypes.POINTER(MethodDesc), I, pd],
        "gfm_set_overlap": [P, I],
        "gfm_set_flux_tile": [P, I],
        "gfm_batch_set_schedule": [P, I],
        "gfm_batch_autotune": [P, ctypes.POINTER(MethodDesc), I, ctypes.c_char_p, I],
        "gfm_set_newton_limit": [P, I],
        "gfm_set_interface_wait": [P, ctypes.c_int64, I],
        "gfm_fp64_peak": [pd, V],
        "gfm_batch_create": [ctypes.POINTER(GridDesc), I, I, ctypes.POINTER(P)],
        "gfm_batch_destroy": [P], "gfm_batch_instance": [P, I, ctypes.POINTER(P)],
        "gfm_batch_set_stream": [P, V], "gfm_batch_synchronize": [P],
        "gfm_step_batched_graph": [P, ctypes.POINTER(MethodDesc), I],
        "gfm_step_batched_sequential": [P, ctypes.POINTER(MethodDesc), I],
        "gfm_case_shock_bubble": [V, I, I, ctypes.POINTER(GridDesc), pd],
        "gfm_mlp_create": [ctypes.c_uint64, ctypes.POINTER(P)], "gfm_mlp_destroy": [P],
        "gfm_mlp_set_params": [P, V], "gfm_mlp_get_params": [P, V],
        "gfm_mlp_generate": [ctypes.c_uint64, I, V, V, ctypes.POINTER(I), V],
        "gfm_mlp_gradient": [P, V, V, I, V, ctypes.POINTER(ctypes.c_float), V],
        "gfm_mlp_train": [P, V, V, I, I, I, ctypes.c_float, ctypes.c_uint64, V, V],
        "gfm_mlp_infer": [P, V, I, V, I, V],
        "gfm_rs_mixed_batch_learned": [P, I, D, D, D, D, V, V, V, V, V, I, V],
        "gfm_set_mlp": [P, P],
        "gfm_capture_interface_problems": [P, V, V, I, V],
        "gfm_get_interface_stats": [P, ctypes.POINTER(ctypes.c_int64), ctypes.POINTER(ctypes.c_int64),
                                    ctypes.POINTER(ctypes.c_int64)],
        "gfm_get_interface_totals": [P, ctypes.POINTER(ctypes.c_int64), ctypes.POINTER(ctypes.c_int64),
                                     ctypes.POINTER(ctypes.c_int64)],
        "gfm_case_init_shock_bubble": [V, ctypes.POINTER(GridDesc), pd, pd, pd],
        "gfm_get_device_status": [P, ctypes.POINTER(ctypes.c_uint32)],
        "gfm_clear_device_status": [P],
        "gfm_get_stats": [P, ctypes.POINTER(ctypes.c_int64)] * 1 + [ctypes.POINTER(ctypes.c_int64)] * 2,
        "gfm_fluid_mass": [P, D, pd],
        "gfm_rs_pure_batch": [I, I, D, D, V, V, V, V, V],
        "gfm_rs_mixed_batch": [I, D, D, D, D, V, V, V, V, V],
        "gfm_case_params": [ctypes.c_char_p, ctypes.c_char_p, I, I, ctypes.POINTER(GridDesc), pd],
        "gfm_case_init": [ctypes.c_char_p, ctypes.c_char_p, ctypes.POINTER(GridDesc), pd, pd, pd],
        "gfm_case_init_z": [ctypes.c_char_p, ctypes.POINTER(GridDesc), pd],
        "gfm_case_init_shock_bubble_z": [V, ctypes.POINTER(GridDesc), pd],
        "gfm_case_init_device": [P, ctypes.c_char_p, ctypes.c_char_p, I],
        "gfm_case_init_shock_bubble_device": [P, V, I],
        "gfm_write_output_files": [ctypes.POINTER(GridDesc), ctypes.c_char_p, I, I, I, pd, pd, pd, pd],
        "gfm_run_sim": [P, ctypes.POINTER(MethodDesc), ctypes.POINTER(GridDesc), ctypes.c_char_p, I, I, pd],
        "gfm_checkpoint_save": [P, ctypes.c_char_p], "gfm_checkpoint_load": [P, ctypes.c_char_p],
        "gfm_checkpoint_write": [ctypes.c_char_p, ctypes.POINTER(GridDesc), I, D, I, pd, pd, pd],
        "gfm_checkpoint_read": [ctypes.c_char_p, ctypes.POINTER(GridDesc), ctypes.POINTER(I), pd, ctypes.POINTER(I),
                                pd, pd, pd],
    }
    for name, args in sig.items():
        f = getattr(L, name)
        f.argtypes = args
        f.restype = ctypes.c_int
    L.gfm_version.restype = ctypes.c_char_p
    L.gfm_version.argtypes = []
    L.gfm_launch_count.restype = ctypes.c_int64
    L.gfm_launch_count.argtypes = []
    L.gfm_mlp_param_count.restype = ctypes.c_int
    L.gfm_mlp_param_count.argtypes = []
    _lib = L
    return L


def _check(rc, what):
    if rc != 0:
        raise GFMError("%s failed with gfm_status_t %d" % (what, rc))


def _dptr(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def status_names(bits):
    return [n for b, n in ST_BITS.items() if bits & b]


# ---------------------------------------------------------------------------
# test cases (set_sim_parameters + set_sim_ICs)
# ---------------------------------------------------------------------------
def case_params(sim_type, test_case, Nx, Ny):
    """Returns (GridDesc, T) of a named test case."""
    d = GridDesc()
    T = ctypes.c_double(0.0)
    _check(lib().gfm_case_params(sim_type.encode(), test_case.encode(), Nx, Ny, ctypes.byref(d), ctypes.byref(T)),
           "gfm_case_params(%s, %s)" % (sim_type, test_case))
    return d, T.value


def case_init(sim_type, test_case, desc):
    """Initial conditions as host arrays: U1 (4,nr,nc), U2 (4,nr,nc) or None, phi (nr,nc) or None."""
    nr, nc = desc.shape
    two = sim_type == "twofluid"
    U1 = np.zeros((4, nr, nc))
    U2 = np.zeros((4, nr, nc)) if two else None
    phi = np.zeros((nr, nc)) if two else None
    _check(lib().gfm_case_init(sim_type.encode(), test_case.encode(), ctypes.byref(desc), _dptr(U1),
                               _dptr(U2) if two else None, _dptr(phi) if two else None),
           "gfm_case_init(%s, %s)" % (sim_type, test_case))
    return U1, U2, phi


def case_init_z(test_case, desc):
    """Volume fraction of fluid 1 (nr, nc) of a two-fluid case: the initial
    interface field of the VOF tracker (itm "PYVOF")."""
    nr, nc = desc.shape
    z = np.zeros((nr, nc))
    _check(lib().gfm_case_init_z(test_case.encode(), ctypes.byref(desc), _dptr(z)),
           "gfm_case_init_z(%s)" % test_case)
    return z


def method(fs="MUSCL", gfm="riemannGFM", itm="LS5", CFL=0.6, T=1.0, reinit_every=None, reinit_iters=5,
           use_extension_vfield=False, use_slip_BCs=False):
    order, every, kind = ITM[itm]
    m = MethodDesc()
    m.itm = kind
    m.fs = FS[fs]
    m.gfm = GFM[gfm]
    m.ls_order = order
    m.reinit_every = every if reinit_every is None else reinit_every
    m.reinit_iters = reinit_iters
    m.use_extension_vfield = int(bool(use_extension_vfield))
    m.use_slip_BCs = int(bool(use_slip_BCs))
    m.CFL = CFL
    m.T = T
    return m


# ---------------------------------------------------------------------------
# device context
# ---------------------------------------------------------------------------
class Context:
    """Device-resident grids of one instance (gfm_ctx)."""

    def __init__(self, desc, two_fluid=True, stream=None, _borrowed=None):
        self.desc = desc
        self.two_fluid = bool(two_fluid)
        self._owned = _borrowed is None
        if _borrowed is not None:   # an instance of a Batch: the batch owns it
            self._p = _borrowed
            return
        self._p = ctypes.c_void_p()
        _check(lib().gfm_ctx_create(ctypes.byref(desc), int(self.two_fluid), ctypes.byref(self._p)),
               "gfm_ctx_create")
        if stream is not None:
            _check(lib().gfm_set_stream(self._p, ctypes.c_void_p(stream)), "gfm_set_stream")

    def close(self):
        if self._p and self._owned:
            lib().gfm_ctx_destroy(self._p)
        self._p = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_stream(self, stream):
        _check(lib().gfm_set_stream(self._p, ctypes.c_void_p(stream)), "gfm_set_stream")

    def upload(self, U1, U2=None, phi=None, t=0.0, numsteps=0):
        U1 = np.ascontiguousarray(U1, dtype=np.float64)
        _check(lib().gfm_upload(self._p, 1, _dptr(U1)), "gfm_upload(1)")
        if self.two_fluid:
            U2 = np.ascontiguousarray(U2, dtype=np.float64)
            phi = np.ascontiguousarray(phi, dtype=np.float64)
            _check(lib().gfm_upload(self._p, 2, _dptr(U2)), "gfm_upload(2)")
            _check(lib().gfm_upload_phi(self._p, _dptr(phi)), "gfm_upload_phi")
        _check(lib().gfm_set_time(self._p, t, numsteps), "gfm_set_time")

    def download(self):
        nr, nc = self.desc.shape
        U1 = np.empty((4, nr, nc))
        _check(lib().gfm_download(self._p, 1, _dptr(U1)), "gfm_download(1)")
        if not self.two_fluid:
            return U1, None, None
        U2 = np.empty((4, nr, nc))
        phi = np.empty((nr, nc))
        _check(lib().gfm_download(self._p, 2, _dptr(U2)), "gfm_download(2)")
        _check(lib().gfm_download_phi(self._p, _dptr(phi)), "gfm_download_phi")
        return U1, U2, phi

    def mask(self):
        nr, nc = self.desc.shape
        out = np.zeros((nr, nc), dtype=np.uint8)
        _check(lib().gfm_download_mask(self._p, out.ctypes.data_as(ctypes.POINTER(ctypes.c_uint8))),
               "gfm_download_mask")
        return out

    def step(self, m, nsteps=1):
        _check(lib().gfm_step(self._p, ctypes.byref(m), nsteps), "gfm_step")

    def time(self):
        t = ctypes.c_double()
        n = ctypes.c_int()
        dt = ctypes.c_double()
        _check(lib().gfm_get_time(self._p, ctypes.byref(t), ctypes.byref(n), ctypes.byref(dt)), "gfm_get_time")
        return t.value, n.value, dt.value

    def realcells(self):
        """(realcells1, realcells2) of the last step, each (imin, imax, jmin, jmax)."""
        rc = (ctypes.c_int * 8)()
        _check(lib().gfm_get_realcells(self._p, rc), "gfm_get_realcells")
        return tuple(rc[:4]), tuple(rc[4:])

    def status(self):
        s = ctypes.c_uint32()
        _check(lib().gfm_get_device_status(self._p, ctypes.byref(s)), "gfm_get_device_status")
        return s.value

    def clear_status(self):
        _check(lib().gfm_clear_device_status(self._p), "gfm_clear_device_status")

    def init_device(self, sim_type, test_case, itm="LS5"):
        """The named case's initial state generated on the device (gfm_case_init_device)."""
        _check(lib().gfm_case_init_device(self._p, sim_type.encode(), test_case.encode(), ITM[itm][2]),
               "gfm_case_init_device")

    def init_shock_bubble_device(self, params, itm="LS5"):
        """A shock-bubble family member generated on the device."""
        _check(lib().gfm_case_init_shock_bubble_device(self._p, ctypes.byref(params), ITM[itm][2]),
               "gfm_case_init_shock_bubble_device")

    def save_checkpoint(self, path):
        """gfm_checkpoint_save: grids, interface field, t and step count."""
        _check(lib().gfm_checkpoint_save(self._p, str(path).encode()), "gfm_checkpoint_save")

    def load_checkpoint(self, path):
        """gfm_checkpoint_load: the state of a checkpoint of the same grid."""
        _check(lib().gfm_checkpoint_load(self._p, str(path).encode()), "gfm_checkpoint_load")

    def velocity(self):
        """The velocity field (2, nr, nc) of the last ghost fill."""
        nr, nc = self.desc.shape
        vel = np.empty((2, nr, nc))
        _check(lib().gfm_download_velocity(self._p, _dptr(vel)), "gfm_download_velocity")
        return vel

    def stats(self):
        a, b, c = ctypes.c_int64(), ctypes.c_int64(), ctypes.c_int64()
        _check(lib().gfm_get_stats(self._p, ctypes.byref(a), ctypes.byref(b), ctypes.byref(c)), "gfm_get_stats")
        return {"n_interfacial": a.value, "rounds": b.value, "newton_iters": c.value}

    def set_overlap(self, mode):
        """Ghost-fill schedule of the Riemann / real GFM: False or "off",
        True or "on" (interface loop on its own SM partition), "auto" (the
        default: on for the Riemann GFM only).  Returns False when the context
        has no partitions to turn it on."""
        code = {False: 0, "off": 0, True: 1, "on": 1, "auto": 2}[mode]
        rc = lib().gfm_set_overlap(self._p, code)
        if rc == 4:
            return False
        _check(rc, "gfm_set_overlap")
        return True

    def set_flux_tile(self, shape):
        """Tile shape of the flux update: "16x32" (default), "16x16", "32x8" or "64x4"
        (results are identical)."""
        code = {"32x8": 0, "16x16": 1, "64x4": 2, "16x32": 3}[shape]
        _check(lib().gfm_set_flux_tile(self._p, code), "gfm_set_flux_tile")

    def set_newton_limit(self, max_iterations):
        """Newton iteration limit of the exact Riemann solves (default 60);
        a solve that reaches it sets GFM_ST_NEWTON_NO_CONVERGE."""
        _check(lib().gfm_set_newton_limit(self._p, int(max_iterations)), "gfm_set_newton_limit")

    def set_interface_wait(self, spin_limit=0, withheld_entry=-1):
        """Polls before an interface-loop wait gives up (0: default), and the
        failure-detection test hook: an interface-list entry left unsolved."""
        _check(lib().gfm_set_interface_wait(self._p, int(spin_limit), int(withheld_entry)),
               "gfm_set_interface_wait")

    def step_timed(self, m, nsteps=1):
        """gfm_step with per-phase device times; returns GFM_NPHASES (9)
        milliseconds summed over the steps."""
        ph = np.zeros(9)
        _check(lib().gfm_step_timed(self._p, ctypes.byref(m), nsteps, _dptr(ph)), "gfm_step_timed")
        return ph

    def set_mlp(self, mlp):
        """Start the interface solves from a learned proposal (an MLP), or
        from the two-shock guess again (None)."""
        _check(lib().gfm_set_mlp(self._p, mlp._p if mlp is not None else None), "gfm_set_mlp")

    def capture_interface_problems(self, X_ptr, Y_ptr, cap, count_ptr):
        """Append each step's gated interface problems (features, exact target)
        to device arrays; X_ptr None stops."""
        _check(lib().gfm_capture_interface_problems(self._p, ctypes.c_void_p(X_ptr), ctypes.c_void_p(Y_ptr), cap,
                                                    ctypes.c_void_p(count_ptr)), "gfm_capture_interface_problems")

    def interface_stats(self):
        a, b, c = ctypes.c_int64(), ctypes.c_int64(), ctypes.c_int64()
        _check(lib().gfm_get_interface_stats(self._p, ctypes.byref(a), ctypes.byref(b), ctypes.byref(c)),
               "gfm_get_interface_stats")
        return {"solves": a.value, "newton_iters": b.value, "proposed": c.value}

    def interface_totals(self):
        """Interface solves, their Newton iterations and the solves started
        from the learned proposal, summed since the last upload / set_time."""
        a, b, c = ctypes.c_int64(), ctypes.c_int64(), ctypes.c_int64()
        _check(lib().gfm_get_interface_totals(self._p, ctypes.byref(a), ctypes.byref(b), ctypes.byref(c)),
               "gfm_get_interface_totals")
        return {"solves": a.value, "newton_iters": b.value, "proposed": c.value}

    def fluid_mass(self, interiorsign):
        m = ctypes.c_double()
        _check(lib().gfm_fluid_mass(self._p, interiorsign, ctypes.byref(m)), "gfm_fluid_mass")
        return m.value


# ---------------------------------------------------------------------------
# batches of instances
# ---------------------------------------------------------------------------
class Batch:
    """Many independent instances stepped together (gfm_batch): `instances`
    are Contexts (upload, download, time, status) owned by the batch."""

    def __init__(self, descs, two_fluid=True, stream=None):
        descs = list(descs)
        arr = (GridDesc * len(descs))(*descs)
        self._p = ctypes.c_void_p()
        _check(lib().gfm_batch_create(arr, len(descs), int(bool(two_fluid)), ctypes.byref(self._p)),
               "gfm_batch_create")
        self.instances = []
        for i, d in enumerate(descs):
            c = ctypes.c_void_p()
            _check(lib().gfm_batch_instance(self._p, i, ctypes.byref(c)), "gfm_batch_instance")
            self.instances.append(Context(d, two_fluid, _borrowed=c))
        if stream is not None:
            _check(lib().gfm_batch_set_stream(self._p, ctypes.c_void_p(stream)), "gfm_batch_set_stream")

    def step(self, m, nsteps=1, graph=True):
        """nsteps steps of every instance: recorded CUDA graph with the
        instances side by side (graph=True), or one instance after another."""
        f = lib().gfm_step_batched_graph if graph else lib().gfm_step_batched_sequential
        _check(f(self._p, ctypes.byref(m), nsteps), "gfm_step_batched_%s" % ("graph" if graph else "sequential"))

    def synchronize(self):
        _check(lib().gfm_batch_synchronize(self._p), "gfm_batch_synchronize")

    def set_schedule(self, schedule):
        """"streams" (each instance's step on its own stream, the default) or
        "phased" (one persistent flux launch over all instances per step)."""
        _check(lib().gfm_batch_set_schedule(self._p, {"streams": 0, "phased": 1}[schedule]),
               "gfm_batch_set_schedule")

    def autotune(self, m, steps=16):
        """Times the flux tile shapes per grid-size class and the two
        schedules on the batch's current state (restored afterwards), keeps
        the fastest; returns the report."""
        import json
        buf = ctypes.create_string_buffer(4096)
        _check(lib().gfm_batch_autotune(self._p, ctypes.byref(m), int(steps), buf, len(buf)), "gfm_batch_autotune")
        return json.loads(buf.value.decode())

    def close(self):
        for c in getattr(self, "instances", []):
            c._p = ctypes.c_void_p()
        if self._p:
            lib().gfm_batch_destroy(self._p)
            self._p = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class BubbleParams(ctypes.Structure):
    _fields_ = [("mach", ctypes.c_double), ("gamma_bubble", ctypes.c_double), ("rho_ratio", ctypes.c_double),
                ("radius_frac", ctypes.c_double)]


def shock_bubble_case(Nx, Ny, mach, gamma_bubble, rho_ratio, radius_frac):
    """Grid, T and initial state of one member of the shock-bubble family
    (gfm_case_shock_bubble / gfm_case_init_shock_bubble)."""
    p = BubbleParams(mach, gamma_bubble, rho_ratio, radius_frac)
    d = GridDesc()
    T = ctypes.c_double(0.0)
    _check(lib().gfm_case_shock_bubble(ctypes.byref(p), Nx, Ny, ctypes.byref(d), ctypes.byref(T)),
           "gfm_case_shock_bubble")
    nr, nc = d.shape
    U1, U2, phi = np.empty((4, nr, nc)), np.empty((4, nr, nc)), np.empty((nr, nc))
    _check(lib().gfm_case_init_shock_bubble(ctypes.byref(p), ctypes.byref(d), _dptr(U1), _dptr(U2), _dptr(phi)),
           "gfm_case_init_shock_bubble")
    return d, T.value, U1, U2, phi


def shock_bubble_case_z(d, mach, gamma_bubble, rho_ratio, radius_frac):
    """The family member's volume fraction of fluid 1 (gfm_case_init_shock_bubble_z)."""
    p = BubbleParams(mach, gamma_bubble, rho_ratio, radius_frac)
    nr, nc = d.shape
    z = np.empty((nr, nc))
    _check(lib().gfm_case_init_shock_bubble_z(ctypes.byref(p), ctypes.byref(d), _dptr(z)),
           "gfm_case_init_shock_bubble_z")
    return z


# ---------------------------------------------------------------------------
# learned star-pressure proposal
# ---------------------------------------------------------------------------
class MLP:
    """The learned proposal (gfm_mlp).  Device arrays are passed as raw
    pointers (e.g. torch tensors' data_ptr())."""

    NPARAM = 9089

    def __init__(self, seed=1):
        self._p = ctypes.c_void_p()
        _check(lib().gfm_mlp_create(seed, ctypes.byref(self._p)), "gfm_mlp_create")

    def params(self):
        out = np.empty(self.NPARAM, dtype=np.float32)
        _check(lib().gfm_mlp_get_params(self._p, out.ctypes.data_as(ctypes.c_void_p)), "gfm_mlp_get_params")
        return out

    def set_params(self, p):
        p = np.ascontiguousarray(p, dtype=np.float32)
        _check(lib().gfm_mlp_set_params(self._p, p.ctypes.data_as(ctypes.c_void_p)), "gfm_mlp_set_params")

    def gradient(self, X_ptr, Y_ptr, n, stream=0):
        g = np.empty(self.NPARAM, dtype=np.float32)
        loss = ctypes.c_float()
        _check(lib().gfm_mlp_gradient(self._p, ctypes.c_void_p(X_ptr), ctypes.c_void_p(Y_ptr), n,
                                      g.ctypes.data_as(ctypes.c_void_p), ctypes.byref(loss), ctypes.c_void_p(stream)),
               "gfm_mlp_gradient")
        return g, loss.value

    def train(self, X_ptr, Y_ptr, n, epochs, batch=8192, lr=2e-3, seed=7, stream=0):
        losses = np.zeros(epochs, dtype=np.float32)
        _check(lib().gfm_mlp_train(self._p, ctypes.c_void_p(X_ptr), ctypes.c_void_p(Y_ptr), n, epochs, batch, lr, seed,
                                   losses.ctypes.data_as(ctypes.c_void_p), ctypes.c_void_p(stream)), "gfm_mlp_train")
        return losses

    def infer(self, X_ptr, n, out_ptr, tensor_cores=True, stream=0):
        _check(lib().gfm_mlp_infer(self._p, ctypes.c_void_p(X_ptr), n, ctypes.c_void_p(out_ptr), int(tensor_cores),
                                   ctypes.c_void_p(stream)), "gfm_mlp_infer")

    def rs_mixed(self, gL, pinfL, gR, pinfR, UL_ptr, UR_ptr, n, out_ptr, iters_ptr, status_ptr, use_net=True,
                 stream=0):
        _check(lib().gfm_rs_mixed_batch_learned(self._p, n, gL, pinfL, gR, pinfR, ctypes.c_void_p(UL_ptr),
                                                ctypes.c_void_p(UR_ptr), ctypes.c_void_p(out_ptr),
                                                ctypes.c_void_p(iters_ptr), ctypes.c_void_p(status_ptr), int(use_net),
                                                ctypes.c_void_p(stream)), "gfm_rs_mixed_batch_learned")

    def close(self):
        if self._p:
            lib().gfm_mlp_destroy(self._p)
            self._p = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def mlp_generate(seed, n, X_ptr, Y_ptr, stream=0):
    """n training problems into device arrays X (n x 10 float) and Y (n)."""
    got = ctypes.c_int(0)
    _check(lib().gfm_mlp_generate(seed, n, ctypes.c_void_p(X_ptr), ctypes.c_void_p(Y_ptr), ctypes.byref(got),
                                  ctypes.c_void_p(stream)), "gfm_mlp_generate")
    return got.value


# ---------------------------------------------------------------------------
# GFM_settingsfile and the simulation drivers
# ---------------------------------------------------------------------------
class GFM_settingsfile:
    """Whitespace 'key value' lines; unknown keys are ignored (headers/GFM_settingsfile.hpp:24-59)."""

    def __init__(self):
        self.Nx = 0
        self.Ny = 0
        self.CFL = 0.0
        self.sim_type = ""
        self.FS = ""
        self.ITM = ""
        self.GFM = ""
        self.test_case = ""
        self.outputpath = ""
        self.basename = ""
        self.nsteps = 0          # 0: run to the test case's end time T
        self.reinit_every = None
        self.reinit_iters = 5

    def read_settings_file(self, filename):
        conv = {"Nx": int, "Ny": int, "CFL": float, "nsteps": int, "reinit_every": int, "reinit_iters": int}
        with open(filename) as f:
            for line in f:
                parts = line.split()
                if not parts:
                    continue
                key = parts[0]
                if len(parts) < 2:
                    continue
                if key in ("Nx", "Ny", "CFL", "sim_type", "FS", "test_case", "ITM", "GFM", "outputpath", "nsteps",
                           "reinit_every", "reinit_iters"):
                    setattr(self, key, conv.get(key, str)(parts[1]))
        if self.sim_type == "onefluid":
            self.basename = "%s%s-%s-%s-%d-%d" % (self.outputpath, self.sim_type, self.test_case, self.FS, self.Nx,
                                                 self.Ny)
        else:
            self.basename = "%s%s-%s-%s-%s-%d-%d" % (self.outputpath, self.GFM, self.ITM, self.test_case, self.FS,
                                                    self.Nx, self.Ny)
        return self


# params.output_freq of set_sim_parameters (sourcecode/sim_twofluid.cpp:347,392,404;
# sourcecode/sim_onefluid.cpp:102)
OUTPUT_FREQ_TWOFLUID = {"GDA": 0, "shocked_helium_bubble": 2}
OUTPUT_FREQ_ONEFLUID = 10 ** 9


class sim_base:
    def run_sim(self, SF):
        raise NotImplementedError

    @staticmethod
    def _run_with_output(ctx, m, desc, SF, output_freq):
        """gfm_run_sim: the reference's loop with its output files under
        SF.basename; returns the loop's wall time in seconds."""
        secs = ctypes.c_double(0.0)
        nsteps = SF.nsteps if SF.nsteps > 0 else 0
        _check(lib().gfm_run_sim(ctx._p, ctypes.byref(m), ctypes.byref(desc), SF.basename.encode(), int(output_freq),
                                 int(nsteps), ctypes.byref(secs)), "gfm_run_sim")
        return secs.value


def checkpoint_write(path, desc, t, numsteps, U1, U2=None, phi=None):
    """gfm_checkpoint_write from host arrays."""
    two = U2 is not None
    arrs = [np.ascontiguousarray(a, dtype=np.float64) if a is not None else None for a in (U1, U2, phi)]
    _check(lib().gfm_checkpoint_write(str(path).encode(), ctypes.byref(desc), int(two), float(t), int(numsteps),
                                      *[_dptr(a) if a is not None else None for a in arrs]),
           "gfm_checkpoint_write")


def checkpoint_read(path):
    """gfm_checkpoint_read: (desc, t, numsteps, U1, U2 or None, phi or None)."""
    d = GridDesc()
    two, ns = ctypes.c_int(0), ctypes.c_int(0)
    t = ctypes.c_double(0.0)
    L = lib()
    _check(L.gfm_checkpoint_read(str(path).encode(), ctypes.byref(d), ctypes.byref(two), ctypes.byref(t),
                                 ctypes.byref(ns), None, None, None), "gfm_checkpoint_read")
    nr, nc = d.shape
    U1 = np.empty((4, nr, nc))
    U2 = np.empty((4, nr, nc)) if two.value else None
    phi = np.empty((nr, nc)) if two.value else None
    _check(L.gfm_checkpoint_read(str(path).encode(), ctypes.byref(d), ctypes.byref(two), ctypes.byref(t),
                                 ctypes.byref(ns), _dptr(U1), _dptr(U2) if U2 is not None else None,
                                 _dptr(phi) if phi is not None else None), "gfm_checkpoint_read")
    return d, t.value, ns.value, U1, U2, phi


def write_output_files(desc, basename, numsteps, U1, U2=None, field=None, vel=None, itm="LS5"):
    """The files of one output of sim_twofluid / sim_onefluid from host
    arrays (gfm_write_output_files)."""
    two = U2 is not None
    arrs = [np.ascontiguousarray(a, dtype=np.float64) if a is not None else None for a in (U1, U2, field, vel)]
    _check(lib().gfm_write_output_files(ctypes.byref(desc), basename.encode(), int(two), ITM[itm][2],
                                        int(numsteps), *[_dptr(a) if a is not None else None for a in arrs]),
           "gfm_write_output_files")


class sim_onefluid(sim_base):
    """sourcecode/sim_onefluid.cpp:12-64 on the GPU."""

    def run_sim(self, SF, stream=None, output=False):
        """output: write the reference's files under SF.basename (gfm_run_sim)."""
        desc, T = case_params("onefluid", SF.test_case, SF.Nx, SF.Ny)
        U1, _, _ = case_init("onefluid", SF.test_case, desc)
        ctx = Context(desc, two_fluid=False, stream=stream)
        ctx.upload(U1)
        m = method(fs=SF.FS, CFL=SF.CFL, T=T)
        if output:
            self.seconds = self._run_with_output(ctx, m, desc, SF, OUTPUT_FREQ_ONEFLUID)
            self.ctx = ctx
            return ctx
        nsteps = SF.nsteps if SF.nsteps > 0 else 10 ** 9
        done = 0
        while done < nsteps:
            chunk = min(256, nsteps - done)
            ctx.step(m, chunk)
            done += chunk
            t, n, _ = ctx.time()
            if t >= T:
                break
        self.ctx = ctx
        return ctx


class sim_twofluid(sim_base):
    """sourcecode/sim_twofluid.cpp:27-103 on the GPU."""

    def run_sim(self, SF, stream=None, output=False):
        """output: write the reference's files under SF.basename (gfm_run_sim)."""
        desc, T = case_params("twofluid", SF.test_case, SF.Nx, SF.Ny)
        U1, U2, phi = case_init("twofluid", SF.test_case, desc)
        if ITM[SF.ITM][2] == ITM_VOF:   # the tracker's field is the volume fraction
            phi = case_init_z(SF.test_case, desc)
        ctx = Context(desc, two_fluid=True, stream=stream)
        ctx.upload(U1, U2, phi)
        m = method(fs=SF.FS, gfm=SF.GFM, itm=SF.ITM, CFL=SF.CFL, T=T, reinit_every=SF.reinit_every,
                   reinit_iters=SF.reinit_iters)
        if output:
            freq = OUTPUT_FREQ_TWOFLUID.get(SF.test_case, 4)
            self.seconds = self._run_with_output(ctx, m, desc, SF, freq)
            self.ctx = ctx
            return ctx
        nsteps = SF.nsteps if SF.nsteps > 0 else 10 ** 9
        done = 0
        while done < nsteps:
            chunk = min(256, nsteps - done)
            ctx.step(m, chunk)
            done += chunk
            t, n, _ = ctx.time()
            if t >= T:
                break
        self.ctx = ctx
        return ctx
