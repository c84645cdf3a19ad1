"""TEST INFRASTRUCTURE: runs the reference checker oracle/_ref/gfm_ref.

Only tests/ may use this module, and only to check the oracle against the
reference's own code (built from its sources by oracle/build_ref.py; see
ref_driver.cpp for what runs).  Each run is a fresh process: the reference's
ghost-fluid methods keep function-static scratch grids sized by the first
call's row count (e.g. sourcecode/GFM_riemann.cpp:20-30), so one process runs
one grid.
"""
import os
import platform
import subprocess
import tempfile

import numpy as np

import build_ref

FS_NAMES = {0: "Godunov", 1: "MUSCL"}
GFM_NAMES = {0: "OGFM", 1: "riemannGFM", 2: "realGFM", 3: "MGFM", 4: "VOFGFM", 5: "OGFMVOF"}
BC_NAMES = {0: "transmissive", 1: "reflective", 2: "periodic"}


def available():
    """The checker can run here: the reference's sources are present (it is
    built for this machine), or it was built on this machine before."""
    return build_ref.available() and platform.machine() in ("x86_64", "aarch64")


def binary():
    path = build_ref.build()
    if path is None:
        raise RuntimeError("the reference's sources are absent: the checker cannot be built")
    return path


def _itm_name(m):
    if m.itm == 1:
        return "PYVOF"
    return "LS%d" % m.ls_order


def _write_state(path, nr, nc, U1, U2, phi, t=0.0, numsteps=0):
    with open(path, "wb") as f:
        np.array([nr, nc, numsteps, 0], dtype="<i4").tofile(f)
        np.array([t], dtype="<f8").tofile(f)
        np.zeros(8, dtype="<i4").tofile(f)
        for a in (U1, U2, phi):
            np.ascontiguousarray(a, dtype="<f8").tofile(f)


def _read_result(path):
    with open(path, "rb") as f:
        h = np.fromfile(f, dtype="<i4", count=4)
        t = float(np.fromfile(f, dtype="<f8", count=1)[0])
        rc = np.fromfile(f, dtype="<i4", count=8)
        nr, nc = int(h[0]), int(h[1])
        plane = nr * nc
        U1 = np.fromfile(f, dtype="<f8", count=4 * plane).reshape(4, nr, nc)
        U2 = np.fromfile(f, dtype="<f8", count=4 * plane).reshape(4, nr, nc)
        phi = np.fromfile(f, dtype="<f8", count=plane).reshape(nr, nc)
        mask = np.fromfile(f, dtype=np.uint8, count=plane).reshape(nr, nc)
        mask_fill = np.fromfile(f, dtype=np.uint8, count=plane).reshape(nr, nc)
        newton = int(np.fromfile(f, dtype="<i8", count=1)[0])
    return {"U1": U1, "U2": U2, "phi": phi, "mask": mask, "mask_ghost_fill": mask_fill, "t": t, "numsteps": int(h[2]),
            "realcells1": tuple(int(x) for x in rc[:4]), "realcells2": tuple(int(x) for x in rc[4:]),
            "newton_iters": newton}


def _run(lines, state=None):
    exe = binary()
    with tempfile.TemporaryDirectory() as d:
        req = os.path.join(d, "request.txt")
        out = os.path.join(d, "result.bin")
        if state is not None:
            sp = os.path.join(d, "state.bin")
            _write_state(sp, *state)
            lines = lines + ["state %s" % sp]
        with open(req, "w") as f:
            f.write("\n".join(lines) + "\n")
        r = subprocess.run([exe, req, out], stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
        if r.returncode != 0:
            raise RuntimeError("reference checker failed (%d): %s" % (r.returncode, r.stdout[-2000:]))
        return _read_result(out)


def _method_lines(m, nsteps):
    return ["FS %s" % FS_NAMES[m.fs], "GFM %s" % GFM_NAMES[m.gfm], "ITM %s" % _itm_name(m),
            "CFL %r" % m.CFL, "nsteps %d" % nsteps, "reinit_every %d" % m.reinit_every,
            "reinit_iters %d" % m.reinit_iters, "use_extension_vfield %d" % m.use_extension_vfield,
            "use_slip_BCs %d" % m.use_slip_BCs]


def _grid_lines(desc, T):
    return ["Nx %d" % desc.Nx, "Ny %d" % desc.Ny, "numGC %d" % desc.numGC, "x0 %r" % desc.x0, "y0 %r" % desc.y0,
            "dx %r" % desc.dx, "dy %r" % desc.dy, "BC_L %s" % BC_NAMES[desc.BC_L], "BC_R %s" % BC_NAMES[desc.BC_R],
            "BC_B %s" % BC_NAMES[desc.BC_B], "BC_T %s" % BC_NAMES[desc.BC_T], "gamma1 %r" % desc.gamma1,
            "pinf1 %r" % desc.pinf1, "gamma2 %r" % desc.gamma2, "pinf2 %r" % desc.pinf2, "T %r" % T]


def twofluid_case(test_case, Nx, Ny, m, nsteps):
    """The reference's own parameters and initial conditions of test_case
    (sim_twofluid::set_sim_parameters / set_sim_ICs), then nsteps steps."""
    return _run(["sim_type twofluid", "test_case %s" % test_case, "Nx %d" % Nx, "Ny %d" % Ny]
                + _method_lines(m, nsteps))


def twofluid_initial(test_case, Nx, Ny, m):
    """The reference's initial conditions of test_case (no step)."""
    return twofluid_case(test_case, Nx, Ny, m, 0)


def twofluid_state(desc, m, U1, U2, phi, nsteps, t=0.0, numsteps=0):
    """nsteps reference steps from a given state (phi holds z for the VOF tracker)."""
    nr, nc = desc.Ny + 2 * desc.numGC, desc.Nx + 2 * desc.numGC
    return _run(["sim_type twofluid"] + _grid_lines(desc, m.T) + _method_lines(m, nsteps),
                state=(nr, nc, U1, U2, phi, t, numsteps))


def onefluid_state(desc, m, U, nsteps, t=0.0, numsteps=0):
    nr, nc = desc.Ny + 2 * desc.numGC, desc.Nx + 2 * desc.numGC
    z = np.zeros((4, nr, nc))
    return _run(["sim_type onefluid"] + _grid_lines(desc, m.T) + _method_lines(m, nsteps),
                state=(nr, nc, U, z, np.zeros((nr, nc)), t, numsteps))
