"""Output files of the reference's drivers (sim_twofluid::output,
output_mass_error, the runtime file; sim_onefluid::output).

The CPU tests check the native writer (gfm_write_output_files, host arrays)
byte for byte against a Python restatement of the reference's output loops
(sourcecode/sim_twofluid.cpp:163-297, sourcecode/sim_onefluid.cpp:169-192),
which print with std::ostream's default %g; the GPU test runs the whole
time loop with its outputs (gfm_run_sim) and compares the files with those
of the oracle's states.
"""
import math
import os

import numpy as np
import pytest

import gfm_gb300 as g
import oracle_binding as orc


def fmt(v):
    return "%g" % v


def prim_line(x, y, U, gm, pinf, i, j):
    rho = U[0, i, j]
    u = U[1, i, j] / rho
    v = U[2, i, j] / rho
    e = (U[3, i, j] / rho) - 0.5 * (u * u + v * v)
    p = (gm - 1.0) * rho * e - gm * pinf
    return " ".join(fmt(a) for a in (x, y, rho, u, v, e, p)) + "\n"


def expected_twofluid(desc, U1, U2, field, vel, vof):
    """The reference's output loops on host arrays."""
    g_ = desc.numGC
    nr, nc = desc.shape
    cx = lambda j: desc.x0 + ((j - g_) + 0.5) * desc.dx   # noqa: E731
    cy = lambda i: desc.y0 + ((i - g_) + 0.5) * desc.dy   # noqa: E731
    sdf = (0.5 - field) if vof else field
    z = field if vof else (field <= 0.0).astype(np.float64)
    prims, ls, vf, zf = [], [], [], []
    for i in range(2, nr - 2):
        for j in range(2, nc - 2):
            x, y = cx(j), cy(i)
            ls.append("%s %s %s\n" % (fmt(x), fmt(y), fmt(sdf[i, j])))
            vf.append("%s %s %s %s\n" % (fmt(x), fmt(y), fmt(vel[0, i, j]), fmt(vel[1, i, j])))
            zf.append("%s %s %s\n" % (fmt(x), fmt(y), fmt(z[i, j])))
            if sdf[i, j] < 0.0:
                prims.append(prim_line(x, y, U1, desc.gamma1, desc.pinf1, i, j))
            else:
                prims.append(prim_line(x, y, U2, desc.gamma2, desc.pinf2, i, j))
        for a in (prims, ls, vf, zf):
            a.append("\n")
    grads = []
    for i in range(g_, desc.Ny + g_):
        for j in range(g_, desc.Nx + g_):
            r = lambda a, b: U1[0, a, b] if sdf[a, b] <= 0.0 else U2[0, a, b]   # noqa: E731
            gx = (r(i, j + 1) - r(i, j - 1)) / (2.0 * desc.dx)
            gy = (r(i + 1, j) - r(i - 1, j)) / (2.0 * desc.dy)
            grads.append(math.sqrt(gx * gx + gy * gy))
    mx = max(grads)
    sch, k = [], 0
    for i in range(g_, desc.Ny + g_):
        for j in range(g_, desc.Nx + g_):
            sch.append("%s %s %s\n" % (fmt(cx(j)), fmt(cy(i)), fmt(grads[k] / mx)))
            k += 1
        sch.append("\n")
    L1 = 0.0
    for i in range(g_, desc.Ny + g_):
        for j in range(g_, desc.Nx + g_):
            dx_, dy_ = cx(j) - 0.5, cy(i) - 0.5
            exact = 1.0 + 1000.0 * math.exp(-(dx_ * dx_ + dy_ * dy_) / (2.0 * 0.1 * 0.1))
            L1 += abs(U1[0, i, j] - exact) * desc.dx * desc.dy
    gda = "%s %s\n" % (fmt(float(desc.Nx)), fmt(L1))
    return {"prims": "".join(prims), "ls": "".join(ls), "vfield": "".join(vf), "z": "".join(zf),
            "schlieren": "".join(sch), "GDAerr": gda}


def read(path):
    with open(path) as f:
        return f.read()


@pytest.mark.parametrize("case,gfm,itm,Nx,Ny", [("shock_bubble", "riemannGFM", "LS5", 40, 16),
                                                ("underwater_explosion_sg", "VOFGFM", "PYVOF", 24, 24)])
def test_twofluid_files_match_reference_loops(tmp_path, case, gfm, itm, Nx, Ny):
    desc, T = g.case_params("twofluid", case, Nx, Ny)
    U1, U2, phi = g.case_init("twofluid", case, desc)
    vof = itm == "PYVOF"
    if vof:
        phi = g.case_init_z(case, desc)
    r = orc.twofluid_run(desc, g.method(gfm=gfm, itm=itm, CFL=0.5, T=T), U1, U2, phi, 6)
    base = str(tmp_path / "run")
    g.write_output_files(desc, base, 6, r["U1"], r["U2"], r["phi"], r["vel"], itm=itm)
    exp = expected_twofluid(desc, r["U1"], r["U2"], r["phi"], r["vel"], vof)
    for k in ("prims", "ls", "vfield", "z", "schlieren"):
        assert read("%s-6-%s.dat" % (base, k)) == exp[k], k
    assert read(base + "-GDAerr.dat") == exp["GDAerr"]


def test_onefluid_prims_file(tmp_path):
    desc, T = g.case_params("onefluid", "TTC1_x", 30, 4)
    U, _, _ = g.case_init("onefluid", "TTC1_x", desc)
    R, _, _, _ = orc.onefluid_run(desc, g.method(CFL=0.8, T=T), U, 5)
    base = str(tmp_path / "one")
    g.write_output_files(desc, base, 5, R)
    nr, nc = desc.shape
    g_ = desc.numGC
    lines = []
    for i in range(nr):
        for j in range(nc):
            x = desc.x0 + ((j - g_) + 0.5) * desc.dx
            y = desc.y0 + ((i - g_) + 0.5) * desc.dy
            lines.append(prim_line(x, y, R, desc.gamma1, desc.pinf1, i, j))
        lines.append("\n")
    assert read(base + "-5-prims.dat") == "".join(lines)


def test_bad_output_path_is_an_error(tmp_path):
    desc, T = g.case_params("onefluid", "TTC1_x", 10, 4)
    U, _, _ = g.case_init("onefluid", "TTC1_x", desc)
    with pytest.raises(g.GFMError):
        g.write_output_files(desc, str(tmp_path / "missing_dir" / "x"), 0, U)


@pytest.mark.gpu
def test_run_sim_outputs_match_oracle(tmp_path):
    """gfm_run_sim on the shock-bubble at 60x24 for 40 steps: output steps as
    the reference's rule picks them, every file of the last output byte-equal
    to the files of the oracle's state, masschange lines within rounding of
    the oracle's sequential mass sums, a runtime file."""
    SF = g.GFM_settingsfile()
    SF.sim_type, SF.test_case, SF.Nx, SF.Ny = "twofluid", "shock_bubble", 60, 24
    SF.FS, SF.GFM, SF.ITM, SF.CFL, SF.nsteps = "MUSCL", "riemannGFM", "LS5", 0.6, 40
    SF.basename = str(tmp_path / "sb")
    sim = g.sim_twofluid()
    ctx = sim.run_sim(SF, output=True)
    ctx.close()
    desc, T = g.case_params("twofluid", "shock_bubble", 60, 24)
    U1, U2, phi = g.case_init("twofluid", "shock_bubble", desc)
    m = g.method(gfm="riemannGFM", itm="LS5", CFL=0.6, T=T)
    # the oracle step by step: output steps and masses
    interval, last = T / 4, 0.0
    outs = [0]
    st = {"U1": U1, "U2": U2, "phi": phi, "t": 0.0, "numsteps": 0}
    mass = lambda sign, U, ph: orc.fluid_mass(desc, sign, U, ph)   # noqa: E731
    m0 = (mass(-1.0, U1, phi), mass(1.0, U2, phi))
    rows = [(0.0, 0.0, 0.0)]
    for s in range(40):
        st = orc.twofluid_run(desc, m, st["U1"], st["U2"], st["phi"], 1, st["t"], st["numsteps"])
        if st["t"] - last > interval:
            outs.append(st["numsteps"])
            last = st["t"]
        m1, m2 = mass(-1.0, st["U1"], st["phi"]), mass(1.0, st["U2"], st["phi"])
        rows.append((st["t"], (m1 - m0[0]) / m0[0], (m2 - m0[1]) / m0[1]))
    outs.append(st["numsteps"])
    for n in outs:
        assert os.path.exists("%s-%d-prims.dat" % (SF.basename, n)), n
    ref = str(tmp_path / "ref")
    g.write_output_files(desc, ref, 40, st["U1"], st["U2"], st["phi"], st["vel"], itm="LS5")
    for k in ("prims", "ls", "vfield", "z", "schlieren"):
        assert read("%s-40-%s.dat" % (SF.basename, k)) == read("%s-40-%s.dat" % (ref, k)), k
    lines = read(SF.basename + "-masschange.dat").split("\n")[:-1]
    assert len(lines) == len(rows)
    for ln, (t, e1, e2) in zip(lines, rows):
        a = [float(x) for x in ln.split()]
        assert a[0] == float("%g" % t)
        assert abs(a[1] - e1) <= 1e-12 + 1e-5 * abs(e1) and abs(a[2] - e2) <= 1e-12 + 1e-5 * abs(e2)
    assert float(read(SF.basename + "-runtime.dat")) > 0.0
