"""The VOF interface tracker and the VOF ghost-fluid methods in the oracle
(CPU): initial volume fractions, the properties its definition promises,
and short GFM_VOF / OGFM_VOF runs against the level-set Riemann GFM.

The reference takes its VOF tracker from an absent library, so these pin
the oracle's own definition (PLIC geometry, advection) by properties; the
GPU path is checked against the oracle bit for bit in test_gpu_vof.py.
"""
import numpy as np
import pytest

import gfm_gb300 as g
import oracle_binding as orc


def inner(desc, a):
    gc = desc.numGC
    return a[..., gc:gc + desc.Ny, gc:gc + desc.Nx]


def test_initial_volume_fraction_of_a_circle():
    """10x10 sub-sampled area fractions (sourcecode/sim_twofluid.cpp:825-856)
    integrate to the disc's area within the sampling error."""
    desc, T = g.case_params("twofluid", "underwater_explosion_sg", 80, 80)
    z = g.case_init_z("underwater_explosion_sg", desc)
    area = inner(desc, z).sum() * desc.dx * desc.dy
    assert abs(area - np.pi * 0.2 ** 2) < 2e-3
    zi = inner(desc, z)
    assert zi.min() == 0.0 and zi.max() == 1.0
    # the planar tube: a clipped linear profile across one cell
    desc2, _ = g.case_params("twofluid", "ST1_x", 50, 4)
    z2 = inner(desc2, g.case_init_z("ST1_x", desc2))
    assert np.all(np.diff(z2[0]) <= 0.0) and z2[0, 0] == 1.0 and z2[0, -1] == 0.0


@pytest.mark.parametrize("gfm", ["VOFGFM", "OGFMVOF"])
def test_vof_gfm_shock_tube_tracks_the_level_set(gfm):
    """ST1_x, a planar two-gas tube: the VOF interface (fluid-1 length)
    stays within two cells of the level set's after 60 steps, z stays in
    [0, 1] and the run raises no status.  An odd cell count puts the
    interface inside a cell: the VOF GFMs act only where a cell is mixed
    (with the interface on a face both grids stay uniform, as in the
    reference)."""
    desc, T = g.case_params("twofluid", "ST1_x", 99, 4)
    U1, U2, phi = g.case_init("twofluid", "ST1_x", desc)
    z = g.case_init_z("ST1_x", desc)
    orc.clear_status()
    mv = g.method(gfm=gfm, itm="PYVOF", CFL=0.5, T=T)
    rv = orc.twofluid_run(desc, mv, U1, U2, z, 60)
    assert orc.status() == 0
    ml = g.method(gfm="riemannGFM", itm="LS5", CFL=0.5, T=T)
    rl = orc.twofluid_run(desc, ml, U1, U2, phi, 60)
    zr = inner(desc, rv["phi"])[1]
    pr = inner(desc, rl["phi"])[1]
    assert zr.min() >= 0.0 and zr.max() <= 1.0
    xv = np.sum(zr)                 # fluid-1 length in cells
    xl = np.argmax(pr > 0.0)        # first fluid-2 cell of the level set
    assert abs(xv - xl) <= 2.0, (xv, xl)
    for k in ("U1", "U2"):
        assert np.isfinite(rv[k]).all()


def test_vof_advection_conserves_and_translates():
    """GDA-like check of the advection alone: with both fluids at rest but a
    uniform velocity (u, v) handed to the tracker, a periodic box keeps
    sum(z) to rounding and moves the fluid's centroid by (u, v) t."""
    desc, T = g.case_params("twofluid", "GDA", 64, 64)
    U1, U2, _ = g.case_init("twofluid", "GDA", desc)
    # a disc of fluid 1 in the periodic box; GDA's flow is uniform (1, 1)
    z = g.case_init_z("underwater_explosion_sg", g.case_params("twofluid", "underwater_explosion_sg", 64, 64)[0])
    z = np.ascontiguousarray(z)
    U2 = U1.copy()
    m = g.method(gfm="VOFGFM", itm="PYVOF", CFL=0.5, T=T)
    r = orc.twofluid_run(desc, m, U1, U2, z, 40)
    z0, z1 = inner(desc, z), inner(desc, r["phi"])
    assert abs(z1.sum() - z0.sum()) <= 1e-9 * z0.sum()
    assert z1.min() >= 0.0 and z1.max() <= 1.0
    ny, nx = z0.shape
    yy, xx = np.mgrid[0:ny, 0:nx]
    c0 = np.array([(z0 * xx).sum(), (z0 * yy).sum()]) / z0.sum()
    c1 = np.array([(z1 * xx).sum(), (z1 * yy).sum()]) / z1.sum()
    shift = (c1 - c0) * desc.dx          # square cells
    assert np.allclose(shift, [r["t"], r["t"]], atol=0.3 * desc.dx), (shift, r["t"])


def test_vof_bubble_runs_clean():
    """Shock-bubble at 120x48 with both VOF GFMs: finite, no status, the
    bubble's volume within 10% of its initial value early on."""
    desc, T = g.case_params("twofluid", "shock_bubble", 120, 48)
    U1, U2, _ = g.case_init("twofluid", "shock_bubble", desc)
    z = g.case_init_z("shock_bubble", desc)
    for gfm in ("VOFGFM", "OGFMVOF"):
        orc.clear_status()
        r = orc.twofluid_run(desc, g.method(gfm=gfm, itm="PYVOF", CFL=0.5, T=T), U1, U2, z, 30)
        assert orc.status() == 0
        assert np.isfinite(r["U1"]).all() and np.isfinite(r["U2"]).all()
        assert abs(inner(desc, r["phi"]).sum() / inner(desc, z).sum() - 1.0) < 0.1
        assert r["n_interfacial"] > 0
