"""The oracle pinned to the reference's own code.

oracle/_ref/gfm_ref is murraycutforth/PhD-2D-GFM's sourcecode/*.cpp compiled
unchanged (oracle/build_ref.py) against stand-in headers for the libraries it
takes from outside its repository; the stand-ins for the absent algorithms
(exact stiffened-gas Riemann solver, EOS, level set, VOF tracker, bilinear
interpolation, cell centres) are the oracle's own definitions, so these tests
check the oracle's restatement of everything that IS in the reference's
repository -- FS_MUSCL / FS_godunov, pure_RS_exact / mixed_RS_exact, the six
GFM_*::set_ghost_states, extrapolate_vector(_mgfm), extrapolate_extension_vfield,
apply_BCs_euler, euler_misc, compute_dt, the time loop and set_sim_ICs --
against that code itself.  The bar is the parity bar (relative L1 <= 1e-10
per field over real cells), then bit equality of the whole padded grids,
the step count and t, the realcells boxes and the interfacial-cell mask.

The reference's sources are needed to build the checker; without them these
tests are skipped.
"""
import numpy as np
import pytest

import gfm_gb300 as g
import oracle_binding as orc
import ref_binding as rb

pytestmark = pytest.mark.skipif(not rb.available(), reason="the reference's sources are absent")
TOL = 1e-10


def rel_l1(a, b):
    den = np.abs(b).sum()
    return np.abs(a - b).sum() / (den if den > 0 else 1.0)


def real(desc, a):
    gc = desc.numGC
    return a[..., gc:gc + desc.Ny, gc:gc + desc.Nx]


def assert_same(desc, o, r, planes=("U1", "U2", "phi")):
    for name in planes:
        a, b = o[name], r[name]
        if a.ndim == 3:
            for k in range(a.shape[0]):
                assert rel_l1(real(desc, a[k]), real(desc, b[k])) <= TOL, (name, k)
        else:
            assert rel_l1(real(desc, a), real(desc, b)) <= TOL, name
        assert np.array_equal(a, b), "%s: not bit-identical (max %.3e)" % (name, np.abs(a - b).max())


# reference test cases whose parameters and initial conditions the reference sets itself
REFERENCE_CASES = [("circularexplosion", 40, 40), ("ST1_x", 64, 12), ("ST2_y", 12, 64), ("GDA", 24, 24),
                   ("shocked_helium_bubble", 65, 18), ("shocked_R22_bubble", 60, 16)]


@pytest.mark.parametrize("case,Nx,Ny", REFERENCE_CASES)
def test_initial_conditions_match_the_reference(case, Nx, Ny):
    """The library's host set-up (gfm_case_params / gfm_case_init / _z)
    against sim_twofluid::set_sim_parameters and set_sim_ICs
    (sourcecode/sim_twofluid.cpp:336-490, 599-1799)."""
    desc, T = g.case_params("twofluid", case, Nx, Ny)
    U1, U2, phi = g.case_init("twofluid", case, desc)
    r = rb.twofluid_initial(case, Nx, Ny, g.method(T=T))
    assert_same(desc, {"U1": U1, "U2": U2, "phi": phi}, r)
    z = g.case_init_z(case, desc)
    rz = rb.twofluid_initial(case, Nx, Ny, g.method(gfm="VOFGFM", itm="PYVOF", T=T))
    assert np.array_equal(z, rz["phi"])


@pytest.mark.parametrize("case,Nx,Ny", REFERENCE_CASES)
def test_steps_from_the_reference_initial_conditions(case, Nx, Ny):
    desc, T = g.case_params("twofluid", case, Nx, Ny)
    m = g.method(fs="MUSCL", gfm="riemannGFM", itm="LS5", CFL=0.5, T=T)
    r = rb.twofluid_case(case, Nx, Ny, m, 20)
    r0 = rb.twofluid_initial(case, Nx, Ny, m)
    o = orc.twofluid_run(desc, m, r0["U1"], r0["U2"], r0["phi"], 20)
    assert o["numsteps"] == r["numsteps"] == 20 and o["t"] == r["t"]
    assert_same(desc, o, r)


TWOFLUID = [
    # case, Nx, Ny, GFM, FS, ITM, reinit_every, steps, extension vfield, slip
    ("shock_bubble", 80, 32, "riemannGFM", "MUSCL", "LS5", 1, 12, False, False),
    ("shock_bubble", 80, 32, "realGFM", "MUSCL", "LS5", 5, 12, False, False),
    ("shock_bubble", 80, 32, "MGFM", "MUSCL", "LS5", 1, 12, False, False),
    ("shock_bubble", 80, 32, "OGFM", "MUSCL", "LS5", 1, 12, False, False),
    ("shock_bubble", 80, 32, "riemannGFM", "Godunov", "LS1", 1, 12, False, False),
    ("shock_bubble", 64, 24, "riemannGFM", "MUSCL", "LS5", 1, 8, True, False),
    ("shock_bubble", 64, 24, "MGFM", "MUSCL", "LS1", 0, 8, True, False),
    ("shock_bubble", 64, 24, "MGFM", "MUSCL", "LS5", 1, 8, False, True),
    ("underwater_explosion_sg", 48, 48, "realGFM", "MUSCL", "LS5", 5, 10, False, False),
    ("underwater_explosion_sg", 40, 40, "riemannGFM", "MUSCL", "LS5", 1, 8, False, False),
    ("ST1_x", 64, 12, "riemannGFM", "MUSCL", "LS5", 1, 15, False, False),
    ("ST2_y", 12, 64, "MGFM", "MUSCL", "LS5", 1, 15, False, False),
    ("GDA", 24, 24, "OGFM", "MUSCL", "LS5", 1, 10, False, False),
    ("shocked_helium_bubble", 64, 20, "riemannGFM", "MUSCL", "LS5", 1, 10, False, False),
    ("circularexplosion", 32, 32, "realGFM", "Godunov", "LS1", 1, 10, False, False),
    ("circularexplosion", 40, 40, "OGFM", "Godunov", "LS1", 1, 12, False, False),
]


@pytest.mark.parametrize("case,Nx,Ny,gfm,fs,itm,reinit,nsteps,ext,slip", TWOFLUID)
def test_twofluid_oracle_matches_reference(case, Nx, Ny, gfm, fs, itm, reinit, nsteps, ext, slip):
    desc, T = g.case_params("twofluid", case, Nx, Ny)
    U1, U2, phi = g.case_init("twofluid", case, desc)
    m = g.method(fs=fs, gfm=gfm, itm=itm, CFL=0.6, T=T, reinit_every=reinit, use_extension_vfield=ext,
                 use_slip_BCs=slip)
    orc.clear_status()
    o = orc.twofluid_run(desc, m, U1, U2, phi, nsteps)
    rc1, rc2 = orc.last_realcells()
    r = rb.twofluid_state(desc, m, U1, U2, phi, nsteps)
    assert o["numsteps"] == r["numsteps"] == nsteps and o["t"] == r["t"]
    assert_same(desc, o, r)
    assert (rc1, rc2) == (r["realcells1"], r["realcells2"])
    assert np.array_equal(orc.interfacial_mask(desc, o["phi"]), r["mask"])
    assert o["n_interfacial"] == int(r["mask_ghost_fill"].sum())
    assert orc.status() == 0


VOF = [
    ("shock_bubble", 64, 24, "VOFGFM", "MUSCL", 12),
    ("shock_bubble", 64, 24, "OGFMVOF", "MUSCL", 12),
    ("circularexplosion", 40, 40, "VOFGFM", "Godunov", 10),
    ("underwater_explosion_sg", 40, 40, "VOFGFM", "MUSCL", 8),
]


@pytest.mark.parametrize("case,Nx,Ny,gfm,fs,nsteps", VOF)
def test_vof_oracle_matches_reference(case, Nx, Ny, gfm, fs, nsteps):
    desc, T = g.case_params("twofluid", case, Nx, Ny)
    U1, U2, _ = g.case_init("twofluid", case, desc)
    z = g.case_init_z(case, desc)
    m = g.method(fs=fs, gfm=gfm, itm="PYVOF", CFL=0.5, T=T)
    o = orc.twofluid_run(desc, m, U1, U2, z, nsteps)
    rc1, rc2 = orc.last_realcells()
    r = rb.twofluid_state(desc, m, U1, U2, z, nsteps)
    assert o["numsteps"] == r["numsteps"] == nsteps and o["t"] == r["t"]
    assert_same(desc, o, r)
    assert (rc1, rc2) == (r["realcells1"], r["realcells2"])


ONEFLUID = [
    ("TTC1_x", 64, 8, "MUSCL"), ("TTC1_y", 8, 64, "MUSCL"), ("TTC2_x", 64, 8, "MUSCL"),
    ("TTC3_x", 64, 8, "MUSCL"), ("TTC4_y", 8, 64, "MUSCL"), ("TTC5_x", 64, 8, "MUSCL"),
    ("TTC1_x", 64, 8, "Godunov"), ("TTC3_y", 8, 64, "Godunov"),
    ("circularexplosion", 40, 40, "MUSCL"), ("circularexplosion", 36, 28, "Godunov"),
]


@pytest.mark.parametrize("case,Nx,Ny,fs", ONEFLUID)
def test_onefluid_oracle_matches_reference(case, Nx, Ny, fs):
    """sim_onefluid's loop: its compute_dt, FS_* and apply_BCs_euler."""
    desc, T = g.case_params("onefluid", case, Nx, Ny)
    U, _, _ = g.case_init("onefluid", case, desc)
    m = g.method(fs=fs, CFL=0.8, T=T)
    R, t, n, _ = orc.onefluid_run(desc, m, U, 25)
    r = rb.onefluid_state(desc, m, U, 25)
    assert n == r["numsteps"] and t == r["t"]
    for k in range(4):
        assert rel_l1(real(desc, R[k]), real(desc, r["U1"][k])) <= TOL
    assert np.array_equal(R, r["U1"])


def test_long_run_matches_reference():
    """600 steps of a coarse shock-bubble: the two codes stay bit-identical
    through the Newton iterations, fallbacks and reinitialisations of a long
    run (the configured runs themselves are pinned by
    tests/golden/fulllength_digests.json, made by the same checker)."""
    desc, T = g.case_params("twofluid", "shock_bubble", 100, 40)
    U1, U2, phi = g.case_init("twofluid", "shock_bubble", desc)
    m = g.method(fs="MUSCL", gfm="riemannGFM", itm="LS5", CFL=0.6, T=T)
    o = orc.twofluid_run(desc, m, U1, U2, phi, 600)
    r = rb.twofluid_state(desc, m, U1, U2, phi, 600)
    assert o["numsteps"] == r["numsteps"] == 600 and o["t"] == r["t"]
    assert_same(desc, o, r)
    assert np.array_equal(orc.interfacial_mask(desc, o["phi"]), r["mask"])


def test_unphysical_state_detected_at_the_reference_abort():
    """On the 100 x 40 shock-bubble the far ghost field of fluid 1 turns
    unphysical after 671 steps: the reference's live assert at the start of
    the ghost fill (sourcecode/GFM_riemann.cpp:37) aborts step 672, and the
    oracle, which records the same check in its status word instead of
    aborting, flags GFM_ST_UNPHYSICAL in the same step and not before."""
    desc, T = g.case_params("twofluid", "shock_bubble", 100, 40)
    U1, U2, phi = g.case_init("twofluid", "shock_bubble", desc)
    m = g.method(fs="MUSCL", gfm="riemannGFM", itm="LS5", CFL=0.6, T=T)
    r = rb.twofluid_state(desc, m, U1, U2, phi, 671)
    with pytest.raises(RuntimeError, match=r"GFM_riemann\.cpp:37.*is_physical_state"):
        rb.twofluid_state(desc, m, U1, U2, phi, 672)
    orc.clear_status()
    o = orc.twofluid_run(desc, m, U1, U2, phi, 671)
    assert orc.status() == 0
    assert_same(desc, o, r)
    orc.twofluid_run(desc, m, o["U1"], o["U2"], o["phi"], 1, t=o["t"], numsteps=o["numsteps"])
    assert orc.status() & 1
