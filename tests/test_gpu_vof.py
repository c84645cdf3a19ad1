"""GFM_VOF and OGFM_VOF with the VOF interface tracker on the GPU (through
the C ABI) against the CPU oracle: bit-identical grids, volume fraction,
mixed-cell counts and realcells boxes (the rel-L1 <= 1e-10 bar is asserted
first)."""
import numpy as np
import pytest

import gfm_gb300 as g
import oracle_binding as orc

pytestmark = pytest.mark.gpu
TOL = 1e-10


def rel_l1(a, b):
    den = np.abs(b).sum()
    return np.abs(a - b).sum() / (den if den > 0 else 1.0)


def real(desc, a):
    gc = desc.numGC
    return a[..., gc:gc + desc.Ny, gc:gc + desc.Nx]


VOF_CASES = [
    # case, Nx, Ny, GFM, FS, steps, slip
    ("shock_bubble", 120, 48, "VOFGFM", "MUSCL", 40, False),
    ("shock_bubble", 120, 48, "OGFMVOF", "MUSCL", 40, False),
    ("shock_bubble", 96, 40, "VOFGFM", "Godunov", 30, True),
    ("underwater_explosion_sg", 64, 64, "VOFGFM", "MUSCL", 30, False),
    ("underwater_explosion_sg", 64, 64, "OGFMVOF", "MUSCL", 30, False),
    ("ST1_x", 99, 8, "VOFGFM", "MUSCL", 40, False),
    ("ST1_x", 99, 8, "OGFMVOF", "MUSCL", 40, False),
    ("ST2_y", 8, 99, "VOFGFM", "MUSCL", 40, False),
    ("circularexplosion", 48, 48, "VOFGFM", "MUSCL", 25, False),
    ("shocked_helium_bubble", 96, 28, "OGFMVOF", "Godunov", 25, False),
]


@pytest.mark.parametrize("case,Nx,Ny,gfm,fs,nsteps,slip", VOF_CASES)
def test_vof_parity(case, Nx, Ny, gfm, fs, nsteps, slip):
    desc, T = g.case_params("twofluid", case, Nx, Ny)
    U1, U2, _ = g.case_init("twofluid", case, desc)
    z = g.case_init_z(case, desc)
    m = g.method(fs=fs, gfm=gfm, itm="PYVOF", CFL=0.5, T=T, use_slip_BCs=slip)
    ctx = g.Context(desc, two_fluid=True)
    ctx.upload(U1, U2, z)
    ctx.step(m, nsteps)
    G1, G2, Gz = ctx.download()
    stats = ctx.stats()
    t, n, _ = ctx.time()
    st = ctx.status()
    ctx.close()
    orc.clear_status()
    ref = orc.twofluid_run(desc, m, U1, U2, z, nsteps)
    assert n == ref["numsteps"] and t == ref["t"]
    f1 = real(desc, Gz) >= 0.5
    f1r = real(desc, ref["phi"]) >= 0.5
    for k in range(4):
        comp_gpu = np.where(f1, real(desc, G1[k]), real(desc, G2[k]))
        comp_ref = np.where(f1r, real(desc, ref["U1"][k]), real(desc, ref["U2"][k]))
        assert rel_l1(comp_gpu, comp_ref) <= TOL
    assert rel_l1(real(desc, Gz), real(desc, ref["phi"])) <= TOL
    assert stats["n_interfacial"] == ref["n_interfacial"] > 0
    assert np.array_equal(Gz, ref["phi"]), "expected a bit-identical volume fraction"
    assert np.array_equal(G1, ref["U1"]) and np.array_equal(G2, ref["U2"]), "expected bit-identical grids"
    assert st == 0 and orc.status() == 0


def test_vof_ogfm_water_air_tube_fails_identically():
    """OGFM_VOF on the water/air tube ST2_y (pressure ratio 1e4, stiffened
    water) leaves the physical states after about 15 steps in the oracle as
    well: the GPU raises the same status and produces the same bits,
    non-finite values included."""
    desc, T = g.case_params("twofluid", "ST2_y", 8, 99)
    U1, U2, _ = g.case_init("twofluid", "ST2_y", desc)
    z = g.case_init_z("ST2_y", desc)
    m = g.method(gfm="OGFMVOF", itm="PYVOF", CFL=0.5, T=T)
    ctx = g.Context(desc, two_fluid=True)
    ctx.upload(U1, U2, z)
    ctx.step(m, 20)
    G1, G2, Gz = ctx.download()
    st = ctx.status()
    ctx.close()
    orc.clear_status()
    ref = orc.twofluid_run(desc, m, U1, U2, z, 20)
    assert st != 0 and st == orc.status()
    assert not np.isfinite(ref["U2"]).all()
    for a, b in ((G1, ref["U1"]), (G2, ref["U2"]), (Gz, ref["phi"])):
        assert np.array_equal(a, b, equal_nan=True)


def test_vof_velocity_field_matches():
    """The velocity field handed to the tracker by the last ghost fill."""
    desc, T = g.case_params("twofluid", "underwater_explosion_sg", 48, 48)
    U1, U2, _ = g.case_init("twofluid", "underwater_explosion_sg", desc)
    z = g.case_init_z("underwater_explosion_sg", desc)
    for gfm in ("VOFGFM", "OGFMVOF"):
        m = g.method(gfm=gfm, itm="PYVOF", CFL=0.5, T=T)
        ctx = g.Context(desc, two_fluid=True)
        ctx.upload(U1, U2, z)
        ctx.step(m, 6)
        vel = ctx.velocity()
        ctx.close()
        ref = orc.twofluid_run(desc, m, U1, U2, z, 6)
        assert np.array_equal(vel, ref["vel"])


def test_vof_rejects_level_set_combinations():
    desc, T = g.case_params("twofluid", "shock_bubble", 64, 24)
    ctx = g.Context(desc, two_fluid=True)
    bad = [g.method(gfm="VOFGFM", itm="LS5", T=T), g.method(gfm="riemannGFM", itm="PYVOF", T=T)]
    for m in bad:
        with pytest.raises(g.GFMError):
            ctx.step(m, 1)
    ctx.close()


def test_vof_settings_file_run():
    """The settings-file path (sim_twofluid.run_sim) with GFM VOFGFM, ITM
    PYVOF: the same steps as direct calls."""
    SF = g.GFM_settingsfile()
    SF.sim_type, SF.test_case, SF.Nx, SF.Ny = "twofluid", "shock_bubble", 80, 32
    SF.FS, SF.GFM, SF.ITM, SF.CFL, SF.nsteps = "MUSCL", "VOFGFM", "PYVOF", 0.5, 10
    ctx = g.sim_twofluid().run_sim(SF)
    G1, G2, Gz = ctx.download()
    ctx.close()
    desc, T = g.case_params("twofluid", "shock_bubble", 80, 32)
    U1, U2, _ = g.case_init("twofluid", "shock_bubble", desc)
    z = g.case_init_z("shock_bubble", desc)
    ref = orc.twofluid_run(desc, g.method(gfm="VOFGFM", itm="PYVOF", CFL=0.5, T=T), U1, U2, z, 10)
    assert np.array_equal(Gz, ref["phi"]) and np.array_equal(G1, ref["U1"]) and np.array_equal(G2, ref["U2"])
