"""The settings-file reader (headers/GFM_settingsfile.hpp:24-59): whitespace
'key value' lines, unknown keys ignored, the output basename built as the
reference builds it; and the GPU run_sim drivers stepping a named case."""
import numpy as np
import pytest

import gfm_gb300 as g


def write(tmp_path, text):
    f = tmp_path / "settingsfile.txt"
    f.write_text(text)
    return str(f)


def test_twofluid_settings(tmp_path):
    SF = g.GFM_settingsfile().read_settings_file(write(tmp_path, """Nx 80
Ny 64
CFL 0.4
sim_type twofluid
FS MUSCL
test_case GDA
outputpath out/
ITM LS5
GFM OGFM
unknown_key 12
""" ))
    assert (SF.Nx, SF.Ny, SF.CFL) == (80, 64, 0.4)
    assert (SF.sim_type, SF.FS, SF.test_case, SF.ITM, SF.GFM) == ("twofluid", "MUSCL", "GDA", "LS5", "OGFM")
    assert SF.basename == "out/OGFM-LS5-GDA-MUSCL-80-64"


def test_onefluid_settings(tmp_path):
    SF = g.GFM_settingsfile().read_settings_file(write(tmp_path, "sim_type onefluid\nFS Godunov\ntest_case TTC1_x\n"
                                                                 "Nx 100\nNy 4\n\nCFL 0.8\n"))
    assert SF.basename == "onefluid-TTC1_x-Godunov-100-4"
    assert SF.CFL == 0.8


@pytest.mark.gpu
def test_run_sim_twofluid_matches_direct_steps(tmp_path):
    SF = g.GFM_settingsfile().read_settings_file(write(tmp_path, """Nx 48
Ny 48
CFL 0.5
sim_type twofluid
FS MUSCL
test_case underwater_explosion_sg
ITM LS5
GFM realGFM
nsteps 12
"""))
    ctx = g.sim_twofluid().run_sim(SF)
    out = ctx.download()
    t, n, _ = ctx.time()
    ctx.close()
    desc, T = g.case_params("twofluid", "underwater_explosion_sg", 48, 48)
    U1, U2, phi = g.case_init("twofluid", "underwater_explosion_sg", desc)
    c2 = g.Context(desc, two_fluid=True)
    c2.upload(U1, U2, phi)
    c2.step(g.method(fs="MUSCL", gfm="realGFM", itm="LS5", CFL=0.5, T=T), 12)
    ref = c2.download()
    c2.close()
    assert n == 12
    for a, b in zip(out, ref):
        assert np.array_equal(a, b)
