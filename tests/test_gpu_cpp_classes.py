"""The reference's C++ class surface (include/gfm_gb300.hpp) used from C++.

tests/cpp/reference_loop.cpp is the reference's time loop written against
the classes (sim_twofluid / sim_onefluid set-up, FS_MUSCL / FS_godunov,
GFM_*::set_ghost_states, Levelset / VOF, apply_BCs_euler, compute_dt) on host
grids, compiled with g++ against the library.  Its results must equal the
oracle's bit for bit (the parity bar, relative L1 <= 1e-10, is implied), and
sim_*::run_sim must write the same files as the library's run through the
Python driver.  The settings-file parsing runs on the CPU.
"""
import os
import subprocess

import numpy as np
import pytest

import gfm_gb300 as g
import oracle_binding as orc

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)


@pytest.fixture(scope="module")
def program(tmp_path_factory):
    libdir = os.path.dirname(g.LIB_PATH)
    exe = str(tmp_path_factory.mktemp("cpp") / "reference_loop")
    r = subprocess.run(["g++", "-std=c++17", "-O2", "-I", os.path.join(ROOT, "include"),
                        os.path.join(HERE, "cpp", "reference_loop.cpp"), "-L", libdir, "-lgfm_gb300",
                        "-Wl,-rpath," + libdir, "-o", exe], stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    assert r.returncode == 0, r.stdout
    return exe


def settings(path, **kv):
    with open(path, "w") as f:
        for k, v in kv.items():
            f.write("%s %s\n" % (k, v))
    return str(path)


def read_result(path, two):
    with open(path, "rb") as f:
        h = np.fromfile(f, dtype="<i4", count=4)
        t = float(np.fromfile(f, dtype="<f8", count=1)[0])
        rc = np.fromfile(f, dtype="<i4", count=8)
        nr, nc = int(h[0]), int(h[1])
        U1 = np.fromfile(f, dtype="<f8", count=4 * nr * nc).reshape(4, nr, nc)
        out = {"numsteps": int(h[2]), "t": t, "rc": (tuple(rc[:4]), tuple(rc[4:])), "U1": U1}
        if two:
            out["U2"] = np.fromfile(f, dtype="<f8", count=4 * nr * nc).reshape(4, nr, nc)
            out["phi"] = np.fromfile(f, dtype="<f8", count=nr * nc).reshape(nr, nc)
    return out


def test_settings_file_basename(program, tmp_path):
    """GFM_settingsfile::read_settings_file: the reference's keys and basename
    (headers/GFM_settingsfile.hpp:24-59), as the Python driver reads them."""
    for kv in ({"sim_type": "twofluid", "Nx": 96, "Ny": 40, "CFL": 0.6, "FS": "MUSCL", "GFM": "riemannGFM",
                "ITM": "LS5", "test_case": "shock_bubble", "outputpath": "./out/", "unused_key": 3},
               {"sim_type": "onefluid", "Nx": 200, "Ny": 200, "CFL": 0.8, "FS": "Godunov",
                "test_case": "circularexplosion", "outputpath": "x_"}):
        path = settings(tmp_path / "sf.txt", **kv)
        r = subprocess.run([program, "basename", path], stdout=subprocess.PIPE, text=True)
        assert r.returncode == 0
        assert r.stdout.strip() == g.GFM_settingsfile().read_settings_file(path).basename


TWOFLUID = [
    # case, Nx, Ny, GFM, FS, ITM, CFL, steps, reinit_every
    ("shock_bubble", 64, 24, "riemannGFM", "MUSCL", "LS5", 0.6, 10, 1),
    ("shock_bubble", 64, 24, "realGFM", "MUSCL", "LS5", 0.6, 10, 1),
    ("shock_bubble", 64, 24, "MGFM", "MUSCL", "LS1", 0.6, 10, 1),
    ("shock_bubble", 64, 24, "OGFM", "Godunov", "LS1", 0.6, 10, 1),
    ("underwater_explosion_sg", 48, 48, "realGFM", "MUSCL", "LS5", 0.5, 12, 5),
    ("shock_bubble", 64, 24, "VOFGFM", "MUSCL", "PYVOF", 0.6, 10, 0),
    ("shock_bubble", 64, 24, "OGFMVOF", "MUSCL", "PYVOF", 0.6, 10, 0),
    ("ST1_x", 64, 12, "riemannGFM", "MUSCL", "LS5", 0.5, 15, 1),
]


@pytest.mark.gpu
@pytest.mark.parametrize("case,Nx,Ny,gfm,fs,itm,CFL,nsteps,reinit", TWOFLUID)
def test_cpp_loop_matches_oracle(program, tmp_path, case, Nx, Ny, gfm, fs, itm, CFL, nsteps, reinit):
    path = settings(tmp_path / "sf.txt", sim_type="twofluid", Nx=Nx, Ny=Ny, CFL=CFL, FS=fs, GFM=gfm, ITM=itm,
                    test_case=case, outputpath=str(tmp_path) + "/", nsteps=nsteps, reinit_every=reinit)
    out = str(tmp_path / "result.bin")
    r = subprocess.run([program, "loop", path, out], stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    assert r.returncode == 0, r.stdout
    res = read_result(out, True)
    desc, T = g.case_params("twofluid", case, Nx, Ny)
    U1, U2, phi = g.case_init("twofluid", case, desc)
    if itm == "PYVOF":
        phi = g.case_init_z(case, desc)
    m = g.method(fs=fs, gfm=gfm, itm=itm, CFL=CFL, T=T, reinit_every=reinit)
    ref = orc.twofluid_run(desc, m, U1, U2, phi, nsteps)
    assert res["numsteps"] == ref["numsteps"] == nsteps and res["t"] == ref["t"]
    gc = desc.numGC
    for name in ("U1", "U2", "phi"):
        a, b = res[name][..., gc:-gc, gc:-gc], ref[name][..., gc:-gc, gc:-gc]
        assert np.abs(a - b).sum() <= 1e-10 * np.abs(b).sum(), name
        assert np.array_equal(res[name], ref[name]), name
    assert res["rc"] == orc.last_realcells()


@pytest.mark.gpu
@pytest.mark.parametrize("case,Nx,Ny,fs", [("circularexplosion", 48, 48, "MUSCL"), ("TTC1_x", 64, 8, "Godunov")])
def test_cpp_onefluid_loop_matches_oracle(program, tmp_path, case, Nx, Ny, fs):
    path = settings(tmp_path / "sf.txt", sim_type="onefluid", Nx=Nx, Ny=Ny, CFL=0.8, FS=fs, test_case=case,
                    outputpath=str(tmp_path) + "/", nsteps=20)
    out = str(tmp_path / "result.bin")
    r = subprocess.run([program, "onefluid", path, out], stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    assert r.returncode == 0, r.stdout
    res = read_result(out, False)
    desc, T = g.case_params("onefluid", case, Nx, Ny)
    U, _, _ = g.case_init("onefluid", case, desc)
    R, t, n, _ = orc.onefluid_run(desc, g.method(fs=fs, CFL=0.8, T=T), U, 20)
    assert res["numsteps"] == n and res["t"] == t
    assert np.array_equal(res["U1"], R)


@pytest.mark.gpu
@pytest.mark.parametrize("kv", [
    {"sim_type": "twofluid", "Nx": 64, "Ny": 24, "CFL": 0.6, "FS": "MUSCL", "GFM": "riemannGFM", "ITM": "LS5",
     "test_case": "shock_bubble", "nsteps": 30},
    {"sim_type": "twofluid", "Nx": 40, "Ny": 40, "CFL": 0.5, "FS": "Godunov", "GFM": "VOFGFM", "ITM": "PYVOF",
     "test_case": "circularexplosion", "nsteps": 20},
    {"sim_type": "onefluid", "Nx": 50, "Ny": 50, "CFL": 0.8, "FS": "MUSCL", "test_case": "circularexplosion"},
])
def test_cpp_run_sim_writes_the_drivers_files(program, tmp_path, kv):
    """sim_*::run_sim from C++ and the Python driver's run_sim(output=True)
    write byte-identical files (the reference's formats; the runtime file,
    a wall-clock time, excepted)."""
    a, b = tmp_path / "cpp", tmp_path / "py"
    a.mkdir()
    b.mkdir()
    pa = settings(tmp_path / "a.txt", outputpath=str(a) + "/", **kv)
    pb = settings(tmp_path / "b.txt", outputpath=str(b) + "/", **kv)
    r = subprocess.run([program, "run_sim", pa], stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    assert r.returncode == 0, r.stdout
    SF = g.GFM_settingsfile().read_settings_file(pb)
    sim = g.sim_onefluid() if kv["sim_type"] == "onefluid" else g.sim_twofluid()
    ctx = sim.run_sim(SF, output=True)
    ctx.close()
    fa = sorted(f for f in os.listdir(a) if not f.endswith("-runtime.dat"))
    fb = sorted(f for f in os.listdir(b) if not f.endswith("-runtime.dat"))
    assert fa == fb and len(fa) >= 2
    for f in fa:
        assert open(a / f, "rb").read() == open(b / f, "rb").read(), f
