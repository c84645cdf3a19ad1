"""Generates tests/golden/reference_goldens.json: digests of small runs made
by the REFERENCE'S OWN CODE (the checker oracle/_ref/gfm_ref, built from
murraycutforth/PhD-2D-GFM's sources by oracle/build_ref.py), for the GPU
tests to compare against on a machine without the reference.

    python tests/golden/make_ref_goldens.py

Cases: every ghost-fluid method with the level set (Godunov and MUSCL, LS1
and LS5, extension velocities, slip BCs), GFM_VOF and OGFM_VOF with the VOF
tracker, the reference's own test cases from its own initial conditions, the
one-fluid tube tests and circular explosion, and the coarse shock-bubble on
which the reference's assert at sourcecode/GFM_riemann.cpp:37 stops the run.
Per case: the step count, t, per field the SHA-256 of the real cells'
float64 bytes and their magnitude sum, the interfacial-cell mask of the last
ghost fill (SHA-256 and count) and the realcells boxes.  Initial conditions
come from the library's host set-up (gfm_case_init), which
tests/test_oracle_vs_reference.py shows to be bit-identical to the
reference's set_sim_ICs for its own cases.  Runs in about a minute.
"""
import json
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
import make_digests as md  # noqa: E402

md._paths()
import gfm_gb300 as g  # noqa: E402
import ref_binding as rb  # noqa: E402

OUT = os.path.join(HERE, "reference_goldens.json")

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
    ("shock_bubble", 160, 64, "riemannGFM", "MUSCL", "LS5", 1, 200, False, False),
    ("underwater_explosion_sg", 48, 48, "realGFM", "MUSCL", "LS5", 5, 10, False, False),
    ("underwater_explosion_sg", 40, 40, "riemannGFM", "MUSCL", "LS5", 1, 8, False, False),
    ("underwater_explosion_sg", 96, 96, "realGFM", "MUSCL", "LS5", 5, 150, False, False),
    ("ST1_x", 64, 12, "riemannGFM", "MUSCL", "LS5", 1, 15, False, False),
    ("ST2_y", 12, 64, "MGFM", "MUSCL", "LS5", 1, 15, False, False),
    ("GDA", 24, 24, "OGFM", "MUSCL", "LS5", 1, 10, False, False),
    ("shocked_helium_bubble", 64, 20, "riemannGFM", "MUSCL", "LS5", 1, 10, False, False),
    ("shocked_R22_bubble", 60, 16, "realGFM", "MUSCL", "LS5", 1, 20, False, False),
    ("circularexplosion", 32, 32, "realGFM", "Godunov", "LS1", 1, 10, False, False),
    ("circularexplosion", 40, 40, "OGFM", "Godunov", "LS1", 1, 12, False, False),
    ("shock_bubble", 100, 40, "riemannGFM", "MUSCL", "LS5", 1, 671, False, False),
]
VOF = [
    ("shock_bubble", 64, 24, "VOFGFM", "MUSCL", 12),
    ("shock_bubble", 64, 24, "OGFMVOF", "MUSCL", 12),
    ("circularexplosion", 40, 40, "VOFGFM", "Godunov", 10),
    ("underwater_explosion_sg", 40, 40, "VOFGFM", "MUSCL", 8),
    ("shock_bubble", 120, 48, "VOFGFM", "MUSCL", 150),
]
ONEFLUID = [
    ("TTC1_x", 64, 8, "MUSCL"), ("TTC1_y", 8, 64, "MUSCL"), ("TTC2_x", 64, 8, "MUSCL"),
    ("TTC3_x", 64, 8, "MUSCL"), ("TTC4_y", 8, 64, "MUSCL"), ("TTC5_x", 64, 8, "MUSCL"),
    ("TTC1_x", 64, 8, "Godunov"), ("TTC3_y", 8, 64, "Godunov"),
    ("circularexplosion", 40, 40, "MUSCL"), ("circularexplosion", 36, 28, "Godunov"),
]


def main():
    out = {"generator": "tests/golden/make_ref_goldens.py (reference checker oracle/_ref/gfm_ref)", "cases": []}
    for case, nx, ny, gfm, fs, itm, reinit, nsteps, ext, slip in TWOFLUID:
        desc, T = g.case_params("twofluid", case, nx, ny)
        U1, U2, phi = g.case_init("twofluid", case, desc)
        m = g.method(fs=fs, gfm=gfm, itm=itm, CFL=0.6, T=T, reinit_every=reinit, use_extension_vfield=ext,
                     use_slip_BCs=slip)
        r = rb.twofluid_state(desc, m, U1, U2, phi, nsteps)
        d = md.digest(desc, r["U1"], r["U2"], r["phi"], None, r["t"], r["numsteps"], r["mask_ghost_fill"],
                      (r["realcells1"], r["realcells2"]))
        d["spec"] = {"sim": "twofluid", "case": case, "Nx": nx, "Ny": ny, "gfm": gfm, "fs": fs, "itm": itm,
                     "reinit_every": reinit, "steps": nsteps, "ext": ext, "slip": slip, "CFL": 0.6}
        out["cases"].append(d)
    for case, nx, ny, gfm, fs, nsteps in VOF:
        desc, T = g.case_params("twofluid", case, nx, ny)
        U1, U2, _ = g.case_init("twofluid", case, desc)
        z = g.case_init_z(case, desc)
        m = g.method(fs=fs, gfm=gfm, itm="PYVOF", CFL=0.5, T=T)
        r = rb.twofluid_state(desc, m, U1, U2, z, nsteps)
        d = md.digest(desc, r["U1"], r["U2"], r["phi"], None, r["t"], r["numsteps"], None,
                      (r["realcells1"], r["realcells2"]))
        d["spec"] = {"sim": "twofluid", "case": case, "Nx": nx, "Ny": ny, "gfm": gfm, "fs": fs, "itm": "PYVOF",
                     "reinit_every": 0, "steps": nsteps, "ext": False, "slip": False, "CFL": 0.5}
        out["cases"].append(d)
    for case, nx, ny, fs in ONEFLUID:
        desc, T = g.case_params("onefluid", case, nx, ny)
        U, _, _ = g.case_init("onefluid", case, desc)
        m = g.method(fs=fs, CFL=0.8, T=T)
        r = rb.onefluid_state(desc, m, U, 25)
        d = md.digest(desc, r["U1"], None, None, None, r["t"], r["numsteps"])
        d["spec"] = {"sim": "onefluid", "case": case, "Nx": nx, "Ny": ny, "fs": fs, "steps": 25, "CFL": 0.8}
        out["cases"].append(d)
    # the step at which the reference's assert stops the coarse shock-bubble:
    # the first step count whose run raises it (bisection over 1..3000)
    desc, T = g.case_params("twofluid", "shock_bubble", 100, 40)
    U1, U2, phi = g.case_init("twofluid", "shock_bubble", desc)
    m = g.method(fs="MUSCL", gfm="riemannGFM", itm="LS5", CFL=0.6, T=T)

    def aborts(n):
        try:
            rb.twofluid_state(desc, m, U1, U2, phi, n)
            return False
        except RuntimeError as e:
            assert "GFM_riemann.cpp:37" in str(e), str(e)
            return True
    lo, hi = 0, 3000
    if not aborts(hi):
        raise SystemExit("expected the reference to stop the coarse shock-bubble within %d steps" % hi)
    while hi - lo > 1:
        mid = (lo + hi) // 2
        if aborts(mid):
            hi = mid
        else:
            lo = mid
    out["reference_abort"] = {"case": "shock_bubble", "Nx": 100, "Ny": 40, "gfm": "riemannGFM", "fs": "MUSCL",
                              "itm": "LS5", "CFL": 0.6, "clean_steps": lo, "abort_step": hi,
                              "assert": "sourcecode/GFM_riemann.cpp:37 is_physical_state(grid1[i][j])"}
    json.dump(out, open(OUT, "w"), indent=1, sort_keys=True)
    print(len(out["cases"]), "cases ->", OUT)


if __name__ == "__main__":
    main()
