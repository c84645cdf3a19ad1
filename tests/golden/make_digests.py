"""Generates tests/golden/fulllength_digests.json: digests of the configured
runs at their configured lengths, computed by the REFERENCE'S OWN CODE (the
checker oracle/_ref/gfm_ref, built from murraycutforth/PhD-2D-GFM's sources
by oracle/build_ref.py) and, with --oracle, confirmed by the CPU oracle.

    python tests/golden/make_digests.py [--oracle] [--jobs N] [--only NAME ...]

Runs (initial conditions from the library's host set-up, gfm_case_init):
  shock_bubble_2000     1000 x 400 shock-bubble, Riemann GFM, LS5, MUSCL,
                        CFL 0.6, 2000 steps (sourcecode/sim_twofluid.cpp:64-88)
  underwater_1500       800 x 800 underwater explosion, real GFM, LS5 with
                        reinitialisation every 5 steps, MUSCL, CFL 0.5, 1500 steps
  shock_bubble_vof_2000 the shock-bubble with GFM_VOF and the VOF tracker
  circular_explosion    200 x 200 one-fluid circular explosion, MUSCL, CFL 0.4,
                        to t = 0.25
  batch_member_K        four members of the 64-instance shock-bubble batch
                        (seeded family, smallest / two middle / largest), 1000 steps

Per run: the step count, t (as a hex float), and per field (U1's and U2's
four planes, phi) the SHA-256 of the real cells' float64 bytes (row-major,
little-endian) and the sum of their magnitudes; the interfacial mask's SHA-256.
Several runs take tens of minutes of one CPU core each (the checker steps
about 0.5 M cell-updates per second); they run in parallel processes.
"""
import argparse
import concurrent.futures as cf
import hashlib
import json
import multiprocessing as mp
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
OUT = os.path.join(HERE, "fulllength_digests.json")


def _paths():
    for p in (os.path.join(ROOT, "phd-2d-gfm_gb300"), os.path.join(ROOT, "oracle"), ROOT):
        if p not in sys.path:
            sys.path.insert(0, p)


def runs():
    _paths()
    import bench
    spec = bench.batch_members()
    order = sorted(range(len(spec)), key=lambda k: spec[k][0] * spec[k][1])
    picks = {"batch_member_smallest": order[0], "batch_member_mid_a": order[len(order) // 3],
             "batch_member_mid_b": order[2 * len(order) // 3], "batch_member_largest": order[-1]}
    out = {
        "shock_bubble_2000": {"sim": "twofluid", "case": "shock_bubble", "Nx": 1000, "Ny": 400, "gfm": "riemannGFM",
                              "fs": "MUSCL", "itm": "LS5", "CFL": 0.6, "reinit_every": 1, "steps": 2000},
        "underwater_1500": {"sim": "twofluid", "case": "underwater_explosion_sg", "Nx": 800, "Ny": 800,
                            "gfm": "realGFM", "fs": "MUSCL", "itm": "LS5", "CFL": 0.5, "reinit_every": 5,
                            "steps": 1500},
        "shock_bubble_vof_2000": {"sim": "twofluid", "case": "shock_bubble", "Nx": 1000, "Ny": 400, "gfm": "VOFGFM",
                                  "fs": "MUSCL", "itm": "PYVOF", "CFL": 0.6, "reinit_every": 0, "steps": 2000},
        "circular_explosion": {"sim": "onefluid", "case": "circularexplosion", "Nx": 200, "Ny": 200, "fs": "MUSCL",
                               "CFL": 0.4, "steps": 100000},
    }
    for name, k in picks.items():
        nx, ny, mach, gb, rr, rf = spec[k]
        out[name] = {"sim": "twofluid", "case": "batch_member", "member": k, "params": [nx, ny, mach, gb, rr, rf],
                     "Nx": nx, "Ny": ny, "gfm": "riemannGFM", "fs": "MUSCL", "itm": "LS5", "CFL": 0.6,
                     "reinit_every": 1, "steps": 1000}
    return out


def initial_state(r):
    """(desc, method, U1, U2, phi) of a run from the library's host set-up."""
    _paths()
    import gfm_gb300 as g
    if r["sim"] == "onefluid":
        desc, T = g.case_params("onefluid", r["case"], r["Nx"], r["Ny"])
        U, _, _ = g.case_init("onefluid", r["case"], desc)
        return desc, g.method(fs=r["fs"], CFL=r["CFL"], T=T), U, None, None
    if r["case"] == "batch_member":
        desc, T, U1, U2, phi = g.shock_bubble_case(*r["params"])
        if r["itm"] == "PYVOF":
            phi = g.shock_bubble_case_z(desc, *r["params"][2:])
    else:
        desc, T = g.case_params("twofluid", r["case"], r["Nx"], r["Ny"])
        U1, U2, phi = g.case_init("twofluid", r["case"], desc)
        if r["itm"] == "PYVOF":
            phi = g.case_init_z(r["case"], desc)
    m = g.method(fs=r["fs"], gfm=r["gfm"], itm=r["itm"], CFL=r["CFL"], T=T, reinit_every=r["reinit_every"])
    return desc, m, U1, U2, phi


def digest(desc, U1, U2, phi, mask, t, numsteps, mask_fill=None, realcells=None):
    g = desc.numGC
    sl = (slice(g, g + desc.Ny), slice(g, g + desc.Nx))
    fields = {}
    named = [("U1_%d" % k, U1[k]) for k in range(4)]
    if U2 is not None:
        named += [("U2_%d" % k, U2[k]) for k in range(4)] + [("phi", phi)]
    for name, a in named:
        real = np.ascontiguousarray(a[sl], dtype="<f8")
        fields[name] = {"sha256": hashlib.sha256(real.tobytes()).hexdigest(), "abs_sum": float(np.abs(real).sum())}
    out = {"numsteps": int(numsteps), "t": float(t).hex(), "fields": fields}
    if mask is not None:
        out["mask_sha256"] = hashlib.sha256(np.ascontiguousarray(mask[sl], dtype=np.uint8).tobytes()).hexdigest()
    if mask_fill is not None:
        m = np.ascontiguousarray(mask_fill[sl], dtype=np.uint8)
        out["ghost_fill_mask_sha256"] = hashlib.sha256(m.tobytes()).hexdigest()
        out["ghost_fill_mask_count"] = int(m.sum())
    if realcells is not None:
        out["realcells"] = [list(realcells[0]), list(realcells[1])]
    return out


def run_one(args):
    name, r, use_oracle = args
    _paths()
    import ref_binding as rb
    desc, m, U1, U2, phi = initial_state(r)
    t0 = time.time()
    if r["sim"] == "onefluid":
        res = rb.onefluid_state(desc, m, U1, r["steps"])
        d = digest(desc, res["U1"], None, None, None, res["t"], res["numsteps"])
    else:
        res = rb.twofluid_state(desc, m, U1, U2, phi, r["steps"])
        d = digest(desc, res["U1"], res["U2"], res["phi"], res["mask"] if r["itm"] != "PYVOF" else None, res["t"],
                   res["numsteps"])
    d["checker_seconds"] = round(time.time() - t0, 1)
    if use_oracle:
        import oracle_binding as orc
        if r["sim"] == "onefluid":
            U, t, n, _ = orc.onefluid_run(desc, m, U1, r["steps"])
            o = digest(desc, U, None, None, None, t, n)
        else:
            o = orc.twofluid_run(desc, m, U1, U2, phi, r["steps"])
            mask = orc.interfacial_mask(desc, o["phi"]) if r["itm"] != "PYVOF" else None
            o = digest(desc, o["U1"], o["U2"], o["phi"], mask, o["t"], o["numsteps"])
        d["oracle_agrees"] = o["fields"] == d["fields"] and o["numsteps"] == d["numsteps"] and o["t"] == d["t"] and \
            o.get("mask_sha256") == d.get("mask_sha256")
    d["run"] = r
    return name, d


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--oracle", action="store_true", help="confirm each digest with the CPU oracle")
    ap.add_argument("--jobs", type=int, default=os.cpu_count())
    ap.add_argument("--only", nargs="*")
    a = ap.parse_args()
    _paths()
    import build_ref
    if build_ref.build() is None:
        sys.exit("the reference's sources are absent: the checker cannot be built")
    todo = runs()
    if a.only:
        todo = {k: v for k, v in todo.items() if k in a.only}
    old = json.load(open(OUT)) if os.path.exists(OUT) else {}
    results = dict(old.get("runs", {}))
    # the longest runs first
    items = sorted(todo.items(), key=lambda kv: -kv[1]["Nx"] * kv[1]["Ny"] * min(kv[1]["steps"], 2000))
    ctx = mp.get_context("spawn")
    with cf.ProcessPoolExecutor(max_workers=a.jobs, mp_context=ctx) as ex:
        for name, d in ex.map(run_one, [(n, r, a.oracle) for n, r in items]):
            results[name] = d
            print(name, d["numsteps"], d.get("checker_seconds"), d.get("oracle_agrees"), flush=True)
            json.dump({"generator": "tests/golden/make_digests.py (reference checker oracle/_ref/gfm_ref)",
                       "runs": results}, open(OUT, "w"), indent=1, sort_keys=True)


if __name__ == "__main__":
    main()
