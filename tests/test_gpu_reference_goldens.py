"""The CUDA path against digests made by the REFERENCE'S OWN CODE.

tests/golden/reference_goldens.json holds, per case, what the reference
checker (murraycutforth/PhD-2D-GFM's sources compiled unchanged against the
oracle's stand-ins for its absent libraries; oracle/build_ref.py) computed:
SHA-256 digests of every field's real cells, the step count, t, the
interfacial-cell mask of the last ghost fill and the realcells boxes.  The GPU
runs the same case through the C ABI and must reproduce them bit for bit
(which implies the parity bar, relative L1 <= 1e-10); on a mismatch the
message gives each differing field's relative difference of magnitude sums.
"""
import json
import os
import sys

import numpy as np
import pytest

import gfm_gb300 as g

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "golden"))
import make_digests as md  # noqa: E402

pytestmark = pytest.mark.gpu
GOLD = json.load(open(os.path.join(HERE, "golden", "reference_goldens.json")))


def _id(c):
    s = c["spec"]
    return "-".join(str(s[k]) for k in ("case", "Nx", "Ny", "gfm", "fs", "itm", "steps") if k in s) + \
        ("-ext" if s.get("ext") else "") + ("-slip" if s.get("slip") else "")


def run_gpu(spec, overlap="auto"):
    """The case on the GPU; returns its digest and the device status."""
    if spec["sim"] == "onefluid":
        desc, T = g.case_params("onefluid", spec["case"], spec["Nx"], spec["Ny"])
        U, _, _ = g.case_init("onefluid", spec["case"], desc)
        m = g.method(fs=spec["fs"], CFL=spec["CFL"], T=T)
        ctx = g.Context(desc, two_fluid=False)
        ctx.upload(U)
        ctx.step(m, spec["steps"])
        G, _, _ = ctx.download()
        t, n, _ = ctx.time()
        st = ctx.status()
        ctx.close()
        return md.digest(desc, G, None, None, None, t, n), st
    desc, T = g.case_params("twofluid", spec["case"], spec["Nx"], spec["Ny"])
    U1, U2, phi = g.case_init("twofluid", spec["case"], desc)
    vof = spec["itm"] == "PYVOF"
    if vof:
        phi = g.case_init_z(spec["case"], desc)
    m = g.method(fs=spec["fs"], gfm=spec["gfm"], itm=spec["itm"], CFL=spec["CFL"], T=T,
                 reinit_every=spec["reinit_every"], use_extension_vfield=spec["ext"], use_slip_BCs=spec["slip"])
    ctx = g.Context(desc, two_fluid=True)
    ctx.set_overlap(overlap)
    ctx.upload(U1, U2, phi)
    ctx.step(m, spec["steps"])
    G1, G2, Gphi = ctx.download()
    mask = None if vof else ctx.mask()
    rc = ctx.realcells()
    t, n, _ = ctx.time()
    st = ctx.status()
    ctx.close()
    return md.digest(desc, G1, G2, Gphi, None, t, n, mask, rc), st


def compare(d, gold):
    assert d["numsteps"] == gold["numsteps"]
    assert d["t"] == gold["t"], "t %s, reference %s" % (float.fromhex(d["t"]), float.fromhex(gold["t"]))
    bad = {}
    for name, f in gold["fields"].items():
        mine = d["fields"][name]
        if mine["sha256"] != f["sha256"]:
            den = f["abs_sum"] if f["abs_sum"] > 0 else 1.0
            bad[name] = abs(mine["abs_sum"] - f["abs_sum"]) / den
    assert not bad, "fields differ from the reference (relative difference of |x| sums): %r" % bad
    if "ghost_fill_mask_sha256" in gold:
        assert d["ghost_fill_mask_count"] == gold["ghost_fill_mask_count"]
        assert d["ghost_fill_mask_sha256"] == gold["ghost_fill_mask_sha256"]
    if "realcells" in gold:
        assert d["realcells"] == gold["realcells"]


@pytest.mark.parametrize("gold", GOLD["cases"], ids=_id)
def test_gpu_matches_reference_code(gold):
    d, st = run_gpu(gold["spec"])
    compare(d, gold)
    assert st == 0


@pytest.mark.parametrize("gold", [c for c in GOLD["cases"] if c["spec"]["sim"] == "twofluid"
                                  and c["spec"]["gfm"] in ("riemannGFM", "realGFM")][:6], ids=_id)
def test_one_stream_schedule_matches_reference_code(gold):
    d, st = run_gpu(gold["spec"], overlap="off")
    compare(d, gold)
    assert st == 0


def test_unphysical_state_flagged_where_the_reference_aborts():
    """The reference's assert (sourcecode/GFM_riemann.cpp:37) stops the coarse
    shock-bubble in step 672; the GPU steps 671 steps clean (bit-identical to
    the reference, above) and flags GFM_ST_UNPHYSICAL in step 672."""
    a = GOLD["reference_abort"]
    desc, T = g.case_params("twofluid", a["case"], a["Nx"], a["Ny"])
    U1, U2, phi = g.case_init("twofluid", a["case"], desc)
    m = g.method(fs=a["fs"], gfm=a["gfm"], itm=a["itm"], CFL=a["CFL"], T=T)
    ctx = g.Context(desc, two_fluid=True)
    ctx.upload(U1, U2, phi)
    ctx.step(m, a["clean_steps"])
    st_clean = ctx.status()
    ctx.step(m, 1)
    st = ctx.status()
    ctx.close()
    assert st_clean == 0
    assert st & 1
