"""The configured runs at their configured lengths on the GPU, against digests
made by the REFERENCE'S OWN CODE.

tests/golden/fulllength_digests.json holds, per run, what the reference
checker (murraycutforth/PhD-2D-GFM's sources compiled unchanged against the
oracle's stand-ins for its absent libraries; oracle/build_ref.py) computed
over the whole run, confirmed by the CPU oracle (tests/golden/make_digests.py):
the step count, t, a SHA-256 of every field's real cells and of the final
interfacial-cell mask.  The GPU steps the same runs through the C ABI and
must reproduce every digest bit for bit: the 1000 x 400 shock-bubble for 2000
steps (both schedules), the 800 x 800 underwater explosion for 1500 steps,
the shock-bubble with GFM_VOF for 2000 steps, the one-fluid circular
explosion to its end time, and four members of the 64-instance batch, stepped
for 1000 steps as part of the whole batch after the autotuner has chosen
tile shapes and the schedule.
"""
import json
import os
import sys

import numpy as np
import pytest

import gfm_gb300 as g
import oracle_binding as orc

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "golden"))
import make_digests as md  # noqa: E402

pytestmark = pytest.mark.gpu
RUNS = json.load(open(os.path.join(HERE, "golden", "fulllength_digests.json")))["runs"]
SINGLE = sorted(k for k in RUNS if not k.startswith("batch_member"))
MEMBERS = sorted(k for k in RUNS if k.startswith("batch_member"))


def compare(d, gold):
    assert d["numsteps"] == gold["numsteps"], (d["numsteps"], gold["numsteps"])
    assert d["t"] == gold["t"], "t %s, reference %s" % (float.fromhex(d["t"]), float.fromhex(gold["t"]))
    bad = {}
    for name, f in gold["fields"].items():
        mine = d["fields"][name]
        if mine["sha256"] != f["sha256"]:
            den = f["abs_sum"] if f["abs_sum"] > 0 else 1.0
            bad[name] = abs(mine["abs_sum"] - f["abs_sum"]) / den
    assert not bad, "fields differ from the reference (relative difference of |x| sums): %r" % bad
    if "mask_sha256" in gold:
        assert d["mask_sha256"] == gold["mask_sha256"]


def digest_of(ctx, desc, vof):
    G1, G2, Gphi = ctx.download()
    t, n, _ = ctx.time()
    mask = None if vof else orc.interfacial_mask(desc, Gphi)
    return md.digest(desc, G1, G2, Gphi, mask, t, n)


def run_single(name, overlap):
    gold = RUNS[name]
    r = gold["run"]
    desc, m, U1, U2, phi = md.initial_state(r)
    if r["sim"] == "onefluid":
        ctx = g.Context(desc, two_fluid=False)
        ctx.upload(U1)
        # the run ends at its end time: steps past it change nothing
        ctx.step(m, gold["numsteps"])
        G, _, _ = ctx.download()
        ctx.step(m, 4)
        G_after, _, _ = ctx.download()
        t, n, _ = ctx.time()
        st = ctx.status()
        ctx.close()
        assert np.array_equal(G, G_after)
        return md.digest(desc, G, None, None, None, t, n), st
    ctx = g.Context(desc, two_fluid=True)
    ctx.set_overlap(overlap)
    ctx.upload(U1, U2, phi)
    ctx.step(m, r["steps"])
    d = digest_of(ctx, desc, r["itm"] == "PYVOF")
    st = ctx.status()
    ctx.close()
    return d, st


@pytest.mark.parametrize("name", SINGLE)
def test_full_length_run_matches_reference_code(name):
    d, st = run_single(name, "auto")
    compare(d, RUNS[name])
    assert st == 0


@pytest.mark.parametrize("name", [n for n in SINGLE if n == "shock_bubble_2000"])
def test_full_length_one_stream_schedule_matches_reference_code(name):
    d, st = run_single(name, "off")
    compare(d, RUNS[name])
    assert st == 0


@pytest.mark.skipif(not MEMBERS, reason="no batch member digests")
def test_tuned_batch_members_match_reference_code():
    """The whole 64-instance batch after gfm_batch_autotune, 1000 steps
    through the recorded graph; the members with digests must match them."""
    import bench
    spec = bench.batch_members()
    cases = [g.shock_bubble_case(*p) for p in spec]
    m = g.method(gfm="riemannGFM", CFL=0.6, T=1.0)
    b = g.Batch([c[0] for c in cases], two_fluid=True)
    for ctx, (d, T, U1, U2, phi) in zip(b.instances, cases):
        ctx.upload(U1, U2, phi)
    report = b.autotune(m, steps=8)
    steps = {RUNS[n]["run"]["steps"] for n in MEMBERS}
    assert len(steps) == 1
    b.step(m, steps.pop(), graph=True)
    b.synchronize()
    results = {}
    for name in MEMBERS:
        r = RUNS[name]["run"]
        k = r["member"]
        assert list(spec[k]) == r["params"]
        ctx = b.instances[k]
        results[name] = (digest_of(ctx, cases[k][0], False), ctx.status())
    b.close()
    assert report["schedule"] in ("streams", "phased")
    for name, (d, st) in results.items():
        compare(d, RUNS[name])
        assert st == 0, name
