"""Batched instances (gfm_batch): each instance of a batch stepped through a
recorded CUDA graph, or one after another, ends bit-identical to the same
instance stepped alone and to the oracle; the graph's device-side choice of
reinitialisation steps matches the host's."""
import numpy as np
import pytest

import gfm_gb300 as g
import oracle_binding as orc

pytestmark = pytest.mark.gpu

MEMBERS = [  # Nx, Ny, Mach, bubble gamma, density ratio, radius / height
    (96, 48, 1.22, 1.648, 0.182, 0.25),
    (64, 64, 2.5, 1.09, 5.0, 0.2),
    (128, 64, 1.6, 1.4, 0.5, 0.3),
]


def members():
    return [g.shock_bubble_case(*p) for p in MEMBERS]


@pytest.mark.parametrize("graph", [True, False])
@pytest.mark.parametrize("reinit_every,nsteps", [(1, 12), (3, 21)])
def test_batch_matches_single_and_oracle(graph, reinit_every, nsteps):
    cases = members()
    m = g.method(gfm="riemannGFM", CFL=0.6, T=1.0, reinit_every=reinit_every)
    b = g.Batch([c[0] for c in cases], two_fluid=True)
    for ctx, (d, T, U1, U2, phi) in zip(b.instances, cases):
        ctx.upload(U1, U2, phi)
    b.step(m, nsteps, graph=graph)
    b.synchronize()
    outs = [ctx.download() for ctx in b.instances]
    times = [ctx.time() for ctx in b.instances]
    stats = [ctx.status() for ctx in b.instances]
    b.close()
    for k, (d, T, U1, U2, phi) in enumerate(cases):
        single = g.Context(d, two_fluid=True)
        single.upload(U1, U2, phi)
        single.step(m, nsteps)
        S = single.download()
        ts = single.time()
        single.close()
        for a, c in zip(outs[k], S):
            assert np.array_equal(a, c), "instance %d differs from its single run" % k
        assert times[k][:2] == ts[:2] and times[k][1] == nsteps
        assert stats[k] == 0
        if k == 0:   # one member against the oracle as well
            ref = orc.twofluid_run(d, m, U1, U2, phi, nsteps)
            assert np.array_equal(outs[k][0], ref["U1"]) and np.array_equal(outs[k][1], ref["U2"])
            assert np.array_equal(outs[k][2], ref["phi"])


def test_batch_graph_after_single_calls():
    """Work issued on an instance stream (an upload, single steps) is ordered
    before the batched graph and the graph before later downloads; the batch
    stream here is the legacy default stream, from which no graph can be
    recorded (the batch records from its own stream and replays on this one)."""
    cases = members()
    m = g.method(gfm="riemannGFM", CFL=0.6, T=1.0)
    b = g.Batch([c[0] for c in cases], two_fluid=True, stream=0)
    for ctx, (d, T, U1, U2, phi) in zip(b.instances, cases):
        ctx.upload(U1, U2, phi)
        ctx.step(m, 3)                      # single-instance steps on the instance stream
    b.step(m, 16, graph=True)               # two graph replays
    outs = [ctx.download() for ctx in b.instances]
    b.close()
    for k, (d, T, U1, U2, phi) in enumerate(cases):
        ref = orc.twofluid_run(d, m, U1, U2, phi, 19)
        assert np.array_equal(outs[k][0], ref["U1"]) and np.array_equal(outs[k][2], ref["phi"])


def test_batch_vof_graph_matches_single():
    """GFM_VOF with the VOF tracker through the recorded graph: the sweep
    order of the advection follows the step number on the device, so every
    replay is right; each instance ends as it would alone, states generated
    on the device."""
    import ctypes
    m = g.method(gfm="VOFGFM", itm="PYVOF", CFL=0.5, T=1.0)
    params = [g.BubbleParams(*p[2:]) for p in MEMBERS]
    descs = [g.shock_bubble_case(*p)[0] for p in MEMBERS]
    b = g.Batch(descs, two_fluid=True)
    for ctx, p in zip(b.instances, params):
        ctx.init_shock_bubble_device(p, itm="PYVOF")
    b.step(m, 17, graph=True)
    b.synchronize()
    outs = [ctx.download() for ctx in b.instances]
    b.close()
    for k, (d, p) in enumerate(zip(descs, params)):
        single = g.Context(d, two_fluid=True)
        single.init_shock_bubble_device(p, itm="PYVOF")
        single.step(m, 17)
        S = single.download()
        single.close()
        for a, c in zip(outs[k], S):
            assert np.array_equal(a, c), "VOF instance %d differs from its single run" % k


@pytest.mark.parametrize("shape", ["32x8", "16x16", "64x4", "16x32"])
def test_flux_tile_shapes_match_oracle(shape):
    """Every tile shape of the flux update gives the oracle's bits (each face
    flux is formed once and each cell sums its faces in the reference's
    order, whatever the tiling)."""
    desc, T = g.case_params("twofluid", "shock_bubble", 80, 32)
    U1, U2, phi = g.case_init("twofluid", "shock_bubble", desc)
    for fs in ("MUSCL", "Godunov"):
        m = g.method(fs=fs, gfm="riemannGFM", CFL=0.6, T=T)
        ctx = g.Context(desc, two_fluid=True)
        ctx.set_overlap("off")
        ctx.set_flux_tile(shape)
        ctx.upload(U1, U2, phi)
        ctx.step(m, 12)
        G = ctx.download()
        st = ctx.status()
        ctx.close()
        ref = orc.twofluid_run(desc, m, U1, U2, phi, 12)
        assert st == 0
        assert np.array_equal(G[0], ref["U1"]) and np.array_equal(G[1], ref["U2"]) and np.array_equal(G[2], ref["phi"])
    d1, T1 = g.case_params("onefluid", "circularexplosion", 72, 40)
    U, _, _ = g.case_init("onefluid", "circularexplosion", d1)
    m1 = g.method(fs="MUSCL", CFL=0.8, T=T1)
    c1 = g.Context(d1, two_fluid=False)
    c1.set_flux_tile(shape)
    c1.upload(U)
    c1.step(m1, 15)
    G1, _, _ = c1.download()
    c1.close()
    R, _, _, _ = orc.onefluid_run(d1, m1, U, 15)
    assert np.array_equal(G1, R)


@pytest.mark.parametrize("reinit_every,nsteps", [(1, 12), (3, 21)])
def test_phased_batch_matches_single(reinit_every, nsteps):
    """The phased schedule (every instance up to its flux update, one
    persistent flux launch per tile shape over all instances, every
    instance's commit), recorded into a graph for 8 steps and issued directly
    for the rest, with mixed tile shapes: each instance ends bit-identical to
    the same instance stepped alone."""
    cases = members()
    m = g.method(gfm="riemannGFM", CFL=0.6, T=1.0, reinit_every=reinit_every)
    b = g.Batch([c[0] for c in cases], two_fluid=True)
    b.set_schedule("phased")
    for ctx, shape, (d, T, U1, U2, phi) in zip(b.instances, ["16x16", "64x4", "32x8"], cases):
        ctx.set_flux_tile(shape)
        ctx.upload(U1, U2, phi)
    b.step(m, nsteps, graph=True)
    b.synchronize()
    outs = [ctx.download() for ctx in b.instances]
    stats = [ctx.status() for ctx in b.instances]
    times = [ctx.time()[:2] for ctx in b.instances]
    b.close()
    for k, (d, T, U1, U2, phi) in enumerate(cases):
        single = g.Context(d, two_fluid=True)
        single.upload(U1, U2, phi)
        single.step(m, nsteps)
        S = single.download()
        ts = single.time()[:2]
        single.close()
        assert stats[k] == 0 and times[k] == ts
        for a, c in zip(outs[k], S):
            assert np.array_equal(a, c), "instance %d differs from its single run" % k


def test_autotune_keeps_the_state_and_the_results():
    """gfm_batch_autotune times tile shapes per size class and the two
    schedules on the batch's state, restores it, and keeps the fastest: the
    run continues bit-identically to an untuned one."""
    cases = members()
    m = g.method(gfm="riemannGFM", CFL=0.6, T=1.0)
    b = g.Batch([c[0] for c in cases], two_fluid=True)
    for ctx, (d, T, U1, U2, phi) in zip(b.instances, cases):
        ctx.upload(U1, U2, phi)
    b.step(m, 3, graph=False)
    report = b.autotune(m, steps=8)
    b.step(m, 9, graph=True)
    b.synchronize()
    outs = [ctx.download() for ctx in b.instances]
    times = [ctx.time()[:2] for ctx in b.instances]
    b.close()
    assert report["schedule"] in ("streams", "phased") and report["steps"] == 8
    assert len(report["classes"]) >= 1
    for c in report["classes"]:
        assert c["tile"] in ("32x8", "16x16", "64x4", "16x32") and min(c["ms_per_step"].values()) > 0
    for k, (d, T, U1, U2, phi) in enumerate(cases):
        single = g.Context(d, two_fluid=True)
        single.upload(U1, U2, phi)
        single.step(m, 12)
        S = single.download()
        ts = single.time()[:2]
        single.close()
        assert times[k] == ts
        for a, c in zip(outs[k], S):
            assert np.array_equal(a, c), "instance %d differs after tuning" % k
