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
