"""Failure detection.  The reference's only error convention is a live
assert that aborts the run: an unphysical state at the flux update
(sourcecode/FS_MUSCL.cpp:167, headers/euler_misc.hpp:99-100), dt <= 0
(sourcecode/sim_twofluid.cpp:155), and a message for a NaN star pressure
(sourcecode/GFM_real.cpp:173-176).  Here kernels OR bits into a device status
word that the host reads after the step, and the context stays usable.

Every failure is made on the host: a poisoned cell in a host initial
condition, a Newton limit set through the C ABI, and an interface-list entry
that the interface loop leaves unpublished so that its dependants' bounded
waits run out.  No test faults, traps or hangs the GPU: device indices
computed from field values are clamped to the grid, and every wait polls a
bounded number of times.  The oracle flags the same conditions where it has
them."""
import numpy as np
import pytest

import gfm_gb300 as g
import oracle_binding as orc

pytestmark = pytest.mark.gpu

ST_UNPHYSICAL = 1 << 0
ST_NEWTON = 1 << 1
ST_DT = 1 << 4
ST_SCHEDULE = 1 << 5


def shock_bubble(nx=96, ny=40):
    desc, T = g.case_params("twofluid", "shock_bubble", nx, ny)
    U1, U2, phi = g.case_init("twofluid", "shock_bubble", desc)
    return desc, T, U1, U2, phi


def poison_rho(U, desc, i_real, j_real):
    """Negate the density of one real cell (rho < 0, e < 0 where the
    reference asserts): 47 cells from the bubble of the 96 x 40 case."""
    U = U.copy()
    gc = desc.numGC
    U[0, gc + i_real, gc + j_real] *= -1.0
    return U


def interior(desc):
    gc = desc.numGC
    return slice(gc, gc + desc.Ny), slice(gc, gc + desc.Nx)


@pytest.mark.parametrize("overlap", ["off", "auto"])
def test_negative_density_sets_unphysical(overlap):
    desc, T, U1, U2, phi = shock_bubble()
    U2p = poison_rho(U2, desc, 20, 10)   # ambient gas (fluid 2) at x ~ 0.026
    m = g.method(fs="MUSCL", gfm="riemannGFM", itm="LS5", CFL=0.6, T=T)
    ctx = g.Context(desc, two_fluid=True)
    ctx.set_overlap(overlap)
    ctx.upload(U1, U2p, phi)
    ctx.step(m, 1)
    st = ctx.status()
    t, n, _ = ctx.time()
    # the context stays usable: a clean state steps without a status bit
    ctx.clear_status()
    ctx.upload(U1, U2, phi)
    ctx.step(m, 2)
    st_clean = ctx.status()
    G1, G2, Gphi = ctx.download()
    ctx.close()
    assert st & ST_UNPHYSICAL
    assert n == 1 and t > 0.0
    assert st_clean == 0
    orc.clear_status()
    ref = orc.twofluid_run(desc, m, U1, U2p, phi, 1)
    assert orc.status() & ST_UNPHYSICAL
    orc.clear_status()
    ref = orc.twofluid_run(desc, m, U1, U2, phi, 2)
    assert np.array_equal(G1, ref["U1"]) and np.array_equal(G2, ref["U2"]) and np.array_equal(Gphi, ref["phi"])


def test_newton_limit_sets_no_converge():
    desc, T, U1, U2, phi = shock_bubble()
    m = g.method(fs="MUSCL", gfm="riemannGFM", itm="LS5", CFL=0.6, T=T)
    ctx = g.Context(desc, two_fluid=True)
    ctx.upload(U1, U2, phi)
    ctx.set_newton_limit(1)      # every solve that needs a second iteration stops after one
    ctx.step(m, 1)
    st = ctx.status()
    ctx.clear_status()
    ctx.set_newton_limit(60)     # the default again: the same step is clean and matches the oracle
    ctx.upload(U1, U2, phi)
    ctx.step(m, 3)
    st_clean = ctx.status()
    G1, G2, Gphi = ctx.download()
    ctx.close()
    assert st & ST_NEWTON
    assert st_clean == 0
    ref = orc.twofluid_run(desc, m, U1, U2, phi, 3)
    assert np.array_equal(G1, ref["U1"]) and np.array_equal(G2, ref["U2"]) and np.array_equal(Gphi, ref["phi"])


def test_newton_limit_rejects_bad_values():
    desc, T, U1, U2, phi = shock_bubble(32, 16)
    ctx = g.Context(desc, two_fluid=True)
    for bad in (0, -3, 5000):
        with pytest.raises(g.GFMError):
            ctx.set_newton_limit(bad)
    ctx.close()


@pytest.mark.parametrize("overlap", ["off", "auto"])
def test_infinite_wave_speed_gives_nonpositive_dt(overlap):
    """A cell with infinite energy has an infinite sound speed, so the CFL
    step is CFL * min(dx / inf, dy / inf) = 0: the reference's assert(dt > 0)
    (sourcecode/sim_twofluid.cpp:151-155)."""
    desc, T, U1, U2, phi = shock_bubble()
    gc = desc.numGC
    U2p = U2.copy()
    U2p[3, gc + 20, gc + 10] = np.inf    # ambient gas, far from the bubble
    m = g.method(fs="MUSCL", gfm="riemannGFM", itm="LS5", CFL=0.6, T=T)
    ctx = g.Context(desc, two_fluid=True)
    ctx.set_overlap(overlap)
    ctx.upload(U1, U2p, phi)
    ctx.step(m, 1)
    st = ctx.status()
    _, _, dt = ctx.time()
    ctx.close()
    assert st & ST_DT
    assert dt == 0.0
    orc.clear_status()
    orc.twofluid_run(desc, m, U1, U2p, phi, 1)
    assert orc.status() & ST_DT


@pytest.mark.parametrize("overlap", ["off", "auto"])
def test_interface_wait_runs_out_and_returns(overlap):
    """The interface loop's first entry is withheld: the cells that read it
    give up after their bounded waits, the kernel returns, the status says
    so, and the context steps correctly once the hook is cleared."""
    desc, T, U1, U2, phi = shock_bubble()
    m = g.method(fs="MUSCL", gfm="riemannGFM", itm="LS5", CFL=0.6, T=T)
    ctx = g.Context(desc, two_fluid=True)
    ctx.set_overlap(overlap)
    ctx.upload(U1, U2, phi)
    ctx.set_interface_wait(spin_limit=1 << 12, withheld_entry=0)
    ctx.step(m, 1)
    st = ctx.status()
    ctx.set_interface_wait(0, -1)
    ctx.clear_status()
    ctx.upload(U1, U2, phi)
    ctx.step(m, 2)
    st_clean = ctx.status()
    G1, G2, Gphi = ctx.download()
    ctx.close()
    assert st & ST_SCHEDULE
    assert st_clean == 0
    ref = orc.twofluid_run(desc, m, U1, U2, phi, 2)
    assert np.array_equal(G1, ref["U1"]) and np.array_equal(G2, ref["U2"]) and np.array_equal(Gphi, ref["phi"])


@pytest.mark.parametrize("graph", [True, False])
def test_poisoned_batch_instance_leaves_the_others_intact(graph):
    members = [(96, 48, 1.22, 1.648, 0.182, 0.25), (96, 40, 1.6, 1.4, 0.5, 0.2), (64, 64, 2.5, 1.09, 5.0, 0.2)]
    cases = [g.shock_bubble_case(*p) for p in members]
    m = g.method(gfm="riemannGFM", CFL=0.6, T=1.0)
    b = g.Batch([c[0] for c in cases], two_fluid=True)
    for k, (ctx, (d, T, U1, U2, phi)) in enumerate(zip(b.instances, cases)):
        ctx.upload(U1, poison_rho(U2, d, 20, 8) if k == 1 else U2, phi)
    b.step(m, 3, graph=graph)
    b.synchronize()
    outs = [ctx.download() for ctx in b.instances]
    stats = [ctx.status() for ctx in b.instances]
    b.close()
    assert stats[1] & ST_UNPHYSICAL
    for k in (0, 2):
        d, T, U1, U2, phi = cases[k]
        assert stats[k] == 0
        single = g.Context(d, two_fluid=True)
        single.upload(U1, U2, phi)
        single.step(m, 3)
        S = single.download()
        single.close()
        for a, c in zip(outs[k], S):
            assert np.array_equal(a, c), "instance %d changed by its poisoned neighbour" % k
