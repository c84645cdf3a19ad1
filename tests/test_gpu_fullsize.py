"""Parity of the CUDA path with the CPU oracle at the benchmark configurations'
full sizes: C1 (one-fluid circular explosion, 200x200, run to T = 0.25),
C2 (shock-bubble 1000x400, Riemann GFM, overlapped schedule) and C3
(underwater explosion 800x800, real GFM, reinitialisation every 5 steps),
over as many steps as the oracle finishes in seconds.  Bar: rel-L1 <= 1e-10
per conserved field of the composite state and for phi, then bit equality;
interfacial counts exact."""
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


def test_c1_circular_explosion_to_end_time():
    """CFL 0.4, the value of the reference's own settings files: 132 steps to T."""
    desc, T = g.case_params("onefluid", "circularexplosion", 200, 200)
    assert T == 0.25
    U, _, _ = g.case_init("onefluid", "circularexplosion", desc)
    m = g.method(fs="MUSCL", CFL=0.4, T=T)
    ctx = g.Context(desc, two_fluid=False)
    ctx.upload(U)
    t = 0.0
    while t < T:
        ctx.step(m, 50)
        t, n, _ = ctx.time()
    G, _, _ = ctx.download()
    st = ctx.status()
    ctx.close()
    orc.clear_status()
    R, tr, nr_, _ = orc.onefluid_run(desc, m, U, n + 10)   # the oracle stops at T by itself
    assert nr_ == n and tr == t and t >= T
    for k in range(4):
        assert rel_l1(real(desc, G[k]), real(desc, R[k])) <= TOL
    assert np.array_equal(G, R)
    assert st == 0 and orc.status() == 0


def test_c1_cfl_08_diverges_identically():
    """At CFL 0.8 the unsplit MUSCL-Hancock update with the reference's dt
    (CFL min(dx/max(|u|+c), dy/max(|v|+c)), sourcecode/sim_onefluid.cpp:68-91)
    is unstable: the oracle's state turns non-finite at step 23.  The GPU
    follows it step for step."""
    desc, T = g.case_params("onefluid", "circularexplosion", 200, 200)
    U, _, _ = g.case_init("onefluid", "circularexplosion", desc)
    m = g.method(fs="MUSCL", CFL=0.8, T=T)
    for nsteps in (22, 30):
        ctx = g.Context(desc, two_fluid=False)
        ctx.upload(U)
        ctx.step(m, nsteps)
        G, _, _ = ctx.download()
        st = ctx.status()
        ctx.close()
        orc.clear_status()
        R, _, _, _ = orc.onefluid_run(desc, m, U, nsteps)
        assert np.array_equal(G, R, equal_nan=True)
        if nsteps == 22:
            assert np.isfinite(G).all() and st == 0 and orc.status() == 0
        else:
            assert not np.isfinite(G).all() and st != 0 and orc.status() != 0


@pytest.mark.parametrize("case,Nx,Ny,gfm,cfl,reinit,nsteps", [
    ("shock_bubble", 1000, 400, "riemannGFM", 0.6, 1, 8),
    ("underwater_explosion_sg", 800, 800, "realGFM", 0.5, 5, 6),
])
def test_twofluid_full_size(case, Nx, Ny, gfm, cfl, reinit, nsteps):
    desc, T = g.case_params("twofluid", case, Nx, Ny)
    U1, U2, phi = g.case_init("twofluid", case, desc)
    m = g.method(gfm=gfm, CFL=cfl, T=T, reinit_every=reinit)
    ctx = g.Context(desc, two_fluid=True)
    ctx.upload(U1, U2, phi)
    ctx.step(m, nsteps)
    G1, G2, Gphi = ctx.download()
    stats = ctx.stats()
    t, n, _ = ctx.time()
    st = ctx.status()
    ctx.close()
    orc.clear_status()
    ref = orc.twofluid_run(desc, m, U1, U2, phi, nsteps)
    assert n == ref["numsteps"] == nsteps and t == ref["t"]
    sgn = real(desc, Gphi) <= 0.0
    sref = real(desc, ref["phi"]) <= 0.0
    for k in range(4):
        comp_gpu = np.where(sgn, real(desc, G1[k]), real(desc, G2[k]))
        comp_ref = np.where(sref, real(desc, ref["U1"][k]), real(desc, ref["U2"][k]))
        assert rel_l1(comp_gpu, comp_ref) <= TOL
    assert rel_l1(real(desc, Gphi), real(desc, ref["phi"])) <= TOL
    assert stats["n_interfacial"] == ref["n_interfacial"]
    assert np.array_equal(G1, ref["U1"]) and np.array_equal(G2, ref["U2"]) and np.array_equal(Gphi, ref["phi"])
    assert st == 0 and orc.status() == 0
