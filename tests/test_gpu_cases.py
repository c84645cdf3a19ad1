"""Initial conditions generated on the device (gfm_case_init_device) against
the host set-up: bit-identical grids, level sets and volume fractions (GDA's
Gaussian density within 1 ulp: its exp differs between host and device)."""
import numpy as np
import pytest

import gfm_gb300 as g

pytestmark = pytest.mark.gpu

ONE = ["TTC1_x", "TTC1_y", "TTC2_x", "TTC2_y", "TTC3_x", "TTC4_y", "TTC5_x", "TTC5_y", "circularexplosion"]
TWO = ["circularexplosion", "ST1_x", "ST2_y", "GDA", "shocked_helium_bubble", "shocked_R22_bubble", "shock_bubble",
       "underwater_explosion_sg"]


def _same(a, b, close=False):
    if close:
        return np.allclose(a, b, rtol=4e-16, atol=0.0)
    return np.array_equal(a.view(np.int64), b.view(np.int64))


@pytest.mark.parametrize("case", ONE)
def test_onefluid_device_ic(case):
    d, T = g.case_params("onefluid", case, 37, 29)
    U, _, _ = g.case_init("onefluid", case, d)
    ctx = g.Context(d, two_fluid=False)
    ctx.init_device("onefluid", case)
    V, _, _ = ctx.download()
    assert ctx.time()[:2] == (0.0, 0)
    ctx.close()
    assert _same(V, U)


@pytest.mark.parametrize("case", TWO)
@pytest.mark.parametrize("itm", ["LS5", "PYVOF"])
def test_twofluid_device_ic(case, itm):
    d, T = g.case_params("twofluid", case, 41, 41 if case == "GDA" else 33)   # periodic grids are square
    U1, U2, phi = g.case_init("twofluid", case, d)
    if itm == "PYVOF":
        phi = g.case_init_z(case, d)
    ctx = g.Context(d, two_fluid=True)
    ctx.init_device("twofluid", case, itm=itm)
    V1, V2, f = ctx.download()
    ctx.close()
    close = case == "GDA"
    assert _same(V1, U1, close) and _same(V2, U2, close) and _same(f, phi)


@pytest.mark.parametrize("itm", ["LS5", "PYVOF"])
def test_shock_bubble_family_device_ic(itm):
    d, T, U1, U2, phi = g.shock_bubble_case(192, 96, 1.8, 1.3, 0.4, 0.22)
    if itm == "PYVOF":
        phi = g.shock_bubble_case_z(d, 1.8, 1.3, 0.4, 0.22)
    ctx = g.Context(d, two_fluid=True)
    ctx.init_shock_bubble_device(g.BubbleParams(1.8, 1.3, 0.4, 0.22), itm=itm)
    V1, V2, f = ctx.download()
    ctx.close()
    assert _same(V1, U1) and _same(V2, U2) and _same(f, phi)


def test_device_initialised_run_matches():
    d, T = g.case_params("twofluid", "shock_bubble", 100, 40)
    U1, U2, phi = g.case_init("twofluid", "shock_bubble", d)
    m = g.method(T=T)
    a = g.Context(d, two_fluid=True)
    a.upload(U1, U2, phi)
    a.step(m, 15)
    ra = a.download()
    a.close()
    b = g.Context(d, two_fluid=True)
    b.init_device("twofluid", "shock_bubble")
    b.step(m, 15)
    rb = b.download()
    b.close()
    for x, y in zip(ra, rb):
        assert np.array_equal(x, y)


def test_state_upload_download_in_one_call():
    """gfm_upload_state / gfm_download_state move the same bytes as the
    per-field calls."""
    import ctypes
    d, T = g.case_params("twofluid", "shock_bubble", 57, 23)
    U1, U2, phi = g.case_init("twofluid", "shock_bubble", d)
    L = g.lib()
    pd = lambda a: a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))   # noqa: E731
    ctx = g.Context(d, two_fluid=True)
    assert L.gfm_upload_state(ctx._p, pd(U1), pd(U2), pd(phi)) == 0
    V1, V2, ph = ctx.download()
    assert np.array_equal(V1, U1) and np.array_equal(V2, U2) and np.array_equal(ph, phi)
    # the asynchronous form, completed by the synchronising download
    Z1, Z2, zp = np.zeros_like(U1), np.zeros_like(U2), np.zeros_like(phi)
    assert L.gfm_upload_state_async(ctx._p, pd(Z1), pd(Z2), pd(zp)) == 0
    assert L.gfm_download_state(ctx._p, pd(V1), pd(V2), pd(ph)) == 0
    assert not V1.any() and not V2.any() and not ph.any()
    assert L.gfm_upload_state_async(ctx._p, pd(U1), pd(U2), pd(phi)) == 0
    assert L.gfm_download_state(ctx._p, pd(V1), pd(V2), pd(ph)) == 0
    assert np.array_equal(V1, U1) and np.array_equal(V2, U2) and np.array_equal(ph, phi)
    ctx.step(g.method(T=T), 3)
    W1, W2, wp = np.empty_like(U1), np.empty_like(U2), np.empty_like(phi)
    assert L.gfm_download_state(ctx._p, pd(W1), pd(W2), pd(wp)) == 0
    X1, X2, xp = ctx.download()
    ctx.close()
    assert np.array_equal(W1, X1) and np.array_equal(W2, X2) and np.array_equal(wp, xp)
