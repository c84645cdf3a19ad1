"""Batched exact Riemann solves on the GPU (C ABI) against the oracle:
bit-identical fluxes and star states over random data, the Toro tests, the
identical-state shortcut and stiffened-gas pairs."""
import json
import os

import numpy as np
import pytest

import gfm_gb300 as g
import oracle_binding as orc

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")
HERE = os.path.dirname(os.path.abspath(__file__))


def cons(gm, pinf, rho, u, v, p):
    e = (p + gm * pinf) / ((gm - 1.0) * rho)
    return np.array([rho, rho * u, rho * v, rho * e + 0.5 * rho * (u * u + v * v)])


def gpu_pure(xdir, gm, pinf, UL, UR):
    dL = torch.tensor(UL, dtype=torch.float64, device="cuda")
    dR = torch.tensor(UR, dtype=torch.float64, device="cuda")
    out = torch.zeros_like(dL)
    st = torch.zeros(1, dtype=torch.int32, device="cuda")
    rc = g.lib().gfm_rs_pure_batch(len(UL), xdir, gm, pinf, dL.data_ptr(), dR.data_ptr(), out.data_ptr(),
                                   st.data_ptr(), torch.cuda.current_stream().cuda_stream)
    assert rc == 0
    torch.cuda.synchronize()
    return out.cpu().numpy(), int(st.item())


def gpu_mixed(gL, pL, gR, pR, UL, UR):
    dL = torch.tensor(UL, dtype=torch.float64, device="cuda")
    dR = torch.tensor(UR, dtype=torch.float64, device="cuda")
    out = torch.zeros_like(dL)
    st = torch.zeros(1, dtype=torch.int32, device="cuda")
    rc = g.lib().gfm_rs_mixed_batch(len(UL), gL, pL, gR, pR, dL.data_ptr(), dR.data_ptr(), out.data_ptr(),
                                    st.data_ptr(), torch.cuda.current_stream().cuda_stream)
    assert rc == 0
    torch.cuda.synchronize()
    return out.cpu().numpy(), int(st.item())


def random_states(rng, n, gm, pinf, rho0, p0):
    rho = rho0 * np.exp(rng.uniform(-2, 2, n))
    p = p0 * np.exp(rng.uniform(-3, 3, n))
    c = np.sqrt(gm * (p + pinf) / rho)
    u = rng.uniform(-1.5, 1.5, n) * c
    v = rng.uniform(-1.5, 1.5, n) * c
    return np.array([cons(gm, pinf, *s) for s in zip(rho, u, v, p)])


@pytest.mark.parametrize("gm,pinf,rho0,p0", [(1.4, 0.0, 1.0, 1.0), (1.648, 0.0, 0.182, 1e5), (4.4, 6e8, 1000.0, 1e5)])
@pytest.mark.parametrize("xdir", [1, 0])
def test_pure_flux_bitwise(gm, pinf, rho0, p0, xdir):
    rng = np.random.default_rng(11)
    n = 4096
    UL = random_states(rng, n, gm, pinf, rho0, p0)
    UR = random_states(rng, n, gm, pinf, rho0, p0)
    UR[: n // 8] = UL[: n // 8]            # identical states
    UR[n // 8: n // 4, 0] *= 1.7           # contact only (same u, p)
    UR[n // 8: n // 4, 1:] *= 1.7
    got, st = gpu_pure(xdir, gm, pinf, UL, UR)
    ref = orc.rs_pure(xdir, gm, pinf, UL, UR)
    ok = np.isfinite(ref).all(axis=1)
    assert ok.mean() > 0.9
    assert np.array_equal(got[ok], ref[ok])


@pytest.mark.parametrize("mat", [(1.4, 0.0, 1.4, 0.0), (1.648, 0.0, 1.4, 0.0), (1.4, 0.0, 4.4, 6e8)])
def test_mixed_bitwise(mat):
    gL, pL, gR, pR = mat
    rng = np.random.default_rng(12)
    UL = random_states(rng, 2048, gL, pL, 1.0 if pL == 0 else 1000.0, 1e5)
    UR = random_states(rng, 2048, gR, pR, 1.0 if pR == 0 else 1000.0, 1e5)
    UL[:, 2] = 0.0
    UR[:, 2] = 0.0
    got, st = gpu_mixed(gL, pL, gR, pR, UL, UR)
    ref = orc.rs_mixed(gL, pL, gR, pR, UL, UR)
    ok = np.isfinite(ref).all(axis=1)
    assert np.array_equal(got[ok], ref[ok])


def test_toro_on_gpu():
    data = json.load(open(os.path.join(HERE, "golden", "toro_table_4_3.json")))
    gm = data["gamma"]
    UL = np.array([cons(gm, 0.0, t["left"][0], t["left"][1], 0.0, t["left"][2]) for t in data["tests"]])
    UR = np.array([cons(gm, 0.0, t["right"][0], t["right"][1], 0.0, t["right"][2]) for t in data["tests"]])
    got, st = gpu_mixed(gm, 0.0, gm, 0.0, UL, UR)
    assert st == 0
    for row, t in zip(got, data["tests"]):
        for v, text in zip(row, t["star"]):
            dec = len(text.split(".")[1])
            assert abs(v - float(text)) <= max(1.01 * 10.0 ** -dec, 4e-6 * abs(float(text)))
