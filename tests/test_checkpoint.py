"""Checkpoint / resume: the file format on the host (CPU) and bit-identical
continuation of a run resumed on the GPU."""
import numpy as np
import pytest

import gfm_gb300 as g


def _state(case="shock_bubble", Nx=40, Ny=16):
    desc, T = g.case_params("twofluid", case, Nx, Ny)
    U1, U2, phi = g.case_init("twofluid", case, desc)
    return desc, T, U1, U2, phi


def test_roundtrip_host(tmp_path):
    desc, T, U1, U2, phi = _state()
    p = tmp_path / "a.ckpt"
    g.checkpoint_write(p, desc, 0.125, 17, U1, U2, phi)
    d, t, n, V1, V2, ph = g.checkpoint_read(p)
    assert (t, n) == (0.125, 17)
    assert (d.Nx, d.Ny, d.numGC, d.dx, d.gamma1, d.BC_T) == (desc.Nx, desc.Ny, desc.numGC, desc.dx, desc.gamma1,
                                                             desc.BC_T)
    assert np.array_equal(V1, U1) and np.array_equal(V2, U2) and np.array_equal(ph, phi)
    # one fluid
    d1, T1 = g.case_params("onefluid", "TTC1_x", 20, 4)
    W, _, _ = g.case_init("onefluid", "TTC1_x", d1)
    g.checkpoint_write(tmp_path / "b.ckpt", d1, 0.0, 0, W)
    d, t, n, V, V2, ph = g.checkpoint_read(tmp_path / "b.ckpt")
    assert np.array_equal(V, W) and V2 is None and ph is None


@pytest.mark.parametrize("damage", ["flip", "truncate", "magic"])
def test_damaged_file_is_rejected(tmp_path, damage):
    desc, T, U1, U2, phi = _state()
    p = tmp_path / "c.ckpt"
    g.checkpoint_write(p, desc, 0.5, 3, U1, U2, phi)
    raw = bytearray(p.read_bytes())
    if damage == "flip":
        raw[len(raw) // 2] ^= 0x10
    elif damage == "truncate":
        raw = raw[:len(raw) - 100]
    else:
        raw[0:8] = b"NOTACKPT"
    p.write_bytes(bytes(raw))
    with pytest.raises(g.GFMError, match="gfm_status_t 5"):
        g.checkpoint_read(p)


def test_missing_file(tmp_path):
    with pytest.raises(g.GFMError, match="gfm_status_t 5"):
        g.checkpoint_read(tmp_path / "none.ckpt")


@pytest.mark.gpu
@pytest.mark.parametrize("gfm,itm,reinit", [("riemannGFM", "LS5", 3), ("OGFMVOF", "PYVOF", 0), ("realGFM", "LS1", 1)])
def test_resume_is_bit_identical(tmp_path, gfm, itm, reinit):
    """20 steps straight against 9 steps, checkpoint, a new context, 11 steps."""
    case = "underwater_explosion_sg" if gfm != "riemannGFM" else "shock_bubble"
    desc, T = g.case_params("twofluid", case, 48, 40)
    U1, U2, phi = g.case_init("twofluid", case, desc)
    if itm == "PYVOF":
        phi = g.case_init_z(case, desc)
    m = g.method(gfm=gfm, itm=itm, CFL=0.5, T=T, reinit_every=reinit)
    a = g.Context(desc, two_fluid=True)
    a.upload(U1, U2, phi)
    a.step(m, 20)
    ref = a.download()
    ta = a.time()
    a.close()
    b = g.Context(desc, two_fluid=True)
    b.upload(U1, U2, phi)
    b.step(m, 9)
    b.save_checkpoint(tmp_path / "r.ckpt")
    b.close()
    c = g.Context(desc, two_fluid=True)
    c.load_checkpoint(tmp_path / "r.ckpt")
    assert c.time()[1] == 9
    c.step(m, 11)
    got = c.download()
    tc = c.time()
    c.close()
    assert ta[:2] == tc[:2]
    for x, y in zip(ref, got):
        assert np.array_equal(x, y)


@pytest.mark.gpu
def test_load_rejects_other_grid(tmp_path):
    desc, T, U1, U2, phi = _state()
    g.checkpoint_write(tmp_path / "d.ckpt", desc, 0.0, 0, U1, U2, phi)
    other, _ = g.case_params("twofluid", "shock_bubble", 44, 16)
    ctx = g.Context(other, two_fluid=True)
    with pytest.raises(g.GFMError):
        ctx.load_checkpoint(tmp_path / "d.ckpt")
    ctx.close()
