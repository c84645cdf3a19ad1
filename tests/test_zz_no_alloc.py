"""gfm_onefluid_step_noalloc: the one-fluid step for callers that cannot
allocate device memory (a host runtime whose memory pool owns the device, or
real-time code that may not block on cudaMalloc after start-up).  Its scratch
is a built-in device array; these tests check, through the C ABI, that two
calls in a row give the same grids, time and step count as the
context-based gfm_step, and that a grid larger than the built-in scratch is
rejected.  The file is collected last on purpose."""
import ctypes

import numpy as np
import pytest

import gfm_gb300 as g

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")
TOL = 1e-10


def _entry():
    L = g.lib()
    f = L.gfm_onefluid_step_noalloc
    f.argtypes = [ctypes.POINTER(g.GridDesc), ctypes.POINTER(g.MethodDesc), ctypes.c_void_p, ctypes.c_int,
                  ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_uint32),
                  ctypes.c_void_p]
    f.restype = ctypes.c_int
    return f


def rel_l1(a, b):
    return np.abs(a - b).sum() / np.abs(b).sum()


@pytest.mark.parametrize("fs", ["MUSCL", "Godunov"])
def test_noalloc_matches_context_on_two_calls(fs):
    step = _entry()
    desc, T = g.case_params("onefluid", "circularexplosion", 120, 100)
    U0, _, _ = g.case_init("onefluid", "circularexplosion", desc)
    m = g.method(fs=fs, CFL=0.8, T=T)
    dU = torch.tensor(U0, dtype=torch.float64, device="cuda").contiguous()
    stream = torch.cuda.current_stream().cuda_stream
    t = ctypes.c_double(0.0)
    n = ctypes.c_int(0)
    st = ctypes.c_uint32(0)
    ctx = g.Context(desc, two_fluid=False)
    ctx.upload(U0)
    gc = desc.numGC
    for call in range(2):
        rc = step(ctypes.byref(desc), ctypes.byref(m), dU.data_ptr(), 15, ctypes.byref(t), ctypes.byref(n),
                  ctypes.byref(st), stream)
        assert rc == 0 and st.value == 0
        ctx.step(m, 15)
        G, _, _ = ctx.download()
        tc, ncs, _ = ctx.time()
        A = dU.cpu().numpy()
        assert n.value == ncs == 15 * (call + 1)
        assert t.value == tc
        for k in range(4):
            assert rel_l1(A[k, gc:-gc, gc:-gc], G[k, gc:-gc, gc:-gc]) <= TOL
        assert np.array_equal(A, G)
    ctx.close()


def test_noalloc_rejects_grids_beyond_its_scratch():
    step = _entry()
    desc, T = g.case_params("onefluid", "circularexplosion", 800, 800)   # 804 x 804 padded cells
    assert (desc.Nx + 2 * desc.numGC) * (desc.Ny + 2 * desc.numGC) > 524272
    m = g.method(fs="MUSCL", CFL=0.8, T=T)
    dU = torch.zeros(8, dtype=torch.float64, device="cuda")
    t = ctypes.c_double(0.0)
    n = ctypes.c_int(0)
    st = ctypes.c_uint32(0)
    rc = step(ctypes.byref(desc), ctypes.byref(m), dU.data_ptr(), 1, ctypes.byref(t), ctypes.byref(n),
              ctypes.byref(st), torch.cuda.current_stream().cuda_stream)
    assert rc == 1
    assert n.value == 0 and t.value == 0.0
