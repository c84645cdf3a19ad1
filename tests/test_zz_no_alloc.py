"""gfm_onefluid_step_noalloc: the one-fluid step for callers that cannot
allocate device memory (a host runtime whose memory pool owns the device, or
real-time code that may not block on cudaMalloc after start-up).  Its scratch
is a built-in device array; these tests check, through the C ABI, that two
calls in a row give the same grids, time and step count as the
context-based gfm_step (transmissive, reflective and periodic sides, and a
call that asks for more steps than reach the end time), that a call after
the first leaves the device's free memory unchanged, and that a grid larger
than the built-in scratch or a bad boundary kind is rejected.  The file is
collected last on purpose."""
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


def _compare_two_calls(step, desc, U0, m, nsteps):
    """Two calls of nsteps each against a context stepped the same way."""
    dU = torch.tensor(U0, dtype=torch.float64, device="cuda").contiguous()
    stream = torch.cuda.current_stream().cuda_stream
    t = ctypes.c_double(0.0)
    n = ctypes.c_int(0)
    st = ctypes.c_uint32(0)
    ctx = g.Context(desc, two_fluid=False)
    ctx.upload(U0)
    gc = desc.numGC
    counts = []
    for call in range(2):
        rc = step(ctypes.byref(desc), ctypes.byref(m), dU.data_ptr(), nsteps, ctypes.byref(t), ctypes.byref(n),
                  ctypes.byref(st), stream)
        assert rc == 0 and st.value == 0
        ctx.step(m, nsteps)
        G, _, _ = ctx.download()
        tc, ncs, _ = ctx.time()
        A = dU.cpu().numpy()
        assert n.value == ncs
        assert t.value == tc
        for k in range(4):
            assert rel_l1(A[k, gc:-gc, gc:-gc], G[k, gc:-gc, gc:-gc]) <= TOL
        assert np.array_equal(A, G)
        counts.append(n.value)
    ctx.close()
    return counts, t.value


@pytest.mark.parametrize("fs", ["MUSCL", "Godunov"])
def test_noalloc_matches_context_on_two_calls(fs):
    step = _entry()
    desc, T = g.case_params("onefluid", "circularexplosion", 120, 100)
    U0, _, _ = g.case_init("onefluid", "circularexplosion", desc)
    counts, _ = _compare_two_calls(step, desc, U0, g.method(fs=fs, CFL=0.8, T=T), 15)
    assert counts == [15, 30]


@pytest.mark.parametrize("bc", ["reflective", "periodic"])
def test_noalloc_matches_context_at_walls_and_periodic_sides(bc):
    step = _entry()
    desc, T = g.case_params("onefluid", "circularexplosion", 96, 96)
    kind = {"reflective": 1, "periodic": 2}[bc]
    desc.BC_L = desc.BC_R = desc.BC_B = desc.BC_T = kind
    U0, _, _ = g.case_init("onefluid", "circularexplosion", desc)
    counts, _ = _compare_two_calls(step, desc, U0, g.method(fs="MUSCL", CFL=0.4, T=T), 12)
    assert counts == [12, 24]


def test_noalloc_stops_at_the_end_time():
    """Steps after t reaches T do nothing: t and the step count stay put."""
    step = _entry()
    desc, _ = g.case_params("onefluid", "circularexplosion", 64, 64)
    U0, _, _ = g.case_init("onefluid", "circularexplosion", desc)
    T = 0.02
    counts, t_end = _compare_two_calls(step, desc, U0, g.method(fs="MUSCL", CFL=0.8, T=T), 400)
    assert 0 < counts[0] < 400
    assert counts[1] == counts[0]
    assert abs(t_end - T) <= 1e-15


def test_noalloc_allocates_no_device_memory():
    """After the first call (which looks up the scratch array's address), a
    call leaves the device's free memory where it was."""
    step = _entry()
    desc, T = g.case_params("onefluid", "circularexplosion", 200, 200)
    U0, _, _ = g.case_init("onefluid", "circularexplosion", desc)
    m = g.method(fs="MUSCL", CFL=0.8, T=T)
    dU = torch.tensor(U0, dtype=torch.float64, device="cuda").contiguous()
    stream = torch.cuda.current_stream().cuda_stream
    t = ctypes.c_double(0.0)
    n = ctypes.c_int(0)
    st = ctypes.c_uint32(0)
    args = (ctypes.byref(desc), ctypes.byref(m), dU.data_ptr(), 5, ctypes.byref(t), ctypes.byref(n),
            ctypes.byref(st), stream)
    assert step(*args) == 0
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    for _ in range(3):
        assert step(*args) == 0
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info()
    assert free1 == free0
    assert n.value == 20 and st.value == 0


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


def test_noalloc_rejects_bad_boundary_kinds():
    step = _entry()
    desc, T = g.case_params("onefluid", "circularexplosion", 32, 32)
    desc.BC_T = 7
    m = g.method(fs="MUSCL", CFL=0.8, T=T)
    dU = torch.zeros(8, dtype=torch.float64, device="cuda")
    t = ctypes.c_double(0.0)
    n = ctypes.c_int(0)
    rc = step(ctypes.byref(desc), ctypes.byref(m), dU.data_ptr(), 1, ctypes.byref(t), ctypes.byref(n), None,
              torch.cuda.current_stream().cuda_stream)
    assert rc == 1
    assert n.value == 0 and t.value == 0.0
