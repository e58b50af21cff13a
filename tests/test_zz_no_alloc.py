"""ts_advance_noalloc: the fused mixed-precision step for callers that are not
allowed to allocate device memory (a host application that owns all device
memory through its own pool or budget, or a latency-critical loop that cannot
afford an allocation's implicit synchronisation).

The caller hands in device buffers for the input and output state; all other
working memory comes from one fixed array inside the library.  These tests
check that two calls in a row give the same states, step counts and times as
the handle API (ts_create / ts_set_state / ts_step / ts_get_state) doing the
same work, within the 1e-12 relative tolerance the other parity tests use --
on the legacy default stream and on a non-blocking stream (every set-up copy
of the call must be ordered on the caller's stream), with and without a
snapshot schedule (SaveSolutionTime) clipping dt -- that a call leaves the
device's free memory unchanged, and that a grid too large for the fixed array
is refused with a clear error.

This file is collected last so that a failure here cannot hide the result of
any other test in a run that stops at the first failure.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _bind(lib):
    from turbostructred_gb300 import capi
    lib.ts_advance_noalloc.argtypes = [C.POINTER(capi.Config), C.c_void_p, C.c_void_p, C.c_int32, C.c_void_p,
                                       C.POINTER(capi.StepInfo)]
    lib.ts_advance_noalloc.restype = C.c_int
    return lib.ts_advance_noalloc


def _rel(a, b):
    return float(np.abs(a - b).max() / np.abs(b).max())


@pytest.mark.parametrize("stream_kind,save_time", [("legacy", 0.0), ("nonblocking", 0.0), ("nonblocking", 3e-4)])
def test_no_alloc_matches_handle_api_on_two_calls_in_a_row(stream_kind, save_time, tslib):
    import torch

    from turbostructred_gb300 import capi
    advance = _bind(tslib)
    sym = (capi.BC_SYMMETRY, 0.0, (0.0, 0.0, 0.0), 0.0)
    case = capi.make_case(ndims=3, nx=40, ny=36, nz=30, periodic=(0, 0, 0), recon=capi.RECON_LINEAR2_LIM,
                          solver=capi.RS_ROE, cfl=0.4, bc=[sym] * 6, save_solution_time=save_time)
    ic = capi.fill_scenario(case, capi.SCENARIO_BLAST, 31, [1.0, 0.1, 10.0, 0.15, 0.01])
    # torch.cuda.Stream() is created with cudaStreamNonBlocking: it does not
    # wait for the legacy default stream
    side = torch.cuda.Stream() if stream_kind == "nonblocking" else None
    handle = None if side is None else C.c_void_p(side.cuda_stream)

    # the handle API, with the state read back between the two segments
    with capi.Solver(case, capi.PRECISION_MIXED) as s:
        s.set_state(ic)
        s.step(7)
        ref1, info1 = s.get_state(), s.info()
        s.step(5)
        ref2, info2 = s.get_state(), s.info()

    cfg, keep = capi.to_config(case, capi.PRECISION_MIXED)
    d_in = torch.from_numpy(ic.copy()).cuda()
    d_out = torch.empty_like(d_in)
    si = capi.StepInfo()
    torch.cuda.synchronize()

    st = advance(C.byref(cfg), d_in.data_ptr(), d_out.data_ptr(), 7, handle, C.byref(si))
    assert st == 0, tslib.ts_last_error()
    out1 = d_out.cpu().numpy()
    assert si.iteration == 7 and si.time == info1["time"]
    assert si.next_solution_time == info1["next_solution_time"]
    assert _rel(out1, ref1) <= 1e-12

    # second call in a row: continue in place from the first call's output,
    # passing back the step info (and with it the snapshot schedule)
    st = advance(C.byref(cfg), d_out.data_ptr(), d_out.data_ptr(), 5, handle, C.byref(si))
    assert st == 0, tslib.ts_last_error()
    out2 = d_out.cpu().numpy()
    assert si.iteration == 12 and si.time == info2["time"]
    assert si.next_solution_time == info2["next_solution_time"]
    assert _rel(out2, ref2) <= 1e-12
    assert si.health == 0
    if save_time > 0:
        # The schedule starts at SaveSolutionTime on the first call (the zeroed
        # step info is a fresh run) and clips dt to land on it.  Plain steps,
        # like the reference's IterationStep outside Kernel::Run, do not move
        # the schedule on, so the time stays at the snapshot time after that.
        assert 0.0 < info1["time"] <= save_time
        assert info2["time"] == save_time == si.time


def test_no_alloc_call_allocates_nothing(tslib):
    """After a first call (which loads the kernels and looks up the fixed
    array's address), a call leaves the device's free memory unchanged."""
    import torch

    from turbostructred_gb300 import capi
    advance = _bind(tslib)
    case = capi.make_case(ndims=3, nx=32, ny=24, nz=20, periodic=(1, 1, 1), recon=capi.RECON_LINEAR2_LIM,
                          solver=capi.RS_HLLC, cfl=0.4)
    ic = capi.fill_scenario(case, capi.SCENARIO_BLAST, 5, [1.0, 0.1, 10.0, 0.2, 0.01])
    cfg, keep = capi.to_config(case, capi.PRECISION_MIXED)
    d_in = torch.from_numpy(ic.copy()).cuda()
    d_out = torch.empty_like(d_in)
    si = capi.StepInfo()
    assert advance(C.byref(cfg), d_in.data_ptr(), d_out.data_ptr(), 2, None, C.byref(si)) == 0
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    si = capi.StepInfo()
    assert advance(C.byref(cfg), d_in.data_ptr(), d_out.data_ptr(), 3, None, C.byref(si)) == 0
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info()
    assert free1 == free0
    assert si.iteration == 3 and si.health == 0


def test_no_alloc_rejects_grids_beyond_its_fixed_array(tslib):
    from turbostructred_gb300 import capi
    advance = _bind(tslib)
    case = capi.make_case(ndims=3, nx=80, ny=80, nz=80, periodic=(1, 1, 1))
    cfg, keep = capi.to_config(case, capi.PRECISION_MIXED)
    si = capi.StepInfo()
    st = advance(C.byref(cfg), C.c_void_p(1), C.c_void_p(1), 1, None, C.byref(si))
    assert st == 1
    assert b"too large" in tslib.ts_last_error()
