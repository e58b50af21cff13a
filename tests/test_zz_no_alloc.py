"""ts_advance_noalloc: the fused mixed-precision step for callers that are not
allowed to allocate device memory (a host application that owns all device
memory through its own pool or budget, or a latency-critical loop that cannot
afford an allocation's implicit synchronisation).

The caller hands in device buffers for the input and output state; all other
working memory comes from one fixed array inside the library.  These tests
check that two calls in a row give the same states, step counts and times as
the handle API (ts_create / ts_set_state / ts_step / ts_get_state) doing the
same work, within the 1e-12 relative tolerance the other parity tests use, and
that a grid too large for the fixed array is refused with a clear error.

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


def test_no_alloc_matches_handle_api_on_two_calls_in_a_row(tslib):
    import torch

    from turbostructred_gb300 import capi
    advance = _bind(tslib)
    sym = (capi.BC_SYMMETRY, 0.0, (0.0, 0.0, 0.0), 0.0)
    case = capi.make_case(ndims=3, nx=40, ny=36, nz=30, periodic=(0, 0, 0), recon=capi.RECON_LINEAR2_LIM,
                          solver=capi.RS_ROE, cfl=0.4, bc=[sym] * 6)
    ic = capi.fill_scenario(case, capi.SCENARIO_BLAST, 31, [1.0, 0.1, 10.0, 0.15, 0.01])

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

    st = advance(C.byref(cfg), d_in.data_ptr(), d_out.data_ptr(), 7, None, C.byref(si))
    assert st == 0, tslib.ts_last_error()
    out1 = d_out.cpu().numpy()
    assert si.iteration == 7 and si.time == info1["time"]
    assert _rel(out1, ref1) <= 1e-12

    # second call in a row: continue in place from the first call's output
    st = advance(C.byref(cfg), d_out.data_ptr(), d_out.data_ptr(), 5, None, C.byref(si))
    assert st == 0, tslib.ts_last_error()
    out2 = d_out.cpu().numpy()
    assert si.iteration == 12 and si.time == info2["time"]
    assert _rel(out2, ref2) <= 1e-12
    assert si.health == 0


def test_no_alloc_rejects_grids_beyond_its_fixed_array(tslib):
    from turbostructred_gb300 import capi
    advance = _bind(tslib)
    case = capi.make_case(ndims=3, nx=80, ny=80, nz=80, periodic=(1, 1, 1))
    cfg, keep = capi.to_config(case, capi.PRECISION_MIXED)
    si = capi.StepInfo()
    st = advance(C.byref(cfg), C.c_void_p(1), C.c_void_p(1), 1, None, C.byref(si))
    assert st == 1
    assert b"too large" in tslib.ts_last_error()
