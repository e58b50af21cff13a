"""The C-ABI library without a GPU: it loads, exports every entry point that
include/*.h declares, and its host-side logic (grid accumulation, scenarios,
configuration checks) is right.  No device work is attempted here."""
import ctypes as C
import os
import re
import subprocess

import numpy as np
import pytest

from conftest import ROOT, golden_names, load_golden


def declared_symbols():
    names = set()
    inc = os.path.join(ROOT, "include")
    for f in os.listdir(inc):
        if not f.endswith(".h"):
            continue
        text = open(os.path.join(inc, f)).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        for m in re.finditer(r"\b(ts_[a-z0-9_]+)\s*\(", text):
            names.add(m.group(1))
    return names


def test_library_exports_all_declared_symbols(tslib):
    from turbostructred_gb300 import capi
    out = subprocess.run(["nm", "-D", "--defined-only", capi.LIB_PATH], capture_output=True, text=True).stdout
    exported = {line.split()[-1] for line in out.splitlines() if line.split()}
    missing = declared_symbols() - exported
    assert not missing, missing
    for name in declared_symbols():
        assert hasattr(tslib, name)


@pytest.mark.parametrize("name", golden_names())
def test_host_grid_matches_reference(name, tslib):
    from turbostructred_gb300 import capi
    g = load_golden(name)
    case = capi.make_case(**g["case"])
    for mine, ref in zip(capi.grid_coordinates(case), (g["x"], g["hx"], g["y"], g["hy"], g["z"], g["hz"])):
        assert np.array_equal(mine, ref)


def test_scenarios_deterministic_and_shaped(tslib):
    from turbostructred_gb300 import capi
    case = capi.make_case(ndims=3, nx=8, ny=6, nz=5)
    a = capi.fill_scenario(case, capi.SCENARIO_BLAST, 3, [1.0, 0.1, 10.0, 0.2, 0.01])
    b = capi.fill_scenario(case, capi.SCENARIO_BLAST, 3, [1.0, 0.1, 10.0, 0.2, 0.01])
    c = capi.fill_scenario(case, capi.SCENARIO_BLAST, 4, [1.0, 0.1, 10.0, 0.2, 0.01])
    assert a.shape == (5, 6, 8, 5)
    assert np.array_equal(a, b) and not np.array_equal(a, c)
    assert np.all(np.abs(a[..., 0] - 1.0) <= 0.01 + 1e-15)
    p = a[..., 4] * 0.4
    assert set(np.round(np.unique(p), 12)) <= {0.1 * 1.0, 10.0}
    # the hash RNG depends on (seed, i, j, k) only
    u = tslib.ts_hash_uniform(3, 1, 2, 3)
    assert 0.0 <= u < 1.0 and u == tslib.ts_hash_uniform(3, 1, 2, 3)


def test_shear_layer_matches_config(tslib):
    from turbostructred_gb300 import capi
    case = capi.make_case(ndims=2, nx=16, ny=16)
    s = capi.fill_scenario(case, capi.SCENARIO_SHEAR_LAYER, 1, [2.0, 1.0, 0.5, 2.5, 0.01])[0]
    y = capi.grid_coordinates(case)[2][1:-1]
    inner = np.abs(y - 0.5) < 0.25
    assert np.all(s[inner, :, 0] == 2.0) and np.all(s[~inner, :, 0] == 1.0)
    assert np.allclose(s[inner, :, 1], 1.0) and np.allclose(s[~inner, :, 1], -0.5)
    v = s[..., 2] / s[..., 0]
    assert np.abs(v).max() <= 0.01 and np.abs(v).max() > 0.005


@pytest.mark.parametrize("bad", [
    dict(ndims=4), dict(nx=1), dict(gamma=1.0), dict(cfl=0.0), dict(recon=7), dict(limiter=5),
    dict(solver=9), dict(solver=2), dict(eps=-1.0), dict(length=(0.0, 1.0, 1.0)),
    dict(ndims=2, ny=1), dict(blocks={0: [(0.0, 1.0, 3)]}),
])
def test_invalid_configurations_rejected(bad, tslib):
    from turbostructred_gb300 import capi
    case = capi.make_case(**dict(dict(ndims=1, nx=8), **bad))
    cfg, keep = capi.to_config(case)
    h = C.c_void_p()
    st = tslib.ts_create(C.byref(cfg), C.byref(h))
    assert st == 1, (st, tslib.ts_last_error())
    assert tslib.ts_last_error()


def test_godunov_limits_reported_unsupported(tslib):
    """The exact solver runs on the FP64 path with the ideal-gas EOS (as the
    reference's); other combinations are refused before any device work."""
    from turbostructred_gb300 import capi
    h = C.c_void_p()
    cfg, keep = capi.to_config(capi.make_case(nx=8, solver=capi.RS_GODUNOV), precision=capi.PRECISION_MIXED)
    assert tslib.ts_create(C.byref(cfg), C.byref(h)) == 2
    cfg, keep = capi.to_config(capi.make_case(nx=8, solver=capi.RS_GODUNOV, eos=capi.EOS_STIFFENED, p_inf=1.0))
    assert tslib.ts_create(C.byref(cfg), C.byref(h)) == 2


def test_state_sizes(tslib):
    from turbostructred_gb300 import capi
    cfg, keep = capi.to_config(capi.make_case(ndims=3, nx=4, ny=5, nz=6))
    assert tslib.ts_state_doubles(C.byref(cfg), 0) == 4 * 5 * 6 * 5
    assert tslib.ts_state_doubles(C.byref(cfg), 1) == 6 * 7 * 8 * 5


@pytest.mark.parametrize("nd,scenario,params", [
    (3, 2, [1.0, 0.1, 10.0, 0.1, 0.01]),
    (2, 1, [2.0, 1.0, 0.5, 2.5, 0.01]),
    (1, 0, [0.5, 1.0, 0.0, 1.0, 0.125, 0.0, 0.1]),
    (2, 3, [1.5, 0.0, 0.0, 1.5, 0.53, 1.2, 0.0, 0.3, 0.14, 1.2, 1.2, 0.03, 0.53, 0.0, 1.2, 0.3]),
])
def test_oracle_scenarios_equal_the_library_scenarios(nd, scenario, params, tslib, oracle_mod):
    """The CPU legs of the bench build their inputs with the oracle's
    restatement of the scenarios; it must give the product's bytes."""
    from turbostructred_gb300 import capi
    stiff = scenario == 0
    case = capi.make_case(ndims=nd, nx=41, ny=27, nz=19, gamma=4.4 if stiff else 1.4,
                          eos=capi.EOS_STIFFENED if stiff else capi.EOS_IDEAL, p_inf=6.0 if stiff else 0.0,
                          blocks={0: [(0.0, 1.03, 41)]})
    a = capi.fill_scenario(case, scenario, 2024, params)
    b = oracle_mod.fill_scenario(case, scenario, 2024, params)
    assert a.shape == b.shape
    assert np.array_equal(a, b)


@pytest.mark.parametrize("name", ["marker2d_plate", "marker3d_split"])
def test_split_markers_equal_the_oracles(name, tslib, oracle_mod):
    """Per-face BC markers of a split side, from the library's grid and from
    the oracle's, are the same arrays (the reference's marker function
    evaluated at the face centres gives the fixture's results)."""
    from turbostructred_gb300 import capi
    g = load_golden(name)
    case = g["case"]
    a = capi.split_markers(capi.make_case(**case))
    b = oracle_mod.split_markers(case)
    assert sorted(a) == sorted(b) and len(a) > 0
    for side in a:
        assert np.array_equal(a[side], b[side])
        assert len(set(a[side].tolist())) == 2  # the split falls inside the side


def test_markers_are_validated(tslib):
    """Markers beyond n_bc_kinds, or on a periodic side, are refused; batches
    refuse position-dependent sides."""
    from turbostructred_gb300 import capi
    nat = (capi.BC_NATURAL, 0.0, (0.0, 0.0, 0.0), 0.0)
    case = capi.make_case(ndims=2, nx=8, ny=6, periodic=(0, 0, 1), bc=[nat] * 6, bc_kinds=[nat],
                          bc_split={2: (0, 0.5, 0, 1)})
    cfg, keep = capi.to_config(case, capi.PRECISION_MIXED)
    assert tslib.ts_batch_problem_bytes(C.byref(cfg)) == 0  # kind 1 does not exist
    case = dict(case, bc_kinds=[nat, nat])
    cfg, keep = capi.to_config(case, capi.PRECISION_MIXED)
    assert tslib.ts_batch_problem_bytes(C.byref(cfg)) == 0  # valid, but batches take no markers
    cfg.periodic[1] = 1  # the split side becomes periodic
    null = C.POINTER(C.c_double)()
    assert tslib.ts_grid_coordinates(C.byref(cfg), *([null] * 6)) == 1
    assert b"periodic" in tslib.ts_last_error()
