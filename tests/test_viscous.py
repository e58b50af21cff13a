"""Viscous flow (ExplicitRungeKuttaFVM.h:81-874 and the viscous terms of
ComputeResidual, :1161-1170, :1220-1248) on the FP64 path.

Bars:
  * oracle vs the reference's own runs (tests/golden/viscous, made by
    make_viscous_golden.py): same step count and, per fixture, bit for bit
    where no boundary least-squares gradient enters (rtol 0: periodic axes,
    the one-dimensional stencil, viscosity only in the spectral radius), else
    relative L-inf <= 1e-13 (the reference solves the boundary least-squares
    problems with Eigen's JacobiSVD, the oracle and the device with the
    normal equations; measured <= 1.2e-16);
  * device vs oracle on the same inputs: bit for bit (the same algorithm in
    the same operation order); on stretched grids the host libm's pow builds
    the grid, so there the device is compared with the oracle run on the same
    host;
  * device vs the reference fixture: the fixture's rtol, or 1e-12 on
    stretched grids (the grid's last bits differ between x86 and Arm libm).
"""
import ctypes as C
import json
import os

import numpy as np
import pytest

from conftest import ROOT

VISC = os.path.join(ROOT, "tests", "golden", "viscous")
NAMES = sorted(f[:-4] for f in os.listdir(VISC) if f.endswith(".npz"))


def load(name):
    d = dict(np.load(os.path.join(VISC, name + ".npz")))
    meta = json.loads(bytes(d.pop("meta")).decode())
    case = meta["case"]
    case["periodic"] = tuple(case["periodic"])
    case["length"] = tuple(case["length"])
    case["bc"] = [(t, dens, tuple(vel), ps) for t, dens, vel, ps in case["bc"]]
    case["blocks"] = {int(k): [tuple(b) for b in v] for k, v in case.get("blocks", {}).items()}
    d["case"], d["meta"] = case, meta
    d["iteration"], d["time"], d["dt"] = int(d["scalars"][0]), float(d["scalars"][1]), float(d["scalars"][2])
    return d


def rel_linf(a, b):
    return float(np.abs(a - b).max() / np.abs(b).max())


def interior(case, full):
    nx, ny, nz = case["nx"], case["ny"], case["nz"]
    nd = case["ndims"]
    return full[(slice(1, nz + 1) if nd > 2 else slice(None)), (slice(1, ny + 1) if nd > 1 else slice(None)),
                slice(1, nx + 1)]


def test_fixture_set_covers_the_viscous_paths():
    metas = [load(n) for n in NAMES]
    assert {m["case"]["ndims"] for m in metas} == {1, 2, 3}
    assert any(not m["case"]["viscous"] and m["case"]["viscosity"] > 0 for m in metas)
    assert any(m["meta"]["rtol"] > 0 for m in metas) and any(m["meta"]["rtol"] == 0 for m in metas)
    assert any(m["case"]["blocks"] for m in metas)


@pytest.mark.parametrize("name", NAMES)
def test_oracle_matches_reference_viscous(name, oracle_mod):
    g = load(name)
    vals, info = oracle_mod.advance(g["case"], g["initial"], g["meta"]["steps"])
    assert info["iteration"] == g["iteration"]
    a, b = interior(g["case"], vals), interior(g["case"], g["values"])
    if g["meta"]["rtol"] == 0:
        assert info["time"] == g["time"] and info["dt"] == g["dt"]
        assert np.array_equal(a, b)
    else:
        assert abs(info["time"] - g["time"]) <= g["meta"]["rtol"] * g["time"]
        assert rel_linf(a, b) <= g["meta"]["rtol"]


def test_viscosity_changes_the_solution(oracle_mod):
    """The fixtures exercise the viscous terms: the inviscid run of the same
    case differs well above the tolerances."""
    g = load("visc2d_channel_walls")
    vals, _ = oracle_mod.advance(g["case"], g["initial"], g["meta"]["steps"])
    inv = dict(g["case"], viscous=False, viscosity=0.0)
    vals0, _ = oracle_mod.advance(inv, g["initial"], g["meta"]["steps"])
    assert rel_linf(interior(inv, vals0), interior(inv, vals)) > 1e-4


def test_viscous_refused_off_the_fp64_path(tslib):
    """Viscous flow, or a nonzero viscosity (which enters the spectral radius),
    runs on the FP64 path only; the mixed path and batches refuse it."""
    from turbostructred_gb300 import capi
    h = C.c_void_p()
    for kw in (dict(viscous=True, viscosity=0.01), dict(viscous=False, viscosity=0.01)):
        cfg, keep = capi.to_config(capi.make_case(nx=8, **kw), precision=capi.PRECISION_MIXED)
        assert tslib.ts_create(C.byref(cfg), C.byref(h)) == 2
    cfg, keep = capi.to_config(capi.make_case(nx=8, viscous=True, viscosity=-1.0))
    assert tslib.ts_create(C.byref(cfg), C.byref(h)) == 1


@pytest.mark.gpu
@pytest.mark.parametrize("name", NAMES)
def test_device_viscous_matches_oracle_and_reference(name, tslib, oracle_mod):
    from turbostructred_gb300 import capi
    g = load(name)
    case = capi.make_case(**g["case"])
    with capi.Solver(case, precision=capi.PRECISION_FP64) as s:
        s.set_state(g["initial"], capi.LAYOUT_WITH_GHOSTS)
        info = s.run() if g["meta"]["steps"] < 0 else s.step(g["meta"]["steps"])
        got = s.get_state(capi.LAYOUT_WITH_GHOSTS)
    ref, rinfo = oracle_mod.advance(g["case"], g["initial"], g["meta"]["steps"])
    assert info["iteration"] == rinfo["iteration"] == g["iteration"]
    assert info["health"] == 0
    a, b = interior(g["case"], got), interior(g["case"], ref)
    assert info["time"] == rinfo["time"] and info["dt"] == rinfo["dt"]
    assert np.array_equal(a, b)
    tol = max(g["meta"]["rtol"], 1e-12 if g["case"]["blocks"] else 0.0)
    fx = interior(g["case"], g["values"])
    if tol == 0:
        assert np.array_equal(a, fx)
    else:
        assert rel_linf(a, fx) <= tol


@pytest.mark.gpu
def test_device_viscous_kernels_launch(tslib):
    """A viscous step launches the gradient kernels (interior and one per
    active axis) in front of the face fluxes."""
    from turbostructred_gb300 import capi
    g = load("visc3d_box")
    case = capi.make_case(**g["case"])
    with capi.Solver(case, precision=capi.PRECISION_FP64) as s:
        s.set_state(g["initial"], capi.LAYOUT_WITH_GHOSTS)
        _, tm = s.step_timed(2)
    names = set(tm["kernels"])
    assert {"k_vgrad", "k_vgrad_bc_x", "k_vgrad_bc_y", "k_vgrad_bc_z"} <= names
