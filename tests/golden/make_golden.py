"""Generates tests/golden/*.npz from the reference solver's own code.

Runs the reference's ExplicitRungeKuttaFVM (compiled from its sources into
oracle/_ref/ by oracle/ref_build/Makefile; needs the reference checkout) on a
set of small cases and stores, per case: the problem dict, the initial state,
the final Kernel::values array (with ghosts), step info, residual norms, the
grid, and for the Toro cases the reference's exact solution and error norms.

    make -C oracle/ref_build REF=<reference checkout>
    python tests/golden/make_golden.py

Initial states come from the product's scenario generator (host code, no GPU)
or, for the Toro cases, from the reference's own cell-averaged quadrature;
either way the fixture stores them, so tests never regenerate them.
"""
from __future__ import annotations

import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import oracle as O  # noqa: E402
from turbostructred_gb300 import capi as T  # noqa: E402

NAT = (O.BC_NATURAL, 0.0, (0.0, 0.0, 0.0), 0.0)
SYM = (O.BC_SYMMETRY, 0.0, (0.0, 0.0, 0.0), 0.0)
WALL = (O.BC_WALL, 0.0, (0.0, 0.0, 0.0), 0.0)
MOVW = (O.BC_MOVING_WALL, 0.0, (0.3, -0.2, 0.1), 0.0)
INLET = (O.BC_SUBSONIC_INLET, 1.2, (0.4, 0.05, 0.0), 1.1)
OUTLET = (O.BC_SUBSONIC_OUTLET, 0.0, (0.0, 0.0, 0.0), 0.0)

SOD = [0.5, 1.0, 0.0, 1.0, 0.125, 0.0, 0.1]


def sod_case(**kw):
    base = dict(ndims=1, nx=1000, periodic=(0, 1, 1), recon=O.RECON_PWC, solver=O.RS_ROE, cfl=0.5,
                max_iter=1000000, max_time=0.2, bc=[NAT] * 6)
    base.update(kw)
    return O.make_case(**base)


def cases():
    out = []
    # C1: 1D Sod, 1000 cells, PWC + Roe, CFL 0.5, t_end 0.2, transmissive ends
    c = sod_case()
    out.append(("c1_sod_pwc_roe", c, ("scenario", T.SCENARIO_SHOCK_TUBE, 0, SOD), -1))
    for name, rec, lim in [("sod_lim_bj", O.RECON_LINEAR2_LIM, O.LIM_BJ),
                           ("sod_lim_venkat", O.RECON_LINEAR2_LIM, O.LIM_VENKAT),
                           ("sod_eno2", O.RECON_ENO2, O.LIM_BJ)]:
        c = sod_case(nx=200, recon=rec, limiter=lim)
        out.append((name, c, ("scenario", T.SCENARIO_SHOCK_TUBE, 0, SOD), -1))
    # Harten entropy fix and a dt clipped by SaveSolutionTime (ExplicitRungeKuttaFVM.h:1433)
    c = sod_case(nx=300, eps=0.05, save_solution_time=0.03, max_time=0.1)
    out.append(("sod_eps_snapshots", c, ("scenario", T.SCENARIO_SHOCK_TUBE, 0, SOD), -1))
    # Toro tests 1-5 through the reference's own ToroTests set-up (quadrature IC)
    # (ToroTests::DefaultSettings :53-83: CFL 0.45, gamma = 0.4 + 1, MaxTime = t_res)
    t_res = {1: 0.25, 2: 0.15, 3: 0.012, 4: 0.035, 5: 0.035}
    # Test 2 (the 1-2-3 problem) is left out: the reference's Roe flux turns
    # it into NaN/inf at this resolution.
    for n in (1, 3, 4, 5):
        c = sod_case(nx=200, cfl=0.45, max_time=t_res[n], gamma=0.4 + 1.0)
        out.append((f"toro{n}_pwc", c, ("toro", n), -1))
    c = sod_case(nx=200, cfl=0.45, max_time=t_res[1], gamma=0.4 + 1.0, recon=O.RECON_LINEAR2_LIM,
                 limiter=O.LIM_VENKAT)
    out.append(("toro1_lim_venkat", c, ("toro", 1), -1))
    # Unlimited central slopes on a smooth periodic wave
    c = O.make_case(ndims=1, nx=128, periodic=(1, 1, 1), recon=O.RECON_LINEAR2, solver=O.RS_ROE, cfl=0.4,
                    max_iter=60, max_time=1e9)
    out.append(("wave_linear2_periodic", c, ("wave",), -1))
    # C2-like 2D shear layer, periodic, limited linear + Roe
    c = O.make_case(ndims=2, nx=32, ny=32, periodic=(1, 1, 1), recon=O.RECON_LINEAR2_LIM, solver=O.RS_ROE,
                    cfl=0.4, max_iter=25, max_time=1e9)
    out.append(("shear2d_bj_roe", c, ("scenario", T.SCENARIO_SHEAR_LAYER, 7, [2.0, 1.0, 0.5, 2.5, 0.01]), -1))
    c = dict(c, limiter=O.LIM_VENKAT, nx=24, ny=20)
    out.append(("shear2d_venkat_roe", c, ("scenario", T.SCENARIO_SHEAR_LAYER, 8, [2.0, 1.0, 0.5, 2.5, 0.01]), -1))
    # every boundary condition type, ENO2
    c = O.make_case(ndims=2, nx=24, ny=20, periodic=(0, 0, 1), recon=O.RECON_ENO2, solver=O.RS_ROE, cfl=0.4,
                    max_iter=15, max_time=1e9, bc=[INLET, OUTLET, MOVW, WALL, NAT, NAT])
    out.append(("bc2d_eno2", c, ("scenario", T.SCENARIO_SHEAR_LAYER, 9, [1.5, 1.0, 0.3, 2.0, 0.02]), -1))
    # stretched grid (CompressionX/Y blocks), symmetry/wall, limited
    c = O.make_case(ndims=2, nx=24, ny=20, periodic=(0, 0, 1), recon=O.RECON_LINEAR2_LIM, solver=O.RS_ROE,
                    cfl=0.4, max_iter=20, max_time=1e9, bc=[NAT, NAT, WALL, SYM, NAT, NAT],
                    blocks={0: [(0.0, 1.05, 10), (0.4, 0.97, 14)], 1: [(0.0, 1.1, 20)]})
    out.append(("stretched2d_bj", c, ("scenario", T.SCENARIO_SHEAR_LAYER, 10, [2.0, 1.0, 0.5, 2.5, 0.01]), -1))
    # C3-like 3D blast with reflective (Symmetry) walls, limited linear + Roe
    c = O.make_case(ndims=3, nx=12, ny=12, nz=12, periodic=(0, 0, 0), recon=O.RECON_LINEAR2_LIM,
                    solver=O.RS_ROE, cfl=0.4, max_iter=10, max_time=1e9, bc=[SYM] * 6)
    out.append(("blast3d_sym_bj_roe", c, ("scenario", T.SCENARIO_BLAST, 11, [1.0, 0.1, 10.0, 0.25, 0.01]), -1))
    # 3D mixed periodic/wall, PWC with Harten fix; odd sizes
    c = O.make_case(ndims=3, nx=9, ny=7, nz=6, periodic=(1, 0, 1), recon=O.RECON_PWC, solver=O.RS_ROE,
                    cfl=0.45, eps=0.05, max_iter=12, max_time=1e9, bc=[NAT, NAT, WALL, WALL, NAT, NAT])
    out.append(("blast3d_mixed_pwc", c, ("scenario", T.SCENARIO_BLAST, 12, [1.0, 0.1, 10.0, 0.3, 0.01]), -1))
    # 3D Venkatakrishnan on anisotropic cells; a mild pressure jump, since the
    # reference's eps^2 (not normalised, Limiters.h:93-112) hardly limits and
    # a strong blast goes negative in the reference itself.
    c = O.make_case(ndims=3, nx=10, ny=8, nz=6, length=(1.0, 0.8, 0.5), periodic=(0, 1, 0),
                    recon=O.RECON_LINEAR2_LIM, limiter=O.LIM_VENKAT, solver=O.RS_ROE, cfl=0.4, max_iter=8,
                    max_time=1e9, bc=[SYM, SYM, NAT, NAT, WALL, NAT])
    out.append(("blast3d_venkat_aniso", c, ("scenario", T.SCENARIO_BLAST, 13, [1.0, 0.5, 1.0, 0.2, 0.01]), -1))
    # source terms (Kernel::ProcessExternalForces / ProcessExternalAcceleration)
    c = sod_case(nx=200, recon=O.RECON_LINEAR2_LIM, external_force=(0.3, 0.1, 0.0), max_time=0.1)
    out.append(("force1d_lim", c, ("scenario", T.SCENARIO_SHOCK_TUBE, 0, SOD), -1))
    c = O.make_case(ndims=2, nx=32, ny=48, periodic=(1, 0, 1), recon=O.RECON_LINEAR2_LIM, cfl=0.4,
                    max_time=1e30, uniform_acceleration=(0.0, -1.0, 0.0), bc=[NAT, NAT, WALL, WALL, NAT, NAT])
    heavy_top = [2.0, 0.0, 0.0, 2.5, 2.0, 0.0, 0.0, 2.5, 1.0, 0.0, 0.0, 2.5, 1.0, 0.0, 0.0, 2.5]
    out.append(("gravity2d_rt", c, ("scenario", T.SCENARIO_QUADRANTS, 0, heavy_top), 40))
    c = O.make_case(ndims=3, nx=12, ny=10, nz=9, periodic=(0, 0, 0), recon=O.RECON_LINEAR2_LIM, cfl=0.4,
                    max_time=1e30, external_force=(0.0, 0.2, -0.1), uniform_acceleration=(0.1, 0.0, -0.5),
                    bc=[SYM] * 6)
    out.append(("sources3d_both", c, ("scenario", T.SCENARIO_BLAST, 21, [1.0, 0.5, 2.0, 0.3, 0.01]), 8))
    # position-dependent sides (DomainBCinfo::isComplex / getMarker): a plate
    # on the bottom side from x = 0.3 on (Symmetry before it, Wall after, as
    # src/Tests/2DTests/BlasiusFlow.h:115-120), inlet on the left
    c = O.make_case(ndims=2, nx=32, ny=16, periodic=(0, 0, 1), recon=O.RECON_LINEAR2_LIM, solver=O.RS_ROE,
                    cfl=0.4, eps=0.05, max_iter=10**6, max_time=1e9, bc=[INLET, NAT, NAT, NAT, NAT, NAT],
                    bc_kinds=[SYM, WALL], bc_split={2: (0, 0.3, 0, 1)})
    out.append(("marker2d_plate", c, ("scenario", T.SCENARIO_SHEAR_LAYER, 31, [1.2, 1.0, 0.4, 2.0, 0.02]), 20))
    # 3D: the z-low side split along y (Wall below y = 0.45, moving wall
    # above), the x-high side split along z (Natural / Symmetry)
    c = O.make_case(ndims=3, nx=12, ny=10, nz=8, periodic=(0, 0, 0), recon=O.RECON_LINEAR2_LIM,
                    solver=O.RS_ROE, cfl=0.4, max_iter=10**6, max_time=1e9, bc=[SYM, NAT, SYM, SYM, NAT, NAT],
                    bc_kinds=[WALL, MOVW, NAT, SYM], bc_split={4: (1, 0.45, 0, 1), 1: (2, 0.55, 2, 3)})
    out.append(("marker3d_split", c, ("scenario", T.SCENARIO_BLAST, 32, [1.0, 0.5, 3.0, 0.3, 0.01]), 8))
    # HLLC and the stiffened gas are not in the reference: no fixture.
    return out


def initial_state(case, spec):
    kind = spec[0]
    if kind == "scenario":
        tcase = T.make_case(**{k: v for k, v in case.items()})
        return T.fill_scenario(tcase, spec[1], spec[2], spec[3])
    if kind == "wave":
        x = O.grid(case)[0][1:-1]
        g = case["gamma"]
        rho = 1.0 + 0.2 * np.sin(2 * np.pi * x)
        u, p = 0.5, 1.0
        ic = np.zeros((1, 1, case["nx"], 5))
        ic[0, 0, :, 0] = rho
        ic[0, 0, :, 1] = rho * u
        ic[0, 0, :, 4] = p / (g - 1) + 0.5 * rho * u * u
        return ic
    return None


def main():
    """python tests/golden/make_golden.py [name ...]: all cases, or the named
    ones (merged into index.json)."""
    if not O.ref_available():
        sys.exit("oracle/_ref/ref_run is not built (make -C oracle/ref_build)")
    only = set(sys.argv[1:])
    index = {}
    ipath = os.path.join(HERE, "index.json")
    if only and os.path.exists(ipath):
        with open(ipath) as f:
            index = json.load(f)
    for name, case, spec, steps in cases():
        if only and name not in only:
            continue
        ic = initial_state(case, spec)
        toro = spec[1] if spec[0] == "toro" else 0
        r = O.run_reference(case, ic, toro=toro, steps=steps)
        rec = dict(initial=r["initial"], values=r["values"], residual=r["residual"],
                   x=r["x"], hx=r["hx"], y=r["y"], hy=r["hy"], z=r["z"], hz=r["hz"],
                   scalars=np.array([r["iteration"], r["time"], r["dt"]]))
        if toro:
            rec["exact"] = r["exact"]
            rec["errors"] = r["errors"]
        meta = dict(case=case, spec=[s if not isinstance(s, np.ndarray) else s.tolist() for s in spec],
                    steps=steps, toro=toro)
        rec["meta"] = np.frombuffer(json.dumps(meta).encode(), dtype=np.uint8)
        np.savez_compressed(os.path.join(HERE, name + ".npz"), **rec)
        index[name] = dict(iteration=r["iteration"], time=r["time"], seconds=r["seconds"])
        print(f"{name:24s} iterations {r['iteration']:5d} t {r['time']!r}")
    with open(ipath, "w") as f:
        json.dump(index, f, indent=1, sort_keys=True)


if __name__ == "__main__":
    main()
