"""Generates tests/golden/viscous/*.npz: viscous-flow runs of the reference.

Runs the reference's ExplicitRungeKuttaFVM with IsViscousFlow / Viscosity
(compiled from its sources into oracle/_ref/ by oracle/ref_build/Makefile;
needs the reference checkout) and stores, per case, the same record as
make_golden.py plus `rtol`: the largest relative difference (max |a - b| /
max |b| over the interior state) the oracle may show against the reference.
It is 0 (bit for bit) where no boundary least-squares gradient enters
(periodic axes, one-dimensional stencils, viscosity only in the spectral
radius) and 1e-13 where the reference's Eigen JacobiSVD and the oracle's
normal equations solve the same small least-squares problems to rounding.

    make -C oracle/ref_build REF=<reference checkout>
    python tests/golden/make_viscous_golden.py
"""
from __future__ import annotations

import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "viscous")
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
SHEAR = [2.0, 1.0, 0.5, 2.5, 0.05]


def cases():
    """(name, case, (scenario, seed, params), steps, rtol)."""
    out = []
    c = O.make_case(ndims=1, nx=100, periodic=(0, 1, 1), recon=O.RECON_PWC, solver=O.RS_ROE, cfl=0.5,
                    max_iter=60, max_time=1e9, bc=[NAT] * 6, viscous=True, viscosity=0.01)
    out.append(("visc1d_sod_pwc", c, (T.SCENARIO_SHOCK_TUBE, 0, SOD), -1, 0.0))
    c = O.make_case(ndims=1, nx=100, periodic=(0, 1, 1), recon=O.RECON_LINEAR2_LIM, solver=O.RS_ROE, cfl=0.5,
                    max_iter=60, max_time=1e9, bc=[NAT] * 6, viscous=False, viscosity=0.01)
    out.append(("viscosity_only_sr_1d", c, (T.SCENARIO_SHOCK_TUBE, 0, SOD), -1, 0.0))
    c = O.make_case(ndims=2, nx=32, ny=32, periodic=(1, 1, 1), recon=O.RECON_LINEAR2_LIM, solver=O.RS_ROE,
                    cfl=0.4, max_iter=20, max_time=1e9, viscous=True, viscosity=1e-3)
    out.append(("visc2d_shear_periodic", c, (T.SCENARIO_SHEAR_LAYER, 7, [2.0, 1.0, 0.5, 2.5, 0.01]), -1, 0.0))
    c = O.make_case(ndims=2, nx=24, ny=16, periodic=(1, 0, 1), recon=O.RECON_LINEAR2_LIM, solver=O.RS_ROE,
                    cfl=0.4, max_iter=20, max_time=1e9, bc=[NAT, NAT, WALL, MOVW, NAT, NAT], viscous=True,
                    viscosity=0.01)
    out.append(("visc2d_channel_walls", c, (T.SCENARIO_SHEAR_LAYER, 8, SHEAR), -1, 1e-13))
    c = O.make_case(ndims=2, nx=24, ny=20, periodic=(0, 0, 1), recon=O.RECON_ENO2, solver=O.RS_ROE, cfl=0.4,
                    max_iter=15, max_time=1e9, bc=[INLET, OUTLET, SYM, WALL, NAT, NAT], viscous=True,
                    viscosity=0.02, blocks={0: [(0.0, 1.05, 10), (0.4, 0.97, 14)], 1: [(0.0, 1.1, 20)]})
    out.append(("visc2d_stretched_inlet", c, (T.SCENARIO_SHEAR_LAYER, 9, [1.5, 1.0, 0.3, 2.0, 0.02]), -1, 1e-13))
    c = O.make_case(ndims=3, nx=12, ny=10, nz=8, periodic=(0, 0, 0), recon=O.RECON_LINEAR2_LIM, solver=O.RS_ROE,
                    cfl=0.4, max_iter=10, max_time=1e9, bc=[SYM, NAT, WALL, WALL, NAT, SYM], viscous=True,
                    viscosity=0.005)
    out.append(("visc3d_box", c, (T.SCENARIO_BLAST, 3, [1.0, 0.5, 2.0, 0.3, 0.05]), -1, 1e-13))
    c = O.make_case(ndims=3, nx=10, ny=8, nz=6, periodic=(1, 0, 1), recon=O.RECON_PWC, solver=O.RS_ROE, cfl=0.45,
                    max_iter=12, max_time=1e9, bc=[NAT, NAT, MOVW, WALL, NAT, NAT], viscous=True, viscosity=0.01)
    out.append(("visc3d_periodic_walls_pwc", c, (T.SCENARIO_BLAST, 4, [1.0, 0.5, 2.0, 0.3, 0.05]), -1, 1e-13))
    return out


def main():
    if not O.ref_available():
        sys.exit("oracle/_ref/ref_run is not built (make -C oracle/ref_build)")
    os.makedirs(OUT, exist_ok=True)
    for name, case, (scen, seed, params), steps, rtol in cases():
        ic = T.fill_scenario(T.make_case(**case), scen, seed, params)
        r = O.run_reference(case, ic, steps=steps)
        rec = dict(initial=r["initial"], values=r["values"], residual=r["residual"],
                   x=r["x"], hx=r["hx"], y=r["y"], hy=r["hy"], z=r["z"], hz=r["hz"],
                   scalars=np.array([r["iteration"], r["time"], r["dt"]]))
        meta = dict(case=case, spec=["scenario", scen, seed, params], steps=steps, rtol=rtol)
        rec["meta"] = np.frombuffer(json.dumps(meta).encode(), dtype=np.uint8)
        np.savez_compressed(os.path.join(OUT, name + ".npz"), **rec)
        print(f"{name:28s} iterations {r['iteration']:5d} t {r['time']!r}")


if __name__ == "__main__":
    main()
