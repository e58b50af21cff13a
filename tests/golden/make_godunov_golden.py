"""Generates tests/golden/godunov/*.npz from the reference's exact Godunov flux.

Runs the reference's ExplicitRungeKuttaFVM with RPSolver::GodunovSolver
(GodunovSolverPerfectGasEOS.h, whose star pressure comes from alglib 3.8.0's
Levenberg-Marquardt minimiser) on small 1D/2D/3D cases and stores the same
records as make_golden.py.  The restatement and the device path solve for the
star pressure by Newton's method, so parity with these fixtures is to the
reference's solver tolerance, not bit for bit.

    make -C oracle/ref_build REF=<reference checkout>
    python tests/golden/make_godunov_golden.py
"""
from __future__ import annotations

import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "godunov")
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import oracle as O  # noqa: E402
from turbostructred_gb300 import capi as T  # noqa: E402

NAT = (O.BC_NATURAL, 0.0, (0.0, 0.0, 0.0), 0.0)
SYM = (O.BC_SYMMETRY, 0.0, (0.0, 0.0, 0.0), 0.0)
WALL = (O.BC_WALL, 0.0, (0.0, 0.0, 0.0), 0.0)
SOD = [0.5, 1.0, 0.0, 1.0, 0.125, 0.0, 0.1]
QUAD = [1.5, 0.0, 0.0, 1.5, 0.53, 1.2, 0.0, 0.3, 0.14, 1.2, 1.2, 0.03, 0.53, 0.0, 1.2, 0.3]


def cases():
    G = O.RS_GODUNOV
    return [
        ("god_sod_pwc", O.make_case(ndims=1, nx=200, periodic=(0, 1, 1), recon=O.RECON_PWC, solver=G, cfl=0.5,
                                    max_time=0.2, max_iter=10**6, bc=[NAT] * 6),
         (T.SCENARIO_SHOCK_TUBE, 0, SOD), -1),
        ("god_sod_lim_bj", O.make_case(ndims=1, nx=200, periodic=(0, 1, 1), recon=O.RECON_LINEAR2_LIM, solver=G,
                                       cfl=0.5, max_time=0.2, max_iter=10**6, bc=[NAT] * 6),
         (T.SCENARIO_SHOCK_TUBE, 0, SOD), -1),
        ("god_sod_eno2_wall", O.make_case(ndims=1, nx=150, periodic=(0, 1, 1), recon=O.RECON_ENO2, solver=G,
                                          cfl=0.5, max_time=0.25, max_iter=10**6, bc=[WALL] * 6),
         (T.SCENARIO_SHOCK_TUBE, 0, SOD), -1),
        ("god_quad2d_pwc", O.make_case(ndims=2, nx=40, ny=32, periodic=(0, 0, 1), recon=O.RECON_PWC, solver=G,
                                       cfl=0.4, max_time=1e30, bc=[NAT] * 6),
         (T.SCENARIO_QUADRANTS, 1, QUAD), 30),
        ("god_shear2d_lim", O.make_case(ndims=2, nx=40, ny=32, periodic=(1, 1, 1), recon=O.RECON_LINEAR2_LIM,
                                        solver=G, cfl=0.4, max_time=1e30),
         (T.SCENARIO_SHEAR_LAYER, 2, [2.0, 1.0, 0.5, 2.5, 0.01]), 30),
        ("god_blast3d_lim", O.make_case(ndims=3, nx=16, ny=14, nz=12, periodic=(0, 0, 0), recon=O.RECON_LINEAR2_LIM,
                                        solver=G, cfl=0.4, max_time=1e30, bc=[SYM] * 6),
         (T.SCENARIO_BLAST, 3, [1.0, 0.1, 10.0, 0.25, 0.01]), 10),
    ]


def main():
    if not O.ref_available():
        sys.exit("oracle/_ref/ref_run is not built (make -C oracle/ref_build)")
    os.makedirs(OUT, exist_ok=True)
    index = {}
    for name, case, (scen, seed, params), steps in cases():
        # the scenario generator validates the configuration: build the state
        # for the same grid with the Roe solver selected
        ic = T.fill_scenario(T.make_case(**dict(case, solver=O.RS_ROE)), scen, seed, params)
        r = O.run_reference(case, ic, steps=steps)
        rec = dict(initial=r["initial"], values=r["values"], residual=r["residual"],
                   scalars=np.array([r["iteration"], r["time"], r["dt"]]))
        meta = dict(case=case, steps=steps)
        rec["meta"] = np.frombuffer(json.dumps(meta).encode(), dtype=np.uint8)
        np.savez_compressed(os.path.join(OUT, name + ".npz"), **rec)
        index[name] = dict(iteration=r["iteration"], time=r["time"])
        print(f"{name:20s} iterations {r['iteration']:5d} t {r['time']!r}")
    with open(os.path.join(OUT, "index.json"), "w") as f:
        json.dump(index, f, indent=1, sort_keys=True)


if __name__ == "__main__":
    main()
