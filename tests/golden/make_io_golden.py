"""Generates tests/golden/io/: the reference's own solution files.

Runs the reference's ExplicitRungeKuttaFVM (oracle/_ref/ref_run, built from its
sources by oracle/ref_build/Makefile) on small 1D/2D/3D cases and stores the
bytes its Kernel::SaveSolution and Kernel::SaveSolutionToTecplot write
(src/kernel/kernel.h:992-1413), plus a Kernel::LoadSolution case: a saved file
loaded into a run that then steps on (time and snapshot schedule restart from
the file, kernel.h:1029-1079).

    make -C oracle/ref_build REF=<reference checkout>
    python tests/golden/make_io_golden.py

Per case: <name>.npz (problem, initial state, final interior state, time,
iteration), <name>.bin (SaveSolution), <name>.dat (SaveSolutionToTecplot).
"""
from __future__ import annotations

import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "io")
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import oracle as O  # noqa: E402
from turbostructred_gb300 import capi as T  # noqa: E402

NAT = (O.BC_NATURAL, 0.0, (0.0, 0.0, 0.0), 0.0)
SYM = (O.BC_SYMMETRY, 0.0, (0.0, 0.0, 0.0), 0.0)
QUAD = [1.5, 0.0, 0.0, 1.5, 0.53, 1.2, 0.0, 0.3, 0.14, 1.2, 1.2, 0.03, 0.53, 0.0, 1.2, 0.3]


def cases():
    # (name, case, scenario, seed, params, steps, molar_mass, gas_constant)
    return [
        ("io_sod1d", O.make_case(ndims=1, nx=100, periodic=(0, 1, 1), recon=O.RECON_PWC, cfl=0.5, max_time=1e30,
                                 bc=[NAT] * 6),
         T.SCENARIO_SHOCK_TUBE, 0, [0.5, 1.0, 0.0, 1.0, 0.125, 0.0, 0.1], 20, 0.029, 8.3144598),
        ("io_quad2d", O.make_case(ndims=2, nx=16, ny=12, periodic=(0, 0, 1), recon=O.RECON_LINEAR2_LIM, cfl=0.4,
                                  max_time=1e30, save_solution_time=0.01, bc=[NAT] * 6),
         T.SCENARIO_QUADRANTS, 1, QUAD, 5, 0.029, 8.3144598),
        ("io_blast3d", O.make_case(ndims=3, nx=8, ny=6, nz=5, periodic=(0, 0, 0), recon=O.RECON_LINEAR2_LIM,
                                   cfl=0.4, max_time=1e30, bc=[SYM] * 6),
         T.SCENARIO_BLAST, 3, [1.0, 0.1, 10.0, 0.3, 0.01], 3, None, None),
    ]


def main():
    if not O.ref_available():
        sys.exit("oracle/_ref/ref_run is not built (make -C oracle/ref_build)")
    os.makedirs(OUT, exist_ok=True)
    index = {}
    saved = {}
    for name, case, scen, seed, params, steps, mm, rg in cases():
        ic = T.fill_scenario(T.make_case(**case), scen, seed, params)
        r = O.run_reference(case, ic, steps=steps, save_solution=True, save_tecplot=True, molar_mass=mm,
                            gas_constant=rg)
        sl = O.interior_slices(case)
        final = r["values"][sl]
        meta = dict(case=case, steps=steps, molar_mass=mm if mm is not None else 0.0,
                    gas_constant=rg if rg is not None else 8.3144598)
        np.savez_compressed(os.path.join(OUT, name + ".npz"), initial=ic, final=final,
                            scalars=np.array([r["iteration"], r["time"]]),
                            meta=np.frombuffer(json.dumps(meta).encode(), dtype=np.uint8))
        with open(os.path.join(OUT, name + ".bin"), "wb") as f:
            f.write(r["solution_bytes"])
        with open(os.path.join(OUT, name + ".dat"), "wb") as f:
            f.write(r["tecplot_bytes"])
        saved[name] = (case, ic, r["solution_bytes"])
        index[name] = dict(iteration=r["iteration"], time=r["time"], bin=len(r["solution_bytes"]),
                           dat=len(r["tecplot_bytes"]))
        print(f"{name:12s} iterations {r['iteration']} t {r['time']!r} bin {len(r['solution_bytes'])} "
              f"dat {len(r['tecplot_bytes'])}")
    # LoadSolution: the 2D file loaded into a fresh run (its own initial state
    # is overwritten), then 4 more steps with the snapshot schedule restarted
    case, ic, blob = saved["io_quad2d"]
    r = O.run_reference(case, np.ones_like(ic), steps=4, load_solution=blob, save_solution=True)
    sl = O.interior_slices(case)
    meta = dict(case=case, steps=4, loads="io_quad2d.bin")
    np.savez_compressed(os.path.join(OUT, "io_load2d.npz"), final=r["values"][sl],
                        scalars=np.array([r["iteration"], r["time"]]),
                        meta=np.frombuffer(json.dumps(meta).encode(), dtype=np.uint8))
    with open(os.path.join(OUT, "io_load2d.bin"), "wb") as f:
        f.write(r["solution_bytes"])
    index["io_load2d"] = dict(iteration=r["iteration"], time=r["time"], bin=len(r["solution_bytes"]))
    print(f"io_load2d    iterations {r['iteration']} t {r['time']!r}")
    with open(os.path.join(OUT, "index.json"), "w") as f:
        json.dump(index, f, indent=1, sort_keys=True)


if __name__ == "__main__":
    main()
