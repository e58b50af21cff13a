"""Seeded synthetic workloads of the batched and served configurations.

tubes():   4096 independent 1D shock tubes (grid sizes log-uniform in
           64..4096 cells; left/right density and pressure log-uniform in
           [0.1, 10], velocity uniform in [-1, 1]; half ideal gas gamma 1.4,
           half stiffened gas gamma 4.4 with p_inf = 6e8 Pa expressed in the
           tube's pressure unit of 1e8 Pa, i.e. p_inf = 6; piecewise-constant
           and limited linear (Barth-Jespersen) reconstruction mixed; Roe flux;
           CFL 0.5; transmissive ends; t_end = 0.1).
stream():  2D ideal-gas four-quadrant Riemann problems arriving as a Poisson
           process (grid side drawn from {64, 128, 256, 512, 1024}; quadrant
           density and pressure uniform in [0.1, 2], |u|, |v| <= 1; Roe or HLLC
           flux at random; 500 RK steps each; limited linear reconstruction,
           CFL 0.4, transmissive boundaries).
"""
from __future__ import annotations

import numpy as np

from . import capi

NAT = (capi.BC_NATURAL, 0.0, (0.0, 0.0, 0.0), 0.0)


def tubes(count: int = 4096, seed: int = 4096, t_end: float = 0.1, max_iter: int = 10_000_000, fill=None):
    """[(case, initial state)] of the batched-tubes configuration.  `fill`
    builds a scenario's state (default: the library's ts_fill_scenario; the
    CPU legs of the bench pass the oracle's bit-identical restatement)."""
    fill = fill or capi.fill_scenario
    rng = np.random.default_rng(seed)
    out = []
    for k in range(count):
        n = int(round(np.exp(rng.uniform(np.log(64), np.log(4096)))))
        rho = np.exp(rng.uniform(np.log(0.1), np.log(10.0), 2))
        p = np.exp(rng.uniform(np.log(0.1), np.log(10.0), 2))
        u = rng.uniform(-1.0, 1.0, 2)
        stiff = k % 2 == 1
        recon = capi.RECON_LINEAR2_LIM if (k // 2) % 2 else capi.RECON_PWC
        case = capi.make_case(ndims=1, nx=n, periodic=(0, 1, 1), gamma=4.4 if stiff else 1.4,
                              eos=capi.EOS_STIFFENED if stiff else capi.EOS_IDEAL, p_inf=6.0 if stiff else 0.0,
                              recon=recon, limiter=capi.LIM_BJ, solver=capi.RS_ROE, cfl=0.5, max_time=t_end,
                              max_iter=max_iter, bc=[NAT] * 6)
        ic = fill(case, capi.SCENARIO_SHOCK_TUBE, seed + k, [0.5, rho[0], u[0], p[0], rho[1], u[1], p[1]])
        out.append((case, ic))
    return out


SIDES = (64, 128, 256, 512, 1024)


def quadrant_case(side: int, solver: int, steps: int = 500):
    return capi.make_case(ndims=2, nx=side, ny=side, periodic=(0, 0, 1), recon=capi.RECON_LINEAR2_LIM,
                          limiter=capi.LIM_BJ, solver=solver, cfl=0.4, max_iter=steps, max_time=1e30,
                          bc=[NAT] * 6)


def stream(rate_hz: float = 200.0, seconds: float = 60.0, seed: int = 200, steps: int = 500, sides=SIDES):
    """[(arrival time s, case, initial state)] of a Poisson request stream."""
    rng = np.random.default_rng(seed)
    t = 0.0
    out = []
    k = 0
    while True:
        t += rng.exponential(1.0 / rate_hz)
        if t >= seconds:
            break
        side = int(sides[rng.integers(len(sides))])
        solver = capi.RS_ROE if rng.integers(2) == 0 else capi.RS_HLLC
        q = []
        for _ in range(4):
            q += [rng.uniform(0.1, 2.0), rng.uniform(-1.0, 1.0), rng.uniform(-1.0, 1.0), rng.uniform(0.1, 2.0)]
        out.append((t, quadrant_case(side, solver, steps), q, seed + k))
        k += 1
    return out


def stream_state(case: dict, params, seed: int, fill=None):
    return (fill or capi.fill_scenario)(case, capi.SCENARIO_QUADRANTS, seed, params)
