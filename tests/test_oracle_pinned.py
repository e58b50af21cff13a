"""The CPU oracle is pinned to the reference's own results.

Every fixture in tests/golden/ was produced by the reference solver's code
(ExplicitRungeKuttaFVM built from its sources, see tests/golden/make_golden.py).
The oracle must reproduce each one bit for bit: state with ghosts, iteration
count, final time (including the dt overshoot past MaxTime), last dt and the
residual norms.
"""
import numpy as np
import pytest

from conftest import golden_names, load_golden


@pytest.mark.parametrize("name", golden_names())
def test_oracle_matches_reference_bitwise(name, oracle_mod):
    g = load_golden(name)
    vals, info = oracle_mod.advance(g["case"], g["initial"], g["meta"]["steps"])
    assert info["iteration"] == g["iteration"]
    assert info["time"] == g["time"]
    assert info["dt"] == g["dt"]
    assert np.array_equal(vals, g["values"])
    assert np.array_equal(np.array(info["residual"]), g["residual"])


@pytest.mark.parametrize("name", golden_names())
def test_oracle_grid_matches_reference(name, oracle_mod):
    g = load_golden(name)
    for mine, ref in zip(oracle_mod.grid(g["case"]), (g["x"], g["hx"], g["y"], g["hy"], g["z"], g["hz"])):
        assert np.array_equal(mine, ref)


def test_c1_sod_known_answer():
    # The headline 1D case: 1746 steps ending at t = 0.20001806774119135
    # (dt is not clipped to MaxTime, kernel.h:1841).
    g = load_golden("c1_sod_pwc_roe")
    assert g["iteration"] == 1746
    assert g["time"] == 0.20001806774119135


@pytest.mark.parametrize("name", ["toro1_pwc", "toro3_pwc", "toro4_pwc", "toro5_pwc"])
def test_exact_riemann_matches_reference_sampler(name, oracle_mod):
    """The oracle's exact Riemann solver (used for the HLLC and stiffened-gas
    checks, which the reference cannot pin) agrees with the reference's exact
    Toro sampler (ToroTests.h:234-392), whose star states are rounded to 5-6
    digits, on nearly every cell."""
    g = load_golden(name)
    case = g["case"]
    n = int(g["meta"]["toro"])
    states = {1: ((1.0, 0.0, 1.0), (0.125, 0.0, 0.1), 0.25), 3: ((1.0, 0.0, 1000.0), (1.0, 0.0, 0.01), 0.012),
              4: ((1.0, 0.0, 0.01), (1.0, 0.0, 100.0), 0.035),
              5: ((5.99924, 19.5975, 460.894), (5.99242, -6.19633, 46.0950), 0.035)}
    left, right, _ = states[n]
    x = g["x"][1:-1] - 0.5
    h = g["hx"][1:-1]
    t = g["time"]
    gam = case["gamma"]
    d2 = 0.5773502691896257
    mine = np.zeros((len(x), 5))
    for i in range(len(x)):
        acc = np.zeros(5)
        for xs in (x[i] - d2 * 0.5 * h[i], x[i] + d2 * 0.5 * h[i]):
            r, u, p = oracle_mod.exact_riemann(gam, 0.0, left, right, xs / t)
            acc += [r, r * u, 0, 0, p / 0.4 + 0.5 * r * u * u]
        mine[i] = 0.5 * acc
    ex = g["exact"]
    rel = np.abs(mine - ex).max(axis=1) / np.abs(ex).max(axis=1)
    assert np.mean(rel < 2e-3) > 0.97
