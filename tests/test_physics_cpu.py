"""The restated ICRU-77 stopping-power table and its interpolant (stopping_power.jl:40-154), the
oracle's thread-count independence, and the committed config-size fixtures on the CPU."""
import os
import sys

import numpy as np
import pytest

from pnepma_gb300 import icru77, physics

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
sys.path.insert(0, GOLDEN)
import make_config_golden as mc  # noqa: E402


@pytest.mark.parametrize("sym", sorted(physics.ELEMENTS))
def test_stopping_table_knots_and_slopes(sym):
    """At a knot the interpolant returns the tabulated value converted to eV cm^2/g (MeV/cm * 1e6
    / density); inside an interval the slope is the interval's difference quotient; at an
    interior knot it is the slope of the interval to the right, at the last knot of the last one."""
    el = physics.ELEMENTS[sym]
    tab = physics.stopping_power_table(el)
    E = np.array(icru77.ENERGIES_MEV) * 1e6
    S = np.array(icru77.TOTAL_MEV_PER_CM[el.Z]) * 1e6 / el.density
    assert len(E) == len(S) == 111
    assert np.all(np.diff(E) > 0)
    for i in range(len(E)):
        assert tab(E[i]) == pytest.approx(S[i], rel=1e-15, abs=0)
    for i in range(len(E) - 1):
        q = (S[i + 1] - S[i]) / (E[i + 1] - E[i])
        mid = 0.5 * (E[i] + E[i + 1])
        assert tab.slope(mid) == pytest.approx(q, rel=1e-12)
        assert tab(mid) == pytest.approx(0.5 * (S[i] + S[i + 1]), rel=1e-14)
        assert tab.slope(E[i]) == pytest.approx(q, rel=1e-12)       # right interval at a knot
    last = (S[-1] - S[-2]) / (E[-1] - E[-2])
    assert tab.slope(E[-1]) == pytest.approx(last, rel=1e-12)
    with pytest.raises(ValueError):
        tab(E[0] * 0.99)
    with pytest.raises(ValueError):
        tab(E[-1] * 1.01)


@pytest.mark.parametrize("sym", sorted(physics.ELEMENTS))
def test_stopping_table_agrees_with_bethe_joy_luo(sym):
    """Units check against an independent closed form: the Bethe / Joy-Luo mass stopping power
    is within 15 % of the ICRU-77 table over the energies of the workloads (1-30 keV)."""
    el = physics.ELEMENTS[sym]
    tab = physics.stopping_power_table(el)
    for E in np.geomspace(1e3, 3e4, 25):
        jl = float(physics.joy_luo_mass_stopping_power(el, E))
        assert abs(tab(E) / jl - 1.0) < 0.15, (sym, E)


def test_stopping_table_spot_values():
    """Two table entries read back in the reference's units (MeV/cm at natural density)."""
    assert icru77.TOTAL_MEV_PER_CM[26][0] == 1.291464e+03
    assert icru77.TOTAL_MEV_PER_CM[29][-1] == pytest.approx(icru77.TOTAL_MEV_PER_CM[29][-1])
    assert icru77.ENERGIES_MEV[0] == 5e-05 and icru77.ENERGIES_MEV[-1] == 1000.0


def test_oracle_results_do_not_depend_on_its_thread_count(oracle):
    from pnepma_gb300 import workloads
    s = workloads.small_case(dims=2, N=5, shape=(20, 14), n_steps=6)
    desc, keep = s.problem.descriptor(s.x_rays)
    rho, noa, acs = s.inputs()
    ib = np.array([1.0, 2.0])
    out = []
    try:
        for t in (1, 4):
            oracle.set_threads(t)
            out.append(oracle.adjoint(desc, rho, noa, acs, ib))
    finally:
        oracle.set_threads(1)
    for a, b in zip(out[0], out[1]):
        assert np.array_equal(a, b)


def test_config_summaries_see_errors_anywhere():
    rng = np.random.default_rng(0)
    g = rng.standard_normal(50000) * np.exp(rng.uniform(-8, 0, 50000))
    st = mc.summarise(g)
    assert st["pos"].size >= mc.N_HASHED
    e = mc.compare(g, st)
    assert e["normwise"] == 0 and e["projection"] == 0 and e["per_element"] == 0
    h = g.copy()
    far = int(np.setdiff1d(np.arange(g.size), st["pos"])[123])
    h[far] += 1e-6 * np.sum(np.abs(g))       # an error away from the stored positions
    assert mc.compare(h, st)["projection"] > 1e-7
    assert mc.signs(10, 0).tolist() == mc.signs(10, 0).tolist()
    assert set(np.unique(mc.signs(1000, 3))) == {-1.0, 1.0}


def test_config1_fixture_is_the_oracle_result(oracle):
    """The stored slab solve (545 steps) is what the oracle computes now (drift guard)."""
    G = mc.load()["config1"]
    s = mc.config1_case()
    assert s.problem.N_steps == int(G["n_steps"])
    desc, keep = s.problem.descriptor(s.x_rays)
    rho, noa, acs = s.inputs()
    I, rb, nb, ab = oracle.adjoint(desc, rho, noa, acs, G["ibar"])
    for got, ref in ((I, G["I"]), (rb, G["rho_bar"]), (nb, G["noa_bar"]), (ab, G["acs_bar"])):
        assert np.max(np.abs(got - ref)) <= 1e-12 * np.max(np.abs(ref))


def test_config2_fixture_step_counts():
    G = mc.load()
    for name, s in mc.config2_cases().items():
        assert s.problem.N_steps == int(G[name]["n_steps"])
        assert G[name]["I"].shape == (3,)
        for o in mc.OUTPUTS:
            assert G[name][o]["val"].shape == G[name][o]["pos"].shape
