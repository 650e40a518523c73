"""Convergence of the march (the oracle restatement): intensities settle as the energy step and
the grid are refined.  The reference has no such test; its strategy lists convergence in N_steps
and in the grid as a check of a correct discretisation.  The march is first order in the energy
step (sub-steps of one explicit half/full/half sweep with per-step coefficients), so halving dE
about halves the change."""
import numpy as np

from pnepma_gb300 import workloads


def _intensities(oracle, M, n_steps):
    s = workloads.small_case(dims=1, N=3, shape=(M,), n_steps=n_steps)
    desc, keep = s.problem.descriptor(s.x_rays)
    rho, noa, acs = s.inputs()
    return s.problem.N_steps, oracle.forward(desc, rho, noa, acs)


def _changes(results):
    ref = np.abs(results[-1])
    return [float(np.max(np.abs(results[i + 1] - results[i]) / ref)) for i in range(len(results) - 1)]


def test_intensities_converge_in_the_energy_step(oracle):
    n0, _ = _intensities(oracle, 32, 10)       # the stable step count of this grid
    res = [_intensities(oracle, 32, n0 * f)[1] for f in (1, 2, 4, 8)]
    d = _changes(res)
    for a, b in zip(d, d[1:]):
        assert b < 0.7 * a, d                  # first order: each halving of dE about halves the change
    assert d[-1] < 5e-3


def test_intensities_converge_in_the_grid(oracle):
    n, _ = _intensities(oracle, 128, 10)       # stable on the finest grid, hence on all of them
    res = [_intensities(oracle, M, n)[1] for M in (16, 32, 64, 128)]
    d = _changes(res)
    for a, b in zip(d, d[1:]):
        assert b < 0.7 * a, d
    assert d[-1] < 5e-3
    ratio = [r[0] / r[1] for r in res]         # the line ratio (what a k-ratio compares) settles too
    assert abs(ratio[-1] - ratio[-2]) < abs(ratio[1] - ratio[0])
