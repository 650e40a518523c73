"""The whole gradient chain of a reconstruction parameter vector on the CPU, as the reference's
sensitivity script checks it (scripts/sensitivities_1d.jl:98-176: a MassFractionSC material with a
Boxed or Bilinear field of a few parameters, adjoint Jacobian against finite differences):
parameters -> material fields (oracle/material_oracle.py) -> march and intensities (the C oracle)
-> adjoint -> material pullback.  The adjoint is the reference's continuous-style one, so it
agrees with finite differences to discretisation level."""
import numpy as np
import pytest

import material_oracle as mo
from pnepma_gb300 import workloads
from pnepma_gb300.material_model import MaterialModel, Slices

UM = 1e-4


@pytest.mark.parametrize("par", ["bilinear", "boxed"])
def test_parameter_gradient_of_the_intensities_against_finite_differences(oracle, par):
    s = workloads.small_case(dims=1, N=3, shape=(24,), n_steps=12)
    if par == "bilinear":
        sl = [Slices.range(-0.55 * UM, 0.05 * UM, 6), Slices.range(0.0, 0.0, 1), Slices.range(0.0, 0.0, 1)]
    else:
        sl = [Slices.vector([-0.6 * UM, -0.35 * UM, -0.2 * UM, -0.1 * UM, 0.05 * UM]),
              Slices.range(-0.5, 0.5, 2), Slices.range(-0.5, 0.5, 2)]
    mm = MaterialModel(s.material.gspec, s.material.elements, "mass_fraction", sc=True, parametrization=par,
                       slices=sl, x_rays=s.x_rays, detector=s.detector,
                       beam_x=s.problem.beam_position.mean[0])
    rng = np.random.default_rng(4)
    P = mm.random_params(rng, 0.3, 0.7)
    desc, keep = s.problem.descriptor(s.x_rays)
    rho, noa, acs = mo.fields(mm, P)
    I0 = oracle.forward(desc, rho, noa, acs)
    ib = np.array([1.0, 0.7]) / np.abs(I0)
    _, rb, nb, ab = oracle.adjoint(desc, rho, noa, acs, ib)
    G = mo.pullback(mm, P, rb, nb, acs, ab)

    def J(Q):
        return float(ib @ oracle.forward(desc, *mo.fields(mm, Q)))

    h = 1e-6
    n_field = mm.n_params - mm.n_par               # the embedding is never sampled here
    assert np.all(G[n_field:] == 0.0)
    fds = []
    for i in range(n_field):
        Qp, Qm = P.copy(), P.copy()
        Qp[i] += h
        Qm[i] -= h
        fds.append((J(Qp) - J(Qm)) / (2 * h))
    fds = np.array(fds)
    assert np.max(np.abs(fds - G[:n_field])) <= 5e-2 * np.max(np.abs(fds)), (fds, G[:n_field])
    d = rng.standard_normal(n_field)
    Qp, Qm = P.copy(), P.copy()
    Qp[:n_field] += h * d
    Qm[:n_field] -= h * d
    fd = (J(Qp) - J(Qm)) / (2 * h)
    assert abs(fd - G[:n_field] @ d) <= 1e-2 * abs(fd)
