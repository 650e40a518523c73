"""Gradient checks on the CPU: exact pullbacks of the material layer, and the reference's adjoint
(continuous-style, pn_intensities.jl:353-413) against central finite differences of the oracle.

The adjoint is not the transpose of the discrete forward, so it matches finite differences only
to discretisation level (the reference's sensitivity script records the difference and asserts
nothing, scripts/sensitivities_1d.jl:150-154); the tolerances below are normwise and loose.
"""
import numpy as np
import pytest

from pnepma_gb300 import workloads
from pnepma_gb300.material import BoxedMassFraction


def _material_inputs(s, vals):
    m = s.material
    mm = BoxedMassFraction(m.elements, m.gspec, vals, sc=m.sc)
    rho = mm.rho_flat()
    noa = mm.number_of_atoms().reshape(-1, mm.n_e)
    acs = mm.absorption(s.x_rays, s.detector, s.problem.beam_position.mean).reshape(-1, len(s.x_rays))
    return mm, rho, noa, acs


@pytest.mark.parametrize("sc", [False, True])
def test_material_pullbacks_are_exact(sc):
    s = workloads.small_case(dims=2, N=3, shape=(7, 6), n_steps=2, elements=("Fe", "Cr", "Ni"))
    m = s.material
    frac = np.concatenate([m.values, 1.0 - m.values.sum(-1, keepdims=True)], -1) if m.sc else m.values
    vals = frac[..., :-1] if sc else frac
    mm = BoxedMassFraction(m.elements, m.gspec, vals, sc=sc)
    acs0 = mm.absorption(s.x_rays, s.detector, (0.0, 0.0, 0.0)).reshape(-1, len(s.x_rays))
    rng = np.random.default_rng(1)
    rb = rng.standard_normal(mm.rho_flat().size)
    nb = rng.standard_normal(mm.number_of_atoms().size)
    ab = rng.standard_normal(acs0.size)
    g = mm.grid_pullback(rb) + mm.noa_pullback(nb.reshape(mm.values.shape[:-1] + (mm.n_e,)))
    g = g + mm.absorption_pullback(s.x_rays, s.detector, (0.0, 0.0, 0.0), acs0, ab)[0]

    def f(v):
        m2 = BoxedMassFraction(m.elements, m.gspec, v, sc=sc)
        return (rb @ m2.rho_flat() + nb @ m2.number_of_atoms().ravel()
                + ab @ m2.absorption(s.x_rays, s.detector, (0.0, 0.0, 0.0)).ravel())

    flat = vals.reshape(-1)
    for q in rng.choice(flat.size, 6, replace=False):
        h = 1e-6
        vp, vm = flat.copy(), flat.copy()
        vp[q] += h
        vm[q] -= h
        fd = (f(vp.reshape(vals.shape)) - f(vm.reshape(vals.shape))) / (2 * h)
        assert abs(fd - g.reshape(-1)[q]) <= 1e-6 * max(1.0, abs(fd))


def _chain_gradient(oracle, s, ib):
    m = s.material
    mm, rho, noa, acs = _material_inputs(s, m.values)
    d, k = s.problem.descriptor(s.x_rays)
    I, rb, nb, ab = oracle.adjoint(d, rho, noa, acs, ib)
    g = mm.grid_pullback(rb)
    g = g + mm.absorption_pullback(s.x_rays, s.detector, s.problem.beam_position.mean, acs, ab)[0]
    g = g + mm.noa_pullback(nb.reshape(mm.values.shape[:-1] + (mm.n_e,)))
    return I, g, d, k


@pytest.mark.parametrize("case", [dict(dims=1, shape=(24,), n_steps=12), dict(dims=2, shape=(12, 10), n_steps=10)],
                         ids=["1d", "2d"])
def test_adjoint_gradient_against_finite_differences(oracle, case):
    s = workloads.small_case(N=3, **case)
    d0, k0 = s.problem.descriptor(s.x_rays)
    mm, rho, noa, acs = _material_inputs(s, s.material.values)
    I0 = oracle.forward(d0, rho, noa, acs)
    ib = np.array([1.0, 0.7]) / np.abs(I0)
    I, g, d, k = _chain_gradient(oracle, s, ib)
    flat = s.material.values.reshape(-1)
    rng = np.random.default_rng(0)

    def J(v):
        _, r, n_, a = _material_inputs(s, v.reshape(s.material.values.shape))
        return float(ib @ oracle.forward(d, r, n_, a))

    h = 1e-6
    # directional derivative along a random direction
    dirn = rng.standard_normal(flat.size)
    fd = (J(flat + h * dirn) - J(flat - h * dirn)) / (2 * h)
    assert abs(fd - g.reshape(-1) @ dirn) <= 1e-2 * abs(fd)
    # single cells, normwise over the sample
    idx = rng.choice(flat.size, 8, replace=False)
    fds, ads = [], []
    for q in idx:
        vp, vm = flat.copy(), flat.copy()
        vp[q] += h
        vm[q] -= h
        fds.append((J(vp) - J(vm)) / (2 * h))
        ads.append(g.reshape(-1)[q])
    fds, ads = np.array(fds), np.array(ads)
    assert np.max(np.abs(fds - ads)) <= 5e-2 * np.max(np.abs(fds))


def test_box_perturbation_equals_full_recomputation():
    """The local input update used by the 3D finite-difference check (one box changed) gives the
    same rho and number of atoms as recomputing the material, and absorption factors to rounding."""
    from pnepma_gb300.material import BoxPerturbation
    s = workloads.small_case(dims=3, N=3, shape=(8, 7, 6), n_steps=2, elements=("Fe", "Cr", "Ni"))
    m = s.material
    base = s.inputs()
    boxes = [(1, 3, 4), (0, 0, 7), (5, 6, 0), (2, 2, 2)]
    bp = BoxPerturbation(m, s.x_rays, s.detector, s.problem.beam_position.mean, boxes, base)
    for b in boxes:
        delta = np.array([1e-3, 0.0, -2e-3])
        rho, noa, acs = bp.inputs(b, delta)
        v = m.values.copy()
        v[b] += delta
        m2 = BoxedMassFraction(m.elements, m.gspec, v, sc=m.sc)
        assert np.array_equal(rho, m2.rho_flat())
        assert np.array_equal(noa, m2.number_of_atoms().reshape(-1, m.n_e))
        a2 = m2.absorption(s.x_rays, s.detector, s.problem.beam_position.mean).reshape(acs.shape)
        assert np.max(np.abs(acs - a2) / a2) < 1e-14
