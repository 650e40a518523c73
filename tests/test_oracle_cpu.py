"""CPU checks of the oracle and of the host-side problem tables (no GPU).

The reference has no test suite, golden vectors or fixtures for this path; its building blocks
are pinned here by known-answer tests and by agreement of two independent restatements.
"""
import math

import numpy as np
import pytest

import np_oracle
from pnepma_gb300 import matrices as mx
from pnepma_gb300 import moments as mo
from pnepma_gb300 import workloads


def rel(a, b):
    a = np.asarray(a, float).ravel()
    b = np.asarray(b, float).ravel()
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))


# ------------------------------------------------------------------ moments and blocks
@pytest.mark.parametrize("N", range(0, 14))
def test_class_sizes_match_closed_forms(N):
    assert mo.class_sizes(N) == mo.class_sizes_closed_form(N)
    assert sum(mo.class_sizes(N)) == (N + 1) ** 2


def test_parity_classes_and_switch():
    assert mo.classes_of_parity(0) == [0, 3, 5, 6]      # eee, eoo, oeo, ooe
    assert mo.classes_of_parity(1) == [1, 2, 4, 7]
    for c in range(8):
        for d in range(3):
            assert mo.switch(mo.switch(c, d), d) == c
            assert mo.parity(mo.switch(c, d)) != mo.parity(c)


@pytest.mark.parametrize("N", [3, 5, 7])
def test_advection_blocks_equal_quadrature(N):
    T, P, W = mx.sphere_rule(2 * N + 4, 4 * N + 8)
    Ys = mx.real_harmonics(N, T, P)
    om = [np.sin(T) * np.cos(P), np.sin(T) * np.sin(P), np.cos(T)]
    ms = mo.class_moments(N)
    for d in range(3):
        for c in range(8):
            A = mx.advection_block(N, c, d)
            if A.size == 0:
                continue
            Q = np.array([[np.sum(om[d] * Ys[a] * Ys[b] * W) for b in ms[mo.switch(c, d)]] for a in ms[c]])
            assert np.max(np.abs(A - Q)) < 1e-13


def _half_range_rule(d, n_mu=120, n_phi=240):
    x, w = np.polynomial.legendre.leggauss(n_mu)
    mu = 0.5 * (x + 1)
    wm = 0.5 * w
    ph = (np.arange(n_phi) + 0.5) * 2 * math.pi / n_phi
    MU, PH = np.meshgrid(mu, ph, indexing="ij")
    Wt = np.outer(wm, np.full(n_phi, 2 * math.pi / n_phi))
    s = np.sqrt(1 - MU ** 2)
    O = [None] * 3
    others = [e for e in range(3) if e != d]
    O[d], O[others[0]], O[others[1]] = MU, s * np.cos(PH), s * np.sin(PH)
    th = np.arccos(np.clip(O[2].ravel(), -1, 1))
    phi = np.arctan2(O[1].ravel(), O[0].ravel())
    return th, phi, Wt.ravel(), O[d].ravel()


@pytest.mark.parametrize("N", [3, 5])
def test_boundary_L_is_the_half_range_integral(N):
    """L_d = 2 int_{Omega_d > 0} Y_i Y_j / Omega_d: the gamma/binomial sums of pn_matrices.jl:191-275."""
    ms = mo.class_moments(N)
    for d in range(3):
        th, ph, W, od = _half_range_rule(d)
        Ys = mx.real_harmonics(N, th, ph)
        for c in range(8):
            if not mo.odd_in(c, d) or not ms[c]:
                continue
            L = mx.boundary_L(N, c, d)
            Q = np.array([[2 * np.sum(Ys[a] * Ys[b] / od * W) for b in ms[c]] for a in ms[c]])
            assert np.max(np.abs(L - Q)) < 1e-12


def test_boundary_blocks_forward_and_adjoint():
    N = 5
    for d in range(3):
        for c in range(8):
            if not mo.odd_in(c, d) or not mo.class_moments(N)[c]:
                continue
            L = mx.boundary_L(N, c, d)
            A = mx.advection_block(N, c, d)
            assert np.allclose(mx.boundary_block(N, c, d), L @ A, rtol=0, atol=1e-14)
            assert np.allclose(mx.boundary_block(N, c, d, adjoint=True), -L.T @ A, rtol=0, atol=1e-14)


def test_beam_moments_converged():
    ms = list(mo.class_moments(7)[4])
    a = mx.beam_moments(ms, (-1.0, 0.0, 0.0), 50.0)
    b = mx._beam_moments(ms, (-1.0, 0.0, 0.0), 50.0, 300, 600)
    assert np.max(np.abs(a - b)) < 1e-12 * np.max(np.abs(a))


# ------------------------------------------------------------------ the two restatements
CASES = [dict(dims=1, N=5, shape=(16,), n_steps=6), dict(dims=2, N=3, shape=(8, 7), n_steps=5),
         dict(dims=3, N=3, shape=(5, 5, 4), n_steps=3)]
# the edges of the domain: the highest orders, one element, four elements, 3D at P5
EDGE_CASES = [dict(dims=2, N=9, shape=(7, 6), n_steps=3), dict(dims=1, N=11, shape=(10,), n_steps=3),
              dict(dims=2, N=3, shape=(7, 6), n_steps=3, elements=("Fe", "Cr", "Ni", "Cu")),
              dict(dims=1, N=3, shape=(10,), n_steps=4, elements=("Cu",)),
              dict(dims=3, N=5, shape=(4, 4, 3), n_steps=2)]


@pytest.mark.parametrize("case", CASES + EDGE_CASES, ids=["1d", "2d", "3d", "2d-N9", "1d-N11", "2d-4el", "1d-1el", "3d-N5"])
def test_numpy_restatement_matches_c_oracle(oracle, case):
    s = workloads.small_case(**case)
    rho, noa, acs = s.inputs()
    desc, keep = s.problem.descriptor(s.x_rays)
    I_c, tape = oracle.forward(desc, rho, noa, acs, with_tape=True)
    I_n, state_n = np_oracle.forward(desc, rho, noa, acs, return_state=True)
    assert rel(I_n, I_c) < 1e-12
    # the whole final state: interior, ghost and corner points of all eight classes
    assert rel(state_n, tape[-1]) < 1e-12


ADJOINT_CASES = CASES + EDGE_CASES[2:3] + [dict(dims=2, N=7, shape=(6, 5), n_steps=3),
                                             dict(dims=1, N=9, shape=(12,), n_steps=3)]


@pytest.mark.parametrize("case", ADJOINT_CASES, ids=["1d", "2d", "3d", "2d-4el", "2d-N7", "1d-N9"])
def test_numpy_adjoint_matches_c_oracle(oracle, case):
    """The adjoint (density integral, intensity pullback, adjoint source and march) restated twice,
    independently: intensities and all three cotangents agree to rounding."""
    s = workloads.small_case(**case)
    rho, noa, acs = s.inputs()
    desc, keep = s.problem.descriptor(s.x_rays)
    I = oracle.forward(desc, rho, noa, acs)
    ib = np.linspace(1.0, 2.0, len(I)) / np.abs(I)
    c = oracle.adjoint(desc, rho, noa, acs, ib)
    n = np_oracle.adjoint(desc, rho, noa, acs, ib)
    for a, b in zip(n, c):
        assert rel(a, b) < 1e-12


@pytest.mark.parametrize("case", CASES, ids=["1d", "2d", "3d"])
def test_numpy_generation_field_matches_c_oracle(oracle, case):
    s = workloads.small_case(**case)
    rho, noa, acs = s.inputs()
    desc, keep = s.problem.descriptor(s.x_rays)
    assert rel(np_oracle.generation_field(desc, rho), oracle.generation_field(desc, rho)) < 1e-12


@pytest.mark.parametrize("case", CASES, ids=["1d", "2d", "3d"])
def test_single_step_matches(oracle, case):
    s = workloads.small_case(**case)
    rho, noa, acs = s.inputs()
    desc, keep = s.problem.descriptor(s.x_rays)
    rng = np.random.default_rng(3)
    u = rng.standard_normal(oracle.state_size(desc))
    a = oracle.step(desc, rho, u, 1)
    b = np_oracle.one_step(desc, rho, u, 1)
    assert rel(b, a) < 1e-12


# ------------------------------------------------------------------ properties
def test_linearity_in_the_source_is_exact(oracle):
    """Doubling the beam source doubles intensities and rho_bar bit for bit (all operations are
    linear in the state); doubling the cotangent doubles the adjoint outputs."""
    s = workloads.small_case(dims=2, N=3, shape=(8, 7), n_steps=5)
    rho, noa, acs = s.inputs()
    d1, k1 = s.problem.descriptor(s.x_rays)
    t = s.problem.tables(s.x_rays)
    ib = np.array([1.0, -0.5])
    I1, rb1, nb1, ab1 = oracle.adjoint(d1, rho, noa, acs, ib)
    t["beam_face"] *= 2.0
    I2, rb2, nb2, ab2 = oracle.adjoint(d1, rho, noa, acs, ib)
    t["beam_face"] /= 2.0
    assert np.array_equal(I2, 2 * I1)
    assert np.array_equal(rb2, 2 * rb1)
    I3, rb3, nb3, ab3 = oracle.adjoint(d1, rho, noa, acs, 2 * ib)
    assert np.array_equal(rb3, 2 * rb1) and np.array_equal(nb3, 2 * nb1) and np.array_equal(ab3, 2 * ab1)


def test_reflection_symmetry_in_y(oracle):
    """A beam at y = 0 on a material that varies only in depth gives a fluence symmetric in y.
    (A y-symmetric box field is not enough: the box lookup puts odd-grid points that sit on a box
    boundary into the right-hand box, biliner_interp.jl:5-16, which breaks the mirror symmetry.)"""
    from pnepma_gb300.grid import GridSpec
    UM = workloads.UM
    g = GridSpec.make((10, 9, 1), (-0.5 * UM, 0.0), (-0.4 * UM, 0.4 * UM), 0.0)
    rng = np.random.default_rng(11)
    depth = rng.uniform(0.2, 0.8, (1, 1, 10))
    w = np.repeat(depth, 9, axis=1)[..., None]
    frac = np.concatenate([w, 1 - w], axis=-1)
    s = workloads.make_solve(3, g, ["Cu", "Ni"], frac, 12.0, beam_y=0.0, beam_sigma=60 * workloads.NM,
                             n_steps=6, E_cut=7000.0, detector=(50 * workloads.NM, 0.0, 0.0))
    rho, noa, acs = s.inputs()
    desc, keep = s.problem.descriptor(s.x_rays)
    I, tape = oracle.forward(desc, rho, noa, acs, with_tape=True)
    nm0 = mo.class_sizes(3)[0]
    u0 = tape[-1][: 9 * 10 * nm0].reshape(9, 10, nm0)[..., 0]   # eee: [y][x]
    assert rel(u0[::-1], u0) < 1e-12


def test_stable_step_counts_follow_the_estimate():
    s = workloads.config1(stabilise=True)
    assert s.problem.N_steps >= 100
    assert s.problem.delta_e <= 0.6 * s.problem.cfl_dt_max(
        workloads.min_stopping(s.material, s.problem, s.problem.E_initial)) * 1.0000001
