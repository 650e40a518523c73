"""The reference-shaped Python API (pnepma_gb300/api.py) on the GPU: calc_intensities_pullback with
the host material and with a GPUMaterial, against the oracle, with another call on the same
problem between the forward and the pullback."""
import numpy as np
import pytest

import material_oracle as mo
from pnepma_gb300 import api, workloads
from pnepma_gb300.material import BoxedMassFraction
from pnepma_gb300.material_model import MaterialModel

pytestmark = pytest.mark.gpu

TOL64 = 1e-10


def _rel(a, b):
    a, b = np.asarray(a, float).ravel(), np.asarray(b, float).ravel()
    return float(np.max(np.abs(a - b)) / np.max(np.abs(b)))


def test_host_material_path_matches_the_oracle(gpu_lib, oracle):
    s = workloads.small_case(dims=2, N=3, shape=(10, 8), n_steps=6)
    m = s.material
    rho, noa, acs = s.inputs()
    desc, keep = s.problem.descriptor(s.x_rays)
    I, pb = api.calc_intensities_pullback(s.problem, m, s.x_rays, s.detector)
    assert _rel(I, oracle.forward(desc, rho, noa, acs)) < TOL64
    ib = np.linspace(1.0, 2.0, len(I)) / np.abs(I)
    other = BoxedMassFraction(m.elements, m.gspec, 0.5 * m.values + 0.2, sc=m.sc)
    api.calc_intensities(s.problem, other, s.x_rays, s.detector)       # uses the same handle
    g = pb(ib)
    _, rb, nb, ab = oracle.adjoint(desc, rho, noa, acs, ib)
    g_o = (m.grid_pullback(rb) + m.absorption_pullback(s.x_rays, s.detector, s.problem.beam_position.mean, acs, ab)[0]
           + m.noa_pullback(nb.reshape(m.values.shape[:-1] + (m.n_e,))))
    assert _rel(g, g_o) < TOL64
    api.clear_handles()


def test_gpu_material_path_matches_the_oracle(gpu_lib, oracle):
    s = workloads.small_case(dims=2, N=3, shape=(10, 8), n_steps=6)
    mm, P = MaterialModel.per_cell_boxed(s.material, s.x_rays, s.detector, beam_x=s.problem.beam_position.mean[0])
    m = api.GPUMaterial(mm, P)
    desc, keep = s.problem.descriptor(s.x_rays)
    rho, noa, acs = mo.fields(mm, P)
    I, pb = api.calc_intensities_pullback(s.problem, m, s.x_rays, s.detector)
    assert _rel(I, oracle.forward(desc, rho, noa, acs)) < TOL64
    ib = np.linspace(1.0, 2.0, len(I)) / np.abs(I)
    api.calc_intensities(s.problem, api.GPUMaterial(mm, 0.9 * P + 0.05), s.x_rays, s.detector)
    G = pb(ib)
    _, rb, nb, ab = oracle.adjoint(desc, rho, noa, acs, ib)
    assert _rel(G, mo.pullback(mm, P, rb, nb, acs, ab)) < TOL64
    api.clear_handles()
