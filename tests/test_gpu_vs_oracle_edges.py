"""The FP64 plain solve against the oracle at the edges of its domain: one element, four elements
(the most a solve may have), order 9, and 3D at order 5 (1e-10 relative, as the other parity
tests)."""
import numpy as np
import pytest

from pnepma_gb300 import capi, workloads

pytestmark = pytest.mark.gpu

TOL64 = 1e-10
EDGES = [dict(dims=1, N=3, shape=(10,), n_steps=4, elements=("Cu",)),
         dict(dims=2, N=5, shape=(8, 7), n_steps=4, elements=("Fe", "Cr", "Ni", "Cu")),
         dict(dims=1, N=9, shape=(14,), n_steps=5),
         dict(dims=3, N=5, shape=(5, 4, 4), n_steps=3)]


def rel(a, b):
    a, b = np.asarray(a, float).ravel(), np.asarray(b, float).ravel()
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))


@pytest.mark.parametrize("case", EDGES, ids=["1d-1el", "2d-4el", "1d-N9", "3d-N5"])
def test_plain_solve_at_the_edges_matches_the_oracle(gpu_lib, oracle, case):
    s = workloads.small_case(**case)
    rho, noa, acs = s.inputs()
    desc, keep = s.problem.descriptor(s.x_rays)
    h = capi.Handle(desc, keep)
    I = h.forward(rho, noa, acs)
    ibar = np.linspace(1.0, 2.0, len(I)) / np.abs(I)
    rb, nb, ab = h.adjoint(ibar)
    h.close()
    I_o, rb_o, nb_o, ab_o = oracle.adjoint(desc, rho, noa, acs, ibar)
    assert rel(I, I_o) < TOL64
    assert rel(rb, rb_o) < TOL64
    assert rel(nb, nb_o) < TOL64
    assert rel(ab, ab_o) < TOL64
