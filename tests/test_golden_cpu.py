"""The oracle reproduces the committed golden vectors (tests/golden/make_golden.py made them from
seeded inputs): a guard against drift of the CPU restatement between rounds and machines."""
import os
import sys

import numpy as np
import pytest

import material_oracle as mo

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
sys.path.insert(0, GOLDEN)
import make_golden as mg  # noqa: E402

TOL = 1e-12   # libm differences between machines only


def _rel(a, b):
    a, b = np.asarray(a, float).ravel(), np.asarray(b, float).ravel()
    return float(np.max(np.abs(a - b)) / np.max(np.abs(b)))


@pytest.mark.parametrize("name", list(mg.SOLVES))
def test_oracle_reproduces_the_golden_solves(oracle, name):
    G = np.load(mg.PATH)
    s, desc, keep, rho, noa, acs, _ = mg.solve_case(name)
    I, rb, nb, ab = oracle.adjoint(desc, rho, noa, acs, G[f"{name}/ibar"])
    assert _rel(I, G[f"{name}/I"]) < TOL
    assert _rel(rb, G[f"{name}/rho_bar"]) < TOL
    assert _rel(nb, G[f"{name}/noa_bar"]) < TOL
    assert _rel(ab, G[f"{name}/acs_bar"]) < TOL


def test_material_restatement_reproduces_the_golden_vectors():
    G = np.load(mg.PATH)
    mm, P, rb, nb, ab = mg.material_case()
    rho, noa, acs = mo.fields(mm, P)
    assert _rel(rho, G["material/rho"]) < TOL
    assert _rel(noa, G["material/noa"]) < TOL
    assert _rel(acs, G["material/acs"]) < TOL
    assert _rel(mo.pullback(mm, P, rb, nb, acs, ab), G["material/params_bar"]) < TOL
