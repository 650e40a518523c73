"""The GPU library against the committed golden vectors (tests/golden/oracle_small_cases.npz, made
by the oracle from seeded inputs): the plain FP64 solve and the device material, compared with
fixed vectors rather than a fresh oracle run."""
import os
import sys

import numpy as np
import pytest

from pnepma_gb300 import capi

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
sys.path.insert(0, GOLDEN)
import make_golden as mg  # noqa: E402

pytestmark = pytest.mark.gpu

TOL64 = 1e-10


def _rel(a, b):
    a, b = np.asarray(a, float).ravel(), np.asarray(b, float).ravel()
    return float(np.max(np.abs(a - b)) / np.max(np.abs(b)))


@pytest.mark.parametrize("name", list(mg.SOLVES))
def test_plain_solve_matches_the_golden_vectors(gpu_lib, name):
    G = np.load(mg.PATH)
    s, desc, keep, rho, noa, acs, _ = mg.solve_case(name)
    h = capi.Handle(desc, keep)
    I = h.forward(rho, noa, acs)
    rb, nb, ab = h.adjoint(G[f"{name}/ibar"])
    h.close()
    assert _rel(I, G[f"{name}/I"]) < TOL64
    assert _rel(rb, G[f"{name}/rho_bar"]) < TOL64
    assert _rel(nb, G[f"{name}/noa_bar"]) < TOL64
    assert _rel(ab, G[f"{name}/acs_bar"]) < TOL64


def test_device_material_matches_the_golden_vectors(gpu_lib):
    torch = pytest.importorskip("torch")
    G = np.load(mg.PATH)
    mm, P, rb, nb, ab = mg.material_case()
    dm = capi.DeviceMaterial(mm)
    dev = lambda a: torch.from_numpy(np.ascontiguousarray(a, dtype=np.float64)).cuda()
    z = lambda n: torch.zeros(int(n), dtype=torch.float64, device="cuda")
    dP = dev(P)
    d_rho, d_noa, d_acs = z(G["material/rho"].size), z(G["material/noa"].size), z(G["material/acs"].size)
    d_G = z(dm.n_params)
    d_rb, d_nb, d_ab = dev(rb), dev(nb), dev(ab)
    dm.fields(dP.data_ptr(), d_rho.data_ptr(), d_noa.data_ptr(), d_acs.data_ptr())
    dm.pullback(dP.data_ptr(), d_G.data_ptr(), d_rb.data_ptr(), d_nb.data_ptr(), d_acs.data_ptr(), d_ab.data_ptr())
    torch.cuda.synchronize()
    dm.close()
    assert _rel(d_rho.cpu().numpy(), G["material/rho"]) < 1e-12
    assert _rel(d_noa.cpu().numpy(), G["material/noa"]) < 1e-12
    assert _rel(d_acs.cpu().numpy(), G["material/acs"]) < 1e-12
    assert _rel(d_G.cpu().numpy(), G["material/params_bar"]) < 1e-11
