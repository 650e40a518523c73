"""GPU parity at the full sizes of the benchmark configurations, against oracle results committed
in tests/golden/oracle_config_cases.npz (made by tests/golden/make_config_golden.py; running the
oracle here would take minutes and tens of GB of host memory per solve).

* the 1D slab (200 cells, P7, the full stable march), FP64 plain: every output within 1e-10;
* one solve per beam energy of the 2D workload (256 x 128, P11, 200 / 356 / 663 steps), FP64
  plain: intensities and all three cotangents within 1e-10;
* the same three solves as one FP32 batch (TMA tiles, FP64 accumulators): intensities within
  1e-4 and all three cotangents within 1e-3 of the FP64 oracle.

Errors are normwise (the largest difference over the largest magnitude), per element at the
stored positions whose magnitude is at least 1e-3 of the largest, and of eight +-1 projections of
the whole array over its 1-norm (an error anywhere in the array moves them).
"""
import os
import sys

import numpy as np
import pytest

from pnepma_gb300 import capi
from pnepma_gb300.problem import PN_FP32

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
sys.path.insert(0, GOLDEN)
import make_config_golden as mc  # noqa: E402

pytestmark = pytest.mark.gpu

TOL64 = 1e-10            # FP64 plain vs the oracle, normwise and projections
TOL64_ELEMENT = 1e-8     # FP64 plain, per element at magnitudes >= 1e-3 of the largest
TOL32_K = 1e-4           # FP32 batch: intensities (k-ratios)
TOL32_GRAD = 1e-3        # FP32 batch: cotangents, normwise and projections
TOL32_ELEMENT = 1e-3     # FP32 batch: per element at magnitudes >= 1e-3 of the largest


@pytest.fixture(scope="module")
def golden():
    return mc.load()


def _rel(a, b):
    a, b = np.asarray(a, float).ravel(), np.asarray(b, float).ravel()
    return float(np.max(np.abs(a - b)) / np.max(np.abs(b)))


def _per_element(a, b):
    a, b = np.asarray(a, float).ravel(), np.asarray(b, float).ravel()
    big = np.abs(b) >= 1e-3 * np.max(np.abs(b))
    return float(np.max(np.abs(a[big] - b[big]) / np.abs(b[big])))


def test_config1_slab_fp64_full_march(gpu_lib, golden):
    G = golden["config1"]
    s = mc.config1_case()
    assert s.problem.N_steps == int(G["n_steps"])
    rho, noa, acs = s.inputs()
    desc, keep = s.problem.descriptor(s.x_rays)
    h = capi.Handle(desc, keep)
    I = h.forward(rho, noa, acs)
    rb, nb, ab = h.adjoint(G["ibar"])
    h.close()
    assert _rel(I, G["I"]) < TOL64
    assert _per_element(I, G["I"]) < TOL64
    for name, got in (("rho_bar", rb), ("noa_bar", nb), ("acs_bar", ab)):
        e, pe = _rel(got, G[name]), _per_element(got, G[name])
        print(f"config1 {name}: normwise {e:.2e}, per element {pe:.2e}")
        assert e < TOL64, name
        assert pe < TOL64_ELEMENT, name


@pytest.mark.parametrize("name", [f"config2_{int(E)}kev" for E in mc.CONFIG2_ENERGIES])
def test_config2_solve_fp64_full_march(gpu_lib, golden, name):
    G = golden[name]
    s = mc.config2_cases()[name]
    assert s.problem.N_steps == int(G["n_steps"])
    rho, noa, acs = s.inputs()
    desc, keep = s.problem.descriptor(s.x_rays)
    h = capi.Handle(desc, keep)
    I = h.forward(rho, noa, acs)
    rb, nb, ab = h.adjoint(G["ibar"])
    h.close()
    assert _rel(I, G["I"]) < TOL64
    assert _per_element(I, G["I"]) < TOL64
    for o, got in zip(mc.OUTPUTS, (rb, nb, ab)):
        err = mc.compare(got, G[o])
        print(f"{name} {o}: {err}")
        assert err["normwise"] < TOL64, o
        assert err["projection"] < TOL64, o
        assert err["per_element"] < TOL64_ELEMENT, o


def test_config2_fp32_batch_full_march(gpu_lib, golden):
    """The three energies in one FP32 batch: the 2D TMA tiles with fused sub-steps and FP64
    accumulators over the full marches, against the FP64 oracle."""
    torch = pytest.importorskip("torch")
    cases = mc.config2_cases(precision=PN_FP32)
    names = list(cases)
    solves = [cases[n] for n in names]
    descs, keep = [], []
    for s in solves:
        d, k = s.problem.descriptor(s.x_rays)
        descs.append(d)
        keep.append(k)
    b = capi.Batch(descs, keep)
    assert b.info().tma_groups == 1
    dev = lambda a: torch.from_numpy(np.ascontiguousarray(a, dtype=np.float64)).cuda()
    ins = [[dev(a) for a in s.inputs()] for s in solves]
    I = [torch.zeros(len(s.x_rays), dtype=torch.float64, device="cuda") for s in solves]
    b.forward([x[0].data_ptr() for x in ins], [x[1].data_ptr() for x in ins], [x[2].data_ptr() for x in ins],
              [t.data_ptr() for t in I])
    ib = [dev(golden[n]["ibar"]) for n in names]
    rb = [torch.zeros(x[0].numel(), dtype=torch.float64, device="cuda") for x in ins]
    nb = [torch.zeros(x[1].numel(), dtype=torch.float64, device="cuda") for x in ins]
    ab = [torch.zeros(x[2].numel(), dtype=torch.float64, device="cuda") for x in ins]
    b.adjoint([t.data_ptr() for t in ib], [t.data_ptr() for t in rb], [t.data_ptr() for t in nb],
              [t.data_ptr() for t in ab])
    torch.cuda.synchronize()
    b.close()
    for q, n in enumerate(names):
        G = golden[n]
        k_err = _rel(I[q].cpu().numpy(), G["I"])
        print(f"{n} FP32 intensities: {k_err:.2e}")
        assert k_err < TOL32_K, n
        for o, got in zip(mc.OUTPUTS, (rb[q], nb[q], ab[q])):
            err = mc.compare(got.cpu().numpy(), G[o])
            print(f"{n} FP32 {o}: {err}")
            assert err["normwise"] < TOL32_GRAD, (n, o)
            assert err["projection"] < TOL32_GRAD, (n, o)
            assert err["per_element"] < TOL32_ELEMENT, (n, o)
