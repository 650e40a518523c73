"""Reconstruction driver on the GPU batch against the same driver on the oracle (FP64)."""
import numpy as np
import pytest

from pnepma_gb300 import reconstruct

from test_reconstruct_cpu import GSPEC, OracleBackend, truth

pytestmark = pytest.mark.gpu


def rel(a, b):
    a, b = np.asarray(a, float).ravel(), np.asarray(b, float).ravel()
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))


def build(factory):
    reconstruct.clear_standards()
    return reconstruct.Reconstruction(3, GSPEC, ["Cu", "Ni"], (10.0, 13.0, 16.0), n_steps=30,
                                      backend_factory=factory)


def test_batched_driver_matches_the_oracle(gpu_lib, oracle):
    pytest.importorskip("torch")
    ref = build(lambda d, k: OracleBackend(oracle, d, k))
    gpu = build(None)
    try:
        for a, b in zip(gpu.std, ref.std):
            assert rel(a, b) < 1e-10
        k_exp = ref.measure(truth(ref))
        p = np.full(ref.shape, 0.5).ravel()
        assert rel(gpu.measure(p), ref.measure(p)) < 1e-10
        fg, gg = gpu.loss_grad(p, k_exp)
        fr, gr = ref.loss_grad(p, k_exp)
        assert abs(fg - fr) <= 1e-9 * fr
        assert rel(gg, gr) < 1e-9
        kg, Jg = gpu.jacobian(p)
        kr, Jr = ref.jacobian(p)
        assert rel(Jg, Jr) < 1e-9
        res = gpu.fit_gauss_newton(np.full(gpu.shape, 0.5), k_exp, iterations=6)
        assert res.loss <= 1e-3 * fg
    finally:
        gpu.close()

