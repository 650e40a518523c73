"""The reconstruction driver fitting a MaterialModel on the GPU (the batch and the device
material set) against the same driver on the oracle and the material restatement (FP64)."""
import numpy as np
import pytest

from pnepma_gb300 import reconstruct

from test_reconstruct_cpu import GSPEC, OracleBackend, OracleMaterialSet, bilinear_model

pytestmark = pytest.mark.gpu


def rel(a, b):
    a, b = np.asarray(a, float).ravel(), np.asarray(b, float).ravel()
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))


def test_batched_driver_with_a_device_material_matches_the_oracle(gpu_lib, oracle):
    """The reference's kind of fit (VolumeFractionSC over a Bilinear field, fixed embedding): the
    batch and the device material set against the oracle and the material restatement."""
    pytest.importorskip("torch")
    reconstruct.clear_standards()
    kw = dict(n_steps=30, model=bilinear_model(), embedding=[1.0])
    ref = reconstruct.Reconstruction(3, GSPEC, ["Cu", "Ni"], (10.0, 13.0, 16.0),
                                     backend_factory=lambda d, k: OracleBackend(oracle, d, k),
                                     material_set_factory=OracleMaterialSet, **kw)
    gpu = reconstruct.Reconstruction(3, GSPEC, ["Cu", "Ni"], (10.0, 13.0, 16.0), **kw)
    try:
        truth_p = np.array([0.9, 0.8, 0.4, 0.3, 0.2])
        k_exp = ref.measure(truth_p)
        p = np.full(ref.shape, 0.5)
        assert rel(gpu.measure(p), ref.measure(p)) < 1e-10
        fg, gg = gpu.loss_grad(p, k_exp)
        fr, gr = ref.loss_grad(p, k_exp)
        assert abs(fg - fr) <= 1e-9 * fr
        assert rel(gg, gr) < 1e-9
        kg, Jg = gpu.jacobian(p)
        kr, Jr = ref.jacobian(p)
        assert rel(Jg, Jr) < 1e-9
    finally:
        gpu.close()
