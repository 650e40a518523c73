"""Reconstruction driver (k-ratio standards cache, loss, gradient, Jacobian, fits) on the CPU,
with the oracle as the solver backend (the driver's GPU backend is the batched library,
tests/test_gpu_reconstruct.py)."""
import numpy as np
import pytest

import material_oracle as mo
from pnepma_gb300 import reconstruct
from pnepma_gb300.grid import GridSpec
from pnepma_gb300.material_model import MaterialModel, Slices
from pnepma_gb300.workloads import UM

GSPEC = GridSpec.make((6, 1, 1), (-0.4 * UM, 0.0), 0.0, 0.0)


class OracleBackend:
    """The oracle behind the driver's backend interface (test infrastructure only)."""
    calls = 0

    def __init__(self, oracle, descs, keep):
        self.o, self.descs, self.keep = oracle, descs, keep

    def forward(self, inputs):
        OracleBackend.calls += 1
        self.inputs = inputs
        return [self.o.forward(d, *x) for d, x in zip(self.descs, inputs)]

    def adjoint(self, ibars):
        out = [self.o.adjoint(d, *x, ib) for d, x, ib in zip(self.descs, self.inputs, ibars)]
        return [o[1] for o in out], [o[2] for o in out], [o[3] for o in out]

    def close(self):
        pass


def make(oracle, **kw):
    return reconstruct.Reconstruction(3, GSPEC, ["Cu", "Ni"], (10.0, 13.0, 16.0), n_steps=30,
                                      backend_factory=lambda d, k: OracleBackend(oracle, d, k), **kw)


def truth(rec):
    p = np.empty(rec.shape)
    p[..., 0] = np.where(np.arange(6) < 3, 0.8, 0.25)
    return p


def test_standards_are_pure_element_intensities_computed_once(oracle):
    reconstruct.clear_standards()
    OracleBackend.calls = 0
    rec = make(oracle)
    assert OracleBackend.calls == 1          # one batch for every problem's standards
    for s, sd in zip(rec.solves, rec.std):
        for r, x in enumerate(s.x_rays):
            e = [el.symbol for el in s.problem.elements].index(x.element)
            m = reconstruct.pure_material(GSPEC, s.problem.elements, e, True)
            d, k = s.problem.descriptor(s.x_rays)
            I = oracle.forward(d, *reconstruct.Solve(s.problem, m, s.x_rays, s.detector).inputs())
            assert sd[r] == I[r]
    OracleBackend.calls = 0
    make(oracle)
    assert OracleBackend.calls == 0          # cached


def test_k_ratios_of_a_standard_are_one(oracle):
    rec = make(oracle)
    k = rec.measure(np.ones(rec.shape))      # pure Cu: its own standard
    assert np.allclose(k[0::2], 1.0, rtol=1e-13)
    assert np.all(np.abs(k[1::2]) < 1e-12)   # no Ni


def test_gradient_equals_jacobian_transpose_residual(oracle):
    rec = make(oracle)
    k_exp = rec.measure(truth(rec))
    p = np.full(rec.shape, 0.5).ravel()
    f, g = rec.loss_grad(p, k_exp)
    k, J = rec.jacobian(p)
    r = k - k_exp
    assert abs(f - r @ r) <= 1e-12 * f
    assert np.max(np.abs(g - 2.0 * J.T @ r)) <= 1e-10 * np.max(np.abs(g))


def test_gradient_against_finite_differences(oracle):
    """The reference's adjoint is continuous-style (not the transpose of the discrete march), so
    adjoint and finite-difference gradients agree at discretisation level."""
    rec = make(oracle)
    k_exp = rec.measure(truth(rec))
    p = np.full(rec.shape, 0.5).ravel()
    _f, g = rec.loss_grad(p, k_exp)
    h = 1e-6
    fd = np.empty_like(g)
    for i in range(p.size):
        e = np.zeros_like(p)
        e[i] = h
        fd[i] = (rec.loss_grad(p + e, k_exp)[0] - rec.loss_grad(p - e, k_exp)[0]) / (2 * h)
    assert np.linalg.norm(g - fd) <= 2e-2 * np.linalg.norm(fd)


@pytest.mark.parametrize("method", ["lbfgs", "gauss_newton"])
def test_fits_lower_the_loss(oracle, method):
    rec = make(oracle)
    k_exp = rec.measure(truth(rec))
    p0 = np.full(rec.shape, 0.5)
    f0 = rec.loss_grad(p0.ravel(), k_exp)[0]
    if method == "lbfgs":
        res = rec.fit_lbfgs(p0, k_exp, maxiter=40)
    else:
        res = rec.fit_gauss_newton(p0, k_exp, iterations=8)
    assert res.loss <= 1e-3 * f0
    assert np.all(res.params >= 0.0) and np.all(res.params <= 1.0)


# ------------------------------------------------------- a MaterialModel (the reference's fits)
class OracleMaterialSet:
    """The material restatement behind the driver's material-set interface (test infrastructure)."""

    def __init__(self, model, solves):
        self.mms = [model.with_geometry(s.x_rays, s.detector, s.problem.beam_position.mean[0]) for s in solves]

    def fields(self, P):
        return [mo.fields(mm, P) for mm in self.mms]

    def pullback(self, i, P, rho_bar, noa_bar, acs, acs_bar):
        return mo.pullback(self.mms[i], P, rho_bar, noa_bar, acs, acs_bar)

    def close(self):
        pass


def bilinear_model(par="bilinear"):
    """VolumeFractionSC over five knots (Bilinear) or five boxes (Boxed) down to -300 nm, the
    embedding (pure Cu) below: reconstructions_1d.jl:115-130 on the test grid."""
    if par == "bilinear":
        sl = [Slices.range(-0.3 * UM, 0.0, 5), Slices.range(0.0, 0.0, 1), Slices.range(0.0, 0.0, 1)]
    else:
        sl = [Slices.range(-0.3 * UM, 0.0, 6), Slices.range(-0.5, 0.5, 2), Slices.range(-0.5, 0.5, 2)]
    return MaterialModel(GSPEC, ["Cu", "Ni"], "volume_fraction", sc=True, parametrization=par, slices=sl)


def make_model(oracle, par="bilinear", **kw):
    return reconstruct.Reconstruction(3, GSPEC, ["Cu", "Ni"], (10.0, 13.0, 16.0), n_steps=30,
                                      backend_factory=lambda d, k: OracleBackend(oracle, d, k),
                                      model=bilinear_model(par), embedding=[1.0],
                                      material_set_factory=OracleMaterialSet, **kw)


def test_model_parameters_exclude_a_fixed_embedding(oracle):
    rec = make_model(oracle)
    assert rec.shape == (5,)
    assert np.array_equal(rec.material(np.zeros(5)), np.r_[np.zeros(5), 1.0])


def test_model_k_ratios_of_a_standard_are_one(oracle):
    rec = make_model(oracle)
    k = rec.measure(np.ones(rec.shape))      # Cu everywhere (the embedding is Cu too)
    assert np.allclose(k[0::2], 1.0, rtol=1e-12)
    assert np.all(np.abs(k[1::2]) < 1e-12)


@pytest.mark.parametrize("par", ["bilinear", "boxed"])
def test_model_gradient_is_consistent_and_matches_finite_differences(oracle, par):
    rec = make_model(oracle, par)
    truth_p = np.linspace(0.9, 0.2, rec.shape[0])
    k_exp = rec.measure(truth_p)
    p = np.full(rec.shape, 0.5)
    f, g = rec.loss_grad(p, k_exp)
    k, J = rec.jacobian(p)
    r = k - k_exp
    assert abs(f - r @ r) <= 1e-12 * f
    assert np.max(np.abs(g - 2.0 * J.T @ r)) <= 1e-10 * np.max(np.abs(g))
    h = 1e-6
    fd = np.array([(rec.loss_grad(p + h * e, k_exp)[0] - rec.loss_grad(p - h * e, k_exp)[0]) / (2 * h)
                   for e in np.eye(p.size)])
    assert np.linalg.norm(g - fd) <= 2e-2 * np.linalg.norm(fd)


def test_model_fit_recovers_the_profile(oracle):
    rec = make_model(oracle)
    truth_p = np.array([0.9, 0.8, 0.4, 0.3, 0.2])
    k_exp = rec.measure(truth_p)
    p0 = np.full(rec.shape, 0.5)
    f0 = rec.loss_grad(p0, k_exp)[0]
    res = rec.fit_gauss_newton(p0, k_exp, iterations=8)
    assert res.loss <= 1e-3 * f0
    assert np.all(res.params >= 0.0) and np.all(res.params <= 1.0)


class FakeDeviceMaterial:
    """Stands in for capi.DeviceMaterial on host memory: reads and writes the buffers behind the
    pointers it is given, with the material restatement doing the arithmetic."""

    def __init__(self, mm):
        self.mm, self.n_params = mm, mm.n_params
        g = mm.gspec
        self.n = dict(rho=sum(g.n_cells(c) for c in range(8)) * mm.n_e,
                      noa=int(np.prod([a.M for a in g.axes])) * mm.n_e,
                      acs=int(np.prod([a.M for a in g.axes])) * len(mm.x_rays))

    @staticmethod
    def _arr(ptr, n):
        import ctypes
        return np.ctypeslib.as_array((ctypes.c_double * n).from_address(ptr))

    def fields(self, params, rho=None, noa=None, acs=None, stream=0):
        P = self._arr(params, self.n_params).copy()
        r, n, a = mo.fields(self.mm, P)
        for ptr, v in ((rho, r), (noa, n), (acs, a)):
            if ptr:
                self._arr(ptr, v.size)[:] = v.ravel()

    def pullback(self, params, params_bar, rho_bar=None, noa_bar=None, acs=None, acs_bar=None, stream=0):
        P = self._arr(params, self.n_params).copy()
        G = mo.pullback(self.mm, P, self._arr(rho_bar, self.n["rho"]).copy(), self._arr(noa_bar, self.n["noa"]).copy(),
                        self._arr(acs, self.n["acs"]).copy(), self._arr(acs_bar, self.n["acs"]).copy())
        self._arr(params_bar, self.n_params)[:] = G

    def close(self):
        pass


def test_device_material_set_passes_buffers_in_order(oracle, monkeypatch):
    """DeviceMaterialSet's buffers, sizes, argument order and reshapes, on host tensors with a fake
    device material: the same fields and gradients as the restatement used directly."""
    pytest.importorskip("torch")
    from pnepma_gb300 import capi
    monkeypatch.setattr(capi, "DeviceMaterial", FakeDeviceMaterial)
    rec = make_model(oracle)
    dset = reconstruct.DeviceMaterialSet(bilinear_model(), rec.solves, device="cpu")
    ref = OracleMaterialSet(bilinear_model(), rec.solves)
    P = rec.material(np.linspace(0.2, 0.8, 5))
    got, want = dset.fields(P), ref.fields(P)
    rng = np.random.default_rng(2)
    for i, (g, w) in enumerate(zip(got, want)):
        for a, b in zip(g, w):
            assert a.shape == np.asarray(b).reshape(a.shape).shape
            assert np.array_equal(a.ravel(), np.asarray(b).ravel())
        rb, nb, ab = (rng.normal(size=np.asarray(x).shape) for x in w)
        assert np.array_equal(dset.pullback(i, P, rb, nb, g[2], ab), ref.pullback(i, P, rb, nb, w[2], ab))
    dset.close()
