"""The reference-shaped Python API (pnepma_gb300/api.py) on the CPU: a pullback reads the tape of
its own forward even when other calls used the shared handle in between, and a GPUMaterial reaches
the device library (which reports that there is no device here)."""
import numpy as np
import pytest

from pnepma_gb300 import api, capi, workloads
from pnepma_gb300.material_model import MaterialModel


class FakeHandle:
    """Records which densities the tape was marched with; the adjoint returns them as rho_bar."""

    def __init__(self, n_noa, n_acs, nr):
        self.tape = None
        self.n_noa, self.n_acs, self.nr = n_noa, n_acs, nr
        self.forwards = 0

    def forward(self, rho, noa, acs):
        self.tape = np.array(rho, copy=True)
        self.forwards += 1
        return np.ones(self.nr)

    def adjoint(self, ibar):
        return self.tape.copy(), np.zeros(self.n_noa), np.zeros(self.n_acs)

    def generation_field(self, rho):
        self.tape = None
        return np.zeros(1)


def test_pullback_marches_its_own_forward_again_after_another_call(monkeypatch):
    s = workloads.small_case(dims=1, N=3, shape=(12,), n_steps=4)
    rho, noa, acs = s.inputs()
    fake = FakeHandle(noa.size, acs.size, len(s.x_rays))
    monkeypatch.setattr(api, "get_handle", lambda problem, x_rays: fake)
    seen = []

    class Mat:
        """The host material protocol; each instance has its own densities."""

        def __init__(self, scale):
            self.scale = scale
            self.n_e = s.material.n_e
            self.values = s.material.values

        def rho_flat(self):
            return rho * self.scale

        def number_of_atoms(self):
            return noa

        def absorption(self, *a):
            return acs

        def grid_pullback(self, rho_bar):
            seen.append(float(rho_bar[np.argmax(np.abs(rho))] / rho[np.argmax(np.abs(rho))]))
            return np.zeros(1)

        def absorption_pullback(self, *a):
            return np.zeros(1), np.zeros(1)

        def noa_pullback(self, nb):
            return np.zeros(1)

    A, B = Mat(1.0), Mat(2.0)
    _, pb_a = api.calc_intensities_pullback(s.problem, A, s.x_rays, s.detector)
    _, pb_b = api.calc_intensities_pullback(s.problem, B, s.x_rays, s.detector)
    assert fake.forwards == 2
    pb_b(np.ones(len(s.x_rays)))          # B still owns the tape: no new forward
    assert fake.forwards == 2 and seen[-1] == pytest.approx(2.0)
    pb_a(np.ones(len(s.x_rays)))          # A's tape was overwritten by B: marched again
    assert fake.forwards == 3 and seen[-1] == pytest.approx(1.0)
    pb_a(np.ones(len(s.x_rays)))
    assert fake.forwards == 3
    api.calc_x_ray_generation_field(s.problem, B, s.x_rays)
    pb_a(np.ones(len(s.x_rays)))          # the generation field replaced the densities
    assert fake.forwards == 4 and seen[-1] == pytest.approx(1.0)
    api.calc_intensities(s.problem, B, s.x_rays, s.detector)     # a plain forward of another material
    assert fake.forwards == 5
    pb_a(np.ones(len(s.x_rays)))
    assert fake.forwards == 6 and seen[-1] == pytest.approx(1.0)


def test_gpu_material_reaches_the_device_library():
    torch = pytest.importorskip("torch")
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    s = workloads.small_case(dims=1, N=3, shape=(12,), n_steps=4)
    mm, P = MaterialModel.per_cell_boxed(s.material, s.x_rays, s.detector)
    m = api.GPUMaterial(mm, P)
    with pytest.raises(capi.PnError) as e:
        m.device(s.x_rays, s.detector, 0.0)
    assert e.value.code == -9
    with pytest.raises(ValueError):
        api.GPUMaterial(mm, P[:-1])


class FakeDeviceHandle:
    """pn_forward_device / pn_adjoint_device on host memory, the oracle doing the march."""

    def __init__(self, oracle, desc):
        self.o, self.desc = oracle, desc
        self.sizes = capi.query_sizes(desc)
        self.forwards = 0

    @staticmethod
    def _arr(ptr, n):
        import ctypes
        return np.ctypeslib.as_array((ctypes.c_double * n).from_address(ptr))

    def forward_device(self, rho, noa, acs, out, stream=0):
        z = self.sizes
        self.inputs = (self._arr(rho, z.n_rho).copy(), self._arr(noa, z.n_noa).copy(), self._arr(acs, z.n_acs).copy())
        I = self.o.forward(self.desc, *self.inputs)
        self._arr(out, I.size)[:] = I
        self.forwards += 1

    def generation_field(self, rho):
        return self.o.generation_field(self.desc, rho)

    def adjoint_device(self, ibar, rho_bar, noa_bar, acs_bar, stream=0):
        z = self.sizes
        ib = self._arr(ibar, self.desc.n_xrays).copy()
        _, rb, nb, ab = self.o.adjoint(self.desc, *self.inputs, ib)
        for ptr, v in ((rho_bar, rb), (noa_bar, nb), (acs_bar, ab)):
            self._arr(ptr, v.size)[:] = np.ravel(v)


def test_gpu_material_path_on_host_buffers(oracle, monkeypatch):
    """The GPUMaterial path's buffers, call order and tape ownership, run on host tensors with a
    fake handle and a fake device material (the oracle and the material restatement doing the
    arithmetic): the intensities and the gradient equal the restatements used directly."""
    pytest.importorskip("torch")
    import material_oracle as mo
    from test_reconstruct_cpu import FakeDeviceMaterial
    s = workloads.small_case(dims=1, N=3, shape=(12,), n_steps=4)
    desc, keep = s.problem.descriptor(s.x_rays)
    fake = FakeDeviceHandle(oracle, desc)
    monkeypatch.setattr(api, "_DEVICE", "cpu")
    monkeypatch.setattr(api, "get_handle", lambda problem, x_rays: fake)
    monkeypatch.setattr(api, "DeviceMaterial", FakeDeviceMaterial)
    mm, P = MaterialModel.per_cell_boxed(s.material, s.x_rays, s.detector, beam_x=s.problem.beam_position.mean[0])
    I, pb = api.calc_intensities_pullback(s.problem, api.GPUMaterial(mm, P), s.x_rays, s.detector)
    rho, noa, acs = mo.fields(mm, P)
    assert np.array_equal(I, oracle.forward(desc, rho, noa, acs))
    api.calc_intensities(s.problem, api.GPUMaterial(mm, 0.9 * P + 0.05), s.x_rays, s.detector)
    assert fake.forwards == 2
    ib = np.array([1.0, 0.5]) / np.abs(I)
    G = pb(ib)
    assert fake.forwards == 3                 # the pullback marched its own forward again
    _, rb, nb, ab = oracle.adjoint(desc, rho, noa, acs, ib)
    assert np.array_equal(G, mo.pullback(mm, P, rb, nb, acs, ab))


def test_gpu_material_generation_field_on_host_buffers(oracle, monkeypatch):
    pytest.importorskip("torch")
    import material_oracle as mo
    from test_reconstruct_cpu import FakeDeviceMaterial
    s = workloads.small_case(dims=1, N=3, shape=(12,), n_steps=4)
    desc, keep = s.problem.descriptor(s.x_rays)
    fake = FakeDeviceHandle(oracle, desc)
    monkeypatch.setattr(api, "_DEVICE", "cpu")
    monkeypatch.setattr(api, "get_handle", lambda problem, x_rays: fake)
    monkeypatch.setattr(api, "DeviceMaterial", FakeDeviceMaterial)
    mm, P = MaterialModel.per_cell_boxed(s.material, s.x_rays, s.detector, beam_x=s.problem.beam_position.mean[0])
    f = api.calc_x_ray_generation_field(s.problem, api.GPUMaterial(mm, P), s.x_rays)
    assert np.array_equal(f, oracle.generation_field(desc, mo.fields(mm, P)[0]))
