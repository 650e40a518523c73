"""Device material kernels (pn_material_fields / pn_material_pullback) against the CPU
restatement of the reference's material code, through the C ABI, and chained with the solve."""
import itertools

import numpy as np
import pytest

import material_oracle as mo
from pnepma_gb300 import capi, physics, workloads
from pnepma_gb300.grid import GridSpec
from pnepma_gb300.material_model import MaterialModel, Slices

pytestmark = pytest.mark.gpu

UM = 1e-4
TOL_FIELDS = 1e-12   # same point location and order of operations; exp and the ray sum's order differ
TOL_GRAD = 1e-11     # FP64 atomics add in a run-dependent order
VARIANTS = [("mass_concentration", False), ("volume_fraction", False), ("volume_fraction", True),
            ("linear_density", False), ("linear_density", True), ("mass_fraction", False), ("mass_fraction", True)]


def _rel(a, b):
    a, b = np.asarray(a, float).ravel(), np.asarray(b, float).ravel()
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))


def _model(variant, par, dims=2, n_int=100):
    model, sc = variant
    if dims == 1:
        g = GridSpec.make((16, 1, 1), (-0.5 * UM, 0.0), 0.0, 0.0)
    elif dims == 2:
        g = GridSpec.make((7, 5, 1), (-0.5 * UM, 0.0), (-0.3 * UM, 0.3 * UM), 0.0)
    else:
        g = GridSpec.make((5, 4, 3), (-0.5 * UM, 0.0), (-0.3 * UM, 0.3 * UM), (-0.2 * UM, 0.2 * UM))
    els = ["Cu", "Ni", "Fe"]
    single = Slices.range(-0.5, 0.5, 2)
    if par == "const":
        sl = None
    elif par == "boxed":
        sl = [Slices.vector([-0.55 * UM, -0.3 * UM, -0.1 * UM, 0.05 * UM]),
              Slices.range(-0.35 * UM, 0.35 * UM, 4) if dims > 1 else single,
              Slices.range(-0.25 * UM, 0.25 * UM, 3) if dims == 3 else single]
    else:
        sl = [Slices.range(-0.6 * UM, 0.1 * UM, 5),
              Slices.range(-0.3 * UM, 0.3 * UM, 3) if dims > 1 else Slices.range(0.0, 0.0, 1),
              Slices.range(-0.2 * UM, 0.2 * UM, 2) if dims == 3 else Slices.range(0.0, 0.0, 1)]
    xr = [physics.XRay(e, "K-L3") for e in ("Cu", "Ni")]
    return MaterialModel(g, els, model, sc=sc, parametrization=par, slices=sl, x_rays=xr,
                         detector=(0.3 * UM, 0.05 * UM, 0.0), beam_x=0.0, n_int_points=n_int)


def _dev(torch, a):
    return torch.from_numpy(np.ascontiguousarray(a, dtype=np.float64)).cuda()


def _run(torch, mm, P, rb, nb, ab):
    dm = capi.DeviceMaterial(mm)
    assert dm.n_params == mm.n_params
    rho_o, noa_o, acs_o = mo.fields(mm, P)
    dP = _dev(torch, P)
    d_rho = torch.full((rho_o.size,), float("nan"), dtype=torch.float64, device="cuda")
    d_noa = torch.full((noa_o.size,), float("nan"), dtype=torch.float64, device="cuda")
    d_acs = torch.full((acs_o.size,), float("nan"), dtype=torch.float64, device="cuda")
    dm.fields(dP.data_ptr(), d_rho.data_ptr(), d_noa.data_ptr(), d_acs.data_ptr())
    torch.cuda.synchronize()
    fields = (d_rho.cpu().numpy(), d_noa.cpu().numpy(), d_acs.cpu().numpy())
    G_o = mo.pullback(mm, P, rb, nb, acs_o, ab)
    d_G = torch.full((mm.n_params,), float("nan"), dtype=torch.float64, device="cuda")
    d_rb, d_nb, d_ab = _dev(torch, rb), _dev(torch, nb), _dev(torch, ab)
    dm.pullback(dP.data_ptr(), d_G.data_ptr(), d_rb.data_ptr(), d_nb.data_ptr(), d_acs.data_ptr(), d_ab.data_ptr())
    torch.cuda.synchronize()
    G = d_G.cpu().numpy()
    dm.close()
    return fields, (rho_o, noa_o, acs_o), G, G_o


@pytest.mark.parametrize("variant,par", list(itertools.product(VARIANTS, ["const", "boxed", "bilinear"])),
                         ids=lambda v: v if isinstance(v, str) else f"{v[0]}{'SC' if v[1] else ''}")
def test_fields_and_pullback_match_the_oracle(gpu_lib, variant, par):
    torch = pytest.importorskip("torch")
    mm = _model(variant, par)
    rng = np.random.default_rng(17)
    P = mm.random_params(rng)
    rho_o, noa_o, acs_o = mo.fields(mm, P)
    rb, nb, ab = rng.normal(size=rho_o.shape), rng.normal(size=noa_o.shape), rng.normal(size=acs_o.shape)
    (rho, noa, acs), (rho_o, noa_o, acs_o), G, G_o = _run(torch, mm, P, rb, nb, ab)
    assert _rel(rho, rho_o) < TOL_FIELDS
    assert _rel(noa, noa_o) < TOL_FIELDS
    assert _rel(acs, acs_o) < TOL_FIELDS
    assert _rel(G, G_o) < TOL_GRAD


@pytest.mark.parametrize("dims,par", [(1, "boxed"), (1, "bilinear"), (3, "boxed"), (3, "bilinear")])
def test_1d_and_3d_grids(gpu_lib, dims, par):
    torch = pytest.importorskip("torch")
    mm = _model(("mass_fraction", True), par, dims=dims)
    rng = np.random.default_rng(23)
    P = mm.random_params(rng)
    rho_o, noa_o, acs_o = mo.fields(mm, P)
    rb, nb, ab = rng.normal(size=rho_o.shape), rng.normal(size=noa_o.shape), rng.normal(size=acs_o.shape)
    (rho, noa, acs), (rho_o, noa_o, acs_o), G, G_o = _run(torch, mm, P, rb, nb, ab)
    assert _rel(rho, rho_o) < TOL_FIELDS and _rel(noa, noa_o) < TOL_FIELDS and _rel(acs, acs_o) < TOL_FIELDS
    assert _rel(G, G_o) < TOL_GRAD


def test_partial_cotangents_and_repeat_calls(gpu_lib):
    """NULL cotangents contribute nothing; params_bar is overwritten on every call."""
    torch = pytest.importorskip("torch")
    mm = _model(("linear_density", True), "bilinear")
    rng = np.random.default_rng(29)
    P = mm.random_params(rng)
    rho_o, noa_o, acs_o = mo.fields(mm, P)
    rb = rng.normal(size=rho_o.shape)
    dm = capi.DeviceMaterial(mm)
    dP, d_rb, d_acs = _dev(torch, P), _dev(torch, rb), _dev(torch, acs_o)
    d_G = torch.zeros(mm.n_params, dtype=torch.float64, device="cuda")
    for _ in range(2):
        dm.pullback(dP.data_ptr(), d_G.data_ptr(), rho_bar=d_rb.data_ptr())
        torch.cuda.synchronize()
        assert _rel(d_G.cpu().numpy(), mo.pullback(mm, P, rho_bar=rb)) < TOL_GRAD
    d_noa = torch.zeros(noa_o.size, dtype=torch.float64, device="cuda")
    dm.fields(dP.data_ptr(), noa=d_noa.data_ptr())
    torch.cuda.synchronize()
    assert _rel(d_noa.cpu().numpy(), noa_o) < TOL_FIELDS
    dm.close()


def test_device_material_chained_with_the_solve(gpu_lib):
    """Fields on the device feed pn_forward_device; the adjoint's outputs feed the device
    pullback; the parameter gradient equals the oracle's material pullback of the same adjoint
    outputs, and the intensities equal those from the host-built inputs."""
    torch = pytest.importorskip("torch")
    s = workloads.small_case(dims=2, N=3, shape=(10, 8), n_steps=6)
    mm, P = MaterialModel.per_cell_boxed(s.material, s.x_rays, s.detector,
                                         beam_x=s.problem.beam_position.mean[0])
    desc, keep = s.problem.descriptor(s.x_rays)
    h = capi.Handle(desc, keep)
    sz = h.sizes
    dm = capi.DeviceMaterial(mm)
    dP = _dev(torch, P)
    z = lambda n: torch.zeros(int(n), dtype=torch.float64, device="cuda")
    d_rho, d_noa, d_acs, d_I = z(sz.n_rho), z(sz.n_noa), z(sz.n_acs), z(desc.n_xrays)
    dm.fields(dP.data_ptr(), d_rho.data_ptr(), d_noa.data_ptr(), d_acs.data_ptr())
    h.forward_device(d_rho.data_ptr(), d_noa.data_ptr(), d_acs.data_ptr(), d_I.data_ptr())
    torch.cuda.synchronize()
    I = d_I.cpu().numpy()
    rho_o, noa_o, acs_o = mo.fields(mm, P)
    I_host = h.forward(rho_o, noa_o, acs_o)
    assert _rel(I, I_host) < 1e-12
    ibar = np.linspace(1.0, 2.0, len(I)) / np.abs(I)
    d_ib = _dev(torch, ibar)
    d_rb, d_nb, d_ab = z(sz.n_rho), z(sz.n_noa), z(sz.n_acs)
    h.forward_device(d_rho.data_ptr(), d_noa.data_ptr(), d_acs.data_ptr(), d_I.data_ptr())
    h.adjoint_device(d_ib.data_ptr(), d_rb.data_ptr(), d_nb.data_ptr(), d_ab.data_ptr())
    d_G = z(mm.n_params)
    dm.pullback(dP.data_ptr(), d_G.data_ptr(), d_rb.data_ptr(), d_nb.data_ptr(), d_acs.data_ptr(), d_ab.data_ptr())
    torch.cuda.synchronize()
    G_o = mo.pullback(mm, P, d_rb.cpu().numpy(), d_nb.cpu().numpy(), d_acs.cpu().numpy(), d_ab.cpu().numpy())
    assert _rel(d_G.cpu().numpy(), G_o) < 1e-10
    dm.close()
    h.close()
