"""The material restatement (oracle/material_oracle.py) on the CPU: point location rules of the
reference, pullbacks against central finite differences for every model and parametrisation, and
agreement with the boxed mass-fraction host path the solves already use."""
import itertools

import numpy as np
import pytest

import material_oracle as mo
from pnepma_gb300 import physics, workloads
from pnepma_gb300.grid import GridSpec
from pnepma_gb300.material import BoxedMassFraction
from pnepma_gb300.material_model import MaterialModel, Slices

UM = 1e-4

VARIANTS = [("mass_concentration", False), ("volume_fraction", False), ("volume_fraction", True),
            ("linear_density", False), ("linear_density", True), ("mass_fraction", False), ("mass_fraction", True)]


def test_range_location_is_floor_of_the_quotient():
    s = Slices.range(0.0, 4.0, 5)              # 0, 1, 2, 3, 4
    assert mo.locate(s, 2.5) == (3, 0.5)
    assert mo.locate(s, 2.0) == (3, 0.0)       # on a slice: the box above it
    assert mo.locate(s, -0.5) == (0, 0.5)
    assert mo.locate(Slices.range(7.0, 7.0, 1), 7.0) == (1, 0.0)


def test_vector_location_follows_the_linear_search():
    s = Slices.vector([0.0, 1.0, 3.0, 4.0])
    assert mo.locate(s, 0.5) == (1, 0.5)
    assert mo.locate(s, 1.0) == (1, 1.0)       # on an interior slice: the box below it
    assert mo.locate(s, 0.0) == (1, 0.0)
    assert mo.locate(s, 2.0) == (2, 0.5)
    assert mo.locate(s, 4.0) == (3, 1.0)
    assert mo.locate(s, -1.0) == (0, -1.0)     # outside: index 0 (the embedding for Boxed)
    assert mo.locate(s, 5.0) == (4, 2.0)


def test_boxed_last_slice_belongs_to_the_last_box():
    g = GridSpec.make((4, 1, 1), (0.0, 3.0), 0.0, 0.0)
    mm = MaterialModel(g, ["Cu", "Ni"], "mass_concentration", parametrization="boxed",
                       slices=[Slices.range(0.0, 3.0, 4), Slices.range(-0.5, 0.5, 2), Slices.range(-0.5, 0.5, 2)])
    assert mo.param_terms(mm, (3.0, 0.0, 0.0)) == [(2, 1.0)]
    assert mo.param_terms(mm, (3.5, 0.0, 0.0)) == [(3, 1.0)]      # embedding


def _model(variant, par, dims=2, n_int=12):
    model, sc = variant
    if dims == 2:
        g = GridSpec.make((5, 4, 1), (-0.5 * UM, 0.0), (-0.3 * UM, 0.3 * UM), 0.0)
    else:
        g = GridSpec.make((4, 3, 3), (-0.5 * UM, 0.0), (-0.3 * UM, 0.3 * UM), (-0.2 * UM, 0.2 * UM))
    els = ["Cu", "Ni", "Fe"]
    if par == "const":
        sl = None
    elif par == "boxed":
        sl = [Slices.vector([-0.55 * UM, -0.3 * UM, -0.1 * UM, 0.05 * UM]), Slices.range(-0.35 * UM, 0.35 * UM, 3),
              Slices.range(-0.5, 0.5, 2) if dims == 2 else Slices.range(-0.25 * UM, 0.25 * UM, 3)]
    else:
        sl = [Slices.range(-0.6 * UM, 0.1 * UM, 4), Slices.range(-0.3 * UM, 0.3 * UM, 3),
              Slices.range(0.0, 0.0, 1) if dims == 2 else Slices.range(-0.2 * UM, 0.2 * UM, 2)]
    xr = [physics.XRay(e, "K-L3") for e in ("Cu", "Ni")]
    return MaterialModel(g, els, model, sc=sc, parametrization=par, slices=sl, x_rays=xr,
                         detector=(0.3 * UM, 0.05 * UM, 0.0), beam_x=0.0, n_int_points=n_int)


@pytest.mark.parametrize("variant,par", list(itertools.product(VARIANTS, ["const", "boxed", "bilinear"])),
                         ids=lambda v: v if isinstance(v, str) else f"{v[0]}{'SC' if v[1] else ''}")
def test_pullback_matches_finite_differences(variant, par):
    mm = _model(variant, par)
    rng = np.random.default_rng(3)
    P = mm.random_params(rng)
    rho, noa, acs = mo.fields(mm, P)
    rb, nb, ab = rng.normal(size=rho.shape), rng.normal(size=noa.shape), rng.normal(size=acs.shape)

    def f(Q):
        r, n, a = mo.fields(mm, Q)
        return float(np.sum(r * rb) + np.sum(n * nb) + np.sum(a * ab))

    G = mo.pullback(mm, P, rb, nb, acs, ab)
    idx = rng.choice(mm.n_params, size=min(6, mm.n_params), replace=False)
    idx = np.unique(np.concatenate([idx, [mm.n_params - 1]]))      # include the embedding
    h = 1e-6
    for i in idx:
        Qp, Qm = P.copy(), P.copy()
        Qp[i] += h
        Qm[i] -= h
        fd = (f(Qp) - f(Qm)) / (2 * h)
        scale = max(1.0, np.max(np.abs(G)))
        assert abs(G[i] - fd) <= 1e-6 * scale, (i, G[i], fd)


def test_3d_bilinear_and_boxed_pullbacks_match_finite_differences():
    for par in ("bilinear", "boxed"):
        mm = _model(("mass_fraction", True), par, dims=3, n_int=8)
        rng = np.random.default_rng(5)
        P = mm.random_params(rng)
        rho, noa, acs = mo.fields(mm, P)
        rb, nb, ab = rng.normal(size=rho.shape), rng.normal(size=noa.shape), rng.normal(size=acs.shape)
        G = mo.pullback(mm, P, rb, nb, acs, ab)
        for i in rng.choice(mm.n_params, size=4, replace=False):
            Qp, Qm = P.copy(), P.copy()
            Qp[i] += 1e-6
            Qm[i] -= 1e-6
            fp = [np.sum(a * b) for a, b in zip(mo.fields(mm, Qp), (rb, nb, ab))]
            fm = [np.sum(a * b) for a, b in zip(mo.fields(mm, Qm), (rb, nb, ab))]
            fd = (sum(fp) - sum(fm)) / 2e-6
            assert abs(G[i] - fd) <= 1e-6 * max(1.0, np.max(np.abs(G)))


def test_per_cell_boxed_model_reproduces_the_host_material_path():
    """On a grid whose coordinates are binary fractions (so the floor rule and the integer rule of
    BoxedMassFraction coincide), the restatement gives the host path's densities on all eight
    grids, number of atoms, absorption factors and pullbacks."""
    g = GridSpec.make((9, 5, 1), (-2.0 ** -13, 0.0), (-2.0 ** -14, 2.0 ** -14), 0.0)
    rng = np.random.default_rng(11)
    els = ["Cu", "Ni"]
    vals = rng.uniform(0.2, 0.8, size=(1, 5, 9, 1))
    mat = BoxedMassFraction(els, g, vals, sc=True)
    xr = [physics.XRay(e, "K-L3") for e in els]
    det = (2.0 ** -13, 2.0 ** -15, 0.0)
    mm, P = MaterialModel.per_cell_boxed(mat, xr, det, beam_x=0.0)
    rho, noa, acs = mo.fields(mm, P)
    np.testing.assert_allclose(rho, mat.rho_flat(), rtol=1e-14, atol=0)
    np.testing.assert_allclose(noa.ravel(), mat.number_of_atoms().ravel(), rtol=1e-14, atol=0)
    acs_h = mat.absorption(xr, det, (0.0, 0.0, 0.0))
    np.testing.assert_allclose(acs.ravel(), acs_h.ravel(), rtol=1e-12, atol=0)
    rb, nb, ab = rng.normal(size=rho.shape), rng.normal(size=noa.shape), rng.normal(size=acs.shape)
    G = mo.pullback(mm, P, rb, nb, acs, ab)
    gh = mat.grid_pullback(rb) + mat.noa_pullback(nb.reshape(mat.number_of_atoms().shape))
    ga, emb = mat.absorption_pullback(xr, det, (0.0, 0.0, 0.0), acs_h, ab)
    gh = gh + ga
    np.testing.assert_allclose(G[:-1], gh.ravel(), rtol=1e-11, atol=1e-11 * np.max(np.abs(gh)))
    np.testing.assert_allclose(G[-1:], emb, rtol=1e-11, atol=1e-11 * np.max(np.abs(gh)))


def test_small_case_material_fields_match_the_solver_inputs():
    """The per-cell model of a solve reproduces the solve's own inputs at the eee points and
    the absorption factors (generic points, no slice ambiguity)."""
    s = workloads.small_case(dims=2, N=3, shape=(10, 8), n_steps=4)
    rho_in, noa_in, acs_in = s.inputs()
    mm, P = MaterialModel.per_cell_boxed(s.material, s.x_rays, s.detector,
                                         beam_x=s.problem.beam_position.mean[0])
    rho, noa, acs = mo.fields(mm, P)
    np.testing.assert_allclose(noa.ravel(), np.asarray(noa_in).ravel(), rtol=1e-14)
    np.testing.assert_allclose(acs.ravel(), np.asarray(acs_in).ravel(), rtol=1e-12)
    n_eee = noa.shape[0] * len(s.material.elements)
    np.testing.assert_allclose(rho[:n_eee], np.asarray(rho_in)[:n_eee], rtol=1e-14)


def test_invalid_material_descriptors_are_errors_not_crashes():
    """Validation happens before any device work, so it runs without a GPU."""
    import ctypes
    from pnepma_gb300 import capi
    L = capi.lib()
    mm = _model(("volume_fraction", True), "boxed")
    for field, value in (("model", 9), ("parametrization", 7), ("n_elements", 0), ("n_xrays", 99)):
        d, keep = mm.descriptor()
        setattr(d, field, value)
        out = ctypes.c_void_p()
        rc = L.pn_material_create(ctypes.byref(d), ctypes.byref(out), None)
        assert rc in (-1, -2), (field, rc)
        assert not out.value
        assert L.pn_last_error(None).decode()
    d, keep = mm.descriptor()
    bad = np.array([0.0, 1.0, 1.0, 2.0])          # not strictly increasing
    d.slices[0].values = bad.ctypes.data
    d.slices[0].n = 4
    out = ctypes.c_void_p()
    assert L.pn_material_create(ctypes.byref(d), ctypes.byref(out), None) == -1
    assert "increasing" in L.pn_last_error(None).decode()


@pytest.mark.parametrize("case", [dict(dims=1, shape=(9,)), dict(dims=2, shape=(7, 5)), dict(dims=3, shape=(5, 4, 3))],
                         ids=["1d", "2d", "3d"])
def test_material_fields_have_the_solver_input_sizes(case):
    """The material's points (all eight class grids, ghosts included) and the solver's buffers
    (pn_query_sizes) agree for every dimension, so device fields feed pn_forward_device as they are."""
    from pnepma_gb300 import capi
    s = workloads.small_case(N=3, n_steps=3, **case)
    desc, keep = s.problem.descriptor(s.x_rays)
    sz = capi.query_sizes(desc)
    mm, P = MaterialModel.per_cell_boxed(s.material, s.x_rays, s.detector, n_int_points=4)
    rho, noa, acs = mo.fields(mm, P)
    assert (rho.size, noa.size, acs.size) == (sz.n_rho, sz.n_noa, sz.n_acs)
    assert mm.coords().size == sum(a.M + (1 if a.M == 1 else a.M + 1) for a in mm.gspec.axes)


def _device_vector_locate(values, x):
    """The vector-slice location of pn_material.cu (locate_axis), step for step: a binary search
    for the first k in [1, n-1] with x <= v[k], then the reference's partition and corrections."""
    n = len(values)
    if n == 1:
        return 1, 0.0
    lo, hi = 1, n - 1
    while lo < hi:
        mid = (lo + hi) >> 1
        if x <= values[mid]:
            hi = mid
        else:
            lo = mid + 1
    i = lo
    d = (x - values[i - 1]) / (values[i] - values[i - 1])
    if d < 0.0:
        i -= 1
    elif d > 1.0:
        i += 1
    return i, d


def test_binary_search_returns_the_linear_search_index():
    """The device's binary search and the reference's linear search agree on every point: random
    points, points exactly on slices, and points outside on either side."""
    rng = np.random.default_rng(8)
    for n in (2, 3, 5, 17):
        for _ in range(20):
            v = np.sort(rng.uniform(-1.0, 1.0, n))
            if np.any(np.diff(v) <= 0):
                continue
            sl = Slices.vector(v)
            xs = np.concatenate([rng.uniform(-1.5, 1.5, 30), v, [v[0] - 1.0, v[-1] + 1.0]])
            for x in xs:
                assert _device_vector_locate(v, float(x)) == mo.locate(sl, float(x)), (v, x)
