"""Reference-shaped entry points over the GPU library.

These keep the names and argument meaning of the reference's Julia API for this path:

* ``calc_intensities(problem, m, x_rays, detector_position)`` -- pn_intensities.jl:325-351
* ``calc_intensities_pullback(problem, m, x_rays, detector_position)`` -- the Zygote adjoint of
  the same function (pn_intensities.jl:353-413): returns the intensities and a pullback that maps
  a cotangent of the intensities to the gradient with respect to the material parameters
* ``calc_x_ray_generation_field(problem, m, x_rays)`` -- pn_intensities.jl:189-212
* ``step_pn(problem, rho, u, i)`` -- one forward energy step of a state (pn_intensities.jl:16-22)

Two kinds of material ``m`` are accepted:

* the per-cell boxed mass-fraction material (:mod:`material`): the densities on the eight grids,
  the number of atoms and the absorption factors are formed on the host, the march and its adjoint
  run on the GPU, and the parameter pullbacks are applied on the host, as the reference's shim
  would do (pn_intensities.jl:406-409);
* a :class:`GPUMaterial` (any model and Const / Boxed / Bilinear parametrisation of
  ``pn_material.jl``): fields, march, adjoint and material pullbacks all run on the device, and
  only the intensities and the parameter gradient (the reference's ``param_vec`` order, embedding
  last) come back to the host; the generation field takes its densities from the device too.
"""
from __future__ import annotations

import numpy as np

from .capi import DeviceMaterial, Handle
from .material_model import MaterialModel
from .problem import ForwardPNProblem

_CACHE: dict = {}
_CACHE_MAX = 8
_DEVICE = "cuda"          # where the GPUMaterial path keeps its buffers


def get_handle(problem: ForwardPNProblem, x_rays) -> Handle:
    """A device handle for (problem, lines), cached (handles keep their tape between calls)."""
    key = (id(problem), tuple(x_rays))
    h = _CACHE.get(key)
    if h is None or h[0] is not problem:
        desc, keep = problem.descriptor(list(x_rays))
        h = (problem, Handle(desc, keep))
        _CACHE[key] = h
        while len(_CACHE) > _CACHE_MAX:
            k0 = next(iter(_CACHE))
            _CACHE.pop(k0)[1].close()
    return h[1]


def clear_handles():
    for _p, h in _CACHE.values():
        h.close()
    _CACHE.clear()


class GPUMaterial:
    """A material whose fields and pullbacks run on the device: a ``MaterialModel`` (its model,
    parametrisation, slices and elements) and its parameter vector.  The measurement geometry of
    each call (lines, detector, beam position) selects a device material, built once and cached."""

    def __init__(self, model: MaterialModel, params):
        self.model = model
        self.params = np.ascontiguousarray(params, dtype=np.float64)
        if self.params.size != model.n_params:
            raise ValueError(f"params has {self.params.size} values, the material needs {model.n_params}")
        self._dev = {}

    def device(self, x_rays, detector_position, beam_x: float) -> DeviceMaterial:
        key = (tuple(x_rays), tuple(float(v) for v in detector_position), float(beam_x))
        dm = self._dev.get(key)
        if dm is None:
            t = self.model
            mm = MaterialModel(t.gspec, t.elements, t.model, sc=t.sc, parametrization=t.parametrization,
                               slices=t.slices, x_rays=list(x_rays), detector=detector_position, beam_x=beam_x,
                               n_int_points=t.n_int_points)
            dm = self._dev[key] = DeviceMaterial(mm)
        return dm


def _mark(h):
    """Record that the handle's tape now belongs to a new forward; returns its token."""
    token = object()
    h._api_forward = token
    return token


def _owns_tape(h, token) -> bool:
    return getattr(h, "_api_forward", None) is token


def _sync(torch):
    if _DEVICE != "cpu":
        torch.cuda.synchronize()


def _device_forward(problem, m: GPUMaterial, x_rays, detector_position):
    """Device fields -> pn_forward_device; every call on the legacy default stream, in order."""
    import torch
    h = get_handle(problem, x_rays)
    dm = m.device(x_rays, detector_position, problem.beam_position.mean[0])
    sz = h.sizes
    f64 = dict(dtype=torch.float64, device=_DEVICE)
    d = {"P": torch.from_numpy(m.params).to(_DEVICE), "rho": torch.empty(sz.n_rho, **f64),
         "noa": torch.empty(sz.n_noa, **f64), "acs": torch.empty(max(sz.n_acs, 1), **f64),
         "I": torch.empty(max(len(x_rays), 1), **f64)}
    dm.fields(d["P"].data_ptr(), d["rho"].data_ptr(), d["noa"].data_ptr(), d["acs"].data_ptr())
    h.forward_device(d["rho"].data_ptr(), d["noa"].data_ptr(), d["acs"].data_ptr(), d["I"].data_ptr())
    d["token"] = _mark(h)
    _sync(torch)
    I = d["I"].cpu().numpy()[:len(x_rays)].copy()
    return h, dm, d, I


def _inputs(problem, m, x_rays, detector_position):
    rho = m.rho_flat()
    noa = m.number_of_atoms().reshape(-1, m.n_e)
    acs = m.absorption(x_rays, detector_position, problem.beam_position.mean).reshape(-1, len(x_rays))
    return rho, noa, acs


def calc_intensities(problem: ForwardPNProblem, m, x_rays, detector_position) -> np.ndarray:
    if isinstance(m, GPUMaterial):
        return _device_forward(problem, m, x_rays, detector_position)[3]
    h = get_handle(problem, x_rays)
    rho, noa, acs = _inputs(problem, m, x_rays, detector_position)
    I = h.forward(rho, noa, acs)
    _mark(h)                 # this forward replaced the tape of any pending pullback
    return I


def calc_intensities_pullback(problem: ForwardPNProblem, m, x_rays, detector_position):
    """(intensities, pullback); pullback(I_bar) -> d(material parameters): the shape of
    ``m.values`` for the host material, the parameter vector's length for a GPUMaterial."""
    if isinstance(m, GPUMaterial):
        return _device_pullback(problem, m, x_rays, detector_position)
    h = get_handle(problem, x_rays)
    rho, noa, acs = _inputs(problem, m, x_rays, detector_position)
    I = h.forward(rho, noa, acs)
    token = [_mark(h)]

    def pullback(I_bar):
        # the handle is shared by every call on (problem, lines): if another forward ran on it
        # since, march this call's forward again so the adjoint reads this call's tape
        if not _owns_tape(h, token[0]):
            h.forward(rho, noa, acs)
            token[0] = _mark(h)
        rho_bar, noa_bar, acs_bar = h.adjoint(np.asarray(I_bar, dtype=float))
        g = m.grid_pullback(rho_bar)
        ga, emb = m.absorption_pullback(x_rays, detector_position, problem.beam_position.mean, acs, acs_bar)
        g = g + ga + m.noa_pullback(noa_bar.reshape(m.values.shape[:-1] + (m.n_e,)))
        return g

    return I, pullback


def _device_pullback(problem, m: GPUMaterial, x_rays, detector_position):
    import torch
    h, dm, d, I = _device_forward(problem, m, x_rays, detector_position)
    sz = h.sizes
    f64 = dict(dtype=torch.float64, device=_DEVICE)

    def pullback(I_bar):
        ib = torch.from_numpy(np.ascontiguousarray(I_bar, dtype=np.float64)).to(_DEVICE)
        rb, nb = torch.empty(sz.n_rho, **f64), torch.empty(sz.n_noa, **f64)
        ab, G = torch.empty(max(sz.n_acs, 1), **f64), torch.empty(dm.n_params, **f64)
        # the adjoint reads the tape of this call's forward; march it again if another call used
        # the handle since
        if not _owns_tape(h, d["token"]):
            h.forward_device(d["rho"].data_ptr(), d["noa"].data_ptr(), d["acs"].data_ptr(), d["I"].data_ptr())
            d["token"] = _mark(h)
        h.adjoint_device(ib.data_ptr(), rb.data_ptr(), nb.data_ptr(), ab.data_ptr())
        dm.pullback(d["P"].data_ptr(), G.data_ptr(), rb.data_ptr(), nb.data_ptr(),
                    d["acs"].data_ptr() if len(x_rays) else None, ab.data_ptr() if len(x_rays) else None)
        _sync(torch)
        return G.cpu().numpy()

    return I, pullback


def calc_x_ray_generation_field(problem: ForwardPNProblem, m, x_rays) -> np.ndarray:
    h = get_handle(problem, x_rays)
    _mark(h)                 # the handle's densities and state change: pending pullbacks re-march
    if isinstance(m, GPUMaterial):
        import torch
        # the densities only: a material without lines (no absorption factors)
        dm = m.device((), (0.0, 0.0, 0.0), problem.beam_position.mean[0])
        P = torch.from_numpy(m.params).to(_DEVICE)
        rho = torch.empty(h.sizes.n_rho, dtype=torch.float64, device=_DEVICE)
        dm.fields(P.data_ptr(), rho.data_ptr())
        _sync(torch)
        return h.generation_field(rho.cpu().numpy())
    return h.generation_field(m.rho_flat())


def step_pn(problem: ForwardPNProblem, rho, u, i: int, x_rays=()) -> np.ndarray:
    """Advance state u (reference layout) by forward step i (0-based); returns the new state."""
    h = get_handle(problem, x_rays)
    _mark(h)
    h.set_state(rho, u)
    h.step(i)
    return h.get_state()
