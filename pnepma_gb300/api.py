"""Reference-shaped entry points over the GPU library.

These keep the names and argument meaning of the reference's Julia API for this path:

* ``calc_intensities(problem, m, x_rays, detector_position)`` -- pn_intensities.jl:325-351
* ``calc_intensities_pullback(problem, m, x_rays, detector_position)`` -- the Zygote adjoint of
  the same function (pn_intensities.jl:353-413): returns the intensities and a pullback that maps
  a cotangent of the intensities to the gradient with respect to the material parameters
* ``calc_x_ray_generation_field(problem, m, x_rays)`` -- pn_intensities.jl:189-212
* ``step_pn(problem, rho, u, i)`` -- one forward energy step of a state (pn_intensities.jl:16-22)

The material model here is the per-cell boxed mass-fraction material (:mod:`material`); the
densities on the eight grids, the number of atoms and the absorption factors are formed on the
host, the march and its adjoint run on the GPU, and the parameter pullbacks are applied on the
host, as the reference's shim would do (pn_intensities.jl:406-409).
"""
from __future__ import annotations

import numpy as np

from .capi import Handle
from .problem import ForwardPNProblem

_CACHE: dict = {}
_CACHE_MAX = 8


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


def _inputs(problem, m, x_rays, detector_position):
    rho = m.rho_flat()
    noa = m.number_of_atoms().reshape(-1, m.n_e)
    acs = m.absorption(x_rays, detector_position, problem.beam_position.mean).reshape(-1, len(x_rays))
    return rho, noa, acs


def calc_intensities(problem: ForwardPNProblem, m, x_rays, detector_position) -> np.ndarray:
    h = get_handle(problem, x_rays)
    rho, noa, acs = _inputs(problem, m, x_rays, detector_position)
    return h.forward(rho, noa, acs)


def calc_intensities_pullback(problem: ForwardPNProblem, m, x_rays, detector_position):
    """(intensities, pullback); pullback(I_bar) -> d(material parameters), shape of ``m.values``."""
    h = get_handle(problem, x_rays)
    rho, noa, acs = _inputs(problem, m, x_rays, detector_position)
    I = h.forward(rho, noa, acs)

    def pullback(I_bar):
        rho_bar, noa_bar, acs_bar = h.adjoint(np.asarray(I_bar, dtype=float))
        g = m.grid_pullback(rho_bar)
        ga, emb = m.absorption_pullback(x_rays, detector_position, problem.beam_position.mean, acs, acs_bar)
        g = g + ga + m.noa_pullback(noa_bar.reshape(m.values.shape[:-1] + (m.n_e,)))
        return g

    return I, pullback


def calc_x_ray_generation_field(problem: ForwardPNProblem, m, x_rays) -> np.ndarray:
    h = get_handle(problem, x_rays)
    return h.generation_field(m.rho_flat())


def step_pn(problem: ForwardPNProblem, rho, u, i: int, x_rays=()) -> np.ndarray:
    """Advance state u (reference layout) by forward step i (0-based); returns the new state."""
    h = get_handle(problem, x_rays)
    h.set_state(rho, u)
    h.step(i)
    return h.get_state()
