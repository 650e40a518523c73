"""Synthetic workloads with the shapes of the benchmark configurations.

No measured data set belongs to this path; every input is generated from a seeded
``numpy.random.Generator(PCG64(seed))``.  Axis convention follows the reference scripts: x is depth
(sample at x <= 0, surface at x = 0), the beam enters through the x = 0 face with direction
(-1, 0, 0), y and z are lateral (``scripts/sensitivities_1d.jl:7-11,100-122``).

The march is explicit and the reference does not enforce its own stability estimate
(``compute_dt_max``, ``pn_intensities.jl:2-8``).  :func:`stable_steps` returns
``max(N_cfg, ceil((E_initial - E_cutoff) / (f dt_max)))`` with dt_max from that estimate at the
initial energy, where the stopping power and hence the admissible step is smallest.  The factor f
comes from the spectral radius of the one-step map of the scheme (constant coefficients, no
scattering): with the reference's ghost-point boundary closure a saw-tooth mode localised at the
boundaries grows above ~0.75 dt_max in 1D for N >= 5, while 2D stays stable up to dt_max (its
estimate is more conservative).  f = 0.6 in 1D and 0.9 otherwise.
"""
from __future__ import annotations

import math
from dataclasses import dataclass

import numpy as np

from . import physics
from .grid import GridSpec
from .material import BoxedMassFraction
from .problem import (PN_FP32, PN_FP64, BeamDirection, BeamEnergy, BeamPosition,
                      ForwardPNProblem)

UM = 1e-4   # cm
NM = 1e-7


@dataclass
class Solve:
    """One forward+adjoint solve: problem, material and measurement geometry."""
    problem: ForwardPNProblem
    material: BoxedMassFraction
    x_rays: list
    detector: tuple
    label: str = ""

    def inputs(self):
        """(rho, noa, acs) in the C-ABI layout (memoised on the material: solves that share a
        material, lines, detector and beam depth share the arrays)."""
        m = self.material
        key = (tuple(self.x_rays), tuple(self.detector), float(self.problem.beam_position.mean[0]))
        memo = m.__dict__.setdefault("_inputs_memo", {})
        if key not in memo:
            rho = m.rho_flat()
            noa = m.number_of_atoms().reshape(-1, m.n_e)
            acs = m.absorption(self.x_rays, self.detector, self.problem.beam_position.mean).reshape(-1, len(self.x_rays))
            memo[key] = (rho, np.ascontiguousarray(noa), np.ascontiguousarray(acs))
        return memo[key]


def min_stopping(material: BoxedMassFraction, problem: ForwardPNProblem, E: float) -> float:
    s = np.array([tab(E) for tab in problem.phys.stopping])
    rho = material.densities_on_grids()
    return float(min(np.min(r @ s) for r in rho))


def stable_steps(problem: ForwardPNProblem, material: BoxedMassFraction, n_cfg: int, safety: float | None = None) -> int:
    if safety is None:
        safety = 0.6 if len(problem.gspec.active_dims) == 1 else 0.9
    Smin = min_stopping(material, problem, problem.E_initial)
    dt_max = problem.cfl_dt_max(Smin, 1.0)
    need = math.ceil((problem.E_initial - problem.E_cutoff) / (safety * dt_max))
    return max(int(n_cfg), int(need))


def _rng(seed):
    return np.random.Generator(np.random.PCG64(seed))


def smooth_fractions(rng, gspec: GridSpec, n_e: int, n_bumps: int = 8, width=(0.1, 0.3),
                     inclusion=None):
    """Softmax of a sum of Gaussian bumps at the eee cell centres: [nz][ny][nx][n_e]."""
    px, py, pz = gspec.class_points(0)
    Z, Y, X = np.meshgrid(pz, py, px, indexing="ij")
    lo = np.array([a.lo for a in gspec.axes])
    hi = np.array([a.hi for a in gspec.axes])
    field = np.zeros(X.shape + (n_e,))
    for _ in range(n_bumps):
        c = lo + (hi - lo) * rng.random(3)
        w = rng.uniform(*width) * UM
        a = rng.standard_normal(n_e)
        r2 = (X - c[0]) ** 2 + (Y - c[1]) ** 2 + (Z - c[2]) ** 2
        field += np.exp(-r2 / (2 * w * w))[..., None] * a
    if inclusion is not None:
        centre, radius, amp = inclusion
        r2 = (X - centre[0]) ** 2 + (Y - centre[1]) ** 2 + (Z - centre[2]) ** 2
        field += (r2 <= radius * radius)[..., None] * amp
    field -= field.max(axis=-1, keepdims=True)
    e = np.exp(field)
    return e / e.sum(axis=-1, keepdims=True)


def make_solve(N, gspec, elements, fractions, beam_kev, beam_y=0.0, beam_sigma=30 * NM, kappa=50.0,
               E_init=None, E_cut=None, n_steps=100, sc=False, detector=(10 * NM, 0.0, 0.0),
               precision=PN_FP64, lines=None, stabilise=True, checkpoint_stride=0, label=""):
    els = [physics.ELEMENTS[e] for e in elements]
    x_rays = lines or [physics.XRay(e, "K-L3") for e in elements]
    E0 = beam_kev * 1e3
    if E_init is None:
        E_init = E0 + 500.0
    if E_cut is None:
        E_cut = min(x.edge for x in x_rays) - 100.0
    values = fractions[..., :-1] if sc else fractions
    mat = BoxedMassFraction(els, gspec, values, sc=sc)
    prob = ForwardPNProblem(N, gspec, els, BeamEnergy(E0, 100.0), BeamPosition((0.0, beam_y, 0.0), beam_sigma),
                            BeamDirection((-1.0, 0.0, 0.0), kappa), E_init, E_cut, n_steps, precision=precision,
                            checkpoint_stride=checkpoint_stride)
    if stabilise:
        ns = stable_steps(prob, mat, n_steps)
        if ns != n_steps:
            prob = ForwardPNProblem(N, gspec, els, prob.beam_energy, prob.beam_position, prob.beam_direction,
                                    E_init, E_cut, ns, precision=precision, checkpoint_stride=checkpoint_stride)
    return Solve(prob, mat, x_rays, tuple(detector), label)


# ---------------------------------------------------------------------------------------- configs
def config1(seed: int = 1, precision=PN_FP64, stabilise=True) -> Solve:
    """1D slab: 200 cells over 1 um, N=7, Cu/Ni in 4 layers, 15 keV, 100 steps to 1 keV."""
    rng = _rng(seed)
    gspec = GridSpec.make((200, 1, 1), (-1 * UM, 0.0), 0.0, 0.0)
    cu = rng.uniform(0.1, 0.9, 4)
    layer = np.minimum((np.arange(200) * 4) // 200, 3)
    w = np.zeros((1, 1, 200, 2))
    w[0, 0, :, 0] = cu[layer]
    w[0, 0, :, 1] = 1.0 - cu[layer]
    return make_solve(7, gspec, ["Cu", "Ni"], w, 15.0, beam_sigma=30 * NM, E_init=15.5e3, E_cut=1.0e3,
                      n_steps=100, sc=True, precision=precision, stabilise=stabilise, label="slab1d")


def config2(seed: int = 2, precision=PN_FP64, stabilise=True, n_positions=20, energies=(10.0, 15.0, 20.0),
            n_steps=200, shape=(128, 256)):
    """2D: 256 (lateral) x 128 (depth) over 2 x 1 um, N=11, Fe/Cr/Ni smooth field, 20 positions x 3 energies."""
    rng = _rng(seed)
    mx, my = shape
    gspec = GridSpec.make((mx, my, 1), (-1 * UM, 0.0), (-1 * UM, 1 * UM), 0.0)
    frac = smooth_fractions(rng, gspec, 3)
    ys = np.linspace(-1 * UM, 1 * UM, n_positions + 2)[1:-1] if n_positions > 1 else [0.0]
    out = []
    mat = None
    for E in energies:
        for y in ys:
            s = make_solve(11, gspec, ["Fe", "Cr", "Ni"], frac, E, beam_y=float(y), beam_sigma=50 * NM,
                           n_steps=n_steps, detector=(100 * NM, 0.0, 0.0), precision=precision,
                           stabilise=stabilise, label=f"2d256x128 E={E} y={y:.3e}")
            if mat is None:
                mat = s.material
            s.material = mat
            out.append(s)
    return out


def config3(seed: int = 3, n_instances: int = 256, stabilise=True):
    """Batched FP32 mix: grids {64x32, 128x64, 256x128}, N in {5,7,11}, 2-4 of Fe/Cr/Ni/Cu."""
    rng = _rng(seed)
    shapes = [(32, 64), (64, 128), (128, 256)]
    pool = ["Fe", "Cr", "Ni", "Cu"]
    out = []
    for i in range(n_instances):
        mx, my = shapes[rng.integers(3)]
        N = int(rng.choice([5, 7, 11]))
        ne = int(rng.integers(2, 5))
        els = list(rng.choice(pool, ne, replace=False))
        E = float(rng.uniform(8.0, 25.0))
        gspec = GridSpec.make((mx, my, 1), (-1 * UM, 0.0), (-1 * UM, 1 * UM), 0.0)
        frac = smooth_fractions(rng, gspec, ne)
        x_rays = [physics.XRay(e, "K-L3") for e in els]
        E_cut = min(x.edge for x in x_rays) - 100.0
        n_steps = max(1, int(round(10 * (E * 1e3 + 500.0 - E_cut) / 1e3)))
        y = float(rng.uniform(-0.5, 0.5) * UM)
        out.append(make_solve(N, gspec, els, frac, E, beam_y=y, beam_sigma=50 * NM, n_steps=n_steps,
                              detector=(100 * NM, 0.0, 0.0), precision=PN_FP32, stabilise=stabilise,
                              label=f"mixed2d[{i}] N={N} {mx}x{my} ne={ne} E={E:.2f}"))
    return out


def config4(seed: int = 4, precision=PN_FP32, stabilise=True, shape=(64, 96, 96), n_steps=300,
            checkpoint_stride=16):
    """3D: 96 x 96 (lateral) x 64 (depth) over 1.5 x 1.5 x 1 um, N=7, 3 elements with an inclusion."""
    rng = _rng(seed)
    mx, my, mz = shape
    gspec = GridSpec.make((mx, my, mz), (-1 * UM, 0.0), (-0.75 * UM, 0.75 * UM), (-0.75 * UM, 0.75 * UM))
    lo = np.array([-0.8 * UM, -0.55 * UM, -0.55 * UM])
    hi = np.array([-0.2 * UM, 0.55 * UM, 0.55 * UM])
    centre = lo + (hi - lo) * rng.random(3)
    amp = rng.standard_normal(3) * 3.0
    frac = smooth_fractions(rng, gspec, 3, inclusion=(centre, 0.2 * UM, amp))
    return make_solve(7, gspec, ["Fe", "Cr", "Ni"], frac, 20.0, beam_sigma=50 * NM, n_steps=n_steps,
                      detector=(100 * NM, 0.0, 0.0), precision=precision, stabilise=stabilise,
                      checkpoint_stride=checkpoint_stride, label="3d96x96x64")


def small_case(dims: int = 2, N: int = 3, shape=None, n_steps: int = 12, seed: int = 7, precision=PN_FP64,
               elements=("Cu", "Ni"), beam_kev: float = 12.0, stabilise=True, checkpoint_stride=0):
    """A small problem for parity tests (runs on the oracle in well under a second)."""
    rng = _rng(seed)
    if dims == 1:
        shape = shape or (24,)
        gspec = GridSpec.make((shape[0], 1, 1), (-0.5 * UM, 0.0), 0.0, 0.0)
    elif dims == 2:
        shape = shape or (12, 10)
        gspec = GridSpec.make((shape[0], shape[1], 1), (-0.5 * UM, 0.0), (-0.4 * UM, 0.4 * UM), 0.0)
    else:
        shape = shape or (8, 7, 6)
        gspec = GridSpec.make(tuple(shape), (-0.5 * UM, 0.0), (-0.4 * UM, 0.4 * UM), (-0.3 * UM, 0.3 * UM))
    frac = smooth_fractions(rng, gspec, len(elements), width=(0.05, 0.2))
    return make_solve(N, gspec, list(elements), frac, beam_kev, beam_sigma=60 * NM, n_steps=n_steps,
                      E_cut=min(physics.ELEMENTS[e].k_edge_ev for e in elements) - 500.0,
                      detector=(50 * NM, 0.1 * UM, 0.0), precision=precision, stabilise=stabilise,
                      checkpoint_stride=checkpoint_stride, label=f"small{dims}d")


@dataclass
class Request:
    """One served request: a reconstruction iteration's solves (positions x energies) on one material."""
    kind: str
    arrival_s: float
    solves: list


def config5_kind(kind: str, seed: int, precision=PN_FP32, positions: int = 16, energies=(10.0, 15.0),
                 stabilise=True):
    """The solves of one request of a kind: '1d' N=7 200 cells over 1 um (Cu/Ni); '2d' N=11
    128 (lateral) x 64 (depth) over 2 x 1 um; '3d' N=5 64 x 64 (lateral) x 48 (depth) over
    1.5 x 1.5 x 1 um (Fe/Cr/Ni).  Composition: a seeded smooth field; beam positions evenly across
    the lateral extent (on the axis in 1D)."""
    rng = _rng(seed)
    if kind == "1d":
        gspec = GridSpec.make((200, 1, 1), (-1 * UM, 0.0), 0.0, 0.0)
        els, N, ys = ["Cu", "Ni"], 7, [0.0] * positions
    elif kind == "2d":
        gspec = GridSpec.make((64, 128, 1), (-1 * UM, 0.0), (-1 * UM, 1 * UM), 0.0)
        els, N = ["Fe", "Cr", "Ni"], 11
        ys = list(np.linspace(-1 * UM, 1 * UM, positions + 2)[1:-1])
    elif kind == "3d":
        gspec = GridSpec.make((48, 64, 64), (-1 * UM, 0.0), (-0.75 * UM, 0.75 * UM), (-0.75 * UM, 0.75 * UM))
        els, N = ["Fe", "Cr", "Ni"], 5
        ys = list(np.linspace(-0.75 * UM, 0.75 * UM, positions + 2)[1:-1])
    else:
        raise ValueError(kind)
    frac = smooth_fractions(rng, gspec, len(els))
    out, mat = [], None
    for E in energies:
        for y in ys:
            s = make_solve(N, gspec, els, frac, E, beam_y=float(y), beam_sigma=50 * NM, n_steps=100,
                           detector=(100 * NM, 0.0, 0.0), precision=precision, stabilise=stabilise,
                           label=f"served {kind} E={E} y={y:.3e}")
            if mat is None:
                mat = s.material
            s.material = mat          # one material per request: the inputs are shared
            out.append(s)
    return out


def config5(n_requests: int = 64, seed: int = 5, rate: float = 200.0, mix=(0.5, 0.4, 0.1),
            precision=PN_FP32, materials_per_kind: int = 3, positions: int = 16, energies=(10.0, 15.0)):
    """Served stream: Poisson arrivals at `rate` requests/s; kinds 1d/2d/3d drawn with `mix`; each
    request is `positions` x `energies` forward+adjoint solves.  The compositions cycle through a
    pool of `materials_per_kind` seeded fields per kind (host preparation of a 3D material takes
    seconds; the device work does not depend on which field a request carries)."""
    rng = _rng(seed)
    kinds = rng.choice(["1d", "2d", "3d"], size=n_requests, p=list(mix))
    t = np.cumsum(rng.exponential(1.0 / rate, size=n_requests))
    t -= t[0]
    pool = {}
    out = []
    counts = {"1d": 0, "2d": 0, "3d": 0}
    for i, k in enumerate(kinds):
        slot = counts[k] % materials_per_kind
        counts[k] += 1
        if (k, slot) not in pool:
            pool[(k, slot)] = config5_kind(k, seed * 1000 + 10 * slot + {"1d": 1, "2d": 2, "3d": 3}[k],
                                           precision=precision, positions=positions, energies=energies)
        out.append(Request(str(k), float(t[i]), pool[(k, slot)]))
    return out
