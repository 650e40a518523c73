"""Host-side problem description: the counterpart of ``ForwardPNProblem`` / ``AdjointPNProblem``.

``ForwardPNProblem`` keeps the reference's constructor arguments (``pn_solver/pn_problem.jl:72``)
and produces the flat tables of the C descriptor (``include/pnepma.h``): coupling and boundary
blocks, the beam source face, and every per-step coefficient of the forward and adjoint energy
marches, evaluated at the energies the reference evaluates them at:

* forward step i uses ``update_problem!(problem, rho, E - dE/2, dE)`` and accumulates the
  intensity at the energy after the step (``pn_intensities.jl:341-349``);
* the adjoint loop evaluates the forward problem at the tape energy E, the cross-sections at E
  and at ``E + dE/2``, and the adjoint problem at ``E + dE/2`` (``pn_intensities.jl:391-404``);
* ``int_fac`` compares the loop index with the *function* ``N_steps``, so it is 1.0 for every
  step; only the two explicit 0.5 calls (initial forward accumulation at ``E_initial`` with a zero
  state, final adjoint accumulation) carry 0.5 (``pn_intensities.jl:339,347,377,393,403``).

Energies are advanced through the pseudo-time t exactly as the reference does
(``E_to_t``/``t_to_E``, ``pn_intensities.jl:10-14``), so every table value is bit-identical to
what the reference would compute from the same physical data.
"""
from __future__ import annotations

import ctypes
import math
from dataclasses import dataclass, field

import numpy as np

from . import physics
from .grid import GridSpec
from .matrices import advection_block, beam_moments, boundary_block
from .moments import N_CLASSES, class_moments, odd_in, switch

PN_ABI_VERSION = 1
PN_FP64, PN_FP32 = 0, 1
PN_FLAG_CHECK_FINITE, PN_FLAG_CHECK_CFL = 1, 2

_ODD_X = (4, 5, 6, 7)


class PnDesc(ctypes.Structure):
    """ctypes mirror of ``pn_desc``."""
    _fields_ = [
        ("abi_version", ctypes.c_int32), ("order", ctypes.c_int32),
        ("n_points", ctypes.c_int32 * 3), ("n_elements", ctypes.c_int32),
        ("n_xrays", ctypes.c_int32), ("n_steps", ctypes.c_int32), ("precision", ctypes.c_int32),
        ("checkpoint_stride", ctypes.c_int32), ("flags", ctypes.c_int32), ("reserved", ctypes.c_int32),
        ("h", ctypes.c_double * 3), ("delta_e", ctypes.c_double), ("dvol", ctypes.c_double),
        ("cfl_limit", ctypes.c_double),
        ("xray_element", ctypes.POINTER(ctypes.c_int32)),
        ("advection", ctypes.POINTER(ctypes.c_double)),
        ("boundary_fwd", ctypes.POINTER(ctypes.c_double)),
        ("boundary_adj", ctypes.POINTER(ctypes.c_double)),
        ("beam_face", ctypes.POINTER(ctypes.c_double)),
        ("fwd_s", ctypes.POINTER(ctypes.c_double)), ("fwd_c", ctypes.POINTER(ctypes.c_double)),
        ("fwd_bc", ctypes.POINTER(ctypes.c_double)), ("fwd_sigma", ctypes.POINTER(ctypes.c_double)),
        ("fwd_weight", ctypes.POINTER(ctypes.c_double)),
        ("adj_int_s", ctypes.POINTER(ctypes.c_double)), ("adj_int_c", ctypes.POINTER(ctypes.c_double)),
        ("adj_int_bc", ctypes.POINTER(ctypes.c_double)), ("adj_sigma", ctypes.POINTER(ctypes.c_double)),
        ("adj_weight", ctypes.POINTER(ctypes.c_double)),
        ("adj_src_sigma", ctypes.POINTER(ctypes.c_double)), ("adj_s", ctypes.POINTER(ctypes.c_double)),
        ("adj_c", ctypes.POINTER(ctypes.c_double)),
    ]


class PnSizes(ctypes.Structure):
    _fields_ = [
        ("n_moments", ctypes.c_int32 * 8), ("shape", (ctypes.c_int32 * 3) * 8),
        ("n_rho", ctypes.c_int64), ("n_eee_cells", ctypes.c_int64), ("n_noa", ctypes.c_int64),
        ("n_acs", ctypes.c_int64), ("n_state", ctypes.c_int64), ("n_beam_face", ctypes.c_int64),
        ("n_advection", ctypes.c_int64), ("n_boundary", ctypes.c_int64), ("device_bytes", ctypes.c_int64),
    ]


@dataclass(frozen=True)
class BeamEnergy:
    mean: float
    std: float


@dataclass(frozen=True)
class BeamPosition:
    mean: tuple          # (x, y, z) cm
    std: float

    def pdf(self, p) -> float:
        """Isotropic 3-D normal density (``MultivariateNormal(mu, sigma)``)."""
        d2 = sum((float(a) - float(b)) ** 2 for a, b in zip(p, self.mean))
        v = self.std * self.std
        return math.exp(-0.5 * d2 / v) / ((2.0 * math.pi * v) ** 1.5)


@dataclass(frozen=True)
class BeamDirection:
    mu: tuple            # mean direction
    kappa: float


@dataclass
class Physics:
    """Per-element physical data; defaults to the stand-ins of :mod:`physics`."""
    elements: list
    stopping: list = field(default=None)
    transport: object = None          # callable (element, E, N) -> array(N+1)
    sigma: object = None              # callable (xray, E) -> float

    def __post_init__(self):
        if self.stopping is None:
            self.stopping = [physics.stopping_power_table(e) for e in self.elements]
        if self.transport is None:
            self.transport = physics.transport_coefficients
        if self.sigma is None:
            self.sigma = physics.ionization_cross_section


class ForwardPNProblem:
    """Mirror of ``ForwardPNProblem{N,T}(gspec, elements, beam_energy, beam_position,
    beam_direction, E_initial, E_cutoff, N_steps)`` (pn_problem.jl:72-106)."""

    def __init__(self, N: int, gspec: GridSpec, elements, beam_energy: BeamEnergy,
                 beam_position: BeamPosition, beam_direction: BeamDirection,
                 E_initial: float, E_cutoff: float, N_steps: int, precision: int = PN_FP64,
                 phys: Physics | None = None, checkpoint_stride: int = 0):
        self.N = int(N)
        self.gspec = gspec
        self.elements = [physics.ELEMENTS[e] if isinstance(e, str) else e for e in elements]
        self.beam_energy = beam_energy
        self.beam_position = beam_position
        self.beam_direction = beam_direction
        self.E_initial = float(E_initial)
        self.E_cutoff = float(E_cutoff)
        self.N_steps = int(N_steps)
        self.precision = precision
        self.checkpoint_stride = int(checkpoint_stride)
        self.phys = phys or Physics(self.elements)
        self._tables_cache = {}

    # -------------------------------------------------------------------------------------------
    @property
    def delta_e(self) -> float:
        return (self.E_initial - self.E_cutoff) / self.N_steps

    def forward_energies(self):
        """(E_mid per step, E after each step) with E_0 = E_initial."""
        dE = self.delta_e
        E = self.E_initial
        mids, ends = [], [E]
        for _ in range(self.N_steps):
            mids.append(E - dE / 2)
            t = self.E_initial - E
            t = t + dE
            E = self.E_initial - t
            ends.append(E)
        return mids, ends

    def adjoint_energies(self):
        """Tape energies Ea_j, j = 0..N_steps (Ea_0 = E_cutoff)."""
        dE = self.delta_e
        E = self.E_cutoff
        out = [E]
        for _ in range(self.N_steps):
            t = E - self.E_cutoff
            t = t + dE
            E = self.E_cutoff + t
            out.append(E)
        return out

    # -------------------------------------------------------------------------------------------
    def _coeffs(self, E: float, adjoint: bool):
        """(s[e], c[e][l]) as update_coefficients! fills them (pn_problem.jl:157-190)."""
        ne, N = len(self.elements), self.N
        s = np.empty(ne)
        c = np.empty((ne, N + 1))
        for i, tab in enumerate(self.phys.stopping):
            s[i] = tab(E)
        for i, el in enumerate(self.elements):
            tc = np.asarray(self.phys.transport(el, E, N), dtype=float)
            base = 0.0 if adjoint else -tab_slope(self.phys.stopping[i], E)
            for l in range(N + 1):
                c[i, l] = base - (tc[l] - tc[0])
        return s, c

    def _bc_weight(self, E: float) -> float:
        dE = self.delta_e
        be = self.beam_energy
        return (physics.normal_cdf(E + dE, be.mean, be.std) - physics.normal_cdf(E, be.mean, be.std)) / dE

    def beam_face(self) -> list[np.ndarray]:
        """gx_temp right-face values per odd-in-x class: array [nz][ny][n_c] (pn_problem.jl:192-203)."""
        ms = class_moments(self.N)
        out = []
        for c in _ODD_X:
            mms = beam_moments(list(ms[c]), self.beam_direction.mu, self.beam_direction.kappa)
            ev = switch(c, 0)
            px, py, pz = self.gspec.class_points(ev)
            nx, ny, nz = self.gspec.class_shape(c)
            face = np.zeros((nz, ny, len(ms[c])))
            for k in range(nz):
                for j in range(ny):
                    # evaluated at the first x point of the even grid (the reference's [1, :, :])
                    pp = self.beam_position.pdf((px[0], py[j], pz[k]))
                    face[k, j, :] = mms * pp
            out.append(face)
        return out

    def tables(self, x_rays) -> dict:
        key = tuple(x_rays)
        if key in self._tables_cache:
            return self._tables_cache[key]
        N, ne, nr, ns = self.N, len(self.elements), len(x_rays), self.N_steps
        el_names = [e.symbol for e in self.elements]
        xray_element = np.array([el_names.index(x.element) for x in x_rays], dtype=np.int32)
        mids, ends = self.forward_energies()
        t = {}
        t["xray_element"] = xray_element
        t["fwd_s"] = np.empty((ns, ne))
        t["fwd_c"] = np.empty((ns, ne, N + 1))
        t["fwd_bc"] = np.empty(ns)
        for i, Em in enumerate(mids):
            t["fwd_s"][i], t["fwd_c"][i] = self._coeffs(Em, adjoint=False)
            t["fwd_bc"][i] = self._bc_weight(Em)
        t["fwd_sigma"] = np.array([[self.phys.sigma(x, E) for x in x_rays] for E in ends]).reshape(ns + 1, nr)
        t["fwd_weight"] = np.ones(ns + 1)
        t["fwd_weight"][0] = 0.5
        Ea = self.adjoint_energies()
        dE = self.delta_e
        t["adj_int_s"] = np.empty((ns + 1, ne))
        t["adj_int_c"] = np.empty((ns + 1, ne, N + 1))
        t["adj_int_bc"] = np.empty(ns + 1)
        t["adj_sigma"] = np.empty((ns + 1, nr))
        t["adj_src_sigma"] = np.zeros((ns + 1, nr))
        t["adj_s"] = np.zeros((ns + 1, ne))
        t["adj_c"] = np.zeros((ns + 1, ne, N + 1))
        for j, E in enumerate(Ea):
            t["adj_int_s"][j], t["adj_int_c"][j] = self._coeffs(E, adjoint=False)
            t["adj_int_bc"][j] = self._bc_weight(E)
            t["adj_sigma"][j] = [self.phys.sigma(x, E) for x in x_rays]
            if j < ns:
                Eh = E + dE / 2
                t["adj_src_sigma"][j] = [self.phys.sigma(x, Eh) for x in x_rays]
                t["adj_s"][j], t["adj_c"][j] = self._coeffs(Eh, adjoint=True)
        t["adj_weight"] = np.ones(ns + 1)
        t["adj_weight"][ns] = 0.5
        # matrices
        adv, bf, ba = [], [], []
        for d in range(3):
            for c in range(N_CLASSES):
                adv.append(advection_block(N, c, d).ravel())
                if odd_in(c, d):
                    bf.append(boundary_block(N, c, d, adjoint=False).ravel())
                    ba.append(boundary_block(N, c, d, adjoint=True).ravel())
        t["advection"] = np.concatenate(adv) if adv else np.zeros(0)
        t["boundary_fwd"] = np.concatenate(bf)
        t["boundary_adj"] = np.concatenate(ba)
        t["beam_face"] = np.concatenate([f.ravel() for f in self.beam_face()])
        for k, v in t.items():
            if k != "xray_element":
                t[k] = np.ascontiguousarray(v, dtype=np.float64)
        self._tables_cache[key] = t
        return t

    def cfl_dt_max(self, rho_min_stopping: float, cfl: float = 1.0) -> float:
        """``compute_dt_max`` (pn_intensities.jl:2-8) for a given minimum of S."""
        dx, dy, dz = self.gspec.h
        m = rho_min_stopping
        return cfl / (1.0 / (dx * m) + 1.0 / (dy * m) + 1.0 / (dz * m))

    def descriptor(self, x_rays, flags: int = 0, cfl_limit: float = 0.0):
        """(PnDesc, keepalive) for this problem and line list."""
        t = self.tables(x_rays)
        d = PnDesc()
        d.abi_version = PN_ABI_VERSION
        d.order = self.N
        for i, a in enumerate(self.gspec.axes):
            d.n_points[i] = a.M
            d.h[i] = a.step
        d.n_elements = len(self.elements)
        d.n_xrays = len(x_rays)
        d.n_steps = self.N_steps
        d.precision = self.precision
        d.checkpoint_stride = self.checkpoint_stride
        d.flags = flags
        d.delta_e = self.delta_e
        d.dvol = self.gspec.dvol
        d.cfl_limit = cfl_limit
        keep = []

        def ptr(a, ct=ctypes.c_double):
            keep.append(a)
            return a.ctypes.data_as(ctypes.POINTER(ct))

        d.xray_element = ptr(t["xray_element"], ctypes.c_int32)
        for name in ("advection", "boundary_fwd", "boundary_adj", "beam_face", "fwd_s", "fwd_c", "fwd_bc",
                     "fwd_sigma", "fwd_weight", "adj_int_s", "adj_int_c", "adj_int_bc", "adj_sigma",
                     "adj_weight", "adj_src_sigma", "adj_s", "adj_c"):
            setattr(d, name, ptr(t[name]))
        return d, keep


def tab_slope(tab, E):
    return tab.slope(E)


class AdjointPNProblem:
    """Mirror of ``AdjointPNProblem(frwd)`` (pn_problem.jl:108-136); its tables are part of the
    forward problem's descriptor (the adjoint march always follows a forward march)."""

    def __init__(self, frwd: ForwardPNProblem):
        self.forward = frwd
        self.N = frwd.N
        self.gspec = frwd.gspec
        self.E_initial, self.E_cutoff, self.N_steps = frwd.E_initial, frwd.E_cutoff, frwd.N_steps
