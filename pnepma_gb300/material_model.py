"""Host description of a material for the device material kernels (``pn_material_*``).

Mirrors the reference's material types (``pn_parametrizations/pn_material.jl``): a model
(MassConcentration, VolumeFraction, LinearDensity, MassFraction, each but the first with an SC
variant) over a parametrisation (Const, Boxed, Bilinear), and the data the solve's inputs need
(element densities and atomic masses, mass absorption coefficients, detector and beam position).
``descriptor()`` builds the ``pn_material_desc`` of ``include/pnepma.h``; the parameter vector is
the reference's ``param_vec`` order (boxes or knots ``[z][y][x][n_par]``, then the embedding).
"""
from __future__ import annotations

import ctypes
from dataclasses import dataclass

import numpy as np

from . import physics
from .grid import GridSpec

MODELS = {"mass_concentration": 0, "volume_fraction": 1, "linear_density": 2, "mass_fraction": 3}
PARAMETRIZATIONS = {"const": 0, "boxed": 1, "bilinear": 2}


class PnSlices(ctypes.Structure):
    _fields_ = [("n", ctypes.c_int32), ("offset", ctypes.c_int32), ("ref", ctypes.c_double),
                ("step", ctypes.c_double), ("values", ctypes.c_void_p)]


class PnMaterialDesc(ctypes.Structure):
    _fields_ = [("model", ctypes.c_int32), ("sc", ctypes.c_int32), ("parametrization", ctypes.c_int32),
                ("n_elements", ctypes.c_int32), ("n_points", ctypes.c_int32 * 3), ("n_xrays", ctypes.c_int32),
                ("n_int_points", ctypes.c_int32), ("reserved", ctypes.c_int32), ("coords", ctypes.c_void_p),
                ("slices", PnSlices * 3), ("rho_pure", ctypes.c_void_p), ("atom_mass", ctypes.c_void_p),
                ("mac", ctypes.c_void_p), ("detector", ctypes.c_double * 3), ("beam_x", ctypes.c_double)]


@dataclass
class Slices:
    """Slice values (Boxed) or knots (Bilinear) along one axis.

    Range form: Julia's ``StepRangeLen`` given by ``ref`` (value at the 1-based index ``offset``),
    ``step`` and length ``n``; value i (1-based) is ref + (i - offset) step.  Vector form:
    explicit increasing ``values`` (Boxed only).
    """
    n: int
    offset: int = 1
    ref: float = 0.0
    step: float = 1.0
    values: np.ndarray | None = None

    @staticmethod
    def range(first: float, last: float, n: int) -> "Slices":
        """``range(first, last, length=n)`` with ref = first (offset 1).  Julia may pick another
        element as its reference; a shim passes the range's own ref, step and offset."""
        if n == 1:
            return Slices(1, 1, float(first), 1.0)
        return Slices(int(n), 1, float(first), (float(last) - float(first)) / (n - 1))

    @staticmethod
    def vector(values) -> "Slices":
        v = np.ascontiguousarray(values, dtype=np.float64)
        return Slices(int(v.size), 1, float(v[0]), 0.0, v)

    def value(self, i: int) -> float:
        """Value at 1-based index i."""
        if self.values is not None:
            return float(self.values[i - 1])
        return self.ref + (i - self.offset) * self.step


class MaterialModel:
    """A material on a staggered grid, with everything the device material kernels need."""

    def __init__(self, gspec: GridSpec, elements, model: str, sc: bool = False, parametrization: str = "const",
                 slices=None, x_rays=(), detector=(0.0, 0.0, 0.0), beam_x: float = 0.0, n_int_points: int = 100):
        self.gspec = gspec
        self.elements = [physics.ELEMENTS[e] if isinstance(e, str) else e for e in elements]
        self.n_e = len(self.elements)
        self.model = model
        self.sc = bool(sc)
        self.parametrization = parametrization
        self.slices = list(slices) if slices is not None else None
        self.x_rays = list(x_rays)
        self.detector = np.asarray(detector, dtype=float)
        self.beam_x = float(beam_x)
        self.n_int_points = int(n_int_points)
        if model not in MODELS or parametrization not in PARAMETRIZATIONS:
            raise ValueError("unknown model or parametrisation")
        if parametrization != "const" and (self.slices is None or len(self.slices) != 3):
            raise ValueError("boxed and bilinear parametrisations need slices for x, y and z")
        self.n_par = self.n_e - 1 if self.sc else self.n_e
        self.rho_pure = np.array([e.density for e in self.elements])
        self.atom_mass = np.array([e.atomic_mass_g for e in self.elements])
        self.mac = np.array([[physics.mass_absorption(x, e) for e in self.elements] for x in self.x_rays]
                            ).reshape(len(self.x_rays), self.n_e)

    # ------------------------------------------------------------------ sizes
    @property
    def grid_shape(self) -> tuple[int, int, int]:
        """(nx, ny, nz) of boxes or knots."""
        if self.parametrization == "const":
            return (1, 1, 1)
        if self.parametrization == "boxed":
            return tuple(s.n - 1 for s in self.slices)
        return tuple(s.n for s in self.slices)

    @property
    def n_params(self) -> int:
        if self.parametrization == "const":
            return self.n_par
        nx, ny, nz = self.grid_shape
        return (nx * ny * nz + 1) * self.n_par

    def coords(self) -> np.ndarray:
        """Per axis: the even points, then the odd points (``points(eo, gspec)``)."""
        parts = []
        for d in range(3):
            ax = self.gspec.axes[d]
            parts.append(ax.points(False))
            parts.append(ax.points(True))
        return np.ascontiguousarray(np.concatenate(parts), dtype=np.float64)

    # ------------------------------------------------------------------ descriptor
    def descriptor(self):
        """(PnMaterialDesc, keepalive): the C descriptor and the arrays its pointers reference."""
        keep = {"coords": self.coords(), "rho_pure": np.ascontiguousarray(self.rho_pure),
                "atom_mass": np.ascontiguousarray(self.atom_mass),
                "mac": np.ascontiguousarray(self.mac, dtype=np.float64)}
        d = PnMaterialDesc()
        d.model = MODELS[self.model]
        d.sc = 1 if self.sc else 0
        d.parametrization = PARAMETRIZATIONS[self.parametrization]
        d.n_elements = self.n_e
        for k in range(3):
            d.n_points[k] = self.gspec.axes[k].M
        d.n_xrays = len(self.x_rays)
        d.n_int_points = self.n_int_points
        d.coords = keep["coords"].ctypes.data
        if self.slices is not None:
            for k, s in enumerate(self.slices):
                d.slices[k].n = s.n
                d.slices[k].offset = s.offset
                d.slices[k].ref = s.ref
                d.slices[k].step = s.step
                if s.values is not None:
                    v = np.ascontiguousarray(s.values, dtype=np.float64)
                    keep[f"slices{k}"] = v
                    d.slices[k].values = v.ctypes.data
        d.rho_pure = keep["rho_pure"].ctypes.data
        d.atom_mass = keep["atom_mass"].ctypes.data
        d.mac = keep["mac"].ctypes.data if self.mac.size else None
        for k in range(3):
            d.detector[k] = float(self.detector[k])
        d.beam_x = self.beam_x
        return d, keep

    def with_geometry(self, x_rays, detector, beam_x: float) -> "MaterialModel":
        """The same material seen from another measurement geometry (lines, detector, beam)."""
        return MaterialModel(self.gspec, self.elements, self.model, sc=self.sc, parametrization=self.parametrization,
                             slices=self.slices, x_rays=list(x_rays), detector=detector, beam_x=beam_x,
                             n_int_points=self.n_int_points)

    @staticmethod
    def per_cell_boxed(mat, x_rays, detector, beam_x: float = 0.0, n_int_points: int = 100):
        """(MaterialModel, params) of a ``material.BoxedMassFraction``: a MassFraction(SC) model
        over one box per eee cell, whose slices are the odd-grid points (a range of M + 1 values
        from lo - h/2); a singleton axis gets one box [p - 1/2, p + 1/2] around its point.  The
        floor rule puts an odd-grid point on the box above its slice (the last on the last box);
        ``BoxedMassFraction`` applies the same rule with integers, which agrees wherever the
        floating-point quotient is exact (grids whose coordinates are binary fractions)."""
        sl = []
        for d in range(3):
            ax = mat.gspec.axes[d]
            if ax.singleton:
                sl.append(Slices.range(ax.lo - 0.5, ax.lo + 0.5, 2))
            else:
                h = ax.step
                sl.append(Slices.range(ax.lo - h / 2, ax.hi + h / 2, ax.M + 1))
        mm = MaterialModel(mat.gspec, mat.elements, "mass_fraction", sc=mat.sc, parametrization="boxed",
                           slices=sl, x_rays=x_rays, detector=detector, beam_x=beam_x, n_int_points=n_int_points)
        params = np.concatenate([np.asarray(mat.values, dtype=float).ravel(),
                                 np.asarray(mat.embedding, dtype=float).ravel()])
        return mm, params

    def random_params(self, rng: np.random.Generator, lo: float = 0.1, hi: float = 0.9) -> np.ndarray:
        """Parameters drawn uniformly; SC variants keep the sum of each vector below 1."""
        p = rng.uniform(lo, hi, size=(self.n_params // self.n_par, self.n_par))
        if self.sc:
            p *= 0.9 / np.maximum(p.sum(axis=1, keepdims=True), 0.9)
        return p.ravel()
