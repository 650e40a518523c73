"""Staggered grid specification (``starmap/src/staggered_grid.jl``).

Each axis is either a singleton (one point, step 1.0, ``staggered_grid.jl:21-24,58-60``) or an
extent ``(lo, hi)`` with ``M`` points.  Classes even in an axis live on the M "even" points
``lo + i h`` (``h = (hi - lo)/(M - 1)``); classes odd in it live on M + 1 points shifted by h/2
with one ghost point outside each end (``OddWithGhostDimension``, ``staggered_grid.jl:25-28,
54-56,75-78``).  ``dvol`` is the product of the three steps (``staggered_grid.jl:166``).
"""
from __future__ import annotations

from dataclasses import dataclass
from fractions import Fraction

import numpy as np

from .moments import N_CLASSES, class_bits


def _linspace_exact(lo: float, hi: float, n: int) -> np.ndarray:
    """Points lo + i (hi - lo)/(n - 1), each rounded once (Julia's range uses extra precision)."""
    if n == 1:
        return np.array([lo])
    flo, fhi = Fraction(lo), Fraction(hi)
    return np.array([float(flo + (fhi - flo) * i / (n - 1)) for i in range(n)])


@dataclass(frozen=True)
class Axis:
    M: int                       # number of even points (1 for a singleton)
    lo: float
    hi: float                    # equal to lo for a singleton

    @property
    def singleton(self) -> bool:
        return self.M == 1 and self.lo == self.hi

    @property
    def step(self) -> float:
        if self.singleton:
            return 1.0
        return (self.hi - self.lo) / (self.M - 1)

    def size(self, odd: bool) -> int:
        if self.singleton:
            return 1
        return self.M + 1 if odd else self.M

    def points(self, odd: bool) -> np.ndarray:
        if self.singleton:
            return np.array([self.lo])
        if not odd:
            return _linspace_exact(self.lo, self.hi, self.M)
        h = self.step
        return _linspace_exact(self.lo - h / 2, self.hi + h / 2, self.M + 1)


@dataclass(frozen=True)
class GridSpec:
    axes: tuple[Axis, Axis, Axis]

    @staticmethod
    def make(M, x, y, z) -> "GridSpec":
        """``make_gridspec(M, x, y, z)``: each of x, y, z is a (lo, hi) tuple or a scalar position."""
        if isinstance(M, int):
            M = (M, M, M)
        axes = []
        for m, e in zip(M, (x, y, z)):
            if isinstance(e, (tuple, list)):
                if m < 2:
                    raise ValueError("an axis with an extent needs at least two points")
                axes.append(Axis(int(m), float(e[0]), float(e[1])))
            else:
                axes.append(Axis(1, float(e), float(e)))
        return GridSpec(tuple(axes))

    @property
    def h(self) -> tuple[float, float, float]:
        return tuple(a.step for a in self.axes)

    @property
    def dvol(self) -> float:
        dx, dy, dz = self.h
        return dx * dy * dz

    @property
    def active_dims(self) -> list[int]:
        return [d for d in range(3) if not self.axes[d].singleton]

    def class_shape(self, c: int) -> tuple[int, int, int]:
        """(nx, ny, nz) of class c including ghost points."""
        bits = class_bits(c)
        return tuple(self.axes[d].size(bool(bits[d])) for d in range(3))

    def class_points(self, c: int) -> tuple[np.ndarray, np.ndarray, np.ndarray]:
        bits = class_bits(c)
        return tuple(self.axes[d].points(bool(bits[d])) for d in range(3))

    def class_active(self, c: int) -> bool:
        """A class odd in a singleton axis is never advanced (its interior range is empty)."""
        bits = class_bits(c)
        return all(not (bits[d] and self.axes[d].singleton) for d in range(3))

    def active_classes(self) -> list[int]:
        return [c for c in range(N_CLASSES) if self.class_active(c)]

    def n_cells(self, c: int) -> int:
        nx, ny, nz = self.class_shape(c)
        return nx * ny * nz

    def interior_ranges(self, c: int) -> tuple[range, range, range]:
        """0-based interior index ranges per axis (``eo_range``, solver_core.jl:7-19)."""
        out = []
        for d, n in enumerate(self.class_shape(c)):
            out.append(range(1, n - 1) if class_bits(c)[d] else range(0, n))
        return tuple(out)
