"""Moment basis of the P_N expansion and its split into the eight staggered-grid classes.

A moment is a real spherical harmonic ``(l, k)`` with ``0 <= l <= N`` and ``-l <= k <= l``.
Under a reflection of one axis each harmonic is either even or odd; the triple of parities
(x, y, z) selects one of eight classes, and each class lives on its own staggered grid.

Reference behaviour restated here:

* parity of ``(l, k)`` per axis -- ``pn_solver/moment_specification.jl:26-36``
* order of all moments (l ascending, then k ascending) -- ``moment_specification.jl:42-44``
* class order eee, eeo, eoe, eoo, oee, oeo, ooe, ooo (x outermost) --
  ``starmap/src/even_odd_classification.jl:19`` (``all_eos``)
* class sizes ``N_eee(N) = 1/2 floor((N+2)/2) floor((N+4)/2)`` and the shifted forms for the other
  classes -- ``pn_solver/pn_variable.jl:2-9``
* class parity (even: eee, ooe, oeo, eoo; odd: the rest) -- ``even_odd_classification.jl:73-81``
"""
from __future__ import annotations

from functools import lru_cache

# class index c = 4*ox + 2*oy + oz with o = 1 for "odd in that axis"
CLASS_NAMES = ("eee", "eeo", "eoe", "eoo", "oee", "oeo", "ooe", "ooo")
N_CLASSES = 8
EVEN_PARITY = 0
ODD_PARITY = 1


def class_index(ox: int, oy: int, oz: int) -> int:
    return 4 * ox + 2 * oy + oz


def class_bits(c: int) -> tuple[int, int, int]:
    """(ox, oy, oz) with 1 meaning odd in that axis."""
    return (c >> 2) & 1, (c >> 1) & 1, c & 1


def odd_in(c: int, dim: int) -> bool:
    return bool(class_bits(c)[dim])


def switch(c: int, dim: int) -> int:
    """Class with the parity of axis ``dim`` flipped (``switch_eo``, even_odd_classification.jl:24-26)."""
    return c ^ (4 >> dim)


def parity(c: int) -> int:
    """0 (even parity) for eee/ooe/oeo/eoo, 1 (odd parity) for oee/eoe/eeo/ooo."""
    ox, oy, oz = class_bits(c)
    return (ox + oy + oz) & 1


def classes_of_parity(p: int) -> list[int]:
    return [c for c in range(N_CLASSES) if parity(c) == p]


def moment_parity(l: int, k: int) -> tuple[int, int, int]:
    """(ox, oy, oz) of harmonic (l, k), 1 = odd.

    x: even iff (k >= 0 and k even) or (k < 0 and k odd)
    y: even iff k >= 0
    z: even iff l + k even
    """
    even_x = (k >= 0 and k % 2 == 0) or (k < 0 and k % 2 != 0)
    even_y = k >= 0
    even_z = (l + k) % 2 == 0
    return (0 if even_x else 1, 0 if even_y else 1, 0 if even_z else 1)


def moment_class(l: int, k: int) -> int:
    return class_index(*moment_parity(l, k))


def all_moments(N: int) -> list[tuple[int, int]]:
    return [(l, k) for l in range(N + 1) for k in range(-l, l + 1)]


@lru_cache(maxsize=None)
def class_moments(N: int) -> tuple[tuple[tuple[int, int], ...], ...]:
    """Moments of each class in reference order (``make_moments``, pn_variable.jl:12)."""
    out: list[list[tuple[int, int]]] = [[] for _ in range(N_CLASSES)]
    for lk in all_moments(N):
        out[moment_class(*lk)].append(lk)
    return tuple(tuple(v) for v in out)


def n_eee(N: int) -> int:
    return max(0, ((N + 2) // 2) * ((N + 4) // 2) // 2)


def class_sizes_closed_form(N: int) -> list[int]:
    """Per-class moment counts from the closed forms of pn_variable.jl:2-9."""
    return [n_eee(N), n_eee(N - 1), n_eee(N - 1), n_eee(N - 2),
            n_eee(N - 1), n_eee(N - 2), n_eee(N - 2), n_eee(N - 3)]


def class_sizes(N: int) -> list[int]:
    return [len(v) for v in class_moments(N)]


def degree_table(N: int) -> list[list[int]]:
    """Degree l of every moment of each class (used to index the per-degree coefficients)."""
    return [[l for (l, _k) in ms] for ms in class_moments(N)]
