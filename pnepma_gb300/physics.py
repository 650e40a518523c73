"""Physical data entering the solve as per-energy tables.

The reference takes these quantities from third-party packages or from a file that is not in
its tree:

* mass stopping power s_e(E) and its slope -- ICRU-77 tables, linearly interpolated
  (``pn_solver/stopping_power.jl:37-154``);
* elastic transport coefficients tc_{e,l}(E) -- ``transport_coefficient_funcs`` from
  ``pn_solver/transport_coefficient.jl``, absent from the reference tree;
* ionisation cross-sections sigma_r(E) -- NeXLCore 0.3.7 ``ionizationcrosssection`` (Bote-Salvat
  2009 via BoteSalvatICX 2.0.2) (``pn_solver/x_ray_intensities.jl:32-37``);
* mass absorption coefficients -- NeXLCore ``mac`` (FFAST) (``x_ray_intensities.jl:117``);
* element densities and atomic masses -- PeriodicTable 1.1.3.

The stopping power is the reference's own in-tree data: ``icru77.py`` restates its ICRU-77
table for the elements modelled here, and ``stopping_power_table`` converts and interpolates it
as ``stopping_power_func`` does.  The other data sets are not available here, so this module
supplies documented stand-ins with the same roles and units (cm, g, eV); every solve consumes
them as tables, so the GPU path and the oracle see identical numbers.  A caller with the real
data passes its own tables instead.

Stand-ins (labelled as such), each a published closed form:

* transport coefficients: Legendre moments of the screened-Rutherford cross-section with a
  Wentzel screening parameter eta = 3.4e-3 Z^(2/3) / E[keV]; the moments use Neumann's integral
  int P_l(mu)/(a-mu) dmu = 2 Q_l(a) (Legendre functions of the second kind);
* ionisation cross-section: Worthington-Tomlin (1956) form
  6.51e-14 n b / (U E_c^2) ln(4U / (1.65 + 2.35 e^(1-U))) cm^2 (E_c in eV), zero below the edge;
* mass absorption coefficient: Kramers-type c Z^4 / (A E^3) with a K-edge jump of 8.

Element densities are PeriodicTable's (the divisor of the stopping-power table); the line and
edge energies are tabulated values.
"""
from __future__ import annotations

import math
from dataclasses import dataclass

import numpy as np

AVOGADRO = 6.02214076e23
AMU_G = 1.66053906660e-24        # one unified atomic mass unit in g
E2_EV_CM = 1.43996448e-7         # e^2 / (4 pi eps0) in eV cm
MC2_EV = 510998.95


@dataclass(frozen=True)
class Element:
    symbol: str
    Z: int
    atomic_mass_u: float     # g/mol == u
    density: float           # g/cm^3
    k_edge_ev: float
    k_l3_ev: float           # K-alpha1 line energy
    k_l2_ev: float           # K-alpha2 line energy

    @property
    def atomic_mass_g(self) -> float:
        """Mass of one atom in g (``convert_strip_mass(el.atomic_mass)``)."""
        return self.atomic_mass_u * AMU_G


ELEMENTS = {
    "Cr": Element("Cr", 24, 51.9961, 7.19, 5989.0, 5414.72, 5405.51),
    "Fe": Element("Fe", 26, 55.845, 7.874, 7112.0, 6403.84, 6390.84),
    "Ni": Element("Ni", 28, 58.6934, 8.908, 8333.0, 7478.15, 7460.89),
    "Cu": Element("Cu", 29, 63.546, 8.96, 8979.0, 8047.78, 8027.83),
}


@dataclass(frozen=True)
class XRay:
    """A characteristic line: emitting element and transition (``K-L3`` or ``K-L2``)."""
    element: str
    transition: str = "K-L3"

    @property
    def energy(self) -> float:
        el = ELEMENTS[self.element]
        return el.k_l3_ev if self.transition == "K-L3" else el.k_l2_ev

    @property
    def edge(self) -> float:
        return ELEMENTS[self.element].k_edge_ev


# ------------------------------------------------------------------------------------------------
# stopping power
# ------------------------------------------------------------------------------------------------
def joy_luo_mass_stopping_power(el: Element, E_ev):
    """Mass stopping power in eV cm^2/g from the Bethe formula with the Joy-Luo (1989) correction.

    Not used by the solve (which takes the ICRU-77 table); kept as an independent closed form that
    the tests compare the table against."""
    E_kev = np.asarray(E_ev, dtype=float) * 1e-3
    J = (9.76 * el.Z + 58.5 * el.Z ** -0.19) * 1e-3
    k = 0.734 * el.Z ** 0.037
    s_kev = 78500.0 * el.Z / (el.atomic_mass_u * E_kev) * np.log(1.166 * (E_kev + k * J) / J)
    return s_kev * 1e3


class LinearTable:
    """Piecewise-linear interpolation on knots, with the slope of the interval holding E.

    Mirrors ``stopping_power_func`` (stopping_power.jl:41-44): Interpolations' gridded linear
    interpolant, value ``y_i (1 - t) + y_{i+1} t`` with ``t = (E - x_i) / (x_{i+1} - x_i)``, and its
    derivative by forward-mode AD, ``y_i (-r) + y_{i+1} r`` with ``r = 1 / (x_{i+1} - x_i)``.  The
    interval holding E is the last one whose left knot is <= E (right-open intervals), the last
    interval at the last knot: at an interior knot the slope is the one of the interval to its
    right.  Outside the knots the call raises, as the reference's interpolant does (its default
    extrapolation throws).
    """

    def __init__(self, knots, values):
        self.x = np.asarray(knots, dtype=float)
        self.y = np.asarray(values, dtype=float)

    def _interval(self, E):
        if not (self.x[0] <= E <= self.x[-1]):
            raise ValueError(f"energy {E} outside the tabulated range")
        i = int(np.searchsorted(self.x, E, side="right") - 1)
        return min(i, len(self.x) - 2)

    def __call__(self, E: float) -> float:
        i = self._interval(E)
        x0, x1, y0, y1 = self.x[i], self.x[i + 1], self.y[i], self.y[i + 1]
        t = (E - x0) / (x1 - x0)
        return float(y0 * (1.0 - t) + y1 * t)

    def slope(self, E: float) -> float:
        i = self._interval(E)
        r = 1.0 / (self.x[i + 1] - self.x[i])
        return float(self.y[i] * -r + self.y[i + 1] * r)


def stopping_power_table(el: Element) -> LinearTable:
    """ICRU-77 total mass stopping power of `el` in eV cm^2/g on knots in eV.

    As ``stopping_power_func`` builds it (stopping_power.jl:40-41): the energies converted MeV -> eV,
    the stopping powers MeV/cm -> eV/cm and divided by the element's density in g/cm^3."""
    from . import icru77
    if el.Z not in icru77.TOTAL_MEV_PER_CM:
        raise ValueError(f"no ICRU-77 stopping-power row for Z = {el.Z}; pass the element's table")
    knots = np.array(icru77.ENERGIES_MEV) * 1000000.0
    values = np.array(icru77.TOTAL_MEV_PER_CM[el.Z]) * 1000000.0 / el.density
    return LinearTable(knots, values)


# ------------------------------------------------------------------------------------------------
# transport coefficients (screened Rutherford)
# ------------------------------------------------------------------------------------------------
def _legendre_q_and_dq(lmax: int, a: float):
    """Q_l(a) and Q_l'(a) for a > 1, l = 0..lmax."""
    q = np.zeros(lmax + 1)
    dq = np.zeros(lmax + 1)
    q[0] = 0.5 * math.log((a + 1.0) / (a - 1.0))
    if lmax >= 1:
        q[1] = a * q[0] - 1.0
    for l in range(1, lmax):
        q[l + 1] = ((2 * l + 1) * a * q[l] - l * q[l - 1]) / (l + 1)
    dq[0] = -1.0 / (a * a - 1.0)
    for l in range(1, lmax + 1):
        dq[l] = l * (a * q[l] - q[l - 1]) / (a * a - 1.0)
    return q, dq


def transport_coefficients(el: Element, E_ev: float, N: int) -> np.ndarray:
    """tc_l(E), l = 0..N, mass-normalised Legendre moments of the elastic cross-section (cm^2/g).

    sigma_l = 2 pi K int_{-1}^{1} P_l(mu) / (1 - mu + 2 eta)^2 dmu = -4 pi K Q_l'(1 + 2 eta),
    K = Z (Z + 1) (e^2 / (p v))^2.  The solve uses tc_l - tc_0.
    """
    E_kev = E_ev * 1e-3
    eta = 3.4e-3 * el.Z ** (2.0 / 3.0) / E_kev
    pc2 = E_ev * (E_ev + 2 * MC2_EV)
    pv = pc2 / (E_ev + MC2_EV)
    K = el.Z * (el.Z + 1) * (E2_EV_CM / pv) ** 2
    _q, dq = _legendre_q_and_dq(N, 1.0 + 2.0 * eta)
    sigma = -4.0 * math.pi * K * dq
    return sigma * (AVOGADRO / el.atomic_mass_u)


# ------------------------------------------------------------------------------------------------
# ionisation cross-section and absorption
# ------------------------------------------------------------------------------------------------
def ionization_cross_section(xray: XRay, E_ev: float) -> float:
    """K-shell ionisation cross-section in cm^2 (Worthington-Tomlin form), 0 below the edge."""
    Ec = xray.edge
    U = E_ev / Ec
    if U <= 1.0:
        return 0.0
    n_s, b_s = 2.0, 0.35
    return 6.51e-14 * n_s * b_s / (U * Ec * Ec) * math.log(4.0 * U / (1.65 + 2.35 * math.exp(1.0 - U)))


def mass_absorption(xray: XRay, absorber: Element) -> float:
    """Mass absorption coefficient of the line in the absorber, cm^2/g."""
    E_kev = xray.energy * 1e-3
    mu = 2.48 * absorber.Z ** 4 / (absorber.atomic_mass_u * E_kev ** 3)
    if xray.energy > absorber.k_edge_ev:
        mu *= 8.0
    return mu


def normal_cdf(x: float, mean: float, std: float) -> float:
    """cdf of Normal(mean, std), erfc form."""
    return 0.5 * math.erfc(-(x - mean) / (std * math.sqrt(2.0)))
