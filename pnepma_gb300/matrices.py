"""Moment-coupling (advection) and boundary matrices of the P_N system, and the beam moments.

Advection blocks ``A_d[c]`` couple the moments of class ``c`` to the moments of ``switch(c, d)``:
``A_d[i, j] = int_{S^2} Omega_d Y_i Y_j dOmega`` for real orthonormal harmonics.  Only degrees
``l' = l +- 1`` couple.  The values follow the three-term recurrences of the real harmonics in
the form the reference writes them (``pn_solver/pn_matrices.jl:1-152``): every coefficient is a
square root of a ratio of small integers evaluated in IEEE double, so the values here are
bit-identical to the reference's.

Boundary blocks ``B_d[c] = L_d[c] @ A_d[c]`` (forward) and ``-L_d[c]^T @ A_d[c]`` (adjoint) act on
the ghost layer of each class odd in ``d`` (``pn_matrices.jl:191-293``).  ``L`` is a double sum of
gamma-function and factorial ratios.  For moment pairs of one class every gamma argument is a
positive integer or half-integer, so each entry equals ``q * sqrt(r)`` with rationals ``q, r``;
it is evaluated exactly here (``fractions``) and rounded once to double.  The reference evaluates
the same expression in a BigFloat/Float64 mix, so entries may differ from it in the last bits.

Beam moments ``-int Y_lk(Omega) vMF(Omega; mu, kappa) dOmega`` (``pn_matrices.jl:331-338``) are
computed with a tensor Gauss-Legendre rule in (theta, phi) that resolves the von Mises-Fisher
peak to ~1e-14; the reference uses adaptive cubature with its default tolerance (~1.5e-8).
"""
from __future__ import annotations

import math
from decimal import Decimal, getcontext
from fractions import Fraction
from functools import lru_cache

import numpy as np

from .moments import N_CLASSES, class_moments, odd_in, switch

X, Y, Z = 0, 1, 2


# ----------------------------------------------------------------------------------------------
# advection coefficients (closed form; pn_matrices.jl:2-144)
# ----------------------------------------------------------------------------------------------
def _sgn_step(k: int) -> int:
    # Theta(k): -1 for k < 0, +1 for k >= 0
    return -1 if k < 0 else 1


def _up(k: int) -> int:
    # order one further away from zero (0 -> 1)
    return 1 if k == 0 else k + (1 if k > 0 else -1)


def _down(k: int) -> int:
    # order one closer to zero (0 -> -1)
    return -1 if k == 0 else k - (1 if k > 0 else -1)


def _ratio_sqrt(num: int, den: int) -> float:
    # Julia evaluates Int/Int as Float64(num)/Float64(den) then sqrt; both exact for small ints
    return math.sqrt(float(num) / float(den))


def _ca(k, l):
    return _ratio_sqrt((l - k + 1) * (l + k + 1), (2 * l + 3) * (2 * l + 1))


def _cb(k, l):
    return _ratio_sqrt((l - k) * (l + k), (2 * l + 1) * (2 * l - 1))


def _cc(k, l):
    v = _ratio_sqrt((l + k + 1) * (l + k + 2), (2 * l + 3) * (2 * l + 1))
    if k < 0:
        return 0.0
    return v if k > 0 else v * math.sqrt(2.0)


def _cd(k, l):
    v = _ratio_sqrt((l - k) * (l - k - 1), (2 * l + 1) * (2 * l - 1))
    if k < 0:
        return 0.0
    return v if k > 0 else v * math.sqrt(2.0)


def _ce(k, l):
    v = _ratio_sqrt((l - k + 1) * (l - k + 2), (2 * l + 3) * (2 * l + 1))
    if k == 1:
        return v * math.sqrt(2.0)
    if k > 1:
        return v
    raise ValueError("order below 1 in the e-coefficient")


def _cf(k, l):
    v = _ratio_sqrt((l + k) * (l + k - 1), (2 * l + 1) * (2 * l - 1))
    if k == 1:
        return v * math.sqrt(2.0)
    if k > 1:
        return v
    raise ValueError("order below 1 in the f-coefficient")


def _coupling_down(l, k, kp, dim):
    """Coefficient of moment (l-1, kp) in Omega_dim * Y_lk, written for target (l, k)."""
    if dim == X:
        if kp == _down(k) and k != -1:
            return 0.5 * _cc(abs(k) - 1, l - 1)
        if kp == _up(k):
            return -0.5 * _ce(abs(k) + 1, l - 1)
        return 0.0
    if dim == Y:
        if kp == -_down(k) and k != 1:
            return (-_sgn_step(k) / 2) * _cc(abs(k) - 1, l - 1)
        if kp == -_up(k):
            return (-_sgn_step(k) / 2) * _ce(abs(k) + 1, l - 1)
        return 0.0
    return _ca(k, l - 1) if kp == k else 0.0


def _coupling_up(l, k, kp, dim):
    """Coefficient of moment (l+1, kp) for target (l, k)."""
    if dim == X:
        if kp == _down(k) and k != -1:
            return -0.5 * _cd(abs(k) - 1, l + 1)
        if kp == _up(k):
            return 0.5 * _cf(abs(k) + 1, l + 1)
        return 0.0
    if dim == Y:
        if kp == -_down(k) and k != 1:
            return (_sgn_step(k) / 2) * _cd(abs(k) - 1, l + 1)
        if kp == -_up(k):
            return (_sgn_step(k) / 2) * _cf(abs(k) + 1, l + 1)
        return 0.0
    return _cb(k, l + 1) if kp == k else 0.0


def coupling(m_to, m_from, dim) -> float:
    l, k = m_to
    lp, kp = m_from
    if l == lp - 1:
        return _coupling_up(l, k, kp, dim)
    if l == lp + 1:
        return _coupling_down(l, k, kp, dim)
    return 0.0


@lru_cache(maxsize=None)
def _advection_block_cached(N: int, c: int, dim: int) -> bytes:
    ms = class_moments(N)
    to, fr = ms[c], ms[switch(c, dim)]
    A = np.zeros((len(to), len(fr)))
    for i, mt in enumerate(to):
        for j, mf in enumerate(fr):
            A[i, j] = coupling(mt, mf, dim)
    return A.tobytes()


def advection_block(N: int, c: int, dim: int) -> np.ndarray:
    """Dense ``A_dim[c]`` of shape (n_c, n_switch(c,dim)) (``make_advection_matrix``)."""
    ms = class_moments(N)
    A = np.frombuffer(_advection_block_cached(N, c, dim), dtype=np.float64)
    return A.reshape(len(ms[c]), len(ms[switch(c, dim)])).copy()


def advection_blocks(N: int) -> list[list[np.ndarray]]:
    """``[dim][class]`` dense advection blocks."""
    return [[advection_block(N, c, d) for c in range(N_CLASSES)] for d in range(3)]


# ----------------------------------------------------------------------------------------------
# boundary coefficients (pn_matrices.jl:191-275), exact evaluation
# ----------------------------------------------------------------------------------------------
class _Alg:
    """Exact value q * pi^(p/2) with rational q (p an integer)."""
    __slots__ = ("q", "p")

    def __init__(self, q, p=0):
        self.q = Fraction(q)
        self.p = p

    def __mul__(self, o):
        if isinstance(o, _Alg):
            return _Alg(self.q * o.q, self.p + o.p)
        return _Alg(self.q * Fraction(o), self.p)

    __rmul__ = __mul__

    def __truediv__(self, o):
        if isinstance(o, _Alg):
            return _Alg(self.q / o.q, self.p - o.p)
        return _Alg(self.q / Fraction(o), self.p)


def _gamma_exact(two_x: int) -> _Alg:
    """Gamma(two_x / 2) for positive integer two_x, exactly."""
    if two_x <= 0:
        raise ValueError("gamma pole in a boundary coefficient")
    if two_x % 2 == 0:
        return _Alg(math.factorial(two_x // 2 - 1), 0)
    n = (two_x - 1) // 2  # Gamma(n + 1/2) = (2n)! / (4^n n!) sqrt(pi)
    return _Alg(Fraction(math.factorial(2 * n), 4 ** n * math.factorial(n)), 1)


def _dfact(n: int) -> int:
    if n < 0:
        return 1
    r = 1
    while n > 1:
        r *= n
        n -= 2
    return r


def _sum_alg(terms: list[_Alg]) -> _Alg:
    terms = [t for t in terms if t.q != 0]
    if not terms:
        return _Alg(0, 0)
    p = terms[0].p
    if any(t.p != p for t in terms):
        raise ValueError("mixed powers of pi in one boundary sum")
    return _Alg(sum((t.q for t in terms), Fraction(0)), p)


def _norm_sq(l: int, k: int) -> Fraction:
    # C(l,k)^2 * 2 pi = (2l+1) (l-|k|)! / (l+|k|)!
    return Fraction((2 * l + 1) * math.factorial(l - abs(k)), math.factorial(l + abs(k)))


def _boundary_coefficient_parts(m1, m2, dim):
    """Return (q, r) with L = q * sqrt(r), exactly; r may be 1."""
    l, k = m1
    lp, kp = m2
    ak, akp = abs(k), abs(kp)
    # C(l,|k|) C(l',|k'|) = s * sqrt(norm) / (2 pi) with sign s = (-1)^|k| (-1)^|k'|
    sgnC = (-1) ** (ak % 2) * (-1) ** (akp % 2)
    nrm = _norm_sq(l, ak) * _norm_sq(lp, akp)
    if dim == Z:
        if k != kp:
            return Fraction(0), Fraction(1)
        terms = []
        for j in range(0, (l - ak) // 2 + 1):
            for q in range(0, (lp - akp) // 2 + 1):
                coef = Fraction(1, (-2) ** (q + j) * math.factorial(q) * math.factorial(j))
                coef *= Fraction(_dfact(2 * (l - j) - 1), math.factorial(l - ak - 2 * j))
                coef *= Fraction(_dfact(2 * (lp - q) - 1), math.factorial(lp - akp - 2 * q))
                g = _gamma_exact(l + lp - 2 * q - 2 * j - 2 * ak) / _gamma_exact(l + lp + 2 - 2 * q - 2 * j)
                terms.append(g * coef)
        s = _sum_alg(terms)
        if s.q == 0:
            return Fraction(0), Fraction(1)
        # result = s * pi * C C * |k|! ; C C = sgnC sqrt(nrm)/(2 pi)
        if s.p != 0:
            raise ValueError("unexpected power of pi")
        return s.q * math.factorial(ak) * sgnC / 2, nrm
    # X or Y
    if (l + lp) % 2 == 1:
        return Fraction(0), Fraction(1)
    terms = []
    for j in range(0, (l - ak) // 2 + 1):
        for q in range(0, (lp - akp) // 2 + 1):
            inner = []
            for i in range(0, (ak - 1) // 2 + 1 if ak >= 1 else 0):
                for s_ in range(0, (akp - 1) // 2 + 1 if akp >= 1 else 0):
                    sign = (-1) ** (s_ + i)
                    if dim == X:
                        if k >= 0 and kp >= 0 and k % 2 == 1 and kp % 2 == 1:
                            t = (_gamma_exact(1 + 2 * (s_ + i)) * _gamma_exact(k + kp - 2 * (s_ + i))
                                 * (sign * math.comb(k, 2 * i) * math.comb(kp, 2 * s_)))
                            inner.append(t)
                        elif k < 0 and kp < 0 and k % 2 == 0 and kp % 2 == 0:
                            t = (_gamma_exact(3 + 2 * (s_ + i)) * _gamma_exact(ak + akp - 2 * (s_ + i) - 2)
                                 * (sign * math.comb(ak, 2 * i + 1) * math.comb(akp, 2 * s_ + 1)))
                            inner.append(t)
                    else:
                        t = (_gamma_exact(ak + akp - 2 * s_ - 2 * i - 1)
                             * (sign * math.factorial(s_ + i) * math.comb(ak, 2 * i + 1) * math.comb(akp, 2 * s_ + 1)))
                        inner.append(t)
            sis = _sum_alg(inner)
            if sis.q == 0:
                continue
            coef = Fraction((-1) ** (q + j), 2 ** (j + q) * math.factorial(j) * math.factorial(q))
            coef *= Fraction(_dfact(2 * (l - j) - 1), math.factorial(l - ak - 2 * j))
            coef *= Fraction(_dfact(2 * (lp - q) - 1), math.factorial(lp - akp - 2 * q))
            g = _gamma_exact(l + lp + 1 - 2 * (q + j) - (ak + akp)) / _gamma_exact(l + lp + 2 - 2 * (q + j))
            terms.append(sis * g * coef)
    s = _sum_alg(terms)
    if s.q == 0:
        return Fraction(0), Fraction(1)
    if s.p != 2:
        raise ValueError("unexpected power of pi")
    # result = C C (1 + (-1)^(l+l')) (-1)^(|k|+|k'|) s ; s = s.q * pi ; C C = sgnC sqrt(nrm) / (2 pi)
    sign2 = (-1) ** ((ak + akp) % 2)
    return s.q * sgnC * sign2 * 2 / 2, nrm


def _to_float(q: Fraction, r: Fraction) -> float:
    if q == 0:
        return 0.0
    getcontext().prec = 60
    v = (Decimal(q.numerator) / Decimal(q.denominator)) * (Decimal(r.numerator) / Decimal(r.denominator)).sqrt()
    return float(v)


@lru_cache(maxsize=None)
def boundary_coefficient(m1: tuple, m2: tuple, dim: int) -> float:
    q, r = _boundary_coefficient_parts(m1, m2, dim)
    return _to_float(q, r)


def boundary_L(N: int, c: int, dim: int) -> np.ndarray:
    ms = class_moments(N)[c]
    L = np.zeros((len(ms), len(ms)))
    for i, a in enumerate(ms):
        for j, b in enumerate(ms):
            L[i, j] = boundary_coefficient(a, b, dim)
    return L


def _matmul_ordered(L: np.ndarray, A: np.ndarray) -> np.ndarray:
    """Double-precision product with a fixed left-to-right summation order."""
    n, m = L.shape[0], A.shape[1]
    out = np.zeros((n, m))
    for i in range(n):
        for j in range(m):
            acc = 0.0
            for k in range(L.shape[1]):
                acc += float(L[i, k]) * float(A[k, j])
            out[i, j] = acc
    return out


@lru_cache(maxsize=None)
def _boundary_block_cached(N: int, c: int, dim: int, adjoint: bool) -> bytes:
    L = boundary_L(N, c, dim)
    A = advection_block(N, c, dim)
    B = -_matmul_ordered(L.T.copy(), A) if adjoint else _matmul_ordered(L, A)
    return B.tobytes()


def boundary_block(N: int, c: int, dim: int, adjoint: bool = False) -> np.ndarray:
    """``L @ A`` (forward) or ``-L^T @ A`` (adjoint) for a class odd in ``dim``."""
    if not odd_in(c, dim):
        raise ValueError("boundary blocks exist only for classes odd in the boundary axis")
    ms = class_moments(N)
    B = np.frombuffer(_boundary_block_cached(N, c, dim, bool(adjoint)), dtype=np.float64)
    return B.reshape(len(ms[c]), len(ms[switch(c, dim)])).copy()


def boundary_blocks(N: int, adjoint: bool = False) -> list[list[np.ndarray | None]]:
    """``[dim][class]`` boundary blocks (None for classes even in that axis)."""
    return [[boundary_block(N, c, d, adjoint) if odd_in(c, d) else None for c in range(N_CLASSES)]
            for d in range(3)]


# ----------------------------------------------------------------------------------------------
# real spherical harmonics and beam moments
# ----------------------------------------------------------------------------------------------
def real_harmonics(N: int, theta: np.ndarray, phi: np.ndarray) -> dict:
    """Orthonormal real harmonics Y_lk(theta, phi) without the Condon-Shortley phase.

    Y_l0 = Nbar_l0 P_l(cos t); Y_lk (k>0) = sqrt2 Nbar_lk P_l^k cos(k phi);
    Y_lk (k<0) = sqrt2 Nbar_l|k| P_l^|k| sin(|k| phi), with P_l^m >= 0 near the pole for m = l.
    This is the convention under which the closed-form advection blocks equal
    int Omega_d Y_i Y_j (checked by quadrature in the tests).
    """
    mu = np.cos(theta)
    s = np.sin(theta)
    # normalised associated Legendre functions by the standard stable recurrences
    P = {}
    pmm = np.full_like(mu, math.sqrt(1.0 / (4 * math.pi)))
    for m in range(0, N + 1):
        if m > 0:
            pmm = pmm * s * math.sqrt((2 * m + 1) / (2 * m))
        P[(m, m)] = pmm
        if m + 1 <= N:
            P[(m + 1, m)] = mu * math.sqrt(2 * m + 3) * pmm
        for l in range(m + 2, N + 1):
            a = math.sqrt((4 * l * l - 1) / (l * l - m * m))
            b = math.sqrt(((l - 1) ** 2 - m * m) / (4 * (l - 1) ** 2 - 1))
            P[(l, m)] = a * (mu * P[(l - 1, m)] - b * P[(l - 2, m)])
    out = {}
    for l in range(N + 1):
        for k in range(-l, l + 1):
            if k == 0:
                out[(l, k)] = P[(l, 0)]
            elif k > 0:
                out[(l, k)] = math.sqrt(2.0) * P[(l, k)] * np.cos(k * phi)
            else:
                out[(l, k)] = math.sqrt(2.0) * P[(l, -k)] * np.sin(-k * phi)
    return out


def sphere_rule(n_theta: int, n_phi: int):
    """Gauss-Legendre in cos(theta) times the trapezoid rule in phi (exact for harmonics)."""
    x, w = np.polynomial.legendre.leggauss(n_theta)
    theta = np.arccos(x)
    phi = (np.arange(n_phi) + 0.5) * (2 * math.pi / n_phi)
    T, P = np.meshgrid(theta, phi, indexing="ij")
    W = np.outer(w, np.full(n_phi, 2 * math.pi / n_phi))
    return T.ravel(), P.ravel(), W.ravel()


def vmf_pdf(direction: np.ndarray, mu_dir, kappa: float) -> np.ndarray:
    """von Mises-Fisher density on S^2: kappa / (4 pi sinh kappa) exp(kappa mu.x)."""
    mu_dir = np.asarray(mu_dir, dtype=float)
    mu_dir = mu_dir / np.linalg.norm(mu_dir)
    dot = direction @ mu_dir
    # kappa/(4 pi sinh k) exp(k dot) = kappa / (2 pi (1 - exp(-2k))) exp(k (dot - 1))
    return kappa / (2 * math.pi * (-math.expm1(-2 * kappa))) * np.exp(kappa * (dot - 1.0))


def beam_moments(moments, mu_dir, kappa: float, n_theta: int = 200, n_phi: int = 400) -> np.ndarray:
    """``-int Y_m(Omega) vMF(Omega) dOmega`` for each moment (``beam_moments``, pn_matrices.jl:331-338)."""
    key = (tuple(tuple(m) for m in moments), tuple(float(v) for v in mu_dir), float(kappa), n_theta, n_phi)
    hit = _BEAM_CACHE.get(key)
    if hit is None:
        hit = _beam_moments(moments, mu_dir, kappa, n_theta, n_phi)
        _BEAM_CACHE[key] = hit
    return hit.copy()


_BEAM_CACHE: dict = {}


def _beam_moments(moments, mu_dir, kappa, n_theta, n_phi):
    if not moments:
        return np.zeros(0)
    N = max(l for (l, _k) in moments)
    # split theta at pi/2 and phi at the peak so the rule resolves the peak on both sides
    T, P, W = _peak_rule(mu_dir, kappa, n_theta, n_phi)
    d = np.stack([np.sin(T) * np.cos(P), np.sin(T) * np.sin(P), np.cos(T)], axis=1)
    f = vmf_pdf(d, mu_dir, kappa) * W
    Ys = real_harmonics(N, T, P)
    return np.array([-float(np.sum(Ys[m] * f)) for m in moments])


def _peak_rule(mu_dir, kappa, n_theta, n_phi):
    # Gauss-Legendre in theta on [0, pi] (in theta, with the sin(theta) weight) split at the
    # polar angle of the peak, and Gauss-Legendre in phi split at the azimuth of the peak.
    mu_dir = np.asarray(mu_dir, dtype=float) / np.linalg.norm(mu_dir)
    th0 = math.acos(max(-1.0, min(1.0, mu_dir[2])))
    ph0 = math.atan2(mu_dir[1], mu_dir[0]) % (2 * math.pi)

    def gl(a, b, n):
        x, w = np.polynomial.legendre.leggauss(n)
        return 0.5 * (b - a) * x + 0.5 * (b + a), 0.5 * (b - a) * w

    ts, tw = [], []
    for a, b in ((0.0, th0), (th0, math.pi)):
        if b - a > 1e-12:
            t, w = gl(a, b, n_theta // 2)
            ts.append(t)
            tw.append(w)
    ps, pw = [], []
    for a, b in ((0.0, ph0), (ph0, 2 * math.pi)):
        if b - a > 1e-12:
            p, w = gl(a, b, n_phi // 2)
            ps.append(p)
            pw.append(w)
    t = np.concatenate(ts)
    wt = np.concatenate(tw) * np.sin(t)
    p = np.concatenate(ps)
    wp = np.concatenate(pw)
    T, P = np.meshgrid(t, p, indexing="ij")
    W = np.outer(wt, wp)
    return T.ravel(), P.ravel(), W.ravel()
