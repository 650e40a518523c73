"""Second CPU restatement of the reference march and its adjoint, in vectorised numpy (test
infrastructure only).

Written independently of ``pn_oracle.c``: whole classes are advanced with array slicing and
``einsum`` instead of per-cell loops, so a mistake in one restatement does not repeat in the other.
It follows the same reference code -- ``starmap/src/solver.jl:107-196`` (boundary, sub-steps),
``solver_core.jl:7-137`` (stencil, right-hand side, expm1div), ``boundary_conditions.jl:67-102``,
``pn_problem.jl:205-249`` (coefficients, source), ``pn_intensities.jl:325-351`` (intensities),
``pn_intensities.jl:129-164,353-413`` and ``x_ray_intensities.jl:155-223`` (the adjoint) --
and the state layout of the C ABI (per class [z][y][x][moment], classes concatenated).  The
tests compare the two restatements, including ghost and corner points, on small grids.
"""
from __future__ import annotations

import numpy as np


def _bit(c, d):
    return (c >> (2 - d)) & 1


def _sw(c, d):
    return c ^ (4 >> d)


class Geometry:
    def __init__(self, desc):
        from pnepma_gb300.moments import class_sizes_closed_form
        self.N = desc.order
        self.ne = desc.n_elements
        self.nr = desc.n_xrays
        self.ns = desc.n_steps
        self.M = [desc.n_points[d] for d in range(3)]
        self.h = [desc.h[d] for d in range(3)]
        self.nm = class_sizes_closed_form(self.N)
        self.shape = []
        for c in range(8):
            sh = []
            for d in range(3):
                if self.M[d] == 1:
                    sh.append(1)
                else:
                    sh.append(self.M[d] + 1 if _bit(c, d) else self.M[d])
            self.shape.append(tuple(sh))   # (nx, ny, nz)
        # blocks
        self.A = [[None] * 8 for _ in range(3)]
        self.Bf = [[None] * 8 for _ in range(3)]
        self.Ba = [[None] * 8 for _ in range(3)]
        off = bo = 0
        adv = np.ctypeslib.as_array(desc.advection, shape=(self._n_adv(),))
        nb = self._n_bnd()
        bf = np.ctypeslib.as_array(desc.boundary_fwd, shape=(nb,))
        ba = np.ctypeslib.as_array(desc.boundary_adj, shape=(nb,))
        for d in range(3):
            for c in range(8):
                r, k = self.nm[c], self.nm[_sw(c, d)]
                self.A[d][c] = adv[off:off + r * k].reshape(r, k)
                off += r * k
                if _bit(c, d):
                    self.Bf[d][c] = bf[bo:bo + r * k].reshape(r, k)
                    self.Ba[d][c] = ba[bo:bo + r * k].reshape(r, k)
                    bo += r * k
        nbeam = sum(self.shape[c][1] * self.shape[c][2] * self.nm[c] for c in (4, 5, 6, 7))
        beam = np.ctypeslib.as_array(desc.beam_face, shape=(max(nbeam, 1),))
        self.gx = {}
        o = 0
        for c in (4, 5, 6, 7):
            n = self.shape[c][1] * self.shape[c][2] * self.nm[c]
            self.gx[c] = beam[o:o + n].reshape(self.shape[c][2], self.shape[c][1], self.nm[c])
            o += n

    def _n_adv(self):
        return sum(self.nm[c] * self.nm[_sw(c, d)] for d in range(3) for c in range(8))

    def _n_bnd(self):
        return sum(self.nm[c] * self.nm[_sw(c, d)] for d in range(3) for c in range(8) if _bit(c, d))

    def split(self, flat, per_point):
        """Flat caller layout -> list of arrays [z][y][x][v] per class."""
        out, o = [], 0
        for c in range(8):
            nx, ny, nz = self.shape[c]
            v = per_point(c)
            n = nx * ny * nz * v
            out.append(flat[o:o + n].reshape(nz, ny, nx, v).copy())
            o += n
        return out


def _axis(d):
    # array axes are [z, y, x, m]
    return 2 - d


def _interior(g, c):
    """Slices of the interior points of class c (eo_range)."""
    sl = []
    for d in (2, 1, 0):   # z, y, x order of array axes
        n = g.shape[c][d]
        sl.append(slice(1, n - 1) if _bit(c, d) else slice(0, n))
    return tuple(sl)


def apply_boundary(g, u, parity, adjoint, bc):
    for d in range(3):
        if g.M[d] == 1:
            continue
        for c in range(8):
            if not _bit(c, d) or ((_bit(c, 0) + _bit(c, 1) + _bit(c, 2)) & 1) != parity:
                continue
            v = u[_sw(c, d)]
            B = g.Ba[d][c] if adjoint else g.Bf[d][c]
            ax = _axis(d)
            n = g.shape[c][d]
            U = u[c]

            def take(arr, i):
                idx = [slice(None)] * 4
                idx[ax] = i
                return arr[tuple(idx)]

            def put(arr, i, val):
                idx = [slice(None)] * 4
                idx[ax] = i
                arr[tuple(idx)] = val

            Bv_left = np.einsum("mn,...n->...m", B, take(v, 0))
            Bv_right = np.einsum("mn,...n->...m", B, take(v, n - 2))
            source = (not adjoint) and d == 0
            if source:
                put(U, 0, 2.0 * (-Bv_left + 0.0) - take(U, 1))
                g_right = g.gx[c] * bc   # [z][y][m] on the x face
                put(U, n - 1, 2.0 * (Bv_right + g_right) - take(U, n - 2))
            else:
                put(U, 0, -2.0 * Bv_left - take(U, 1))
                put(U, n - 1, 2.0 * Bv_right - take(U, n - 2))


def expm1div(c):
    small = np.abs(c) <= 0.0002
    with np.errstate(divide="ignore", invalid="ignore"):
        big = (np.exp(c) - 1.0) / c
    return np.where(small, 1.0 + 0.5 * c + 1.0 / 6.0 * (c * c), big)


def calc_du(g, u, rho, s, cdeg, Q, parity, dt, use_exp, adjoint):
    from pnepma_gb300.moments import degree_table
    degs = degree_table(g.N)
    du = {}
    for c in range(8):
        if ((_bit(c, 0) + _bit(c, 1) + _bit(c, 2)) & 1) != parity:
            continue
        inner = _interior(g, c)
        if any(sl.stop is not None and sl.start >= sl.stop for sl in inner):
            continue
        if g.nm[c] == 0:
            continue
        acc = np.zeros(u[c][inner].shape)
        for d in range(3):
            if g.shape[c][d] == 1:
                continue
            f = u[_sw(c, d)]
            ax = _axis(d)
            # neighbour slices: other axes as the target's interior; along d the two neighbours
            if _bit(c, d):   # odd target io reads even io (right) and io - 1 (left)
                right = list(inner)
                right[ax] = slice(1, g.shape[c][d] - 1)
                left = list(inner)
                left[ax] = slice(0, g.shape[c][d] - 2)
            else:            # even target ie reads odd ie + 1 (right) and ie (left)
                right = list(inner)
                right[ax] = slice(1, g.shape[c][d] + 1)
                left = list(inner)
                left[ax] = slice(0, g.shape[c][d])
            diff = (f[tuple(right)] - f[tuple(left)]) / g.h[d]
            A = -g.A[d][c] if adjoint else g.A[d][c]
            acc = acc + np.einsum("mn,...n->...m", A, diff)
        r = rho[c][inner]                                   # [...][e]
        S = np.einsum("...e,e->...", r, s)[..., None]
        C = np.einsum("...e,el->...l", r, cdeg)[..., degs[c]]
        U = u[c][inner]
        q = Q[c][inner] if Q is not None else 0.0
        num = (q - acc) - C * U
        if use_exp:
            du[c] = num / S * expm1div(-C / S * dt)
        else:
            du[c] = num / S
    return du


def step(g, u, rho, s, cdeg, bc, dt, adjoint=False, Q=None):
    def half(parity, h):
        du = calc_du(g, u, rho, s, cdeg, Q, parity, h, True, adjoint)
        for c, v in du.items():
            u[c][_interior(g, c)] += h * v

    apply_boundary(g, u, 0, adjoint, bc)
    half(1, dt / 2)
    apply_boundary(g, u, 1, adjoint, bc)
    half(0, dt)
    apply_boundary(g, u, 0, adjoint, bc)
    half(1, dt / 2)


def forward(desc, rho_flat, noa, acs, return_state=False, tape=None):
    """Intensities of the forward march (pn_intensities.jl:325-351); with a list as ``tape``, every
    state of the march (initial state first) is appended to it."""
    g = Geometry(desc)
    N1 = g.N + 1
    rho = g.split(np.asarray(rho_flat, float), lambda c: g.ne)
    u = [np.zeros((sh[2], sh[1], sh[0], g.nm[c])) for c, sh in enumerate(g.shape)]
    fs = np.ctypeslib.as_array(desc.fwd_s, shape=(g.ns * g.ne,)).reshape(g.ns, g.ne)
    fc = np.ctypeslib.as_array(desc.fwd_c, shape=(g.ns * g.ne * N1,)).reshape(g.ns, g.ne, N1)
    fbc = np.ctypeslib.as_array(desc.fwd_bc, shape=(g.ns,))
    sig = np.ctypeslib.as_array(desc.fwd_sigma, shape=((g.ns + 1) * g.nr,)).reshape(g.ns + 1, g.nr)
    w = np.ctypeslib.as_array(desc.fwd_weight, shape=(g.ns + 1,))
    xel = np.ctypeslib.as_array(desc.xray_element, shape=(g.nr,))
    W = np.asarray(acs).reshape(-1, g.nr) * np.asarray(noa).reshape(-1, g.ne)[:, xel]
    I = np.zeros(g.nr)
    for i in range(g.ns + 1):
        if i > 0:
            step(g, u, rho, fs[i - 1], fc[i - 1], fbc[i - 1], desc.delta_e)
        if tape is not None:
            tape.append([x.copy() for x in u])
        integral = W.T @ u[0][..., 0].ravel()
        I = I + desc.delta_e * desc.dvol * sig[i] * integral * w[i]
    if return_state:
        return I, np.concatenate([x.ravel() for x in u])
    return I


def one_step(desc, rho_flat, state_flat, i):
    g = Geometry(desc)
    N1 = g.N + 1
    rho = g.split(np.asarray(rho_flat, float), lambda c: g.ne)
    u = g.split(np.asarray(state_flat, float), lambda c: g.nm[c])
    fs = np.ctypeslib.as_array(desc.fwd_s, shape=(g.ns * g.ne,)).reshape(g.ns, g.ne)
    fc = np.ctypeslib.as_array(desc.fwd_c, shape=(g.ns * g.ne * N1,)).reshape(g.ns, g.ne, N1)
    fbc = np.ctypeslib.as_array(desc.fwd_bc, shape=(g.ns,))
    step(g, u, rho, fs[i], fc[i], fbc[i], desc.delta_e)
    return np.concatenate([x.ravel() for x in u])


def adjoint(desc, rho_flat, noa, acs, Ibar):
    """(I, rho_bar, noa_bar, acs_bar) of the reference's adjoint (pn_intensities.jl:353-413),
    written independently of pn_oracle.c.  Iteration j = 0..n_steps takes tape state n_steps - j
    (the initial state last) and, as the reference's pullback loop does:

    * integrate_adjoint_densities! (pn_intensities.jl:129-164): the forward problem at the tape
      energy sets the tape state's ghost points (both parities, beam source included), du of every
      class without the exponential factor, and rho_bar += lambda . (s_e du + c_{e,l} u) dvol dE w;
    * integrate_step_and_add_pullback! (x_ray_intensities.jl:196-223): the cotangents of the
      absorption factors and numbers of atoms from the eee cells' first moment;
    * for j < n_steps, compute_adjoint_source! at E + dE/2 (x_ray_intensities.jl:155-170) and one
      step of the adjoint problem (its coefficients at E + dE/2, zero boundary source).
    """
    from pnepma_gb300.moments import degree_table
    g = Geometry(desc)
    N1, ne, nr, ns = g.N + 1, g.ne, g.nr, g.ns
    dE = desc.delta_e
    rho = g.split(np.asarray(rho_flat, float), lambda c: ne)
    tape = []
    I = forward(desc, rho_flat, noa, acs, tape=tape)
    arr = lambda p, n: np.ctypeslib.as_array(p, shape=(n,))
    ais = arr(desc.adj_int_s, (ns + 1) * ne).reshape(ns + 1, ne)
    aic = arr(desc.adj_int_c, (ns + 1) * ne * N1).reshape(ns + 1, ne, N1)
    aibc = arr(desc.adj_int_bc, ns + 1)
    asig = arr(desc.adj_sigma, (ns + 1) * nr).reshape(ns + 1, nr)
    aw = arr(desc.adj_weight, ns + 1)
    asrc = arr(desc.adj_src_sigma, max(ns * nr, 1))[:ns * nr].reshape(ns, nr)
    as_ = arr(desc.adj_s, ns * ne).reshape(ns, ne)
    ac = arr(desc.adj_c, ns * ne * N1).reshape(ns, ne, N1)
    xel = arr(desc.xray_element, nr)
    noa2 = np.asarray(noa, float).reshape(-1, ne)
    acs2 = np.asarray(acs, float).reshape(-1, nr)
    Ib = np.asarray(Ibar, float)
    degs = degree_table(g.N)
    lam = [np.zeros_like(x) for x in tape[0]]
    rho_bar = [np.zeros(x.shape[:3] + (ne,)) for x in tape[0]]
    noa_bar = np.zeros_like(noa2)
    acs_bar = np.zeros_like(acs2)
    for j in range(ns + 1):
        u = [x.copy() for x in tape[ns - j]]
        apply_boundary(g, u, 0, False, aibc[j])
        apply_boundary(g, u, 1, False, aibc[j])
        du = calc_du(g, u, rho, ais[j], aic[j], None, 0, dE, False, False)
        du.update(calc_du(g, u, rho, ais[j], aic[j], None, 1, dE, False, False))
        fac = desc.dvol * dE * aw[j]
        for c, d in du.items():
            inner = _interior(g, c)
            lc, uc = lam[c][inner], u[c][inner]
            P = np.einsum("...m,...m->...", lc, d)                        # sum_m lambda_m du_m
            R = np.einsum("...m,em->...e", lc * uc, aic[j][:, degs[c]])   # sum_m lambda_m c_{e,l(m)} u_m
            rho_bar[c][inner] += (P[..., None] * ais[j][None, :] + R) * fac
        u0 = u[0][..., 0].ravel()
        w = dE * desc.dvol * asig[j] * aw[j] * Ib                               # [r]
        acs_bar += noa2[:, xel] * u0[:, None] * w[None, :]
        for r in range(nr):
            noa_bar[:, xel[r]] += acs2[:, r] * u0 * w[r]
        if j == ns:
            break
        Q = [np.zeros_like(x) for x in lam]
        Q[0][..., 0] = -(acs2 * noa2[:, xel] * asrc[j][None, :] * Ib[None, :]).sum(axis=1).reshape(Q[0].shape[:3])
        step(g, lam, rho, as_[j], ac[j], 0.0, dE, adjoint=True, Q=Q)
    return I, np.concatenate([x.ravel() for x in rho_bar]), noa_bar, acs_bar


def generation_field(desc, rho_flat):
    """calc_x_ray_generation_field (pn_intensities.jl:189-212 with
    integrate_step_and_add_x_ray_generation!, x_ray_intensities.jl:226-234): per eee cell and line,
    the sum over the states of the forward march of u_eee[cell, 0] dE sigma_r(E) w."""
    g = Geometry(desc)
    nr, ns = g.nr, g.ns
    tape = []
    ncell = g.shape[0][0] * g.shape[0][1] * g.shape[0][2]
    forward(desc, rho_flat, np.zeros(ncell * g.ne), np.zeros(ncell * max(nr, 1)), tape=tape)
    sig = np.ctypeslib.as_array(desc.fwd_sigma, shape=((ns + 1) * nr,)).reshape(ns + 1, nr)
    w = np.ctypeslib.as_array(desc.fwd_weight, shape=(ns + 1,))
    field = np.zeros((ncell, nr))
    for i, u in enumerate(tape):
        field += u[0][..., 0].ravel()[:, None] * (desc.delta_e * sig[i] * w[i])[None, :]
    return field
