"""CPU restatement of the reference's material evaluation and material pullbacks (test
infrastructure only: the tests use it as the checker of the device material kernels; the library
never imports it).

Follows, point by point and in the reference's loop and summation order:

* ``find_index_smaller_and_partition`` for ranges and vectors (``biliner_interp.jl:5-36``);
* Const / Boxed / Bilinear ``parametrization!`` and ``parametrization_pullback!``
  (``pn_parametrization_const.jl``, ``pn_parametrization_boxed.jl:137-175``,
  ``pn_parametrization_bilinear.jl:122-130`` with ``biliner_interp.jl:63-111,163-218``);
* ``component_densities!`` and ``component_densities_pullback!`` of the four material models and
  their SC variants (``pn_material.jl:71-264``);
* all eight grids (``pn_material_utils.jl:74-91``), the number of atoms and its pullback
  (``x_ray_intensities.jl:43-96``), the 100-sample absorption factors and their pullback
  (``x_ray_intensities.jl:100-153``).

Parity status: "parity unpinned" against the reference itself (Julia is not available here, and
the reference's own pn_material_test.jl checks its pullbacks only against finite differences).  This
restatement is pinned the same way: by central finite differences of its own fields for every
model and parametrisation, by the reference's point-location rules as known answers, and by the
host boxed mass-fraction path, which it reproduces to 1e-14 (tests/test_material_cpu.py).

Sums run left to right as Julia's ``sum`` and the broadcast expressions do for short vectors;
``dot`` and ``mul!`` (BLAS in Julia) are written as left-to-right sums, which can differ from the
BLAS result in the last bits.  Inputs come from a ``MaterialModel`` (``pnepma_gb300``), the same
object the device descriptor is built from.
"""
from __future__ import annotations

import math

import numpy as np


def _seqsum(v):
    s = 0.0
    for a in v:
        s = s + float(a)
    return s


def _dot(a, b):
    s = 0.0
    for x, y in zip(a, b):
        s = s + float(x) * float(y)
    return s


def approx_zero(a: float) -> bool:
    """``isapproxzero`` (biliner_interp.jl:45-47)."""
    return abs(a) < 1e-20


def locate(sl, x: float):
    """(1-based index, partition) of x in slices `sl` (biliner_interp.jl:5-36)."""
    if sl.n == 1:
        return 1, 0.0
    if sl.values is None:
        d = x - sl.ref
        f = math.floor(d / sl.step)
        return int(f) + sl.offset, (d - f * sl.step) / sl.step
    rg = sl.values
    i = 1
    while x > rg[i] and i < sl.n - 1:     # rg[i+1] in 1-based indexing is rg[i] here
        i += 1
    d = (x - rg[i - 1]) / (rg[i] - rg[i - 1])
    if d < 0.0:
        i -= 1
    elif d > 1.0:
        i += 1
    return i, d


def param_terms(mm, x):
    """[(vector index, weight)] of the parametrisation at point x, in the reference's order; the
    embedding is the vector index after the boxes or knots."""
    if mm.parametrization == "const":
        return [(0, 1.0)]
    nb = mm.grid_shape
    emb = nb[0] * nb[1] * nb[2]
    loc = [locate(mm.slices[d], x[d]) for d in range(3)]
    if mm.parametrization == "boxed":
        idx = []
        inside = True
        for d in range(3):
            i, p = loc[d]
            if i == mm.slices[d].n and approx_zero(p):
                i -= 1
            inside = inside and 1 <= i <= mm.slices[d].n - 1
            idx.append(i)
        if not inside:
            return [(emb, 1.0)]
        return [(((idx[2] - 1) * nb[1] + (idx[1] - 1)) * nb[0] + (idx[0] - 1), 1.0)]
    # bilinear: the branch of biliner_interp.jl:63-111 chosen by the partitions that are ~0
    ix, iy, iz = (loc[d][0] for d in range(3))
    px, py, pz = (loc[d][1] for d in range(3))
    zx, zy, zz = approx_zero(px), approx_zero(py), approx_zero(pz)

    def key(cx, cy, cz):
        if cx < 1 or cx > nb[0] or cy < 1 or cy > nb[1] or cz < 1 or cz > nb[2]:
            return emb
        return ((cz - 1) * nb[1] + (cy - 1)) * nb[0] + (cx - 1)

    if zx and zy and zz:
        return [(key(ix, iy, iz), 1.0)]
    if zx and zy:
        return [(key(ix, iy, iz), 1.0 - pz), (key(ix, iy, iz + 1), pz)]
    if zy and zz:
        return [(key(ix, iy, iz), 1.0 - px), (key(ix + 1, iy, iz), px)]
    if zx and zz:
        return [(key(ix, iy, iz), 1.0 - py), (key(ix, iy + 1, iz), py)]
    if zx:
        return [(key(ix, iy, iz), (1.0 - py) * (1.0 - pz)), (key(ix, iy + 1, iz), py * (1.0 - pz)),
                (key(ix, iy, iz + 1), (1.0 - py) * pz), (key(ix, iy + 1, iz + 1), py * pz)]
    if zy:
        return [(key(ix, iy, iz), (1.0 - px) * (1.0 - pz)), (key(ix + 1, iy, iz), px * (1.0 - pz)),
                (key(ix, iy, iz + 1), (1.0 - px) * pz), (key(ix + 1, iy, iz + 1), px * pz)]
    if zz:
        return [(key(ix, iy, iz), (1.0 - px) * (1.0 - py)), (key(ix + 1, iy, iz), px * (1.0 - py)),
                (key(ix, iy + 1, iz), (1.0 - px) * py), (key(ix + 1, iy + 1, iz), px * py)]
    return [(key(ix, iy, iz), (1.0 - px) * (1.0 - py) * (1.0 - pz)),
            (key(ix + 1, iy, iz), px * (1.0 - py) * (1.0 - pz)),
            (key(ix, iy + 1, iz), (1.0 - px) * py * (1.0 - pz)),
            (key(ix, iy, iz + 1), (1.0 - px) * (1.0 - py) * pz),
            (key(ix + 1, iy + 1, iz), px * py * (1.0 - pz)),
            (key(ix + 1, iy, iz + 1), px * (1.0 - py) * pz),
            (key(ix, iy + 1, iz + 1), (1.0 - px) * py * pz),
            (key(ix + 1, iy + 1, iz + 1), px * py * pz)]


def param_value(mm, P, x):
    """``parametrization!`` at x: the n_par values."""
    V = P.reshape(-1, mm.n_par)
    terms = param_terms(mm, x)
    if len(terms) == 1:
        return V[terms[0][0]].copy()
    out = np.empty(mm.n_par)
    for q in range(mm.n_par):
        s = terms[0][1] * V[terms[0][0], q]
        for k, w in terms[1:]:
            s = s + w * V[k, q]
        out[q] = s
    return out


def _full(mm, p):
    if not mm.sc:
        return [float(a) for a in p]
    return [float(a) for a in p] + [1.0 - _seqsum(p)]


def densities(mm, p):
    """``component_densities!`` from the parametrisation value p (pn_material.jl)."""
    f = _full(mm, p)
    rp = mm.rho_pure
    if mm.model == "mass_concentration":
        return np.array(f)
    if mm.model == "volume_fraction":
        return np.array([f[e] * rp[e] for e in range(mm.n_e)])
    if mm.model == "linear_density":
        dt = _dot(f, rp)
        return np.array([f[e] * dt for e in range(mm.n_e)])
    R = _seqsum([f[e] / rp[e] for e in range(mm.n_e)])
    return np.array([f[e] / R for e in range(mm.n_e)])


def model_pullback(mm, p, rb):
    """``component_densities_pullback!`` up to the parametrisation: the n_par cotangent."""
    rp = mm.rho_pure
    ne = mm.n_e
    if mm.model == "mass_concentration":
        g = [float(a) for a in rb]
    elif mm.model == "volume_fraction":
        g = [rb[e] * rp[e] for e in range(ne)]
    elif mm.model == "linear_density":
        f = _full(mm, p)
        dpr, dpb = _dot(f, rp), _dot(f, rb)
        g = [rb[e] * dpr + rp[e] * dpb for e in range(ne)]
    else:
        f = _full(mm, p)
        R = _seqsum([f[e] / rp[e] for e in range(ne)])
        Rb = -_dot(f, rb) / (R * R)
        g = [rb[e] / R + Rb / rp[e] for e in range(ne)]
    if mm.sc:
        return np.array([g[q] - g[ne - 1] for q in range(mm.n_par)])
    return np.array(g[:mm.n_par])


def _scatter(mm, G, x, pb):
    V = G.reshape(-1, mm.n_par)
    terms = param_terms(mm, x)
    if len(terms) == 1:
        V[terms[0][0]] += pb
        return
    for k, w in terms:
        V[k] += w * pb


def _grids(mm):
    """Class grids in class order: [(c, xs, ys, zs)], x fastest within a class."""
    out = []
    for c in range(8):
        xs, ys, zs = mm.gspec.class_points(c)
        out.append((c, xs, ys, zs))
    return out


def _points(xs, ys, zs):
    for z in zs:
        for y in ys:
            for x in xs:
                yield (float(x), float(y), float(z))


def _ray(mm, o):
    d = [mm.detector[k] - o[k] for k in range(3)]
    lam = max((mm.beam_x - o[0]) / d[0], 0.0)
    nrm = math.sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2])
    return d, lam, nrm * lam / mm.n_int_points


def _sample(mm, o, d, lam, k):
    n = mm.n_int_points
    l = lam * (k / (n - 1)) if n > 1 else 0.0
    return (o[0] + l * d[0], o[1] + l * d[1], o[2] + l * d[2])


def fields(mm, P):
    """(rho [n_rho], noa [eee][n_e], acs [eee][n_r]) from parameters P."""
    P = np.asarray(P, dtype=float)
    rho = []
    for c, xs, ys, zs in _grids(mm):
        for x in _points(xs, ys, zs):
            rho.append(densities(mm, param_value(mm, P, x)))
    rho = np.concatenate(rho)
    xs, ys, zs = mm.gspec.class_points(0)
    eee = list(_points(xs, ys, zs))
    noa = np.array([densities(mm, param_value(mm, P, x)) / mm.atom_mass for x in eee])
    nr = len(mm.x_rays)
    acs = np.zeros((len(eee), nr))
    for ci, o in enumerate(eee if nr else []):      # no lines: no absorption factors to form
        d, lam, dx = _ray(mm, o)
        ac = [0.0] * nr
        for k in range(mm.n_int_points):
            r = densities(mm, param_value(mm, P, _sample(mm, o, d, lam, k)))
            for q in range(nr):
                ac[q] = ac[q] - _dot(mm.mac[q], r)
        acs[ci] = [math.exp(a * dx) for a in ac]
    return rho, noa, acs


def pullback(mm, P, rho_bar=None, noa_bar=None, acs=None, acs_bar=None):
    """Parameter gradient [n_params]: component_densities_pullback on the eight grids, then
    compute_absorption_coefficient_pullback, then compute_number_of_atoms_pullback (the order
    of pn_intensities.jl:406-409)."""
    P = np.asarray(P, dtype=float)
    G = np.zeros(mm.n_params)
    ne = mm.n_e
    if rho_bar is not None:
        rb = np.asarray(rho_bar, dtype=float).reshape(-1, ne)
        q = 0
        for c, xs, ys, zs in _grids(mm):
            for x in _points(xs, ys, zs):
                _scatter(mm, G, x, model_pullback(mm, param_value(mm, P, x), rb[q]))
                q += 1
    xs, ys, zs = mm.gspec.class_points(0)
    eee = list(_points(xs, ys, zs))
    if acs_bar is not None:
        a = np.asarray(acs, dtype=float).reshape(len(eee), -1)
        ab = np.asarray(acs_bar, dtype=float).reshape(len(eee), -1)
        nr = a.shape[1]
        for ci, o in enumerate(eee):
            d, lam, dx = _ray(mm, o)
            aa = [-a[ci, r] * dx * ab[ci, r] for r in range(nr)]
            radj = np.array([_dot([mm.mac[r][e] for r in range(nr)], aa) for e in range(ne)])
            for k in range(mm.n_int_points):
                x = _sample(mm, o, d, lam, k)
                _scatter(mm, G, x, model_pullback(mm, param_value(mm, P, x), radj))
    if noa_bar is not None:
        nb = np.asarray(noa_bar, dtype=float).reshape(len(eee), ne)
        for ci, x in enumerate(eee):
            _scatter(mm, G, x, model_pullback(mm, param_value(mm, P, x), nb[ci] / mm.atom_mass))
    return G
