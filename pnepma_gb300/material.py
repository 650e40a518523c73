"""Material model on the staggered grids: per-cell boxed mass fractions.

This is the input side of the solve (what the reference computes before its march) and the
last step of the gradient (what it does after the adjoint march):

* ``MassFractionPNMaterial(SC)``: rho_e = w_e / sum_j (w_j / rho_pure_j); the SC variant carries
  n_e - 1 parameters and sets the last fraction to 1 - sum of the others
  (``pn_parametrizations/pn_material.jl:199-264``), with the hand-written pullbacks of the same
  lines;
* ``BoxedPNParametrization``: piecewise constant on boxes bounded by slices, outside value
  ``embedding`` (``pn_parametrization_boxed.jl:137-175``, ``biliner_interp.jl:5-16``).  Boxes here
  are one per eee cell, bounded by the odd-grid points; a point of the odd grid maps to the box
  of the same index and the last one to the last box (the ``isapproxzero`` rule), done with
  integer indices;
* densities on all eight class grids (``pn_material_utils.jl:74-91``), number of atoms
  (``x_ray_intensities.jl:43-55``) and the 100-point absorption ray march with its pullback
  (``x_ray_intensities.jl:100-153``).
"""
from __future__ import annotations

import math

import numpy as np

from . import physics
from .grid import GridSpec
from .moments import N_CLASSES


class BoxedMassFraction:
    """Mass-fraction material with one box per eee cell.

    values: array [nz][ny][nx][n_par] of box parameters (n_par = n_e, or n_e - 1 with ``sc``).
    """

    def __init__(self, elements, gspec: GridSpec, values, sc: bool = False, embedding=None):
        self.elements = [physics.ELEMENTS[e] if isinstance(e, str) else e for e in elements]
        self.gspec = gspec
        self.sc = sc
        self.n_e = len(self.elements)
        self.n_par = self.n_e - 1 if sc else self.n_e
        shape = gspec.class_shape(0)[::-1]
        v = np.asarray(values, dtype=float)
        if v.shape != shape + (self.n_par,):
            raise ValueError(f"values must have shape {shape + (self.n_par,)}, got {v.shape}")
        self.values = v.copy()
        self.embedding = np.full(self.n_par, 0.5) if embedding is None else np.asarray(embedding, float)
        self.rho_pure = np.array([e.density for e in self.elements])
        self.atomic_mass = np.array([e.atomic_mass_g for e in self.elements])

    # ---------------------------------------------------------------- point evaluation
    def _fractions(self, p):
        """Full mass-fraction vectors from parameter vectors p [..., n_par]."""
        if self.sc:
            last = 1.0 - np.sum(p, axis=-1, keepdims=True)
            return np.concatenate([p, last], axis=-1)
        return p

    def densities_from_params(self, p):
        w = self._fractions(p)
        R = np.sum(w / self.rho_pure, axis=-1, keepdims=True)
        return w / R

    def params_pullback(self, p, rho_bar):
        """d(params) from d(rho) at parameter vectors p (MassFraction(SC) pullback)."""
        w = self._fractions(p)
        R = np.sum(w / self.rho_pure, axis=-1, keepdims=True)
        R_bar = -np.sum(w * rho_bar, axis=-1, keepdims=True) / R ** 2
        w_bar = rho_bar / R + R_bar / self.rho_pure
        if self.sc:
            return w_bar[..., :-1] - w_bar[..., -1:]
        return w_bar

    # ---------------------------------------------------------------- grid mapping
    def _axis_box_index(self, d: int, odd: bool) -> np.ndarray:
        ax = self.gspec.axes[d]
        n = ax.size(odd)
        if ax.singleton:
            return np.zeros(1, dtype=np.int64)
        idx = np.arange(n)
        return np.minimum(idx, ax.M - 1) if odd else idx

    def class_box_indices(self, c: int):
        bits = ((c >> 2) & 1, (c >> 1) & 1, c & 1)
        return [self._axis_box_index(d, bool(bits[d])) for d in range(3)]

    def class_params(self, c: int) -> np.ndarray:
        ix, iy, iz = self.class_box_indices(c)
        return self.values[np.ix_(iz, iy, ix)]

    def densities_on_grids(self) -> list[np.ndarray]:
        """rho per class as [nz][ny][nx][n_e]."""
        return [self.densities_from_params(self.class_params(c)) for c in range(N_CLASSES)]

    def rho_flat(self) -> np.ndarray:
        return np.concatenate([r.ravel() for r in self.densities_on_grids()])

    def number_of_atoms(self) -> np.ndarray:
        """[nz][ny][nx][n_e] on the eee grid."""
        return self.densities_on_grids()[0] / self.atomic_mass

    # ---------------------------------------------------------------- arbitrary points
    def _slices(self, d):
        ax = self.gspec.axes[d]
        h = ax.step
        return ax.lo - h / 2, h, ax.M

    def params_at_points(self, pts: np.ndarray) -> np.ndarray:
        """Boxed lookup at arbitrary points [n, 3] (floor rule; outside -> embedding)."""
        out = np.empty((pts.shape[0], self.n_par))
        inside = np.ones(pts.shape[0], dtype=bool)
        idx = []
        for d in range(3):
            ax = self.gspec.axes[d]
            if ax.singleton:
                idx.append(np.zeros(pts.shape[0], dtype=np.int64))
                continue
            lo, h, M = self._slices(d)
            t = (pts[:, d] - lo) / h
            i = np.floor(t).astype(np.int64)
            frac = t - i
            last = (i == M) & (np.abs(frac) < 1e-20)
            i = np.where(last, M - 1, i)
            inside &= (i >= 0) & (i <= M - 1)
            idx.append(np.clip(i, 0, M - 1))
        out[:] = self.embedding
        sel = np.nonzero(inside)[0]
        out[sel] = self.values[idx[2][sel], idx[1][sel], idx[0][sel]]
        return out, inside, idx

    def absorption(self, x_rays, detector, beam_pos, n_int_points: int = 100):
        """[nz][ny][nx][n_r] absorption factors on the eee grid."""
        macs = np.array([[physics.mass_absorption(x, e) for e in self.elements] for x in x_rays])
        px, py, pz = self.gspec.class_points(0)
        Z, Y, X = np.meshgrid(pz, py, px, indexing="ij")
        origin = np.stack([X.ravel(), Y.ravel(), Z.ravel()], axis=1)
        det = np.asarray(detector, float)
        d = det[None, :] - origin
        lam = np.maximum((beam_pos[0] - origin[:, 0]) / d[:, 0], 0.0)
        dx = np.linalg.norm(d, axis=1) * lam / n_int_points
        ac = np.zeros((origin.shape[0], len(x_rays)))
        for k in range(n_int_points):
            l = lam * (k / (n_int_points - 1))
            p = origin + l[:, None] * d
            par, _, _ = self.params_at_points(p)
            rho = self.densities_from_params(par)
            ac -= rho @ macs.T
        ac = np.exp(ac * dx[:, None])
        return ac.reshape(Z.shape + (len(x_rays),))

    # ---------------------------------------------------------------- pullbacks
    def grid_pullback(self, rho_bar_flat: np.ndarray) -> np.ndarray:
        """d(values) from d(rho) on all eight grids (component_densities_pullback)."""
        gbar = np.zeros_like(self.values)
        off = 0
        for c in range(N_CLASSES):
            shp = self.gspec.class_shape(c)[::-1] + (self.n_e,)
            n = int(np.prod(shp))
            rb = rho_bar_flat[off:off + n].reshape(shp)
            off += n
            p = self.class_params(c)
            pb = self.params_pullback(p, rb)
            ix, iy, iz = self.class_box_indices(c)
            IZ, IY, IX = np.meshgrid(iz, iy, ix, indexing="ij")
            np.add.at(gbar, (IZ, IY, IX), pb)
        return gbar

    def noa_pullback(self, noa_bar: np.ndarray) -> np.ndarray:
        p = self.class_params(0)
        pb = self.params_pullback(p, noa_bar / self.atomic_mass)
        return pb  # boxes of the eee grid coincide with its cells

    def absorption_pullback(self, x_rays, detector, beam_pos, acs, acs_bar, n_int_points: int = 100):
        macs = np.array([[physics.mass_absorption(x, e) for e in self.elements] for x in x_rays])
        px, py, pz = self.gspec.class_points(0)
        Z, Y, X = np.meshgrid(pz, py, px, indexing="ij")
        origin = np.stack([X.ravel(), Y.ravel(), Z.ravel()], axis=1)
        det = np.asarray(detector, float)
        d = det[None, :] - origin
        lam = np.maximum((beam_pos[0] - origin[:, 0]) / d[:, 0], 0.0)
        dx = np.linalg.norm(d, axis=1) * lam / n_int_points
        a = acs.reshape(-1, len(x_rays))
        ab = -a * dx[:, None] * acs_bar.reshape(-1, len(x_rays))
        rho_adj = ab @ macs          # [cells][n_e]
        gbar = np.zeros_like(self.values)
        emb = np.zeros(self.n_par)
        for k in range(n_int_points):
            l = lam * (k / (n_int_points - 1))
            p = origin + l[:, None] * d
            par, inside, idx = self.params_at_points(p)
            pb = self.params_pullback(par, rho_adj)
            sel = np.nonzero(inside)[0]
            np.add.at(gbar, (idx[2][sel], idx[1][sel], idx[0][sel]), pb[sel])
            emb += pb[~inside].sum(axis=0)
        return gbar, emb


class BoxPerturbation:
    """Inputs (rho, noa, acs) of a material with one box's parameters changed, updated locally.

    A central finite difference of the k-ratio functional with respect to one cell's mass
    fractions needs the solver inputs twice per cell.  Recomputing them for a 3D grid costs seconds
    (the 100-point absorption march over every cell), so this keeps the unperturbed arrays and
    changes only what depends on the box: rho at the grid points of the box on all eight grids,
    the box's number of atoms, and, for every cell whose absorption ray has samples in the box,
    its absorption factor.  With E_c = -sum_samples rho(p) . mu the factor is exp(E_c dx_c), so a
    change d rho in the box multiplies it by exp(-count_c (d rho . mu) dx_c), count_c being the
    number of the cell's samples inside the box (the sample rule of ``absorption``).
    """

    def __init__(self, mat: BoxedMassFraction, x_rays, detector, beam_pos, boxes, base, n_int_points: int = 100):
        self.mat = mat
        self.boxes = [tuple(int(v) for v in b) for b in boxes]   # (iz, iy, ix)
        self.rho0, self.noa0, self.acs0 = (np.array(a, dtype=float, copy=True) for a in base)
        self.macs = np.array([[physics.mass_absorption(x, e) for e in mat.elements] for x in x_rays])
        g = mat.gspec
        M = [g.axes[d].M for d in range(3)]
        self.M = M
        # grid points of each box on each class grid (flat offsets into rho, element 0)
        self.points = {b: [] for b in self.boxes}
        off = 0
        for c in range(N_CLASSES):
            ix, iy, iz = mat.class_box_indices(c)
            nz, ny, nx = len(iz), len(iy), len(ix)
            for b in self.boxes:
                zs = np.nonzero(iz == b[0])[0]
                ys = np.nonzero(iy == b[1])[0]
                xs = np.nonzero(ix == b[2])[0]
                if len(zs) and len(ys) and len(xs):
                    Zs, Ys, Xs = np.meshgrid(zs, ys, xs, indexing="ij")
                    pts = ((Zs * ny + Ys) * nx + Xs).ravel()
                    self.points[b].append(off + pts * mat.n_e)
            off += nz * ny * nx * mat.n_e
        for b in self.boxes:
            self.points[b] = np.concatenate(self.points[b]) if self.points[b] else np.zeros(0, dtype=np.int64)
        # rays: per box, the cells with samples inside it and their counts
        px, py, pz = g.class_points(0)
        Z, Y, X = np.meshgrid(pz, py, px, indexing="ij")
        origin = np.stack([X.ravel(), Y.ravel(), Z.ravel()], axis=1)
        det = np.asarray(detector, float)
        dvec = det[None, :] - origin
        lam = np.maximum((beam_pos[0] - origin[:, 0]) / dvec[:, 0], 0.0)
        self.dx = np.linalg.norm(dvec, axis=1) * lam / n_int_points
        lin = np.array([(b[0] * M[1] + b[1]) * M[0] + b[2] for b in self.boxes])
        order = np.argsort(lin)
        lin_sorted = lin[order]
        counts = np.zeros((len(self.boxes), origin.shape[0]), dtype=np.int32)
        for k in range(n_int_points):
            l = lam * (k / (n_int_points - 1))
            p = origin + l[:, None] * dvec
            _, inside, idx = mat.params_at_points(p)
            boxid = np.where(inside, (idx[2] * M[1] + idx[1]) * M[0] + idx[0], -1)
            hit = np.nonzero(np.isin(boxid, lin_sorted))[0]
            if hit.size:
                which = order[np.searchsorted(lin_sorted, boxid[hit])]
                np.add.at(counts, (which, hit), 1)
        self.rays = {}
        for q, b in enumerate(self.boxes):
            cells = np.nonzero(counts[q])[0]
            self.rays[b] = (cells, counts[q][cells])

    def inputs(self, box, param_delta):
        """(rho, noa, acs) with the box's parameter vector changed by `param_delta` [n_par]."""
        m = self.mat
        b = tuple(int(v) for v in box)
        p_old = m.values[b]
        p_new = p_old + np.asarray(param_delta, float)
        r_old = m.densities_from_params(p_old[None, :])[0]
        r_new = m.densities_from_params(p_new[None, :])[0]
        rho = self.rho0.copy()
        pts = self.points[b]
        for e in range(m.n_e):
            rho[pts + e] = r_new[e]
        noa = self.noa0.copy()
        cell = (b[0] * self.M[1] + b[1]) * self.M[0] + b[2]
        noa.reshape(-1, m.n_e)[cell] = r_new / m.atomic_mass
        acs = self.acs0.copy().reshape(-1, self.macs.shape[0])
        cells, cnt = self.rays[b]
        if cells.size:
            dmu = (r_new - r_old) @ self.macs.T          # [n_r]
            acs[cells] *= np.exp(-(cnt[:, None] * dmu[None, :]) * self.dx[cells, None])
        return rho, noa, acs.reshape(self.acs0.shape)
