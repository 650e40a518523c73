"""Reconstruction driver over the batched solves: k-ratio standards cache, loss, gradient,
Jacobian, and L-BFGS-B / Gauss-Newton fits of the per-cell mass fractions.

The callers of the hot path in the reference (``scripts/reconstructions_1d.jl:56-185``,
``scripts/2d_full_reconstruction_test.jl:104-234``) evaluate, for every beam energy and position,

* ``measure(m) = calc_intensities(problem_i, m, x_rays, detector) ./ std_ints[i]`` - k-ratios
  against pure-element standards computed once (``reconstructions_1d.jl:56-58``);
* ``loss(m) = sum((measure(m) - k_exp).^2)`` (``:68-71``), its gradient through the adjoint of
  ``calc_intensities`` and the material pullbacks (``Zygote.withgradient``, ``:150-163``);
* ``optimize(only_fg!(loss_fg!), 0, 1, p, Fminbox(BFGS()))`` (``:175-183``).

Here every (energy, position) problem of one iteration runs as one ``pn_batch``: the forward of
all problems in one call, the adjoint of all problems in one call, with the cotangent
``I_bar = 2 (k - k_exp) / I_std`` formed from the forward's intensities.  The batch is created once
per problem set and reused every iteration (its CUDA graphs are captured once).  The standards'
intensities are computed once per problem signature in one batch and kept in a process-wide cache.
The material pullbacks (densities on the eight grids, number of atoms, absorption ray march) run on
the host as in the reference, where they follow the adjoint.

The Jacobian of the k-ratios (for Gauss-Newton) takes one adjoint per k-ratio: the problems are
repeated once per line in a second batch, each copy with the unit cotangent of its line.
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

from . import physics
from .grid import GridSpec
from .material import BoxedMassFraction
from .problem import PN_FP64
from .workloads import NM, Solve, make_solve, stable_steps


# ------------------------------------------------------------------------------------ backends
class BatchBackend:
    """Solves a fixed list of descriptors as one ``pn_batch`` on the GPU (device buffers through
    torch).  ``forward`` then ``adjoint`` on the same inputs, as ``pn_batch_forward/_adjoint``."""

    def __init__(self, descs, keep, memory_budget: int = 0, device: int = 0):
        import torch
        from . import capi
        self.torch = torch
        self.dev = torch.device("cuda", device)
        torch.cuda.set_device(self.dev)
        self.batch = capi.Batch(descs, keep, memory_budget=memory_budget)
        self.sizes = [capi.query_sizes(d) for d in descs]
        self.nr = [d.n_xrays for d in descs]
        self._inputs = None

    def _dv(self, a):
        return self.torch.from_numpy(np.ascontiguousarray(a, dtype=np.float64)).to(self.dev)

    def forward(self, inputs):
        """inputs: list of (rho, noa, acs) host arrays; returns the intensities (host)."""
        t = self.torch
        self._inputs = [tuple(self._dv(a) for a in x) for x in inputs]
        I = [t.zeros(nr, dtype=t.float64, device=self.dev) for nr in self.nr]
        self.batch.forward([x[0].data_ptr() for x in self._inputs], [x[1].data_ptr() for x in self._inputs],
                           [x[2].data_ptr() for x in self._inputs], [v.data_ptr() for v in I])
        t.cuda.synchronize(self.dev)
        return [v.cpu().numpy() for v in I]

    def adjoint(self, ibars):
        """Cotangents of the intensities of the last forward; returns (rho_bar, noa_bar, acs_bar)."""
        t = self.torch
        ib = [self._dv(x) for x in ibars]
        rb = [t.zeros(s.n_rho, dtype=t.float64, device=self.dev) for s in self.sizes]
        nb = [t.zeros(s.n_noa, dtype=t.float64, device=self.dev) for s in self.sizes]
        ab = [t.zeros(max(s.n_acs, 1), dtype=t.float64, device=self.dev) for s in self.sizes]
        self.batch.adjoint([v.data_ptr() for v in ib], [v.data_ptr() for v in rb], [v.data_ptr() for v in nb],
                           [v.data_ptr() for v in ab])
        t.cuda.synchronize(self.dev)
        return [v.cpu().numpy() for v in rb], [v.cpu().numpy() for v in nb], [v.cpu().numpy() for v in ab]

    def close(self):
        self.batch.close()


# --------------------------------------------------------------------------- standards cache
_STANDARDS: dict = {}


def problem_signature(s: Solve):
    """What a standard's intensities depend on: the descriptor (order, grid, energies, step count,
    beam, precision, lines) and the measurement geometry; not the sample material."""
    p = s.problem
    g = p.gspec
    return (p.N, tuple(a.M for a in g.axes), tuple((a.lo, a.hi) for a in g.axes), tuple(e.symbol for e in p.elements),
            p.beam_energy.mean, tuple(p.beam_position.mean), p.beam_position.std, p.E_initial, p.E_cutoff,
            p.N_steps, p.precision, tuple((x.element, x.transition) for x in s.x_rays), tuple(s.detector))


def pure_material(gspec: GridSpec, elements, e: int, sc: bool) -> BoxedMassFraction:
    """The pure-element standard of element e on the sample's grid."""
    shape = gspec.class_shape(0)[::-1]
    w = np.zeros(shape + (len(elements),))
    w[..., e] = 1.0
    return BoxedMassFraction(elements, gspec, w[..., :-1] if sc else w, sc=sc)


def standard_intensities(solves, backend_factory, sc: bool):
    """I_std[i][r]: line r of problem i in the pure standard of the line's element; computed once
    per problem signature (one batch for all missing ones) and cached for the process."""
    missing = [i for i, s in enumerate(solves) if problem_signature(s) not in _STANDARDS]
    if missing:
        jobs, descs, keep, inputs = [], [], [], []
        for i in missing:
            s = solves[i]
            els = s.problem.elements
            for e in range(len(els)):
                m = pure_material(s.problem.gspec, els, e, sc)
                std = Solve(s.problem, m, s.x_rays, s.detector, label="standard")
                d, k = s.problem.descriptor(s.x_rays)
                descs.append(d)
                keep.append(k)
                inputs.append(std.inputs())
                jobs.append((i, e))
        be = backend_factory(descs, keep)
        try:
            I = be.forward(inputs)
        finally:
            be.close()
        per = {}
        for (i, e), v in zip(jobs, I):
            per.setdefault(i, {})[e] = v
        for i in missing:
            s = solves[i]
            sym = [el.symbol for el in s.problem.elements]
            _STANDARDS[problem_signature(s)] = np.array(
                [per[i][sym.index(x.element)][r] for r, x in enumerate(s.x_rays)])
    return [_STANDARDS[problem_signature(s)] for s in solves]


def clear_standards():
    _STANDARDS.clear()


# ------------------------------------------------------------------------------ reconstruction
@dataclass
class FitResult:
    params: np.ndarray
    loss: float
    losses: list = field(default_factory=list)
    iterations: int = 0
    message: str = ""


class Reconstruction:
    """k-ratio reconstruction of boxed per-cell mass fractions (one box per eee cell).

    problems: one per (beam energy, beam position); all share the grid, order, elements, lines
    and detector.  The energy-step count of each problem is the larger of ``n_steps`` and the
    stable count for the lowest stopping power of the pure elements, so that every mixture the
    fit visits (and every standard) marches stably.  ``backend_factory(descs, keep)`` returns an
    object with ``forward(inputs)``, ``adjoint(ibars)`` and ``close()``; by default the GPU batch.
    """

    def __init__(self, N: int, gspec: GridSpec, elements, energies_kev, beam_ys=(0.0,), detector=(50 * NM, 0.0, 0.0),
                 n_steps: int = 100, precision: int = PN_FP64, sc: bool = True, beam_sigma: float = 30 * NM,
                 E_cut=None, backend_factory=None, memory_budget: int = 0):
        self.gspec = gspec
        self.elements = [physics.ELEMENTS[e] if isinstance(e, str) else e for e in elements]
        self.sc = sc
        self.n_e = len(self.elements)
        self.n_par = self.n_e - 1 if sc else self.n_e
        self.shape = gspec.class_shape(0)[::-1] + (self.n_par,)
        self.backend_factory = backend_factory or (lambda d, k: BatchBackend(d, k, memory_budget=memory_budget))
        names = [e.symbol for e in self.elements]
        mix = np.full(gspec.class_shape(0)[::-1] + (self.n_e,), 1.0 / self.n_e)
        self.solves = []
        for E in energies_kev:
            for y in beam_ys:
                kw = dict(beam_y=y, beam_sigma=beam_sigma, E_cut=E_cut, sc=sc, detector=detector,
                          precision=precision, stabilise=False)
                s = make_solve(N, gspec, names, mix, E, n_steps=n_steps, **kw)
                # a mixture's stopping power lies between the pure elements': the slowest one bounds
                # the stable step for every material the fit can visit
                ns = max(stable_steps(s.problem, pure_material(gspec, self.elements, e, sc), n_steps)
                         for e in range(self.n_e))
                if ns != n_steps:
                    s = make_solve(N, gspec, names, mix, E, n_steps=ns, **kw)
                self.solves.append(s)
        self.std = standard_intensities(self.solves, self.backend_factory, sc)
        self._be = None
        self._jac_be = None

    # ------------------------------------------------------------------ material and inputs
    def material(self, p) -> BoxedMassFraction:
        return BoxedMassFraction(self.elements, self.gspec, np.asarray(p, float).reshape(self.shape), sc=self.sc)

    def _inputs(self, m):
        return [Solve(s.problem, m, s.x_rays, s.detector).inputs() for s in self.solves]

    def _backend(self):
        if self._be is None:
            descs, keep = zip(*[s.problem.descriptor(s.x_rays) for s in self.solves])
            self._be = self.backend_factory(list(descs), list(keep))
        return self._be

    def close(self):
        for be in (self._be, self._jac_be):
            if be is not None:
                be.close()
        self._be = self._jac_be = None

    # ---------------------------------------------------------------------------- evaluations
    def measure(self, p) -> np.ndarray:
        """k-ratios of every problem and line (problem-major), one batched forward."""
        I = self._backend().forward(self._inputs(self.material(p)))
        return np.concatenate([v / sd for v, sd in zip(I, self.std)])

    def _pullback(self, m, inputs, rb, nb, ab):
        g = np.zeros(self.shape)
        for s, (rho, noa, acs), r_, n_, a_ in zip(self.solves, inputs, rb, nb, ab):
            g += m.grid_pullback(r_)
            g += m.noa_pullback(n_.reshape(self.shape[:-1] + (self.n_e,)))
            g += m.absorption_pullback(s.x_rays, s.detector, s.problem.beam_position.mean, acs, a_)[0]
        return g

    def loss_grad(self, p, k_exp):
        """sum (k - k_exp)^2 and its gradient with respect to the parameters: one batched forward,
        one batched adjoint with I_bar = 2 (k - k_exp) / I_std, the material pullbacks."""
        m = self.material(p)
        inputs = self._inputs(m)
        be = self._backend()
        I = be.forward(inputs)
        k = np.concatenate([v / sd for v, sd in zip(I, self.std)])
        r = k - np.asarray(k_exp, float)
        loss = float(r @ r)
        nr = [len(sd) for sd in self.std]
        rs = np.split(r, np.cumsum(nr)[:-1])
        rb, nb, ab = be.adjoint([2.0 * ri / sd for ri, sd in zip(rs, self.std)])
        return loss, self._pullback(m, inputs, rb, nb, ab).ravel()

    def jacobian(self, p):
        """(k, J) with J[i, :] = d k_i / d params: the problems repeated once per line in one batch,
        each copy's adjoint with the unit cotangent of its line (divided by the standard)."""
        m = self.material(p)
        inputs = self._inputs(m)
        rows = [(i, r) for i, sd in enumerate(self.std) for r in range(len(sd))]
        if self._jac_be is None:
            descs, keep = [], []
            for i, _r in rows:
                d, k = self.solves[i].problem.descriptor(self.solves[i].x_rays)
                descs.append(d)
                keep.append(k)
            self._jac_be = self.backend_factory(descs, keep)
        be = self._jac_be
        I = be.forward([inputs[i] for i, _r in rows])
        k = np.array([I[q][r] / self.std[i][r] for q, (i, r) in enumerate(rows)])
        ibars = []
        for i, r in rows:
            e = np.zeros(len(self.std[i]))
            e[r] = 1.0 / self.std[i][r]
            ibars.append(e)
        rb, nb, ab = be.adjoint(ibars)
        J = np.empty((len(rows), int(np.prod(self.shape))))
        for q, (i, r) in enumerate(rows):
            s = self.solves[i]
            acs = inputs[i][2]
            g = m.grid_pullback(rb[q]) + m.noa_pullback(nb[q].reshape(self.shape[:-1] + (self.n_e,)))
            g = g + m.absorption_pullback(s.x_rays, s.detector, s.problem.beam_position.mean, acs, ab[q])[0]
            J[q] = g.ravel()
        return k, J

    # ----------------------------------------------------------------------------------- fits
    def fit_lbfgs(self, p0, k_exp, maxiter: int = 50, bounds=(0.0, 1.0)) -> FitResult:
        """Box-constrained quasi-Newton fit (the reference's Fminbox(BFGS()) on [0, 1])."""
        from scipy.optimize import minimize
        losses = []

        def fg(x):
            f, g = self.loss_grad(x, k_exp)
            losses.append(f)
            return f, g

        x0 = np.clip(np.asarray(p0, float).ravel(), bounds[0], bounds[1])
        res = minimize(fg, x0, jac=True, method="L-BFGS-B", bounds=[bounds] * x0.size,
                       options={"maxiter": maxiter})
        return FitResult(res.x.reshape(self.shape), float(res.fun), losses, int(res.nit), str(res.message))

    def fit_gauss_newton(self, p0, k_exp, iterations: int = 10, damping: float = 1e-3,
                         bounds=(0.0, 1.0)) -> FitResult:
        """Projected Levenberg-Marquardt: (J^T J + lambda diag(J^T J)) dp = -J^T r, clipped to the box;
        lambda grows when a step does not lower the loss and shrinks when it does."""
        p = np.clip(np.asarray(p0, float).ravel(), bounds[0], bounds[1])
        k_exp = np.asarray(k_exp, float)
        k, J = self.jacobian(p)
        r = k - k_exp
        loss = float(r @ r)
        losses = [loss]
        lam = damping
        for it in range(iterations):
            A = J.T @ J
            g = J.T @ r
            step = np.linalg.solve(A + lam * np.diag(np.maximum(np.diag(A), 1e-30)), -g)
            q = np.clip(p + step, bounds[0], bounds[1])
            kq = self.measure(q)
            rq = kq - k_exp
            lq = float(rq @ rq)
            if lq < loss:
                p, loss = q, lq
                lam = max(lam / 3.0, 1e-12)
                k, J = self.jacobian(p)
                r = k - k_exp
            else:
                lam *= 4.0
            losses.append(loss)
        return FitResult(p.reshape(self.shape), loss, losses, iterations, "done")
