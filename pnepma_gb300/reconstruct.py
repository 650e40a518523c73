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

The fitted material is either the per-cell boxed mass fractions (host material and pullbacks) or
any ``MaterialModel`` -- the reference's reconstructions fit a VolumeFractionSC material over a
Boxed or Bilinear field of ten parameters with a fixed embedding (``reconstructions_1d.jl:115-130``)
-- whose fields and pullbacks run on the device through one ``pn_material`` per measurement
geometry (:class:`DeviceMaterialSet`).
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

from . import physics
from .grid import GridSpec
from .material import BoxedMassFraction
from .material_model import MaterialModel
from .problem import PN_FP64
from .workloads import NM, Solve, make_solve, stable_steps


# ------------------------------------------------------------------------------------ backends
class BatchBackend:
    """Solves a fixed list of descriptors as one ``pn_batch`` on the GPU (device buffers through
    torch).  ``forward`` then ``adjoint`` on the same inputs, as ``pn_batch_forward/_adjoint``."""

    def __init__(self, descs, keep, memory_budget: int = 0, device: int = 0):
        import torch
        from . import autotune, capi
        self.torch = torch
        self.dev = torch.device("cuda", device)
        torch.cuda.set_device(self.dev)
        # the autotuner's configuration for this batch's key, when its table has one
        self.batch = capi.Batch(descs, keep, memory_budget=memory_budget, **autotune.options_for(descs))
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


class DeviceMaterialSet:
    """The fields and pullbacks of a ``MaterialModel`` for every problem of a reconstruction, on the
    device: one ``pn_material`` per measurement geometry (lines, detector, beam position), shared by
    the problems that have the same one.  Host arrays in and out, as the batch backend takes them."""

    def __init__(self, model: MaterialModel, solves, device=0):
        import torch
        from . import capi
        self.torch = torch
        self.dev = torch.device(device) if isinstance(device, str) else torch.device("cuda", device)
        cache, self.mats, self.sizes = {}, [], []
        for s in solves:
            key = (tuple(s.x_rays), tuple(float(v) for v in s.detector), float(s.problem.beam_position.mean[0]))
            if key not in cache:
                cache[key] = capi.DeviceMaterial(model.with_geometry(s.x_rays, s.detector, key[2]))
            self.mats.append(cache[key])
            d, k = s.problem.descriptor(s.x_rays)
            self.sizes.append(capi.query_sizes(d))
        self._owned = list(cache.values())
        self.ne, self.nr = model.n_e, [len(s.x_rays) for s in solves]

    def _dv(self, a):
        return self.torch.from_numpy(np.ascontiguousarray(a, dtype=np.float64)).to(self.dev)

    def _z(self, n):
        return self.torch.zeros(max(int(n), 1), dtype=self.torch.float64, device=self.dev)

    def _sync(self):
        if self.dev.type == "cuda":
            self.torch.cuda.synchronize(self.dev)

    def fields(self, P):
        """[(rho, noa [cells][n_e], acs [cells][n_r])] per problem."""
        dP = self._dv(P)
        out = []
        for dm, sz in zip(self.mats, self.sizes):
            rho, noa, acs = self._z(sz.n_rho), self._z(sz.n_noa), self._z(sz.n_acs)
            dm.fields(dP.data_ptr(), rho.data_ptr(), noa.data_ptr(), acs.data_ptr())
            out.append((rho, noa, acs))
        self._sync()
        res = []
        for (rho, noa, acs), sz, nr in zip(out, self.sizes, self.nr):
            res.append((rho.cpu().numpy()[:sz.n_rho], noa.cpu().numpy()[:sz.n_noa].reshape(-1, self.ne),
                        acs.cpu().numpy()[:sz.n_acs].reshape(-1, max(nr, 1))))
        return res

    def pullback(self, i, P, rho_bar, noa_bar, acs, acs_bar):
        """Parameter gradient of problem i from its adjoint outputs."""
        dm = self.mats[i]
        G = self._z(dm.n_params)
        dP, rb, nb, a, ab = (self._dv(x) for x in (P, rho_bar, noa_bar, acs, acs_bar))
        dm.pullback(dP.data_ptr(), G.data_ptr(), rb.data_ptr(), nb.data_ptr(), a.data_ptr(), ab.data_ptr())
        self._sync()
        return G.cpu().numpy()[:dm.n_params]

    def close(self):
        for dm in self._owned:
            dm.close()
        self._owned = []


class _BoxedMaterials:
    """Per-cell boxed mass fractions: host material, host pullbacks (the parameters are the
    ``values`` of a ``BoxedMassFraction``)."""

    def __init__(self, rec):
        self.rec = rec
        self.shape = rec.gspec.class_shape(0)[::-1] + (rec.n_par,)

    def inputs(self, p):
        r = self.rec
        m = BoxedMassFraction(r.elements, r.gspec, np.asarray(p, float).reshape(self.shape), sc=r.sc)
        return m, [Solve(s.problem, m, s.x_rays, s.detector).inputs() for s in r.solves]

    def pullback(self, m, i, inputs_i, rb, nb, ab):
        s = self.rec.solves[i]
        g = m.grid_pullback(rb) + m.noa_pullback(nb.reshape(self.shape[:-1] + (self.rec.n_e,)))
        g = g + m.absorption_pullback(s.x_rays, s.detector, s.problem.beam_position.mean, inputs_i[2], ab)[0]
        return g.ravel()

    def close(self):
        pass


class _ModelMaterials:
    """A ``MaterialModel`` through a material set (fields and per-problem pullbacks); the free
    parameters are its parameter vector, without the embedding when that is fixed."""

    def __init__(self, rec, model: MaterialModel, embedding, material_set_factory):
        if model.gspec != rec.gspec or [e.symbol for e in model.elements] != [e.symbol for e in rec.elements]:
            raise ValueError("the material model must live on the reconstruction's grid and elements")
        if model.sc != rec.sc:
            raise ValueError("the material model's SC flag must match the reconstruction's")
        self.model = model
        self.embedding = None if embedding is None else np.asarray(embedding, dtype=float).ravel()
        if self.embedding is not None and self.embedding.size != model.n_par:
            raise ValueError(f"the embedding has {model.n_par} values")
        self.n_free = model.n_params - (model.n_par if self.embedding is not None else 0)
        self.shape = (self.n_free,)
        factory = material_set_factory or (lambda mm, solves: DeviceMaterialSet(mm, solves))
        self.set = factory(model, rec.solves)

    def full(self, p):
        p = np.asarray(p, dtype=float).ravel()
        return np.concatenate([p, self.embedding]) if self.embedding is not None else p

    def inputs(self, p):
        P = self.full(p)
        return P, self.set.fields(P)

    def pullback(self, P, i, inputs_i, rb, nb, ab):
        return self.set.pullback(i, P, rb, nb, inputs_i[2], ab)[:self.n_free]

    def close(self):
        self.set.close()


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

    With ``model`` (a ``MaterialModel`` on the same grid and elements) the fitted parameters are the
    model's parameter vector, without the embedding when ``embedding`` fixes it (the reference's
    ``BoxedPNParametrization{false}`` / ``BilinearPNParametrization{false}``).
    ``material_set_factory(model, solves)`` returns an object with ``fields(P)``,
    ``pullback(i, P, rho_bar, noa_bar, acs, acs_bar)`` and ``close()``; by default
    :class:`DeviceMaterialSet`.
    """

    def __init__(self, N: int, gspec: GridSpec, elements, energies_kev, beam_ys=(0.0,), detector=(50 * NM, 0.0, 0.0),
                 n_steps: int = 100, precision: int = PN_FP64, sc: bool = True, beam_sigma: float = 30 * NM,
                 E_cut=None, backend_factory=None, memory_budget: int = 0, model: MaterialModel | None = None,
                 embedding=None, material_set_factory=None):
        self.gspec = gspec
        self.elements = [physics.ELEMENTS[e] if isinstance(e, str) else e for e in elements]
        self.sc = sc
        self.n_e = len(self.elements)
        self.n_par = self.n_e - 1 if sc else self.n_e
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
        self.mat = (_ModelMaterials(self, model, embedding, material_set_factory) if model is not None
                    else _BoxedMaterials(self))
        self.shape = self.mat.shape

    # ------------------------------------------------------------------ material and inputs
    def material(self, p):
        """The material of parameters p: a ``BoxedMassFraction``, or the model's full parameter
        vector (embedding included)."""
        return self.mat.inputs(p)[0] if isinstance(self.mat, _BoxedMaterials) else self.mat.full(p)

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
        self.mat.close()

    # ---------------------------------------------------------------------------- evaluations
    def measure(self, p) -> np.ndarray:
        """k-ratios of every problem and line (problem-major), one batched forward."""
        I = self._backend().forward(self.mat.inputs(p)[1])
        return np.concatenate([v / sd for v, sd in zip(I, self.std)])

    def _pullback(self, m, inputs, rb, nb, ab):
        g = np.zeros(int(np.prod(self.shape)))
        for i in range(len(self.solves)):
            g += self.mat.pullback(m, i, inputs[i], rb[i], nb[i], ab[i])
        return g.reshape(self.shape)

    def loss_grad(self, p, k_exp):
        """sum (k - k_exp)^2 and its gradient with respect to the parameters: one batched forward,
        one batched adjoint with I_bar = 2 (k - k_exp) / I_std, the material pullbacks."""
        m, inputs = self.mat.inputs(p)
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
        m, inputs = self.mat.inputs(p)
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
            J[q] = self.mat.pullback(m, i, inputs[i], rb[q], nb[q], ab[q])
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
