"""Autotuner of batched solves: for each key (precision, order, active axes, grid of the solves in a
batch) it measures the batch engine's configurations and keeps the one whose forward + adjoint runs
fastest, in a table that persists as JSON.

The configurations are the batch engine's own runtime choices:

* the kernel family: TMA tile kernels, the default for FP32 2D and 3D groups, or the generic
  kernels (``PN_BATCH_GENERIC_KERNELS``);
* the launch mode: sweeps captured as CUDA graphs at creation, the default, kernels issued from
  the host on every call (``PN_BATCH_DIRECT_LAUNCH``), or the TMA steps of each sweep as one
  persistent cooperative launch (``PN_BATCH_SWEEP_LAUNCH``);
* the tape schedule: the automatic choice within the memory budget, or a fixed checkpoint stride;
* the persistent grid of the TMA tile kernels: resident CTAs per SM (``PN_BATCH_CTAS_PER_SM_SHIFT``
  bits of the flags), i.e. how many tiles each CTA walks;
* the 2D tile shape: one tile per target class, the default, or parity tiles that update both
  target classes of a parity at one position (``PN_BATCH_PARITY_TILES``).

The tile box (32 x 4 points) and the points per thread are compile-time constants of the TMA
kernels (``PN_TMA_TY``, ``PN_TMA_PPT``) and are not among the runtime choices.  ``options_for``
returns the tuned configuration of a batch's key from the table; the reconstruction driver's
batches (``reconstruct.BatchBackend``) are built with it.  A configuration
that does not change anything for a batch is skipped: the kernel family and the CTA count only
matter for FP32 groups with two or three active axes.
"""
from __future__ import annotations

import json
import math
import os
from dataclasses import asdict, dataclass

import numpy as np

PN_BATCH_GENERIC_KERNELS = 1
PN_BATCH_DIRECT_LAUNCH = 2
PN_BATCH_SWEEP_LAUNCH = 16
PN_BATCH_PARITY_TILES = 32
PN_BATCH_CTAS_PER_SM_SHIFT = 8
PN_FP32 = 1


@dataclass(frozen=True)
class Config:
    flags: int = 0
    checkpoint_stride: int = 0

    @property
    def ctas_per_sm(self) -> int:
        return (self.flags >> PN_BATCH_CTAS_PER_SM_SHIFT) & 15

    def label(self) -> str:
        kern = "generic" if self.flags & PN_BATCH_GENERIC_KERNELS else "tma"
        if self.flags & PN_BATCH_PARITY_TILES:
            kern += "-parity"
        launch = ("direct" if self.flags & PN_BATCH_DIRECT_LAUNCH else
                  "sweep" if self.flags & PN_BATCH_SWEEP_LAUNCH else "graphs")
        tape = f"K={self.checkpoint_stride}" if self.checkpoint_stride else "K=auto"
        ctas = f"/ctas={self.ctas_per_sm}" if self.ctas_per_sm else ""
        return f"{kern}/{launch}/{tape}{ctas}"


DEFAULT_CANDIDATES = (
    Config(0, 0),
    Config(PN_BATCH_DIRECT_LAUNCH, 0),
    Config(PN_BATCH_GENERIC_KERNELS, 0),
    Config(0, 2),
    Config(0, 4),
    Config(PN_BATCH_SWEEP_LAUNCH, 0),
    Config(3 << PN_BATCH_CTAS_PER_SM_SHIFT, 0),
    Config(4 << PN_BATCH_CTAS_PER_SM_SHIFT, 0),
    Config(PN_BATCH_PARITY_TILES, 0),
)


# the table `bench.py --autotune` writes and the library's batch users read
DEFAULT_TABLE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "_build", "autotune.json")


def options_for(descs, path: str | None = DEFAULT_TABLE) -> dict:
    """``capi.Batch`` keyword arguments (flags, checkpoint_stride) of the configuration the table
    holds for the batch's key, or {} (the engine's defaults) when the table or the key is absent."""
    if not path or not os.path.exists(path):
        return {}
    try:
        with open(path) as f:
            entry = json.load(f).get(batch_key(descs))
    except (OSError, ValueError):
        return {}
    if not entry:
        return {}
    cfg = Config(**entry["config"])
    return {"flags": cfg.flags, "checkpoint_stride": cfg.checkpoint_stride}


def key_of(desc) -> str:
    """The key of one solve: precision, order, active axes and grid."""
    axes = "".join("xyz"[d] for d in range(3) if desc.n_points[d] > 1) or "0d"
    grid = "x".join(str(int(desc.n_points[d])) for d in range(3))
    return f"{'fp32' if desc.precision == PN_FP32 else 'fp64'}-N{desc.order}-{axes}-{grid}"


def batch_key(descs) -> str:
    """The key of a batch: the distinct keys of its solves, in sorted order."""
    return "+".join(sorted({key_of(d) for d in descs}))


def applies(cfg: Config, descs) -> bool:
    """False when the configuration runs the batch exactly as the default does."""
    tiles = any(d.precision == PN_FP32 and sum(d.n_points[k] > 1 for k in range(3)) >= 2 for d in descs)
    if cfg.flags & PN_BATCH_PARITY_TILES:
        return any(d.precision == PN_FP32 and sum(d.n_points[k] > 1 for k in range(3)) == 2 for d in descs)
    if cfg.flags & (PN_BATCH_GENERIC_KERNELS | PN_BATCH_SWEEP_LAUNCH) or cfg.ctas_per_sm:
        return tiles
    return True


class Autotuner:
    """Measures candidate configurations once per batch key and remembers the fastest.

    ``path``: JSON file of the table (read at creation, written after every new key); None keeps
    the table in memory only."""

    def __init__(self, path: str | None = None, candidates=DEFAULT_CANDIDATES):
        self.path = path
        self.candidates = list(candidates)
        self.table: dict = {}
        if path and os.path.exists(path):
            with open(path) as f:
                self.table = json.load(f)

    def lookup(self, descs) -> Config | None:
        entry = self.table.get(batch_key(descs))
        return Config(**entry["config"]) if entry else None

    def tune(self, descs, measure) -> Config:
        """The fastest configuration for the batch's key.  ``measure(config)`` returns the seconds
        of one forward + adjoint of the batch under that configuration (None if it cannot run);
        it is called only for keys not in the table."""
        cached = self.lookup(descs)
        if cached is not None:
            return cached
        results = []
        for cfg in self.candidates:
            if not applies(cfg, descs):
                continue
            t = measure(cfg)
            if t is not None and math.isfinite(t) and t > 0:
                results.append((float(t), cfg))
        if not results:
            raise RuntimeError("no candidate configuration could be measured")
        t, best = min(results, key=lambda r: r[0])
        self.table[batch_key(descs)] = {
            "config": asdict(best), "label": best.label(), "seconds": t,
            "measured": [{"config": asdict(c), "label": c.label(), "seconds": s} for s, c in results]}
        self.save()
        return best

    def save(self):
        if not self.path:
            return
        tmp = self.path + f".tmp{os.getpid()}"
        with open(tmp, "w") as f:
            json.dump(self.table, f, indent=1, sort_keys=True)
        os.replace(tmp, self.path)


def batch_timer(descs, keep, inputs, ibars, memory_budget: int = 0, reps: int = 2, device: int = 0):
    """``measure`` for :meth:`Autotuner.tune` on the GPU: builds the batch with the configuration,
    runs one forward + adjoint to warm up, then times ``reps`` of them with CUDA events, inputs
    resident on the device.  Returns seconds per forward + adjoint."""
    import torch
    from . import capi
    dev = torch.device("cuda", device)
    dv = lambda a: torch.from_numpy(np.ascontiguousarray(a, dtype=np.float64)).to(dev)
    z = lambda n: torch.zeros(max(int(n), 1), dtype=torch.float64, device=dev)
    ins = [tuple(dv(a) for a in x) for x in inputs]
    ib = [dv(x) for x in ibars]
    sizes = [capi.query_sizes(d) for d in descs]
    out_I = [z(d.n_xrays) for d in descs]
    out_b = [(z(s.n_rho), z(s.n_noa), z(s.n_acs)) for s in sizes]
    ptr = lambda ts: [t.data_ptr() for t in ts]

    def measure(cfg: Config):
        b = capi.Batch(descs, keep, memory_budget=memory_budget, checkpoint_stride=cfg.checkpoint_stride,
                       flags=cfg.flags)
        try:
            def run():
                b.forward(ptr(x[0] for x in ins), ptr(x[1] for x in ins), ptr(x[2] for x in ins), ptr(out_I))
                b.adjoint(ptr(ib), ptr(o[0] for o in out_b), ptr(o[1] for o in out_b), ptr(o[2] for o in out_b))
            run()
            torch.cuda.synchronize(dev)
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            for _ in range(reps):
                run()
            e1.record()
            torch.cuda.synchronize(dev)
            return e0.elapsed_time(e1) / 1e3 / reps
        finally:
            b.close()

    return measure
