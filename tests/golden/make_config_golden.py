"""Regenerate tests/golden/oracle_config_cases.npz: oracle results at the benchmark configurations.

    python tests/golden/make_config_golden.py          (about 3 minutes on 8 host threads)

The reference ships no golden vectors for this path and cannot run here, so these come from the
CPU restatement (oracle/) at the full sizes of the workloads, where running the oracle inside a
GPU test would take minutes and tens of GB of host memory for its tape:

* ``config1``: the 1D slab, 200 cells, P7, Cu/Ni in four layers, 15 keV, the full stable march
  (forward + adjoint); every output is stored in full.
* ``config2_{10,15,20}kev``: one solve of the 2D workload per beam energy (256 x 128 cells, P11,
  Fe/Cr/Ni, beam position 7 of 20), the full stable march each.  The cotangents are summarised
  (:func:`summarise`): values at 2048 positions (the 512 largest in magnitude and 1536 chosen by
  a hash of the index), projections on eight +-1 vectors made from the same hash, the 1-norm and
  the largest magnitude.  A GPU result is compared entry by entry at the stored positions and
  through the projections, which see an error anywhere in the array.

Every input is regenerated from its seed by ``pnepma_gb300.workloads``.  The cotangent of each
solve is ``linspace(1, 2, n_lines) / |I|`` (the scale of a squared k-ratio loss).
"""
from __future__ import annotations

import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
PATH = os.path.join(HERE, "oracle_config_cases.npz")

CONFIG2_POSITION = 7
CONFIG2_ENERGIES = (10.0, 15.0, 20.0)
N_TOP, N_HASHED, N_PROJ = 512, 1536, 8
OUTPUTS = ("rho_bar", "noa_bar", "acs_bar")


def _mix(x):
    """splitmix64 finaliser on uint64 arrays (wraps modulo 2^64): a hash independent of numpy's
    random streams, so the positions and signs are the same on every machine."""
    x = np.asarray(x, dtype=np.uint64)
    with np.errstate(over="ignore"):
        x = x + np.uint64(0x9E3779B97F4A7C15)
        x = (x ^ (x >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
        x = (x ^ (x >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
        return x ^ (x >> np.uint64(31))


def signs(n: int, k: int) -> np.ndarray:
    """The k-th +-1 projection vector of length n."""
    h = _mix(np.arange(n, dtype=np.uint64) + np.uint64((k + 1) << 40))
    return 1.0 - 2.0 * (h >> np.uint64(63)).astype(np.float64)


def hashed_positions(n: int, count: int) -> np.ndarray:
    h = _mix(np.arange(n, dtype=np.uint64) ^ np.uint64(0x5DEECE66D))
    return np.sort(np.argsort(h, kind="stable")[:min(count, n)])


def summarise(g: np.ndarray, positions=None) -> dict:
    """Positions, values, projections, 1-norm and largest magnitude of a flat array.  With
    `positions` given (the stored ones), the values are taken there."""
    g = np.asarray(g, dtype=np.float64).ravel()
    if positions is None:
        top = np.argsort(-np.abs(g), kind="stable")[:N_TOP]
        positions = np.union1d(top, hashed_positions(g.size, N_HASHED))
    return {
        "pos": np.asarray(positions, dtype=np.int64),
        "val": g[positions],
        "proj": np.array([signs(g.size, k) @ g for k in range(N_PROJ)]),
        "l1": np.array(np.sum(np.abs(g))),
        "amax": np.array(np.max(np.abs(g))),
        "n": np.array(g.size),
    }


def compare(got: np.ndarray, stored: dict) -> dict:
    """Errors of `got` against a stored summary: normwise (largest difference at the stored
    positions over the largest magnitude), per element at the stored positions whose magnitude
    is at least 1e-3 of the largest, and of the projections over the 1-norm."""
    got = np.asarray(got, dtype=np.float64).ravel()
    assert got.size == int(stored["n"])
    pos, ref = stored["pos"], stored["val"]
    amax = float(stored["amax"])
    d = np.abs(got[pos] - ref)
    big = np.abs(ref) >= 1e-3 * amax
    proj = np.array([signs(got.size, k) @ got for k in range(N_PROJ)])
    return {
        "normwise": float(np.max(d) / amax),
        "per_element": float(np.max(d[big] / np.abs(ref[big]))) if big.any() else 0.0,
        "projection": float(np.max(np.abs(proj - stored["proj"])) / float(stored["l1"])),
        "amax": float(abs(np.max(np.abs(got)) - amax) / amax),
    }


def config1_case():
    from pnepma_gb300 import workloads
    return workloads.config1()


def config2_cases(precision=None):
    """The three config-2 solves (one per energy, position CONFIG2_POSITION), FP64 unless given."""
    from pnepma_gb300 import workloads
    from pnepma_gb300.problem import PN_FP64
    sv = workloads.config2(precision=precision if precision is not None else PN_FP64)
    per_e = len(sv) // len(CONFIG2_ENERGIES)
    return {f"config2_{int(E)}kev": sv[i * per_e + CONFIG2_POSITION] for i, E in enumerate(CONFIG2_ENERGIES)}


def load() -> dict:
    """The stored fixtures as {case: {"I", "ibar", output: full array or summary}}."""
    Z = np.load(PATH)
    out: dict = {}
    for key in Z.files:
        parts = key.split("/")
        d = out.setdefault(parts[0], {})
        if len(parts) == 2:
            d[parts[1]] = Z[key]
        else:
            d.setdefault(parts[1], {})[parts[2]] = Z[key]
    return out


def _solve(oracle, s):
    desc, keep = s.problem.descriptor(s.x_rays)
    rho, noa, acs = s.inputs()
    I0 = oracle.forward(desc, rho, noa, acs)
    ibar = np.linspace(1.0, 2.0, len(I0)) / np.abs(I0)
    I, rb, nb, ab = oracle.adjoint(desc, rho, noa, acs, ibar)
    return ibar, I, rb, nb, ab


def generate():
    for p in (ROOT, os.path.join(ROOT, "oracle")):
        if p not in sys.path:
            sys.path.insert(0, p)
    import oracle
    oracle.set_threads(os.cpu_count() or 1)
    out = {}
    t0 = time.time()
    s = config1_case()
    ibar, I, rb, nb, ab = _solve(oracle, s)
    out.update({"config1/ibar": ibar, "config1/I": I, "config1/rho_bar": rb, "config1/noa_bar": nb,
                "config1/acs_bar": ab, "config1/n_steps": np.array(s.problem.N_steps)})
    print(f"config1: {s.problem.N_steps} steps, {time.time() - t0:.1f} s", flush=True)
    for name, s in config2_cases().items():
        t0 = time.time()
        ibar, I, rb, nb, ab = _solve(oracle, s)
        out[f"{name}/ibar"] = ibar
        out[f"{name}/I"] = I
        out[f"{name}/n_steps"] = np.array(s.problem.N_steps)
        for o, g in zip(OUTPUTS, (rb, nb, ab)):
            for k, v in summarise(g).items():
                out[f"{name}/{o}/{k}"] = v
        print(f"{name}: {s.problem.N_steps} steps, {time.time() - t0:.1f} s", flush=True)
    np.savez_compressed(PATH, **out)
    return out


if __name__ == "__main__":
    generate()
    print(PATH, os.path.getsize(PATH), "bytes")
