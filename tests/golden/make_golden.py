"""Regenerate the golden vectors of tests/golden/oracle_small_cases.npz from the oracle.

    python tests/golden/make_golden.py

The reference ships no golden vectors or fixtures for this path, and it cannot run here (Julia is
absent), so these vectors come from the CPU restatement (oracle/): forward intensities and
adjoint outputs of seeded small solves in 1D, 2D and 3D, and the device-material fields and
pullback of a seeded Bilinear MassFractionSC material.  They pin the oracle against drift
(tests/test_golden_cpu.py) and give the GPU tests committed vectors to compare with
(tests/test_gpu_vs_golden.py).  Every input is regenerated from its seed by the case functions below.
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
PATH = os.path.join(HERE, "oracle_small_cases.npz")

SOLVES = {
    "1d_n7": dict(dims=1, N=7, shape=(24,), n_steps=10),
    "2d_n5": dict(dims=2, N=5, shape=(12, 9), n_steps=8),
    "3d_n3": dict(dims=3, N=3, shape=(7, 6, 5), n_steps=6),
}
UM = 1e-4


def solve_case(name):
    """(solve, desc, keep, rho, noa, acs, ibar) of a seeded solve case."""
    from pnepma_gb300 import workloads
    s = workloads.small_case(**SOLVES[name])
    desc, keep = s.problem.descriptor(s.x_rays)
    rho, noa, acs = s.inputs()
    ibar = np.linspace(1.0, 2.0, len(s.x_rays))
    return s, desc, keep, rho, noa, acs, ibar


def material_case():
    """(MaterialModel, params, rho_bar, noa_bar, acs, acs_bar shapes filled by seeds)."""
    from pnepma_gb300 import physics
    from pnepma_gb300.grid import GridSpec
    from pnepma_gb300.material_model import MaterialModel, Slices
    g = GridSpec.make((7, 5, 1), (-0.5 * UM, 0.0), (-0.3 * UM, 0.3 * UM), 0.0)
    sl = [Slices.range(-0.6 * UM, 0.1 * UM, 5), Slices.range(-0.3 * UM, 0.3 * UM, 3), Slices.range(0.0, 0.0, 1)]
    mm = MaterialModel(g, ["Cu", "Ni", "Fe"], "mass_fraction", sc=True, parametrization="bilinear", slices=sl,
                       x_rays=[physics.XRay(e, "K-L3") for e in ("Cu", "Ni")], detector=(0.3 * UM, 0.05 * UM, 0.0),
                       beam_x=0.0, n_int_points=100)
    rng = np.random.default_rng(31)
    P = mm.random_params(rng)
    n_eee = 7 * 5
    n_rho = sum(g.n_cells(c) for c in range(8)) * mm.n_e
    rb = rng.normal(size=n_rho)
    nb = rng.normal(size=(n_eee, mm.n_e))
    ab = rng.normal(size=(n_eee, len(mm.x_rays)))
    return mm, P, rb, nb, ab


def generate():
    for p in (ROOT, os.path.join(ROOT, "oracle")):
        if p not in sys.path:
            sys.path.insert(0, p)
    import material_oracle as mo
    import oracle
    out = {}
    for name in SOLVES:
        s, desc, keep, rho, noa, acs, ibar = solve_case(name)
        ib = ibar / np.abs(oracle.forward(desc, rho, noa, acs))
        I, rb, nb, ab = oracle.adjoint(desc, rho, noa, acs, ib)
        out[f"{name}/ibar"] = ib
        out[f"{name}/I"] = I
        out[f"{name}/rho_bar"] = rb
        out[f"{name}/noa_bar"] = nb
        out[f"{name}/acs_bar"] = ab
    mm, P, rb, nb, ab = material_case()
    rho, noa, acs = mo.fields(mm, P)
    out["material/rho"], out["material/noa"], out["material/acs"] = rho, noa, acs
    out["material/params_bar"] = mo.pullback(mm, P, rb, nb, acs, ab)
    np.savez_compressed(PATH, **out)
    return out


if __name__ == "__main__":
    out = generate()
    print(PATH, {k: v.shape for k, v in out.items()})
