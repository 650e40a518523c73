"""ctypes front end of the CPU oracle (test infrastructure only: the tests, the smoke check and
the benchmark's CPU-baseline leg use it as the checker; the library never imports it)."""
from __future__ import annotations

import ctypes
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
import build as _build  # noqa: E402

_lib = None


def lib():
    global _lib
    if _lib is None:
        path = _build.build()
        L = ctypes.CDLL(path)
        P = ctypes.c_void_p
        L.ora_state_size.argtypes = [P]
        L.ora_state_size.restype = ctypes.c_int64
        L.ora_rho_size.argtypes = [P]
        L.ora_rho_size.restype = ctypes.c_int64
        L.ora_forward.argtypes = [P, P, P, P, P, P]
        L.ora_adjoint.argtypes = [P, P, P, P, P, P, P, P, P]
        L.ora_generation_field.argtypes = [P, P, P]
        L.ora_step.argtypes = [P, P, P, ctypes.c_int]
        L.ora_solve_many.argtypes = [P] * 9 + [ctypes.c_int, ctypes.c_int]
        L.ora_set_threads.argtypes = [ctypes.c_int]
        L.ora_set_threads.restype = ctypes.c_int
        L.ora_openmp.restype = ctypes.c_int
        _lib = L
    return _lib


def set_threads(n: int) -> int:
    """Host threads of each following solve; returns the count in effect (1 without OpenMP)."""
    return int(lib().ora_set_threads(int(n)))


def threads_available() -> int:
    """Threads a solve can use: the host's cores when the oracle was built with OpenMP, else 1."""
    return (os.cpu_count() or 1) if lib().ora_openmp() else 1


def _p(a):
    return a.ctypes.data_as(ctypes.c_void_p) if a is not None else None


def _f64(a):
    return np.ascontiguousarray(a, dtype=np.float64)


def state_size(desc) -> int:
    return int(lib().ora_state_size(ctypes.byref(desc)))


def forward(desc, rho, noa, acs, with_tape: bool = False):
    rho, noa, acs = _f64(rho), _f64(noa), _f64(acs)
    I = np.zeros(desc.n_xrays)
    tape = np.zeros((desc.n_steps + 1, state_size(desc))) if with_tape else None
    rc = lib().ora_forward(ctypes.byref(desc), _p(rho), _p(noa), _p(acs), _p(I), _p(tape))
    if rc:
        raise RuntimeError(f"oracle forward failed ({rc})")
    return (I, tape) if with_tape else I


def adjoint(desc, rho, noa, acs, Ibar):
    rho, noa, acs, Ibar = _f64(rho), _f64(noa), _f64(acs), _f64(Ibar)
    I = np.zeros(desc.n_xrays)
    rho_bar = np.zeros_like(rho)
    noa_bar = np.zeros_like(noa)
    acs_bar = np.zeros_like(acs)
    rc = lib().ora_adjoint(ctypes.byref(desc), _p(rho), _p(noa), _p(acs), _p(Ibar), _p(I), _p(rho_bar),
                           _p(noa_bar), _p(acs_bar))
    if rc:
        raise RuntimeError(f"oracle adjoint failed ({rc})")
    return I, rho_bar, noa_bar, acs_bar


def generation_field(desc, rho):
    rho = _f64(rho)
    ncell = None
    # eee cells = product of M over non-singleton axes
    ncell = 1
    for d in range(3):
        ncell *= desc.n_points[d]
    out = np.zeros((ncell, desc.n_xrays))
    rc = lib().ora_generation_field(ctypes.byref(desc), _p(rho), _p(out))
    if rc:
        raise RuntimeError(f"oracle generation field failed ({rc})")
    return out


def step(desc, rho, state, i):
    rho = _f64(rho)
    st = _f64(state).copy()
    rc = lib().ora_step(ctypes.byref(desc), _p(rho), _p(st), int(i))
    if rc:
        raise RuntimeError(f"oracle step failed ({rc})")
    return st


def solve_many(descs, rhos, noas, acss, Ibars, threads: int):
    """Forward + adjoint of many independent solves on `threads` host threads."""
    n = len(descs)
    outs_I = [np.zeros(d.n_xrays) for d in descs]
    outs_rb = [np.zeros_like(r) for r in rhos]
    outs_nb = [np.zeros_like(a) for a in noas]
    outs_ab = [np.zeros_like(a) for a in acss]

    def arr(lst):
        A = (ctypes.c_void_p * n)()
        for i, x in enumerate(lst):
            A[i] = ctypes.addressof(x) if isinstance(x, ctypes.Structure) else x.ctypes.data
        return A

    rc = lib().ora_solve_many(arr(descs), arr(rhos), arr(noas), arr(acss), arr(Ibars), arr(outs_I),
                              arr(outs_rb), arr(outs_nb), arr(outs_ab), n, int(threads))
    if rc:
        raise RuntimeError(f"oracle solve_many failed ({rc})")
    return outs_I, outs_rb, outs_nb, outs_ab
