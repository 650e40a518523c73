"""ctypes binding of ``libpnepma_gb300.so`` (the C ABI in ``include/pnepma.h``).

The library is loaded from the in-tree build directory.  There is no fallback: if the library is
missing or cannot be loaded, :func:`lib` raises, so no solve can silently run anywhere but on the
GPU kernels.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

from .problem import PnDesc, PnSizes

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libpnepma_gb300.so")

STATUS = {
    0: "PN_OK", -1: "PN_ERR_INVALID", -2: "PN_ERR_UNSUPPORTED", -3: "PN_ERR_CFL", -4: "PN_ERR_NO_MEMORY",
    -5: "PN_ERR_DIVERGED", -6: "PN_ERR_TIMEOUT", -7: "PN_ERR_CUDA", -8: "PN_ERR_STATE", -9: "PN_ERR_NO_DEVICE",
}

class PnHandleInfo(ctypes.Structure):
    _fields_ = [("checkpoint_stride", ctypes.c_int32), ("precision", ctypes.c_int32),
                ("device_bytes", ctypes.c_int64), ("forward_kernels", ctypes.c_int64),
                ("adjoint_kernels", ctypes.c_int64)]


class PnBatchOptions(ctypes.Structure):
    _fields_ = [("memory_budget", ctypes.c_int64), ("checkpoint_stride", ctypes.c_int32),
                ("reserved", ctypes.c_int32)]


class PnBatchInfo(ctypes.Structure):
    _fields_ = [("n_solves", ctypes.c_int32), ("n_groups", ctypes.c_int32),
                ("checkpoint_stride", ctypes.c_int32), ("reserved", ctypes.c_int32),
                ("device_bytes", ctypes.c_int64), ("forward_kernels", ctypes.c_int64),
                ("adjoint_kernels", ctypes.c_int64)]


EXPORTS = ("pn_batch_create", "pn_batch_forward", "pn_batch_adjoint", "pn_batch_query", "pn_batch_destroy",
           "pn_forward_noalloc", "pn_query_handle", "pn_query_sizes", "pn_create", "pn_forward", "pn_adjoint", "pn_forward_device", "pn_adjoint_device",
           "pn_generation_field", "pn_set_state", "pn_step", "pn_get_state", "pn_destroy", "pn_last_error",
           "pn_abi_version", "pn_compiled_orders")


class PnError(RuntimeError):
    def __init__(self, code: int, message: str):
        super().__init__(f"{STATUS.get(code, code)}: {message}")
        self.code = code


_lib = None


def lib():
    """Load the library (raises if it has not been built)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(f"{LIB_PATH} is missing: build it with `python -m pnepma_gb300.build` "
                               "(or __graft_entry__.build()); there is no CPU fallback")
        L = ctypes.CDLL(LIB_PATH)
        P = ctypes.c_void_p
        L.pn_query_sizes.argtypes = [ctypes.POINTER(PnDesc), ctypes.POINTER(PnSizes)]
        L.pn_create.argtypes = [ctypes.POINTER(PnDesc), ctypes.POINTER(P)]
        L.pn_forward.argtypes = [P, P, P, P, P]
        L.pn_adjoint.argtypes = [P, P, P, P, P]
        L.pn_forward_device.argtypes = [P, P, P, P, P, P]
        L.pn_adjoint_device.argtypes = [P, P, P, P, P, P]
        L.pn_generation_field.argtypes = [P, P, P]
        L.pn_set_state.argtypes = [P, P, P]
        L.pn_step.argtypes = [P, ctypes.c_int32]
        L.pn_get_state.argtypes = [P, P]
        L.pn_batch_create.argtypes = [P, ctypes.c_int32, ctypes.POINTER(PnBatchOptions), ctypes.POINTER(P)]
        L.pn_batch_create.restype = ctypes.c_int
        L.pn_batch_forward.argtypes = [P, P, P, P, P, P]
        L.pn_batch_forward.restype = ctypes.c_int
        L.pn_batch_adjoint.argtypes = [P, P, P, P, P, P]
        L.pn_batch_adjoint.restype = ctypes.c_int
        L.pn_batch_query.argtypes = [P, ctypes.POINTER(PnBatchInfo)]
        L.pn_batch_query.restype = ctypes.c_int
        L.pn_batch_destroy.argtypes = [P]
        L.pn_batch_destroy.restype = None
        L.pn_forward_noalloc.argtypes = [ctypes.POINTER(PnDesc), P, P, P, P, P]
        L.pn_forward_noalloc.restype = ctypes.c_int
        L.pn_query_handle.argtypes = [P, ctypes.POINTER(PnHandleInfo)]
        L.pn_query_handle.restype = ctypes.c_int
        L.pn_destroy.argtypes = [P]
        L.pn_destroy.restype = None
        L.pn_last_error.argtypes = [P]
        L.pn_last_error.restype = ctypes.c_char_p
        L.pn_abi_version.restype = ctypes.c_int32
        L.pn_compiled_orders.restype = ctypes.c_int64
        for name in ("pn_query_sizes", "pn_create", "pn_forward", "pn_adjoint", "pn_forward_device",
                     "pn_adjoint_device", "pn_generation_field", "pn_set_state", "pn_step", "pn_get_state"):
            getattr(L, name).restype = ctypes.c_int
        _lib = L
    return _lib


def _ptr(a):
    if a is None:
        return None
    if isinstance(a, int):
        return ctypes.c_void_p(a)
    return a.ctypes.data_as(ctypes.c_void_p)


def _f64(a):
    return np.ascontiguousarray(a, dtype=np.float64)


def query_sizes(desc: PnDesc) -> PnSizes:
    s = PnSizes()
    rc = lib().pn_query_sizes(ctypes.byref(desc), ctypes.byref(s))
    if rc:
        raise PnError(rc, lib().pn_last_error(None).decode())
    return s


class Handle:
    """Owns one ``pn_handle``: a problem compiled onto the GPU with its tape."""

    def __init__(self, desc: PnDesc, keepalive=None):
        self.desc = desc
        self._keep = keepalive
        self.sizes = query_sizes(desc)
        h = ctypes.c_void_p()
        rc = lib().pn_create(ctypes.byref(desc), ctypes.byref(h))
        if rc:
            raise PnError(rc, lib().pn_last_error(None).decode())
        self._h = h

    def _check(self, rc):
        if rc:
            raise PnError(rc, lib().pn_last_error(self._h).decode())

    def info(self) -> PnHandleInfo:
        out = PnHandleInfo()
        self._check(lib().pn_query_handle(self._h, ctypes.byref(out)))
        return out

    def close(self):
        if getattr(self, "_h", None):
            lib().pn_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def forward(self, rho, noa, acs):
        rho, noa, acs = _f64(rho), _f64(noa), _f64(acs)
        self._check_len(rho, self.sizes.n_rho, "rho")
        self._check_len(noa, self.sizes.n_noa, "noa")
        self._check_len(acs, self.sizes.n_acs, "acs")
        I = np.zeros(self.desc.n_xrays)
        self._check(lib().pn_forward(self._h, _ptr(rho), _ptr(noa), _ptr(acs), _ptr(I)))
        return I

    def adjoint(self, ibar):
        ibar = _f64(ibar)
        rho_bar = np.zeros(self.sizes.n_rho)
        noa_bar = np.zeros(self.sizes.n_noa)
        acs_bar = np.zeros(self.sizes.n_acs)
        self._check(lib().pn_adjoint(self._h, _ptr(ibar), _ptr(rho_bar), _ptr(noa_bar), _ptr(acs_bar)))
        return rho_bar, noa_bar.reshape(-1, self.desc.n_elements), acs_bar.reshape(-1, self.desc.n_xrays)

    def forward_device(self, rho, noa, acs, out, stream=0):
        """Device pointers (ints) in and out; ordered on `stream` (a cudaStream_t as int)."""
        self._check(lib().pn_forward_device(self._h, _ptr(rho), _ptr(noa), _ptr(acs), _ptr(out), _ptr(stream)))

    def adjoint_device(self, ibar, rho_bar, noa_bar, acs_bar, stream=0):
        self._check(lib().pn_adjoint_device(self._h, _ptr(ibar), _ptr(rho_bar), _ptr(noa_bar), _ptr(acs_bar),
                                            _ptr(stream)))

    def generation_field(self, rho):
        rho = _f64(rho)
        out = np.zeros((self.sizes.n_eee_cells, self.desc.n_xrays))
        self._check(lib().pn_generation_field(self._h, _ptr(rho), _ptr(out)))
        return out

    def set_state(self, rho, state):
        rho, state = _f64(rho), _f64(state)
        self._check_len(state, self.sizes.n_state, "state")
        self._check(lib().pn_set_state(self._h, _ptr(rho), _ptr(state)))

    def step(self, i: int):
        self._check(lib().pn_step(self._h, int(i)))

    def get_state(self):
        out = np.zeros(self.sizes.n_state)
        self._check(lib().pn_get_state(self._h, _ptr(out)))
        return out

    @staticmethod
    def _check_len(a, n, name):
        if a.size != n:
            raise ValueError(f"{name} has {a.size} values, expected {n}")


def _ptr_array(ptrs):
    arr = (ctypes.c_void_p * len(ptrs))()
    for i, p in enumerate(ptrs):
        arr[i] = int(p)
    return arr


class Batch:
    """Owns one ``pn_batch``: many solves marched together (device-pointer interface)."""

    def __init__(self, descs, keepalive=None, memory_budget: int = 0, checkpoint_stride: int = 0):
        self.descs = list(descs)
        self._keep = keepalive
        self.sizes = [query_sizes(d) for d in self.descs]
        arr = (ctypes.c_void_p * len(self.descs))()
        for i, d in enumerate(self.descs):
            arr[i] = ctypes.addressof(d)
        self._arr = arr
        opt = PnBatchOptions(int(memory_budget), int(checkpoint_stride), 0)
        b = ctypes.c_void_p()
        rc = lib().pn_batch_create(arr, len(self.descs), ctypes.byref(opt), ctypes.byref(b))
        if rc:
            raise PnError(rc, lib().pn_last_error(None).decode())
        self._b = b

    def _check(self, rc):
        if rc:
            raise PnError(rc, lib().pn_last_error(None).decode())

    def info(self) -> PnBatchInfo:
        out = PnBatchInfo()
        self._check(lib().pn_batch_query(self._b, ctypes.byref(out)))
        return out

    def forward(self, rho, noa, acs, intensities, stream=0):
        """Lists of device pointers (ints), one per solve."""
        self._check(lib().pn_batch_forward(self._b, _ptr_array(rho), _ptr_array(noa), _ptr_array(acs),
                                           _ptr_array(intensities), _ptr(stream)))

    def adjoint(self, ibar, rho_bar, noa_bar, acs_bar, stream=0):
        self._check(lib().pn_batch_adjoint(self._b, _ptr_array(ibar), _ptr_array(rho_bar), _ptr_array(noa_bar),
                                           _ptr_array(acs_bar), _ptr(stream)))

    def close(self):
        if getattr(self, "_b", None):
            lib().pn_batch_destroy(self._b)
            self._b = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
