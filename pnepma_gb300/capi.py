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


PN_BATCH_GENERIC_KERNELS = 1
PN_BATCH_DIRECT_LAUNCH = 2
PN_BATCH_TEST_EXPIRE_WAIT = 4
PN_BATCH_SWEEP_LAUNCH = 16
PN_BATCH_PARITY_TILES = 32
PN_BATCH_CTAS_PER_SM_SHIFT = 8


class PnBatchOptions(ctypes.Structure):
    _fields_ = [("memory_budget", ctypes.c_int64), ("checkpoint_stride", ctypes.c_int32),
                ("flags", ctypes.c_int32)]


class PnBatchInfo(ctypes.Structure):
    _fields_ = [("n_solves", ctypes.c_int32), ("n_groups", ctypes.c_int32),
                ("checkpoint_stride", ctypes.c_int32), ("tma_groups", ctypes.c_int32),
                ("device_bytes", ctypes.c_int64), ("forward_kernels", ctypes.c_int64),
                ("adjoint_kernels", ctypes.c_int64), ("recomputed_steps", ctypes.c_int64)]


class PnServerOptions(ctypes.Structure):
    _fields_ = [("memory_budget", ctypes.c_int64), ("max_waves", ctypes.c_int32),
                ("max_wave_solves", ctypes.c_int32), ("checkpoint_stride", ctypes.c_int32),
                ("reserved", ctypes.c_int32 * 3)]


class PnRequest(ctypes.Structure):
    _fields_ = [("n_solves", ctypes.c_int32), ("adjoint", ctypes.c_int32)] + [
        (name, ctypes.c_void_p) for name in ("descs", "rho", "noa", "acs", "intensities_bar", "intensities",
                                             "rho_bar", "noa_bar", "acs_bar")]


class PnTicketInfo(ctypes.Structure):
    _fields_ = [("done", ctypes.c_int32), ("status", ctypes.c_int32), ("wave", ctypes.c_int32),
                ("reserved", ctypes.c_int32), ("queued_ms", ctypes.c_double), ("total_ms", ctypes.c_double)]


class PnServerInfo(ctypes.Structure):
    _fields_ = [(name, ctypes.c_int64) for name in ("memory_budget", "bytes_in_use", "peak_bytes",
                                                     "requests_submitted", "requests_done", "solves_done",
                                                     "waves_launched")] + [
        ("waves_in_flight", ctypes.c_int32), ("max_waves_in_flight", ctypes.c_int32),
        ("wave_build_us", ctypes.c_int64)]


SERVER_EXPORTS = ("pn_server_create", "pn_submit", "pn_poll", "pn_wait", "pn_server_query", "pn_server_destroy")

EXPORTS = SERVER_EXPORTS + ("pn_batch_create", "pn_batch_forward", "pn_batch_adjoint", "pn_batch_query", "pn_batch_destroy",
           "pn_forward_noalloc", "pn_query_handle", "pn_query_sizes", "pn_create", "pn_forward", "pn_adjoint", "pn_forward_device", "pn_adjoint_device",
           "pn_generation_field", "pn_set_state", "pn_step", "pn_get_state", "pn_destroy", "pn_last_error",
           "pn_abi_version", "pn_compiled_orders", "pn_probe_fp64_fma", "pn_material_create", "pn_material_fields",
           "pn_material_pullback", "pn_material_destroy")


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
        L.pn_server_create.argtypes = [ctypes.POINTER(PnServerOptions), ctypes.POINTER(P)]
        L.pn_submit.argtypes = [P, ctypes.POINTER(PnRequest), ctypes.POINTER(ctypes.c_uint64)]
        L.pn_poll.argtypes = [P, ctypes.c_uint64, ctypes.POINTER(PnTicketInfo)]
        L.pn_wait.argtypes = [P, ctypes.c_uint64, ctypes.c_int64]
        L.pn_server_query.argtypes = [P, ctypes.POINTER(PnServerInfo)]
        for name in ("pn_server_create", "pn_submit", "pn_poll", "pn_wait", "pn_server_query"):
            getattr(L, name).restype = ctypes.c_int
        L.pn_server_destroy.argtypes = [P]
        L.pn_server_destroy.restype = None
        L.pn_selftest_phi1.argtypes = [ctypes.c_int32, P, P, P]
        L.pn_selftest_phi1.restype = ctypes.c_int
        L.pn_selftest_phi1_f64.argtypes = [ctypes.c_int32, P, P]
        L.pn_selftest_phi1_f64.restype = ctypes.c_int
        L.pn_probe_fp64_fma.argtypes = [ctypes.c_int32, ctypes.c_int32, P, P]
        L.pn_probe_fp64_fma.restype = ctypes.c_int
        L.pn_material_create.argtypes = [P, ctypes.POINTER(P), ctypes.POINTER(ctypes.c_int64)]
        L.pn_material_create.restype = ctypes.c_int
        L.pn_material_fields.argtypes = [P, P, P, P, P, P]
        L.pn_material_fields.restype = ctypes.c_int
        L.pn_material_pullback.argtypes = [P, P, P, P, P, P, P, P]
        L.pn_material_pullback.restype = ctypes.c_int
        L.pn_material_destroy.argtypes = [P]
        L.pn_material_destroy.restype = None
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
        arr[i] = p.ctypes.data if isinstance(p, np.ndarray) else int(p)
    return arr


class Batch:
    """Owns one ``pn_batch``: many solves marched together (device-pointer interface)."""

    def __init__(self, descs, keepalive=None, memory_budget: int = 0, checkpoint_stride: int = 0, flags: int = 0):
        self.descs = list(descs)
        self._keep = keepalive
        self.sizes = [query_sizes(d) for d in self.descs]
        arr = (ctypes.c_void_p * len(self.descs))()
        for i, d in enumerate(self.descs):
            arr[i] = ctypes.addressof(d)
        self._arr = arr
        opt = PnBatchOptions(int(memory_budget), int(checkpoint_stride), int(flags))
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


class Ticket:
    """One submitted request: keeps its inputs and descriptors alive and owns its host outputs."""

    def __init__(self, server, tid, solves, adjoint, keep):
        self.server = server
        self.id = tid
        self.adjoint = adjoint
        self._keep = keep
        self.intensities = keep["I"]
        self.rho_bar = keep["rb"] if adjoint else None
        self.noa_bar = keep["nb"] if adjoint else None
        self.acs_bar = keep["ab"] if adjoint else None

    def info(self) -> PnTicketInfo:
        out = PnTicketInfo()
        rc = lib().pn_poll(self.server._s, self.id, ctypes.byref(out))
        if rc:
            raise PnError(rc, lib().pn_last_error(None).decode())
        return out

    def done(self) -> bool:
        return bool(self.info().done)

    def wait(self, timeout_ms: int = -1):
        """Block until done; raises PnError if the request failed.  Returns (I, rho_bar, noa_bar,
        acs_bar) lists, one entry per solve (the adjoint lists are None for a forward request)."""
        rc = lib().pn_wait(self.server._s, self.id, int(timeout_ms))
        if rc:
            raise PnError(rc, lib().pn_last_error(None).decode())
        return self.intensities, self.rho_bar, self.noa_bar, self.acs_bar


class Server:
    """Owns one ``pn_server``: continuous batching of host-buffer requests on one GPU."""

    def __init__(self, memory_budget: int = 0, max_waves: int = 0, max_wave_solves: int = 0,
                 checkpoint_stride: int = 0):
        opt = PnServerOptions(int(memory_budget), int(max_waves), int(max_wave_solves), int(checkpoint_stride))
        s = ctypes.c_void_p()
        rc = lib().pn_server_create(ctypes.byref(opt), ctypes.byref(s))
        if rc:
            raise PnError(rc, lib().pn_last_error(None).decode())
        self._s = s

    def submit(self, solves, adjoint: bool = True, outputs=None) -> Ticket:
        """solves: list of (desc, rho, noa, acs, ibar) with host numpy inputs (ibar ignored for a
        forward request).  Arrays passed as the same object are uploaded once per wave.  `outputs`
        optionally gives, per solve, contiguous float64 arrays (intensities, rho_bar, noa_bar,
        acs_bar) of the sizes pn_query_sizes states, which receive the results instead of new
        arrays."""
        n = len(solves)
        descs = (ctypes.c_void_p * n)()
        keep = {"descs": [], "in": [], "I": [], "rb": [], "nb": [], "ab": []}
        conv = {}

        def host(a):
            k = id(a)
            if k not in conv:
                conv[k] = _f64(a)
                keep["in"].append((a, conv[k]))
            return conv[k]

        arrs = {k: [] for k in ("rho", "noa", "acs", "ibar")}
        for i, (d, rho, noa, acs, ibar) in enumerate(solves):
            descs[i] = ctypes.addressof(d)
            keep["descs"].append(d)
            z = query_sizes(d)
            arrs["rho"].append(host(rho))
            arrs["noa"].append(host(noa))
            arrs["acs"].append(host(acs))
            arrs["ibar"].append(host(ibar) if adjoint else None)
            if outputs is not None:
                oI, orb, onb, oab = outputs[i]
                for a, nmin in ((oI, d.n_xrays), (orb, z.n_rho), (onb, z.n_noa), (oab, z.n_acs)):
                    if a.dtype != np.float64 or not a.flags["C_CONTIGUOUS"] or a.size < nmin:
                        raise ValueError("outputs must be contiguous float64 arrays of the queried sizes")
                keep["I"].append(oI)
                if adjoint:
                    keep["rb"].append(orb)
                    keep["nb"].append(onb)
                    keep["ab"].append(oab)
                continue
            keep["I"].append(np.zeros(d.n_xrays))
            if adjoint:
                keep["rb"].append(np.zeros(z.n_rho))
                keep["nb"].append(np.zeros(z.n_noa))
                keep["ab"].append(np.zeros(z.n_acs))
        req = PnRequest()
        req.n_solves = n
        req.adjoint = 1 if adjoint else 0
        ptrs = {"descs": descs, "rho": _ptr_array(arrs["rho"]), "noa": _ptr_array(arrs["noa"]),
                "acs": _ptr_array(arrs["acs"]), "intensities": _ptr_array(keep["I"])}
        if adjoint:
            ptrs.update(intensities_bar=_ptr_array(arrs["ibar"]), rho_bar=_ptr_array(keep["rb"]),
                        noa_bar=_ptr_array(keep["nb"]), acs_bar=_ptr_array(keep["ab"]))
        for k, v in ptrs.items():
            setattr(req, k, ctypes.cast(v, ctypes.c_void_p))
        keep["ptrs"] = ptrs
        tid = ctypes.c_uint64()
        rc = lib().pn_submit(self._s, ctypes.byref(req), ctypes.byref(tid))
        if rc:
            raise PnError(rc, lib().pn_last_error(None).decode())
        return Ticket(self, tid.value, solves, adjoint, keep)

    def info(self) -> PnServerInfo:
        out = PnServerInfo()
        rc = lib().pn_server_query(self._s, ctypes.byref(out))
        if rc:
            raise PnError(rc, lib().pn_last_error(None).decode())
        return out

    def close(self):
        if getattr(self, "_s", None):
            lib().pn_server_destroy(self._s)
            self._s = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class DeviceMaterial:
    """Owns one ``pn_material``: a material model whose fields and pullbacks run on the GPU.

    `model` is a ``material_model.MaterialModel``.  The calls take device pointers (ints) and are
    ordered on `stream` (a cudaStream_t as int, 0 = legacy default stream)."""

    def __init__(self, model):
        self.model = model
        self.desc, self._keep = model.descriptor()
        m = ctypes.c_void_p()
        n = ctypes.c_int64()
        rc = lib().pn_material_create(ctypes.byref(self.desc), ctypes.byref(m), ctypes.byref(n))
        if rc:
            raise PnError(rc, lib().pn_last_error(None).decode())
        self._m = m
        self.n_params = int(n.value)

    def _check(self, rc):
        if rc:
            raise PnError(rc, lib().pn_last_error(None).decode())

    def fields(self, params, rho=None, noa=None, acs=None, stream=0):
        self._check(lib().pn_material_fields(self._m, _ptr(params), _ptr(rho), _ptr(noa), _ptr(acs), _ptr(stream)))

    def pullback(self, params, params_bar, rho_bar=None, noa_bar=None, acs=None, acs_bar=None, stream=0):
        self._check(lib().pn_material_pullback(self._m, _ptr(params), _ptr(rho_bar), _ptr(noa_bar), _ptr(acs),
                                               _ptr(acs_bar), _ptr(params_bar), _ptr(stream)))

    def close(self):
        if getattr(self, "_m", None):
            lib().pn_material_destroy(self._m)
            self._m = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
