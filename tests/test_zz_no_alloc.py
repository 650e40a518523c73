"""pn_forward_noalloc: the forward march for callers that cannot allocate device memory.

Those callers (a process whose GPU memory belongs to another allocator, a latency-bound loop that
must not call cudaMalloc/cudaFree) pass device buffers they own; the entry point takes all of its
scratch from one fixed library array.  These tests call it through the C ABI twice in a row (on the
legacy default stream, then on a stream of the caller's) and compare with pn_forward, within the
FP64 parity tolerance of the other GPU tests, and check that it rejects what pn_create rejects.  The file is
named so that pytest collects it last.
"""
import ctypes

import numpy as np
import pytest

from pnepma_gb300 import capi, workloads

pytestmark = pytest.mark.gpu

TOL64 = 1e-10
PN_ERR_UNSUPPORTED = -2
PN_ERR_NO_MEMORY = -4


def _rel(a, b):
    return float(np.max(np.abs(np.asarray(a) - np.asarray(b))) / np.max(np.abs(b)))


def _dev(torch, a):
    return torch.from_numpy(np.ascontiguousarray(a, dtype=np.float64)).cuda()


@pytest.mark.parametrize("case", [dict(dims=2, N=5, shape=(12, 9), n_steps=8),
                                  dict(dims=1, N=7, shape=(24,), n_steps=10),
                                  dict(dims=3, N=3, shape=(7, 6, 5), n_steps=6)],
                         ids=["2d-N5", "1d-N7", "3d-N3"])
def test_noalloc_matches_pn_forward_twice(gpu_lib, case):
    torch = pytest.importorskip("torch")
    L = capi.lib()
    s = workloads.small_case(**case)
    rho, noa, acs = s.inputs()
    desc, keep = s.problem.descriptor(s.x_rays)
    h = capi.Handle(desc, keep)
    I_ref = h.forward(rho, noa, acs)
    h.close()
    d_rho, d_noa, d_acs = _dev(torch, rho), _dev(torch, noa), _dev(torch, acs)
    d_I = torch.full((len(s.x_rays),), float("nan"), dtype=torch.float64, device="cuda")
    side = torch.cuda.Stream()
    # two calls in a row: on the legacy default stream, then on a stream of the caller's
    for stream in (None, side):
        d_I.fill_(float("nan"))
        torch.cuda.synchronize()
        rc = L.pn_forward_noalloc(ctypes.byref(desc), ctypes.c_void_p(d_rho.data_ptr()),
                                  ctypes.c_void_p(d_noa.data_ptr()), ctypes.c_void_p(d_acs.data_ptr()),
                                  ctypes.c_void_p(d_I.data_ptr()),
                                  None if stream is None else ctypes.c_void_p(stream.cuda_stream))
        assert rc == 0, L.pn_last_error(None).decode()
        torch.cuda.synchronize()
        assert _rel(d_I.cpu().numpy(), I_ref) < TOL64


def test_noalloc_rejects_problems_beyond_its_scratch(gpu_lib):
    L = capi.lib()
    s = workloads.small_case(dims=2, N=11, shape=(400, 400), n_steps=2, stabilise=False)
    desc, keep = s.problem.descriptor(s.x_rays)
    one = np.zeros(1)
    p = ctypes.c_void_p(one.ctypes.data)
    rc = L.pn_forward_noalloc(ctypes.byref(desc), p, p, p, p, None)
    assert rc == PN_ERR_NO_MEMORY
    msg = L.pn_last_error(None).decode()
    assert "bytes of scratch" in msg


def test_noalloc_rejects_grids_beyond_the_cell_packing(gpu_lib):
    """A z extent above 1000 cells does not fit the packed face-cell index; the entry point rejects
    it before any device work, as pn_create does."""
    L = capi.lib()
    s = workloads.small_case(dims=3, N=1, shape=(3, 3, 1001), n_steps=1, stabilise=False)
    desc, keep = s.problem.descriptor(s.x_rays)
    assert desc.n_points[2] == 1001
    one = np.zeros(1)
    p = ctypes.c_void_p(one.ctypes.data)
    rc = L.pn_forward_noalloc(ctypes.byref(desc), p, p, p, p, None)
    assert rc == PN_ERR_UNSUPPORTED
    assert "cell packing" in L.pn_last_error(None).decode()
