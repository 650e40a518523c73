"""Served solves (pn_server_*): continuous batching of host-buffer requests.

Each result must be the same alone and in a mix of requests of other orders, dimensions and
grids that share its wave or overlap it on the GPU (bit for bit: a solve's arithmetic and
reduction order do not depend on its neighbours, and the checkpoint stride does not change
results).  The FP64 results are also checked against the oracle.
"""
import time

import numpy as np
import pytest

from pnepma_gb300 import capi, workloads
from pnepma_gb300.problem import PN_FP32, PN_FP64

pytestmark = pytest.mark.gpu


def rel(a, b):
    a = np.asarray(a, float).ravel()
    b = np.asarray(b, float).ravel()
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))


def request(kind, precision, seed):
    """A list of solves sharing one material (as one reconstruction iteration's positions x
    energies do), with the cotangent weights of a k-ratio loss."""
    if kind == "1d":
        base = dict(dims=1, N=7, shape=(20,), n_steps=11)
    elif kind == "2d":
        base = dict(dims=2, N=3, shape=(10, 8), n_steps=9)
    elif kind == "2d5":
        base = dict(dims=2, N=5, shape=(9, 9), n_steps=7)
    else:
        base = dict(dims=3, N=3, shape=(6, 5, 5), n_steps=4)
    out = []
    for j, kev in enumerate((11.0, 12.5)):
        s = workloads.small_case(seed=seed, precision=precision, beam_kev=kev, **base)
        d, keep = s.problem.descriptor(s.x_rays)
        rho, noa, acs = s.inputs()
        ib = np.linspace(1.0, 2.0, len(s.x_rays)) * (1.0 + j)
        out.append((s, d, keep, rho, noa, acs, ib))
    return out


def submit(server, req, adjoint=True):
    return server.submit([(d, rho, noa, acs, ib) for (s, d, keep, rho, noa, acs, ib) in req], adjoint=adjoint)


def outputs(t):
    I, rb, nb, ab = t.wait(timeout_ms=120000)
    return [np.array(x) for x in I], [np.array(x) for x in (rb or [])], [np.array(x) for x in (nb or [])], \
        [np.array(x) for x in (ab or [])]


@pytest.mark.parametrize("precision", [PN_FP32, PN_FP64], ids=["fp32", "fp64"])
def test_result_is_the_same_alone_and_in_a_mix(gpu_lib, oracle, precision):
    target = request("2d", precision, seed=21)
    with capi.Server(memory_budget=2 << 30) as srv:
        alone = outputs(submit(srv, target))
        assert srv.info().waves_launched == 1
    others = [request(k, precision, seed=30 + i) for i, k in enumerate(("1d", "3d", "2d5", "1d", "2d"))]
    with capi.Server(memory_budget=2 << 30, max_waves=3, max_wave_solves=4) as srv:
        ts = [submit(srv, r) for r in others[:3]]
        tt = submit(srv, target)
        ts += [submit(srv, r) for r in others[3:]]
        mixed = outputs(tt)
        for t in ts:
            outputs(t)
        info = srv.info()
        assert info.requests_done == 6 and info.solves_done == 12
    for a, b in zip(alone, mixed):
        for x, y in zip(a, b):
            assert np.array_equal(x, y)
    if precision == PN_FP64:
        for q, (s, d, keep, rho, noa, acs, ib) in enumerate(target):
            I_o, rb_o, nb_o, ab_o = oracle.adjoint(d, rho, noa, acs, ib)
            assert rel(mixed[0][q], I_o) < 1e-10
            assert rel(mixed[1][q], rb_o) < 1e-10
            assert rel(mixed[2][q], nb_o) < 1e-10
            assert rel(mixed[3][q], ab_o) < 1e-10


def test_waves_overlap_and_requests_join_while_others_run(gpu_lib):
    reqs = [request(k, PN_FP32, seed=40 + i) for i, k in enumerate(("3d", "2d", "1d", "2d5", "3d", "2d", "1d", "2d5"))]
    with capi.Server(memory_budget=4 << 30, max_waves=4, max_wave_solves=2) as srv:
        tickets = []
        for r in reqs:
            tickets.append(submit(srv, r))
            time.sleep(0.002)
        for t in tickets:
            outputs(t)
        info = srv.info()
        infos = [t.info() for t in tickets]
    assert info.max_waves_in_flight >= 2
    assert info.waves_launched >= 4
    assert all(i.done and i.status == 0 for i in infos)
    assert all(0.0 <= i.queued_ms <= i.total_ms for i in infos)
    assert info.bytes_in_use == 0 and 0 < info.peak_bytes <= info.memory_budget


def test_memory_budget_admits_one_wave_at_a_time(gpu_lib):
    r = request("2d5", PN_FP64, seed=50)
    with capi.Server(memory_budget=1 << 30, checkpoint_stride=1) as srv:
        ref = outputs(submit(srv, r))
        foot = srv.info().peak_bytes
    budget = int(foot * 1.5)
    with capi.Server(memory_budget=budget, checkpoint_stride=1, max_waves=4, max_wave_solves=2) as srv:
        ts = [submit(srv, r) for _ in range(3)]
        got = [outputs(t) for t in ts]
        info = srv.info()
    assert info.max_waves_in_flight == 1
    assert info.peak_bytes <= budget
    for g in got:
        for a, b in zip(g, ref):
            for x, y in zip(a, b):
                assert np.array_equal(x, y)


def test_request_larger_than_the_budget_fails_cleanly(gpu_lib):
    s = workloads.small_case(dims=3, N=5, shape=(18, 16, 14), n_steps=4, seed=60)
    d, keep = s.problem.descriptor(s.x_rays)
    rho, noa, acs = s.inputs()
    assert capi.query_sizes(d).n_state * 8 > 1 << 20   # one state alone exceeds the budget
    with capi.Server(memory_budget=1 << 20) as srv:
        t = srv.submit([(d, rho, noa, acs, np.ones(len(s.x_rays)))])
        with pytest.raises(capi.PnError) as e:
            t.wait(timeout_ms=60000)
        assert e.value.code == -4
        # the server still serves a request that fits
        small = request("1d", PN_FP64, seed=61)
        ok = outputs(submit(srv, small))
        assert all(np.all(np.isfinite(x)) for x in ok[0])


def test_forward_only_request(gpu_lib, oracle):
    r = request("2d", PN_FP64, seed=70)
    with capi.Server(memory_budget=1 << 30) as srv:
        I, rb, nb, ab = submit(srv, r, adjoint=False).wait(timeout_ms=60000)
    assert rb is None
    for q, (s, d, keep, rho, noa, acs, ib) in enumerate(r):
        assert rel(I[q], oracle.forward(d, rho, noa, acs)) < 1e-10
