"""Failure detection of the plain path, injected on the host (no GPU fault, trap or hang): an
energy step above the stated stability limit is rejected at creation with PN_FLAG_CHECK_CFL, and a
march fed non-finite densities reports PN_ERR_DIVERGED with PN_FLAG_CHECK_FINITE.  The reference
checks neither (its compute_dt_max is only printed, pn_intensities.jl:2-8)."""
import numpy as np
import pytest

from pnepma_gb300 import capi, workloads

pytestmark = pytest.mark.gpu

PN_FLAG_CHECK_FINITE, PN_FLAG_CHECK_CFL = 1, 2
PN_ERR_CFL, PN_ERR_DIVERGED = -3, -5


def test_cfl_flag_rejects_an_energy_step_above_the_limit(gpu_lib):
    s = workloads.small_case(dims=1, N=3, shape=(12,), n_steps=4)
    desc, keep = s.problem.descriptor(s.x_rays)
    desc.flags = PN_FLAG_CHECK_CFL
    desc.cfl_limit = 0.5 * desc.delta_e
    with pytest.raises(capi.PnError) as e:
        capi.Handle(desc, keep)
    assert e.value.code == PN_ERR_CFL
    desc.cfl_limit = 2.0 * desc.delta_e
    h = capi.Handle(desc, keep)
    h.close()


def test_non_finite_densities_report_a_diverged_march(gpu_lib):
    s = workloads.small_case(dims=1, N=3, shape=(12,), n_steps=4)
    rho, noa, acs = s.inputs()
    desc, keep = s.problem.descriptor(s.x_rays)
    desc.flags = PN_FLAG_CHECK_FINITE
    h = capi.Handle(desc, keep)
    with pytest.raises(capi.PnError) as e:
        h.forward(np.full_like(rho, np.nan), noa, acs)
    assert e.value.code == PN_ERR_DIVERGED
    I = h.forward(rho, noa, acs)            # the handle stays usable
    assert np.all(np.isfinite(I))
    h.close()


PN_ERR_TIMEOUT = -6


def test_expired_tile_wait_reports_a_timeout_and_the_batch_recovers(gpu_lib):
    """The failure path of the TMA tiles' bounded waits, driven without a hang: with
    PN_BATCH_TEST_EXPIRE_WAIT the first tile wait of the batch is reported as run out after its
    copies have landed, so the CTA records PN_ERR_TIMEOUT, drains its copies and returns.
    pn_batch_query reports the timeout; the next forward clears it, and forward + adjoint then give
    the results of a batch created without the hook, bit for bit."""
    torch = pytest.importorskip("torch")
    from pnepma_gb300.problem import PN_FP32
    solves = [workloads.small_case(dims=2, N=3, shape=(40, 12), n_steps=7, seed=11, precision=PN_FP32),
              workloads.small_case(dims=2, N=5, shape=(40, 12), n_steps=5, seed=12, precision=PN_FP32)]
    descs, keep = [], []
    for s in solves:
        d, k = s.problem.descriptor(s.x_rays)
        descs.append(d)
        keep.append(k)
    dev = lambda a: torch.from_numpy(np.ascontiguousarray(a, dtype=np.float64)).cuda()
    ins = [[dev(a) for a in s.inputs()] for s in solves]

    def run(b, ibar):
        I = [torch.zeros(len(s.x_rays), dtype=torch.float64, device="cuda") for s in solves]
        rb = [torch.zeros(x[0].numel(), dtype=torch.float64, device="cuda") for x in ins]
        nb = [torch.zeros(x[1].numel(), dtype=torch.float64, device="cuda") for x in ins]
        ab = [torch.zeros(x[2].numel(), dtype=torch.float64, device="cuda") for x in ins]
        b.forward([x[0].data_ptr() for x in ins], [x[1].data_ptr() for x in ins], [x[2].data_ptr() for x in ins],
                  [t.data_ptr() for t in I])
        ib = [dev(x) for x in ibar]
        b.adjoint([t.data_ptr() for t in ib], [t.data_ptr() for t in rb], [t.data_ptr() for t in nb],
                  [t.data_ptr() for t in ab])
        torch.cuda.synchronize()
        return [[t.cpu().numpy() for t in ts] for ts in (I, rb, nb, ab)]

    ibar = [np.array([1.0e6, 2.0e6]), np.array([3.0e6, 1.0e6])]
    ref_b = capi.Batch(descs, keep)
    assert ref_b.info().tma_groups == 2
    ref = run(ref_b, ibar)
    ref_b.close()

    b = capi.Batch(descs, keep, flags=capi.PN_BATCH_TEST_EXPIRE_WAIT)
    run(b, ibar)                               # the first launch takes its timeout path
    with pytest.raises(capi.PnError) as e:
        b.info()
    assert e.value.code == PN_ERR_TIMEOUT
    got = run(b, ibar)                         # the batch stays usable
    info = b.info()
    assert info.tma_groups == 2
    b.close()
    for x, y in zip(got, ref):
        for u, v in zip(x, y):
            assert np.array_equal(u, v)
