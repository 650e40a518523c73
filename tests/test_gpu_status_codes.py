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
