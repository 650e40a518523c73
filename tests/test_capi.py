"""The C-ABI library loads and exports every entry point declared in include/pnepma.h (no GPU)."""
import ctypes
import os
import re

from pnepma_gb300 import capi, workloads

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    text = open(os.path.join(ROOT, "include", "pnepma.h")).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(pn_[a-z_]+)\s*\(", text)))


def test_library_exports_every_declared_symbol():
    L = capi.lib()
    names = declared_symbols()
    assert "pn_create" in names and "pn_forward" in names
    for n in names:
        assert hasattr(L, n), n
        assert ctypes.cast(getattr(L, n), ctypes.c_void_p).value


def test_abi_version_and_orders():
    L = capi.lib()
    assert L.pn_abi_version() == 1
    mask = L.pn_compiled_orders()
    for N in (1, 3, 5, 7, 9, 11):
        assert mask & (1 << N)


def test_query_sizes_matches_host_layout():
    s = workloads.small_case(dims=2, N=5, shape=(12, 9))
    desc, keep = s.problem.descriptor(s.x_rays)
    sz = capi.query_sizes(desc)
    rho, noa, acs = s.inputs()
    assert sz.n_rho == rho.size
    assert sz.n_noa == noa.size
    assert sz.n_acs == acs.size
    t = s.problem.tables(s.x_rays)
    assert sz.n_advection == t["advection"].size
    assert sz.n_boundary == t["boundary_fwd"].size
    assert sz.n_beam_face == t["beam_face"].size


def test_invalid_descriptor_is_an_error_not_a_crash():
    s = workloads.small_case(dims=1, N=3, shape=(8,))
    desc, keep = s.problem.descriptor(s.x_rays)
    desc.abi_version = 99
    try:
        capi.query_sizes(desc)
    except capi.PnError as e:
        assert e.code == -1
    else:
        raise AssertionError("expected PN_ERR_INVALID")
