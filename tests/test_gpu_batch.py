"""Batched solves (pn_batch_*) against the CPU oracle: mixed orders, grids and step counts."""
import numpy as np
import pytest

from pnepma_gb300 import capi, workloads
from pnepma_gb300.problem import PN_FP32, PN_FP64

pytestmark = pytest.mark.gpu


def rel(a, b):
    a = np.asarray(a, float).ravel()
    b = np.asarray(b, float).ravel()
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))


def mixed_solves(precision):
    out = [
        workloads.small_case(dims=2, N=3, shape=(10, 8), n_steps=9, seed=1, precision=precision),
        workloads.small_case(dims=2, N=3, shape=(12, 7), n_steps=5, seed=2, precision=precision),
        workloads.small_case(dims=2, N=5, shape=(9, 9), n_steps=7, seed=3, precision=precision),
        workloads.small_case(dims=1, N=7, shape=(20,), n_steps=11, seed=4, precision=precision),
        workloads.small_case(dims=2, N=3, shape=(8, 11), n_steps=9, seed=5, precision=precision,
                             elements=("Fe", "Cr", "Ni")),
        workloads.small_case(dims=3, N=3, shape=(6, 5, 5), n_steps=4, seed=6, precision=precision),
    ]
    return out


def run_batch(torch, solves, K=0, flags=0, ibar=None, budget=0):
    descs, keep = [], []
    for s in solves:
        d, k = s.problem.descriptor(s.x_rays)
        descs.append(d)
        keep.append(k)
    b = capi.Batch(descs, keep, checkpoint_stride=K, flags=flags, memory_budget=budget)
    ins, outs = [], []
    for s in solves:
        rho, noa, acs = s.inputs()
        ins.append([torch.from_numpy(np.ascontiguousarray(a)).cuda() for a in (rho, noa, acs)])
    I = [torch.zeros(len(s.x_rays), dtype=torch.float64, device="cuda") for s in solves]
    b.forward([x[0].data_ptr() for x in ins], [x[1].data_ptr() for x in ins], [x[2].data_ptr() for x in ins],
              [t.data_ptr() for t in I])
    torch.cuda.synchronize()
    Ih = [t.cpu().numpy() for t in I]
    if ibar is None:
        ibar = [np.linspace(1.0, 2.0, len(x)) / np.abs(x) for x in Ih]
    ib = [torch.from_numpy(np.ascontiguousarray(x)).cuda() for x in ibar]
    rb = [torch.zeros(x[0].numel(), dtype=torch.float64, device="cuda") for x in ins]
    nb = [torch.zeros(x[1].numel(), dtype=torch.float64, device="cuda") for x in ins]
    ab = [torch.zeros(x[2].numel(), dtype=torch.float64, device="cuda") for x in ins]
    b.adjoint([t.data_ptr() for t in ib], [t.data_ptr() for t in rb], [t.data_ptr() for t in nb],
              [t.data_ptr() for t in ab])
    torch.cuda.synchronize()
    info = b.info()
    b.close()
    return Ih, [t.cpu().numpy() for t in ib], [t.cpu().numpy() for t in rb], [t.cpu().numpy() for t in nb], \
        [t.cpu().numpy() for t in ab], info


def test_batch_fp64_matches_oracle(gpu_lib, oracle):
    torch = pytest.importorskip("torch")
    solves = mixed_solves(PN_FP64)
    I, ib, rb, nb, ab, info = run_batch(torch, solves)
    assert info.n_solves == len(solves) and info.n_groups == 4
    for q, s in enumerate(solves):
        rho, noa, acs = s.inputs()
        d, k = s.problem.descriptor(s.x_rays)
        I_o, rb_o, nb_o, ab_o = oracle.adjoint(d, rho, noa, acs, ib[q])
        assert rel(I[q], I_o) < 1e-10, q
        assert rel(rb[q], rb_o) < 1e-10, q
        assert rel(nb[q], nb_o) < 1e-10, q
        assert rel(ab[q], ab_o) < 1e-10, q


def test_batch_checkpoint_stride_does_not_change_results(gpu_lib):
    torch = pytest.importorskip("torch")
    solves = mixed_solves(PN_FP64)
    ref = run_batch(torch, solves, K=1)
    for K in (2, 3, 5):
        got = run_batch(torch, solves, K=K)
        for a, b in zip(got[:5], ref[:5]):
            for x, y in zip(a, b):
                assert np.array_equal(x, y), K


def test_batch_fp32_against_fp64_oracle(gpu_lib, oracle):
    torch = pytest.importorskip("torch")
    solves = mixed_solves(PN_FP32)
    I, ib, rb, nb, ab, info = run_batch(torch, solves)
    for q, s in enumerate(solves):
        rho, noa, acs = s.inputs()
        s.problem.precision = PN_FP64
        d, k = s.problem.descriptor(s.x_rays)
        I_o, rb_o, nb_o, ab_o = oracle.adjoint(d, rho, noa, acs, ib[q])
        assert rel(I[q], I_o) < 1e-4, q
        assert rel(rb[q], rb_o) < 1e-3, q
        assert rel(nb[q], nb_o) < 1e-3, q
        assert rel(ab[q], ab_o) < 1e-3, q


def tma_solves():
    """FP32 2D solves on grids wide enough for the TMA box tiles (partial tiles at the edges)."""
    return [
        workloads.small_case(dims=2, N=3, shape=(40, 12), n_steps=7, seed=11, precision=PN_FP32),
        workloads.small_case(dims=2, N=5, shape=(40, 12), n_steps=5, seed=12, precision=PN_FP32),
        workloads.small_case(dims=2, N=7, shape=(44, 16), n_steps=6, seed=13, precision=PN_FP32,
                             elements=("Fe", "Cr", "Ni")),
        workloads.small_case(dims=2, N=11, shape=(40, 12), n_steps=4, seed=14, precision=PN_FP32),
        workloads.small_case(dims=2, N=3, shape=(70, 9), n_steps=9, seed=15, precision=PN_FP32),
        workloads.small_case(dims=2, N=5, shape=(32, 20), n_steps=6, seed=16, precision=PN_FP32),
        workloads.small_case(dims=2, N=11, shape=(20, 8), n_steps=3, seed=17, precision=PN_FP32),
    ]


def tma_solves_3d():
    """FP32 3D solves for the TMA tiles: every class, z faces on both sides, narrow z extents."""
    return [
        workloads.small_case(dims=3, N=3, shape=(36, 9, 6), n_steps=5, seed=21, precision=PN_FP32),
        workloads.small_case(dims=3, N=5, shape=(40, 8, 5), n_steps=4, seed=22, precision=PN_FP32),
        workloads.small_case(dims=3, N=7, shape=(33, 10, 4), n_steps=3, seed=23, precision=PN_FP32,
                             elements=("Fe", "Cr", "Ni")),
        workloads.small_case(dims=3, N=3, shape=(12, 5, 3), n_steps=6, seed=24, precision=PN_FP32),
    ]


@pytest.mark.parametrize("K", [1, 3])
def test_tma_tiles_match_the_generic_kernels(gpu_lib, K):
    """Every cell update and ghost point is the same arithmetic on both paths, so states and
    gradients agree bit for bit; the intensity partial sums group the cells by the path's own
    tiles, so intensities agree to rounding."""
    torch = pytest.importorskip("torch")
    solves = tma_solves() + tma_solves_3d()
    ref = run_batch(torch, solves, K=K, flags=capi.PN_BATCH_GENERIC_KERNELS)
    got = run_batch(torch, solves, K=K, ibar=ref[1])
    assert got[5].tma_groups == got[5].n_groups == 7
    assert ref[5].tma_groups == 0
    for x, y in zip(got[0], ref[0]):
        assert rel(x, y) < 1e-13
    for a, b in zip(got[1:5], ref[1:5]):
        for x, y in zip(a, b):
            assert np.array_equal(x, y)


def test_tma_tiles_against_the_oracle(gpu_lib, oracle):
    torch = pytest.importorskip("torch")
    solves = tma_solves()[:2]
    I, ib, rb, nb, ab, info = run_batch(torch, solves)
    assert info.tma_groups == 2
    for q, s in enumerate(solves):
        rho, noa, acs = s.inputs()
        s.problem.precision = PN_FP64
        d, k = s.problem.descriptor(s.x_rays)
        I_o, rb_o, nb_o, ab_o = oracle.adjoint(d, rho, noa, acs, ib[q])
        assert rel(I[q], I_o) < 1e-4
        assert rel(rb[q], rb_o) < 1e-3
        assert rel(nb[q], nb_o) < 1e-3
        assert rel(ab[q], ab_o) < 1e-3


def test_tma_tiles_3d_against_the_oracle(gpu_lib, oracle):
    torch = pytest.importorskip("torch")
    solves = [tma_solves_3d()[3]]
    I, ib, rb, nb, ab, info = run_batch(torch, solves)
    assert info.tma_groups == 1
    s = solves[0]
    rho, noa, acs = s.inputs()
    s.problem.precision = PN_FP64
    d, k = s.problem.descriptor(s.x_rays)
    I_o, rb_o, nb_o, ab_o = oracle.adjoint(d, rho, noa, acs, ib[0])
    assert rel(I[0], I_o) < 1e-4
    assert rel(rb[0], rb_o) < 1e-3
    assert rel(nb[0], nb_o) < 1e-3
    assert rel(ab[0], ab_o) < 1e-3


def test_direct_launches_match_the_graphs(gpu_lib):
    """PN_BATCH_DIRECT_LAUNCH issues the same kernels from the host instead of replaying the
    captured graphs: identical results."""
    torch = pytest.importorskip("torch")
    solves = mixed_solves(PN_FP32) + tma_solves()[:2] + tma_solves_3d()[:1]
    ref = run_batch(torch, solves)
    got = run_batch(torch, solves, flags=capi.PN_BATCH_DIRECT_LAUNCH, ibar=ref[1])
    for a, b in zip(got[:5], ref[:5]):
        for x, y in zip(a, b):
            assert np.array_equal(x, y)


def test_budgeted_tape_gives_the_full_tape_results(gpu_lib):
    """Within a budget below the full tape the batch keeps the first states in full and
    checkpoints the rest (recomputing them in the adjoint): identical results, TMA and generic
    groups, fused and unfused forward sweeps."""
    torch = pytest.importorskip("torch")
    solves = tma_solves()[:3] + tma_solves_3d()[:1] + mixed_solves(PN_FP32)[:2]
    ref = run_batch(torch, solves, K=1)
    assert ref[5].recomputed_steps == 0
    full = ref[5].device_bytes
    seen = 0
    for frac in (0.7, 0.5, 0.35):
        try:
            got = run_batch(torch, solves, ibar=ref[1], budget=int(full * frac))
        except capi.PnError:
            continue
        if got[5].checkpoint_stride > 1:
            seen += 1
            assert got[5].recomputed_steps > 0
        for a, b in zip(got[:5], ref[:5]):
            for x, y in zip(a, b):
                assert np.array_equal(x, y), frac
    assert seen >= 1


def test_sweep_launch_matches_step_launches(gpu_lib):
    """One persistent launch per sweep (PN_BATCH_SWEEP_LAUNCH) against one launch per step (the
    default): the same tiles with the same arithmetic in the same order per solve, so identical
    states and gradients; intensities agree to rounding."""
    torch = pytest.importorskip("torch")
    solves = tma_solves() + tma_solves_3d()[:2]
    for K in (1, 3):
        ref = run_batch(torch, solves, K=K)
        got = run_batch(torch, solves, K=K, ibar=ref[1], flags=capi.PN_BATCH_SWEEP_LAUNCH)
        assert got[5].tma_groups == ref[5].tma_groups > 0
        assert got[5].forward_kernels < ref[5].forward_kernels
        for x, y in zip(got[0], ref[0]):
            assert rel(x, y) < 1e-13
        for a, b in zip(got[1:5], ref[1:5]):
            for x, y in zip(a, b):
                assert np.array_equal(x, y), K


def test_parity_tiles_match_the_class_tiles(gpu_lib):
    """2D: parity tiles (both targets of a parity at one 32 x 4 position, PN_BATCH_PARITY_TILES)
    against one tile per target class (the default).  Every point runs the same arithmetic, and the
    intensity partials are reduced over the same 32 x 4 eee positions in the same order, so
    intensities, states and gradients agree bit for bit; also with the sweep launch."""
    torch = pytest.importorskip("torch")
    solves = tma_solves()
    for K, extra in ((1, 0), (3, 0), (3, capi.PN_BATCH_SWEEP_LAUNCH)):
        ref = run_batch(torch, solves, K=K, flags=extra)
        got = run_batch(torch, solves, K=K, ibar=ref[1], flags=capi.PN_BATCH_PARITY_TILES | extra)
        assert got[5].tma_groups == ref[5].tma_groups == ref[5].n_groups
        for a, b in zip(got[:5], ref[:5]):
            for x, y in zip(a, b):
                assert np.array_equal(x, y), (K, extra)
