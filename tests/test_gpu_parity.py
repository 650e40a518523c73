"""GPU parity against the CPU oracle through the C ABI (FP64 plain path: 1e-10 relative)."""
import numpy as np
import pytest

from pnepma_gb300 import capi, workloads
from pnepma_gb300.problem import PN_FP32

pytestmark = pytest.mark.gpu

TOL64 = 1e-10


def rel(a, b):
    a = np.asarray(a, float).ravel()
    b = np.asarray(b, float).ravel()
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))


CASES = [
    dict(dims=1, N=1, shape=(16,)),
    dict(dims=1, N=7, shape=(24,)),
    dict(dims=2, N=3, shape=(10, 8)),
    dict(dims=2, N=5, shape=(12, 9)),
    dict(dims=2, N=11, shape=(9, 7), n_steps=6),
    dict(dims=3, N=3, shape=(7, 6, 5), n_steps=6),
    dict(dims=3, N=7, shape=(6, 5, 5), n_steps=5),
]


@pytest.mark.parametrize("case", CASES, ids=lambda c: f"{c['dims']}d-N{c['N']}")
def test_forward_adjoint_fp64(gpu_lib, oracle, case):
    kw = dict(n_steps=8)
    kw.update(case)
    s = workloads.small_case(**kw)
    rho, noa, acs = s.inputs()
    desc, keep = s.problem.descriptor(s.x_rays)
    h = capi.Handle(desc, keep)
    I = h.forward(rho, noa, acs)
    ibar = np.linspace(1.0, 2.0, len(I)) / np.abs(I)
    rb, nb, ab = h.adjoint(ibar)
    I_o, rb_o, nb_o, ab_o = oracle.adjoint(desc, rho, noa, acs, ibar)
    assert rel(I, I_o) < TOL64
    assert rel(rb, rb_o) < TOL64
    assert rel(nb, nb_o) < TOL64
    assert rel(ab, ab_o) < TOL64
    h.close()


def test_checkpointing_matches_full_tape(gpu_lib):
    base = workloads.small_case(dims=2, N=3, shape=(10, 8), n_steps=11)
    rho, noa, acs = base.inputs()
    out = []
    for K in (1, 3, 4, 11):
        base.problem.checkpoint_stride = K
        desc, keep = base.problem.descriptor(base.x_rays)
        h = capi.Handle(desc, keep)
        I = h.forward(rho, noa, acs)
        rb, nb, ab = h.adjoint(np.ones_like(I) / np.abs(I))
        out.append((I, rb, nb, ab))
        h.close()
    for o in out[1:]:
        for a, b in zip(o, out[0]):
            assert np.array_equal(a, b)


def test_deterministic_repeat(gpu_lib):
    s = workloads.small_case(dims=2, N=5, shape=(12, 9), n_steps=6)
    rho, noa, acs = s.inputs()
    desc, keep = s.problem.descriptor(s.x_rays)
    h = capi.Handle(desc, keep)
    r1 = (h.forward(rho, noa, acs),) + h.adjoint(np.array([1e230, -2e230]))
    r2 = (h.forward(rho, noa, acs),) + h.adjoint(np.array([1e230, -2e230]))
    for a, b in zip(r1, r2):
        assert np.array_equal(a, b)
    h.close()


def test_generation_field(gpu_lib, oracle):
    s = workloads.small_case(dims=2, N=3, shape=(10, 8), n_steps=9)
    rho, noa, acs = s.inputs()
    desc, keep = s.problem.descriptor(s.x_rays)
    h = capi.Handle(desc, keep)
    f = h.generation_field(rho)
    f_o = oracle.generation_field(desc, rho)
    assert rel(f, f_o) < TOL64
    h.close()


def _live_mask(h, desc):
    """True for state entries that the library maintains (not multi-axis ghosts, active classes)."""
    sz = h.sizes
    mask = []
    for c in range(8):
        nx, ny, nz = sz.shape[c]
        nm = sz.n_moments[c]
        if nm == 0:
            continue
        bits = ((c >> 2) & 1, (c >> 1) & 1, c & 1)
        act = [desc.n_points[d] > 1 for d in range(3)]
        active = all(not (bits[d] and not act[d]) for d in range(3))
        K, J, I = np.meshgrid(np.arange(nz), np.arange(ny), np.arange(nx), indexing="ij")
        g = np.zeros(K.shape, int)
        for d, idx, n in ((0, I, nx), (1, J, ny), (2, K, nz)):
            if bits[d] and act[d]:
                g += (idx == 0) | (idx == n - 1)
        m = (g < 2) & active
        mask.append(np.repeat(m.ravel(), nm))
    return np.concatenate(mask)


@pytest.mark.parametrize("dims", [1, 2, 3])
def test_step_state(gpu_lib, oracle, dims):
    s = workloads.small_case(dims=dims, N=3, n_steps=6)
    rho, noa, acs = s.inputs()
    desc, keep = s.problem.descriptor(s.x_rays)
    h = capi.Handle(desc, keep)
    rng = np.random.default_rng(5)
    u0 = rng.standard_normal(h.sizes.n_state)
    live = _live_mask(h, desc)
    u0 = u0 * live
    h.set_state(rho, u0)
    ref = u0.copy()
    for i in range(3):
        h.step(i)
        ref = oracle.step(desc, rho, ref, i)
    got = h.get_state()
    assert rel(got[live], ref[live]) < TOL64
    assert np.all(got[~live] == 0.0)
    h.close()


def test_fp32_against_fp64_oracle(gpu_lib, oracle):
    s = workloads.small_case(dims=2, N=5, shape=(12, 9), n_steps=8)
    rho, noa, acs = s.inputs()
    d64, k64 = s.problem.descriptor(s.x_rays)
    I_o, rb_o, nb_o, ab_o = oracle.adjoint(d64, rho, noa, acs, np.ones(2))
    s.problem.precision = PN_FP32
    d32, k32 = s.problem.descriptor(s.x_rays)
    h = capi.Handle(d32, k32)
    I = h.forward(rho, noa, acs)
    ibar = np.ones_like(I) / np.abs(I_o)
    I_o2, rb_o, nb_o, ab_o = oracle.adjoint(d64, rho, noa, acs, ibar)
    rb, nb, ab = h.adjoint(ibar)
    assert rel(I, I_o) < 1e-4
    assert rel(rb, rb_o) < 1e-3
    assert rel(nb, nb_o) < 1e-3
    assert rel(ab, ab_o) < 1e-3
    h.close()


def test_shared_tape_buffer_gives_the_checkpointed_results(gpu_lib):
    """Handles whose full tape exceeds 2 GiB keep it in the device's shared buffer.  Interleaving
    two of them (the second forward overwrites the first tape before the first adjoint, which then
    records it again) gives bit for bit the results of handles that checkpoint every 7 states."""
    from pnepma_gb300 import workloads
    solves = workloads.config2(n_positions=2, energies=(15.0,))
    outs = {}
    for label, stride in (("pool", 0), ("ck7", 7)):
        hs, ins = [], []
        for s in solves:
            s.problem.checkpoint_stride = stride
            d, k = s.problem.descriptor(s.x_rays)
            h = capi.Handle(d, k)
            assert h.info().checkpoint_stride == (1 if stride == 0 else 7)
            hs.append(h)
            ins.append(s.inputs())
        I = [h.forward(*x) for h, x in zip(hs, ins)]
        grads = [h.adjoint(1.0 / np.abs(Ii)) for h, Ii in zip(hs, I)]
        outs[label] = (I, grads)
        for h in hs:
            h.close()
    for a, b in zip(outs["pool"][0], outs["ck7"][0]):
        assert np.array_equal(a, b)
    for ga, gb in zip(outs["pool"][1], outs["ck7"][1]):
        for x, y in zip(ga, gb):
            assert np.array_equal(x, y)
