"""The batch autotuner's logic on the CPU (a fake timer in place of the GPU): keys, which
configurations apply, the choice of the fastest, the table kept across runs."""
import json

import pytest

from pnepma_gb300 import autotune, workloads
from pnepma_gb300.problem import PN_FP32


def _descs(**kw):
    s = workloads.small_case(n_steps=3, **kw)
    d, k = s.problem.descriptor(s.x_rays)
    return d, k


def test_keys_name_precision_order_axes_and_grid():
    d1, k1 = _descs(dims=1, N=3, shape=(12,))
    d2, k2 = _descs(dims=2, N=5, shape=(8, 7), precision=PN_FP32)
    assert autotune.key_of(d1) == "fp64-N3-x-12x1x1"
    assert autotune.key_of(d2) == "fp32-N5-xy-8x7x1"
    assert autotune.batch_key([d2, d1, d2]) == autotune.batch_key([d1, d2]) == "fp32-N5-xy-8x7x1+fp64-N3-x-12x1x1"


def test_generic_kernels_only_matter_for_fp32_2d_and_3d():
    g = autotune.Config(autotune.PN_BATCH_GENERIC_KERNELS, 0)
    d1, k1 = _descs(dims=1, N=3, shape=(12,), precision=PN_FP32)
    d2, k2 = _descs(dims=2, N=3, shape=(8, 7))
    d3, k3 = _descs(dims=2, N=3, shape=(8, 7), precision=PN_FP32)
    assert not autotune.applies(g, [d1]) and not autotune.applies(g, [d2])
    assert autotune.applies(g, [d3]) and autotune.applies(g, [d1, d3])
    assert autotune.applies(autotune.Config(autotune.PN_BATCH_DIRECT_LAUNCH, 0), [d2])


def test_parity_tiles_only_matter_for_fp32_2d():
    p = autotune.Config(autotune.PN_BATCH_PARITY_TILES, 0)
    d2, k2 = _descs(dims=2, N=3, shape=(8, 7), precision=PN_FP32)
    d3, k3 = _descs(dims=3, N=3, shape=(8, 7, 5), precision=PN_FP32)
    d64, k64 = _descs(dims=2, N=3, shape=(8, 7))
    assert autotune.applies(p, [d2]) and autotune.applies(p, [d3, d2])
    assert not autotune.applies(p, [d3]) and not autotune.applies(p, [d64])
    assert p.label() == "tma-parity/graphs/K=auto"


def test_tune_keeps_the_fastest_and_remembers_it(tmp_path):
    d, k = _descs(dims=2, N=3, shape=(8, 7), precision=PN_FP32)
    times = {c: 1.0 + i for i, c in enumerate(autotune.DEFAULT_CANDIDATES)}
    fastest = autotune.Config(0, 4)
    times[fastest] = 0.25
    times[autotune.Config(0, 2)] = None            # cannot run: skipped
    calls = []

    def measure(cfg):
        calls.append(cfg)
        return times[cfg]

    path = str(tmp_path / "tune.json")
    tuner = autotune.Autotuner(path)
    assert tuner.tune([d], measure) == fastest
    assert len(calls) == len(autotune.DEFAULT_CANDIDATES)
    assert tuner.tune([d], measure) == fastest      # remembered: nothing measured again
    assert len(calls) == len(autotune.DEFAULT_CANDIDATES)
    again = autotune.Autotuner(path)                  # and kept across runs
    assert again.lookup([d]) == fastest
    entry = json.load(open(path))[autotune.batch_key([d])]
    assert entry["label"] == "tma/graphs/K=4" and entry["seconds"] == 0.25
    assert len(entry["measured"]) == len(autotune.DEFAULT_CANDIDATES) - 1


def test_tune_skips_configurations_that_change_nothing():
    d, k = _descs(dims=1, N=3, shape=(12,))
    seen = []
    autotune.Autotuner().tune([d], lambda c: seen.append(c) or 1.0)
    assert autotune.Config(autotune.PN_BATCH_GENERIC_KERNELS, 0) not in seen


def test_tune_without_any_measurable_configuration_is_an_error():
    d, k = _descs(dims=1, N=3, shape=(12,))
    with pytest.raises(RuntimeError):
        autotune.Autotuner().tune([d], lambda c: None)


def test_options_for_reads_the_tuned_configuration(tmp_path):
    """The batch users' view of the table: the tuned flags and stride of the batch's key, nothing
    (the engine's defaults) for a key the table does not hold or when there is no table."""
    d, k = _descs(dims=2, N=5, shape=(8, 7), precision=PN_FP32)
    path = str(tmp_path / "table.json")
    assert autotune.options_for([d], path) == {}
    tuner = autotune.Autotuner(path)
    best = autotune.Config(4 << autotune.PN_BATCH_CTAS_PER_SM_SHIFT, 0)
    tuner.tune([d], lambda cfg: 0.5 if cfg == best else 1.0)
    assert autotune.options_for([d], path) == {"flags": best.flags, "checkpoint_stride": 0}
    other, k2 = _descs(dims=2, N=3, shape=(8, 7), precision=PN_FP32)
    assert autotune.options_for([other], path) == {}
    assert autotune.options_for([d], None) == {}
