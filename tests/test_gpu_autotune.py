"""The autotuner (Batch.tune): candidate launch schedules of the FFT-pair pass (threads per
CTA, Stockham radix) and of the tensor-core pass (CTAs per SM, tile order), timed on a live
batch; the members' states come back unchanged, the fastest schedule per lane extent is used
by the later steps, and the tuned propagation stays within FP32 accuracy of the FP64 oracle."""
import json

import numpy as np
import pytest

from oracle import scenarios as S
from tests.gpu_common import ensure_built, rel_l2

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def so():
    ensure_built()
    import split_operator_gb300 as so
    return so


def _members(precision):
    from split_operator_gb300 import workloads as W
    sizes = [(512, 32, 3), (1024, 64, 4), (2048, 128, 5), (1024, 256, 6)]
    return [W.radial_angular_2d(nr=nr, nth=nth, step_no=100, seed=sd, r0=25.0, precision=precision)[0]
            for nr, nth, sd in sizes], sizes


def test_tune_restores_states_and_picks_a_schedule_per_extent(so, tmp_path):
    so.reset_schedules()
    props, sizes = _members("fp32_bf16x6")
    b = so.Batch(props)
    b.steps(2)
    before = [p.get_array() for p in props]
    losses = [p.all_losses() for p in props]
    cache = tmp_path / "schedules.json"
    rep = b.tune(str(cache), trial_steps=2)
    # the states, losses and step counts the trials ran over are restored
    for p, a, l in zip(props, before, losses):
        np.testing.assert_array_equal(p.get_array(), a)
        assert p.all_losses() == l
        assert p.steps_done() == 2
    classes = {(c["pass"], c["n"]) for c in rep["classes"]}
    assert {("tensor_core", nth) for _, nth, _ in sizes} <= classes
    assert {("fft_pair", nr) for nr, _, _ in sizes} <= classes
    for c in rep["classes"]:
        ms = [x["ms"] for x in c["candidates"]]
        assert all(m > 0 for m in ms)
        assert ms[c["chosen"]] == min(ms)
    assert rep["tuned_ms"] <= rep["default_ms"]
    written = json.loads(cache.read_text())
    assert written == rep["schedules"]
    # the tuned schedules drive the next steps: the propagation continues within FP32 accuracy
    b.steps(4)
    for (nr, nth, sd), p in zip(sizes, props):
        o, _ = S.radial_angular_2d(nr=nr, nth=nth, step_no=100, seed=sd, r0=25.0)
        o.propagate(6)
        assert rel_l2(p.get_array(), o.wave_function.array) < 6e-6, (nr, nth)
    so.reset_schedules()


@pytest.mark.parametrize("threads,radix", [(128, 16), (512, 8), (256, 8)])
def test_fft_pair_schedules_match_the_oracle(so, threads, radix, tmp_path):
    """Every FFT-pair schedule the tuner can pick computes the same step: each one loaded from
    a cache file and run against the FP64 oracle."""
    nr, nth = 2048, 32
    cache = tmp_path / "c.json"
    cache.write_text(json.dumps({"fft_pair": [{"n": nr, "fp64": 0, "threads": threads, "radix": radix}],
                                 "tensor_core": [{"n": nth, "mode": 0, "ctas_per_sm": 1,
                                                  "blocked": 1}]}))
    so.load_schedules(str(cache))
    from split_operator_gb300 import workloads as W
    p = W.radial_angular_2d(nr=nr, nth=nth, step_no=10, seed=9, r0=25.0, precision="fp32_tf32x3")[0]
    p.set_timing(True)
    p.steps(3)
    names = " ".join(t[0] for t in p.kernel_times())
    assert ("fftpair r8" in names) == (radix == 8), names
    o, _ = S.radial_angular_2d(nr=nr, nth=nth, step_no=10, seed=9, r0=25.0)
    o.propagate(3)
    assert rel_l2(p.get_array(), o.wave_function.array) < 3e-6
    so.reset_schedules()
