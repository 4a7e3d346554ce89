"""Batched stepping of many propagations (so_batch_*) against stepping each alone."""
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


SHAPES = [(256, 32), (512, 64), (256, 128), (512, 32), (256, 256), (1024, 64)]


@pytest.mark.parametrize("precision", ["fp32_tf32x3", "fp64"])
def test_batch_equals_individual_propagations(so, precision):
    from split_operator_gb300 import workloads as W
    steps = 7
    batch_props, solo_props = [], []
    for k, (nr, nth) in enumerate(SHAPES):
        kw = dict(nr=nr, nth=nth, step_no=steps, r0=20.0 + k, seed=100 + k, precision=precision)
        batch_props.append(W.radial_angular_2d(**kw)[0])
        solo_props.append(W.radial_angular_2d(**kw)[0])
    b = so.Batch(batch_props)
    b.steps(steps)
    assert b.launches_per_step() >= 2
    for pb, ps in zip(batch_props, solo_props):
        ps.steps(steps)
        a, r = pb.get_array(), ps.get_array()
        # the same kernels on the same tiles: identical results
        assert rel_l2(a, r) == 0.0
        assert pb.all_losses() == ps.all_losses()
    # and a second call continues from there
    b.steps(3)
    for ps in solo_props:
        ps.steps(3)
    for pb, ps in zip(batch_props, solo_props):
        assert rel_l2(pb.get_array(), ps.get_array()) == 0.0


def test_batch_fp64_matches_oracle(so):
    from split_operator_gb300 import workloads as W
    steps = 12
    props, oracles = [], []
    for k, (nr, nth) in enumerate([(256, 32), (128, 16), (256, 64)]):
        props.append(W.radial_angular_2d(nr=nr, nth=nth, step_no=steps, r0=25.0, seed=7 + k, precision="fp64")[0])
        oracles.append(S.radial_angular_2d(nr=nr, nth=nth, step_no=steps, r0=25.0, seed=7 + k)[0])
    so.Batch(props).steps(steps)
    for p, o in zip(props, oracles):
        o.propagate(steps)
        assert rel_l2(p.get_array(), o.wave_function.array) < 1e-11


def test_batch_graph_path_long_run(so):
    """Enough steps for the CUDA-graph replay of the repeated passes."""
    from split_operator_gb300 import workloads as W
    steps = 40
    props = [W.radial_angular_2d(nr=256, nth=32, step_no=steps, r0=22.0, seed=3, precision="fp32_tf32x3")[0]]
    solo = W.radial_angular_2d(nr=256, nth=32, step_no=steps, r0=22.0, seed=3, precision="fp32_tf32x3")[0]
    so.Batch(props).steps(steps)
    solo.steps(steps)
    assert rel_l2(props[0].get_array(), solo.get_array()) == 0.0
