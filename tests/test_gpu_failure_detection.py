"""Failure detection on the GPU without a fault: a tensor-core pipeline barrier that nothing
completes makes both bounded wait forms give up after their limit, the kernel returns a
status the host reads, and the context stays usable."""
import numpy as np
import pytest

from tests.gpu_common import ensure_built, rel_l2

pytestmark = pytest.mark.gpu


def test_bounded_waits_give_up_and_context_survives():
    ensure_built()
    import split_operator_gb300 as so
    from split_operator_gb300 import api, workloads as W
    limit = 2_000_000  # 2 ms per wait form
    a, b, ns = api.selftest_bounded_wait(limit)
    assert a and b
    assert 2 * limit <= ns < 1_000_000_000
    # a propagation on the same context still runs and agrees with a fresh one
    p = W.radial_angular_2d(nr=256, nth=32, step_no=5, seed=9, precision="fp32_tf32x3")[0]
    q = W.radial_angular_2d(nr=256, nth=32, step_no=5, seed=9, precision="fp32_tf32x3")[0]
    p.steps(5)
    q.steps(5)
    assert rel_l2(p.get_array(), q.get_array()) == 0.0
    assert np.isfinite(p.norm())
    with pytest.raises(Exception):
        api.selftest_bounded_wait(0)  # the host rejects a zero limit before any launch
