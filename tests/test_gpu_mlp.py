"""Learned-start MLP kernels: gradients against the FP64 numpy oracle, and training."""
import numpy as np
import pytest

from oracle import mlp_oracle as M
from tests.gpu_common import ensure_built

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def so():
    ensure_built()
    import split_operator_gb300 as so
    return so


@pytest.mark.parametrize("widths,batch", [([5, 32, 32, 16], 40), ([5, 256, 256, 256, 512], 128)])
def test_gradients_match_oracle(so, widths, batch):
    rng = np.random.default_rng(len(widths) + batch)
    net = so.Mlp(widths, seed=3)
    p = net.get_params()
    x = rng.uniform(-1, 1, (batch, widths[0])).astype(np.float32)
    t = rng.standard_normal((batch, widths[-1])).astype(np.float32) * 0.3
    loss, g = net.gradients(x, t)
    loss_ref, g_ref = M.loss_and_gradients(p.astype(np.float64), widths, x, t)
    assert abs(loss - loss_ref) <= 1e-5 * abs(loss_ref)
    # FP32 accumulation against FP64 with identical BF16 weights
    assert np.linalg.norm(g - g_ref) <= 1e-4 * np.linalg.norm(g_ref)
    y = net.forward(x)
    y_ref = M.forward(p.astype(np.float64), widths, x)[-1]
    assert np.max(np.abs(y - y_ref)) <= 1e-4 * np.max(np.abs(y_ref))


def test_training_reduces_loss(so):
    rng = np.random.default_rng(11)
    widths = [5, 64, 64, 8]
    x = rng.uniform(-1, 1, (256, 5)).astype(np.float32)
    t = np.stack([np.sin(x @ rng.standard_normal(5)) for _ in range(8)], axis=1).astype(np.float32)
    net = so.Mlp(widths, seed=1)
    losses = net.train(x, t, steps=400, lr=3e-3)
    assert losses[-1] < 0.05 * losses[0]
    # deterministic: a second identical network trains to the same parameters
    net2 = so.Mlp(widths, seed=1)
    net2.train(x, t, steps=400, lr=3e-3)
    np.testing.assert_array_equal(net.get_params(), net2.get_params())
