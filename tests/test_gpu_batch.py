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


@pytest.mark.parametrize("precision", ["fp32_tf32x3", "fp64", "float_float"])
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


@pytest.mark.parametrize("precision", ["fp64", "float_float"])
def test_batch_fp64_matches_oracle(so, precision):
    from split_operator_gb300 import workloads as W
    steps = 12
    props, oracles = [], []
    for k, (nr, nth) in enumerate([(256, 32), (128, 16), (256, 64)]):
        props.append(W.radial_angular_2d(nr=nr, nth=nth, step_no=steps, r0=25.0, seed=7 + k, precision=precision)[0])
        oracles.append(S.radial_angular_2d(nr=nr, nth=nth, step_no=steps, r0=25.0, seed=7 + k)[0])
    so.Batch(props).steps(steps)
    tol = 1e-11 if precision == "fp64" else 1e-10
    for p, o in zip(props, oracles):
        o.propagate(steps)
        assert rel_l2(p.get_array(), o.wave_function.array) < tol


def test_batch_graph_path_long_run(so):
    """Enough steps for the CUDA-graph replay of the repeated passes."""
    from split_operator_gb300 import workloads as W
    steps = 40
    props = [W.radial_angular_2d(nr=256, nth=32, step_no=steps, r0=22.0, seed=3, precision="fp32_tf32x3")[0]]
    solo = W.radial_angular_2d(nr=256, nth=32, step_no=steps, r0=22.0, seed=3, precision="fp32_tf32x3")[0]
    so.Batch(props).steps(steps)
    solo.steps(steps)
    assert rel_l2(props[0].get_array(), solo.get_array()) == 0.0


@pytest.mark.parametrize("precision", ["fp32_tf32x3", "fp64"])
def test_batch_host_arrays_pinned_and_pageable(so, precision):
    """so_batch_set_arrays / so_batch_get_arrays: page-locked buffers (read and written by
    the layout kernels directly) and pageable ones (staged copies) give the same states as
    the per-propagation calls, bit for bit."""
    torch = pytest.importorskip("torch")
    from split_operator_gb300 import workloads as W
    shapes = [(256, 32), (512, 64), (128, 128), (256, 256)]
    props = [W.radial_angular_2d(nr=nr, nth=nth, step_no=10, seed=300 + k, precision=precision)[0]
             for k, (nr, nth) in enumerate(shapes)]
    b = so.Batch(props)
    rng = np.random.default_rng(11)
    states = [rng.normal(size=s) + 1j * rng.normal(size=s) for s in shapes]

    # pageable in, pageable out, against the single-propagation calls
    b.set_arrays(states)
    got = b.get_arrays()
    for p, g in zip(props, got):
        assert np.array_equal(g, p.get_array())
    if precision == "fp64":
        for g, s in zip(got, states):
            assert np.array_equal(g, s)
    else:
        for g, s in zip(got, states):
            assert np.array_equal(g, s.astype(np.complex64).astype(np.complex128))

    # page-locked in and out: same bits
    pins = [torch.from_numpy(s.view(np.float64).ravel().copy()).pin_memory() for s in states]
    outs = [torch.empty_like(t).pin_memory() for t in pins]
    b.set_arrays_ptr([t.data_ptr() for t in pins])
    b.get_arrays_ptr([t.data_ptr() for t in outs])
    for o, g in zip(outs, got):
        assert np.array_equal(o.numpy().view(np.complex128).reshape(g.shape), g)

    # and a step from a pinned start equals a step from a pageable start
    b.set_arrays_ptr([t.data_ptr() for t in pins])
    b.steps(2)
    after_pinned = b.get_arrays()
    b.set_arrays(states)
    b.steps(2)
    for a, c in zip(after_pinned, b.get_arrays()):
        assert np.array_equal(a, c)
    with pytest.raises(Exception):
        b.set_arrays_ptr([t.data_ptr() for t in pins[:-1]])  # count differs from the batch size


def _stored(s, precision):
    """What a state of the precision holds of the complex128 array s: FP64 s itself, FP32
    its rounding, float-float hi = s rounded to FP32 plus lo = the remainder rounded (their
    sum is exact in FP64)."""
    if precision == "fp64":
        return s
    hi = s.astype(np.complex64).astype(np.complex128)
    if precision != "float_float":
        return hi
    return hi + (s - hi).astype(np.complex64).astype(np.complex128)


@pytest.mark.parametrize("precision", ["fp32_simt", "fp64", "float_float"])
def test_single_host_array_ragged_transpose_tiles(so, precision):
    """A radial x angular state whose extents are not multiples of the 32 x 32 transpose
    tile: pinned and pageable buffers through so_propagation_set_array / get_array."""
    torch = pytest.importorskip("torch")
    from split_operator_gb300 import workloads as W
    nr, nth = 300, 17
    p = W.radial_angular_2d(nr=nr, nth=nth, step_no=10, seed=5, precision=precision)[0]
    rng = np.random.default_rng(12)
    s = rng.normal(size=(nr, nth)) + 1j * rng.normal(size=(nr, nth))
    want = _stored(s, precision)
    p.set_array(s)
    assert np.array_equal(p.get_array(), want)
    pin = torch.from_numpy(s.view(np.float64).ravel().copy()).pin_memory()
    out = torch.zeros_like(pin).pin_memory()
    p.set_array(np.zeros_like(s))
    p.set_array_ptr(pin.data_ptr())
    p.get_array_ptr(out.data_ptr())
    assert np.array_equal(out.numpy().view(np.complex128).reshape(nr, nth), want)


def test_batch_steps_host_pipeline_equals_separate_calls(so):
    """so_batch_steps_host (chunked, overlapped copies) gives the same states and losses as
    set_arrays + steps + get_arrays, bit for bit; in and out may be the same buffers."""
    torch = pytest.importorskip("torch")
    from split_operator_gb300 import workloads as W
    shapes = [(256, 32), (512, 64), (128, 128), (256, 256), (512, 32), (256, 64)]
    mk = lambda: [W.radial_angular_2d(nr=nr, nth=nth, step_no=10, seed=400 + k, precision="fp32_tf32x3")[0]
                  for k, (nr, nth) in enumerate(shapes)]
    pa, pb = mk(), mk()
    ba, bb = so.Batch(pa), so.Batch(pb)
    rng = np.random.default_rng(13)
    states = [rng.normal(size=s) + 1j * rng.normal(size=s) for s in shapes]
    pins = [torch.from_numpy(s.view(np.float64).ravel().copy()).pin_memory() for s in states]
    outs = [torch.empty_like(t).pin_memory() for t in pins]
    ba.steps_host_ptr([t.data_ptr() for t in pins], [t.data_ptr() for t in outs], 3)
    bb.set_arrays(states)
    bb.steps(3)
    want = bb.get_arrays()
    for o, w in zip(outs, want):
        assert np.array_equal(o.numpy().view(np.complex128).reshape(w.shape), w)
    for x, y in zip(pa, pb):
        assert x.all_losses() == y.all_losses()
    # in place: the outputs of one call are the inputs of the next
    ba.steps_host_ptr([t.data_ptr() for t in outs], [t.data_ptr() for t in outs], 2)
    bb.steps(2)
    for o, w in zip(outs, bb.get_arrays()):
        assert np.array_equal(o.numpy().view(np.complex128).reshape(w.shape), w)


def test_batch_steps_host_back_to_back_arrays(so, monkeypatch):
    """Host arrays back to back in one pinned buffer (in member order): each pipeline chunk
    moves with one copy per direction through the chunk's staging buffer.  The results equal
    set_arrays + steps + get_arrays bit for bit, in place as well, and with only the inputs
    back to back (outputs in separate buffers: copied per member)."""
    torch = pytest.importorskip("torch")
    from split_operator_gb300 import workloads as W
    monkeypatch.setenv("SO_HOST_CHUNKS", "2")  # two chunks of three members
    shapes = [(256, 32), (512, 64), (128, 128), (256, 256), (512, 32), (256, 64)]
    mk = lambda: [W.radial_angular_2d(nr=nr, nth=nth, step_no=10, seed=500 + k, precision="fp32_bf16x6")[0]
                  for k, (nr, nth) in enumerate(shapes)]
    pa, pb = mk(), mk()
    ba, bb = so.Batch(pa), so.Batch(pb)
    rng = np.random.default_rng(17)
    states = [rng.normal(size=s) + 1j * rng.normal(size=s) for s in shapes]
    sizes = [2 * nr * nth for nr, nth in shapes]
    offs = np.concatenate([[0], np.cumsum(sizes)]).astype(np.int64)
    big_in = torch.empty(int(offs[-1]), dtype=torch.float64).pin_memory()
    big_out = torch.empty_like(big_in).pin_memory()
    views_in = [big_in[int(offs[k]):int(offs[k + 1])] for k in range(len(shapes))]
    views_out = [big_out[int(offs[k]):int(offs[k + 1])] for k in range(len(shapes))]
    for v, s in zip(views_in, states):
        v.numpy()[:] = s.view(np.float64).ravel()
    ba.steps_host_ptr([v.data_ptr() for v in views_in], [v.data_ptr() for v in views_out], 3)
    bb.set_arrays(states)
    bb.steps(3)
    for v, w in zip(views_out, bb.get_arrays()):
        assert np.array_equal(v.numpy().view(np.complex128).reshape(w.shape), w)
    for x, y in zip(pa, pb):
        assert x.all_losses() == y.all_losses()
    # in place on the back-to-back buffer
    ba.steps_host_ptr([v.data_ptr() for v in views_out], [v.data_ptr() for v in views_out], 2)
    bb.steps(2)
    for v, w in zip(views_out, bb.get_arrays()):
        assert np.array_equal(v.numpy().view(np.complex128).reshape(w.shape), w)
    # inputs back to back, outputs separate
    seps = [torch.empty(n, dtype=torch.float64).pin_memory() for n in sizes]
    ba.steps_host_ptr([v.data_ptr() for v in views_out], [t.data_ptr() for t in seps], 1)
    bb.steps(1)
    for t, w in zip(seps, bb.get_arrays()):
        assert np.array_equal(t.numpy().view(np.complex128).reshape(w.shape), w)
