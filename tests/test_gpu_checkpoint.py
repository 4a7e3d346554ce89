"""Checkpoint / resume through the C ABI: a propagation that takes a checkpoint after N
steps, restored into a freshly built propagation, continues bit for bit like the one that
took it -- state, norm, every loss checker, the leak-control norm (imaginary-time energy)
and the saver frames -- and, in FP64, bit for bit like the run that never stopped.  The reference keeps these values in loss_checker.rs:49-68,
leak_control.rs:31-45 and wave_function_saver.rs:42-64, and steps them in
propagation.rs:134-190."""
import numpy as np
import pytest

from tests.gpu_common import ensure_built, rel_l2

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def so():
    ensure_built()
    import split_operator_gb300 as so
    return so


def _two_d(precision, nr=512, nth=32, seed=7):
    from split_operator_gb300 import workloads as W
    return W.radial_angular_2d(nr=nr, nth=nth, step_no=1000, seed=seed, r0=25.0, precision=precision)[0]


@pytest.mark.parametrize("precision", ["fp64", "float_float", "fp32_tf32x3", "fp32_bf16x6"])
def test_resume_equals_uninterrupted_2d(so, precision):
    """The restored propagation continues bit for bit like the one that took the checkpoint
    (a float-float checkpoint carries the state's device words).  In FP64 that is also bit
    for bit the run that never stopped.  In FP32 and float-float a run split at a step
    boundary closes its last pass there (the uninterrupted run fuses the end of one step with
    the start of the next into one pass), and those precisions round the same operations in
    another order, so they differ from the uninterrupted run by rounding only."""
    n = 7
    whole = _two_d(precision)
    whole.steps(2 * n)
    first = _two_d(precision)
    first.steps(n)
    blob = first.checkpoint()
    assert first.steps_done() == n
    resumed = _two_d(precision)
    resumed.restore(blob)
    assert resumed.steps_done() == n
    resumed.steps(n)
    assert resumed.steps_done() == 2 * n
    # the propagation that took the checkpoint goes on as before, and the resumed one with it
    first.steps(n)
    np.testing.assert_array_equal(resumed.get_array(), first.get_array())
    assert resumed.all_losses() == first.all_losses()
    assert resumed.norm() == first.norm()
    if precision == "fp64":
        np.testing.assert_array_equal(resumed.get_array(), whole.get_array())
        assert resumed.all_losses() == whole.all_losses()
        assert resumed.norm() == whole.norm()
    else:
        tol = 1e-12 if precision == "float_float" else 1e-5
        assert rel_l2(resumed.get_array(), whole.get_array()) < tol
        assert abs(resumed.all_losses()[0] - whole.all_losses()[0]) < tol / 100


def _harmonic_imaginary(so, frames=10, steps=40):
    grid = so.Grid.new_linear_continuos("space", -4.0, 4.0, 256, 0)
    wf = so.WaveFunction(so.gaussian_distribution(grid.nodes, 1.0, 0.3, 0.0), [grid])
    wf.normalize(1.0)
    tg = so.TimeGrid(3.0, steps, True)
    leak = so.LeakControl()
    leak.add_loss_checker("leak control")
    saver = so.StateSaver("h", tg, grid, frames)
    st = so.OperationStack()
    st.add_control(leak, so.FIRST_HALF | so.SECOND_HALF)
    st.add_saver(saver, so.FIRST_HALF)
    st.add_propagator(so.one_dim_into_propagator(so.harmonic(grid.nodes, 0.0, 5903.5, 0.001), grid, tg, so.HALF))
    st.add_transformation(so.FFTTransformation(grid, "momentum"), so.NORMAL)
    st.add_propagator(so.one_dim_into_propagator(so.kinetic_hamiltonian(grid, 5903.5), grid, tg, so.FULL))
    return so.Propagation(wf, tg, st, "fp64"), saver


def test_resume_imaginary_time_with_leak_control_saver_and_energy(so, tmp_path):
    whole, wsaver = _harmonic_imaginary(so)
    whole.steps(40)
    first, _ = _harmonic_imaginary(so)
    first.steps(17)  # mid-way between two saver frames
    path = str(tmp_path / "ckpt.npy")
    first.save_checkpoint(path)
    resumed, rsaver = _harmonic_imaginary(so)
    resumed.load_checkpoint(path)
    resumed.steps(23)
    np.testing.assert_array_equal(resumed.get_array(), whole.get_array())
    np.testing.assert_array_equal(rsaver.data, wsaver.data)
    np.testing.assert_array_equal(rsaver.times, wsaver.times)
    assert resumed.all_losses() == whole.all_losses()
    assert resumed.mean_energy() == whole.mean_energy()


def test_resume_after_batched_steps(so):
    """A member of a batch checkpointed after batched steps continues on its own exactly
    as the batch continues it (the batched and the single-propagation passes agree bit for
    bit)."""
    p = [_two_d("fp32_tf32x3", nr=1024, nth=64, seed=s) for s in (11, 12)]
    b = so.Batch(p)
    b.steps(6)
    blob = p[1].checkpoint()
    assert p[1].steps_done() == 6
    b.steps(5)
    alone = _two_d("fp32_tf32x3", nr=1024, nth=64, seed=12)
    alone.restore(blob)
    alone.steps(5)
    np.testing.assert_array_equal(alone.get_array(), p[1].get_array())
    assert alone.all_losses() == p[1].all_losses()
    assert alone.steps_done() == p[1].steps_done() == 11


def test_restore_rejects_a_checkpoint_that_does_not_fit(so):
    from split_operator_gb300._lib import SplitOperatorError

    a = _two_d("fp64")
    a.steps(2)
    blob = a.checkpoint()
    before = a.get_array()
    with pytest.raises(SplitOperatorError):
        _two_d("fp32_tf32x3").restore(blob)  # another precision
    with pytest.raises(SplitOperatorError):
        _two_d("fp64", nr=1024).restore(blob)  # another shape
    with pytest.raises(SplitOperatorError):
        a.restore(blob[:-9])  # truncated
    with pytest.raises(SplitOperatorError):
        a.restore(b"not a checkpoint at all")
    # a failed restore changes nothing
    np.testing.assert_array_equal(a.get_array(), before)
    assert a.steps_done() == 2
