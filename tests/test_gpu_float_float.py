"""The float-float state precision (SO_PRECISION_FLOAT_FLOAT) against the reference's
golden outputs, numpy's FFT and the FP64 oracle, through the C ABI.

Every real of the state and of the tables is an unevaluated sum of two FP32 numbers
(about 48 significand bits), and the FP64 path's kernels run with float-float arithmetic,
so the propagation follows the reference's FP64 algorithm (propagation.rs:134-190) to
about 1e-13 per step instead of the FP32 state's 1e-7."""
import math

import numpy as np
import pytest

from oracle import scenarios as S
from oracle import split_operator_oracle as O
from tests.gpu_common import ensure_built, load_golden, rel_l2

pytestmark = pytest.mark.gpu

PREC = "float_float"


@pytest.fixture(scope="module")
def so():
    ensure_built()
    import split_operator_gb300 as so
    return so


@pytest.mark.parametrize("n", [12, 16, 100, 256, 4096])
def test_fft_and_kinetic_phase_match_oracle(so, n):
    """Unitary lane FFT (fft_transformation.rs:53-88; Stockham stages for powers of two, the
    direct DFT otherwise) with a kinetic phase between the forward and inverse transform,
    against the FP64 oracle step by step."""
    rng = np.random.default_rng(n)
    a = rng.standard_normal(n) + 1j * rng.standard_normal(n)
    g, og = so.Grid.new_linear_continuos("x", -3.0, 3.0, n, 0), O.Grid.new_linear_continuos("x", -3.0, 3.0, n, 0)
    tg, otg = so.TimeGrid(0.05, 3), O.TimeGrid(0.05, 3)
    st, ost = so.OperationStack(), O.OperationStack()
    st.add_transformation(so.FFTTransformation(g, "k"), so.NORMAL)
    st.add_propagator(so.one_dim_into_propagator(so.kinetic_hamiltonian(g, 1.5), g, tg, so.FULL))
    ost.add_transformation(O.FFTTransformation(og, "k"), O.NORMAL)
    ost.add_propagator(O.one_dim_into_propagator(O.kinetic_hamiltonian(og, 1.5), og, otg, O.FULL))
    prop = so.Propagation(so.WaveFunction(a, [g]), tg, st, PREC)
    oprop = O.Propagation(O.WaveFunction(a.copy(), [og]), otg, ost)
    prop.set_timing(True)
    for k in range(3):
        prop.steps(1)
        oprop.step()
        assert rel_l2(prop.get_array(), oprop.wave_function.array) < 1e-12 * (k + 1)
    names = [t[0] for t in prop.kernel_times() if "axis" in t[0]]
    assert names and all(nm.startswith("ff ") for nm in names), names


def _harmonic_trap(so, im_time):
    grid = so.Grid.new_linear_continuos("space", -4.0, 4.0, 256, 0)
    wf = so.WaveFunction(so.gaussian_distribution(grid.nodes, 2.0, 0.2, 0.0), [grid])
    wf.normalize(1.0)
    tg = so.TimeGrid(3.0, 1000, im_time)
    mu = O.MU_LI6_LI7
    saver = so.StateSaver("harmonic", tg, grid, 50)
    st = so.OperationStack()
    st.add_saver(saver, so.FIRST_HALF)
    st.add_control(so.LeakControl(), so.FIRST_HALF | so.SECOND_HALF)
    st.add_propagator(so.one_dim_into_propagator(so.harmonic(grid.nodes, 0.0, mu, 0.001), grid, tg, so.HALF))
    st.add_transformation(so.FFTTransformation(grid, "momentum"), so.NORMAL)
    st.add_propagator(so.one_dim_into_propagator(so.kinetic_hamiltonian(grid, mu), grid, tg, so.FULL))
    return so.Propagation(wf, tg, st, PREC), saver


@pytest.mark.parametrize("im_time,name", [(False, "harmonic"), (True, "harmonic_imaginary")])
def test_harmonic_trap_matches_reference_golden(so, im_time, name):
    """The harmonic trap of tests/harmonic_tests.rs:10-33 (real and imaginary time, 1000
    steps): the saved frames against the reference's committed goldens."""
    prop, saver = _harmonic_trap(so, im_time)
    prop.propagate()
    assert rel_l2(saver.data, load_golden(f"{name}.npy")) < 1e-10
    np.testing.assert_array_equal(saver.times, load_golden(f"{name}_time.npy"))


def test_lj_ground_state_matches_reference_golden_and_energy(so):
    """The imaginary-time Lennard-Jones ground state of tests/ground_state_tests.rs:32-150
    (leak control with a loss checker, 1000 steps): frames against the reference's golden,
    the energy against the oracle's."""
    grid = so.Grid.new_linear_continuos("space", 8.0, 20.0, 512, 0)
    mu = O.MU_LI6_LI7
    mom = math.sqrt(2.0 * mu * 1e-7 * O.KELVIN_TO_AU)
    wf = so.WaveFunction(so.gaussian_distribution(grid.nodes, 14.0, 2.0, mom), [grid])
    wf.normalize(1.0)
    tg = so.TimeGrid(50.0, 1000, True)
    leak = so.LeakControl()
    leak.add_loss_checker("leak control")
    saver = so.StateSaver("lj", tg, grid, 120)
    st = so.OperationStack()
    st.add_control(leak, so.FIRST_HALF | so.SECOND_HALF)
    st.add_saver(saver, so.FIRST_HALF)
    st.add_propagator(so.one_dim_into_propagator(so.lennard_jones(grid.nodes, 0.0003, 9.7), grid, tg, so.HALF))
    st.add_transformation(so.FFTTransformation(grid, "momentum"), so.NORMAL)
    st.add_propagator(so.one_dim_into_propagator(so.kinetic_hamiltonian(grid, mu), grid, tg, so.FULL))
    prop = so.Propagation(wf, tg, st, PREC)
    prop.propagate()
    assert rel_l2(saver.data, load_golden("lj_ground_space.npy")) < 1e-10
    oprop, _ = S.lj_ground_state()
    oprop.propagate()
    e_ref = oprop.mean_energy()
    assert abs(prop.mean_energy() - e_ref) <= 1e-10 * abs(e_ref)


def test_radial_angular_step_matches_oracle_and_fp64(so):
    """The 2-D radial x polar step (Morse + P2, Legendre transform, border damping with a
    loss checker) against the FP64 oracle step by step, and after 20 steps against the FP64
    GPU path: float-float stays within 1e-11 where FP32 drifts by 1e-6."""
    from split_operator_gb300 import workloads as W
    nr, nth, steps = 512, 64, 20
    prop, _ = W.radial_angular_2d(nr=nr, nth=nth, step_no=steps, seed=13, precision=PREC)
    p64, _ = W.radial_angular_2d(nr=nr, nth=nth, step_no=steps, seed=13, precision="fp64")
    oprop, _ = S.radial_angular_2d(nr=nr, nth=nth, step_no=steps, seed=13)
    prop.set_timing(True)
    for k in range(3):
        prop.steps(1)
        p64.steps(1)
        oprop.step()
        assert rel_l2(prop.get_array(), oprop.wave_function.array) < 1e-11 * (k + 1), k
    names = " ".join(t[0] for t in prop.kernel_times())
    assert "ff sweep" in names and "mat" in names, names
    prop.steps(steps - 3)
    p64.steps(steps - 3)
    assert rel_l2(prop.get_array(), p64.get_array()) < 1e-11
    assert abs(prop.norm() - p64.norm()) < 1e-12
    assert abs(prop.all_losses()[0] - p64.all_losses()[0]) < 1e-12
