"""GPU parity of the split-operator path against the FP64 oracle and the
reference's golden outputs, through the C ABI (ctypes)."""
import math

import numpy as np
import pytest

from oracle import scenarios as S
from oracle import split_operator_oracle as O
from tests.gpu_common import ensure_built, load_golden, rel_l2

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def so():
    ensure_built()
    import split_operator_gb300 as so
    return so


# ----------------------------------------------------------------- known answers
def test_fft_known_answer_exact(so):
    """tests/fft_tests.rs:11-78: forward result and bitwise round trip."""
    import os
    ka = np.load(os.path.join(os.path.dirname(__file__), "golden", "fft_known_answer.npz"))
    g1 = so.Grid.new_linear_countable("a", 0.0, 1.0, 4, 0)
    g2 = so.Grid.new_linear_countable("b", 0.0, 1.0, 4, 1)
    wf = so.WaveFunction(ka["input"], [g1, g2])
    fft = so.FFTTransformation(g1, "a_fft")
    n1 = wf.norm()
    fft.transform(wf)
    np.testing.assert_array_equal(wf.array, ka["forward"])
    assert wf.grid(0).name == "a_fft"
    n2 = wf.norm()
    fft.inverse_transform(wf)
    np.testing.assert_array_equal(wf.array, ka["input"])
    n3 = wf.norm()
    assert n1 == n3
    assert wf.grid(0).name == "a"
    assert n2 > 0


@pytest.mark.parametrize("n", [8, 16, 64, 256, 1024, 4096])
def test_fft_lane_matches_numpy(so, n):
    rng = np.random.default_rng(n)
    a = rng.standard_normal((n, 3)) + 1j * rng.standard_normal((n, 3))
    g = so.Grid.new_linear_continuos("x", 0.0, 1.0, n, 0)
    g2 = so.Grid.new_linear_countable("y", 0.0, 2.0, 3, 1)
    wf = so.WaveFunction(a, [g, g2])
    f = so.FFTTransformation(g, "k")
    f.transform(wf)
    assert rel_l2(wf.array, np.fft.fft(a, axis=0, norm="ortho")) < 1e-14
    f.inverse_transform(wf)
    assert rel_l2(wf.array, a) < 1e-14


@pytest.mark.parametrize("n", [3, 5, 12, 100])
def test_fft_non_power_of_two(so, n):
    rng = np.random.default_rng(n)
    a = rng.standard_normal(n) + 1j * rng.standard_normal(n)
    g = so.Grid.new_linear_continuos("x", 0.0, 1.0, n, 0)
    wf = so.WaveFunction(a, [g])
    so.FFTTransformation(g, "k").transform(wf)
    assert rel_l2(wf.array, np.fft.fft(a, norm="ortho")) < 1e-13


# ------------------------------------------------------------ reference goldens
def _harmonic_trap(so, im_time):
    grid = so.Grid.new_linear_continuos("space", -4.0, 4.0, 256, 0)
    wf = so.WaveFunction(so.gaussian_distribution(grid.nodes, 2.0, 0.2, 0.0), [grid])
    wf.normalize(1.0)
    tg = so.TimeGrid(3.0, 1000, im_time)
    mu = O.MU_LI6_LI7
    v = so.harmonic(grid.nodes, 0.0, mu, 0.001)
    saver = so.StateSaver("harmonic", tg, grid, 50)
    st = so.OperationStack()
    st.add_saver(saver, so.FIRST_HALF)
    st.add_control(so.LeakControl(), so.FIRST_HALF | so.SECOND_HALF)
    st.add_propagator(so.one_dim_into_propagator(v, grid, tg, so.HALF))
    st.add_transformation(so.FFTTransformation(grid, "momentum"), so.NORMAL)
    st.add_propagator(so.one_dim_into_propagator(so.kinetic_hamiltonian(grid, mu), grid, tg, so.FULL))
    return so.Propagation(wf, tg, st, "fp64"), saver


@pytest.mark.parametrize("im_time,name", [(False, "harmonic"), (True, "harmonic_imaginary")])
def test_harmonic_trap_matches_reference_golden(so, im_time, name):
    prop, saver = _harmonic_trap(so, im_time)
    prop.propagate()
    assert rel_l2(saver.data, load_golden(f"{name}.npy")) < 1e-12
    np.testing.assert_array_equal(saver.times, load_golden(f"{name}_time.npy"))


def test_lj_ground_state_matches_reference_golden_and_energy(so):
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
    prop = so.Propagation(wf, tg, st, "fp64")
    prop.propagate()
    assert rel_l2(saver.data, load_golden("lj_ground_space.npy")) < 1e-12
    e_gpu = prop.mean_energy()
    oprop, _ = S.lj_ground_state()
    oprop.propagate()
    e_ref = oprop.mean_energy()
    assert abs(e_gpu - e_ref) <= 1e-12 * abs(e_ref)


# ------------------------------------------------------------ 1-D workload
def test_harmonic_1d_fp64_matches_oracle_and_ehrenfest(so):
    from split_operator_gb300 import workloads as W
    prop, _ = W.harmonic_1d(step_no=1000)
    oprop = S.harmonic_1d(step_no=1000)
    x = np.linspace(-20.0, 20.0, 1024)
    dx = x[1] - x[0]
    for k in range(10):
        prop.steps(100)
        oprop.propagate(100)
        a = prop.get_array()
        assert rel_l2(a, oprop.wave_function.array) < 1e-11 * (k + 1)
        t = 0.01 * 100 * (k + 1)
        d = np.abs(a) ** 2
        xm = np.sum(x * d) / np.sum(d)
        # Ehrenfest: <x>(t) = x0 cos(omega t) for any Gaussian in a harmonic trap
        assert abs(xm - 2.0 * math.cos(t)) < 2e-4
    assert abs(prop.norm() - 1.0) < 1e-12


def test_harmonic_1d_real_time_energy(so):
    from split_operator_gb300 import workloads as W
    prop, _ = W.harmonic_1d(step_no=10)
    oprop = S.harmonic_1d(step_no=10)
    e = prop.mean_energy()
    eo = oprop.mean_energy()
    assert abs(e - eo) < 1e-10 * abs(eo)


# ------------------------------------------------------------ 2-D workload
@pytest.mark.parametrize("nr,nth,steps", [(256, 16, 40), (512, 32, 20)])
def test_radial_angular_fp64_per_step_parity(so, nr, nth, steps):
    from split_operator_gb300 import workloads as W
    prop, h = W.radial_angular_2d(nr=nr, nth=nth, step_no=steps, r0=25.0)
    oprop, odamp = S.radial_angular_2d(nr=nr, nth=nth, step_no=steps, r0=25.0)
    for k in range(steps):
        prop.steps(1)
        oprop.step()
        err = rel_l2(prop.get_array(), oprop.wave_function.array)
        assert err < 1e-12 * (k + 1), (k, err)
    lo = odamp.loss().loss()
    lg = h["damp"].loss()
    assert abs(lg - lo) <= 1e-12 + 1e-9 * abs(lo)
    assert prop.all_losses() == [lg]


@pytest.mark.parametrize("nr,nth", [(16, 8), (32, 16), (512, 32), (1024, 64), (2048, 32), (4096, 32), (8192, 32)])
def test_fft_pair_pass_matches_general_pass(nr, nth, monkeypatch):
    """The fused FFT-pair kernel (registers at both FFTs' outer stages, reversed radix order
    for the second transform) against the general lane-sweep pass on the same FP32
    problem: same physics, different rounding order."""
    ensure_built()
    from split_operator_gb300 import workloads as W
    kw = dict(nr=nr, nth=nth, step_no=20, seed=31, precision="fp32_simt")
    fused = W.radial_angular_2d(**kw)[0]
    monkeypatch.setenv("SO_FFT_PAIR", "0")
    general = W.radial_angular_2d(**kw)[0]
    monkeypatch.delenv("SO_FFT_PAIR")
    fused.set_timing(True)
    general.set_timing(True)
    fused.steps(20)
    general.steps(20)
    assert any("fftpair" in k[0] for k in fused.kernel_times())
    assert not any("fftpair" in k[0] for k in general.kernel_times())
    a, b = fused.get_array(), general.get_array()
    assert rel_l2(a, b) < 2e-6, rel_l2(a, b)
    assert abs(fused.norm() - general.norm()) < 1e-6


@pytest.mark.parametrize("nr,nth", [(512, 32), (1024, 32), (2048, 32), (4096, 32), (8192, 32)])
def test_fixed_shape_fft_pair_matches_general_shape(nr, nth, monkeypatch):
    """The fixed-shape FFT-pair kernel (radices, spans, twiddle offsets and strides as
    compile-time constants, directions folded into the butterflies) performs the same FP32
    operations in the same order as the general-shape one: the results agree to rounding
    (in practice bit for bit), single and batched."""
    ensure_built()
    import split_operator_gb300 as so
    from split_operator_gb300 import workloads as W
    kw = dict(nr=nr, nth=nth, step_no=20, seed=37, precision="fp32_tf32x3")
    ct = [W.radial_angular_2d(**kw)[0] for _ in range(2)]
    monkeypatch.setenv("SO_FFT_PAIR_CT", "0")
    gen = [W.radial_angular_2d(**kw)[0] for _ in range(2)]
    monkeypatch.delenv("SO_FFT_PAIR_CT")
    for p in (ct[0], gen[0]):
        p.set_timing(True)
        p.steps(6)
    names_ct = " ".join(k[0] for k in ct[0].kernel_times())
    names_gen = " ".join(k[0] for k in gen[0].kernel_times())
    assert "fftpair ct" in names_ct and "fftpair" in names_gen and "fftpair ct" not in names_gen
    assert rel_l2(ct[0].get_array(), gen[0].get_array()) < 1e-6
    assert abs(ct[0].norm() - gen[0].norm()) < 1e-7
    # batched (a batch of one member each: the batched kernels)
    so.Batch([ct[1]]).steps(6)
    so.Batch([gen[1]]).steps(6)
    assert rel_l2(ct[1].get_array(), gen[1].get_array()) < 1e-6
    np.testing.assert_array_equal(ct[1].get_array(), ct[0].get_array())


@pytest.mark.parametrize("nr", [512, 2048, 8192])
def test_fixed_shape_fft_pair_step_matches_oracle(nr):
    """The FP32 2-D step with the fixed-shape FFT pair against the FP64 oracle, 3 steps."""
    ensure_built()
    from split_operator_gb300 import workloads as W
    nth = 32
    kw = dict(nr=nr, nth=nth, step_no=20, seed=41)
    prop = W.radial_angular_2d(precision="fp32_bf16x6", **kw)[0]
    prop.set_timing(True)
    oprop, _ = S.radial_angular_2d(**kw)
    for k in range(3):
        prop.steps(1)
        oprop.step()
        assert rel_l2(prop.get_array(), oprop.wave_function.array) < 2e-6 * (k + 1)
    assert any("fftpair ct" in t[0] for t in prop.kernel_times())


# ------------------------------------------------------------ lane-matrix operators
def _unitary(rng, n, count):
    z = rng.standard_normal((count, n, n)) + 1j * rng.standard_normal((count, n, n))
    return np.stack([np.linalg.qr(m)[0] for m in z])


@pytest.mark.parametrize("precision,tol", [("fp64", 1e-12), ("float_float", 1e-11), ("fp32_simt", 2e-6)])
@pytest.mark.parametrize("count", [40, 64])
def test_non_diag_propagator_matches_oracle(so, precision, tol, count):
    """NonDiagPropagator (non_diagonal_propagator.rs:9-66): a matrix per lane along axis 1,
    lanes in ndarray lanes_mut order; with fewer matrices than lanes the rest stay as they
    are (Iterator::zip)."""
    nx, ny, steps = 64, 24, 3
    rng = np.random.default_rng(count)
    psi = rng.standard_normal((nx, ny)) + 1j * rng.standard_normal((nx, ny))
    ops = _unitary(rng, ny, count)
    gx = so.Grid.new_linear_continuos("x", -4.0, 4.0, nx, 0)
    gy = so.Grid.new_linear_continuos("y", -2.0, 2.0, ny, 1)
    ox = O.Grid.new_linear_continuos("x", -4.0, 4.0, nx, 0)
    oy = O.Grid.new_linear_continuos("y", -2.0, 2.0, ny, 1)
    v = np.sin(np.linspace(0.0, 3.0, nx))
    tg, otg = so.TimeGrid(0.1, steps), O.TimeGrid(0.1, steps)
    st, ost = so.OperationStack(), O.OperationStack()
    nd = so.NonDiagPropagator(1)
    nd.set_operators(ops)
    ond = O.NonDiagPropagator(1)
    ond.set_operators(list(ops))
    st.add_propagator(so.one_dim_into_propagator(v, gx, tg, so.HALF))
    st.add_propagator(nd)
    ost.add_propagator(O.one_dim_into_propagator(v, ox, otg, O.HALF))
    ost.add_propagator(ond)
    prop = so.Propagation(so.WaveFunction(psi, [gx, gy]), tg, st, precision)
    oprop = O.Propagation(O.WaveFunction(psi.copy(), [ox, oy]), otg, ost)
    for k in range(steps):
        prop.steps(1)
        oprop.step()
        assert rel_l2(prop.get_array(), oprop.wave_function.array) < tol * (k + 1)


@pytest.mark.parametrize("precision,tol", [("fp64", 1e-12), ("float_float", 1e-11), ("fp32_simt", 2e-6)])
def test_state_matrix_transformation_matches_oracle(so, precision, tol):
    """StateMatrixTransformation (state_matrix_transformation.rs:8-73): matrix i acts along
    axis 0 on slice i of the dependent axis 1; transform in the first half-step, inverse in
    the second, a diagonal propagator between them."""
    nth, nom, steps = 16, 6, 3
    rng = np.random.default_rng(5)
    psi = rng.standard_normal((nth, nom)) + 1j * rng.standard_normal((nth, nom))
    ts = _unitary(rng, nth, nom)
    tinvs = np.conj(np.transpose(ts, (0, 2, 1)))
    g0 = so.Grid.new_linear_countable("th", 0.0, 1.0, nth, 0)
    g1 = so.Grid.new_linear_countable("om", 0.0, 1.0, nom, 1)
    gl = so.Grid.new_linear_countable("l", 0.0, 1.0, nth, 0)
    o0 = O.Grid.new_linear_countable("th", 0.0, 1.0, nth, 0)
    o1 = O.Grid.new_linear_countable("om", 0.0, 1.0, nom, 1)
    ol = O.Grid.new_linear_countable("l", 0.0, 1.0, nth, 0)
    h = rng.standard_normal((nth, nom))
    tg, otg = so.TimeGrid(0.05, steps), O.TimeGrid(0.05, steps)
    smt = so.StateMatrixTransformation(1, g0, gl)
    smt.set_diagonalization_matrices(ts, tinvs)
    osmt = O.StateMatrixTransformation(1, o0, ol)
    osmt.set_diagonalization_matrices(list(ts), list(tinvs))
    st, ost = so.OperationStack(), O.OperationStack()
    st.add_transformation(smt, so.NORMAL)
    st.add_propagator(so.n_dim_into_propagator(h, tg, so.FULL))
    ost.add_transformation(osmt, O.NORMAL)
    ost.add_propagator(O.n_dim_into_propagator(h, otg, O.FULL))
    prop = so.Propagation(so.WaveFunction(psi, [g0, g1]), tg, st, precision)
    oprop = O.Propagation(O.WaveFunction(psi.copy(), [o0, o1]), otg, ost)
    for k in range(steps):
        prop.steps(1)
        oprop.step()
        assert rel_l2(prop.get_array(), oprop.wave_function.array) < tol * (k + 1)


@pytest.mark.parametrize("precision,tol", [("fp64", 1e-12), ("float_float", 1e-11), ("fp32_simt", 3e-6)])
def test_three_dim_two_fft_axes_matches_oracle(so, precision, tol):
    """A 3-D state with FFTs along axes 0 and 2 (a power-of-two lane and a 24-point lane, so
    the passes run strided lanes and the direct DFT), kinetic phases along both, and a full
    3-D potential: the engine's storage permutation and lane-axis switches against the
    oracle's straightforward ndarray arithmetic."""
    nx, ny, nz, steps = 32, 6, 24, 4
    rng = np.random.default_rng(3)
    psi = rng.standard_normal((nx, ny, nz)) + 1j * rng.standard_normal((nx, ny, nz))
    m = 1.7
    g = [so.Grid.new_linear_continuos("x", -5.0, 5.0, nx, 0), so.Grid.new_linear_countable("y", 0.0, 1.0, ny, 1),
         so.Grid.new_linear_continuos("z", -3.0, 3.0, nz, 2)]
    o = [O.Grid.new_linear_continuos("x", -5.0, 5.0, nx, 0), O.Grid.new_linear_countable("y", 0.0, 1.0, ny, 1),
         O.Grid.new_linear_continuos("z", -3.0, 3.0, nz, 2)]
    v = 0.3 * rng.standard_normal((nx, ny, nz))
    tg, otg = so.TimeGrid(0.02, steps), O.TimeGrid(0.02, steps)
    st, ost = so.OperationStack(), O.OperationStack()
    st.add_propagator(so.n_dim_into_propagator(v, tg, so.HALF))
    st.add_transformation(so.FFTTransformation(g[0], "kx"), so.NORMAL)
    st.add_transformation(so.FFTTransformation(g[2], "kz"), so.NORMAL)
    st.add_propagator(so.one_dim_into_propagator(so.kinetic_hamiltonian(g[0], m), g[0], tg, so.FULL))
    st.add_propagator(so.one_dim_into_propagator(so.kinetic_hamiltonian(g[2], m), g[2], tg, so.FULL))
    ost.add_propagator(O.n_dim_into_propagator(v, otg, O.HALF))
    ost.add_transformation(O.FFTTransformation(o[0], "kx"), O.NORMAL)
    ost.add_transformation(O.FFTTransformation(o[2], "kz"), O.NORMAL)
    ost.add_propagator(O.one_dim_into_propagator(O.kinetic_hamiltonian(o[0], m), o[0], otg, O.FULL))
    ost.add_propagator(O.one_dim_into_propagator(O.kinetic_hamiltonian(o[2], m), o[2], otg, O.FULL))
    prop = so.Propagation(so.WaveFunction(psi, g), tg, st, precision)
    oprop = O.Propagation(O.WaveFunction(psi.copy(), o), otg, ost)
    for k in range(steps):
        prop.steps(1)
        oprop.step()
        assert rel_l2(prop.get_array(), oprop.wave_function.array) < tol * (k + 1)
    assert abs(prop.norm() - oprop.wave_function.norm()) < 10 * tol * abs(oprop.wave_function.norm())


@pytest.mark.parametrize("precision,n", [("fp32_simt", 16384), ("fp64", 16384), ("float_float", 16384)])
def test_lanes_beyond_the_tile_limit_are_rejected(so, precision, n):
    """A lane longer than a CTA tile holds (8192 points) is refused with a status before any
    kernel runs; the context stays usable."""
    from split_operator_gb300 import workloads as W
    with pytest.raises(so.SplitOperatorError) as e:
        p = W.radial_angular_2d(nr=n, nth=8, step_no=2, precision=precision)[0]
        p.steps(1)
    assert "not supported" in str(e.value)
    q = W.radial_angular_2d(nr=256, nth=8, step_no=2, precision=precision)[0]
    q.steps(1)
    assert np.isfinite(q.norm())


def test_fp64_lanes_beyond_4096_need_the_fft_pair_form(so):
    """FP64 lanes of 4097..8192 points run only in FFT-pair passes (one in-place lane buffer);
    a 1-D propagation whose FFT pass also folds norms is refused with a status."""
    from split_operator_gb300 import workloads as W
    with pytest.raises(so.SplitOperatorError) as e:
        W.harmonic_1d(n=8192, step_no=2)[0].steps(1)
    assert "not supported" in str(e.value)


@pytest.mark.parametrize("precision,tol", [("fp64", 1e-12), ("float_float", 1e-11), ("fp32_tf32x3", 1e-6),
                                           ("fp32_bf16x6", 1e-6)])
def test_radial_angular_8192_lanes_match_oracle(so, precision, tol):
    """Nr = 8192 (the longest radial lanes of the batched workload): the FP64 FFT-pair kernel
    (radix-8 stages, 16 values per thread) and the FP32 tensor-core + FFT-pair step against the
    FP64 oracle, step by step."""
    from split_operator_gb300 import workloads as W
    nr, nth, steps = 8192, 32, 3
    prop, _ = W.radial_angular_2d(nr=nr, nth=nth, step_no=steps, seed=41, precision=precision)
    oprop, _ = S.radial_angular_2d(nr=nr, nth=nth, step_no=steps, seed=41)
    prop.set_timing(True)
    for k in range(steps):
        prop.steps(1)
        oprop.step()
        assert rel_l2(prop.get_array(), oprop.wave_function.array) < tol * (k + 1), k
    assert abs(prop.all_losses()[0] - oprop.all_losses()[0][1]) < tol
    assert any("fftpair" in t[0] for t in prop.kernel_times())


@pytest.mark.parametrize("precision,tol", [("fp64", 1e-12), ("float_float", 1e-11), ("fp32_simt", 3e-6)])
def test_two_dim_savers_match_oracle(so, precision, tol):
    """WaveFunctionSaver (|psi|^2 frames) and StateSaver (state_density along an axis) on a
    2-D propagation, saved at the first half of every step_no / frames_no-th step
    (wave_function_saver.rs:6-183): frames and their times against the oracle."""
    nx, ny, steps, frames = 64, 12, 20, 5
    rng = np.random.default_rng(8)
    psi = rng.standard_normal((nx, ny)) + 1j * rng.standard_normal((nx, ny))
    g = [so.Grid.new_linear_continuos("x", -6.0, 6.0, nx, 0), so.Grid.new_linear_continuos("y", -1.0, 1.0, ny, 1)]
    o = [O.Grid.new_linear_continuos("x", -6.0, 6.0, nx, 0), O.Grid.new_linear_continuos("y", -1.0, 1.0, ny, 1)]
    v = 0.2 * rng.standard_normal((nx, ny))
    tg, otg = so.TimeGrid(0.05, steps), O.TimeGrid(0.05, steps)
    wsave, osave = so.WaveFunctionSaver("w", tg, g[0], g[1], frames), O.WaveFunctionSaver("w", otg, o[0], o[1], frames)
    ssave, ossave = so.StateSaver("s", tg, g[1], frames), O.StateSaver("s", otg, o[1], frames)
    st, ost = so.OperationStack(), O.OperationStack()
    st.add_saver(wsave, so.FIRST_HALF)
    st.add_saver(ssave, so.FIRST_HALF)
    st.add_propagator(so.n_dim_into_propagator(v, tg, so.HALF))
    st.add_transformation(so.FFTTransformation(g[0], "kx"), so.NORMAL)
    st.add_propagator(so.one_dim_into_propagator(so.kinetic_hamiltonian(g[0], 2.0), g[0], tg, so.FULL))
    ost.add_saver(osave, O.FIRST_HALF)
    ost.add_saver(ossave, O.FIRST_HALF)
    ost.add_propagator(O.n_dim_into_propagator(v, otg, O.HALF))
    ost.add_transformation(O.FFTTransformation(o[0], "kx"), O.NORMAL)
    ost.add_propagator(O.one_dim_into_propagator(O.kinetic_hamiltonian(o[0], 2.0), o[0], otg, O.FULL))
    prop = so.Propagation(so.WaveFunction(psi, g), tg, st, precision)
    oprop = O.Propagation(O.WaveFunction(psi.copy(), o), otg, ost)
    prop.propagate()
    oprop.propagate()
    assert rel_l2(wsave.data, osave.data) < tol * steps
    assert rel_l2(ssave.data, ossave.data) < tol * steps
    np.testing.assert_allclose(wsave.times, osave.times, rtol=1e-15)
    np.testing.assert_allclose(ssave.times, ossave.times, rtol=1e-15)
