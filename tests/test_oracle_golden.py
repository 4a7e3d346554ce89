"""Pin the CPU oracle against the reference's own golden outputs (no GPU).

The fixtures in tests/golden/ are the reference crate's FP64 results written by
its integration tests (tests/harmonic_tests.rs, tests/ground_state_tests.rs) and
the 4x4 FFT known answer of tests/fft_tests.rs:11-78.
"""
import math
import os

import numpy as np
import pytest

from oracle import scenarios as S
from oracle import split_operator_oracle as O

GOLD = os.path.join(os.path.dirname(__file__), "golden")


def _load(name):
    return np.load(os.path.join(GOLD, name))


def rel_l2(a, b):
    return float(np.linalg.norm(np.asarray(a) - np.asarray(b)) / np.linalg.norm(np.asarray(b)))


@pytest.mark.parametrize("im_time,name", [(False, "harmonic"), (True, "harmonic_imaginary")])
def test_harmonic_trap_matches_reference_golden(im_time, name):
    prop, saver = S.harmonic_trap(im_time)
    grid = prop.wave_function.grids[0]
    np.testing.assert_array_equal(grid.nodes, _load(f"{name}_space_grid.npy"))
    v = O.harmonic(grid.nodes, 0.0, O.MU_LI6_LI7, 0.001)
    np.testing.assert_array_equal(v, _load(f"{name}_potential.npy"))
    prop.propagate()
    assert rel_l2(saver.data, _load(f"{name}.npy")) < 1e-12
    np.testing.assert_array_equal(np.array(saver.times), _load(f"{name}_time.npy"))


def test_lj_ground_state_matches_reference_golden():
    prop, saver = S.lj_ground_state()
    prop.propagate()
    assert rel_l2(saver.data, _load("lj_ground_space.npy")) < 1e-12
    np.testing.assert_array_equal(np.array(saver.times), _load("lj_ground_space_time.npy"))
    # imaginary-time energy of the relaxed LJ state is finite and negative (bound)
    e = prop.mean_energy()
    assert math.isfinite(e) and e < 0


def test_fft_known_answer_and_exact_round_trip():
    ka = np.load(os.path.join(GOLD, "fft_known_answer.npz"))
    g1 = O.Grid.new_linear_countable("a", 0.0, 1.0, 4, 0)
    g2 = O.Grid.new_linear_countable("b", 0.0, 1.0, 4, 1)
    wf = O.WaveFunction(ka["input"], [g1, g2])
    fft = O.FFTTransformation(g1, "a_fft")
    n1 = wf.norm()
    fft.transform(wf)
    np.testing.assert_array_equal(wf.array, ka["forward"])
    assert wf.grids[0].name == "a_fft"
    fft.inverse_transform(wf)
    np.testing.assert_array_equal(wf.array, ka["input"])
    assert wf.grids[0].name == "a"
    assert wf.norm() == n1


def test_legendre_round_trip_with_gauss_legendre_quadrature():
    x, w = O.gauss_legendre(32)
    polar = O.Grid.new_custom("polar", np.arccos(x), w, 1)
    t, tinv = O.legendre_matrices(polar)
    np.testing.assert_allclose((tinv @ t).real, np.eye(32), atol=1e-12)
    np.testing.assert_allclose((t @ tinv).real, np.eye(32), atol=1e-12)
    assert np.all(t.imag == 0) and np.all(tinv.imag == 0)
    # rows follow numpy's Legendre polynomials
    for l in (0, 1, 5, 31):
        pl = np.polynomial.legendre.Legendre.basis(l)(x)
        np.testing.assert_allclose(tinv[:, l].real, math.sqrt(l + 0.5) * pl, rtol=1e-12, atol=1e-12)


def test_momentum_grid_and_weights():
    g = O.Grid.new_linear_continuos("x", -3.0, 5.0, 16, 0)
    k = O.fft_momentum_grid(g, "k")
    dk = 2 * math.pi / (16 * (8.0 / 15))
    np.testing.assert_allclose(k.nodes, np.fft.fftfreq(16, d=8.0 / 15) * 2 * math.pi, rtol=1e-13, atol=1e-13)
    assert k.weights[7] == pytest.approx(dk / 2) and k.weights[8] == pytest.approx(dk / 2)
    assert k.weights[0] == pytest.approx(dk)


def test_norm_cache_semantics():
    g = O.Grid.new_linear_continuos("x", -3.0, 3.0, 64, 0)
    wf = O.WaveFunction(O.gaussian_distribution(g.nodes, 0.0, 0.5, 1.0), [g])
    wf.normalize(2.0)
    # normalize records the requested norm, not a recomputed one
    assert wf.norm() == 2.0 and not wf.change_observer.possible_norm_change


def test_radial_angular_oracle_conserves_norm_without_damping():
    prop, damp = S.radial_angular_2d(nr=256, nth=16, dt=0.5, step_no=20, with_loss=True)
    n0 = prop.wave_function.norm()
    prop.propagate()
    # the packet starts far from the absorbing border: the loss stays tiny and the norm is kept
    assert abs(damp.loss().loss()) < 1e-8
    prop.wave_function.change_observer.possible_norm_change = True
    assert abs(prop.wave_function.norm() - n0) < 1e-8
