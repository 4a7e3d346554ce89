"""Learned starting states: a small end-to-end run shows the trained network
starting imaginary-time relaxation closer to the ground state than the plain
Gaussian start (fewer steps to |E - E*| <= 1e-8)."""
import numpy as np
import pytest

from tests.gpu_common import ensure_built

pytestmark = pytest.mark.gpu


def test_learned_start_beats_gaussian_start_small():
    ensure_built()
    from split_operator_gb300 import learned_start as LS
    g = LS.Grid2D(nr=256, nth=16, r_min=0.5, r_max=12.5)
    ptrain = LS.param_sets(96, 5)
    states, energies, nsteps = LS.ground_states(ptrain, g, tol=1e-10, every=20, max_steps=20000)
    # the anisotropic term can pull a ground energy below zero; it cannot go below min V
    r = g.r[:, None]
    p2 = 0.5 * (3.0 * g.x[None, :] ** 2 - 1.0)
    vmin = np.array([np.min(d * (1 - np.exp(-a * (r - re))) ** 2 + beta * np.exp(-r / 2) * p2)
                     for d, a, re, beta, _ in ptrain])
    assert np.all(np.isfinite(energies)) and np.all(energies > vmin)
    basis = LS.RadialBasis(states, ptrain, g, modes=16)
    # the basis represents the training states well
    s0 = states[0].astype(np.float64)
    rec = basis.state(basis.coefficients(s0, ptrain[0]), ptrain[0])
    assert np.linalg.norm(rec - s0) / np.linalg.norm(s0) < 1e-3
    model = LS.LearnedStart(basis, hidden=(64, 64, 64), seed=0)
    losses = model.fit(ptrain, states, steps=1500, lr=2e-3)
    assert losses[-1] < 0.1 * losses[0]
    res = LS.evaluate(model, LS.param_sets(8, 6), g, every=5)
    assert res["converged_learned"] == 8 and res["converged_gaussian"] == 8
    assert res["steps_learned_mean"] < res["steps_gaussian_mean"], res


def test_committed_model_reaches_the_ground_state_in_a_third_of_the_time():
    """The network and basis trained at the full configuration (4096 FP64 ground states on the
    2048 x 64 grid, 64 radial modes per l, trained on the library's tensor-core MLP kernels) on
    eight held-out parameter sets: relaxation from the learned start reaches |E - E*| <= 1e-8
    (E* = the plain FP64 solver's converged energy) in at most a third of the wall time of the
    plain Gaussian start, network and basis evaluation included."""
    ensure_built()
    from split_operator_gb300 import learned_start as LS
    res = LS.time_to_ground_state(count=8, first=0)
    assert res["converged"] == [8, 8], res
    assert res["wall_ratio_learned_over_gaussian"] <= 1.0 / 3.0, res
    assert res["steps_learned_mean"] < 0.5 * res["steps_gaussian_mean"], res
