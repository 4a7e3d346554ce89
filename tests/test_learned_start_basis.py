"""Host side of the learned start: the radial basis in the well's scaled coordinate
represents held-out ground states it was not built from.  Analytic Morse ground states
(isotropic, beta = 0) stand in for the solver's states; no GPU needed."""
import math

import numpy as np

from split_operator_gb300 import learned_start as LS


def morse_ground_state(g, prm):
    """psi_0(r) = z^(lambda - 1/2) e^(-z/2), z = 2 lambda e^(-a (r - re)), lambda = (2 m D)^(1/2) / a."""
    d, a, re, _, m = prm
    lam = math.sqrt(2.0 * m * d) / a
    z = 2.0 * lam * np.exp(-a * (g.r - re))
    lp = (lam - 0.5) * np.log(z) - z / 2.0
    st = np.exp(lp - lp.max())[:, None] * np.ones(g.nth)[None, :]
    return st / np.linalg.norm(st)


def test_scaled_coordinate_basis_represents_heldout_states():
    g = LS.Grid2D(nr=1024, nth=8)
    ptrain, pheld = LS.param_sets(128, 5), LS.param_sets(8, 6)
    states = np.stack([morse_ground_state(g, p) for p in ptrain]).astype(np.float32)
    basis = LS.RadialBasis(states, ptrain, g, modes=8)
    for p in pheld:
        s0 = morse_ground_state(g, p)
        rec = basis.state(basis.coefficients(s0, p), p)
        assert np.linalg.norm(rec - s0) / np.linalg.norm(s0) < 1e-5


def test_well_frame_matches_harmonic_width():
    # the harmonic ground state exp(-(m omega / 2) (r - re)^2) is a unit Gaussian in xi
    d, a, re, m = 0.1, 1.0, 3.0, 1000.0
    c, s = LS.well_frame([d, a, re, 0.0, m])
    omega = a * math.sqrt(2.0 * d / m)
    assert c == re and abs(s * s - m * omega) < 1e-12


def test_physics_features_span_the_unit_box():
    f = LS.physics_features(LS.param_sets(4096, 3))
    assert f.shape == (4096, 5) and f.dtype == np.float32
    assert np.all(f >= -1.0 - 1e-6) and np.all(f <= 1.0 + 1e-6)
    assert np.all(f.max(axis=0) - f.min(axis=0) > 1.5)  # each feature uses most of its range
