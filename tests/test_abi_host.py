"""C-ABI library: loads, exports every symbol of include/split_operator.h, and its
host-side (set-up time) functions agree with the oracle.  No GPU needed."""
import math
import os
import re

import numpy as np
import pytest

from oracle import split_operator_oracle as O

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def so():
    from split_operator_gb300 import _lib
    if not os.path.exists(_lib.LIB_PATH):
        from split_operator_gb300 import build
        build.build()
    import split_operator_gb300 as so
    return so


def declared_symbols():
    src = open(os.path.join(ROOT, "include", "split_operator.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(so_[a-z0-9_]+)\s*\(", src)))


def test_library_exports_every_declared_symbol(so):
    from split_operator_gb300 import _lib
    h = _lib.lib()
    names = declared_symbols()
    assert len(names) > 90
    missing = [n for n in names if not hasattr(h, n)]
    assert not missing, missing
    # every declared symbol has a Python signature
    bound = set(_lib.SIGNATURES) | set(_lib.VOID) | set(_lib.OTHER)
    assert not [n for n in names if n not in bound]


def test_grids_match_oracle(so):
    g = so.Grid.new_linear_continuos("space", -4.0, 4.0, 256, 0)
    o = O.Grid.new_linear_continuos("space", -4.0, 4.0, 256, 0)
    np.testing.assert_array_equal(g.nodes, o.nodes)
    np.testing.assert_array_equal(g.weights, o.weights)
    g2 = so.Grid.new_linear_countable("l", 0.0, 7.0, 8, 1)
    o2 = O.Grid.new_linear_countable("l", 0.0, 7.0, 8, 1)
    np.testing.assert_array_equal(g2.weights, o2.weights)
    assert g2.dimension_no == 1 and g2.name == "l"


def test_hamiltonians_and_potentials_match_oracle(so):
    g = so.Grid.new_linear_continuos("r", 0.5, 60.0, 64, 0)
    o = O.Grid.new_linear_continuos("r", 0.5, 60.0, 64, 0)
    np.testing.assert_allclose(so.kinetic_hamiltonian(g, 1000.0), O.kinetic_hamiltonian(o, 1000.0), rtol=1e-15)
    x, w = O.gauss_legendre(8)
    p = so.Grid.new_custom("polar", np.arccos(x), w, 1)
    po = O.Grid.new_custom("polar", np.arccos(x), w, 1)
    np.testing.assert_allclose(so.rotational_hamiltonian(g, p, 1000.0, 0.1),
                               O.rotational_hamiltonian(o, po, 1000.0, 0.1), rtol=1e-15)
    r = o.nodes
    np.testing.assert_array_equal(so.harmonic(r, 0.0, 2.0, 0.5), O.harmonic(r, 0.0, 2.0, 0.5))
    np.testing.assert_allclose(so.lennard_jones(r, 3e-4, 9.7), O.lennard_jones(r, 3e-4, 9.7), rtol=1e-14)
    np.testing.assert_allclose(so.morse(r, 0.1, 1.0, 3.0), O.morse(r, 0.1, 1.0, 3.0), rtol=1e-14)
    np.testing.assert_allclose(so.dispersion(r, -6, 2.0), O.dispersion(r, -6, 2.0), rtol=1e-14)
    m = so.dumping_end(5.0, 0.0, g)
    np.testing.assert_allclose(m, O.dumping_end(5.0, 0.0, o), rtol=0, atol=1e-16)
    shp = (64, 8)
    h2 = O.rotational_hamiltonian(o, po, 1000.0, 0.0)
    np.testing.assert_array_equal(so.two_dim_into_n_dim_operator(shp, h2, g, p),
                                  O.two_dim_into_n_dim_operator(shp, h2, o, po))


def test_gauss_legendre_matches_numpy(so):
    # numpy's leggauss weights carry ~1e-11 relative error near the ends at n >= 128
    # (checked against 40-digit values); the library's Newton weights are closer.
    for n in (1, 2, 7, 32, 128, 256):
        x, w = so.gauss_legendre(n)
        xr, wr = np.polynomial.legendre.leggauss(n)
        np.testing.assert_allclose(x, xr, atol=2e-15)
        np.testing.assert_allclose(w, wr, rtol=5e-11, atol=1e-15)
        # exact for polynomials up to degree 2n - 1
        for k in range(0, 2 * n, max(1, n // 4)):
            exact = 0.0 if k % 2 else 2.0 / (k + 1)
            assert abs(np.sum(w * x ** k) - exact) < 1e-13


def test_legendre_polynomials_match_oracle(so):
    for x in (-1.0, -0.3, 0.0, 0.7, 1.0):
        np.testing.assert_allclose(so.legendre_polynomials(20, x), O.legendre_polynomials(20, x), rtol=1e-15,
                                   atol=1e-300)
        for m in (-3, 2, 5):
            np.testing.assert_allclose(so.associated_legendre_polynomials(20, m, x),
                                       O.associated_legendre_polynomials(20, m, x), rtol=1e-14, atol=1e-300)


def test_gaussian_matches_oracle(so):
    x = np.linspace(-3, 7, 101)
    np.testing.assert_allclose(so.gaussian_distribution(x, 2.0, 0.5, 1.3), O.gaussian_distribution(x, 2.0, 0.5, 1.3),
                               rtol=1e-15)


def test_errors_are_status_codes(so):
    with pytest.raises(ValueError):
        so.Grid.new_custom("bad", [0.0, 1.0], [1.0], 0)
    with pytest.raises(so.SplitOperatorError) as e:
        so.legendre_polynomials(0, 0.5)
    assert e.value.status == 1
    p = so.OneDimPropagator(4, 0)
    with pytest.raises(so.SplitOperatorError) as e:
        p.set_operator(np.ones(5))
    assert e.value.status == 2
    st = so.OperationStack()
    with pytest.raises(so.SplitOperatorError):
        st.add_propagator(so.LeakControl())  # wrong operator kind
    tg = so.TimeGrid(1.0, 10)
    g = so.Grid.new_linear_continuos("x", 0, 1, 8, 0)
    with pytest.raises(so.SplitOperatorError):
        so.StateSaver("s", tg, g, 11)  # frames_no > step_no (the reference divides by zero)


def test_legendre_operator_matrices_are_built(so):
    x, w = O.gauss_legendre(6)
    p = so.Grid.new_custom("polar", np.arccos(x), w, 1)
    t = so.legendre_diagonalization_operator(p)
    assert t.grid_transformation.name == "angular_momentum"
    np.testing.assert_array_equal(t.grid_transformation.weights, np.ones(6))


def test_without_a_gpu_the_device_path_fails_loudly(so):
    """Wave functions live in GPU memory: with no device the call returns SO_ERR_CUDA with a
    message (no host fallback).  Batch entry points reject null handles before any device work."""
    import ctypes
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    from split_operator_gb300 import _lib
    g = so.Grid.new_linear_continuos("x", -4.0, 4.0, 64, 0)
    with pytest.raises(so.SplitOperatorError) as e:
        so.WaveFunction(so.gaussian_distribution(g.nodes, 0.0, 0.5, 0.0), [g])
    assert e.value.status == 3 and "CUDA" in str(e.value)
    h = _lib.lib()
    out = ctypes.c_void_p()
    assert h.so_batch_new(None, 0, ctypes.byref(out)) == 1 and h.so_last_error() == b"null argument"
    assert h.so_batch_steps(None, 1) == 1
    assert h.so_batch_steps_host(None, None, None, 0, 1) == 1
