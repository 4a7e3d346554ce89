"""GPU propagations with the associated Legendre transforms against the FP64 oracle,
through the C ABI.

* associated_legendre_operator (legendre_diagonalization.rs:83-109): a
  StateMatrixTransformation (state_matrix_transformation.rs:48-73) along the polar axis
  whose matrix depends on the Omega index of a third axis, in a radial x polar x Omega
  propagation [V/2, P_l^Omega, Rot/2, FFT, K];
* associated_legendre_diagonalization_operator (legendre_diagonalization.rs:48-80) at a
  fixed Omega in the 2-D radial x polar step, on the tensor cores for 256 polar points: even
  Omega keeps the parity structure (split GEMMs), odd Omega runs as the full GEMM.
"""
import numpy as np
import pytest

from oracle import split_operator_oracle as O
from tests.gpu_common import ensure_built, rel_l2

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def so():
    ensure_built()
    import split_operator_gb300 as so
    return so


def _radial_polar_omega(lib, nr, nth, nom, mass, dt):
    """The same problem built with the product API (lib = the package) or the oracle (lib = O)."""
    radial = lib.Grid.new_linear_continuos("radial", 1.0, 20.0, nr, 0)
    x, w = np.polynomial.legendre.leggauss(nth)
    polar = lib.Grid.new_custom("polar", np.arccos(x), w, 1)
    omega = lib.Grid.new_linear_countable("omega", 0.0, float(nom - 1), nom, 2)
    r = np.asarray(radial.nodes)
    rng = np.random.default_rng(31)
    v = (0.05 * (1.0 - np.exp(-(r - 4.0))) ** 2)[:, None, None] + 0.01 * np.exp(-r / 3.0)[:, None, None] * (
        0.5 * (3 * x * x - 1))[None, :, None] + np.zeros((1, 1, nom))
    l = np.arange(nth)[None, :, None]
    om = np.arange(nom)[None, None, :]
    rot = (l * (l + 1) - om * om) / (2.0 * mass * r[:, None, None] ** 2) + np.zeros((nr, nth, nom))
    psi = (np.exp(-((r - 9.0) / 2.0) ** 2)[:, None, None] * (rng.standard_normal((1, nth, nom)) +
                                                            1j * rng.standard_normal((1, nth, nom))))
    tg = lib.TimeGrid(dt, 10)
    st = lib.OperationStack()
    st.add_propagator(lib.n_dim_into_propagator(v, tg, lib.HALF))
    st.add_transformation(lib.associated_legendre_operator(polar, omega), lib.NORMAL)
    st.add_propagator(lib.n_dim_into_propagator(rot, tg, lib.HALF))
    st.add_transformation(lib.FFTTransformation(radial, "momentum"), lib.NORMAL)
    st.add_propagator(lib.one_dim_into_propagator(lib.kinetic_hamiltonian(radial, mass), radial, tg, lib.FULL))
    wf = lib.WaveFunction(psi, [radial, polar, omega])
    wf.normalize(1.0)
    return wf, tg, st


@pytest.mark.parametrize("precision,tol", [("fp64", 1e-12), ("float_float", 1e-11), ("fp32_simt", 2e-6)])
def test_associated_legendre_operator_propagation_matches_oracle(so, precision, tol):
    nr, nth, nom, steps = 128, 16, 3, 4
    wf, tg, st = _radial_polar_omega(so, nr, nth, nom, 50.0, 0.2)
    owf, otg, ost = _radial_polar_omega(O, nr, nth, nom, 50.0, 0.2)
    prop = so.Propagation(wf, tg, st, precision)
    oprop = O.Propagation(owf, otg, ost)
    for k in range(steps):
        prop.steps(1)
        oprop.step()
        assert rel_l2(prop.get_array(), oprop.wave_function.array) < tol * (k + 1), k
    assert abs(prop.norm() - oprop.wave_function.norm()) < tol * steps


@pytest.mark.parametrize("precision,tol", [("fp32_bf16x6", 2e-6), ("fp32_tf32x3", 2e-6)])
def test_associated_legendre_operator_on_tensor_cores_matches_oracle(so, precision, tol):
    """The state-matrix transformation (one P_l^Omega matrix per Omega) as a grouped GEMM on
    the tensor cores: every tile's columns share one Omega, and the tile streams that
    Omega's operand images (state_matrix_transformation.rs:48-73,
    legendre_diagonalization.rs:83-109)."""
    nr, nth, nom, steps = 128, 64, 3, 4
    wf, tg, st = _radial_polar_omega(so, nr, nth, nom, 50.0, 0.2)
    owf, otg, ost = _radial_polar_omega(O, nr, nth, nom, 50.0, 0.2)
    prop = so.Propagation(wf, tg, st, precision)
    oprop = O.Propagation(owf, otg, ost)
    prop.set_timing(True)
    for k in range(steps):
        prop.steps(1)
        oprop.step()
        assert rel_l2(prop.get_array(), oprop.wave_function.array) < tol * (k + 1), k
    assert abs(prop.norm() - oprop.wave_function.norm()) < tol * steps
    names = " ".join(t[0] for t in prop.kernel_times())
    assert ("tcbf16x6" if precision == "fp32_bf16x6" else "tc3xtf32") in names and "mat_slice" in names, names


def _radial_polar_fixed_omega(lib, nr, nth, omega, mass, dt):
    radial = lib.Grid.new_linear_continuos("radial", 1.0, 30.0, nr, 0)
    x, w = np.polynomial.legendre.leggauss(nth)
    polar = lib.Grid.new_custom("polar", np.arccos(x), w, 1)
    r = np.asarray(radial.nodes)
    v = (0.08 * (1.0 - np.exp(-(r - 3.0))) ** 2)[:, None] + (0.02 * np.exp(-r / 2.0))[:, None] * (
        0.5 * (3 * x * x - 1))[None, :]
    l = np.arange(nth)[None, :]
    rot = l * (l + 1) / (2.0 * mass * r[:, None] ** 2) + np.zeros((nr, nth))
    # a smooth angular state built from P_l^Omega components with l >= Omega
    _, tinv = O.associated_legendre_matrices(O.Grid.new_custom("p", np.arccos(x), w, 1), omega)
    rng = np.random.default_rng(omega + 3)
    coef = np.zeros(nth, dtype=np.complex128)
    coef[omega:omega + 5] = rng.standard_normal(5) + 1j * rng.standard_normal(5)
    ang = tinv.real @ coef
    psi = np.exp(-((r - 12.0) / 2.0) ** 2 - 3j * r)[:, None] * ang[None, :]
    tg = lib.TimeGrid(dt, 10)
    st = lib.OperationStack()
    st.add_propagator(lib.n_dim_into_propagator(v, tg, lib.HALF))
    st.add_transformation(lib.associated_legendre_diagonalization_operator(polar, omega), lib.NORMAL)
    st.add_propagator(lib.n_dim_into_propagator(rot, tg, lib.HALF))
    st.add_transformation(lib.FFTTransformation(radial, "momentum"), lib.NORMAL)
    st.add_propagator(lib.one_dim_into_propagator(lib.kinetic_hamiltonian(radial, mass), radial, tg, lib.FULL))
    wf = lib.WaveFunction(psi, [radial, polar])
    wf.normalize(1.0)
    return wf, tg, st


@pytest.mark.parametrize("omega", [1, 2])
@pytest.mark.parametrize("precision,tol", [("fp64", 1e-12), ("fp32_tf32x3", 1e-6)])
def test_associated_legendre_fixed_omega_matches_oracle(so, omega, precision, tol):
    nr, nth, steps = 512, 256, 3
    wf, tg, st = _radial_polar_fixed_omega(so, nr, nth, omega, 200.0, 0.5)
    owf, otg, ost = _radial_polar_fixed_omega(O, nr, nth, omega, 200.0, 0.5)
    prop = so.Propagation(wf, tg, st, precision)
    oprop = O.Propagation(owf, otg, ost)
    if precision != "fp64":
        prop.set_timing(True)
    for k in range(steps):
        prop.steps(1)
        oprop.step()
        assert rel_l2(prop.get_array(), oprop.wave_function.array) < tol * (k + 1), k
    if precision != "fp64":
        names = " ".join(t[0] for t in prop.kernel_times())
        assert "tc3xtf32" in names
        # even Omega keeps the parity structure of the Legendre pair; odd Omega does not
        assert ("parity" in names) == (omega % 2 == 0), names
