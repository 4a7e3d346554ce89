"""Oracle-side builders of the reference's own test setups and of the synthetic
workloads (test infrastructure only; see ``oracle/__init__.py``).

* ``harmonic_trap`` follows the reference's ``tests/harmonic_trap.rs:34-111``.
* ``lj_ground_state`` follows ``tests/ground_state_tests.rs:54-144``.
* ``harmonic_1d`` is the 1-D harmonic trap workload (m=1, omega=1, 1024 points on
  [-20, 20], Gaussian of width 1 at x0=2, dt=0.01).
* ``radial_angular_2d`` is the 2-D radial x angular Morse + beta e^{-r/2} P2(cos th)
  workload (mass 1000, border damping on the last 10% of r), built with the same
  operator stack the reference would use: [Damp, V/2, Legendre, Rot/2, FFT, K].
"""
import math

import numpy as np

from . import split_operator_oracle as O


def harmonic_trap(im_time: bool, step_no: int = 1000):
    grid = O.Grid.new_linear_continuos("space", -4.0, 4.0, 256, 0)
    wf = O.WaveFunction(O.gaussian_distribution(grid.nodes, 2.0, 0.2, 0.0), [grid])
    wf.normalize(1.0)
    tg = O.TimeGrid(3.0, step_no, im_time)
    mu = O.MU_LI6_LI7
    v = O.harmonic(grid.nodes, 0.0, mu, 0.001)
    saver = O.StateSaver("harmonic", tg, grid, 50)
    st = O.OperationStack()
    st.add_saver(saver, O.FIRST_HALF)
    st.add_control(O.LeakControl(), O.FIRST_HALF | O.SECOND_HALF)
    st.add_propagator(O.one_dim_into_propagator(v, grid, tg, O.HALF))
    st.add_transformation(O.FFTTransformation(grid, "momentum"), O.NORMAL)
    st.add_propagator(O.one_dim_into_propagator(O.kinetic_hamiltonian(grid, mu), grid, tg, O.FULL))
    return O.Propagation(wf, tg, st), saver


def lj_ground_state(step_no: int = 1000):
    grid = O.Grid.new_linear_continuos("space", 8.0, 20.0, 512, 0)
    mu = O.MU_LI6_LI7
    mom = math.sqrt(2.0 * mu * 1e-7 * O.KELVIN_TO_AU)
    wf = O.WaveFunction(O.gaussian_distribution(grid.nodes, 14.0, 2.0, mom), [grid])
    wf.normalize(1.0)
    tg = O.TimeGrid(50.0, step_no, True)
    v = O.lennard_jones(grid.nodes, 0.0003, 9.7)
    leak = O.LeakControl()
    leak.add_loss_checker(O.LossChecker("leak control"))
    saver = O.StateSaver("lj_ground_space", tg, grid, 120)
    st = O.OperationStack()
    st.add_control(leak, O.FIRST_HALF | O.SECOND_HALF)
    st.add_saver(saver, O.FIRST_HALF)
    st.add_propagator(O.one_dim_into_propagator(v, grid, tg, O.HALF))
    st.add_transformation(O.FFTTransformation(grid, "momentum"), O.NORMAL)
    st.add_propagator(O.one_dim_into_propagator(O.kinetic_hamiltonian(grid, mu), grid, tg, O.FULL))
    return O.Propagation(wf, tg, st), saver


def harmonic_1d(n=1024, dt=0.01, step_no=1000, im_time=False, with_loss=False):
    grid = O.Grid.new_linear_continuos("space", -20.0, 20.0, n, 0)
    wf = O.WaveFunction(O.gaussian_distribution(grid.nodes, 2.0, 1.0, 0.0), [grid])
    wf.normalize(1.0)
    tg = O.TimeGrid(dt, step_no, im_time)
    v = O.harmonic(grid.nodes, 0.0, 1.0, 1.0)
    leak = O.LeakControl()
    if with_loss:
        leak.add_loss_checker(O.LossChecker("leak control"))
    st = O.OperationStack()
    st.add_control(leak, O.FIRST_HALF | O.SECOND_HALF)
    st.add_propagator(O.one_dim_into_propagator(v, grid, tg, O.HALF))
    st.add_transformation(O.FFTTransformation(grid, "momentum"), O.NORMAL)
    st.add_propagator(O.one_dim_into_propagator(O.kinetic_hamiltonian(grid, 1.0), grid, tg, O.FULL))
    return O.Propagation(wf, tg, st)


def radial_angular_inputs(nr=4096, nth=128, seed=2026, d=0.1, a=1.0, re=3.0, beta=0.02,
                          mass=1000.0, r0=15.0, sigma=1.5, k0=5.0, lmax_init=4, r_min=0.5, r_max=60.0):
    """Host arrays shared by the oracle and the product builders of the 2-D workload."""
    radial = O.Grid.new_linear_continuos("radial", r_min, r_max, nr, 0)
    x, w = O.gauss_legendre(nth)
    theta = np.arccos(x)
    polar = O.Grid.new_custom("polar", theta, w, 1)
    r = radial.nodes
    p2 = 0.5 * (3.0 * x * x - 1.0)
    v = O.morse(r, d, a, re)[:, None] + (beta * np.exp(-r / 2.0))[:, None] * p2[None, :]
    rng = np.random.default_rng(seed)
    c = rng.standard_normal(lmax_init + 1) + 1j * rng.standard_normal(lmax_init + 1)
    ang = np.zeros(nth, dtype=np.complex128)
    for l in range(lmax_init + 1):
        pl = np.polynomial.legendre.Legendre.basis(l)(x)
        ang += c[l] * math.sqrt(l + 0.5) * pl
    # the reference Gaussian carries e^{-i (r - r0) p}: p = +k0 moves the packet to smaller r
    psi = O.gaussian_distribution(r, r0, sigma, k0)[:, None] * ang[None, :]
    mask = O.dumping_end(0.1 * (r_max - r_min), 0.0, radial) ** (1.0 / 8.0)
    return dict(radial=radial, polar=polar, v=v, psi=psi, mask=mask, mass=mass)


def radial_angular_2d(nr=4096, nth=128, dt=0.5, step_no=10000, seed=2026, with_loss=True, im_time=False, **kw):
    inp = radial_angular_inputs(nr, nth, seed, **kw)
    radial, polar = inp["radial"], inp["polar"]
    wf = O.WaveFunction(inp["psi"], [radial, polar])
    wf.normalize(1.0)
    tg = O.TimeGrid(dt, step_no, im_time)
    damp = O.BorderDumping(inp["mask"], radial)
    if with_loss:
        damp.add_loss_checker(O.LossChecker("border"))
    vprop = O.n_dim_into_propagator(inp["v"], tg, O.HALF)
    leg = O.legendre_diagonalization_operator(polar)
    rot = O.n_dim_into_propagator(O.rotational_hamiltonian(radial, polar, inp["mass"], 0.0), tg, O.HALF)
    fft = O.FFTTransformation(radial, "momentum")
    kin = O.one_dim_into_propagator(O.kinetic_hamiltonian(radial, inp["mass"]), radial, tg, O.FULL)
    st = O.OperationStack()
    st.add_control(damp, O.FIRST_HALF | O.SECOND_HALF)
    st.add_propagator(vprop)
    st.add_transformation(leg, O.NORMAL)
    st.add_propagator(rot)
    st.add_transformation(fft, O.NORMAL)
    st.add_propagator(kin)
    return O.Propagation(wf, tg, st), damp
