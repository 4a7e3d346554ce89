"""Builders of the benchmark / parity workloads through the product API.

* ``harmonic_1d``: 1-D harmonic trap, m = 1, omega = 1, 1024 points on [-20, 20],
  Gaussian of width 1 displaced to x0 = 2, dt = 0.01, stack [Leak, V/2, FFT, K].
* ``radial_angular_2d``: radial x angular (Gauss-Legendre) grid, Morse
  D(1 - e^{-a(r - re)})^2 plus beta e^{-r/2} P2(cos th), mass 1000, seeded
  Gaussian packet times a random l <= 4 superposition, border damping
  (sine ramp)^(1/8) over the last 10% of r with a loss checker, stack
  [Damp, V/2, Legendre, Rot/2, FFT, K] (the order the reference's operator
  API composes for this problem).

Host-side set-up arrays come from ``radial_angular_inputs`` (numpy, seeded).
"""
import math

import numpy as np

from . import api as so


def harmonic_1d(n=1024, dt=0.01, step_no=1000, precision="fp64", im_time=False, with_loss=False):
    grid = so.Grid.new_linear_continuos("space", -20.0, 20.0, n, 0)
    x = grid.nodes
    wf = so.WaveFunction(so.gaussian_distribution(x, 2.0, 1.0, 0.0), [grid])
    wf.normalize(1.0)
    tg = so.TimeGrid(dt, step_no, im_time)
    leak = so.LeakControl()
    if with_loss:
        leak.add_loss_checker("leak control")
    st = so.OperationStack()
    st.add_control(leak, so.FIRST_HALF | so.SECOND_HALF)
    st.add_propagator(so.one_dim_into_propagator(so.harmonic(x, 0.0, 1.0, 1.0), grid, tg, so.HALF))
    st.add_transformation(so.FFTTransformation(grid, "momentum"), so.NORMAL)
    st.add_propagator(so.one_dim_into_propagator(so.kinetic_hamiltonian(grid, 1.0), grid, tg, so.FULL))
    return so.Propagation(wf, tg, st, precision), dict(grid=grid, leak=leak)


def gauss_legendre_polar(nth):
    x, w = so.gauss_legendre(nth)
    return x, w


def radial_angular_inputs(nr=4096, nth=128, seed=2026, d=0.1, a=1.0, re=3.0, beta=0.02, mass=1000.0, r0=15.0,
                          sigma=1.5, k0=5.0, lmax_init=4, r_min=0.5, r_max=60.0):
    step = (r_max - r_min) / (nr - 1.0)
    r = np.array([r_min + step * i for i in range(nr)])
    x, w = np.polynomial.legendre.leggauss(nth)
    p2 = 0.5 * (3.0 * x * x - 1.0)
    e = np.exp(-a * (r - re))
    v = (d * (1.0 - e) ** 2)[:, None] + (beta * np.exp(-r / 2.0))[:, None] * p2[None, :]
    rng = np.random.default_rng(seed)
    c = rng.standard_normal(lmax_init + 1) + 1j * rng.standard_normal(lmax_init + 1)
    ang = np.zeros(nth, dtype=np.complex128)
    for l in range(lmax_init + 1):
        ang += c[l] * math.sqrt(l + 0.5) * np.polynomial.legendre.Legendre.basis(l)(x)
    q = (r - r0) / (2.0 * sigma)
    radial_part = np.exp(-q * q - 1j * (r - r0) * k0)
    psi = radial_part[:, None] * ang[None, :]
    return dict(r=r, x=x, w=w, v=v, psi=psi, mass=mass, r_min=r_min, r_max=r_max)


NR_CHOICES = (512, 1024, 2048, 4096, 8192)
NTH_CHOICES = (32, 64, 128, 256)


def batched_instance_params(count=512, seed_base=1000):
    """Seeded per-instance sizes and Morse parameters of the batched workload:
    Nr uniform over {512..8192}, Ntheta over {32..256}, D in [0.05, 0.2], a in [0.6, 1.4],
    re in [2, 4], beta in [0, 0.05] (instance i draws from default_rng(seed_base + i))."""
    out = []
    for i in range(count):
        rng = np.random.default_rng(seed_base + i)
        nr = int(rng.choice(NR_CHOICES))
        nth = int(rng.choice(NTH_CHOICES))
        out.append(dict(nr=nr, nth=nth, d=float(rng.uniform(0.05, 0.2)), a=float(rng.uniform(0.6, 1.4)),
                        re=float(rng.uniform(2.0, 4.0)), beta=float(rng.uniform(0.0, 0.05)), seed=seed_base + i))
    return out


def batched_radial_angular(count=512, seed_base=1000, precision="fp32_tf32x3", dt=0.5, step_no=2000, params=None):
    """The batched workload: `count` independent radial x angular propagations of uneven
    sizes, each with its own seeded potential and initial state (mass 1000).  `params`
    (a sub-list of batched_instance_params, e.g. one rank's shard) replaces the first
    `count` instances."""
    props = []
    for prm in (params if params is not None else batched_instance_params(count, seed_base)):
        p, _ = radial_angular_2d(nr=prm["nr"], nth=prm["nth"], dt=dt, step_no=step_no, seed=prm["seed"],
                                 precision=precision, d=prm["d"], a=prm["a"], re=prm["re"], beta=prm["beta"])
        props.append(p)
    return props


def radial_angular_2d(nr=4096, nth=128, dt=0.5, step_no=10000, seed=2026, precision="fp64", with_loss=True,
                      im_time=False, **kw):
    inp = radial_angular_inputs(nr, nth, seed, **kw)
    radial = so.Grid.new_linear_continuos("radial", inp["r_min"], inp["r_max"], nr, 0)
    polar = so.Grid.new_custom("polar", np.arccos(inp["x"]), inp["w"], 1)
    wf = so.WaveFunction(inp["psi"], [radial, polar])
    wf.normalize(1.0)
    tg = so.TimeGrid(dt, step_no, im_time)
    mask = so.dumping_end(0.1 * (inp["r_max"] - inp["r_min"]), 0.0, radial) ** (1.0 / 8.0)
    damp = so.BorderDumping(mask, radial)
    if with_loss:
        damp.add_loss_checker("border")
    st = so.OperationStack()
    st.add_control(damp, so.FIRST_HALF | so.SECOND_HALF)
    st.add_propagator(so.n_dim_into_propagator(inp["v"], tg, so.HALF))
    st.add_transformation(so.legendre_diagonalization_operator(polar), so.NORMAL)
    st.add_propagator(so.n_dim_into_propagator(so.rotational_hamiltonian(radial, polar, inp["mass"], 0.0), tg,
                                               so.HALF))
    st.add_transformation(so.FFTTransformation(radial, "momentum"), so.NORMAL)
    st.add_propagator(so.one_dim_into_propagator(so.kinetic_hamiltonian(radial, inp["mass"]), radial, tg, so.FULL))
    return so.Propagation(wf, tg, st, precision), dict(damp=damp, radial=radial, polar=polar)
