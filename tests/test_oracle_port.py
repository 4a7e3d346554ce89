"""The C++ FP64 restatement (timed CPU baseline) agrees with the numpy oracle."""
import numpy as np

from oracle import cpu_port as P
from oracle import scenarios as S


def rel_l2(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def test_port_radial_angular_matches_oracle():
    port = P.RadialAngular(128, 16, r0=25.0)
    oprop, damp = S.radial_angular_2d(nr=128, nth=16, step_no=30, r0=25.0)
    port.run(30, threads=2)
    oprop.propagate(30)
    assert rel_l2(port.psi, oprop.wave_function.array) < 1e-12
    assert abs(port.loss[0] - damp.loss().loss()) < 1e-14


def test_port_radial_angular_absorbs_at_border_like_oracle():
    # packet launched outward (k0 < 0) reaches the damping region
    port = P.RadialAngular(128, 8, dt=2.0, r0=50.0, k0=-3.0)
    oprop, damp = S.radial_angular_2d(nr=128, nth=8, dt=2.0, step_no=40, r0=50.0, k0=-3.0)
    port.run(40, threads=1)
    oprop.propagate(40)
    assert damp.loss().loss() > 1e-4
    assert abs(port.loss[0] - damp.loss().loss()) < 1e-12
    assert rel_l2(port.psi, oprop.wave_function.array) < 1e-11


def test_port_harmonic_1d_matches_oracle():
    port = P.Harmonic1D(1024)
    oprop = S.harmonic_1d(step_no=200)
    port.run(200)
    oprop.propagate(200)
    assert rel_l2(port.psi, oprop.wave_function.array) < 1e-12


def test_port_matches_oracle_on_batch_instance_parameters():
    """The reference arm times the port on instances of the batched workload (seeded Morse
    D, a, re and P2 strength beta per instance): the port follows the oracle there too."""
    from split_operator_gb300 import workloads as W
    for prm in W.batched_instance_params(3):
        kw = dict(seed=prm["seed"], d=prm["d"], a=prm["a"], re=prm["re"], beta=prm["beta"])
        port = P.RadialAngular(256, 32, **kw)
        oprop, damp = S.radial_angular_2d(nr=256, nth=32, step_no=10, **kw)
        port.run(10, threads=2)
        oprop.propagate(10)
        assert rel_l2(port.psi, oprop.wave_function.array) < 1e-12
        assert abs(port.loss[0] - damp.loss().loss()) < 1e-14
