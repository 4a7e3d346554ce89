"""Build and call the C++ FP64 restatement (``cpu_port.cpp``); test and
baseline infrastructure only (see ``oracle/__init__.py``)."""
import ctypes as C
import os
import subprocess

import numpy as np

from . import split_operator_oracle as O
from . import scenarios as S

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "_build")
LIB = os.path.join(OUT, "libcpu_port.so")


def build():
    os.makedirs(OUT, exist_ok=True)
    src = os.path.join(HERE, "cpu_port.cpp")
    if os.path.exists(LIB) and os.path.getmtime(LIB) >= os.path.getmtime(src):
        return LIB
    tmp = LIB + ".tmp"
    subprocess.run(["g++", "-O3", "-std=c++17", "-fopenmp", "-shared", "-fPIC", src, "-o", tmp], check=True)
    os.replace(tmp, LIB)
    return LIB


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        _lib = C.CDLL(LIB)
        dp = C.POINTER(C.c_double)
        _lib.cpu_port_radial_angular.argtypes = [C.c_int, C.c_int] + [dp] * 9 + [C.c_int, C.c_int, dp, dp]
        _lib.cpu_port_harmonic_1d.argtypes = [C.c_int, dp, dp, dp, dp, C.c_int, dp]
    return _lib


def _p(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


class RadialAngular:
    """The 2-D radial x angular workload (same inputs as ``scenarios.radial_angular_2d``)."""

    def __init__(self, nr, nth, dt=0.5, seed=2026, **kw):
        inp = S.radial_angular_inputs(nr, nth, seed, **kw)
        radial, polar = inp["radial"], inp["polar"]
        tg = O.TimeGrid(dt, 1, False)
        wf = O.WaveFunction(inp["psi"], [radial, polar])
        wf.normalize(1.0)
        self.psi = np.ascontiguousarray(wf.array)
        self.v = np.ascontiguousarray(np.exp(-1j * inp["v"] * O.select_step(O.HALF, tg)))
        rot = O.rotational_hamiltonian(radial, polar, inp["mass"], 0.0)
        self.rot = np.ascontiguousarray(np.exp(-1j * rot * O.select_step(O.HALF, tg)))
        self.kin = np.ascontiguousarray(np.exp(-1j * O.kinetic_hamiltonian(radial, inp["mass"]) * O.select_step(O.FULL, tg)))
        self.mask = np.ascontiguousarray(inp["mask"].astype(np.complex128))
        t, ti = O.legendre_matrices(polar)
        self.t, self.ti = np.ascontiguousarray(t), np.ascontiguousarray(ti)
        self.wr, self.wth = radial.weights.copy(), polar.weights.copy()
        self.nr, self.nth = nr, nth
        self.loss = np.zeros(1)
        self.cache = np.ones(1)

    def run(self, steps, threads=0):
        r = lib().cpu_port_radial_angular(
            self.nr, self.nth, _p(self.psi.view(np.float64)), _p(self.v.view(np.float64)),
            _p(self.rot.view(np.float64)), _p(self.kin.view(np.float64)), _p(self.mask.view(np.float64)),
            _p(self.t.view(np.float64)), _p(self.ti.view(np.float64)), _p(self.wr), _p(self.wth), steps, threads,
            _p(self.loss), _p(self.cache))
        assert r == 0


class Harmonic1D:
    def __init__(self, n=1024, dt=0.01):
        prop = S.harmonic_1d(n=n, dt=dt, step_no=1)
        st = prop.operation_stack.stack
        self.psi = np.ascontiguousarray(prop.wave_function.array.copy())
        self.v = np.ascontiguousarray(st[1].obj.operator)
        self.kin = np.ascontiguousarray(st[3].obj.operator)
        self.w = prop.wave_function.grids[0].weights.copy()
        self.n = n
        self.cache = np.ones(1)

    def run(self, steps):
        r = lib().cpu_port_harmonic_1d(self.n, _p(self.psi.view(np.float64)), _p(self.v.view(np.float64)),
                                       _p(self.kin.view(np.float64)), _p(self.w), steps, _p(self.cache))
        assert r == 0
