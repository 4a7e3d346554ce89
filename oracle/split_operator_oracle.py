"""FP64 CPU restatement of the split_operator propagation path (numpy).

TEST INFRASTRUCTURE ONLY.  This module is the oracle: only the test suite,
``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline leg may import it,
and only to check or time against.  The product (``split_operator_gb300``) never
imports it and has no CPU fallback.

It restates, in numpy, the algorithm of the Rust crate ``split_operator``
(Wleter/split_operator).  Every class and function cites the reference file and
lines it follows.  Semantics that matter for parity are kept exactly:

* the norm cache of ``WaveFunction``/``ChangeObserver`` (a norm is recomputed only
  after an operator marked it dirty, and ``normalize`` records the *requested*
  norm, not a recomputed one);
* the representation weights: a transformation swaps the axis grid, and the norm
  uses the weights of the grid currently in place;
* the palindromic ``Propagation::step`` order (forward pass, then the reversed
  stack without its last element);
* ``LossChecker`` / ``LeakControl`` / ``BorderDumping`` bookkeeping;
* the saver frame schedule (``step_no / frames_no``).

Third-party arithmetic: the reference's FFT is ``rustfft 6.2.0`` (forward kernel
e^{-2 pi i jk/N}, unnormalised both ways, the crate divides by sqrt(N)); here it
is numpy's pocketfft with ``norm="ortho"``, which is the same transform.  Dense
lane products are ``ndarray 0.16.1`` ``.dot``; here ``numpy.tensordot``.  The
only difference to the reference is floating-point summation order (~1e-16).

Parity pin: this restatement reproduces the reference's committed FP64 outputs
``tests/test_data/harmonic.npy``, ``harmonic_imaginary.npy`` and
``lj_ground_space.npy`` (copied to ``tests/golden/``) and the 4x4 FFT known
answer of ``tests/fft_tests.rs:11-78``; see ``tests/test_oracle_golden.py``.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field
from typing import List, Optional

import numpy as np

# Hartree per kelvin (CODATA 2018), the unit constant the reference's tests take
# from the un-vendored ``quantum`` crate (Energy(x, Kelvin) -> au).
KELVIN_TO_AU = 3.1668115634556e-6
# Reduced mass of Li6-Li7 in atomic units, as implied by the reference's own
# ``harmonic_potential.npy`` (V = 0.5*mu*omega^2*x^2 with omega = 0.001).
MU_LI6_LI7 = 5903.538543342382


# --------------------------------------------------------------------------- grid
@dataclass
class Grid:
    """1-D grid (grid.rs:14-20)."""

    name: str
    dimension_no: int
    nodes_no: int
    nodes: np.ndarray
    weights: np.ndarray

    @staticmethod
    def new_linear_continuos(name, start, end, nodes_no, dimension_no):
        """Trapezoid weights, half weight at both ends (grid.rs:24-48)."""
        step = (end - start) / (nodes_no - 1.0)
        nodes = np.array([start + step * i for i in range(nodes_no)], dtype=np.float64)
        weights = np.full(nodes_no, 1.0 * step)
        weights[0] = 0.5 * step
        weights[nodes_no - 1] = 0.5 * step
        return Grid(name, dimension_no, nodes_no, nodes, weights)

    @staticmethod
    def new_linear_countable(name, start, end, nodes_no, dimension_no):
        """Uniform weights (grid.rs:51-73)."""
        step = (end - start) / (nodes_no - 1.0)
        nodes = np.array([start + step * i for i in range(nodes_no)], dtype=np.float64)
        weights = np.full(nodes_no, 1.0 * step)
        return Grid(name, dimension_no, nodes_no, nodes, weights)

    @staticmethod
    def new_custom(name, nodes, weights, dimension_no):
        """grid.rs:76-84"""
        nodes = np.asarray(nodes, dtype=np.float64).copy()
        weights = np.asarray(weights, dtype=np.float64).copy()
        return Grid(name, dimension_no, len(nodes), nodes, weights)

    def copy(self):
        return Grid(self.name, self.dimension_no, self.nodes_no, self.nodes.copy(), self.weights.copy())


# ---------------------------------------------------------------------- time grid
@dataclass
class TimeGrid:
    """time_grid.rs:7-11"""

    step: float
    step_no: int
    im_time: bool = False


FULL, HALF = 0, 1


def select_step(step_kind: int, time: TimeGrid) -> complex:
    """time_grid.rs:22-33: Full or Half step; imaginary time gives -i*dt."""
    ts = time.step if step_kind == FULL else time.step / 2.0
    if time.im_time:
        return -ts * 1j
    return complex(ts)


# ------------------------------------------------------------------ wave function
class ChangeObserver:
    """change_observer.rs:7-46 (norm cache + grid-name change detection)."""

    def __init__(self, grids):
        self.last_grid_names = [g.name for g in grids]
        self._last_norm = 1.0
        self.possible_norm_change = True

    def observe_grid(self, grids):
        self.last_grid_names = [g.name for g in grids]

    def observe_norm(self, n):
        self._last_norm = n
        self.possible_norm_change = False

    def last_norm(self):
        return self._last_norm

    def has_grid_changed(self, grids):
        return any(a != g.name for a, g in zip(self.last_grid_names, grids))


def _weight_amplitude(shape, grids):
    """wave_function.rs:23-47: W = prod_axis sqrt(w_axis) (stored complex, imag 0)."""
    w = np.ones(shape, dtype=np.complex128)
    for axis in range(len(shape)):
        s = [1] * len(shape)
        s[axis] = shape[axis]
        w = w * np.sqrt(grids[axis].weights).astype(np.complex128).reshape(s)
    return w


class WaveFunction:
    """wave_function.rs:11-149"""

    def __init__(self, array, grids):
        self.array = np.array(array, dtype=np.complex128)
        self.grids = [g.copy() for g in grids]
        self.change_observer = ChangeObserver(self.grids)
        self._w = _weight_amplitude(self.array.shape, self.grids)

    def clone(self):
        other = WaveFunction.__new__(WaveFunction)
        other.array = self.array.copy()
        other.grids = [g.copy() for g in self.grids]
        co = ChangeObserver(other.grids)
        co.last_grid_names = list(self.change_observer.last_grid_names)
        co._last_norm = self.change_observer._last_norm
        co.possible_norm_change = self.change_observer.possible_norm_change
        other.change_observer = co
        other._w = self._w.copy()
        return other

    def _update_weights(self):
        self._w = _weight_amplitude(self.array.shape, self.grids)

    def weight_sq(self):
        """|W|^2 for the current representation (what the norm multiplies by)."""
        if self.change_observer.has_grid_changed(self.grids):
            self._update_weights()
            self.change_observer.observe_grid(self.grids)
        return np.abs(self._w) ** 2

    def norm(self) -> float:
        """wave_function.rs:68-85 (cached unless an operator marked it dirty)."""
        if not self.change_observer.possible_norm_change:
            return self.change_observer.last_norm()
        if self.change_observer.has_grid_changed(self.grids):
            self._update_weights()
            self.change_observer.observe_grid(self.grids)
        n = float(np.sum((self.array.real ** 2 + self.array.imag ** 2) * (self._w.real ** 2 + self._w.imag ** 2)))
        self.change_observer.observe_norm(n)
        return n

    def dot(self, other: "WaveFunction") -> complex:
        """wave_function.rs:87-101: <self|other> weighted, divided by sqrt(n1*n2)."""
        n1 = self.norm()
        n2 = other.norm()
        assert np.array_equal(self._w, other._w)
        d = np.sum(self.array * np.conj(other.array) * (np.abs(self._w) ** 2))
        return complex(d / math.sqrt(n1 * n2))

    def normalize(self, new_norm: float):
        """wave_function.rs:104-109"""
        n = self.norm()
        self.array *= complex(math.sqrt(new_norm / n))
        self.change_observer.observe_norm(new_norm)

    def density(self):
        """wave_function.rs:112-118"""
        return self.array.real ** 2 + self.array.imag ** 2

    def state_density(self, axis: int):
        """wave_function.rs:121-148 (1-D: unweighted |psi|^2)."""
        if self.change_observer.has_grid_changed(self.grids):
            self._update_weights()
            self.change_observer.observe_grid(self.grids)
        d = self.density()
        if d.ndim == 1:
            return d
        wd = d * (np.abs(self._w) ** 2)
        other = tuple(a for a in range(d.ndim) if a != axis)
        return np.sum(wd, axis=other)


def gaussian_distribution(x, x0, sigma, momentum):
    """wave_function.rs:152-154: exp(-((x-x0)/(2 sigma))^2 - i (x-x0) p)."""
    x = np.asarray(x, dtype=np.float64)
    return np.exp(-(((x - x0) / (2.0 * sigma)) ** 2) - 1j * (x - x0) * momentum)


# ------------------------------------------------------------------ loss checker
class LossChecker:
    """loss_checker.rs:7-69 (LossSaver folded in as an optional frame list)."""

    def __init__(self, name: str, frames_no: int = 0, time_grid: Optional[TimeGrid] = None):
        self.name = name
        self._loss = 0.0
        self.current_norm = 1.0
        self.saver = LossSaver(frames_no, time_grid) if frames_no else None

    def loss(self):
        return self._loss

    def check_before(self, wf: WaveFunction):
        self.current_norm = wf.norm()

    def check_after(self, wf: WaveFunction):
        new = wf.norm()
        self._loss += self.current_norm - new
        if self.saver is not None:
            self.saver.monitor(self._loss)
        self.current_norm = new

    def reset(self):
        self._loss = 0.0


class LossSaver:
    """loss_saver.rs:17-39: cumulative loss sampled twice per step."""

    def __init__(self, frames_no, time_grid):
        self.losses, self.times = [], []
        self.current_frame = 0
        self.frames_no = frames_no
        self.total_frames = time_grid.step_no
        self.step = time_grid.step

    def monitor(self, loss):
        freq = 2 * self.total_frames // self.frames_no
        if self.current_frame % freq == 0 and self.current_frame // freq < self.frames_no:
            self.losses.append(loss)
            self.times.append((self.current_frame + 1.0) / 2.0 * self.step)
        self.current_frame += 1


# -------------------------------------------------------------------- propagators
def _bshape(nd, axis, n):
    s = [1] * nd
    s[axis] = n
    return s


class OneDimPropagator:
    """one_dim_propagator.rs:9-76: every lane along ``dimension_no`` *= op."""

    def __init__(self, shape: int, dimension_no: int):
        self.dimension_no = dimension_no
        self.operator = np.ones(shape, dtype=np.complex128)
        self.loss_checked: Optional[LossChecker] = None

    def set_operator(self, op):
        op = np.asarray(op, dtype=np.complex128)
        assert op.shape[0] == self.operator.shape[0]
        self.operator = op.copy()

    def add_operator(self, op):
        op = np.asarray(op, dtype=np.complex128)
        assert op.shape[0] == self.operator.shape[0]
        self.operator = self.operator * op

    def set_loss_checked(self, lc: LossChecker):
        self.loss_checked = lc

    def apply_unchecked(self, wf: WaveFunction):
        wf.change_observer.possible_norm_change = True
        wf.array *= self.operator.reshape(_bshape(wf.array.ndim, self.dimension_no, len(self.operator)))

    def apply(self, wf: WaveFunction):
        if self.loss_checked:
            self.loss_checked.check_before(wf)
        self.apply_unchecked(wf)
        if self.loss_checked:
            self.loss_checked.check_after(wf)

    def loss(self):
        return self.loss_checked

    def loss_reset(self):
        if self.loss_checked:
            self.loss_checked.reset()


class NDimPropagator:
    """n_dim_propagator.rs:8-65: psi *= op (full-size table)."""

    def __init__(self):
        self.operator = np.zeros((1,), dtype=np.complex128)
        self.loss_checked: Optional[LossChecker] = None

    def set_operator(self, op):
        self.operator = np.array(op, dtype=np.complex128)

    def add_operator(self, op):
        op = np.asarray(op, dtype=np.complex128)
        assert op.shape == self.operator.shape
        self.operator = self.operator * op

    def set_loss_checked(self, lc):
        self.loss_checked = lc

    def apply(self, wf):
        if self.loss_checked:
            self.loss_checked.check_before(wf)
        wf.change_observer.possible_norm_change = True
        wf.array *= self.operator
        if self.loss_checked:
            self.loss_checked.check_after(wf)

    def loss(self):
        return self.loss_checked

    def loss_reset(self):
        if self.loss_checked:
            self.loss_checked.reset()


class NonDiagPropagator:
    """non_diagonal_propagator.rs:9-66: lane_i = op_i . lane_i along ``dimension_no``.

    Lanes are enumerated in ndarray's ``lanes_mut`` order: row-major over the
    remaining axes.
    """

    def __init__(self, dimension_no: int):
        self.dimension_no = dimension_no
        self.operators: List[np.ndarray] = []
        self.loss_checked: Optional[LossChecker] = None

    def set_operators(self, ops):
        self.operators = [np.asarray(o, dtype=np.complex128) for o in ops]

    def set_loss_checked(self, lc):
        self.loss_checked = lc

    def apply(self, wf):
        if self.loss_checked:
            self.loss_checked.check_before(wf)
        wf.change_observer.possible_norm_change = True
        a = np.moveaxis(wf.array, self.dimension_no, -1)
        lanes = a.reshape(-1, a.shape[-1])
        # zip stops at the shorter of (operators, lanes), as Iterator::zip does
        for i, op in zip(range(lanes.shape[0]), self.operators):
            lanes[i] = op @ lanes[i]
        wf.array = np.ascontiguousarray(np.moveaxis(lanes.reshape(a.shape), -1, self.dimension_no))
        if self.loss_checked:
            self.loss_checked.check_after(wf)

    def loss(self):
        return self.loss_checked

    def loss_reset(self):
        if self.loss_checked:
            self.loss_checked.reset()


# ------------------------------------------------------------ propagator factory
def one_dim_into_propagator(hamiltonian, grid: Grid, time: TimeGrid, step_kind: int):
    """propagator_factory.rs:10-22: exp(-i H dt) along ``grid.dimension_no``."""
    dt = select_step(step_kind, time)
    p = OneDimPropagator(grid.nodes_no, grid.dimension_no)
    p.set_operator(np.exp(-1j * np.asarray(hamiltonian, dtype=np.float64) * dt))
    return p


def n_dim_into_propagator(hamiltonian, time: TimeGrid, step_kind: int):
    """propagator_factory.rs:25-36"""
    dt = select_step(step_kind, time)
    p = NDimPropagator()
    p.set_operator(np.exp(-1j * np.asarray(hamiltonian, dtype=np.float64) * dt))
    return p


def complex_n_dim_into_propagator(hamiltonian, time: TimeGrid, step_kind: int):
    """propagator_factory.rs:39-50"""
    dt = select_step(step_kind, time)
    p = NDimPropagator()
    p.set_operator(np.exp(-1j * np.asarray(hamiltonian, dtype=np.complex128) * dt))
    return p


# --------------------------------------------------------------- transformations
NORMAL, INVERSE_FIRST = 0, 1


def fft_momentum_grid(grid: Grid, name: str) -> Grid:
    """fft_transformation.rs:28-43: k in FFT order, weights dk halved at N/2-1 and N/2."""
    n = grid.nodes_no
    dk = 2.0 * math.pi / (grid.nodes[-1] - grid.nodes[0]) * (1.0 - 1.0 / n)
    idx = list(range(0, n // 2)) + list(range(-(n // 2), 0))
    momenta = np.array([i * dk for i in idx], dtype=np.float64)
    w = np.full(len(momenta), dk)
    w[n // 2 - 1] *= 0.5
    w[n // 2] *= 0.5
    return Grid.new_custom(name, momenta, w, grid.dimension_no)


class FFTTransformation:
    """fft_transformation.rs:11-89: unitary DFT along one axis (divide by sqrt(N))."""

    def __init__(self, grid: Grid, transformed_grid_name: str):
        self.dimension_no = grid.dimension_no
        self.dimension_size = grid.nodes_no
        self.grid_transformation = fft_momentum_grid(grid, transformed_grid_name)

    def _swap(self, wf):
        d = self.dimension_no
        wf.grids[d], self.grid_transformation = self.grid_transformation, wf.grids[d]
        wf.change_observer.possible_norm_change = True

    def transform(self, wf):
        self._swap(wf)
        wf.array = np.fft.fft(wf.array, axis=self.dimension_no, norm="ortho")

    def inverse_transform(self, wf):
        self._swap(wf)
        wf.array = np.fft.ifft(wf.array, axis=self.dimension_no, norm="ortho")


def _lane_matmul(T, array, axis):
    """lane <- T . lane for every lane along ``axis``."""
    out = np.tensordot(T, array, axes=([1], [axis]))
    return np.ascontiguousarray(np.moveaxis(out, 0, axis))


class MatrixTransformation:
    """matrix_transformation.rs:8-75: dense N x N matrix on every lane of one axis."""

    def __init__(self, grid: Grid, grid_transformation: Grid):
        self.dimension_no = grid.dimension_no
        self.dimension_size = grid.nodes_no
        n = grid.nodes_no
        self.transformation = np.zeros((n, n), dtype=np.complex128)
        self.inverse_transformation = np.zeros((n, n), dtype=np.complex128)
        self.grid_transformation = grid_transformation.copy()

    def set_diagonalization_matrix(self, t, tinv):
        t = np.asarray(t, dtype=np.complex128)
        tinv = np.asarray(tinv, dtype=np.complex128)
        n = self.dimension_size
        assert t.shape == (n, n) and tinv.shape == (n, n)
        self.transformation = t.copy()
        self.inverse_transformation = tinv.copy()

    def _swap(self, wf):
        d = self.dimension_no
        wf.grids[d], self.grid_transformation = self.grid_transformation, wf.grids[d]
        wf.change_observer.possible_norm_change = True

    def transform(self, wf):
        self._swap(wf)
        wf.array = _lane_matmul(self.transformation, wf.array, self.dimension_no)

    def inverse_transform(self, wf):
        self._swap(wf)
        wf.array = _lane_matmul(self.inverse_transformation, wf.array, self.dimension_no)


class StateMatrixTransformation:
    """state_matrix_transformation.rs:8-73: matrix i acts on slice i of a dependent axis."""

    def __init__(self, dimension_no_dependent: int, grid: Grid, grid_transformation: Grid):
        assert dimension_no_dependent > grid.dimension_no
        self.dimension_no = grid.dimension_no
        self.dimension_no_dependent = dimension_no_dependent
        self.transformations: List[np.ndarray] = []
        self.inverse_transformations: List[np.ndarray] = []
        self.grid_transformation = grid_transformation.copy()

    def set_diagonalization_matrices(self, ts, tinvs):
        self.transformations = [np.asarray(t, dtype=np.complex128) for t in ts]
        self.inverse_transformations = [np.asarray(t, dtype=np.complex128) for t in tinvs]

    def _swap(self, wf):
        d = self.dimension_no
        wf.grids[d], self.grid_transformation = self.grid_transformation, wf.grids[d]
        wf.change_observer.possible_norm_change = True

    def _apply(self, wf, mats):
        dep = self.dimension_no_dependent
        arr = wf.array.copy()
        for i, t in zip(range(arr.shape[dep]), mats):
            sl = [slice(None)] * arr.ndim
            sl[dep] = i
            sub = arr[tuple(sl)]  # the dependent axis is removed; dimension_no < dep keeps its index
            arr[tuple(sl)] = _lane_matmul(t, sub, self.dimension_no)
        wf.array = arr

    def transform(self, wf):
        self._swap(wf)
        self._apply(wf, self.transformations)

    def inverse_transform(self, wf):
        self._swap(wf)
        self._apply(wf, self.inverse_transformations)


# ------------------------------------------------------------------------ controls
FIRST_HALF, SECOND_HALF = 1, 2


class LeakControl:
    """leak_control.rs:6-54: remember the norm at the first half, restore it at the second."""

    def __init__(self):
        self.norm = 0.0
        self.loss_checked: Optional[LossChecker] = None

    def name(self):
        return "LeakControl"

    def add_loss_checker(self, lc):
        self.loss_checked = lc

    def first_half(self, wf):
        self.norm = wf.norm()
        if self.loss_checked:
            self.loss_checked.check_before(wf)

    def second_half(self, wf):
        if self.loss_checked:
            self.loss_checked.check_after(wf)
        wf.normalize(self.norm)

    def loss(self):
        return self.loss_checked


def dumping_end(mask_width: float, mask_end: float, grid: Grid):
    """border_dumping.rs:14-33: sine ramp over the last ``mask_width`` of the grid."""
    r_max = grid.nodes[-1]
    out = np.empty(grid.nodes_no, dtype=np.complex128)
    for i, x in enumerate(grid.nodes):
        if x < r_max - mask_width:
            out[i] = 1.0
        elif x > r_max - mask_end:
            out[i] = 0.0
        else:
            out[i] = math.sin(math.pi / 2.0 * (r_max - x) / mask_width)
    return out


class BorderDumping:
    """border_dumping.rs:36-93: mask multiply on both halves, optional loss check."""

    def __init__(self, mask, grid: Grid):
        self.operator = OneDimPropagator(len(mask), grid.dimension_no)
        self.operator.set_operator(mask)
        self.loss_checked: Optional[LossChecker] = None

    def name(self):
        return "BorderDumping"

    def add_loss_checker(self, lc):
        self.loss_checked = lc

    def _half(self, wf):
        if self.loss_checked:
            self.loss_checked.check_before(wf)
        self.operator.apply(wf)
        if self.loss_checked:
            self.loss_checked.check_after(wf)

    def first_half(self, wf):
        self._half(wf)

    def second_half(self, wf):
        self._half(wf)

    def loss(self):
        return self.loss_checked


# -------------------------------------------------------------------------- savers
class StateSaver:
    """wave_function_saver.rs:101-183: state_density(axis) every step_no/frames_no steps."""

    def __init__(self, name, time_grid: TimeGrid, state_grid: Grid, frames_no: int):
        self.name = name
        self.current_frame = 0
        self.frames_no = frames_no
        self.time_grid = time_grid
        self.state_grid = state_grid.copy()
        self.data = np.zeros((state_grid.nodes_no, frames_no))
        self.times: List[float] = []

    def monitor(self, wf):
        freq = self.time_grid.step_no // self.frames_no
        if self.current_frame % freq == 0 and self.current_frame // freq < self.frames_no:
            self.data[:, self.current_frame // freq] = wf.state_density(self.state_grid.dimension_no)
            self.times.append(self.time_grid.step * (self.current_frame + 1.0))
        self.current_frame += 1

    def reset(self):
        self.data = np.zeros((self.state_grid.nodes_no, self.frames_no))


class WaveFunctionSaver:
    """wave_function_saver.rs:6-98: |psi|^2 frames of a 2-D wave function."""

    def __init__(self, name, time_grid, x_grid, y_grid, frames_no):
        self.name = name
        self.current_frame = 0
        self.frames_no = frames_no
        self.time_grid = time_grid
        self.data = np.zeros((x_grid.nodes_no, y_grid.nodes_no, frames_no))
        self.times: List[float] = []

    def monitor(self, wf):
        assert wf.array.ndim == 2
        freq = self.time_grid.step_no // self.frames_no
        if self.current_frame % freq == 0 and self.current_frame // freq < self.frames_no:
            self.data[:, :, self.current_frame // freq] = wf.density()
            self.times.append(self.time_grid.step * (self.current_frame + 1.0))
        self.current_frame += 1

    def reset(self):
        self.data = np.zeros_like(self.data)


# ------------------------------------------------------------ stack + propagation
@dataclass
class _Op:
    kind: str  # "propagator" | "transformation" | "saver" | "control"
    obj: object
    flag: int = 0  # Order for transformations, Apply bits for savers/controls


@dataclass
class OperationStack:
    """propagation.rs:26-65"""

    stack: List[_Op] = field(default_factory=list)

    def add_propagator(self, p):
        self.stack.append(_Op("propagator", p))

    def add_transformation(self, t, order=NORMAL):
        self.stack.append(_Op("transformation", t, order))

    def add_saver(self, s, apply):
        assert apply != 0
        self.stack.append(_Op("saver", s, apply))

    def add_control(self, c, apply):
        self.stack.append(_Op("control", c, apply))


class Propagation:
    """propagation.rs:72-292"""

    def __init__(self, wave_function: WaveFunction, time_grid: TimeGrid, stack: OperationStack):
        self.wave_function = wave_function
        self.time_grid = time_grid
        self.operation_stack = stack

    def step(self):
        """propagation.rs:134-182"""
        wf = self.wave_function
        ops = self.operation_stack.stack
        for op in ops:
            if op.kind == "propagator":
                op.obj.apply(wf)
            elif op.kind == "transformation":
                (op.obj.transform if op.flag == NORMAL else op.obj.inverse_transform)(wf)
            elif op.kind == "saver":
                if op.flag & FIRST_HALF:
                    op.obj.monitor(wf)
            else:
                if op.flag & FIRST_HALF:
                    op.obj.first_half(wf)
        for op in list(reversed(ops))[1:]:
            if op.kind == "propagator":
                op.obj.apply(wf)
            elif op.kind == "transformation":
                (op.obj.inverse_transform if op.flag == NORMAL else op.obj.transform)(wf)
            elif op.kind == "saver":
                if op.flag & SECOND_HALF:
                    op.obj.monitor(wf)
            else:
                if op.flag & SECOND_HALF:
                    op.obj.second_half(wf)

    def propagate(self, steps: Optional[int] = None):
        """propagation.rs:185-190 (``steps`` overrides ``time_grid.step_no``)."""
        for _ in range(self.time_grid.step_no if steps is None else steps):
            self.step()

    def get_losses(self):
        """propagation.rs:213-231: losses of *propagators* only."""
        out = []
        for op in self.operation_stack.stack:
            if op.kind == "propagator" and op.obj.loss() is not None:
                out.append(op.obj.loss().loss())
        return out

    def all_losses(self):
        """Losses of propagators and controls, in stack order (print_losses, :193-210)."""
        out = []
        for op in self.operation_stack.stack:
            if op.kind in ("propagator", "control") and op.obj.loss() is not None:
                out.append((op.obj.loss().name, op.obj.loss().loss()))
        return out

    def reset_losses(self):
        for op in self.operation_stack.stack:
            if op.kind == "propagator":
                op.obj.loss_reset()

    def mean_energy(self) -> float:
        """propagation.rs:245-291"""
        if self.time_grid.im_time:
            op0 = self.operation_stack.stack[0]
            assert op0.kind == "control" and op0.obj.name() == "LeakControl"
            lc = op0.obj.loss()
            assert lc is not None
            lc.reset()
            self.step()
            decay = lc.loss()
            return -math.log(self.wave_function.norm() - decay) / self.time_grid.step / 2.0
        before = self.wave_function.clone()
        self.step()
        after = self.wave_function.clone()
        return -np.angle(after.dot(before)) / self.time_grid.step


# --------------------------------------------------------------- hamiltonians
def momenta_fft_order(grid: Grid):
    """kinetic_operator.rs:9-16 (same momentum grid as fft_transformation.rs:28-33)."""
    n = grid.nodes_no
    dk = 2.0 * math.pi / (grid.nodes[-1] - grid.nodes[0]) * (1.0 - 1.0 / n)
    idx = list(range(0, n // 2)) + list(range(-(n // 2), 0))
    return np.array([i * dk for i in idx], dtype=np.float64)


def kinetic_hamiltonian(grid: Grid, red_mass: float):
    """kinetic_operator.rs:8-21: k^2 / (2 mu); mu given directly."""
    k = momenta_fft_order(grid)
    return k * k / (2.0 * red_mass)


def rotational_hamiltonian(radial: Grid, polar: Grid, red_mass: float, rotational_const: float):
    """rotational_operator.rs:7-26: l(l+1) (B + 1/(2 mu r^2)) on (r, l)."""
    l = np.arange(polar.nodes_no, dtype=np.int64)
    ll = (l * (l + 1)).astype(np.float64)
    r = radial.nodes
    return ll[None, :] * (rotational_const + 1.0 / (2.0 * red_mass * r[:, None] * r[:, None]))


def two_dim_into_n_dim_operator(shape, hamiltonian, grid1: Grid, grid2: Grid):
    """hamiltonian_broadcasting.rs:6-23: broadcast (grid1, grid2) table to the full shape."""
    nd = len(shape)
    out = np.zeros(shape, dtype=np.float64)
    view = np.moveaxis(out, [grid1.dimension_no, grid2.dimension_no], [nd - 2, nd - 1])
    view += np.asarray(hamiltonian, dtype=np.float64)
    return out


def legendre_polynomials(j: int, x: float):
    """special_functions.rs:3-14 (writes p[1], so j >= 1)."""
    p = [0.0] * (j + 1)
    p[0] = 1.0
    p[1] = x
    for i in range(2, j + 1):
        p[i] = ((2 * i - 1) / i) * x * p[i - 1] - ((i - 1) / i) * p[i - 2]
    return p


def double_factorial(n: int) -> float:
    """special_functions.rs:43-55 (as written: n * (n-2 ... ) over range(2, n-1) step -2)."""
    assert n < 100
    if n == 0:
        return 1.0
    value = float(n)
    for k in range(n - 2, 1, -2):  # (2..n-1).rev().step_by(2): n-2, n-4, ... > 1
        value *= float(k)
    return value


def _negate_m(l: int, m: int) -> float:
    """special_functions.rs:57-83"""
    assert m < 50
    if m > 0:
        v = (-1.0) ** m
        for k in range(l - m, l + m):
            v /= k + 1.0
        return v
    if m < 0:
        v = (-1.0) ** m
        for k in range(l + m, l - m):
            v *= k + 1.0
        return v
    return 1.0


def normalization(l: int, m: int) -> float:
    """special_functions.rs:85-116"""
    assert m < 50
    if m > 0:
        v = 1.0
        for k in range(l - m, l + m):
            v /= k + 1.0
    elif m < 0:
        v = 1.0
        for k in range(l + m, l - m):
            v *= k + 1.0
    else:
        v = 1.0
    return math.sqrt(v * (l + 0.5))


def associated_legendre_polynomials(j: int, m: int, x: float):
    """special_functions.rs:17-41"""
    mu = abs(m)
    if m == 0:
        return legendre_polynomials(j, x)
    p = [0.0] * (j + 1)
    p[mu] = (-1.0) ** m * double_factorial(2 * mu - 1) * (1.0 - x * x) ** (mu / 2.0)
    if m < 0:
        p[mu] *= _negate_m(mu, mu)
        p[mu + 1] = x * p[mu]
    else:
        p[mu + 1] = x * (2.0 * mu + 1.0) * p[mu]
    for i in range(mu + 2, j + 1):
        l = i - 1
        p[i] = ((2 * l + 1) * x * p[i - 1] - (l + m) * p[i - 2]) / (l - m + 1.0)
    return p


def legendre_matrices(polar: Grid):
    """legendre_diagonalization.rs:13-45: T[l,j] = sqrt(l+1/2) P_l(cos th_j) w_j, T^-1 = (unweighted)^T."""
    n = polar.nodes_no
    lmax = n - 1
    t = np.zeros((n, n), dtype=np.float64)
    for j in range(n):
        pl = legendre_polynomials(lmax, math.cos(polar.nodes[j]))
        for i in range(n):
            t[i, j] = math.sqrt(i + 0.5) * pl[i]
    tinv = t.T.copy()
    t = t * polar.weights[None, :]
    return t.astype(np.complex128), tinv.astype(np.complex128)


def legendre_diagonalization_operator(polar: Grid) -> MatrixTransformation:
    """legendre_diagonalization.rs:13-45"""
    n = polar.nodes_no
    lgrid = Grid.new_linear_countable("angular_momentum", 0.0, float(n - 1), n, polar.dimension_no)
    mt = MatrixTransformation(polar, lgrid)
    t, tinv = legendre_matrices(polar)
    mt.set_diagonalization_matrix(t, tinv)
    return mt


def associated_legendre_matrices(polar: Grid, omega: int):
    """legendre_diagonalization.rs:48-80"""
    n = polar.nodes_no
    lmax = n - 1
    t = np.zeros((n, n), dtype=np.float64)
    for j in range(n):
        pl = associated_legendre_polynomials(lmax, omega, math.cos(polar.nodes[j]))
        for i in range(abs(omega), n):
            t[i, j] = normalization(i, omega) * pl[i]
    tinv = t.T.copy()
    t = t * polar.weights[None, :]
    return t.astype(np.complex128), tinv.astype(np.complex128)


def associated_legendre_diagonalization_operator(polar: Grid, omega: int) -> MatrixTransformation:
    n = polar.nodes_no
    lgrid = Grid.new_linear_countable("angular_momentum", 0.0, float(n - 1), n, polar.dimension_no)
    mt = MatrixTransformation(polar, lgrid)
    t, tinv = associated_legendre_matrices(polar, omega)
    mt.set_diagonalization_matrix(t, tinv)
    return mt


def associated_legendre_operator(polar: Grid, omega_grid: Grid) -> StateMatrixTransformation:
    """legendre_diagonalization.rs:83-109"""
    n = polar.nodes_no
    lgrid = Grid.new_linear_countable("angular_momentum", 0.0, float(n - 1), n, polar.dimension_no)
    smt = StateMatrixTransformation(omega_grid.dimension_no, polar, lgrid)
    ts, tis = [], []
    for om in omega_grid.nodes:
        t, ti = associated_legendre_matrices(polar, int(om))
        ts.append(t)
        tis.append(ti)
    smt.set_diagonalization_matrices(ts, tis)
    return smt


# ------------------------------------------------------------------- potentials
def _nan_to_inf(v):
    return np.where(np.isnan(v), np.inf, v)


def dispersion(r, n, cn):
    """analytic_potentials.rs:2-10"""
    return _nan_to_inf(cn * np.asarray(r, dtype=np.float64) ** n)


def lennard_jones(r, d6, r6):
    """analytic_potentials.rs:13-22"""
    rr = (r6 / np.asarray(r, dtype=np.float64)) ** 6
    return _nan_to_inf(d6 * rr * (rr - 2.0))


def harmonic(r, r0, mass, omega):
    """analytic_potentials.rs:24-32"""
    return _nan_to_inf(0.5 * mass * omega ** 2 * (np.asarray(r, dtype=np.float64) - r0) ** 2)


def morse(r, d, a, re):
    """Morse term D (1 - e^{-a (r - re)})^2 (no reference counterpart)."""
    e = np.exp(-a * (np.asarray(r, dtype=np.float64) - re))
    return _nan_to_inf(d * (1.0 - e) ** 2)


def gauss_legendre(n: int):
    """Gauss-Legendre nodes x (ascending) and weights on [-1, 1] (numpy leggauss)."""
    return np.polynomial.legendre.leggauss(n)
