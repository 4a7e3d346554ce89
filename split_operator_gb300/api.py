"""Python mirror of the split_operator crate's API over the C ABI.

Names, argument meaning and error behaviour follow the Rust crate
(Wleter/split_operator): ``Grid``, ``WaveFunction``, ``TimeGrid``,
``one_dim_into_propagator`` ... ``Propagation``.  Every call goes through
``libsplit_operator_gb300.so``; arrays are numpy complex128 on the host side and
live in GPU memory inside the library.
"""
import ctypes as C
from typing import List, Optional, Sequence

import numpy as np

from ._lib import SplitOperatorError, TimeGridC, call, lib  # noqa: F401

# time_grid.rs:15-18, transformation.rs:13-16, control.rs:19-26
FULL, HALF = 0, 1
NORMAL, INVERSE_FIRST = 0, 1
APPLY_NONE, FIRST_HALF, SECOND_HALF = 0, 1, 2

PRECISION = {"fp64": 0, "fp32_tf32x3": 1, "fp32_bf16x3": 2, "fp32_simt": 3, "fp32_bf16x6": 4, "float_float": 5}


def _dp(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def _c128(a):
    return np.ascontiguousarray(np.asarray(a, dtype=np.complex128))


def _f64(a):
    return np.ascontiguousarray(np.asarray(a, dtype=np.float64))


def _sizes(shape):
    return (C.c_size_t * len(shape))(*shape)


class _Handle:
    _free = None

    def __init__(self, h):
        self._h = h

    @property
    def handle(self):
        return self._h

    def __del__(self):
        h = getattr(self, "_h", None)
        if h and self._free:
            try:
                getattr(lib(), self._free)(h)
            except Exception:
                pass
            self._h = None


def _new(fn, *args):
    out = C.c_void_p()
    call(fn, *args, C.byref(out))
    return out


class TimeGrid:
    """time_grid.rs:7-11"""

    def __init__(self, step: float, step_no: int, im_time: bool = False):
        self.step, self.step_no, self.im_time = float(step), int(step_no), bool(im_time)

    def c(self):
        return TimeGridC(self.step, self.step_no, 1 if self.im_time else 0)


class Grid(_Handle):
    """grid.rs:14-89"""

    _free = "so_grid_free"

    @staticmethod
    def new_linear_continuos(name, start, end, nodes_no, dimension_no):
        return Grid(_new("so_grid_new_linear_continuos", name.encode(), start, end, nodes_no, dimension_no))

    @staticmethod
    def new_linear_countable(name, start, end, nodes_no, dimension_no):
        return Grid(_new("so_grid_new_linear_countable", name.encode(), start, end, nodes_no, dimension_no))

    @staticmethod
    def new_custom(name, nodes, weights, dimension_no):
        n, w = _f64(nodes), _f64(weights)
        if len(n) != len(w):
            raise ValueError("nodes and weights differ in length")
        return Grid(_new("so_grid_new_custom", name.encode(), _dp(n), _dp(w), len(n), dimension_no))

    @property
    def nodes_no(self):
        v = C.c_size_t()
        call("so_grid_nodes_no", self._h, C.byref(v))
        return v.value

    @property
    def dimension_no(self):
        v = C.c_size_t()
        call("so_grid_dimension_no", self._h, C.byref(v))
        return v.value

    @property
    def name(self):
        buf = C.create_string_buffer(256)
        call("so_grid_name", self._h, buf, 256)
        return buf.value.decode()

    @property
    def nodes(self):
        a = np.empty(self.nodes_no)
        call("so_grid_nodes", self._h, _dp(a))
        return a

    @property
    def weights(self):
        a = np.empty(self.nodes_no)
        call("so_grid_weights", self._h, _dp(a))
        return a


class WaveFunction(_Handle):
    """wave_function.rs:11-149 (array in GPU memory)."""

    _free = "so_wave_function_free"

    def __init__(self, array=None, grids: Sequence[Grid] = (), _handle=None):
        if _handle is not None:
            super().__init__(_handle)
            return
        a = _c128(array)
        gs = (C.c_void_p * len(grids))(*[g.handle for g in grids])
        super().__init__(
            _new("so_wave_function_new", _dp(a.view(np.float64)), _sizes(a.shape), a.ndim,
                 C.cast(gs, C.POINTER(C.c_void_p)))
        )

    @property
    def shape(self):
        nd = C.c_size_t()
        shp = (C.c_size_t * 8)()
        call("so_wave_function_ndim", self._h, C.byref(nd), shp)
        return tuple(shp[i] for i in range(nd.value))

    @property
    def array(self):
        out = np.empty(self.shape, dtype=np.complex128)
        call("so_wave_function_get_array", self._h, _dp(out.view(np.float64)))
        return out

    @array.setter
    def array(self, value):
        a = _c128(value)
        if a.shape != self.shape:
            raise ValueError("shape differs")
        call("so_wave_function_set_array", self._h, _dp(a.view(np.float64)))

    def grid(self, axis) -> Grid:
        return Grid(_new("so_wave_function_grid", self._h, axis))

    @property
    def grids(self) -> List[Grid]:
        return [self.grid(a) for a in range(len(self.shape))]

    def clone(self):
        return WaveFunction(_handle=_new("so_wave_function_clone", self._h))

    def norm(self) -> float:
        v = C.c_double()
        call("so_wave_function_norm", self._h, C.byref(v))
        return v.value

    def normalize(self, new_norm: float):
        call("so_wave_function_normalize", self._h, new_norm)

    def dot(self, other: "WaveFunction") -> complex:
        out = np.empty(2)
        call("so_wave_function_dot", self._h, other.handle, _dp(out))
        return complex(out[0], out[1])

    def density(self):
        out = np.empty(self.shape)
        call("so_wave_function_density", self._h, _dp(out))
        return out

    def state_density(self, axis: int):
        shp = self.shape
        out = np.empty(shp[0] if len(shp) == 1 else shp[axis])
        if len(shp) == 1:
            out = np.empty(shp)
        call("so_wave_function_state_density", self._h, axis, _dp(out))
        return out


def gaussian_distribution(x, x0, sigma, momentum):
    """wave_function.rs:152-154"""
    x = _f64(np.atleast_1d(x))
    out = np.empty(len(x), dtype=np.complex128)
    call("so_gaussian_distribution", _dp(x), len(x), x0, sigma, momentum, _dp(out.view(np.float64)))
    return out


class Operator(_Handle):
    _free = "so_operator_free"


class Propagator(Operator):
    """propagator.rs:12-18"""

    def apply(self, wf: WaveFunction):
        call("so_propagator_apply", self._h, wf.handle)

    def set_loss_checked(self, name: str):
        call("so_propagator_set_loss_checked", self._h, name.encode())

    def loss(self) -> Optional[float]:
        v, has = C.c_double(), C.c_int()
        call("so_propagator_loss", self._h, C.byref(v), C.byref(has))
        return v.value if has.value else None

    def loss_reset(self):
        call("so_propagator_loss_reset", self._h)


class OneDimPropagator(Propagator):
    """one_dim_propagator.rs:9-76"""

    def __init__(self, shape: int, dimension_no: int):
        super().__init__(_new("so_one_dim_propagator_new", shape, dimension_no))

    def set_operator(self, op):
        a = _c128(op)
        call("so_one_dim_propagator_set_operator", self._h, _dp(a.view(np.float64)), len(a))

    def add_operator(self, op):
        a = _c128(op)
        call("so_one_dim_propagator_add_operator", self._h, _dp(a.view(np.float64)), len(a))


class NDimPropagator(Propagator):
    """n_dim_propagator.rs:8-65"""

    def __init__(self, _handle=None):
        super().__init__(_handle if _handle is not None else _new("so_n_dim_propagator_new"))

    def set_operator(self, op):
        a = _c128(op)
        call("so_n_dim_propagator_set_operator", self._h, _dp(a.view(np.float64)), _sizes(a.shape), a.ndim)

    def add_operator(self, op):
        a = _c128(op)
        call("so_n_dim_propagator_add_operator", self._h, _dp(a.view(np.float64)), _sizes(a.shape), a.ndim)


class NonDiagPropagator(Propagator):
    """non_diagonal_propagator.rs:9-66"""

    def __init__(self, dimension_no: int):
        super().__init__(_new("so_non_diag_propagator_new", dimension_no))

    def set_operators(self, ops):
        a = _c128(ops)
        count, n, _ = a.shape
        call("so_non_diag_propagator_set_operators", self._h, _dp(a.view(np.float64)), count, n)


def one_dim_into_propagator(hamiltonian, grid: Grid, time: TimeGrid, step: int) -> OneDimPropagator:
    """propagator_factory.rs:10-22"""
    h = _f64(hamiltonian)
    p = OneDimPropagator.__new__(OneDimPropagator)
    Operator.__init__(p, _new("so_one_dim_into_propagator", _dp(h), grid.handle, time.c(), step))
    return p


def n_dim_into_propagator(hamiltonian, time: TimeGrid, step: int) -> NDimPropagator:
    """propagator_factory.rs:25-36"""
    h = _f64(hamiltonian)
    return NDimPropagator(_handle=_new("so_n_dim_into_propagator", _dp(h), _sizes(h.shape), h.ndim, time.c(), step))


def complex_n_dim_into_propagator(hamiltonian, time: TimeGrid, step: int) -> NDimPropagator:
    """propagator_factory.rs:39-50"""
    h = _c128(hamiltonian)
    return NDimPropagator(
        _handle=_new("so_complex_n_dim_into_propagator", _dp(h.view(np.float64)), _sizes(h.shape), h.ndim, time.c(),
                     step)
    )


class Transformation(Operator):
    """transformation.rs:5-11"""

    def transform(self, wf: WaveFunction):
        call("so_transformation_transform", self._h, wf.handle)

    def inverse_transform(self, wf: WaveFunction):
        call("so_transformation_inverse_transform", self._h, wf.handle)

    @property
    def grid_transformation(self) -> Grid:
        return Grid(_new("so_transformation_grid", self._h))


class FFTTransformation(Transformation):
    """fft_transformation.rs:11-89"""

    def __init__(self, grid: Grid, transformed_grid_name: str):
        super().__init__(_new("so_fft_transformation_new", grid.handle, transformed_grid_name.encode()))


class MatrixTransformation(Transformation):
    """matrix_transformation.rs:8-75"""

    def __init__(self, grid: Grid = None, grid_transformation: Grid = None, _handle=None):
        super().__init__(_handle if _handle is not None else
                         _new("so_matrix_transformation_new", grid.handle, grid_transformation.handle))

    def set_diagonalization_matrix(self, t, tinv):
        a, b = _c128(t), _c128(tinv)
        call("so_matrix_transformation_set_diagonalization_matrix", self._h, _dp(a.view(np.float64)),
             _dp(b.view(np.float64)), a.shape[0])


class StateMatrixTransformation(Transformation):
    """state_matrix_transformation.rs:8-73"""

    def __init__(self, dimension_no_dependent=0, grid: Grid = None, grid_transformation: Grid = None, _handle=None):
        super().__init__(_handle if _handle is not None else
                         _new("so_state_matrix_transformation_new", dimension_no_dependent, grid.handle,
                              grid_transformation.handle))

    def set_diagonalization_matrices(self, ts, tinvs):
        a, b = _c128(ts), _c128(tinvs)
        count, n, _ = a.shape
        call("so_state_matrix_transformation_set_diagonalization_matrices", self._h, _dp(a.view(np.float64)),
             _dp(b.view(np.float64)), count, n)


# ------------------------------------------------------------ hamiltonian factory
def kinetic_hamiltonian(grid: Grid, red_mass: float):
    """kinetic_operator.rs:8-21"""
    out = np.empty(grid.nodes_no)
    call("so_kinetic_hamiltonian", grid.handle, red_mass, _dp(out))
    return out


def rotational_hamiltonian(radial: Grid, polar: Grid, red_mass: float, rotational_const: float):
    """rotational_operator.rs:7-26"""
    out = np.empty((radial.nodes_no, polar.nodes_no))
    call("so_rotational_hamiltonian", radial.handle, polar.handle, red_mass, rotational_const, _dp(out))
    return out


def two_dim_into_n_dim_operator(shape, hamiltonian, grid1: Grid, grid2: Grid):
    """hamiltonian_broadcasting.rs:6-23"""
    h = _f64(hamiltonian)
    out = np.empty(tuple(shape))
    call("so_two_dim_into_n_dim_operator", _sizes(shape), len(shape), _dp(h), grid1.handle, grid2.handle, _dp(out))
    return out


def legendre_diagonalization_operator(polar: Grid) -> MatrixTransformation:
    """legendre_diagonalization.rs:13-45"""
    return MatrixTransformation(_handle=_new("so_legendre_diagonalization_operator", polar.handle))


def associated_legendre_diagonalization_operator(polar: Grid, omega: int) -> MatrixTransformation:
    """legendre_diagonalization.rs:48-80"""
    return MatrixTransformation(_handle=_new("so_associated_legendre_diagonalization_operator", polar.handle, omega))


def associated_legendre_operator(polar: Grid, omega_grid: Grid) -> StateMatrixTransformation:
    """legendre_diagonalization.rs:83-109"""
    return StateMatrixTransformation(_handle=_new("so_associated_legendre_operator", polar.handle, omega_grid.handle))


def legendre_polynomials(j: int, x: float):
    out = np.empty(j + 1)
    call("so_legendre_polynomials", j, x, _dp(out))
    return out


def associated_legendre_polynomials(j: int, m: int, x: float):
    out = np.empty(j + 1)
    call("so_associated_legendre_polynomials", j, m, x, _dp(out))
    return out


def gauss_legendre(n: int):
    x, w = np.empty(n), np.empty(n)
    call("so_gauss_legendre", n, _dp(x), _dp(w))
    return x, w


def _pot(fn, r, *args):
    r = _f64(r)
    out = np.empty(r.shape)
    call(fn, _dp(r), r.size, *args, _dp(out))
    return out


def dispersion(r, n, cn):
    return _pot("so_dispersion", r, n, cn)


def lennard_jones(r, d6, r6):
    return _pot("so_lennard_jones", r, d6, r6)


def harmonic(r, r0, mass, omega):
    return _pot("so_harmonic", r, r0, mass, omega)


def morse(r, d, a, re):
    return _pot("so_morse", r, d, a, re)


# ------------------------------------------------------------------------ controls
class Control(Operator):
    """control.rs:6-17"""

    def first_half(self, wf: WaveFunction):
        call("so_control_first_half", self._h, wf.handle)

    def second_half(self, wf: WaveFunction):
        call("so_control_second_half", self._h, wf.handle)

    def loss(self) -> Optional[float]:
        v, has = C.c_double(), C.c_int()
        call("so_control_loss", self._h, C.byref(v), C.byref(has))
        return v.value if has.value else None


class LeakControl(Control):
    """leak_control.rs:6-54"""

    def __init__(self):
        super().__init__(_new("so_leak_control_new"))

    def add_loss_checker(self, name: str):
        call("so_leak_control_add_loss_checker", self._h, name.encode())


def dumping_end(mask_width: float, mask_end: float, grid: Grid):
    """border_dumping.rs:14-33"""
    out = np.empty(grid.nodes_no, dtype=np.complex128)
    call("so_dumping_end", mask_width, mask_end, grid.handle, _dp(out.view(np.float64)))
    return out


class BorderDumping(Control):
    """border_dumping.rs:36-93"""

    def __init__(self, mask, grid: Grid):
        m = _c128(mask)
        super().__init__(_new("so_border_dumping_new", _dp(m.view(np.float64)), len(m), grid.handle))

    def add_loss_checker(self, name: str):
        call("so_border_dumping_add_loss_checker", self._h, name.encode())


# -------------------------------------------------------------------------- savers
class Saver(Operator):
    """saver.rs:5-14"""

    def frames(self):
        pts, fr = C.c_size_t(), C.c_size_t()
        call("so_saver_shape", self._h, C.byref(pts), C.byref(fr))
        data = np.empty(pts.value * fr.value)
        times = np.empty(fr.value)
        taken = C.c_size_t()
        call("so_saver_frames", self._h, _dp(data), _dp(times), C.byref(taken))
        return data, times[: taken.value]

    def save(self):
        call("so_saver_save", self._h)

    def reset(self):
        call("so_saver_reset", self._h)

    def monitor(self, wf: WaveFunction):
        call("so_saver_monitor", self._h, wf.handle)


class StateSaver(Saver):
    """wave_function_saver.rs:101-183"""

    def __init__(self, name: str, time: TimeGrid, state_grid: Grid, frames_no: int):
        super().__init__(_new("so_state_saver_new", name.encode(), time.c(), state_grid.handle, frames_no))
        self._n = state_grid.nodes_no

    @property
    def data(self):
        d, _ = self.frames()
        return d.reshape(self._n, -1)

    @property
    def times(self):
        return self.frames()[1]


class WaveFunctionSaver(Saver):
    """wave_function_saver.rs:6-98"""

    def __init__(self, name: str, time: TimeGrid, x_grid: Grid, y_grid: Grid, frames_no: int):
        super().__init__(_new("so_wave_function_saver_new", name.encode(), time.c(), x_grid.handle, y_grid.handle,
                              frames_no))
        self._shape = (x_grid.nodes_no, y_grid.nodes_no)

    @property
    def data(self):
        d, _ = self.frames()
        return d.reshape(self._shape[0], self._shape[1], -1)

    @property
    def times(self):
        return self.frames()[1]


# ---------------------------------------------------------------- stack + propagation
class OperationStack(_Handle):
    """propagation.rs:26-65"""

    _free = "so_operation_stack_free"

    def __init__(self):
        super().__init__(_new("so_operation_stack_new"))
        self._ops = []

    def add_propagator(self, p: Propagator):
        call("so_operation_stack_add_propagator", self._h, p.handle)
        self._ops.append(p)

    def add_transformation(self, t: Transformation, order: int = NORMAL):
        call("so_operation_stack_add_transformation", self._h, t.handle, order)
        self._ops.append(t)

    def add_saver(self, s: Saver, apply: int):
        call("so_operation_stack_add_saver", self._h, s.handle, apply)
        self._ops.append(s)

    def add_control(self, c: Control, apply: int):
        call("so_operation_stack_add_control", self._h, c.handle, apply)
        self._ops.append(c)

    def operations_len(self):
        v = C.c_size_t()
        call("so_operation_stack_len", self._h, C.byref(v))
        return v.value


class Propagation(_Handle):
    """propagation.rs:72-292 (``precision``: 'fp64', 'fp32_tf32x3', 'fp32_bf16x3', 'fp32_bf16x6',
    'fp32_simt', 'float_float')."""

    _free = "so_propagation_free"

    def __init__(self, wave_function: WaveFunction, time_grid: TimeGrid, operation_stack: OperationStack,
                 precision: str = "fp64"):
        super().__init__(_new("so_propagation_new", wave_function.handle, time_grid.c(), operation_stack.handle,
                              PRECISION[precision]))
        self._stack = operation_stack
        self.time_grid = time_grid

    def propagate(self):
        call("so_propagation_propagate", self._h)

    def steps(self, n: int):
        call("so_propagation_steps", self._h, n)

    def mean_energy(self) -> float:
        v = C.c_double()
        call("so_propagation_mean_energy", self._h, C.byref(v))
        return v.value

    def _losses(self, fn):
        cnt = C.c_size_t()
        call(fn, self._h, None, 0, C.byref(cnt))
        out = np.empty(cnt.value)
        call(fn, self._h, _dp(out), cnt.value, C.byref(cnt))
        return list(out)

    def get_losses(self):
        return self._losses("so_propagation_get_losses")

    def all_losses(self):
        return self._losses("so_propagation_all_losses")

    def reset_losses(self):
        call("so_propagation_reset_losses", self._h)

    def reset_savers_state(self):
        call("so_propagation_reset_savers_state", self._h)

    def savers_save(self):
        call("so_propagation_savers_save", self._h)

    def wave_function(self) -> WaveFunction:
        return WaveFunction(_handle=_new("so_propagation_wave_function", self._h))

    def get_array(self, out=None):
        wf_shape = self.wave_function_shape()
        if out is None:
            out = np.empty(wf_shape, dtype=np.complex128)
        call("so_propagation_get_array", self._h, _dp(out.view(np.float64)))
        return out

    def set_array(self, a):
        a = _c128(a)
        call("so_propagation_set_array", self._h, _dp(a.view(np.float64)))

    def set_array_ptr(self, host_ptr: int):
        """Replace the state from a host buffer (complex128, logical order) given by address."""
        call("so_propagation_set_array", self._h, C.cast(C.c_void_p(host_ptr), C.POINTER(C.c_double)))

    def get_array_ptr(self, host_ptr: int):
        call("so_propagation_get_array", self._h, C.cast(C.c_void_p(host_ptr), C.POINTER(C.c_double)))

    def wave_function_shape(self):
        if not hasattr(self, "_shape"):
            self._shape = self.wave_function().shape
        return self._shape

    def norm(self) -> float:
        v = C.c_double()
        call("so_propagation_norm", self._h, C.byref(v))
        return v.value

    def set_stream(self, stream_ptr: int):
        call("so_propagation_set_stream", self._h, C.c_void_p(stream_ptr))

    def synchronize(self):
        call("so_propagation_synchronize", self._h)

    def describe(self) -> str:
        buf = C.create_string_buffer(1 << 16)
        call("so_propagation_describe", self._h, buf, 1 << 16)
        return buf.value.decode()

    def set_timing(self, enabled: bool):
        call("so_propagation_set_timing", self._h, 1 if enabled else 0)

    def steps_done(self) -> int:
        v = C.c_uint64()
        call("so_propagation_steps_done", self._h, C.byref(v))
        return v.value

    def checkpoint(self) -> bytes:
        """Everything the next steps read (state, norm cache, losses, leak norm, savers,
        step count) as one byte string; restore() on a propagation built the same way
        continues bit for bit."""
        n = C.c_size_t()
        call("so_propagation_checkpoint", self._h, None, 0, C.byref(n))
        buf = C.create_string_buffer(n.value)
        call("so_propagation_checkpoint", self._h, buf, n.value, C.byref(n))
        return buf.raw[: n.value]

    def restore(self, blob: bytes):
        call("so_propagation_restore", self._h, C.c_char_p(blob), len(blob))

    def save_checkpoint(self, path: str):
        """The checkpoint as a one-dimensional uint8 .npy file."""
        np.save(path, np.frombuffer(self.checkpoint(), dtype=np.uint8))

    def load_checkpoint(self, path: str):
        self.restore(np.load(path).tobytes())

    def kernel_times(self):
        """[(pass name, launches, total_ms, algorithmic bytes)] since the last call."""
        buf = C.create_string_buffer(1 << 16)
        call("so_propagation_kernel_times", self._h, buf, 1 << 16)
        out = []
        for line in buf.value.decode().splitlines():
            name, n, ms, b = line.split("\t")
            out.append((name, int(n), float(ms), float(b)))
        return out


class Batch(_Handle):
    """Many independent propagations stepped together (batched launches, CUDA graph)."""

    _free = "so_batch_free"

    def __init__(self, propagations: Sequence[Propagation]):
        arr = (C.c_void_p * len(propagations))(*[p.handle for p in propagations])
        super().__init__(_new("so_batch_new", C.cast(arr, C.POINTER(C.c_void_p)), len(propagations)))
        self._props = list(propagations)

    def steps(self, n: int):
        call("so_batch_steps", self._h, n)

    def set_timing(self, enabled: bool):
        call("so_batch_set_timing", self._h, 1 if enabled else 0)

    def kernel_times(self):
        buf = C.create_string_buffer(1 << 18)
        call("so_batch_kernel_times", self._h, buf, 1 << 18)
        out = []
        for line in buf.value.decode().splitlines():
            name, n, ms, b = line.split("\t")
            out.append((name, int(n), float(ms), float(b)))
        return out

    def launches_per_step(self) -> int:
        v = C.c_size_t()
        call("so_batch_launches_per_step", self._h, C.byref(v))
        return v.value

    def set_arrays_ptr(self, host_ptrs: Sequence[int]):
        """Every member's state from host addresses (logical complex128 each; page-locked
        buffers are read by the layout kernels directly)."""
        arr = (C.c_void_p * len(host_ptrs))(*host_ptrs)
        call("so_batch_set_arrays", self._h, C.cast(arr, C.POINTER(C.c_void_p)), len(host_ptrs))

    def get_arrays_ptr(self, host_ptrs: Sequence[int]):
        """Every member's state into host addresses; returns when all are written."""
        arr = (C.c_void_p * len(host_ptrs))(*host_ptrs)
        call("so_batch_get_arrays", self._h, C.cast(arr, C.POINTER(C.c_void_p)), len(host_ptrs))

    def tune(self, cache_path: Optional[str] = None, trial_steps: int = 4) -> dict:
        """Autotune the launch schedules of the batch's FFT-pair and tensor-core passes on the
        live workload (states restored afterwards); returns the trial report."""
        import json
        buf = C.create_string_buffer(1 << 16)
        call("so_batch_tune", self._h, cache_path.encode() if cache_path else None, trial_steps, buf, 1 << 16)
        return json.loads(buf.value.decode())

    def steps_host_ptr(self, in_ptrs: Sequence[int], out_ptrs: Sequence[int], n: int):
        """States in from host addresses, n steps, states out to host addresses: one
        pipelined call (chunks of members overlap their copies and steps)."""
        a = (C.c_void_p * len(in_ptrs))(*in_ptrs)
        b = (C.c_void_p * len(out_ptrs))(*out_ptrs)
        call("so_batch_steps_host", self._h, C.cast(a, C.POINTER(C.c_void_p)), C.cast(b, C.POINTER(C.c_void_p)),
             len(in_ptrs), n)

    def set_arrays(self, arrays):
        arrs = [np.ascontiguousarray(a, dtype=np.complex128) for a in arrays]
        for a, p in zip(arrs, self._props):
            if a.shape != tuple(p.wave_function_shape()):
                raise ValueError("state shape differs from the propagation's grid")
        self.set_arrays_ptr([a.ctypes.data for a in arrs])

    def get_arrays(self):
        outs = [np.empty(tuple(p.wave_function_shape()), dtype=np.complex128) for p in self._props]
        self.get_arrays_ptr([o.ctypes.data for o in outs])
        return outs


def _fp(a):
    return a.ctypes.data_as(C.POINTER(C.c_float))


class Mlp(_Handle):
    """Multilayer perceptron trained by the library's CUDA kernels (tanh hidden layers)."""

    _free = "so_mlp_free"

    def __init__(self, widths: Sequence[int], seed: int = 0):
        w = (C.c_int * len(widths))(*widths)
        super().__init__(_new("so_mlp_new", w, len(widths), seed))
        self.widths = list(widths)

    def num_params(self) -> int:
        v = C.c_size_t()
        call("so_mlp_num_params", self._h, C.byref(v))
        return v.value

    def get_params(self):
        out = np.empty(self.num_params(), dtype=np.float32)
        call("so_mlp_get_params", self._h, _fp(out))
        return out

    def set_params(self, p):
        p = np.ascontiguousarray(p, dtype=np.float32)
        call("so_mlp_set_params", self._h, _fp(p))

    def forward(self, x):
        x = np.ascontiguousarray(x, dtype=np.float32)
        y = np.empty((x.shape[0], self.widths[-1]), dtype=np.float32)
        call("so_mlp_forward", self._h, _fp(x), x.shape[0], _fp(y))
        return y

    def gradients(self, x, t):
        x = np.ascontiguousarray(x, dtype=np.float32)
        t = np.ascontiguousarray(t, dtype=np.float32)
        g = np.empty(self.num_params(), dtype=np.float32)
        loss = C.c_double()
        call("so_mlp_gradients", self._h, _fp(x), _fp(t), x.shape[0], C.byref(loss), _fp(g))
        return loss.value, g

    def train(self, x, t, steps: int, lr: float = 1e-3):
        x = np.ascontiguousarray(x, dtype=np.float32)
        t = np.ascontiguousarray(t, dtype=np.float32)
        losses = np.empty(steps)
        call("so_mlp_train", self._h, _fp(x), _fp(t), x.shape[0], steps, lr, _dp(losses))
        return losses


def selftest_bounded_wait(limit_ns: int):
    """(try_wait form timed out, polling form timed out, elapsed ns) of a device wait on a
    barrier that nothing completes."""
    out = (C.c_uint64 * 3)()
    call("so_selftest_bounded_wait", limit_ns, out)
    return bool(out[0]), bool(out[1]), int(out[2])


def launch_count() -> int:
    v = C.c_uint64()
    call("so_launch_count", C.byref(v))
    return v.value


def load_schedules(path: str):
    """Launch schedules from a cache file the autotuner wrote (process-wide)."""
    call("so_schedules_load", path.encode())


def save_schedules(path: str):
    call("so_schedules_save", path.encode())


def reset_schedules():
    """Back to the built-in launch schedules."""
    call("so_schedules_reset")
