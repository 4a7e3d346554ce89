"""ctypes binding of the C ABI declared in include/split_operator.h.

The shared object is built in-tree (``split_operator_gb300/_build``) by
``split_operator_gb300.build``; importing this module without it raises
immediately: there is no fallback implementation.
"""
import ctypes as C
import os

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_build", "libsplit_operator_gb300.so")


class SplitOperatorError(RuntimeError):
    def __init__(self, status, message):
        super().__init__(f"[status {status}] {message}")
        self.status = status


class TimeGridC(C.Structure):
    _fields_ = [("step", C.c_double), ("step_no", C.c_uint64), ("im_time", C.c_int)]


_P = C.c_void_p
_PP = C.POINTER(C.c_void_p)
_D = C.c_double
_DP = C.POINTER(C.c_double)
_S = C.c_size_t
_SP = C.POINTER(C.c_size_t)
_I = C.c_int
_STR = C.c_char_p

# name -> argtypes (restype int unless listed in _VOID / _OTHER)
SIGNATURES = {
    "so_version": [],
    "so_launch_count": [C.POINTER(C.c_uint64)],
    "so_selftest_bounded_wait": [C.c_uint64, C.POINTER(C.c_uint64)],
    "so_grid_new_linear_continuos": [_STR, _D, _D, _S, _S, _PP],
    "so_grid_new_linear_countable": [_STR, _D, _D, _S, _S, _PP],
    "so_grid_new_custom": [_STR, _DP, _DP, _S, _S, _PP],
    "so_grid_nodes_no": [_P, _SP],
    "so_grid_dimension_no": [_P, _SP],
    "so_grid_name": [_P, C.c_char_p, _S],
    "so_grid_nodes": [_P, _DP],
    "so_grid_weights": [_P, _DP],
    "so_wave_function_new": [_DP, _SP, _S, _PP, _PP],
    "so_wave_function_clone": [_P, _PP],
    "so_wave_function_ndim": [_P, _SP, _SP],
    "so_wave_function_norm": [_P, _DP],
    "so_wave_function_dot": [_P, _P, _DP],
    "so_wave_function_normalize": [_P, _D],
    "so_wave_function_density": [_P, _DP],
    "so_wave_function_state_density": [_P, _S, _DP],
    "so_wave_function_get_array": [_P, _DP],
    "so_wave_function_set_array": [_P, _DP],
    "so_wave_function_grid": [_P, _S, _PP],
    "so_gaussian_distribution": [_DP, _S, _D, _D, _D, _DP],
    "so_one_dim_propagator_new": [_S, _S, _PP],
    "so_one_dim_propagator_set_operator": [_P, _DP, _S],
    "so_one_dim_propagator_add_operator": [_P, _DP, _S],
    "so_n_dim_propagator_new": [_PP],
    "so_n_dim_propagator_set_operator": [_P, _DP, _SP, _S],
    "so_n_dim_propagator_add_operator": [_P, _DP, _SP, _S],
    "so_non_diag_propagator_new": [_S, _PP],
    "so_non_diag_propagator_set_operators": [_P, _DP, _S, _S],
    "so_propagator_set_loss_checked": [_P, _STR],
    "so_propagator_apply": [_P, _P],
    "so_propagator_loss": [_P, _DP, C.POINTER(C.c_int)],
    "so_propagator_loss_reset": [_P],
    "so_one_dim_into_propagator": [_DP, _P, TimeGridC, _I, _PP],
    "so_n_dim_into_propagator": [_DP, _SP, _S, TimeGridC, _I, _PP],
    "so_complex_n_dim_into_propagator": [_DP, _SP, _S, TimeGridC, _I, _PP],
    "so_fft_transformation_new": [_P, _STR, _PP],
    "so_matrix_transformation_new": [_P, _P, _PP],
    "so_matrix_transformation_set_diagonalization_matrix": [_P, _DP, _DP, _S],
    "so_state_matrix_transformation_new": [_S, _P, _P, _PP],
    "so_state_matrix_transformation_set_diagonalization_matrices": [_P, _DP, _DP, _S, _S],
    "so_transformation_transform": [_P, _P],
    "so_transformation_inverse_transform": [_P, _P],
    "so_transformation_grid": [_P, _PP],
    "so_kinetic_hamiltonian": [_P, _D, _DP],
    "so_rotational_hamiltonian": [_P, _P, _D, _D, _DP],
    "so_two_dim_into_n_dim_operator": [_SP, _S, _DP, _P, _P, _DP],
    "so_legendre_diagonalization_operator": [_P, _PP],
    "so_associated_legendre_diagonalization_operator": [_P, _I, _PP],
    "so_associated_legendre_operator": [_P, _P, _PP],
    "so_legendre_polynomials": [_S, _D, _DP],
    "so_associated_legendre_polynomials": [_S, _I, _D, _DP],
    "so_gauss_legendre": [_S, _DP, _DP],
    "so_dispersion": [_DP, _S, _I, _D, _DP],
    "so_lennard_jones": [_DP, _S, _D, _D, _DP],
    "so_harmonic": [_DP, _S, _D, _D, _D, _DP],
    "so_morse": [_DP, _S, _D, _D, _D, _DP],
    "so_leak_control_new": [_PP],
    "so_leak_control_add_loss_checker": [_P, _STR],
    "so_dumping_end": [_D, _D, _P, _DP],
    "so_border_dumping_new": [_DP, _S, _P, _PP],
    "so_border_dumping_add_loss_checker": [_P, _STR],
    "so_control_first_half": [_P, _P],
    "so_control_second_half": [_P, _P],
    "so_control_loss": [_P, _DP, C.POINTER(C.c_int)],
    "so_state_saver_new": [_STR, TimeGridC, _P, _S, _PP],
    "so_wave_function_saver_new": [_STR, TimeGridC, _P, _P, _S, _PP],
    "so_saver_frames": [_P, _DP, _DP, _SP],
    "so_saver_shape": [_P, _SP, _SP],
    "so_saver_save": [_P],
    "so_saver_reset": [_P],
    "so_saver_monitor": [_P, _P],
    "so_operation_stack_new": [_PP],
    "so_operation_stack_add_propagator": [_P, _P],
    "so_operation_stack_add_transformation": [_P, _P, _I],
    "so_operation_stack_add_saver": [_P, _P, _I],
    "so_operation_stack_add_control": [_P, _P, _I],
    "so_operation_stack_len": [_P, _SP],
    "so_propagation_new": [_P, TimeGridC, _P, _I, _PP],
    "so_propagation_propagate": [_P],
    "so_propagation_steps": [_P, C.c_uint64],
    "so_propagation_mean_energy": [_P, _DP],
    "so_propagation_get_losses": [_P, _DP, _S, _SP],
    "so_propagation_all_losses": [_P, _DP, _S, _SP],
    "so_propagation_reset_losses": [_P],
    "so_propagation_reset_savers_state": [_P],
    "so_propagation_savers_save": [_P],
    "so_propagation_wave_function": [_P, _PP],
    "so_propagation_get_array": [_P, _DP],
    "so_propagation_set_array": [_P, _DP],
    "so_propagation_norm": [_P, _DP],
    "so_propagation_set_stream": [_P, _P],
    "so_propagation_synchronize": [_P],
    "so_propagation_describe": [_P, C.c_char_p, _S],
    "so_propagation_set_timing": [_P, _I],
    "so_propagation_kernel_times": [_P, C.c_char_p, _S],
    "so_batch_tune": [_P, _STR, _I, C.c_char_p, _S],
    "so_schedules_load": [_STR],
    "so_schedules_save": [_STR],
    "so_schedules_reset": [],
    "so_propagation_checkpoint": [_P, _P, _S, _SP],
    "so_propagation_restore": [_P, _P, _S],
    "so_propagation_steps_done": [_P, C.POINTER(C.c_uint64)],
    "so_fft_norm_noalloc": [_P, _S, _S, _I, _P, _P, _P, _P],
    "so_batch_new": [_PP, _S, _PP],
    "so_batch_steps": [_P, C.c_uint64],
    "so_batch_set_timing": [_P, _I],
    "so_batch_kernel_times": [_P, C.c_char_p, _S],
    "so_batch_launches_per_step": [_P, _SP],
    "so_batch_set_arrays": [_P, _PP, _S],
    "so_batch_get_arrays": [_P, _PP, _S],
    "so_batch_steps_host": [_P, _PP, _PP, _S, C.c_uint64],
    "so_mlp_new": [C.POINTER(C.c_int), _S, C.c_uint64, _PP],
    "so_mlp_num_params": [_P, _SP],
    "so_mlp_get_params": [_P, C.POINTER(C.c_float)],
    "so_mlp_set_params": [_P, C.POINTER(C.c_float)],
    "so_mlp_forward": [_P, C.POINTER(C.c_float), _S, C.POINTER(C.c_float)],
    "so_mlp_gradients": [_P, C.POINTER(C.c_float), C.POINTER(C.c_float), _S, _DP, C.POINTER(C.c_float)],
    "so_mlp_train": [_P, C.POINTER(C.c_float), C.POINTER(C.c_float), _S, _S, C.c_float, _DP],
}
VOID = {
    "so_grid_free": [_P],
    "so_wave_function_free": [_P],
    "so_operator_free": [_P],
    "so_operation_stack_free": [_P],
    "so_propagation_free": [_P],
    "so_batch_free": [_P],
    "so_mlp_free": [_P],
}
OTHER = {"so_last_error": ([], C.c_char_p)}

_lib = None


def lib():
    """Load (once) and return the library with every signature applied."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise ImportError(
            f"split_operator_gb300 native library not built: {LIB_PATH} is missing "
            "(run `python -m split_operator_gb300.build`)"
        )
    h = C.CDLL(LIB_PATH)
    for name, args in SIGNATURES.items():
        f = getattr(h, name)
        f.argtypes = args
        f.restype = C.c_int
    for name, args in VOID.items():
        f = getattr(h, name)
        f.argtypes = args
        f.restype = None
    for name, (args, res) in OTHER.items():
        f = getattr(h, name)
        f.argtypes = args
        f.restype = res
    _lib = h
    return h


def check(status):
    if status != 0:
        msg = lib().so_last_error().decode(errors="replace")
        raise SplitOperatorError(status, msg)
    return status


def call(name, *args):
    return check(getattr(lib(), name)(*args))
