/*
 * split_operator.h -- C ABI of the GB300 (sm_103a) split-operator propagation path.
 *
 * Each entry point replaces one item of the Rust crate split_operator
 * (Wleter/split_operator); the comment above it cites the reference file:line.
 * Conventions:
 *   - every function returns an so_status (0 = SO_OK); so_last_error() gives a
 *     message for the calling thread's last failure;
 *   - handles are opaque and reference counted: adding an operator to a stack or
 *     a stack to a propagation shares it, so_*_free drops the caller's reference;
 *   - complex arrays are interleaved float64 pairs (re, im) in row-major order of
 *     the reference's logical axes (ndarray's default layout);
 *   - the library owns all device memory; wave functions live in GPU memory;
 *   - a propagation issues all work on one CUDA stream (so_propagation_set_stream).
 * The reference reports misuse with assert!/panic!; here the same conditions
 * return SO_ERR_INVALID / SO_ERR_SHAPE and leave the objects unchanged.
 */
#ifndef SPLIT_OPERATOR_H
#define SPLIT_OPERATOR_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif
#if defined(__GNUC__)
#pragma GCC visibility push(default)
#endif

typedef enum {
  SO_OK = 0,
  SO_ERR_INVALID = 1,      /* bad argument or handle */
  SO_ERR_SHAPE = 2,        /* shape mismatch (reference: assert! on shapes) */
  SO_ERR_CUDA = 3,         /* CUDA runtime error or no device */
  SO_ERR_UNSUPPORTED = 4,  /* valid request outside what the kernels implement */
  SO_ERR_STATE = 5,        /* call not valid in the object's state (reference: panic!) */
  SO_ERR_NONFINITE = 6,    /* a norm became NaN or infinite */
  SO_ERR_TIMEOUT = 7,      /* a bounded device-side wait gave up */
  SO_ERR_IO = 8            /* saver could not write its files */
} so_status;

typedef struct so_grid_t* so_grid;
typedef struct so_wave_function_t* so_wave_function;
typedef struct so_operator_t* so_operator; /* propagator, transformation, control or saver */
typedef struct so_operation_stack_t* so_operation_stack;
typedef struct so_propagation_t* so_propagation;

/* time_grid.rs:7-11 */
typedef struct {
  double step;
  uint64_t step_no;
  int im_time;
} so_time_grid;

enum { SO_STEP_FULL = 0, SO_STEP_HALF = 1 };                      /* time_grid.rs:15-18 */
enum { SO_ORDER_NORMAL = 0, SO_ORDER_INVERSE_FIRST = 1 };         /* transformation.rs:13-16 */
enum { SO_APPLY_NONE = 0, SO_APPLY_FIRST_HALF = 1, SO_APPLY_SECOND_HALF = 2 }; /* control.rs:19-26 */

/* Arithmetic of a propagation (no reference counterpart: the reference is FP64 only). */
enum {
  SO_PRECISION_FP64 = 0,        /* FP64 state, tables and transforms */
  SO_PRECISION_FP32_TF32X3 = 1, /* FP32 state; real lane matrices as 3xTF32 tensor-core GEMM */
  SO_PRECISION_FP32_BF16X3 = 2, /* FP32 state; real lane matrices as split-BF16x3 tensor-core GEMM */
  SO_PRECISION_FP32_SIMT = 3,   /* FP32 state; lane matrices on FP32 CUDA cores */
  SO_PRECISION_FP32_BF16X6 = 4, /* FP32 state; real lane matrices as split-BF16x6 tensor-core GEMM:
                                   three fixed-point bf16 slices per operand, exact FP32 sums */
  SO_PRECISION_FLOAT_FLOAT = 5  /* float-float state and tables (each real an unevaluated sum of two
                                   FP32 numbers, ~48 significand bits); the FP64 path's kernels
                                   with float-float arithmetic on the FP32 pipes */
};

/* ---- library ------------------------------------------------------------ */
const char* so_last_error(void);
int so_version(void);
/* Kernels this library has launched since load (all devices, all handles). */
int so_launch_count(uint64_t* out);
/* Failure-detection self-test (no reference counterpart): one CTA waits on a tensor-core
 * pipeline barrier that nothing completes, with the kernel's two bounded wait forms and a
 * limit of limit_ns each.  out[0], out[1]: 1 if the wait gave up as intended; out[2]: the
 * elapsed device time in ns.  The context stays usable afterwards. */
int so_selftest_bounded_wait(uint64_t limit_ns, uint64_t* out);

/* ---- Grid: grid.rs:14-89 ------------------------------------------------ */
/* grid.rs:24-48 */
int so_grid_new_linear_continuos(const char* name, double start, double end, size_t nodes_no,
                                 size_t dimension_no, so_grid* out);
/* grid.rs:51-73 */
int so_grid_new_linear_countable(const char* name, double start, double end, size_t nodes_no,
                                 size_t dimension_no, so_grid* out);
/* grid.rs:76-84 */
int so_grid_new_custom(const char* name, const double* nodes, const double* weights, size_t nodes_no,
                       size_t dimension_no, so_grid* out);
int so_grid_nodes_no(so_grid g, size_t* out);
int so_grid_dimension_no(so_grid g, size_t* out);
int so_grid_name(so_grid g, char* buf, size_t cap);
int so_grid_nodes(so_grid g, double* out);
int so_grid_weights(so_grid g, double* out);
void so_grid_free(so_grid g);

/* ---- WaveFunction: wave_function.rs:11-149 ------------------------------- */
/* wave_function.rs:23-47 (the array is copied to GPU memory; grids are copied) */
int so_wave_function_new(const double* array, const size_t* shape, size_t ndim, const so_grid* grids,
                         so_wave_function* out);
int so_wave_function_clone(so_wave_function wf, so_wave_function* out);
int so_wave_function_ndim(so_wave_function wf, size_t* ndim, size_t* shape /* cap 8 */);
/* wave_function.rs:68-85 (cached unless an operator marked it dirty) */
int so_wave_function_norm(so_wave_function wf, double* out);
/* wave_function.rs:87-101: out = {re, im} of <a|b> / sqrt(|a| |b|) */
int so_wave_function_dot(so_wave_function a, so_wave_function b, double* out);
/* wave_function.rs:104-109 */
int so_wave_function_normalize(so_wave_function wf, double new_norm);
/* wave_function.rs:112-118 */
int so_wave_function_density(so_wave_function wf, double* out);
/* wave_function.rs:121-148 */
int so_wave_function_state_density(so_wave_function wf, size_t axis, double* out);
/* `array` field read / write (pub in the reference: wave_function.rs:12) */
int so_wave_function_get_array(so_wave_function wf, double* out);
int so_wave_function_set_array(so_wave_function wf, const double* in);
/* `grids` field (pub: wave_function.rs:13): copy of the grid now on `axis` */
int so_wave_function_grid(so_wave_function wf, size_t axis, so_grid* out);
void so_wave_function_free(so_wave_function wf);
/* wave_function.rs:152-154 (host helper: out[i] = gaussian at x[i], complex) */
int so_gaussian_distribution(const double* x, size_t n, double x0, double sigma, double momentum, double* out);

/* ---- Propagators: propagator.rs:12-18 ------------------------------------ */
/* one_dim_propagator.rs:16-35 */
int so_one_dim_propagator_new(size_t shape, size_t dimension_no, so_operator* out);
int so_one_dim_propagator_set_operator(so_operator p, const double* op, size_t n);
int so_one_dim_propagator_add_operator(so_operator p, const double* op, size_t n);
/* n_dim_propagator.rs:14-30 */
int so_n_dim_propagator_new(so_operator* out);
int so_n_dim_propagator_set_operator(so_operator p, const double* op, const size_t* shape, size_t ndim);
int so_n_dim_propagator_add_operator(so_operator p, const double* op, const size_t* shape, size_t ndim);
/* non_diagonal_propagator.rs:16-27: `count` matrices n x n (complex), lane i uses matrix i */
int so_non_diag_propagator_new(size_t dimension_no, so_operator* out);
int so_non_diag_propagator_set_operators(so_operator p, const double* ops, size_t count, size_t n);
/* set_loss_checked(LossChecker::new(name)): one_dim_propagator.rs:48-50, n_dim_propagator.rs:38-40 */
int so_propagator_set_loss_checked(so_operator p, const char* name);
/* Propagator::apply (propagator.rs:13) on a stand-alone wave function */
int so_propagator_apply(so_operator p, so_wave_function wf);
/* Propagator::loss (propagator.rs:15): *has = 0 when no loss checker is attached */
int so_propagator_loss(so_operator p, double* out, int* has);
int so_propagator_loss_reset(so_operator p);

/* propagator_factory.rs:10-22 */
int so_one_dim_into_propagator(const double* hamiltonian, so_grid grid, so_time_grid time, int step,
                               so_operator* out);
/* propagator_factory.rs:25-36 */
int so_n_dim_into_propagator(const double* hamiltonian, const size_t* shape, size_t ndim, so_time_grid time,
                             int step, so_operator* out);
/* propagator_factory.rs:39-50 (complex hamiltonian) */
int so_complex_n_dim_into_propagator(const double* hamiltonian, const size_t* shape, size_t ndim,
                                     so_time_grid time, int step, so_operator* out);

/* ---- Transformations: transformation.rs:5-11 ----------------------------- */
/* fft_transformation.rs:24-48 */
int so_fft_transformation_new(so_grid grid, const char* transformed_grid_name, so_operator* out);
/* matrix_transformation.rs:19-51 */
int so_matrix_transformation_new(so_grid grid, so_grid grid_transformation, so_operator* out);
int so_matrix_transformation_set_diagonalization_matrix(so_operator t, const double* transformation,
                                                        const double* inverse_transformation, size_t n);
/* state_matrix_transformation.rs:19-45: `count` (matrix, inverse) pairs, n x n complex */
int so_state_matrix_transformation_new(size_t dimension_no_dependent, so_grid grid, so_grid grid_transformation,
                                       so_operator* out);
int so_state_matrix_transformation_set_diagonalization_matrices(so_operator t, const double* transformations,
                                                                const double* inverses, size_t count, size_t n);
/* Transformation::transform / inverse_transform on a stand-alone wave function */
int so_transformation_transform(so_operator t, so_wave_function wf);
int so_transformation_inverse_transform(so_operator t, so_wave_function wf);
/* `grid_transformation` (pub field): copy of the grid the transformation holds now */
int so_transformation_grid(so_operator t, so_grid* out);

/* ---- Hamiltonian factory ------------------------------------------------- */
/* kinetic_operator.rs:8-21 (the reduced mass is passed directly) */
int so_kinetic_hamiltonian(so_grid grid, double red_mass, double* out);
/* rotational_operator.rs:7-26: out is (radial, polar) row-major */
int so_rotational_hamiltonian(so_grid radial, so_grid polar, double red_mass, double rotational_const,
                              double* out);
/* hamiltonian_broadcasting.rs:6-23: broadcast a (grid1, grid2) table into `shape` */
int so_two_dim_into_n_dim_operator(const size_t* shape, size_t ndim, const double* hamiltonian, so_grid grid1,
                                   so_grid grid2, double* out);
/* legendre_diagonalization.rs:13-45 */
int so_legendre_diagonalization_operator(so_grid polar_grid, so_operator* out);
/* legendre_diagonalization.rs:48-80 */
int so_associated_legendre_diagonalization_operator(so_grid polar_grid, int omega, so_operator* out);
/* legendre_diagonalization.rs:83-109 */
int so_associated_legendre_operator(so_grid polar_grid, so_grid omega_grid, so_operator* out);
/* special_functions.rs:3-14 (j >= 1) */
int so_legendre_polynomials(size_t j, double x, double* out);
/* special_functions.rs:17-41 */
int so_associated_legendre_polynomials(size_t j, int m, double x, double* out);
/* Gauss-Legendre nodes (ascending, on [-1, 1]) and weights: the reference expects the user to
 * supply them through Grid::new_custom (no generator in the crate). */
int so_gauss_legendre(size_t n, double* nodes, double* weights);
/* analytic_potentials.rs:2-10, :13-22, :24-32 (NaN -> +inf), plus a Morse term */
int so_dispersion(const double* r, size_t n, int power, double cn, double* out);
int so_lennard_jones(const double* r, size_t n, double d6, double r6, double* out);
int so_harmonic(const double* r, size_t n, double r0, double mass, double omega, double* out);
int so_morse(const double* r, size_t n, double d, double a, double re, double* out);

/* ---- Controls: control.rs:6-17 ------------------------------------------- */
/* leak_control.rs:13-24 */
int so_leak_control_new(so_operator* out);
int so_leak_control_add_loss_checker(so_operator c, const char* name);
/* border_dumping.rs:14-33 (complex mask) */
int so_dumping_end(double mask_width, double mask_end, so_grid grid, double* out);
/* border_dumping.rs:42-55 */
int so_border_dumping_new(const double* mask, size_t n, so_grid grid, so_operator* out);
int so_border_dumping_add_loss_checker(so_operator c, const char* name);
/* Control::first_half / second_half on a stand-alone wave function */
int so_control_first_half(so_operator c, so_wave_function wf);
int so_control_second_half(so_operator c, so_wave_function wf);
/* Control::loss (control.rs:15) */
int so_control_loss(so_operator c, double* out, int* has);

/* ---- Savers: saver.rs:5-14 ----------------------------------------------- */
/* wave_function_saver.rs:112-131 */
int so_state_saver_new(const char* name, so_time_grid time, so_grid state_grid, size_t frames_no,
                       so_operator* out);
/* wave_function_saver.rs:20-41 */
int so_wave_function_saver_new(const char* name, so_time_grid time, so_grid x_grid, so_grid y_grid,
                               size_t frames_no, so_operator* out);
/* frames taken so far: data is (points, frames_no) row-major as in the reference; times[frames] */
int so_saver_frames(so_operator s, double* data, double* times, size_t* frames_taken);
int so_saver_shape(so_operator s, size_t* points, size_t* frames_no);
/* Saver::save (writes <name>.npy and companions in the working directory) */
int so_saver_save(so_operator s);
int so_saver_reset(so_operator s);
/* Saver::monitor on a stand-alone wave function */
int so_saver_monitor(so_operator s, so_wave_function wf);

void so_operator_free(so_operator op);

/* ---- OperationStack: propagation.rs:26-65 -------------------------------- */
int so_operation_stack_new(so_operation_stack* out);
int so_operation_stack_add_propagator(so_operation_stack s, so_operator p);
int so_operation_stack_add_transformation(so_operation_stack s, so_operator t, int order);
int so_operation_stack_add_saver(so_operation_stack s, so_operator saver, int apply);
int so_operation_stack_add_control(so_operation_stack s, so_operator c, int apply);
int so_operation_stack_len(so_operation_stack s, size_t* out);
void so_operation_stack_free(so_operation_stack s);

/* ---- Propagation: propagation.rs:72-292 ---------------------------------- */
/* propagation.rs:82-88; the wave function is copied in; `precision` is an SO_PRECISION_* value */
int so_propagation_new(so_wave_function wf, so_time_grid time, so_operation_stack stack, int precision,
                       so_propagation* out);
/* propagation.rs:185-190: time.step_no steps (the per-step println is not reproduced) */
int so_propagation_propagate(so_propagation p);
/* `steps` steps of Propagation::step (propagation.rs:134-182) */
int so_propagation_steps(so_propagation p, uint64_t steps);
/* propagation.rs:245-291 */
int so_propagation_mean_energy(so_propagation p, double* out);
/* propagation.rs:213-231: losses of loss-checked propagators, in stack order */
int so_propagation_get_losses(so_propagation p, double* out, size_t cap, size_t* count);
/* losses of propagators and controls in stack order (what print_losses prints, :193-210) */
int so_propagation_all_losses(so_propagation p, double* out, size_t cap, size_t* count);
int so_propagation_reset_losses(so_propagation p);       /* propagation.rs:125-131 */
int so_propagation_reset_savers_state(so_propagation p); /* propagation.rs:116-122 */
int so_propagation_savers_save(so_propagation p);        /* propagation.rs:234-243 */
/* wave_function() (propagation.rs:111-113): a stand-alone FP64 copy of the current state */
int so_propagation_wave_function(so_propagation p, so_wave_function* out);
/* host copy of the current array (logical row-major, complex128) and its replacement.
 * get returns once `out` is written.  A page-locked `in` is read on the propagation's
 * stream after set returns (the layout kernel reads it directly): keep it unchanged until
 * a later call that waits on the stream (get_array, norm, steps).  Pageable `in` is copied
 * before set returns. */
int so_propagation_get_array(so_propagation p, double* out);
int so_propagation_set_array(so_propagation p, const double* in);
/* norm of the current state with the current representation's weights */
int so_propagation_norm(so_propagation p, double* out);
/* CUDA stream (cudaStream_t) all later work of `p` is issued on; NULL = legacy default stream */
int so_propagation_set_stream(so_propagation p, void* stream);
int so_propagation_synchronize(so_propagation p);
/* Human-readable description of the fused device passes of one step (for tests and profiling). */
int so_propagation_describe(so_propagation p, char* buf, size_t cap);
/* Per-pass device timing (no reference counterpart): when enabled, every pass launch is
 * bracketed by CUDA events on the propagation's stream.  so_propagation_kernel_times
 * synchronizes, writes one line per pass kind "name<TAB>launches<TAB>total_ms<TAB>algorithmic_bytes"
 * and clears the record. */
int so_propagation_set_timing(so_propagation p, int enabled);
int so_propagation_kernel_times(so_propagation p, char* buf, size_t cap);
/* Checkpoint / resume (no counterpart in the reference, whose savers keep frames only).
 * A checkpoint holds everything the next steps read: the state (exactly, in the
 * propagation's storage precision), the norm cache, every loss checker's loss and last
 * norm, the leak-control norm, the savers' frames and the step count; the fields the
 * reference steps are loss_checker.rs:49-68, leak_control.rs:31-45 and the savers of
 * wave_function_saver.rs:42-64.  so_propagation_checkpoint with buf == NULL only reports
 * the size; a cap below the size is SO_ERR_INVALID.  so_propagation_restore accepts a
 * checkpoint of a propagation with the same shape, precision and operator stack (any
 * propagation built the same way, in this process or another) and continues exactly as
 * the propagation that took it would have: bit for bit. */
int so_propagation_checkpoint(so_propagation p, void* buf, size_t cap, size_t* size);
int so_propagation_restore(so_propagation p, const void* buf, size_t size);
/* steps of Propagation::step taken since creation (restore sets the checkpoint's count) */
int so_propagation_steps_done(so_propagation p, uint64_t* out);
void so_propagation_free(so_propagation p);

/* ---- Batched propagation (no counterpart in the reference, which runs one
 * Propagation at a time) ----
 * Steps many independent propagations together: each pass of the steady-state step
 * becomes one launch per kernel / shape class covering every instance's tiles, and
 * the repeated part is replayed from a captured CUDA graph.  The propagations keep
 * their own state (so_propagation_get_array, losses, norms stay valid) and must share
 * the step's pass structure (same operator stack kinds); savers are not allowed.
 * Work is issued on the first propagation's stream.  The batch shares its members: a
 * propagation freed by the caller first stays alive until so_batch_free. */
typedef struct so_batch_t* so_batch;
int so_batch_new(const so_propagation* props, size_t count, so_batch* out);
/* `steps` steps of every propagation (Propagation::step, propagation.rs:134-182) */
int so_batch_steps(so_batch b, uint64_t steps);
int so_batch_set_timing(so_batch b, int enabled);
int so_batch_kernel_times(so_batch b, char* buf, size_t cap);
/* launches of the repeated part of one step (after the first) */
int so_batch_launches_per_step(so_batch b, size_t* out);
/* Every member's state from / to host arrays (count == the batch size; array i is the
 * logical row-major complex128 state of propagation i, as so_propagation_set_array /
 * so_propagation_get_array).  Page-locked host arrays are read and written by the
 * layout kernels directly; get queues every export and waits once. */
int so_batch_set_arrays(so_batch b, const double* const* in, size_t count);
int so_batch_get_arrays(so_batch b, double* const* out, size_t count);
/* so_batch_set_arrays(in), so_batch_steps(steps), so_batch_get_arrays(out) as one call,
 * pipelined: the members are split into chunks (16 by default; SO_HOST_CHUNKS: 1..64, read
 * at the batch's first such call) on streams of their own, each
 * copied in (copy engines), stepped and copied out, so the host link's two directions
 * and the chunks' steps overlap.  `in` and `out` may be the same arrays.  A chunk whose
 * members' arrays lie back to back in one allocation (in member order) moves with one copy
 * per direction. */
int so_batch_steps_host(so_batch b, const double* const* in, double* const* out, size_t count, uint64_t steps);
/* Autotuner (no counterpart in the reference, whose lane loops over rayon --
 * fft_transformation.rs:59-68, matrix_transformation.rs:64-65 -- have no launch shape to pick).
 * For every lane extent of the batch's passes it times candidate launch schedules on the live
 * workload with CUDA events, `trial_steps` steps each: FFT-pair pass threads per CTA (lanes per
 * tile) and Stockham radix; tensor-core pass CTAs per SM and tile order.  The fastest per extent
 * goes into the process-wide schedule table that every later pass launch reads; the table is
 * written to `cache_path` as JSON (NULL: no file).  Every member's state, losses and step count
 * are restored afterwards.  `report` (may be NULL) receives a JSON report of the trials. */
int so_batch_tune(so_batch b, const char* cache_path, int trial_steps, char* report, size_t cap);
void so_batch_free(so_batch b);

/* The process-wide launch schedule table (read by every pass launch): load a cache file the
 * tuner wrote, save the current table, or return to the built-in defaults. */
int so_schedules_load(const char* path);
int so_schedules_save(const char* path);
int so_schedules_reset(void);

/* ---- Learned starting states (no counterpart in the reference) ----
 * A multilayer perceptron (tanh hidden layers, linear output) trained with hand-written
 * CUDA kernels: BF16 weights in the forward and backward products, FP32 accumulation,
 * FP32 master weights updated by Adam.  Used to predict the starting wave function of
 * imaginary-time relaxation from the potential parameters.  Host arrays are FP32. */
typedef struct so_mlp_t* so_mlp;
int so_mlp_new(const int* widths, size_t count, uint64_t seed, so_mlp* out);
int so_mlp_num_params(so_mlp m, size_t* out);
/* parameters layer by layer: W (out x in, row-major) then b */
int so_mlp_get_params(so_mlp m, float* out);
int so_mlp_set_params(so_mlp m, const float* in);
int so_mlp_forward(so_mlp m, const float* x, size_t batch, float* y);
/* mean squared error of forward(x) against target and its gradient (parameter order above) */
int so_mlp_gradients(so_mlp m, const float* x, const float* target, size_t batch, double* loss, float* grads);
/* `steps` full-batch Adam steps; losses[i] (may be NULL) = loss before step i */
int so_mlp_train(so_mlp m, const float* x, const float* target, size_t batch, size_t steps, float lr,
                 double* losses);
void so_mlp_free(so_mlp m);

/* ---- Allocation-free lane FFT + norm (no counterpart in the reference) ----
 * For callers that must not allocate GPU memory, or let a library allocate it, while
 * they run: code inside a strict device memory pool, or a host framework that hands
 * over only pre-sized buffers.  Every pointer is the caller's device memory.
 * In place on psi (complex128, `lanes` contiguous lanes of `n` points, row-major):
 * every lane becomes its unitary discrete Fourier transform,
 *   psi'[l][k] = n^(-1/2) sum_x psi[l][x] exp(direction * 2 pi i x k / n)
 * (direction -1 forward, +1 inverse); then, when `weights` is given,
 *   *norm_out = sum_{l,x} |psi'[l][x]|^2 lane_weights[l] weights[x].
 * `lane_weights`, `weights` and `norm_out` are all given or all NULL.  Issued on
 * `stream` (cudaStream_t; NULL = legacy stream).
 * Limits: n <= 4096 and at most 65536 CTAs of lanes (SO_ERR_UNSUPPORTED beyond).
 * The kernel's scratch (norm partials, a ticket counter) and the twiddle table are
 * fixed file-scope device arrays (about 0.6 MiB, held by every GPU that loads the
 * library until exit); no cudaMalloc / cudaFree is called.  The first call on a
 * device looks up those arrays' device addresses: make it before any stream
 * capture.  All calls share the arrays, which keep the last call's contents (every
 * call rebuilds the twiddle table and clears the counter itself): calls that overlap
 * on the GPU (other streams, other threads) race. */
int so_fft_norm_noalloc(double* psi, size_t lanes, size_t n, int direction, const double* lane_weights,
                        const double* weights, double* norm_out, void* stream);

#if defined(__GNUC__)
#pragma GCC visibility pop
#endif
#ifdef __cplusplus
}
#endif
#endif /* SPLIT_OPERATOR_H */
