// Host-side model of the split-operator API (C++), mirroring the Rust crate's
// types: Grid, WaveFunction (+ ChangeObserver norm cache), the propagators,
// transformations, controls, savers, LossChecker, OperationStack and
// Propagation.  The objects hold FP64 host tables; the arrays they act on live
// in GPU memory inside an Engine, which turns the stream of actions the host
// logic emits into fused lane-sweep passes.
#pragma once
#include <complex>
#include <functional>
#include <map>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#include "../../include/split_operator.h"
#include "common.cuh"

namespace so {

using cplx = std::complex<double>;

struct Error : std::runtime_error {
  int status;
  Error(int s, const std::string& m) : std::runtime_error(m), status(s) {}
};

void cuda_check(cudaError_t e, const char* what);

// ------------------------------------------------------------------ grid.rs
struct Grid {
  std::string name;
  size_t dimension_no = 0;
  std::vector<double> nodes, weights;
  uint64_t uid = 0;  // identifies the weight vector on the device
  static uint64_t next_uid();
  static Grid linear_continuos(const std::string&, double, double, size_t, size_t);
  static Grid linear_countable(const std::string&, double, double, size_t, size_t);
  static Grid custom(const std::string&, std::vector<double>, std::vector<double>, size_t);
  size_t size() const { return nodes.size(); }
};

// factory.cpp
std::vector<double> momenta_fft_order(const Grid& g);
Grid fft_momentum_grid(const Grid& g, const std::string& name);
std::vector<double> kinetic_hamiltonian(const Grid& g, double red_mass);
std::vector<double> rotational_hamiltonian(const Grid& radial, const Grid& polar, double red_mass, double b);
std::vector<double> legendre_polynomials(size_t j, double x);
std::vector<double> associated_legendre_polynomials(size_t j, int64_t m, double x);
void legendre_matrices(const Grid& polar, int64_t omega, std::vector<cplx>& t, std::vector<cplx>& tinv);
void gauss_legendre(size_t n, std::vector<double>& x, std::vector<double>& w);
std::vector<cplx> twiddles(size_t n);
double pot_dispersion(double r, int n, double cn);
double pot_lennard_jones(double r, double d6, double r6);
double pot_harmonic(double r, double r0, double mass, double omega);
double pot_morse(double r, double d, double a, double re);
cplx gaussian(double x, double x0, double sigma, double p);
std::vector<cplx> dumping_end(double width, double end, const Grid& g);
cplx select_step(int step, const so_time_grid& t);
std::vector<cplx> phase_table(const double* h, size_t n, cplx dt);
std::vector<cplx> phase_table_complex(const cplx* h, size_t n, cplx dt);

// ------------------------------------------------------------ device memory
struct DeviceBuffer {
  void* ptr = nullptr;
  size_t bytes = 0;
  DeviceBuffer() = default;
  explicit DeviceBuffer(size_t b);
  DeviceBuffer(const DeviceBuffer&) = delete;
  DeviceBuffer& operator=(const DeviceBuffer&) = delete;
  DeviceBuffer(DeviceBuffer&& o) noexcept : ptr(o.ptr), bytes(o.bytes) { o.ptr = nullptr; o.bytes = 0; }
  DeviceBuffer& operator=(DeviceBuffer&& o) noexcept;
  ~DeviceBuffer();
  template <typename T>
  T* as() const { return reinterpret_cast<T*>(ptr); }
};

class Engine;

// Scalars of an operator (loss, current norm, leak norm) that live in device
// slots while an engine uses them, and on the host otherwise.
struct ScalarState {
  std::vector<double> host;
  Engine* home = nullptr;
  std::vector<int> slots;
  explicit ScalarState(size_t n = 0) : host(n, 0.0) {}
  ScalarState(const ScalarState&) = delete;
  ~ScalarState();
  const std::vector<int>& bind(Engine* e);
  void unbind();  // copies device values back to `host`
  double get(size_t i);
  void set(size_t i, double v);
};

// One emitted unit of work: a device op (with the lane axis it needs, -1 for
// point-wise and scalar ops) or a host callback (saver frames).
struct Action {
  DevOp op{};
  int lane_axis = -1;
  int host_call = -1;
};

// A pass captured instead of launched (batched execution of many propagations).
struct RecordedPass {
  enum Kind { Generic, TensorCore, Scalar, Resident } kind;
  int real;  // state precision (kRealF32, kRealF64, kRealFF)
  PassParams p;
  std::vector<unsigned char> tcp;  // TcParams bytes (TensorCore)
  int threads;
  size_t smem;
  std::string name;
  double bytes;
};

class Engine {
 public:
  // real: the state precision, kRealF32, kRealF64 or kRealFF (float-float)
  Engine(const std::vector<size_t>& shape, const std::vector<int>& perm, int real);
  ~Engine();

  int real;
  bool fp64;  // 16-byte complex values (FP64 or float-float): the FP64 kernels' shapes
  std::vector<size_t> shape;  // logical
  std::vector<int> perm;      // storage position -> logical axis
  DeviceBuffer psi;
  cudaStream_t stream = nullptr;
  int nonfinite_slot = 0;
  int timeout_slot = 0;
  // real lane matrices on the tensor cores (FP32 state only): 3xTF32, split-BF16x3 or
  // split-BF16x6 (exact tensor-core sums)
  bool tc_tf32 = false;
  bool tc_bf16 = false;
  bool tc_bf16x6 = false;
  // operand mode of the tensor-core pass (0 3xTF32, 1 split-BF16x3, 2 split-BF16x6), -1: none
  int tc_mode() const { return tc_tf32 ? 0 : (tc_bf16 ? 1 : (tc_bf16x6 ? 2 : -1)); }
  bool fft_pair = true;  // FP32 FFT-pair passes run the fused register kernel (SO_FFT_PAIR=0: the general pass)
  bool fft_pair_ct = true;  // ... its fixed-shape form where it applies (SO_FFT_PAIR_CT=0: the general shape)

  size_t points() const;
  size_t elem_bytes() const { return fp64 ? 16 : 8; }
  Geometry geometry(int sweep_axis, bool resident) const;
  bool resident_capable() const;

  // scalar slots
  int alloc_slot(double init);
  void free_slot(int s);
  void write_slot(int s, double v);
  double read_slot(int s);  // synchronizes
  double* slots() const { return slots_.as<double>(); }

  // device copies of host tables (state precision), cached by key
  const void* table_1d(const void* key, uint64_t version, const std::vector<cplx>& t);
  const void* table_nd(const void* key, uint64_t version, const std::vector<cplx>& t);
  // parity (optional): float-float single real matrices with the parity structure of a
  // Legendre pair get 1 or 2 (the kind) and the returned pointer is then the half matrix
  const void* matrices(const void* key, uint64_t version, const std::vector<cplx>& m, size_t n, size_t count,
                       bool& real, int* parity = nullptr);
  const double* weights(const Grid& g);
  const void* twiddle(size_t n, int radix = 0);  // radix 0: the precision's default stage order

  // pass building
  void submit(const Action& a);
  void flush();
  void run_resident(const std::vector<Action>& prog, int repeat);
  void sync();
  // logical complex128 -> storage; copy_engine: staged cudaMemcpyAsync even for page-locked
  // memory (no SMs busy on the host link, so the copy overlaps kernels of other streams)
  void import_host(const double* host, bool copy_engine = false);
  // import_host / export_host split at the staging buffer: copy engine and SM halves
  void stage_in(const double* host);
  void unstage_in();
  void stage_out();
  void unstage_out(double* host);
  // the layout halves alone, from / to a logical complex128 array already in device memory
  void import_device(const double* dev);
  void export_device(double* dev);
  void export_host(double* host, bool sync = true, bool copy_engine = false);  // storage -> logical complex128
  void check_nonfinite();

  std::vector<ScalarState*> bound;
  double* record_dev = nullptr;

  // When set, passes are appended here instead of being launched.
  std::vector<RecordedPass>* recording = nullptr;

  // Per-pass device timing with CUDA events on the engine stream.
  bool timing = false;
  void timed_begin(const std::string& name);
  void timed_end();
  std::string collect_timing();  // "name\tlaunches\ttotal_ms\tbytes\n" lines; synchronizes and resets

 private:
  void launch(const std::vector<DevOp>& ops, int axis, bool resident, int repeat);
  struct TimedLaunch {
    std::string name;
    cudaEvent_t a, b;
    double bytes;
  };
  std::vector<TimedLaunch> timed_;
  std::vector<cudaEvent_t> event_pool_;
  cudaEvent_t take_event();
  double pass_bytes(const std::vector<DevOp>& ops, const Geometry& g) const;
  DeviceBuffer slots_, partials_, counter_, staging_;
  size_t partials_cap_ = 0;
  std::vector<int> free_slots_;
  int next_slot_ = 1;
  struct Cached {
    uint64_t version;
    DeviceBuffer buf;
    bool real;
    int parity = 0;     // float-float: kind of the parity structure, half matrix in half_buf
    DeviceBuffer half_buf;
    // A-operand chunk images of the tensor-core passes, and the same for the parity-split
    // form (when the matrix has it): shared by every engine of the process whose matrix has
    // the same values (all propagations on one polar grid), so one copy stays hot in L2
    std::shared_ptr<DeviceBuffer> tc_images, tc_par_images;
    std::shared_ptr<DeviceBuffer> tc_pack_images;  // block-diagonal 128 x 128 form (packed tiles of n < 128)
    DeviceBuffer tc_slice_images;                  // state matrices: every matrix's images, one after another
  };
  std::map<std::pair<const void*, int>, Cached> tables_;
  std::map<const void*, const float*> tc_images_by_matrix_;
  std::map<const void*, const float*> tc_pack_by_matrix_;
  std::map<const void*, std::pair<int, const float*>> tc_parity_by_matrix_;  // parity kind, split images
  std::map<const void*, std::pair<const float*, int64_t>> tc_slice_by_matrix_;  // images, floats per matrix
  bool try_launch_tc(const std::vector<DevOp>& ops, int axis, PassParams& p);
  static void shared_tc_images(const std::vector<double>& md, int n, int mode, cudaStream_t s,
                               std::shared_ptr<DeviceBuffer>& img, std::shared_ptr<DeviceBuffer>& par, int& kind);
  std::map<uint64_t, DeviceBuffer> weights_;
  std::map<std::pair<size_t, int>, DeviceBuffer> twiddles_;  // by (n, stage radix)
  // open pass
  std::vector<DevOp> cur_;
  int cur_axis_ = -1;
  int cur_red_ = 0;
  std::vector<int> cur_written_;
};

// ------------------------------------------------------------ wave function
struct WaveFunction {
  std::vector<size_t> shape;
  std::vector<Grid> grids;
  std::vector<std::string> last_grid_names;  // change_observer.rs:8
  bool possible_norm_change = true;          // change_observer.rs:11
  std::unique_ptr<Engine> eng;
  int cache_slot = -1;  // change_observer.rs:10 (last_norm), on the device

  WaveFunction(const std::vector<size_t>& shape, const std::vector<Grid>& grids, const std::vector<int>& perm,
               int real);
  std::vector<const double*> weight_ptrs();
  void set_weights(DevOp& op);  // op.w / op.wf: FP64 and FP32 weights per logical axis
  size_t points() const;
};

// Where the host logic sends its actions: straight to the engine, or recorded.
struct Emitter {
  Engine* eng;
  std::vector<Action>* rec = nullptr;
  std::vector<std::function<void()>>* calls = nullptr;
  void emit(const Action& a) {
    if (rec)
      rec->push_back(a);
    else
      eng->submit(a);
  }
  void host(std::function<void()> f);
};

// wave_function.rs:68-85 on the host side: returns the slot holding the norm,
// emitting a norm reduction only when the cache is dirty.
int norm_slot(WaveFunction& wf, Emitter& em);
void normalize_to_slot(WaveFunction& wf, Emitter& em, int target_slot);

// ------------------------------------------------------------ operators
struct LossChecker {  // loss_checker.rs:7-69 (LossSaver not reproduced)
  std::string name;
  ScalarState st{2};  // 0: loss, 1: current_norm
  explicit LossChecker(const std::string& n) : name(n) { st.host[1] = 1.0; }
  void check_before(WaveFunction& wf, Emitter& em);
  void check_after(WaveFunction& wf, Emitter& em);
  void reset(Emitter* em);
  double loss() { return st.get(0); }
};

enum class OpClass { Propagator, Transformation, Control, Saver };

struct Operator {
  OpClass cls;
  std::string type;
  uint64_t version = 1;
  explicit Operator(OpClass c, const std::string& t) : cls(c), type(t) {}
  virtual ~Operator() = default;
  // Propagator
  virtual void apply(WaveFunction&, Emitter&) { throw Error(SO_ERR_INVALID, "not a propagator"); }
  virtual LossChecker* loss_checker() { return nullptr; }
  // Transformation
  virtual void transform(WaveFunction&, Emitter&) { throw Error(SO_ERR_INVALID, "not a transformation"); }
  virtual void inverse_transform(WaveFunction&, Emitter&) { throw Error(SO_ERR_INVALID, "not a transformation"); }
  virtual Grid* grid_transformation() { return nullptr; }
  // Control
  virtual std::string name() const { return type; }
  virtual void first_half(WaveFunction&, Emitter&) { throw Error(SO_ERR_INVALID, "not a control"); }
  virtual void second_half(WaveFunction&, Emitter&) { throw Error(SO_ERR_INVALID, "not a control"); }
  // Saver
  virtual void monitor(WaveFunction&, Emitter&) { throw Error(SO_ERR_INVALID, "not a saver"); }
  virtual void reset() {}
  // Device-or-host scalars the operator carries between steps (checkpoints)
  virtual std::vector<ScalarState*> scalar_states() {
    std::vector<ScalarState*> v;
    if (LossChecker* lc = loss_checker()) v.push_back(&lc->st);
    return v;
  }
};

struct OneDimPropagator : Operator {
  size_t dimension_no;
  std::vector<cplx> op;
  std::unique_ptr<LossChecker> lc;
  OneDimPropagator(size_t shape, size_t dim)
      : Operator(OpClass::Propagator, "OneDimPropagator"), dimension_no(dim), op(shape, cplx(1, 0)) {}
  void apply_unchecked(WaveFunction& wf, Emitter& em);
  void apply(WaveFunction& wf, Emitter& em) override;
  LossChecker* loss_checker() override { return lc.get(); }
};

struct NDimPropagator : Operator {
  std::vector<size_t> shape{1};
  std::vector<cplx> op{cplx(0, 0)};
  std::unique_ptr<LossChecker> lc;
  NDimPropagator() : Operator(OpClass::Propagator, "NDimPropagator") {}
  void apply(WaveFunction& wf, Emitter& em) override;
  LossChecker* loss_checker() override { return lc.get(); }
};

struct NonDiagPropagator : Operator {
  size_t dimension_no;
  size_t n = 0, count = 0;
  std::vector<cplx> ops;  // count x n x n
  std::unique_ptr<LossChecker> lc;
  explicit NonDiagPropagator(size_t dim) : Operator(OpClass::Propagator, "NonDiagPropagator"), dimension_no(dim) {}
  void apply(WaveFunction& wf, Emitter& em) override;
  LossChecker* loss_checker() override { return lc.get(); }
};

struct FFTTransformation : Operator {
  size_t dimension_no, dimension_size;
  Grid grid_trans;
  FFTTransformation(const Grid& g, const std::string& name);
  void transform(WaveFunction& wf, Emitter& em) override;
  void inverse_transform(WaveFunction& wf, Emitter& em) override;
  Grid* grid_transformation() override { return &grid_trans; }
};

struct MatrixTransformation : Operator {
  size_t dimension_no, dimension_size;
  std::vector<cplx> t, tinv;
  Grid grid_trans;
  MatrixTransformation(const Grid& g, const Grid& gt);
  void transform(WaveFunction& wf, Emitter& em) override;
  void inverse_transform(WaveFunction& wf, Emitter& em) override;
  Grid* grid_transformation() override { return &grid_trans; }
};

struct StateMatrixTransformation : Operator {
  size_t dimension_no, dependent, n, count = 0;
  std::vector<cplx> ts, tinvs;
  Grid grid_trans;
  StateMatrixTransformation(size_t dep, const Grid& g, const Grid& gt);
  void transform(WaveFunction& wf, Emitter& em) override;
  void inverse_transform(WaveFunction& wf, Emitter& em) override;
  Grid* grid_transformation() override { return &grid_trans; }
};

struct LeakControl : Operator {  // leak_control.rs
  ScalarState st{1};
  std::unique_ptr<LossChecker> lc;
  LeakControl() : Operator(OpClass::Control, "LeakControl") {}
  std::string name() const override { return "LeakControl"; }
  void first_half(WaveFunction& wf, Emitter& em) override;
  void second_half(WaveFunction& wf, Emitter& em) override;
  LossChecker* loss_checker() override { return lc.get(); }
  std::vector<ScalarState*> scalar_states() override {
    std::vector<ScalarState*> v{&st};
    if (lc) v.push_back(&lc->st);
    return v;
  }
};

struct BorderDumping : Operator {  // border_dumping.rs:36-93
  OneDimPropagator op;
  std::unique_ptr<LossChecker> lc;
  BorderDumping(const std::vector<cplx>& mask, const Grid& g);
  std::string name() const override { return "BorderDumping"; }
  void half(WaveFunction& wf, Emitter& em);
  void first_half(WaveFunction& wf, Emitter& em) override { half(wf, em); }
  void second_half(WaveFunction& wf, Emitter& em) override { half(wf, em); }
  LossChecker* loss_checker() override { return lc.get(); }
};

struct StateSaver : Operator {  // wave_function_saver.rs:101-183 (StateSaver) and :6-98 (2-D saver)
  bool two_d;
  std::string fname;
  so_time_grid time;
  Grid grid_a, grid_b;  // state grid (or x grid), y grid
  size_t frames_no, current_frame = 0, points;
  std::vector<double> data;  // (points, frames_no) row-major
  std::vector<double> times;
  StateSaver(const std::string& name, so_time_grid t, const Grid& a, const Grid* b, size_t frames);
  void monitor(WaveFunction& wf, Emitter& em) override;
  void reset() override;
  void record_frame(WaveFunction& wf, size_t frame);
  void save() const;
};

// ------------------------------------------------------------ stack + propagation
struct StackEntry {
  std::shared_ptr<Operator> op;
  int flag;  // Order or Apply bits
};

struct OperationStack {
  std::vector<StackEntry> stack;
};

class Propagation {
 public:
  Propagation(WaveFunction& wf, so_time_grid time, std::shared_ptr<OperationStack> stack, int precision);
  ~Propagation();
  void steps(uint64_t n);
  void propagate() { steps(time_.step_no); }
  void reset_savers();
  void savers_save();
  double mean_energy();
  std::vector<double> losses(bool include_controls);
  void reset_losses();
  std::unique_ptr<WaveFunction> snapshot();
  // sync false: queued on the engine stream; copy_engine: staged through cudaMemcpyAsync
  void get_array(double* out, bool sync = true, bool copy_engine = false);
  void set_array(const double* in, bool copy_engine = false);
  void state_replaced() { wf_->possible_norm_change = true; }  // after a direct engine import
  double norm();
  std::string describe();
  void set_stream(cudaStream_t s) { wf_->eng->stream = s; }
  void synchronize();
  void set_timing(bool on) { wf_->eng->timing = on; }
  std::string kernel_times() { return wf_->eng->collect_timing(); }
  Engine& engine() { return *wf_->eng; }
  // Run the host logic of `n` steps, capturing the passes instead of launching them.
  std::vector<RecordedPass> record_steps(uint64_t n);
  bool has_savers() const;
  // Steps taken since creation (or since the restored checkpoint was taken).
  uint64_t steps_done() const { return steps_done_; }
  void count_steps(uint64_t n) { steps_done_ += n; }  // steps run by a batch on this propagation
  // Everything a later run needs to continue exactly where this one stands: the state in
  // its storage precision, the norm cache, every loss checker, leak-control norm and saver,
  // and the step count.  restore() checks that the blob fits this propagation's shape,
  // precision and operator stack, then replaces the lot.
  std::vector<unsigned char> checkpoint();
  void restore(const unsigned char* data, size_t size);

  int precision;

 private:
  uint64_t steps_done_ = 0;
  void step(Emitter& em);
  std::unique_ptr<WaveFunction> wf_;
  so_time_grid time_;
  std::shared_ptr<OperationStack> stack_;
  std::vector<std::shared_ptr<Operator>> keep_;
};

// Many independent propagations stepped together: every pass position of the
// steady-state step becomes a few batched launches (one per kernel / shape class)
// covering all instances; the periodic part is captured once as a CUDA graph.
class Batch {
 public:
  explicit Batch(std::vector<Propagation*> props);
  ~Batch();
  // wait false: return once the launches are queued (the batch's stream runs them)
  // sync_members false: members whose stream is the batch's are not waited on by the host
  void steps(uint64_t n, bool wait = true, bool sync_members = true);
  void set_timing(bool on) { timing_ = on; }
  std::string kernel_times();
  size_t launches_per_step() const { return launches_per_step_; }
  size_t size() const { return props_.size(); }
  // every member's state from / to host arrays (logical complex128); get waits once at the end
  void set_arrays(const double* const* in);
  void get_arrays(double* const* out);
  // set_arrays, steps(n), get_arrays as one pipeline over member chunks on separate streams
  void steps_host(const double* const* in, double* const* out, uint64_t n);

 private:
  struct Group {
    RecordedPass::Kind kind;
    int real;
    bool sweep = false;  // lane-sweep groups: every member's pass runs the compact sweep kernel
    int threads;
    size_t smem;
    int64_t blocks;
    int count;
    DeviceBuffer params, offsets;
    DeviceBuffer owners;  // tensor-core groups: (pass index, tile within the pass) per global tile
    std::string name;
    double bytes;
    int64_t n = 0;  // lane extent of the members' passes (the schedule class)
    int ct_lgn = 0;  // fixed-shape FFT-pair kernel: log2 of the lane extent (0: general shape)
  };
  std::vector<Group> build_groups(const std::vector<std::vector<RecordedPass>>& rec, size_t pos);
  std::vector<std::vector<RecordedPass>> cached_rec_;  // the passes the cached groups were built from
  uint64_t cached_epoch_ = 0;                          // the launch schedules they were built with
  std::vector<std::vector<Group>> cached_pos_;
  struct Chunk {
    size_t first = 0, count = 0;
    cudaStream_t stream = nullptr;
    // the chunk's copies in and its copies out are done (the next chunk's copies wait on them)
    cudaEvent_t in_done = nullptr, out_done = nullptr;
    std::unique_ptr<Batch> batch;
    // the chunk's members' logical complex128 arrays back to back (used when the caller's
    // host arrays are back to back too: one copy per direction instead of one per member)
    DeviceBuffer stage;
  };
  std::vector<Chunk> chunks_;  // steps_host pipeline (built on first use)
  struct TraceBuf {
    DeviceBuffer buf;
    int64_t tiles = 0;
    std::string name;
  };
  std::vector<TraceBuf> traces_;  // SO_TC_TRACE_BATCH diagnostics
  // concurrent: the groups of one pass position (disjoint members) on forked streams, so
  // that each launch's last wave overlaps the others' (untimed runs only)
  void run_groups(std::vector<Group>& gs, bool concurrent = false);
  std::vector<Propagation*> props_;
  cudaStream_t stream_ = nullptr;
  bool own_stream_ = false;
  std::vector<cudaStream_t> side_;  // forked streams of the concurrent groups
  std::vector<cudaEvent_t> joins_;  // one per side stream
  cudaEvent_t fork_ = nullptr;
  bool timing_ = false;
  size_t launches_per_step_ = 0;
  struct Timed {
    std::string name;
    cudaEvent_t a, b;
    double bytes;
    int cls_kind = -1;  // 0 FFT-pair pass, 1 tensor-core pass, -1 other
    int64_t cls_n = 0;
    int cls_mode = 0;   // FFT pair: 1 for FP64; tensor core: operand mode
  };
  std::vector<Timed> timed_;

 public:
  // Autotuner: times the candidate launch schedules of every lane extent of the batch's FFT-pair
  // and tensor-core passes on the live workload (CUDA events, `trial_steps` steps per
  // candidate), keeps the fastest per extent in the process-wide schedule table, writes the
  // table to `cache_path` (JSON; empty: no file) and restores every member's state.
  // Returns a JSON report: per extent, each candidate's milliseconds and the one chosen.
  std::string tune(const std::string& cache_path, int trial_steps);
};

}  // namespace so
