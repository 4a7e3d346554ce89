// Shared device-side definitions of the split-operator GB300 library.
//
// A wave function lives in GPU memory as interleaved complex values (double2 or
// float2) in "storage order": row-major over the logical axes permuted by
// `perm` (storage position p holds logical axis perm[p]); the propagation puts
// its FFT axis last so radial FFT lanes are contiguous.
//
// Work is issued as *passes*.  A pass owns whole lanes along one axis (the
// sweep axis): every CTA loads a tile of complete lanes into shared memory,
// runs a short program of ops on it (diagonal multiplies, FFT or lane matrix
// along the sweep axis, FP64 norm partial sums), stores it back, and the last
// CTA to finish folds the norm partials in a fixed order (deterministic) and
// runs the program's scalar bookkeeping (loss accumulation, slot copies).
#pragma once
#include <cstdint>
#include <cstring>
#include <string>
#include <vector>
#include <cuda_runtime.h>

namespace so {

constexpr int kMaxDims = 4;
// state precisions: FP32 (float2), FP64 (double2), float-float (two FP32 per real, 16 bytes
// per complex value like FP64)
constexpr int kRealF32 = 0, kRealF64 = 1, kRealFF = 2;
constexpr int kMaxOps = 24;
constexpr int kMaxRed = 8;      // norm reductions per pass
constexpr int kNumSlots = 256;  // FP64 scalar slots per engine

enum OpKind : int32_t {
  OP_DIAG1D = 0,     // psi *= table[coord(axis)]
  OP_DIAGND = 1,     // psi *= table[storage index]
  OP_FFT = 2,        // unitary DFT along the sweep axis, dir = -1 forward, +1 inverse
  OP_MAT = 3,        // lane <- M lane along the sweep axis (one matrix)
  OP_MAT_LANE = 4,   // matrix per lane (non-diagonal propagator)
  OP_MAT_SLICE = 5,  // matrix per index of a dependent axis (state matrix transformation)
  OP_NORM = 6,       // slot[a] = sum |psi|^2 prod_axis w_axis (FP64)
  OP_COPY = 7,       // slot[a] = slot[b]
  OP_LOSS = 8,       // slot[a] += slot[b] - slot[c]
  OP_SCALE = 9,      // psi *= sqrt(slot[b] / slot[c])
  OP_SETC = 10,      // slot[a] = value
  OP_RECORD = 11,    // record[count] = slot[a]
  OP_DOT = 12        // slot[a] + i slot[b] = sum psi conj(other) prod w  (other = ptr, same layout)
};

struct DevOp {
  int32_t kind;
  int32_t axis;   // logical axis (DIAG1D), dependent axis (MAT_SLICE)
  int32_t dir;    // FFT direction
  int32_t a, b, c;
  int32_t red;    // reduction index inside the pass (NORM, DOT uses red and red+1)
  int32_t flags;  // bit0: matrix is real
  int64_t count;  // matrices available (MAT_LANE / MAT_SLICE), record index (RECORD)
  double value;   // SETC
  const void* ptr;               // table / matrix base / other wave function
  const double* w[kMaxDims];     // NORM / DOT weights per logical axis
  const float* wf[kMaxDims];     // the same weights rounded to FP32 (FP32 passes)
};

struct Geometry {
  int32_t ndim;
  int32_t perm[kMaxDims];       // storage position -> logical axis
  int64_t sshape[kMaxDims];     // storage shape
  int32_t spos;                 // storage position of the sweep axis
  int32_t sweep_axis;           // logical sweep axis
  int64_t n;                    // sweep axis extent
  int64_t inner;                // product of storage dims after spos
  int64_t outer;                // product of storage dims before spos
  int32_t lanes_per_tile;       // L
  int32_t tiles_per_outer;      // inner > 1: inner / L; inner == 1: 1
  int64_t tiles;                // grid size
  int32_t vals;                 // V: values a thread holds in FFT/MAT ops
  int32_t lane_stride;          // padded shared-memory lane stride (complex units)
};

struct PassParams {
  Geometry g;
  void* psi;
  double* slots;
  double* partials;             // [kMaxRed][tiles]
  unsigned int* counter;        // last-block ticket (reset by the last block)
  const void* twiddle;          // n entries, state precision: stage-major (stage_twiddle_exponent) for
                                // power-of-two n >= 16, else exp(-2 pi i j / n) at j
  double* record;
  int32_t nops;
  int32_t nred;
  int32_t repeat;               // resident mode: program repetitions
  int32_t resident;             // 1: single CTA owns the whole array, scalars are immediate
  int32_t nonfinite_slot;       // slot set to 1 if a norm is not finite
  int32_t one_buffer;           // 1: no op needs the second tile buffer (FFT stages run in place)
  int32_t sweep;                // 1: only point-wise ops, norms, scalars and power-of-two FFTs
  int32_t fused;                // 1: an FFT pair with point-wise ops, run by fft_pair_kernel
  int32_t radix;                // fused: radix of the Stockham stages (16 or 8; the twiddle table's order)
  int32_t ct;                   // fused FP32: log2 n of the fixed-shape kernel (0: the general-shape kernel)
  DevOp ops[kMaxOps];
};

// Radix sequence of the Stockham stages of a power-of-two lane FFT: rmax while at least
// rmax points remain, then one smaller closing radix; `reversed` lists it backwards.
// Returns the number of stages (at most 13).
__host__ __device__ inline int fft_radices(int64_t n, int rmax, bool reversed, int* rs) {
  int c = 0;
  for (int64_t p = 1; p < n;) {
    const int64_t r = n / p >= rmax ? rmax : n / p;
    rs[c++] = (int)r;
    p *= r;
  }
  if (reversed)
    for (int a = 0, b = c - 1; a < b; ++a, --b) {
      const int t = rs[a];
      rs[a] = rs[b];
      rs[b] = t;
    }
  return c;
}

// Twiddle table of a power-of-two lane FFT (n >= 16) in stage-major order: stage (RS, p)
// with p > 1 owns (RS - 1) * p consecutive entries, entry (r - 1) * p + k holding
// w^(r k n / (RS p)), w = exp(-2 pi i / n).  Threads of a stage read consecutive k, so the
// shared-memory reads are free of bank conflicts.  Returns the exponent of entry e for the
// stages in fft_radices order (0 past the end: a table occupies at most n entries).  The
// device table holds the forward order in entries [0, n) and the reversed order in [n, 2n).
__host__ __device__ inline int64_t stage_twiddle_exponent(int64_t e, int64_t n, int rmax, bool reversed = false) {
  int rs[16];
  const int c = fft_radices(n, rmax, reversed, rs);
  int64_t p = 1, off = 0;
  for (int s = 0; s < c; ++s) {
    const int64_t r_s = rs[s];
    if (p > 1) {
      const int64_t cnt = (r_s - 1) * p;
      if (e < off + cnt) {
        const int64_t q = e - off, r = q / p + 1, k = q - (r - 1) * p;
        return r * k * (n / (r_s * p));
      }
      off += cnt;
    }
    p *= r_s;
  }
  return 0;
}
__host__ __device__ inline bool stage_twiddles(int64_t n) { return n >= 16 && (n & (n - 1)) == 0; }
// A pass copies its twiddle table into shared memory, except for power-of-two lanes in tiles
// of fewer than 4 lanes: there the copy would cost a load and a store per point, and the
// stages read their consecutive table slices straight through L1 / L2 instead.
__host__ __device__ inline bool twiddles_in_smem(const Geometry& g) {
  return !(stage_twiddles(g.n) && g.lanes_per_tile < 4);
}

// Launch schedules (schedule.cpp), per lane extent n; 0 fields mean the built-in default.
// FFT-pair pass: threads per CTA (128, 256 or 512; lanes per tile = 16 threads / n) and the
// radix of its Stockham stages (16 or 8).  Tensor-core pass: persistent CTAs per SM (1 or 2)
// and the batched tile order (0 strided, 1 one run of consecutive tiles per CTA).
struct PairSchedule {
  int threads, radix;
};
struct TcSchedule {
  int ctas_per_sm, blocked;
};
PairSchedule pair_schedule(int64_t n, bool fp64);
TcSchedule tc_schedule(int64_t n, int mode);
void set_pair_schedule(int64_t n, bool fp64, PairSchedule s);
void set_tc_schedule(int64_t n, int mode, TcSchedule s);
void reset_schedules();
uint64_t schedule_epoch();  // changes whenever a schedule does
std::string schedules_json();
bool schedules_from_json(const std::string& text);

// FFT pair pass (lane_sweep.cu): [FFT] [DIAG1D along / DIAGND]* [FFT] [DIAG1D along / DIAGND]*
// over contiguous power-of-two FP32 lanes, every thread holding 16 values in registers.
// fft_pair_plan checks the pass and sets its tiling (lanes per tile, tiles) and p.fused.
bool fft_pair_plan(PassParams& p, int real, bool resident);
int fft_pair_threads(const Geometry& g);  // the default threads per CTA
int fft_pair_block(const Geometry& g);    // threads per CTA of a planned pass (lanes per tile x n / 16)

// Host launchers (lane_sweep.cu)
cudaError_t launch_pass_f64(const PassParams& p, cudaStream_t s);
cudaError_t launch_pass_ff(const PassParams& p, cudaStream_t s);
cudaError_t launch_pass_f32(const PassParams& p, cudaStream_t s);
size_t pass_smem_bytes(const PassParams& p, bool fp64);
int pass_threads(const Geometry& g);
// sets p.one_buffer and p.sweep from the pass's ops and geometry (call once p.ops, p.nops, p.g are set)
void pass_choose_buffers(PassParams& p, bool fp64);

// Tensor-core angular sweep (angular_tc.cu): FP32 state, real lane matrices as 3xTF32.
int angular_tc_columns(int n);  // complex columns of the inner axis per CTA tile
bool angular_tc_eligible(const Geometry& g);
// column groups one tile of this pass packs into the tensor core's 128 rows (1: none)
int angular_tc_pack(const Geometry& g, const DevOp* ops, int nops, int mode);
// the pass's point-wise ops fit the per-tile tables of the tensor-core kernel
bool angular_tc_ops_fit(const DevOp* ops, int nops, int sweep_axis);
// operand modes of the tensor-core pass: 0 3xTF32, 1 split-BF16x3, 2 split-BF16x6 (exact sums)
size_t angular_tc_smem_bytes(int n, bool par = false, int mode = 0);
// A-operand chunk images of an operand mode, raw bytes in a float vector
void angular_tc_images(const double* m, int n, int mode, std::vector<float>& out);
// parity structure of a real n x n lane matrix (0 none, 1 row signs, 2 column signs; n = 256 only)
int angular_tc_parity(const double* m, int n);
void angular_tc_parity_images(const double* m, int n, int kind, int mode, std::vector<float>& out);
// parity: per matrix 0 / 1 / 2 (all 0, or all non-zero with the split images); trace: optional
// per-tile phase timestamps (angular_tc_trace_slots() per tile), nullptr: off
cudaError_t launch_angular_tc(const PassParams& p, const int* mat_op, int nmat, const float* const* images,
                              int error_slot, const int* parity, int mode, cudaStream_t s,
                              unsigned long long* trace = nullptr, int ctas_per_sm = 0, int pack = 1,
                              const int* slice_axis = nullptr, const int64_t* slice_stride = nullptr);
int angular_tc_trace_slots();
// one CTA waits (limit_ns, both wait forms) on an mbarrier nothing completes; out[3]:
// timed out (try_wait form), timed out (polling form), elapsed ns
cudaError_t bounded_wait_selftest(uint64_t limit_ns, unsigned long long* host_out);

// Batched launches over many propagations' passes (block -> (instance, tile) by offsets)
cudaError_t launch_pass_batched(int real, bool sweep, bool fused, const PassParams* params_dev,
                                const int64_t* offsets_dev, int count, int64_t blocks, int threads, size_t smem,
                                cudaStream_t s, int radix = 0, int ct_lgn = 0);
// log2 n when a planned FP32 FFT-pair pass can run the fixed-shape kernel, else 0
int fft_pair_ct_lgn(const PassParams& p, bool fp64);
size_t tc_params_bytes();
void tc_params_set_trace(void* params, unsigned long long* trace);  // the TcParams' trace field
// slice_axis[m] >= 0: matrix m is a state matrix, one image per coordinate of that logical
// axis, slice_stride[m] floats apart (the coordinate is constant over every tile)
void make_tc_params(const PassParams& p, const int* mat_op, int nmat, const float* const* images, int error_slot,
                    const int* parity, void* out, int pack = 1, const int* slice_axis = nullptr,
                    const int64_t* slice_stride = nullptr);
// persistent CTAs a launch of `tiles` tensor-core tiles runs on (CTA k takes the tiles at
// positions k, k + grid, k + 2 grid, ... of the owners table)
int64_t angular_tc_grid(int64_t tiles, int ctas_per_sm = 0);
// owners_dev: blocks pairs (pass index, tile within the pass), uint32 each, in global tile order
cudaError_t launch_angular_tc_batched(const void* params_dev, const void* owners_dev, int64_t blocks, size_t smem,
                                      int mode, cudaStream_t s, int ctas_per_sm = 0, int pack = 1);

// Auxiliary kernels (aux_kernels.cu)
cudaError_t launch_scalar_program(const PassParams& p, cudaStream_t s);
// real: the state precision of the device side (kRealF32, kRealF64, kRealFF)
// dst (storage order, precision of dst) <- src (logical row-major complex128)
cudaError_t launch_import(void* dst, int dst_real, const double* src, const Geometry& g, cudaStream_t s);
// storage order is the logical order / the transpose of a two-axis logical order (the
// layouts whose import and export stay coalesced on both sides)
bool layout_is_identity(const Geometry& g);
bool layout_is_transpose2(const Geometry& g);
// dst (logical row-major complex128) <- src (storage order)
cudaError_t launch_export(double* dst, const void* src, int src_real, const Geometry& g, cudaStream_t s);
// density |psi|^2 in logical order, and its weighted marginal along one logical axis
cudaError_t launch_density(double* dst, const void* src, int real, const Geometry& g, cudaStream_t s);
cudaError_t launch_state_density(double* dst, const void* src, int real, const Geometry& g, int axis,
                                 const double* const* w, double* partials, cudaStream_t s);
cudaError_t launch_copy_convert(void* dst, int dst_real, const void* src, int src_real, int64_t n,
                                cudaStream_t s);
cudaError_t launch_table_convert(void* dst, bool dst_fp64, const double* src_dev, int64_t count, cudaStream_t s);

void count_launch(uint64_t k = 1);
uint64_t launch_count();

}  // namespace so
