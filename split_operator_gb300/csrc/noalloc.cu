// Allocation-free entry point: the lane FFT + weighted norm pass for callers
// that cannot allocate GPU memory themselves or let a library do it -- for
// example code running inside a memory pool that forbids cudaMalloc while it
// holds the device, or a host framework that hands over only pre-sized buffers.
//
// It runs the same lane-sweep pass kernel as the rest of the library, but the
// kernel's scratch (per-CTA norm partials, the last-CTA ticket counter) and the
// FFT twiddle table live in file-scope __device__ arrays of fixed size instead of
// library-allocated buffers.  Every GPU that loads the library holds these arrays
// (about 0.6 MiB) until the process exits.
#include <algorithm>
#include <cmath>
#include <cstdio>

#include "../../include/split_operator.h"
#include "common.cuh"

namespace so {
void set_last_error(const char* msg);  // api.cpp: the message so_last_error() returns

namespace {

constexpr int64_t kMaxTiles = 65536;  // CTAs of one call (norm partials)
constexpr int64_t kMaxLane = 4096;    // FP64 lane length (twiddle table)
constexpr int kMaxDevices = 64;

static __device__ __align__(256) double g_partials[kMaxTiles];
static __device__ __align__(256) unsigned int g_counter[4];
static __device__ __align__(256) double2 g_twiddle[kMaxLane];

struct DeviceScratch {
  bool ready = false;
  double* partials = nullptr;
  unsigned int* counter = nullptr;
  double2* twiddle = nullptr;
};
DeviceScratch g_dev[kMaxDevices];

// exp(-2 pi i m / n) from sincospi (exact at multiples of a quarter turn); m = j, or the
// stage-major exponent of entry j for the FP64 Stockham stages of power-of-two n >= 16
__global__ void twiddle_kernel(double2* tw, int64_t n) {
  for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < n; j += (int64_t)gridDim.x * blockDim.x) {
    const int64_t m = stage_twiddles(n) ? stage_twiddle_exponent(j, n, 8) : j;
    double s, c;
    sincospi(2.0 * (double)m / (double)n, &s, &c);
    tw[j] = make_double2(c, -s);
  }
}

int fail(int status, const char* msg) {
  set_last_error(msg);
  return status;
}

}  // namespace
}  // namespace so

extern "C" int so_fft_norm_noalloc(double* psi, size_t lanes, size_t n, int direction, const double* lane_weights,
                                   const double* weights, double* norm_out, void* stream_ptr) {
  using namespace so;
  if (!psi || lanes == 0 || n < 2 || (direction != -1 && direction != 1))
    return fail(SO_ERR_INVALID, "so_fft_norm_noalloc: bad argument");
  if ((weights == nullptr) != (norm_out == nullptr) || (weights && !lane_weights))
    return fail(SO_ERR_INVALID, "so_fft_norm_noalloc: weights, lane_weights and norm_out go together");
  if ((int64_t)n > kMaxLane) return fail(SO_ERR_UNSUPPORTED, "so_fft_norm_noalloc: lane longer than 4096 points");
  cudaStream_t stream = (cudaStream_t)stream_ptr;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices)
    return fail(SO_ERR_CUDA, "so_fft_norm_noalloc: no current CUDA device");

  // geometry: [lanes][n], lanes contiguous, tiles of L lanes (the heuristic of the library's engine)
  Geometry g{};
  g.ndim = 2;
  g.perm[0] = 0;
  g.perm[1] = 1;
  g.sshape[0] = (int64_t)lanes;
  g.sshape[1] = (int64_t)n;
  g.spos = 1;
  g.sweep_axis = 1;
  g.n = (int64_t)n;
  g.inner = 1;
  g.outer = (int64_t)lanes;
  g.vals = 8;
  auto pow2_floor = [](int64_t v) {
    int64_t p = 1;
    while (p * 2 <= v) p *= 2;
    return p;
  };
  const int64_t lmax = std::max<int64_t>(1, pow2_floor(kMaxLane / g.n));
  int64_t want = pow2_floor(std::max<int64_t>(1, g.outer / 304));
  want = std::max<int64_t>(want, pow2_floor(std::max<int64_t>(1, 1024 / g.n)));
  const int64_t L = std::min(want, lmax);
  g.lanes_per_tile = (int32_t)L;
  g.tiles_per_outer = 1;
  g.tiles = (g.outer + L - 1) / L;
  int64_t ls = g.n + (g.n >> 4);
  if (ls % 2 == 0) ls += 1;
  g.lane_stride = (int32_t)ls;
  if (g.tiles > kMaxTiles)
    return fail(SO_ERR_UNSUPPORTED, "so_fft_norm_noalloc: more than 65536 CTAs of lanes (too many lanes)");

  // set-up once per device, with that device current: device addresses of the scratch arrays
  DeviceScratch& d = g_dev[dev];
  if (!d.ready) {
    if (cudaGetSymbolAddress((void**)&d.partials, g_partials) != cudaSuccess ||
        cudaGetSymbolAddress((void**)&d.counter, g_counter) != cudaSuccess ||
        cudaGetSymbolAddress((void**)&d.twiddle, g_twiddle) != cudaSuccess) {
      cudaGetLastError();
      return fail(SO_ERR_CUDA, "so_fft_norm_noalloc: cudaGetSymbolAddress failed");
    }
    d.ready = true;
  }
  // the ticket counter must start at zero (the kernel's last CTA resets it too)
  if (cudaMemsetAsync(d.counter, 0, sizeof(unsigned int), stream) != cudaSuccess)
    return fail(SO_ERR_CUDA, "so_fft_norm_noalloc: counter reset failed");
  // the twiddle table is rebuilt on every call (n <= 4096 entries, one small kernel): a
  // table kept from an earlier call could belong to another lane length by the time this
  // call's pass runs, whatever order the caller's work reaches the GPU in
  twiddle_kernel<<<(unsigned)std::min<int64_t>(64, (g.n + 255) / 256), 256, 0, stream>>>(d.twiddle, g.n);
  if (cudaGetLastError() != cudaSuccess) return fail(SO_ERR_CUDA, "so_fft_norm_noalloc: twiddle kernel failed");
  count_launch();

  PassParams p{};
  p.g = g;
  p.psi = psi;
  p.slots = norm_out;  // the norm op writes slot 0
  p.partials = d.partials;
  p.counter = d.counter;
  p.twiddle = d.twiddle;
  p.record = nullptr;
  p.repeat = 1;
  p.resident = 0;
  p.nonfinite_slot = -1;
  p.nops = 1;
  p.ops[0].kind = OP_FFT;
  p.ops[0].dir = direction;
  if (weights) {
    p.nops = 2;
    p.nred = 1;
    p.ops[1].kind = OP_NORM;
    p.ops[1].a = 0;
    p.ops[1].red = 0;
    p.ops[1].w[0] = lane_weights;
    p.ops[1].w[1] = weights;
  }
  if (launch_pass_f64(p, stream) != cudaSuccess) return fail(SO_ERR_CUDA, "so_fft_norm_noalloc: launch failed");
  return SO_OK;
}
