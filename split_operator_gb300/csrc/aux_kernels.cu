// Auxiliary kernels: scalar-only pass programs, layout import/export between the
// host's logical row-major complex128 arrays and the device storage order,
// precision conversion, and the saver reductions (density, state_density of
// wave_function.rs:112-148).
#include <atomic>

#include "common.cuh"
#include "ff.cuh"

namespace so {

// f(T{}) with T the device complex type of a state precision
template <typename F>
static cudaError_t by_real(int real, F f) {
  switch (real) {
    case kRealF64: return f(double2{});
    case kRealFF: return f(ffc{});
    default: return f(float2{});
  }
}

static std::atomic<uint64_t> g_launches{0};
void count_launch(uint64_t k) { g_launches.fetch_add(k, std::memory_order_relaxed); }
uint64_t launch_count() { return g_launches.load(std::memory_order_relaxed); }

__global__ void scalar_program_kernel(const __grid_constant__ PassParams p) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  double* s = p.slots;
  for (int i = 0; i < p.nops; ++i) {
    const DevOp& op = p.ops[i];
    switch (op.kind) {
      case OP_COPY:
        s[op.a] = s[op.b];
        break;
      case OP_LOSS:
        s[op.a] += s[op.b] - s[op.c];
        break;
      case OP_SETC:
        s[op.a] = op.value;
        break;
      case OP_RECORD:
        if (p.record) p.record[op.count] = s[op.a];
        break;
      default:
        break;
    }
  }
}

cudaError_t launch_scalar_program(const PassParams& p, cudaStream_t st) {
  scalar_program_kernel<<<1, 32, 0, st>>>(p);
  count_launch();
  return cudaGetLastError();
}

struct Perm {
  int nd;
  int perm[kMaxDims];
  int64_t sshape[kMaxDims];
  int64_t lstride[kMaxDims];  // logical row-major stride of each logical axis
};

static Perm make_perm(const Geometry& g) {
  Perm p{};
  p.nd = g.ndim;
  int64_t lshape[kMaxDims] = {1, 1, 1, 1};
  for (int q = 0; q < g.ndim; ++q) {
    p.perm[q] = g.perm[q];
    p.sshape[q] = g.sshape[q];
    lshape[g.perm[q]] = g.sshape[q];
  }
  int64_t st = 1;
  for (int a = g.ndim - 1; a >= 0; --a) {
    p.lstride[a] = st;
    st *= lshape[a];
  }
  return p;
}

__device__ __forceinline__ int64_t logical_of_storage(const Perm& P, int64_t s) {
  int64_t li = 0;
  for (int q = P.nd - 1; q >= 0; --q) {
    const int64_t c = s % P.sshape[q];
    s /= P.sshape[q];
    li += c * P.lstride[P.perm[q]];
  }
  return li;
}

template <typename D>
__global__ void import_kernel(D* dst, const double2* src, Perm P, int64_t total) {
  for (int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; s < total; s += (int64_t)gridDim.x * blockDim.x) {
    const double2 v = src[logical_of_storage(P, s)];
    dst[s] = D{(decltype(dst->x))v.x, (decltype(dst->x))v.y};
  }
}

template <typename S>
__global__ void export_kernel(double2* dst, const S* src, Perm P, int64_t total) {
  for (int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; s < total; s += (int64_t)gridDim.x * blockDim.x) {
    const S v = src[s];
    dst[logical_of_storage(P, s)] = double2{(double)v.x, (double)v.y};
  }
}

template <typename S>
__global__ void density_kernel(double* dst, const S* src, Perm P, int64_t total) {
  for (int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; s < total; s += (int64_t)gridDim.x * blockDim.x) {
    const S v = src[s];
    dst[logical_of_storage(P, s)] = (double)v.x * (double)v.x + (double)v.y * (double)v.y;
  }
}

// Two-axis layouts whose storage order is the transpose of the logical order (the radial
// FFT axis, logical axis 0, stored last): a 32 x 32 tile is read along the source's
// contiguous axis and written along the destination's, through shared memory, so both
// sides are coalesced.  This matters most when one side is pinned host memory read or
// written directly by the kernel over the host link.
//   import: logical [a0][a1] (complex128)  ->  storage [a1][a0] (D)
//   export: storage [a1][a0] (S)           ->  logical [a0][a1] (complex128)
constexpr int kTT = 32;

template <typename D>
__global__ void __launch_bounds__(256) import_transpose_kernel(D* __restrict__ dst, const double2* __restrict__ src,
                                                               int64_t n0, int64_t n1) {
  __shared__ double2 tile[kTT][kTT + 1];
  const int64_t a1 = blockIdx.x * (int64_t)kTT, a0 = blockIdx.y * (int64_t)kTT;
  const int tx = threadIdx.x, ty = threadIdx.y;
  for (int i = ty; i < kTT; i += 8) {
    const int64_t r = a0 + i, c = a1 + tx;
    if (r < n0 && c < n1) tile[i][tx] = src[r * n1 + c];
  }
  __syncthreads();
  for (int i = ty; i < kTT; i += 8) {
    const int64_t c = a1 + i, r = a0 + tx;
    if (r < n0 && c < n1) {
      const double2 v = tile[tx][i];
      dst[c * n0 + r] = D{(decltype(dst->x))v.x, (decltype(dst->x))v.y};
    }
  }
}

template <typename S>
__global__ void __launch_bounds__(256) export_transpose_kernel(double2* __restrict__ dst, const S* __restrict__ src,
                                                               int64_t n0, int64_t n1) {
  __shared__ double2 tile[kTT][kTT + 1];
  const int64_t a1 = blockIdx.x * (int64_t)kTT, a0 = blockIdx.y * (int64_t)kTT;
  const int tx = threadIdx.x, ty = threadIdx.y;
  for (int i = ty; i < kTT; i += 8) {
    const int64_t c = a1 + i, r = a0 + tx;
    if (r < n0 && c < n1) {
      const S v = src[c * n0 + r];
      tile[tx][i] = double2{(double)v.x, (double)v.y};
    }
  }
  __syncthreads();
  for (int i = ty; i < kTT; i += 8) {
    const int64_t r = a0 + i, c = a1 + tx;
    if (r < n0 && c < n1) dst[r * n1 + c] = tile[i][tx];
  }
}

bool layout_is_transpose2(const Geometry& g) { return g.ndim == 2 && g.perm[0] == 1 && g.perm[1] == 0; }
bool layout_is_identity(const Geometry& g) {
  for (int q = 0; q < g.ndim; ++q)
    if (g.perm[q] != q) return false;
  return true;
}

static dim3 transpose_grid(const Geometry& g) {  // g.sshape = {n1, n0}
  return dim3((unsigned)((g.sshape[0] + kTT - 1) / kTT), (unsigned)((g.sshape[1] + kTT - 1) / kTT));
}

static int64_t total_of(const Geometry& g) {
  int64_t t = 1;
  for (int q = 0; q < g.ndim; ++q) t *= g.sshape[q];
  return t;
}

static unsigned blocks_for(int64_t total) {
  int64_t b = (total + 255) / 256;
  if (b > 152 * 32) b = 152 * 32;
  if (b < 1) b = 1;
  return (unsigned)b;
}

cudaError_t launch_import(void* dst, int dst_real, const double* src, const Geometry& g, cudaStream_t st) {
  const int64_t total = total_of(g);
  if (layout_is_transpose2(g)) {
    const dim3 grid = transpose_grid(g), block(kTT, 8);
    if (grid.y > 65535u) return cudaErrorInvalidConfiguration;
    const cudaError_t e = by_real(dst_real, [&](auto t) {
      using D = decltype(t);
      import_transpose_kernel<D><<<grid, block, 0, st>>>((D*)dst, (const double2*)src, g.sshape[1], g.sshape[0]);
      return cudaGetLastError();
    });
    count_launch();
    return e;
  }
  const Perm P = make_perm(g);
  const cudaError_t e = by_real(dst_real, [&](auto t) {
    using D = decltype(t);
    import_kernel<D><<<blocks_for(total), 256, 0, st>>>((D*)dst, (const double2*)src, P, total);
    return cudaGetLastError();
  });
  count_launch();
  return e;
}

cudaError_t launch_export(double* dst, const void* src, int src_real, const Geometry& g, cudaStream_t st) {
  const int64_t total = total_of(g);
  if (layout_is_transpose2(g)) {
    const dim3 grid = transpose_grid(g), block(kTT, 8);
    if (grid.y > 65535u) return cudaErrorInvalidConfiguration;
    const cudaError_t e = by_real(src_real, [&](auto t) {
      using S = decltype(t);
      export_transpose_kernel<S><<<grid, block, 0, st>>>((double2*)dst, (const S*)src, g.sshape[1], g.sshape[0]);
      return cudaGetLastError();
    });
    count_launch();
    return e;
  }
  const Perm P = make_perm(g);
  const cudaError_t e = by_real(src_real, [&](auto t) {
    using S = decltype(t);
    export_kernel<S><<<blocks_for(total), 256, 0, st>>>((double2*)dst, (const S*)src, P, total);
    return cudaGetLastError();
  });
  count_launch();
  return e;
}

cudaError_t launch_density(double* dst, const void* src, int real, const Geometry& g, cudaStream_t st) {
  const int64_t total = total_of(g);
  const Perm P = make_perm(g);
  const cudaError_t e = by_real(real, [&](auto t) {
    using S = decltype(t);
    density_kernel<S><<<blocks_for(total), 256, 0, st>>>(dst, (const S*)src, P, total);
    return cudaGetLastError();
  });
  count_launch();
  return e;
}

// state_density: out[i] = sum over all other axes of |psi|^2 prod_a w_a (wave_function.rs:121-148).
// One block per index of `axis`; fixed-order block tree.
struct WPtrs {
  const double* w[kMaxDims];
};

template <typename S>
__global__ void state_density_kernel(double* dst, const S* src, Perm P, int axis, WPtrs W, int64_t total) {
  __shared__ double scratch[32];
  const int64_t i = blockIdx.x;
  // storage position of `axis`
  int qa = 0;
  for (int q = 0; q < P.nd; ++q)
    if (P.perm[q] == axis) qa = q;
  int64_t after = 1;
  for (int q = qa + 1; q < P.nd; ++q) after *= P.sshape[q];
  const int64_t na = P.sshape[qa];
  const int64_t rest = total / na;
  double acc = 0.0;
  for (int64_t r = threadIdx.x; r < rest; r += blockDim.x) {
    const int64_t hi = r / after, lo = r - hi * after;
    int64_t s = (hi * na + i) * after + lo;
    const S v = src[s];
    double w = 1.0;
    int64_t t = s;
    for (int q = P.nd - 1; q >= 0; --q) {
      const int64_t c = t % P.sshape[q];
      t /= P.sshape[q];
      w *= W.w[P.perm[q]][c];
    }
    acc += ((double)v.x * (double)v.x + (double)v.y * (double)v.y) * w;
  }
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, off);
  if ((threadIdx.x & 31) == 0) scratch[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    double s = 0.0;
    for (int k = 0; k < (int)(blockDim.x >> 5); ++k) s += scratch[k];
    dst[i] = s;
  }
}

cudaError_t launch_state_density(double* dst, const void* src, int real, const Geometry& g, int axis,
                                 const double* const* w, double* /*partials*/, cudaStream_t st) {
  const int64_t total = total_of(g);
  const Perm P = make_perm(g);
  WPtrs W{};
  for (int a = 0; a < g.ndim; ++a) W.w[a] = w[a];
  int64_t na = 1;
  for (int q = 0; q < g.ndim; ++q)
    if (g.perm[q] == axis) na = g.sshape[q];
  const cudaError_t e = by_real(real, [&](auto t) {
    using S = decltype(t);
    state_density_kernel<S><<<(unsigned)na, 256, 0, st>>>(dst, (const S*)src, P, axis, W, total);
    return cudaGetLastError();
  });
  count_launch();
  return e;
}

template <typename D, typename S>
__global__ void convert_kernel(D* dst, const S* src, int64_t n) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    dst[i] = D{(decltype(dst->x))src[i].x, (decltype(dst->x))src[i].y};
}

cudaError_t launch_copy_convert(void* dst, int dst_real, const void* src, int src_real, int64_t n,
                                cudaStream_t st) {
  const cudaError_t e = by_real(dst_real, [&](auto td) {
    return by_real(src_real, [&](auto ts) {
      using D = decltype(td);
      using S = decltype(ts);
      convert_kernel<D, S><<<blocks_for(n), 256, 0, st>>>((D*)dst, (const S*)src, n);
      return cudaGetLastError();
    });
  });
  count_launch();
  return e;
}

__global__ void table_convert_kernel(float* dst, const double* src, int64_t n) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    dst[i] = (float)src[i];
}

cudaError_t launch_table_convert(void* dst, bool dst_fp64, const double* src_dev, int64_t count, cudaStream_t st) {
  if (dst_fp64) return cudaMemcpyAsync(dst, src_dev, count * sizeof(double), cudaMemcpyDeviceToDevice, st);
  table_convert_kernel<<<blocks_for(count), 256, 0, st>>>((float*)dst, src_dev, count);
  count_launch();
  return cudaGetLastError();
}

}  // namespace so
