// Lane-sweep pass kernel: one CTA owns a tile of complete lanes along the pass's
// sweep axis in shared memory and runs the pass program on it.
//
// Replaces, fused into single passes, the reference's per-operator full-array
// sweeps: OneDimPropagator::apply (one_dim_propagator.rs:37-46),
// NDimPropagator::apply (n_dim_propagator.rs:32-36), FFTTransformation
// (fft_transformation.rs:53-88), MatrixTransformation (matrix_transformation.rs:60-75),
// NonDiagPropagator (non_diagonal_propagator.rs:29-37), StateMatrixTransformation
// (state_matrix_transformation.rs:48-73) and the norm folds of WaveFunction::norm
// (wave_function.rs:68-85) used by LossChecker / LeakControl.
//
// State precisions: FP32 (float2), FP64 (double2) and float-float (ffc, ff.cuh: FP64's
// kernels with float-float arithmetic).
// FFT: Stockham autosort between two shared-memory buffers (radix 8 stages for FP64 and
// float-float, radix 16 for FP32, one smaller closing stage), register butterflies,
// twiddles from an FP64-built table, the 1/sqrt(N) of the reference folded into the last
// stage.
// Lanes shorter than 16 or of non power-of-two length use a direct DFT with the natural
// table.  The lane matrix product also writes into the second buffer.
// Norms: per-thread sums (FP32 in FP32 passes, FP64 in FP64 ones), fixed-order warp/block
// trees, per-CTA partials folded by the last CTA in a fixed order, so results do not
// depend on scheduling.
// The radial pass of the 2-D step ([FFT] [point-wise] [FFT] [point-wise] on contiguous
// power-of-two FP32 lanes) runs the separate register-resident FFT-pair kernel below.
#include <cstdio>
#include <type_traits>

#include "common.cuh"
#include "ff.cuh"

namespace so {

template <typename R>
struct Cx;
template <>
struct Cx<double> {
  using T = double2;
};
template <>
struct Cx<float> {
  using T = float2;
};
template <>
struct Cx<ff> {
  using T = ffc;
};

template <typename R>
constexpr bool kIsFF = std::is_same<R, ff>::value;

// read-only cached load of a state-precision value
template <typename T>
__device__ __forceinline__ T ldg_(const T* p) {
  if constexpr (std::is_same<T, ff>::value || std::is_same<T, ffc>::value)
    return ldg_ff(p);
  else
    return __ldg(p);
}

template <typename C>
__device__ __forceinline__ C cmul(C a, C b) {
  return {a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x};
}
template <typename C>
__device__ __forceinline__ C cadd(C a, C b) {
  return {a.x + b.x, a.y + b.y};
}
template <typename C>
__device__ __forceinline__ C csub(C a, C b) {
  return {a.x - b.x, a.y - b.y};
}
// multiply by s*i (s = +1 or -1)
template <typename C>
__device__ __forceinline__ C mul_si(C a, int s) {
  return s > 0 ? C{-a.y, a.x} : C{a.y, -a.x};
}

__device__ __forceinline__ int sidx(int l, int j, int ls) { return l * ls + j + (j >> 4); }

// ---------------------------------------------------------------- butterflies
template <typename C>
__device__ __forceinline__ void dft2(C& a0, C& a1) {
  C t = a0;
  a0 = cadd(t, a1);
  a1 = csub(t, a1);
}

template <typename C>
__device__ __forceinline__ void dft4(C& a0, C& a1, C& a2, C& a3, int s) {
  C e0 = cadd(a0, a2), e1 = csub(a0, a2);
  C o0 = cadd(a1, a3), o1 = mul_si(csub(a1, a3), s);
  a0 = cadd(e0, o0);
  a2 = csub(e0, o0);
  a1 = cadd(e1, o1);
  a3 = csub(e1, o1);
}

// The rotation constants of the radix-8/16 butterflies, as FP64 values and, for the
// FP32 path, as hi + lo pairs: a single rounded FP32 constant has |e^{i phi}| != 1 by
// a fixed amount, and since every butterfly reuses the same few constants that error
// would shrink (or grow) the norm systematically, stage after stage.
constexpr double kC1 = 0.92387953251128675613;  // cos(pi/8)
constexpr double kC2 = 0.70710678118654752440;  // cos(pi/4)
constexpr double kC3 = 0.38268343236508977173;  // sin(pi/8)

template <typename R>
struct RotConst {
  R hi, lo;
};
// FP32: hi = the constant rounded to FP32, lo = the FP32 rounding of the remainder
// (literal values, so no FP64 arithmetic runs per butterfly); FP64: the constant itself
template <typename R>
__device__ __forceinline__ RotConst<R> rot_const(int which) {
  if constexpr (sizeof(R) == 4) {
    constexpr float hi[3] = {0x1.d906bcp-1f, 0x1.6a09e6p-1f, 0x1.87de2ap-2f};
    constexpr float lo[3] = {0x1.e651a8p-26f, 0x1.9fcef4p-27f, 0x1.abaa58p-28f};
    return {hi[which], lo[which]};
  } else {
    constexpr double v[3] = {kC1, kC2, kC3};
    return {v[which], 0.0};
  }
}
// fused multiply-add in the state precision
template <typename R>
__device__ __forceinline__ R fmar(R a, R b, R c) {
  if constexpr (kIsFF<R>)
    return a * b + c;
  else if constexpr (sizeof(R) == 4)
    return fmaf(a, b, c);
  else
    return fma(a, b, c);
}
// x * c with the constant carried as hi + lo
template <typename R>
__device__ __forceinline__ R mulc(R x, RotConst<R> c) {
  if constexpr (sizeof(R) == 4)
    return fmaf(x, c.hi, x * c.lo);
  else
    return x * c.hi;
}

template <typename C>
__device__ __forceinline__ void dft8(C* a, int s) {
  using R = decltype(a[0].x);
  const RotConst<R> h = rot_const<R>(1);
  C e0 = a[0], e1 = a[2], e2 = a[4], e3 = a[6];
  C o0 = a[1], o1 = a[3], o2 = a[5], o3 = a[7];
  dft4(e0, e1, e2, e3, s);
  dft4(o0, o1, o2, o3, s);
  // o_q *= w8^q, w8 = e^{s 2 pi i / 8}
  o1 = C{mulc<R>(o1.x - s * o1.y, h), mulc<R>(s * o1.x + o1.y, h)};
  o2 = mul_si(o2, s);
  o3 = C{mulc<R>(-o3.x - s * o3.y, h), mulc<R>(s * o3.x - o3.y, h)};
  a[0] = cadd(e0, o0);
  a[4] = csub(e0, o0);
  a[1] = cadd(e1, o1);
  a[5] = csub(e1, o1);
  a[2] = cadd(e2, o2);
  a[6] = csub(e2, o2);
  a[3] = cadd(e3, o3);
  a[7] = csub(e3, o3);
}

template <typename C>
__device__ __forceinline__ void dft16(C* a, int s) {
  using R = decltype(a[0].x);
  C e[8], o[8];
#pragma unroll
  for (int q = 0; q < 8; ++q) {
    e[q] = a[2 * q];
    o[q] = a[2 * q + 1];
  }
  dft8(e, s);
  dft8(o, s);
  // o_q *= w16^q = (cos(q pi/8), s sin(q pi/8)): q = 4 is (0, s); the others use the
  // hi + lo constants (c x - s' y with both products corrected)
  const RotConst<R> c1 = rot_const<R>(0), c2 = rot_const<R>(1), c3 = rot_const<R>(2);
  const RotConst<R> cs[8] = {{(R)1, (R)0}, c1, c2, c3, {(R)0, (R)0}, {-c3.hi, -c3.lo}, {-c2.hi, -c2.lo},
                             {-c1.hi, -c1.lo}};
  const RotConst<R> sn[8] = {{(R)0, (R)0}, c3, c2, c1, {(R)1, (R)0}, c1, c2, c3};
#pragma unroll
  for (int q = 1; q < 8; ++q) {
    if (q == 4) {
      o[q] = mul_si(o[q], s);
      continue;
    }
    const C x = o[q];
    const R ys = (R)s * x.y, xs = (R)s * x.x;
    // (c x - s' y, s' x + c y) with the lo parts of c and s' folded in first
    const R re = fmar(x.x, cs[q].hi, fmar(-ys, sn[q].hi, x.x * cs[q].lo - ys * sn[q].lo));
    const R im = fmar(xs, sn[q].hi, fmar(x.y, cs[q].hi, xs * sn[q].lo + x.y * cs[q].lo));
    o[q] = C{re, im};
  }
#pragma unroll
  for (int q = 0; q < 8; ++q) {
    a[q] = cadd(e[q], o[q]);
    a[q + 8] = csub(e[q], o[q]);
  }
}

template <int RS, typename C>
__device__ __forceinline__ void dft_r(C* a, int s) {
  if constexpr (RS == 2) {
    dft2(a[0], a[1]);
  } else if constexpr (RS == 4) {
    dft4(a[0], a[1], a[2], a[3], s);
  } else if constexpr (RS == 8) {
    dft8(a, s);
  } else {
    dft16(a, s);
  }
}

// One Stockham stage of radix RS from src to dst (ping-pong buffers): each
// thread walks its butterflies one at a time, so it holds RS values at most.
template <int RS, typename C, typename R>
__device__ __forceinline__ void stockham_stage(const C* __restrict__ src, C* __restrict__ dst, int L, int n, int ls,
                                               int p, int dir, const C* __restrict__ tw, bool last, R sc) {
  const int nb = n / RS;
  const int total = L * nb;
  for (int b = threadIdx.x; b < total; b += blockDim.x) {
    const int l = b / nb, i = b - l * nb;
    const int k = i & (p - 1);
    C reg[RS];
#pragma unroll
    for (int r = 0; r < RS; ++r) {
      C x = src[sidx(l, i + r * nb, ls)];
      if (r > 0 && k > 0) {
        C w = tw[(r - 1) * p + k];  // this stage's part of the shared-memory table
        if (dir > 0) w.y = -w.y;
        x = cmul(x, w);
      }
      reg[r] = x;
    }
    dft_r<RS>(reg, dir);
    const int base = (i - k) * RS + k;
#pragma unroll
    for (int q = 0; q < RS; ++q) {
      C v = reg[q];
      if (last) v = C{v.x * sc, v.y * sc};
      dst[sidx(l, base + q * p, ls)] = v;
    }
  }
  __syncthreads();
}

// 1 / sqrt(2^lg) in the state precision: a power of two, times 1/sqrt(2) for odd lg
// (no FP64 division or square root per thread: both are long sequences on this GPU)
template <typename R>
__device__ __forceinline__ R inv_sqrt_pow2(int lg) {
  R s = (R)1;
  for (int k = 0; k < lg / 2; ++k) s *= (R)0.5;
  return (lg & 1) ? s * (R)0.70710678118654752440 : s;
}

// Unitary DFT of every lane of the tile (radix RMAX stages, then one smaller
// stage); the result ends in `alt`, and the two buffer pointers are swapped.
template <int RMAX, typename C>
__device__ void fft_stockham(C*& buf, C*& alt, const Geometry& g, int dir, const C* __restrict__ tw) {
  using R = decltype(buf[0].x);
  const int n = (int)g.n, L = g.lanes_per_tile, ls = g.lane_stride;
  const R scale = inv_sqrt_pow2<R>(__ffs(n) - 1);
  int p = 1, off = 0;  // off: the stage's first entry in the stage-major table
  while (p < n) {
    const int rem = n / p;
    const C* ts = tw + off;
    int rs;
    if (rem >= RMAX) {
      stockham_stage<RMAX>(buf, alt, L, n, ls, p, dir, ts, rem == RMAX, scale);
      rs = RMAX;
    } else if (rem == 8) {
      stockham_stage<8>(buf, alt, L, n, ls, p, dir, ts, true, scale);
      rs = 8;
    } else if (rem == 4) {
      stockham_stage<4>(buf, alt, L, n, ls, p, dir, ts, true, scale);
      rs = 4;
    } else {
      stockham_stage<2>(buf, alt, L, n, ls, p, dir, ts, true, scale);
      rs = 2;
    }
    if (p > 1) off += (rs - 1) * p;
    p *= rs;
    C* t = buf;
    buf = alt;
    alt = t;
  }
}

// Direct DFT for short or non power-of-two lanes: out_j = scale sum_k x_k w^{jk}.
template <typename C>
__device__ void dft_direct(C*& buf, C*& alt, const Geometry& g, int dir, const C* __restrict__ tw) {
  using R = decltype(buf[0].x);
  const int n = (int)g.n, L = g.lanes_per_tile, ls = g.lane_stride;
  const int total = L * n;
  const R sc = (R)(1.0 / sqrt((double)n));
  for (int o = threadIdx.x; o < total; o += blockDim.x) {
    const int l = o / n, j = o - l * n;
    C s = C{(R)0, (R)0};
    for (int k = 0; k < n; ++k) {
      C w = tw[(int)(((int64_t)j * k) % n)];
      if (dir > 0) w.y = -w.y;
      s = cadd(s, cmul(buf[sidx(l, k, ls)], w));
    }
    alt[sidx(l, j, ls)] = C{s.x * sc, s.y * sc};
  }
  __syncthreads();
  C* t = buf;
  buf = alt;
  alt = t;
}

// Float-float lane <- M lane for a real matrix with the parity structure of a Legendre
// pair (flags bits 1-2; the matrix in op.ptr is then the half matrix H, h = n / 2):
//   kind 1, M[a][n-1-b] = (-1)^a M[a][b] (a transform with quadrature weights):
//     out_a = sum_{b<h} H[a][b] (x_b + (-1)^a x_{n-1-b}),   H stored HT[b n + a];
//   kind 2, M[n-1-b][a] = (-1)^a M[b][a] (its inverse): with E_b / O_b the sums over the
//     even / odd a of H[b][a] x_a, out_b = E_b + O_b and out_{n-1-b} = E_b - O_b,
//     H stored HT[a h + b].
// Half the products of the plain form.  The result ends in buf (the pointers swap for kind 2).
template <typename C>
__device__ void mat_apply_parity_ff(C*& buf, C*& alt, const Geometry& g, const DevOp& op, int kind) {
  const int n = (int)g.n, L = g.lanes_per_tile, ls = g.lane_stride, h = n / 2;
  const ff* ht = reinterpret_cast<const ff*>(op.ptr);
  if (kind == 1) {
    // S_b = x_b + x_{n-1-b} and D_b = x_b - x_{n-1-b} into alt (S at b, D at h + b)
    for (int o = threadIdx.x; o < L * h; o += blockDim.x) {
      const int l = o / h, b = o - l * h;
      const C x0 = buf[sidx(l, b, ls)], x1 = buf[sidx(l, n - 1 - b, ls)];
      alt[sidx(l, b, ls)] = cadd(x0, x1);
      alt[sidx(l, h + b, ls)] = csub(x0, x1);
    }
    __syncthreads();
    for (int o = threadIdx.x; o < L * n; o += blockDim.x) {
      const int l = o / n, a = o - l * n, off = (a & 1) ? h : 0;
      FfDot sr, si;
      for (int b = 0; b < h; ++b) {
        const ff m = ldg_ff(ht + (int64_t)b * n + a);
        const C x = alt[sidx(l, off + b, ls)];
        sr.add(m, x.x);
        si.add(m, x.y);
      }
      buf[sidx(l, a, ls)] = C{sr.value(), si.value()};
    }
  } else {
    for (int o = threadIdx.x; o < L * h; o += blockDim.x) {
      const int l = o / h, b = o - l * h;
      FfDot er, ei, orr, oi;
      for (int a = 0; a < n; a += 2) {
        const ff me = ldg_ff(ht + (int64_t)a * h + b), mo = ldg_ff(ht + (int64_t)(a + 1) * h + b);
        const C xe = buf[sidx(l, a, ls)], xo = buf[sidx(l, a + 1, ls)];
        er.add(me, xe.x);
        ei.add(me, xe.y);
        orr.add(mo, xo.x);
        oi.add(mo, xo.y);
      }
      const ff e_r = er.value(), e_i = ei.value(), o_r = orr.value(), o_i = oi.value();
      alt[sidx(l, b, ls)] = C{e_r + o_r, e_i + o_i};
      alt[sidx(l, n - 1 - b, ls)] = C{e_r - o_r, e_i - o_i};
    }
    C* t = buf;
    buf = alt;
    alt = t;
  }
  __syncthreads();
}

// lane <- M lane.  Matrices are stored transposed (MT[k*n + j] = M[j][k]) so that
// threads with consecutive j read consecutive addresses; real matrices store one
// real per entry.  `sel` picks the matrix of a lane (-1: leave the lane as it is).
template <typename C>
__device__ void mat_apply(C*& buf, C*& alt, const Geometry& g, const DevOp& op, const int* lane_sel) {
  using R = decltype(buf[0].x);
  if constexpr (kIsFF<R>) {
    const int par = (op.flags >> 1) & 3;
    if (par && !lane_sel) {
      mat_apply_parity_ff(buf, alt, g, op, par);
      return;
    }
  }
  const int n = (int)g.n, L = g.lanes_per_tile, ls = g.lane_stride;
  const int total = L * n;
  const bool real = op.flags & 1;
  for (int o = threadIdx.x; o < total; o += blockDim.x) {
    const int l = o / n, j = o - l * n;
    const int sel = lane_sel ? lane_sel[l] : 0;
    C res;
    if (sel < 0) {
      res = buf[sidx(l, j, ls)];
    } else if (real) {
      const R* mt = reinterpret_cast<const R*>(op.ptr) + (int64_t)sel * n * n;
      if constexpr (kIsFF<R>) {
        // float-float: compensated dot products (FfDot)
        FfDot sr, si;
        for (int k = 0; k < n; ++k) {
          const R m = ldg_(mt + (int64_t)k * n + j);
          const C x = buf[sidx(l, k, ls)];
          sr.add(m, x.x);
          si.add(m, x.y);
        }
        res = C{sr.value(), si.value()};
      } else {
        R sr = 0, si = 0;
        for (int k = 0; k < n; ++k) {
          const R m = __ldg(mt + (int64_t)k * n + j);
          const C x = buf[sidx(l, k, ls)];
          sr += m * x.x;
          si += m * x.y;
        }
        res = C{sr, si};
      }
    } else {
      const C* mt = reinterpret_cast<const C*>(op.ptr) + (int64_t)sel * n * n;
      C s = C{(R)0, (R)0};
      for (int k = 0; k < n; ++k) {
        const C m = mt[(int64_t)k * n + j];
        s = cadd(s, cmul(m, buf[sidx(l, k, ls)]));
      }
      res = s;
    }
    alt[sidx(l, j, ls)] = res;
  }
  __syncthreads();
  C* t = buf;
  buf = alt;
  alt = t;
}

// Fixed-order block sum of one double per thread; result valid in thread 0.
__device__ double block_sum(double v, double* scratch) {
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) v += __shfl_down_sync(0xffffffffu, v, off);
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (lane == 0) scratch[w] = v;
  __syncthreads();
  double r = 0.0;
  if (threadIdx.x == 0) {
    const int nw = (blockDim.x + 31) >> 5;
    for (int i = 0; i < nw; ++i) r += scratch[i];
  }
  __syncthreads();
  return r;
}

__device__ __forceinline__ double ld_slot(const double* s, int i) { return __ldcg(s + i); }

// scalar bookkeeping of one op, run by a single thread
__device__ void run_scalar(const PassParams& p, const DevOp& op, const double* totals) {
  double* s = p.slots;
  switch (op.kind) {
    case OP_NORM: {
      const double v = totals[op.red];
      s[op.a] = v;
      if (!isfinite(v) && p.nonfinite_slot >= 0) s[p.nonfinite_slot] = 1.0;
      break;
    }
    case OP_DOT:
      s[op.a] = totals[op.red];
      s[op.b] = totals[op.red + 1];
      break;
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

// global loads a thread keeps in flight in the load and table phases of a pass
// (64 bytes: 8 FP32 or 4 FP64 complex values)
template <typename C>
__host__ __device__ constexpr int load_batch() { return 64 / (int)sizeof(C); }

// SWEEP: the pass has only point-wise ops, norms, scalar bookkeeping and power-of-two FFTs
// (16 or more points): the lane-matrix, direct-DFT and overlap paths are compiled out,
// which keeps the kernel small (instruction-cache misses stalled the general interpreter).
template <typename R, int RMAX, bool SWEEP>
__device__ __forceinline__ void pass_tile(const PassParams& p, const int64_t tile) {
  using C = typename Cx<R>::T;
  constexpr bool kF64 = sizeof(R) == 8;
  constexpr int kLoadBatch = load_batch<C>();
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const Geometry& g = p.g;
  const int L = g.lanes_per_tile, n = (int)g.n, ls = g.lane_stride;
  const int T = blockDim.x, tid = threadIdx.x;
  const size_t tile_bytes = ((size_t)L * ls * sizeof(C) + 15) & ~(size_t)15;
  C* buf = reinterpret_cast<C*>(smem_raw);
  C* alt = p.one_buffer ? nullptr : reinterpret_cast<C*>(smem_raw + tile_bytes);
  size_t off = (p.one_buffer ? 1 : 2) * tile_bytes;
  int64_t* lane_base = reinterpret_cast<int64_t*>(smem_raw + off);
  off += (size_t)L * sizeof(int64_t);
  double* lane_w = reinterpret_cast<double*>(smem_raw + off);
  off += (size_t)L * sizeof(double);
  int* lane_coord = reinterpret_cast<int*>(smem_raw + off);
  off += (size_t)L * kMaxDims * sizeof(int);
  int* lane_sel = reinterpret_cast<int*>(smem_raw + off);
  off += (size_t)L * sizeof(int);
  off = (off + 15) & ~(size_t)15;
  C* tw_s = reinterpret_cast<C*>(smem_raw + off);  // the lane's twiddles (passes with an FFT)
  __shared__ double scratch[32];
  __shared__ double blk_red[kMaxRed];
  __shared__ double totals[kMaxRed];
  __shared__ double scale_s;
  __shared__ int s_last;

  const bool pow2 = (n & (n - 1)) == 0;
  const int lg = pow2 ? __ffs(n) - 1 : 0;

  // lane metadata
  for (int l = tid; l < L; l += T) {
    int64_t o, i;
    bool valid;
    if (g.inner == 1) {
      o = tile * L + l;
      i = 0;
      valid = o < g.outer;
    } else {
      o = tile / g.tiles_per_outer;
      i = (tile - o * g.tiles_per_outer) * L + l;
      valid = (o < g.outer) && (i < g.inner);
    }
    lane_base[l] = valid ? o * g.n * g.inner + i : -1;
    int64_t ro = valid ? o : 0, ri = valid ? i : 0;
    for (int q = g.ndim - 1; q > g.spos; --q) {
      lane_coord[l * kMaxDims + g.perm[q]] = (int)(ri % g.sshape[q]);
      ri /= g.sshape[q];
    }
    for (int q = g.spos - 1; q >= 0; --q) {
      lane_coord[l * kMaxDims + g.perm[q]] = (int)(ro % g.sshape[q]);
      ro /= g.sshape[q];
    }
    lane_coord[l * kMaxDims + g.sweep_axis] = 0;
  }
  __syncthreads();

  auto split = [&](int pt, int& l, int& x) {
    if (g.inner == 1) {
      l = pow2 ? (pt >> lg) : pt / n;
      x = pt - l * n;
    } else {
      x = pt / L;
      l = pt - x * L;
    }
  };

  C* psi = reinterpret_cast<C*>(p.psi);
  const int total = L * n;
  // kLoadBatch independent global loads in flight per thread, then the shared stores
  for (int p0 = tid; p0 < total; p0 += kLoadBatch * T) {
    C v[kLoadBatch];
#pragma unroll
    for (int u = 0; u < kLoadBatch; ++u) {
      const int pt = p0 + u * T;
      v[u] = C{(R)0, (R)0};
      if (pt < total) {
        int l, x;
        split(pt, l, x);
        const int64_t b = lane_base[l];
        if (b >= 0) v[u] = psi[b + (int64_t)x * g.inner];
      }
    }
#pragma unroll
    for (int u = 0; u < kLoadBatch; ++u) {
      const int pt = p0 + u * T;
      if (pt < total) {
        int l, x;
        split(pt, l, x);
        buf[sidx(l, x, ls)] = v[u];
      }
    }
  }
  // twiddles in shared memory (stage-major for the Stockham stages: consecutive reads), or
  // read from the cached global table when the tile has few lanes
  const C* tw = reinterpret_cast<const C*>(p.twiddle);
  if (tw && twiddles_in_smem(g)) {
    for (int k = tid; k < n; k += T) tw_s[k] = tw[k];
    tw = tw_s;
  }
  __syncthreads();
  for (int rep = 0; rep < p.repeat; ++rep) {
    for (int oi = 0; oi < p.nops; ++oi) {
      const DevOp& op = p.ops[oi];
      switch (op.kind) {
        case OP_DIAG1D: {
          const C* t = reinterpret_cast<const C*>(op.ptr);
          const bool along = op.axis == g.sweep_axis;
          for (int pt = tid; pt < total; pt += T) {
            const int l = pow2 ? (pt >> lg) : pt / n, x = pt - l * n;
            const int k = along ? x : lane_coord[l * kMaxDims + op.axis];
            const int si = sidx(l, x, ls);
            buf[si] = cmul(buf[si], ldg_(reinterpret_cast<const typename Cx<R>::T*>(t) + k));
          }
          __syncthreads();
          break;
        }
        case OP_DIAGND: {
          const C* t = reinterpret_cast<const C*>(op.ptr);
          for (int p0 = tid; p0 < total; p0 += kLoadBatch * T) {
            C tv[kLoadBatch];
#pragma unroll
            for (int u = 0; u < kLoadBatch; ++u) {
              const int pt = p0 + u * T;
              tv[u] = C{(R)1, (R)0};
              if (pt < total) {
                int l, x;
                split(pt, l, x);
                const int64_t b = lane_base[l];
                if (b >= 0) tv[u] = t[b + (int64_t)x * g.inner];
              }
            }
#pragma unroll
            for (int u = 0; u < kLoadBatch; ++u) {
              const int pt = p0 + u * T;
              if (pt < total) {
                int l, x;
                split(pt, l, x);
                const int si = sidx(l, x, ls);
                buf[si] = cmul(buf[si], tv[u]);
              }
            }
          }
          __syncthreads();
          break;
        }
        case OP_SCALE: {
          // one thread forms sqrt(target / norm) in FP64, the block reads it back
          if (tid == 0) {
            // FP32 uses the factor rounded to FP32; FP64 and float-float the FP64 value
            const double f = sqrt(ld_slot(p.slots, op.b) / ld_slot(p.slots, op.c));
            if constexpr (sizeof(R) == 4)
              scale_s = (double)(float)f;
            else
              scale_s = f;
          }
          __syncthreads();
          const R fr = (R)scale_s;
          for (int pt = tid; pt < total; pt += T) {
            const int l = pow2 ? (pt >> lg) : pt / n, x = pt - l * n;
            const int si = sidx(l, x, ls);
            buf[si] = C{buf[si].x * fr, buf[si].y * fr};
          }
          __syncthreads();
          break;
        }
        case OP_FFT:
          if (SWEEP || (pow2 && n >= 16))
            fft_stockham<RMAX>(buf, alt, g, op.dir, tw);
          else if constexpr (!SWEEP)
            dft_direct(buf, alt, g, op.dir, tw);
          break;
        case OP_MAT:
          if constexpr (!SWEEP) mat_apply(buf, alt, g, op, nullptr);
          break;
        case OP_MAT_LANE:
        case OP_MAT_SLICE: {
          if constexpr (!SWEEP) {
          for (int l = tid; l < L; l += T) {
            int64_t idx;
            if (op.kind == OP_MAT_SLICE) {
              idx = lane_coord[l * kMaxDims + op.axis];
            } else {
              // ndarray lanes_mut order: row-major over the logical axes other than the sweep axis
              idx = 0;
              for (int a = 0; a < g.ndim; ++a) {
                if (a == g.sweep_axis) continue;
                int64_t ext = 0;
                for (int q = 0; q < g.ndim; ++q)
                  if (g.perm[q] == a) ext = g.sshape[q];
                idx = idx * ext + lane_coord[l * kMaxDims + a];
              }
            }
            lane_sel[l] = (lane_base[l] >= 0 && idx < op.count) ? (int)idx : -1;
          }
          __syncthreads();
          mat_apply(buf, alt, g, op, lane_sel);
          }
          break;
        }
        case OP_NORM:
        case OP_DOT: {
          const bool f32_norm = !kF64 && op.kind == OP_NORM;
          float* lane_wf = reinterpret_cast<float*>(lane_w);  // FP32 lane weights share the space
          for (int l = tid; l < L; l += T) {
            if (f32_norm) {
              float w = 0.0f;
              if (lane_base[l] >= 0) {
                w = 1.0f;
                for (int a = 0; a < g.ndim; ++a)
                  if (a != g.sweep_axis) w *= op.wf[a][lane_coord[l * kMaxDims + a]];
              }
              lane_wf[l] = w;
              continue;
            }
            double w = 1.0;
            if (lane_base[l] < 0) {
              w = 0.0;
            } else {
              for (int a = 0; a < g.ndim; ++a)
                if (a != g.sweep_axis) w *= op.w[a][lane_coord[l * kMaxDims + a]];
            }
            lane_w[l] = w;
          }
          __syncthreads();
          const double* wx = op.w[g.sweep_axis];
          double acc = 0.0, acc_i = 0.0;
          const C* other = reinterpret_cast<const C*>(op.ptr);
          if (f32_norm) {
            // FP32 state: FP32 products and per-thread partial sum, folded in FP64 once
            const float* wxf = op.wf[g.sweep_axis];
            float part = 0.0f;
            for (int pt = tid; pt < total; pt += T) {
              int l, x;
              split(pt, l, x);
              const C v = buf[sidx(l, x, ls)];
              const float w = lane_wf[l] * __ldg(wxf + x);
              part = fmaf(fmaf((float)v.x, (float)v.x, (float)v.y * (float)v.y), w, part);
            }
            acc = (double)part;
          }
          for (int pt = tid; pt < total && !f32_norm; pt += T) {
            int l, x;
            split(pt, l, x);
            const C v = buf[sidx(l, x, ls)];
            const double w = lane_w[l] * __ldg(wx + x);
            if (op.kind == OP_NORM) {
              acc += ((double)v.x * (double)v.x + (double)v.y * (double)v.y) * w;
            } else if (lane_base[l] >= 0) {
              const C o = other[lane_base[l] + (int64_t)x * g.inner];
              // v * conj(o)
              acc += ((double)v.x * (double)o.x + (double)v.y * (double)o.y) * w;
              acc_i += ((double)v.y * (double)o.x - (double)v.x * (double)o.y) * w;
            }
          }
          const double tsum = block_sum(acc, scratch);
          double tsum_i = 0.0;
          if (op.kind == OP_DOT) tsum_i = block_sum(acc_i, scratch);
          if (tid == 0) {
            if (p.resident) {
              totals[op.red] = tsum;
              if (op.kind == OP_DOT) totals[op.red + 1] = tsum_i;
              run_scalar(p, op, totals);
            } else {
              blk_red[op.red] = tsum;
              if (op.kind == OP_DOT) blk_red[op.red + 1] = tsum_i;
            }
          }
          __syncthreads();
          break;
        }
        default:  // COPY / LOSS / SETC / RECORD
          if (p.resident) {
            if (tid == 0) run_scalar(p, op, totals);
            __syncthreads();
          }
          break;
      }
    }
  }

  for (int pt = tid; pt < total; pt += T) {
    int l, x;
    split(pt, l, x);
    const int64_t b = lane_base[l];
    if (b >= 0) psi[b + (int64_t)x * g.inner] = buf[sidx(l, x, ls)];
  }
  if (p.resident) return;

  // ---- deterministic finalize by the last CTA
  if (p.nred == 0 && p.nops == 0) return;
  __syncthreads();
  if (tid == 0) {
    for (int r = 0; r < p.nred; ++r) p.partials[(int64_t)r * g.tiles + tile] = blk_red[r];
    __threadfence();
    const unsigned int ticket = atomicAdd(p.counter, 1u);
    s_last = ticket == (unsigned int)(g.tiles - 1);
  }
  __syncthreads();
  if (!s_last) return;
  __threadfence();
  const int w = tid >> 5, lane = tid & 31;
  for (int r = w; r < p.nred; r += (T >> 5)) {
    double v = 0.0;
    for (int64_t b = lane; b < g.tiles; b += 32) v += __ldcg(p.partials + (int64_t)r * g.tiles + b);
#pragma unroll
    for (int o2 = 16; o2 > 0; o2 >>= 1) v += __shfl_down_sync(0xffffffffu, v, o2);
    if (lane == 0) totals[r] = v;
  }
  __syncthreads();
  if (tid == 0) {
    for (int oi = 0; oi < p.nops; ++oi) run_scalar(p, p.ops[oi], totals);
    __threadfence();
    *p.counter = 0u;
  }
}

// ------------------------------------------------------------------ FFT pair pass
// [FFT] [point-wise ops] [FFT] [point-wise ops] over L contiguous FP32 lanes of n points
// (power of two, 16 .. 8192): the 2-D step's radial pass (F, K, F^-1, Rot/2).  Every
// thread holds kPairV = 16 values (L n = 16 T) and runs 16 / RS butterflies of each
// radix-RS stage, b = t + j T, so a stage can run in place in one shared buffer (read,
// barrier, compute, write, barrier).  The first FFT's first stage (p = 1) reads global
// memory directly, its last stage keeps its outputs in registers (index k + q p_last of
// butterfly k), the point-wise ops between the FFTs run on them, and the second FFT runs
// its radices in the reverse order, so that its first stage's inputs (i + r nb, nb = n /
// RS) are exactly those registers.  Its last stage applies the closing point-wise ops and
// writes global memory directly.  Twiddles come from the stage-major table (forward order
// in [0, n), reversed order in [n, 2n)) through L1.  Compared with the general pass this
// drops the tile load and store through shared memory, the shared-memory round trips of
// both FFTs' outer stages and of the point-wise ops, and the second tile buffer.
constexpr int kPairV = 16;

template <int RS, typename C>
__device__ __forceinline__ void pair_load_smem(C (&v)[kPairV], const C* buf, int t, int T, int lgnb,
                                               int ls) {
  const int nb = 1 << lgnb;
#pragma unroll
  for (int j = 0; j < kPairV / RS; ++j) {
    const int b = t + j * T, l = b >> lgnb, i = b & (nb - 1);
#pragma unroll
    for (int r = 0; r < RS; ++r) v[j * RS + r] = buf[sidx(l, i + r * nb, ls)];
  }
}

template <int RS, typename C>
__device__ __forceinline__ void pair_store_smem(const C (&v)[kPairV], C* buf, int t, int T, int lgnb,
                                                int p, int ls) {
  const int nb = 1 << lgnb;
#pragma unroll
  for (int j = 0; j < kPairV / RS; ++j) {
    const int b = t + j * T, l = b >> lgnb, i = b & (nb - 1), k = i & (p - 1);
    const int base = (i - k) * RS + k;
#pragma unroll
    for (int q = 0; q < RS; ++q) buf[sidx(l, base + q * p, ls)] = v[j * RS + q];
  }
}

// first stage (p = 1) inputs straight from the lanes in global memory (invalid lanes: 0)
// (psi: the tile's first lane; nl: its valid lanes; offsets within a tile fit 32 bits)
template <int RS, typename C>
__device__ __forceinline__ void pair_load_global(C (&v)[kPairV], const C* __restrict__ psi, int t, int T, int lgnb,
                                                 int nl, int n) {
  const int nb = 1 << lgnb;
#pragma unroll
  for (int j = 0; j < kPairV / RS; ++j) {
    const int b = t + j * T, l = b >> lgnb, i = b & (nb - 1);
    const int o = l * n + i;
#pragma unroll
    for (int r = 0; r < RS; ++r) v[j * RS + r] = l < nl ? psi[o + r * nb] : C{0, 0};
  }
}

template <int RS, typename C>
__device__ __forceinline__ void pair_butterflies(C (&v)[kPairV], int t, int T, int lgnb, int p, int dir,
                                                 const C* __restrict__ tw) {
  const int nb = 1 << lgnb;
#pragma unroll
  for (int j = 0; j < kPairV / RS; ++j) {
    const int b = t + j * T, i = b & (nb - 1), k = i & (p - 1);
    if (k > 0) {
#pragma unroll
      for (int r = 1; r < RS; ++r) {
        C w = ldg_(tw + (r - 1) * p + k);
        if (dir > 0) w.y = -w.y;
        v[j * RS + r] = cmul(v[j * RS + r], w);
      }
    }
    dft_r<RS>(&v[j * RS], dir);
  }
}

// point-wise ops [ob, oe) on the outputs of a last stage: value j RS + q sits at lane
// b >> lgnb, point x = k + q p with k = b & (p - 1), p = 2^lgnb
template <int RS, typename C, typename R>
__device__ __forceinline__ void pair_pointwise(C (&v)[kPairV], const PassParams& pp, int ob, int oe, int t, int T,
                                               int lgnb, int64_t lane0, int nl, R sc) {
  const int p = 1 << lgnb, n = (int)pp.g.n;
#pragma unroll
  for (int e = 0; e < kPairV; ++e) v[e] = C{v[e].x * sc, v[e].y * sc};
  for (int oi = ob; oi < oe; ++oi) {
    const DevOp& op = pp.ops[oi];
    const bool nd = op.kind == OP_DIAGND;
    // DIAGND: the tile's rows of the full table; DIAG1D along the lane: the lane table
    const C* tab = reinterpret_cast<const C*>(op.ptr) + (nd ? lane0 * n : 0);
#pragma unroll
    for (int j = 0; j < kPairV / RS; ++j) {
      const int b = t + j * T, l = b >> lgnb, k = b & (p - 1);
      if (!nd || l < nl) {
        const int row = nd ? l * n : 0;
#pragma unroll
        for (int q = 0; q < RS; ++q) v[j * RS + q] = cmul(v[j * RS + q], ldg_(tab + row + k + q * p));
      }
    }
  }
}

template <int RS, typename C>
__device__ __forceinline__ void pair_store_global(const C (&v)[kPairV], C* __restrict__ psi, int t, int T, int lgnb,
                                                  int nl, int n) {
  const int p = 1 << lgnb;
#pragma unroll
  for (int j = 0; j < kPairV / RS; ++j) {
    const int b = t + j * T, l = b >> lgnb, k = b & (p - 1);
    if (l < nl) {
      const int o = l * n + k;
#pragma unroll
      for (int q = 0; q < RS; ++q) psi[o + q * p] = v[j * RS + q];
    }
  }
}

// one stage of radix rs (a runtime value: 2, 4, 8 or 16) in one of the pair's forms
enum PairIn { PIN_GLOBAL, PIN_SMEM, PIN_REGS };
enum PairOut { POUT_SMEM, POUT_REGS, POUT_GLOBAL };

template <int RS, typename C, typename R>
__device__ __forceinline__ void pair_stage_rs(C (&v)[kPairV], C* buf, const PassParams& pp, int in, int out, int p,
                                              int dir, const C* tw, int ob, int oe, int64_t lane0, R sc) {
  const Geometry& g = pp.g;
  const int t = threadIdx.x, T = blockDim.x, n = (int)g.n, ls = g.lane_stride;
  const int lgnb = __ffs(n / RS) - 1;
  const int64_t rem = g.outer - lane0;
  const int nl = rem < g.lanes_per_tile ? (int)rem : g.lanes_per_tile;  // valid lanes of the tile
  C* tile_psi = reinterpret_cast<C*>(pp.psi) + lane0 * n;
  if (in == PIN_GLOBAL) {
    pair_load_global<RS, C>(v, tile_psi, t, T, lgnb, nl, n);
  } else if (in == PIN_SMEM) {
    pair_load_smem<RS, C>(v, buf, t, T, lgnb, ls);
    __syncthreads();  // every read of the stage before any write (in place)
  }
  pair_butterflies<RS, C>(v, t, T, lgnb, p, dir, tw);
  if (out == POUT_SMEM) {
    pair_store_smem<RS, C>(v, buf, t, T, lgnb, p, ls);
    __syncthreads();
  } else {
    // a last stage: p = n / RS = nb, outputs at k + q p
    pair_pointwise<RS, C, R>(v, pp, ob, oe, t, T, lgnb, lane0, nl, sc);
    if (out == POUT_GLOBAL) pair_store_global<RS, C>(v, tile_psi, t, T, lgnb, nl, n);
  }
}

template <int RMAX, typename C, typename R>
__device__ __forceinline__ void pair_stage(int rs, C (&v)[kPairV], C* buf, const PassParams& pp, int in, int out,
                                           int p, int dir, const C* tw, int ob, int oe, int64_t lane0, R sc) {
  if constexpr (RMAX == 16) {
    if (rs == 16) {
      pair_stage_rs<16, C, R>(v, buf, pp, in, out, p, dir, tw, ob, oe, lane0, sc);
      return;
    }
  }
  switch (rs) {
    case 8: pair_stage_rs<8, C, R>(v, buf, pp, in, out, p, dir, tw, ob, oe, lane0, sc); break;
    case 4: pair_stage_rs<4, C, R>(v, buf, pp, in, out, p, dir, tw, ob, oe, lane0, sc); break;
    default: pair_stage_rs<2, C, R>(v, buf, pp, in, out, p, dir, tw, ob, oe, lane0, sc); break;
  }
}

// RMAX: the radix of the stages (16 for FP32, 8 for FP64: the radix of the stage-major
// twiddle table each precision builds), S - 1 stages of RMAX and one closing radix rl
template <typename R, int RMAX>
__device__ __forceinline__ void fft_pair_tile(const PassParams& pp, int64_t tile) {
  using C = typename Cx<R>::T;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  C* buf = reinterpret_cast<C*>(smem_raw);
  const Geometry& g = pp.g;
  const int n = (int)g.n;
  const int64_t lane0 = tile * g.lanes_per_tile;
  const C* tw = reinterpret_cast<const C*>(pp.twiddle);
  const R sc = inv_sqrt_pow2<R>(__ffs(n) - 1);
  int f1 = 1;
  while (f1 < pp.nops && pp.ops[f1].kind != OP_FFT) ++f1;
  // the radices of fft_radices(n, RMAX, ...): S - 1 stages of RMAX and the closing radix rl
  // (the forward order ends with it, the reversed order starts with it)
  constexpr int kLgR = RMAX == 16 ? 4 : 3;
  const int lg = __ffs(n) - 1, S = (lg + kLgR - 1) / kLgR, rl = 1 << (lg - kLgR * (S - 1));
  C v[kPairV];
  int p = 1, off = 0;
  for (int s = 0; s < S; ++s) {
    const int rs = s + 1 < S ? RMAX : rl;
    const int in = s == 0 ? PIN_GLOBAL : PIN_SMEM, out = s + 1 < S ? POUT_SMEM : POUT_REGS;
    pair_stage<RMAX, C, R>(rs, v, buf, pp, in, out, p, pp.ops[0].dir, tw + off, 1, f1, lane0, sc);
    if (p > 1) off += (rs - 1) * p;
    p *= rs;
  }
  p = 1;
  off = 0;
  for (int s = 0; s < S; ++s) {
    const int rs = s == 0 ? rl : RMAX;
    const int in = s == 0 ? PIN_REGS : PIN_SMEM, out = s + 1 < S ? POUT_SMEM : POUT_GLOBAL;
    pair_stage<RMAX, C, R>(rs, v, buf, pp, in, out, p, pp.ops[f1].dir, tw + n + off, f1 + 1, pp.nops, lane0, sc);
    if (p > 1) off += (rs - 1) * p;
    p *= rs;
  }
}

__global__ void __launch_bounds__(512, 2) fft_pair_kernel(const __grid_constant__ PassParams p) {
  fft_pair_tile<float, 16>(p, blockIdx.x);
}

// FP32 with radix-8 stages (one more stage than radix 16, fewer registers per butterfly)
__global__ void __launch_bounds__(512, 2) fft_pair_kernel_r8(const __grid_constant__ PassParams p) {
  fft_pair_tile<float, 8>(p, blockIdx.x);
}

// FP64 lanes of 8192 points (one lane of 16 values per thread for 512 threads: one CTA per
// SM, whose 139 KB lane buffer leaves no room for a second)
__global__ void __launch_bounds__(512, 1) fft_pair_kernel_f64(const __grid_constant__ PassParams p) {
  fft_pair_tile<double, 8>(p, blockIdx.x);
}

// float-float lanes of 512-8192 points (radix-8 stages, the FP64 table order)
__global__ void __launch_bounds__(512, 1) fft_pair_kernel_ff(const __grid_constant__ PassParams p) {
  fft_pair_tile<ff, 8>(p, blockIdx.x);
}

template <typename R, int RMAX>
__device__ __forceinline__ void fft_pair_batched_tile(const PassParams* __restrict__ params,
                                                      const int64_t* __restrict__ offsets, int count) {
  const int64_t b = blockIdx.x;
  int lo = 0, hi = count - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (offsets[mid] <= b)
      lo = mid;
    else
      hi = mid - 1;
  }
  __shared__ __align__(16) PassParams sp;
  for (int k = threadIdx.x; k < (int)(sizeof(PassParams) / 4); k += blockDim.x)
    reinterpret_cast<uint32_t*>(&sp)[k] = reinterpret_cast<const uint32_t*>(params + lo)[k];
  __syncthreads();
  fft_pair_tile<R, RMAX>(sp, b - offsets[lo]);
}

__global__ void __launch_bounds__(512, 2) fft_pair_kernel_batched(const PassParams* __restrict__ params,
                                                                  const int64_t* __restrict__ offsets, int count) {
  fft_pair_batched_tile<float, 16>(params, offsets, count);
}

__global__ void __launch_bounds__(512, 1) fft_pair_kernel_batched_f64(const PassParams* __restrict__ params,
                                                                      const int64_t* __restrict__ offsets, int count) {
  fft_pair_batched_tile<double, 8>(params, offsets, count);
}

__global__ void __launch_bounds__(512, 2) fft_pair_kernel_batched_r8(const PassParams* __restrict__ params,
                                                                     const int64_t* __restrict__ offsets, int count) {
  fft_pair_batched_tile<float, 8>(params, offsets, count);
}

__global__ void __launch_bounds__(512, 1) fft_pair_kernel_batched_ff(const PassParams* __restrict__ params,
                                                                     const int64_t* __restrict__ offsets, int count) {
  fft_pair_batched_tile<ff, 8>(params, offsets, count);
}

static size_t fft_pair_smem(const Geometry& g, bool fp64);

// ------------------------------------------------------------------ FFT pair, fixed shape
// The same FP32 pass for lanes of 2^LGN points (512 .. 8192: the radial extents of the batched
// step) with the shape fixed at compile time: every stage's radix, span and twiddle offset,
// and the shared-memory lane stride, are constants.  A butterfly's 16 shared-memory, global
// and twiddle addresses are then one base plus immediate offsets, and the two directions (a
// forward transform, then an inverse one) fold into the butterflies' signs.  The arithmetic
// and its order are those of fft_pair_tile, so the results are the same.
__host__ __device__ constexpr int lg2c(int x) { return x <= 1 ? 0 : 1 + lg2c(x / 2); }

template <int LGN>
struct PairShape {
  static constexpr int kN = 1 << LGN;
  static constexpr int kS = (LGN + 3) / 4;              // stages of radix 16, the last one rl
  static constexpr int kRl = 1 << (LGN - 4 * (kS - 1));  // closing radix
  static constexpr int kLs = ((kN + (kN >> 4)) % 2 == 0) ? kN + (kN >> 4) + 1 : kN + (kN >> 4);
  // stage s of the forward order (16, ..., rl) and of the reversed order (rl, 16, ...)
  __host__ __device__ static constexpr int rs(bool rev, int s) { return rev ? (s == 0 ? kRl : 16) : (s + 1 < kS ? 16 : kRl); }
  __host__ __device__ static constexpr int span(bool rev, int s) { return s == 0 ? 1 : span(rev, s - 1) * rs(rev, s - 1); }
  // first entry of stage s in the stage-major twiddle table (reversed order: from entry n)
  __host__ __device__ static constexpr int twoff(bool rev, int s) {
    return s == 0 ? (rev ? kN : 0) : twoff(rev, s - 1) + (span(rev, s - 1) > 1 ? (rs(rev, s - 1) - 1) * span(rev, s - 1) : 0);
  }
};

// point-wise ops [ob, oe) on the outputs of a last stage (span P = n / RS): value j RS + q
// sits at lane b >> lg P, point k + q P, k = b & (P - 1)
template <int LGN, int RS>
__device__ __forceinline__ void pair_pointwise_ct(float2 (&v)[kPairV], const PassParams& pp, int ob, int oe, int t,
                                                  int T, int64_t lane0, int nl, float sc) {
  constexpr int kN = 1 << LGN, kP = kN / RS, kLgP = LGN - lg2c(RS);
#pragma unroll
  for (int e = 0; e < kPairV; ++e) v[e] = float2{v[e].x * sc, v[e].y * sc};
  for (int oi = ob; oi < oe; ++oi) {
    const DevOp& op = pp.ops[oi];
    const bool nd = op.kind == OP_DIAGND;
    const float2* tab = reinterpret_cast<const float2*>(op.ptr) + (nd ? lane0 * kN : 0);
#pragma unroll
    for (int j = 0; j < kPairV / RS; ++j) {
      const int b = t + j * T, l = b >> kLgP, k = b & (kP - 1);
      if (!nd || l < nl) {
        const float2* tr = tab + (nd ? l * kN : 0) + k;
#pragma unroll
        for (int q = 0; q < RS; ++q) v[j * RS + q] = cmul(v[j * RS + q], __ldg(tr + q * kP));
      }
    }
  }
}

// one stage: radix RS, span P, twiddles from entry OFF; IN / OUT as in pair_stage_rs
template <int LGN, int RS, int P, int OFF, int IN, int OUT, int DIR>
__device__ __forceinline__ void pair_stage_ct(float2 (&v)[kPairV], float2* buf, const PassParams& pp,
                                              float2* tile_psi, const float2* __restrict__ tw, int ob, int oe,
                                              int64_t lane0, int nl, float sc) {
  constexpr int kN = 1 << LGN, kNb = kN / RS, kLgNb = LGN - lg2c(RS), kLs = PairShape<LGN>::kLs;
  const int t = threadIdx.x, T = blockDim.x;
  if constexpr (IN == PIN_GLOBAL) {
#pragma unroll
    for (int j = 0; j < kPairV / RS; ++j) {
      const int b = t + j * T, l = b >> kLgNb, i = b & (kNb - 1);
      const float2* src = tile_psi + l * kN + i;
      const bool ok = l < nl;
#pragma unroll
      for (int r = 0; r < RS; ++r) v[j * RS + r] = ok ? src[r * kNb] : float2{0.0f, 0.0f};
    }
  } else if constexpr (IN == PIN_SMEM) {
    // element l ls + x + (x >> 4) of x = i + r nb: the padding term splits as (i >> 4) + (r nb >> 4)
#pragma unroll
    for (int j = 0; j < kPairV / RS; ++j) {
      const int b = t + j * T, l = b >> kLgNb, i = b & (kNb - 1);
      const float2* src = buf + l * kLs + i + (i >> 4);
#pragma unroll
      for (int r = 0; r < RS; ++r) v[j * RS + r] = src[r * kNb + ((r * kNb) >> 4)];
    }
    __syncthreads();  // every read of the stage before any write (in place)
  }
#pragma unroll
  for (int j = 0; j < kPairV / RS; ++j) {
    if constexpr (P > 1) {
      // k = i & (P - 1) = b & (P - 1) (P <= nb); entry 0 of every twiddle row is exactly 1
      const float2* w = tw + OFF + ((t + j * T) & (P - 1));
#pragma unroll
      for (int r = 1; r < RS; ++r) {
        float2 wv = __ldg(w + (r - 1) * P);
        if (DIR > 0) wv.y = -wv.y;
        v[j * RS + r] = cmul(v[j * RS + r], wv);
      }
    }
    dft_r<RS>(&v[j * RS], DIR);
  }
  if constexpr (OUT == POUT_SMEM) {
    // outputs base + q P, base = (i - k) RS + k: the padding term splits as (base >> 4) + (q P >> 4)
#pragma unroll
    for (int j = 0; j < kPairV / RS; ++j) {
      const int b = t + j * T, l = b >> kLgNb, i = b & (kNb - 1), k = i & (P - 1);
      const int base = (i - k) * RS + k;
      float2* dst = buf + l * kLs + base + (base >> 4);
#pragma unroll
      for (int q = 0; q < RS; ++q) dst[q * P + ((q * P) >> 4)] = v[j * RS + q];
    }
    __syncthreads();
  } else {
    pair_pointwise_ct<LGN, RS>(v, pp, ob, oe, t, T, lane0, nl, sc);
    if constexpr (OUT == POUT_GLOBAL) {
#pragma unroll
      for (int j = 0; j < kPairV / RS; ++j) {
        const int b = t + j * T, l = b >> kLgNb, k = b & (kNb - 1);
        if (l < nl) {
          float2* dst = tile_psi + l * kN + k;
#pragma unroll
          for (int q = 0; q < RS; ++q) dst[q * kNb] = v[j * RS + q];
        }
      }
    }
  }
}

// the stages S .. of one transform (REV: the reversed order of the second transform)
template <int LGN, bool REV, int S, int DIR>
__device__ __forceinline__ void pair_fft_ct(float2 (&v)[kPairV], float2* buf, const PassParams& pp, float2* tile_psi,
                                            const float2* tw, int ob, int oe, int64_t lane0, int nl, float sc) {
  using Sh = PairShape<LGN>;
  constexpr int kIn = S == 0 ? (REV ? PIN_REGS : PIN_GLOBAL) : PIN_SMEM;
  constexpr int kOut = S + 1 < Sh::kS ? POUT_SMEM : (REV ? POUT_GLOBAL : POUT_REGS);
  pair_stage_ct<LGN, Sh::rs(REV, S), Sh::span(REV, S), Sh::twoff(REV, S), kIn, kOut, DIR>(v, buf, pp, tile_psi, tw, ob,
                                                                                         oe, lane0, nl, sc);
  if constexpr (S + 1 < Sh::kS) pair_fft_ct<LGN, REV, S + 1, DIR>(v, buf, pp, tile_psi, tw, ob, oe, lane0, nl, sc);
}

// [F (forward), point-wise, F^-1, point-wise] on the tile's lanes of 2^LGN points
template <int LGN>
__device__ __forceinline__ void fft_pair_tile_ct(const PassParams& pp, int64_t tile) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  float2* buf = reinterpret_cast<float2*>(smem_raw);
  const Geometry& g = pp.g;
  const int64_t lane0 = tile * g.lanes_per_tile;
  const int64_t rem = g.outer - lane0;
  const int nl = rem < g.lanes_per_tile ? (int)rem : g.lanes_per_tile;
  float2* tile_psi = reinterpret_cast<float2*>(pp.psi) + lane0 * (1 << LGN);
  const float2* tw = reinterpret_cast<const float2*>(pp.twiddle);
  const float sc = inv_sqrt_pow2<float>(LGN);
  int f1 = 1;
  while (f1 < pp.nops && pp.ops[f1].kind != OP_FFT) ++f1;
  float2 v[kPairV];
  pair_fft_ct<LGN, false, 0, -1>(v, buf, pp, tile_psi, tw, 1, f1, lane0, nl, sc);
  pair_fft_ct<LGN, true, 0, 1>(v, buf, pp, tile_psi, tw, f1 + 1, pp.nops, lane0, nl, sc);
}

template <int LGN>
__global__ void __launch_bounds__(512, 2) fft_pair_kernel_ct(const __grid_constant__ PassParams p) {
  fft_pair_tile_ct<LGN>(p, blockIdx.x);
}

template <int LGN>
__global__ void __launch_bounds__(512, 2) fft_pair_kernel_batched_ct(const PassParams* __restrict__ params,
                                                                     const int64_t* __restrict__ offsets, int count) {
  const int64_t b = blockIdx.x;
  int lo = 0, hi = count - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (offsets[mid] <= b)
      lo = mid;
    else
      hi = mid - 1;
  }
  __shared__ __align__(16) PassParams sp;
  for (int k = threadIdx.x; k < (int)(sizeof(PassParams) / 4); k += blockDim.x)
    reinterpret_cast<uint32_t*>(&sp)[k] = reinterpret_cast<const uint32_t*>(params + lo)[k];
  __syncthreads();
  fft_pair_tile_ct<LGN>(sp, b - offsets[lo]);
}

// log2 n when a planned FP32 pair can run the fixed-shape kernel (radix 16, n = 512 .. 8192,
// the padded lane stride of the geometry, a forward transform then an inverse one), else 0
int fft_pair_ct_lgn(const PassParams& p, bool fp64) {
  if (fp64 || !p.fused || p.radix != 16) return 0;
  const int64_t n = p.g.n;
  if (n < 512 || n > 8192 || (n & (n - 1)) != 0) return 0;
  int64_t ls = n + (n >> 4);
  if (ls % 2 == 0) ls += 1;
  if (p.g.lane_stride != ls || p.nops < 2 || p.ops[0].kind != OP_FFT || p.ops[0].dir != -1) return 0;
  int f1 = 1;
  while (f1 < p.nops && p.ops[f1].kind != OP_FFT) ++f1;
  if (f1 >= p.nops || p.ops[f1].dir != 1) return 0;
  int lg = 0;
  while ((int64_t)1 << lg < n) ++lg;
  return lg;
}

template <typename K>
static cudaError_t configure_once(K kern, bool& done) {
  if (done) return cudaSuccess;
  cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, 220 * 1024);
  if (e == cudaSuccess) done = true;
  return e;
}

template <int LGN>
static cudaError_t launch_pair_ct(const PassParams& p, cudaStream_t s) {
  static bool done = false;
  cudaError_t e = configure_once(fft_pair_kernel_ct<LGN>, done);
  if (e != cudaSuccess) return e;
  fft_pair_kernel_ct<LGN><<<(unsigned)p.g.tiles, fft_pair_block(p.g), fft_pair_smem(p.g, false), s>>>(p);
  return cudaGetLastError();
}

template <int LGN>
static cudaError_t launch_pair_batched_ct(const PassParams* params_dev, const int64_t* offsets_dev, int count,
                                          int64_t blocks, int threads, size_t smem, cudaStream_t s) {
  static bool done = false;
  cudaError_t e = configure_once(fft_pair_kernel_batched_ct<LGN>, done);
  if (e != cudaSuccess) return e;
  fft_pair_kernel_batched_ct<LGN><<<(unsigned)blocks, threads, smem, s>>>(params_dev, offsets_dev, count);
  return cudaGetLastError();
}

static cudaError_t launch_pair_ct_any(int lgn, const PassParams& p, cudaStream_t s) {
  switch (lgn) {
    case 9: return launch_pair_ct<9>(p, s);
    case 10: return launch_pair_ct<10>(p, s);
    case 11: return launch_pair_ct<11>(p, s);
    case 12: return launch_pair_ct<12>(p, s);
    case 13: return launch_pair_ct<13>(p, s);
    default: return cudaErrorInvalidValue;
  }
}

static cudaError_t launch_pair_batched_ct_any(int lgn, const PassParams* params_dev, const int64_t* offsets_dev,
                                              int count, int64_t blocks, int threads, size_t smem, cudaStream_t s) {
  switch (lgn) {
    case 9: return launch_pair_batched_ct<9>(params_dev, offsets_dev, count, blocks, threads, smem, s);
    case 10: return launch_pair_batched_ct<10>(params_dev, offsets_dev, count, blocks, threads, smem, s);
    case 11: return launch_pair_batched_ct<11>(params_dev, offsets_dev, count, blocks, threads, smem, s);
    case 12: return launch_pair_batched_ct<12>(params_dev, offsets_dev, count, blocks, threads, smem, s);
    case 13: return launch_pair_batched_ct<13>(params_dev, offsets_dev, count, blocks, threads, smem, s);
    default: return cudaErrorInvalidValue;
  }
}

int fft_pair_threads(const Geometry& g) { return g.n >= 8192 ? 512 : 256; }

int fft_pair_block(const Geometry& g) { return (int)((int64_t)g.lanes_per_tile * g.n / kPairV); }

bool fft_pair_plan(PassParams& p, int real, bool resident) {
  Geometry& g = p.g;
  const bool fp64 = real != kRealF32;
  if (resident || g.inner != 1 || !stage_twiddles(g.n) || g.n > 8192 || p.twiddle == nullptr) return false;
  // FP64: only the lanes longer than the general pass's FP64 tile (4096 points) take the pair
  // kernel; shorter FP64 lanes keep the general pass.  Float-float: lanes of 512 points and
  // more (measured on the 512-instance batch: the radial passes 14.2 -> 13.1 ms per step)
  if (real == kRealF64 && g.n <= 4096) return false;
  if (real == kRealFF && g.n < 512) return false;
  if (p.nops < 2 || p.ops[0].kind != OP_FFT) return false;
  int ffts = 0;
  for (int i = 0; i < p.nops; ++i) {
    const DevOp& op = p.ops[i];
    if (op.kind == OP_FFT) {
      ++ffts;
    } else if (op.kind == OP_DIAGND || (op.kind == OP_DIAG1D && op.axis == g.sweep_axis)) {
      // point-wise, in registers
    } else {
      return false;
    }
  }
  if (ffts != 2) return false;
  // the tuned schedule when it is valid for this lane: T threads hold kPairV values each, so
  // a tile is L = kPairV T / n >= 1 whole lanes; FP64 stays at radix 8 (its table's order)
  const PairSchedule sc = pair_schedule(g.n, fp64);
  int T = fft_pair_threads(g);
  if ((sc.threads == 128 || sc.threads == 256 || sc.threads == 512) && (int64_t)kPairV * sc.threads >= g.n &&
      !(fp64 && sc.threads != 512))
    T = sc.threads;
  const int64_t L = (int64_t)kPairV * T / g.n;
  g.lanes_per_tile = (int32_t)L;
  g.tiles_per_outer = 1;
  g.tiles = (g.outer + L - 1) / L;
  p.fused = 1;
  p.radix = fp64 ? 8 : (sc.radix == 8 ? 8 : 16);
  return true;
}

static size_t fft_pair_smem(const Geometry& g, bool fp64) {
  return ((size_t)g.lanes_per_tile * g.lane_stride * (fp64 ? sizeof(double2) : sizeof(float2)) + 15) & ~(size_t)15;
}

template <typename R, int RMAX, bool SWEEP>
__global__ void __launch_bounds__(512, 2) pass_kernel(const __grid_constant__ PassParams p) {
  pass_tile<R, RMAX, SWEEP>(p, blockIdx.x);
}

// Many propagations' passes in one launch: block b runs tile (b - offsets[i]) of
// params[i], offsets[i] <= b < offsets[i + 1].
template <typename R, int RMAX, bool SWEEP>
__global__ void __launch_bounds__(512, 2) pass_kernel_batched(const PassParams* __restrict__ params,
                                                           const int64_t* __restrict__ offsets, int count) {
  const int64_t b = blockIdx.x;
  int lo = 0, hi = count - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (offsets[mid] <= b)
      lo = mid;
    else
      hi = mid - 1;
  }
  // the pass description is read throughout the tile: keep a shared-memory copy
  __shared__ __align__(16) PassParams sp;
  static_assert(sizeof(PassParams) % 4 == 0, "PassParams is copied as 32-bit words");
  for (int k = threadIdx.x; k < (int)(sizeof(PassParams) / 4); k += blockDim.x)
    reinterpret_cast<uint32_t*>(&sp)[k] = reinterpret_cast<const uint32_t*>(params + lo)[k];
  __syncthreads();
  pass_tile<R, RMAX, SWEEP>(sp, b - offsets[lo]);
}

template <typename R, int RMAX, bool SWEEP>
static cudaError_t launch_batched_impl(const PassParams* params_dev, const int64_t* offsets_dev, int count,
                                       int64_t blocks, int threads, size_t smem, cudaStream_t s) {
  auto kern = pass_kernel_batched<R, RMAX, SWEEP>;
  static bool configured = false;
  if (!configured) {
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, 220 * 1024);
    if (e != cudaSuccess) return e;
    configured = true;
  }
  if (smem > 220 * 1024 || threads > 512) return cudaErrorInvalidValue;
  kern<<<(unsigned)blocks, threads, smem, s>>>(params_dev, offsets_dev, count);
  count_launch();
  return cudaGetLastError();
}

cudaError_t launch_pass_batched(int real, bool sweep, bool fused, const PassParams* params_dev,
                                const int64_t* offsets_dev, int count, int64_t blocks, int threads, size_t smem,
                                cudaStream_t s, int radix, int ct_lgn) {
  const bool fp64 = real != kRealF32;
  if (real == kRealFF) {
    if (fused) {
      if (smem > 220 * 1024 || threads > 512) return cudaErrorInvalidValue;
      static bool configured = false;
      if (!configured) {
        cudaError_t e =
            cudaFuncSetAttribute(fft_pair_kernel_batched_ff, cudaFuncAttributeMaxDynamicSharedMemorySize, 220 * 1024);
        if (e != cudaSuccess) return e;
        configured = true;
      }
      fft_pair_kernel_batched_ff<<<(unsigned)blocks, threads, smem, s>>>(params_dev, offsets_dev, count);
      count_launch();
      return cudaGetLastError();
    }
    return sweep ? launch_batched_impl<ff, 8, true>(params_dev, offsets_dev, count, blocks, threads, smem, s)
                 : launch_batched_impl<ff, 8, false>(params_dev, offsets_dev, count, blocks, threads, smem, s);
  }
  if (fused) {
    if (smem > 220 * 1024 || threads > 512) return cudaErrorInvalidValue;
    if (ct_lgn > 0 && !fp64 && radix != 8) {
      const cudaError_t e = launch_pair_batched_ct_any(ct_lgn, params_dev, offsets_dev, count, blocks, threads, smem, s);
      if (e == cudaSuccess) count_launch();
      return e;
    }
    static bool configured[3] = {false, false, false};
    const int which = fp64 ? 1 : (radix == 8 ? 2 : 0);
    const void* kerns[3] = {(const void*)fft_pair_kernel_batched, (const void*)fft_pair_kernel_batched_f64,
                            (const void*)fft_pair_kernel_batched_r8};
    if (!configured[which]) {
      cudaError_t e = cudaFuncSetAttribute(kerns[which], cudaFuncAttributeMaxDynamicSharedMemorySize, 220 * 1024);
      if (e != cudaSuccess) return e;
      configured[which] = true;
    }
    if (which == 1)
      fft_pair_kernel_batched_f64<<<(unsigned)blocks, threads, smem, s>>>(params_dev, offsets_dev, count);
    else if (which == 2)
      fft_pair_kernel_batched_r8<<<(unsigned)blocks, threads, smem, s>>>(params_dev, offsets_dev, count);
    else
      fft_pair_kernel_batched<<<(unsigned)blocks, threads, smem, s>>>(params_dev, offsets_dev, count);
    count_launch();
    return cudaGetLastError();
  }
  if (fp64)
    return sweep ? launch_batched_impl<double, 8, true>(params_dev, offsets_dev, count, blocks, threads, smem, s)
                 : launch_batched_impl<double, 8, false>(params_dev, offsets_dev, count, blocks, threads, smem, s);
  return sweep ? launch_batched_impl<float, 16, true>(params_dev, offsets_dev, count, blocks, threads, smem, s)
               : launch_batched_impl<float, 16, false>(params_dev, offsets_dev, count, blocks, threads, smem, s);
}

size_t pass_smem_bytes(const PassParams& p, bool fp64) {
  const Geometry& g = p.g;
  if (p.fused) return fft_pair_smem(g, fp64);
  const bool fft = p.twiddle != nullptr;
  const size_t cs = fp64 ? 16 : 8;
  size_t b = (p.one_buffer ? 1 : 2) * (((size_t)g.lanes_per_tile * g.lane_stride * cs + 15) & ~(size_t)15);
  b += (size_t)g.lanes_per_tile * (sizeof(int64_t) + sizeof(double) + kMaxDims * sizeof(int) + sizeof(int));
  b = (b + 15) & ~(size_t)15;
  if (fft && twiddles_in_smem(g)) b += (size_t)g.n * cs;
  return b;
}

void pass_choose_buffers(PassParams& p, bool fp64) {
  (void)fp64;
  p.one_buffer = 0;  // every pass keeps the ping-pong pair of tile buffers
  const Geometry& g = p.g;
  bool sweep = true;
  for (int i = 0; i < p.nops; ++i) {
    const int k = p.ops[i].kind;
    if (k == OP_MAT || k == OP_MAT_LANE || k == OP_MAT_SLICE || k == OP_DOT) sweep = false;
    if (k == OP_FFT && !((g.n & (g.n - 1)) == 0 && g.n >= 16)) sweep = false;
  }
  p.sweep = sweep ? 1 : 0;
}

int pass_threads(const Geometry& g) {
  const int64_t pts = (int64_t)g.lanes_per_tile * g.n;
  int64_t t = (pts + g.vals - 1) / g.vals;
  t = ((t + 31) / 32) * 32;
  if (t < 32) t = 32;
  if (t > 512) t = 512;
  return (int)t;
}

template <typename R, int RMAX, bool SWEEP>
static cudaError_t launch_impl(const PassParams& p, cudaStream_t s) {
  const size_t smem = pass_smem_bytes(p, sizeof(R) == 8);
  auto kern = pass_kernel<R, RMAX, SWEEP>;
  static bool configured = false;
  if (!configured) {
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, 220 * 1024);
    if (e != cudaSuccess) return e;
    configured = true;
  }
  if (smem > 220 * 1024) return cudaErrorInvalidValue;
  const int threads = pass_threads(p.g);
  kern<<<(unsigned)p.g.tiles, threads, smem, s>>>(p);
  count_launch();
  return cudaGetLastError();
}

cudaError_t launch_pass_f64(const PassParams& p, cudaStream_t s) {
  if (p.fused) {
    static bool configured = false;
    if (!configured) {
      cudaError_t e =
          cudaFuncSetAttribute(fft_pair_kernel_f64, cudaFuncAttributeMaxDynamicSharedMemorySize, 220 * 1024);
      if (e != cudaSuccess) return e;
      configured = true;
    }
    const size_t smem = fft_pair_smem(p.g, true);
    if (smem > 220 * 1024) return cudaErrorInvalidValue;
    fft_pair_kernel_f64<<<(unsigned)p.g.tiles, fft_pair_block(p.g), smem, s>>>(p);
    count_launch();
    return cudaGetLastError();
  }
  return p.sweep ? launch_impl<double, 8, true>(p, s) : launch_impl<double, 8, false>(p, s);
}
cudaError_t launch_pass_ff(const PassParams& p, cudaStream_t s) {
  if (p.fused) {
    static bool configured = false;
    if (!configured) {
      cudaError_t e = cudaFuncSetAttribute(fft_pair_kernel_ff, cudaFuncAttributeMaxDynamicSharedMemorySize, 220 * 1024);
      if (e != cudaSuccess) return e;
      configured = true;
    }
    const size_t smem = fft_pair_smem(p.g, true);
    if (smem > 220 * 1024) return cudaErrorInvalidValue;
    fft_pair_kernel_ff<<<(unsigned)p.g.tiles, fft_pair_block(p.g), smem, s>>>(p);
    count_launch();
    return cudaGetLastError();
  }
  return p.sweep ? launch_impl<ff, 8, true>(p, s) : launch_impl<ff, 8, false>(p, s);
}
cudaError_t launch_pass_f32(const PassParams& p, cudaStream_t s) {
  if (p.fused) {
    static bool configured[2] = {false, false};
    const bool r8 = p.radix == 8;
    const void* kern = r8 ? (const void*)fft_pair_kernel_r8 : (const void*)fft_pair_kernel;
    if (!configured[r8 ? 1 : 0]) {
      cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, 220 * 1024);
      if (e != cudaSuccess) return e;
      configured[r8 ? 1 : 0] = true;
    }
    const size_t smem = fft_pair_smem(p.g, false);
    if (smem > 220 * 1024) return cudaErrorInvalidValue;
    if (p.ct > 0 && !r8) {
      const cudaError_t e = launch_pair_ct_any(p.ct, p, s);
      if (e == cudaSuccess) count_launch();
      return e;
    }
    if (r8)
      fft_pair_kernel_r8<<<(unsigned)p.g.tiles, fft_pair_block(p.g), smem, s>>>(p);
    else
      fft_pair_kernel<<<(unsigned)p.g.tiles, fft_pair_block(p.g), smem, s>>>(p);
    count_launch();
    return cudaGetLastError();
  }
  return p.sweep ? launch_impl<float, 16, true>(p, s) : launch_impl<float, 16, false>(p, s);
}

}  // namespace so
