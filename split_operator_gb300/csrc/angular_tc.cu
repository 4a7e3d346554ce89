// Angular (lane-matrix) sweep on the 5th-generation tensor cores, FP32 state.
//
// Replaces, fused into one pass, MatrixTransformation::transform /
// inverse_transform (matrix_transformation.rs:60-75) for real matrices -- the
// Legendre transforms of legendre_diagonalization.rs:13-45 -- together with the
// diagonal propagators, border damping and norm folds the step applies between
// and around them (n_dim_propagator.rs:32-36, one_dim_propagator.rs:37-46,
// border_dumping.rs:57-93, wave_function.rs:68-85).
//
// Layout: the state is stored [outer][n][inner] (n = lane axis, e.g. theta, 32..128;
// inner = radial points).  A CTA owns a tile of kBN = 64 complex columns of the inner
// axis for all n rows.  Treating (re, im) as two real columns, each lane matrix
// product is a real GEMM D[128 x 128] = A[128 x n] . B[n x 128] with A the (zero-
// padded) matrix and B the tile.  3xTF32: A = A_hi + A_lo (split once from the FP64
// matrix on the host), B = B_hi + B_lo (split on the fly), D = A_hi B_hi + A_hi B_lo
// + A_lo B_hi accumulated in FP32 in tensor memory.
//
//   prologue  (thread = column): load tile, pre-ops, split -> B_hi/B_lo (smem)
//   GEMM 1    (one thread issues tcgen05.mma; A chunks stream in by bulk TMA)
//   epilogue 1 (thread = row, tcgen05.ld from TMEM): mid-ops, split -> B for GEMM 2
//   GEMM 2
//   epilogue 2: post-ops -> staging -> coalesced store
//   FP64 norm partials folded by the last CTA in a fixed order (as lane_sweep.cu).
// Every mbarrier wait is bounded; on a timeout the CTA records an error in a slot,
// waits (bounded) for its own copies, frees its tensor memory and returns.
#include "common.cuh"
#include "tc_common.cuh"

namespace so {

namespace {

constexpr int kBN = 64;             // complex columns per tile
constexpr int kNC = 2 * kBN;        // fp32 columns = MMA N
constexpr int kM = 128;             // MMA M (matrix rows, zero padded)
constexpr int kChunkK = 32;         // K per A chunk
constexpr int kChunkBytes = kM * kChunkK * 4;  // one of hi / lo
constexpr int kLboB = 144;          // B: core matrices along K (16 B padding vs 128)
constexpr int kStageRow = 132;      // output staging row stride in floats (528 B)
constexpr uint64_t kWaitLimit = 2000000000ull;  // 2 s per wait
constexpr int kThreads = 128;

struct TcSmemLayout {
  uint32_t stage0, stage1, bhi, blo, bars, sbo_b, bbytes, total;
};

__host__ __device__ inline TcSmemLayout tc_layout(int n) {
  TcSmemLayout L{};
  L.sbo_b = (uint32_t)((n + 3) / 4) * kLboB + 16;
  L.bbytes = 16u * L.sbo_b;  // 16 groups of 8 columns
  L.bbytes = (L.bbytes + 127u) & ~127u;
  const uint32_t stage_bytes = 2u * kChunkBytes;
  L.stage0 = 0;
  L.stage1 = stage_bytes;
  L.bhi = 2 * stage_bytes;
  L.blo = L.bhi + L.bbytes;
  L.bars = L.blo + L.bbytes;
  L.total = L.bars + 64;
  return L;
}

__device__ __forceinline__ uint32_t boff(int q, int k, uint32_t sbo) {
  return (uint32_t)(q >> 3) * sbo + (uint32_t)(k >> 2) * kLboB + (uint32_t)(q & 7) * 16u + (uint32_t)(k & 3) * 4u;
}

__device__ __forceinline__ float2 cmulf(float2 a, float2 b) { return {a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x}; }

__device__ double block_sum128(double v, double* scratch) {
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) v += __shfl_down_sync(0xffffffffu, v, off);
  if ((threadIdx.x & 31) == 0) scratch[threadIdx.x >> 5] = v;
  __syncthreads();
  double r = 0.0;
  if (threadIdx.x == 0) r = scratch[0] + scratch[1] + scratch[2] + scratch[3];
  __syncthreads();
  return r;
}

// logical coordinate of axis `a` for element (outer o, inner i) (a != sweep axis)
__device__ __forceinline__ int64_t coord_of(const Geometry& g, int a, int64_t o, int64_t i) {
  int64_t v = i;
  for (int q = g.ndim - 1; q > g.spos; --q) {
    const int64_t c = v % g.sshape[q];
    if (g.perm[q] == a) return c;
    v /= g.sshape[q];
  }
  v = o;
  for (int q = g.spos - 1; q >= 0; --q) {
    const int64_t c = v % g.sshape[q];
    if (g.perm[q] == a) return c;
    v /= g.sshape[q];
  }
  return 0;
}

// One point-wise op on the complex value at (row j, outer o, inner i); global index idx.
__device__ __forceinline__ float2 point_op(const PassParams& p, const DevOp& op, int oi, float2 v, int j, int64_t o,
                                           int64_t i, int64_t idx, double* acc, const double* sc) {
  const Geometry& g = p.g;
  switch (op.kind) {
    case OP_DIAG1D: {
      const float2* t = reinterpret_cast<const float2*>(op.ptr);
      const int64_t k = op.axis == g.sweep_axis ? j : coord_of(g, op.axis, o, i);
      return cmulf(v, __ldg(t + k));
    }
    case OP_DIAGND:
      return cmulf(v, __ldg(reinterpret_cast<const float2*>(op.ptr) + idx));
    case OP_SCALE: {
      const float f = (float)sc[oi];
      return {v.x * f, v.y * f};
    }
    case OP_NORM: {
      double w = op.w[g.sweep_axis][j];
      for (int a = 0; a < g.ndim; ++a)
        if (a != g.sweep_axis) w *= op.w[a][coord_of(g, a, o, i)];
      acc[op.red] += ((double)v.x * v.x + (double)v.y * v.y) * w;
      return v;
    }
    default:
      return v;
  }
}

__device__ void run_scalar_tc(const PassParams& p, const DevOp& op, const double* totals) {
  double* s = p.slots;
  switch (op.kind) {
    case OP_NORM: {
      const double v = totals[op.red];
      s[op.a] = v;
      if (!isfinite(v) && p.nonfinite_slot >= 0) s[p.nonfinite_slot] = 1.0;
      break;
    }
    case OP_COPY: s[op.a] = s[op.b]; break;
    case OP_LOSS: s[op.a] += s[op.b] - s[op.c]; break;
    case OP_SETC: s[op.a] = op.value; break;
    case OP_RECORD:
      if (p.record) p.record[op.count] = s[op.a];
      break;
    default: break;
  }
}

}  // namespace

struct TcParams {
  PassParams p;
  int32_t mat_op[2];      // op indices of the (one or two) lane matrices
  int32_t nmat;
  const float* images[2]; // A chunk images per matrix: nchunks x (hi 16 KB, lo 16 KB)
  int32_t error_slot;
};

__device__ __forceinline__ void tc_tile(const TcParams& tp, const int64_t tile) {
  using namespace tc;
  const PassParams& p = tp.p;
  const Geometry& g = p.g;
  extern __shared__ __align__(1024) unsigned char sm[];
  __shared__ uint32_t tmem_base_s;
  __shared__ double scratch[4];
  __shared__ double blk_red[kMaxRed];
  __shared__ double totals[kMaxRed];
  __shared__ double scale_v[kMaxOps];
  __shared__ int s_last, s_fail;

  const int n = (int)g.n;
  const TcSmemLayout L = tc_layout(n);
  unsigned char* stage[2] = {sm + L.stage0, sm + L.stage1};
  float* bhi = reinterpret_cast<float*>(sm + L.bhi);
  float* blo = reinterpret_cast<float*>(sm + L.blo);
  uint64_t* bars = reinterpret_cast<uint64_t*>(sm + L.bars);
  uint64_t* full = bars;       // [2]
  uint64_t* empty = bars + 2;  // [2]
  uint64_t* dbar = bars + 4;
  const int tid = threadIdx.x, warp = tid >> 5;
  const int nk = (n + kChunkK - 1) / kChunkK;
  const int total_chunks = nk * tp.nmat;

  const int64_t o = tile / g.tiles_per_outer;
  const int64_t i0 = (tile - o * g.tiles_per_outer) * kBN;
  const int64_t base = o * g.n * g.inner + i0;  // element (row 0, column 0) of the tile
  float2* psi = reinterpret_cast<float2*>(p.psi);

  if (tid == 0) {
    mbar_init(&full[0], 1);
    mbar_init(&full[1], 1);
    mbar_init(&empty[0], 1);
    mbar_init(&empty[1], 1);
    mbar_init(dbar, 1);
    fence_mbar_init();
    s_fail = 0;
  }
  if (tid < kMaxOps) {
    const DevOp& op = p.ops[tid < p.nops ? tid : 0];
    scale_v[tid] = (tid < p.nops && op.kind == OP_SCALE) ? sqrt(__ldcg(p.slots + op.b) / __ldcg(p.slots + op.c)) : 0.0;
  }
  if (warp == 0) tmem_alloc(&tmem_base_s, 256);
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = tmem_base_s;

  // A producer (thread 0): chunk c of the whole sequence -> stage c & 1
  auto issue_chunk = [&](int c) {
    const int m = c / nk, q = c - m * nk;
    const int s = c & 1;
    mbar_expect_tx(&full[s], 2u * kChunkBytes);
    bulk_g2s(stage[s], tp.images[m] + (size_t)q * 2 * (kChunkBytes / 4), 2u * kChunkBytes, &full[s]);
  };
  if (tid == 0) {
    issue_chunk(0);
    if (total_chunks > 1) issue_chunk(1);
  }

  // ops before the first matrix run in the prologue, the others in the epilogue that follows their matrix
  const int seg_end0 = tp.mat_op[0];
  double acc[kMaxRed];
#pragma unroll
  for (int r = 0; r < kMaxRed; ++r) acc[r] = 0.0;

  // ---- prologue: thread = complex column c, rows of parity h
  {
    const int c = tid & (kBN - 1), h = tid >> 6;
    const int64_t i = i0 + c;
    for (int k = h; k < n; k += 2) {
      const int64_t idx = base + (int64_t)k * g.inner + c;
      float2 v = psi[idx];
      for (int oi = 0; oi < seg_end0; ++oi) v = point_op(p, p.ops[oi], oi, v, k, o, i, idx, acc, scale_v);
      float rh, rl, ih, il;
      split_tf32(v.x, rh, rl);
      split_tf32(v.y, ih, il);
      const uint32_t a0 = boff(2 * c, k, L.sbo_b) >> 2, a1 = boff(2 * c + 1, k, L.sbo_b) >> 2;
      bhi[a0] = rh;
      blo[a0] = rl;
      bhi[a1] = ih;
      blo[a1] = il;
    }
    // rows n..(K rounded to 8) stay zero in the K remainder (n is a multiple of 32 here)
  }
  fence_proxy_async();
  __syncthreads();

  const uint32_t idesc = idesc_tf32(kM, kNC);
  // MMA issue for matrix m into TMEM columns [m * 128, m * 128 + 128)
  auto run_gemm = [&](int m) -> bool {
    const uint32_t d = tmem + (uint32_t)(m * kNC);
    for (int q = 0; q < nk; ++q) {
      const int c = m * nk + q, s = c & 1;
      if (!mbar_wait(&full[s], (uint32_t)((c >> 1) & 1), kWaitLimit)) return false;
      tc_fence_after();
      const int ksteps = min(kChunkK, n - q * kChunkK) / 8;
      for (int ks = 0; ks < ksteps; ++ks) {
        const int kg = q * kChunkK + ks * 8;
        const uint64_t ahi = smem_desc(stage[s] + ks * 256, 128, 1024);
        const uint64_t alo = smem_desc(stage[s] + kChunkBytes + ks * 256, 128, 1024);
        const uint64_t bh = smem_desc(reinterpret_cast<unsigned char*>(bhi) + (kg >> 2) * kLboB, kLboB, L.sbo_b);
        const uint64_t bl = smem_desc(reinterpret_cast<unsigned char*>(blo) + (kg >> 2) * kLboB, kLboB, L.sbo_b);
        mma_tf32(d, ahi, bh, idesc, (q > 0 || ks > 0) ? 1u : 0u);
        mma_tf32(d, ahi, bl, idesc, 1u);
        mma_tf32(d, alo, bh, idesc, 1u);
      }
      mma_commit(&empty[s]);
      // refill the stage of the previous chunk with chunk c + 1 (its MMAs were issued earlier)
      if (c >= 1 && c + 1 < total_chunks) {
        const int ps = (c - 1) & 1;
        if (!mbar_wait(&empty[ps], (uint32_t)(((c - 1) >> 1) & 1), kWaitLimit)) return false;
        issue_chunk(c + 1);
      }
    }
    mma_commit(dbar);
    return true;
  };

  // ---- GEMMs and epilogues
  for (int m = 0; m < tp.nmat; ++m) {
    if (tid == 0 && !s_fail) {
      if (!run_gemm(m)) s_fail = 1;
    }
    __syncthreads();
    bool ok = !s_fail;
    if (ok && !mbar_wait(dbar, (uint32_t)(m & 1), kWaitLimit)) ok = false;
    // every thread takes the same branch (tcgen05.ld below is warp-collective)
    ok = __syncthreads_and(ok ? 1 : 0) != 0;
    if (!ok) {
      if (tid == 0) s_fail = 1;
      break;
    }
    tc_fence_after();
    const bool last = m + 1 == tp.nmat;
    // ops between this matrix and the next one (or the end of the program)
    const int sb = tp.mat_op[m] + 1, se = last ? p.nops : tp.mat_op[m + 1];
    const int j = tid;  // row = TMEM lane
    const bool row_ok = j < n;
    float* stg = bhi;  // output staging reuses the B_hi area once the last GEMM is done
    for (int cc = 0; cc < kNC / 32; ++cc) {
      float v[32];
      tmem_ld32(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)(m * kNC + cc * 32), v);
      if (row_ok) {
#pragma unroll
        for (int pp = 0; pp < 16; pp += 2) {
          float2 x0 = {v[2 * pp], v[2 * pp + 1]}, x1 = {v[2 * pp + 2], v[2 * pp + 3]};
          const int c0 = cc * 16 + pp;
          const int64_t idx0 = base + (int64_t)j * g.inner + c0;
          for (int oi = sb; oi < se; ++oi) {
            x0 = point_op(p, p.ops[oi], oi, x0, j, o, i0 + c0, idx0, acc, scale_v);
            x1 = point_op(p, p.ops[oi], oi, x1, j, o, i0 + c0 + 1, idx0 + 1, acc, scale_v);
          }
          if (last) {
            *reinterpret_cast<float4*>(stg + j * kStageRow + 2 * c0) = make_float4(x0.x, x0.y, x1.x, x1.y);
          } else {
            float h0, l0;
            split_tf32(x0.x, h0, l0);
            bhi[boff(2 * c0, j, L.sbo_b) >> 2] = h0;
            blo[boff(2 * c0, j, L.sbo_b) >> 2] = l0;
            split_tf32(x0.y, h0, l0);
            bhi[boff(2 * c0 + 1, j, L.sbo_b) >> 2] = h0;
            blo[boff(2 * c0 + 1, j, L.sbo_b) >> 2] = l0;
            split_tf32(x1.x, h0, l0);
            bhi[boff(2 * c0 + 2, j, L.sbo_b) >> 2] = h0;
            blo[boff(2 * c0 + 2, j, L.sbo_b) >> 2] = l0;
            split_tf32(x1.y, h0, l0);
            bhi[boff(2 * c0 + 3, j, L.sbo_b) >> 2] = h0;
            blo[boff(2 * c0 + 3, j, L.sbo_b) >> 2] = l0;
          }
        }
      }
    }
    fence_proxy_async();
    tc_fence_before();
    __syncthreads();
  }

  if (!s_fail) {
    // coalesced store of the staged tile: thread = complex column
    const int c = tid & (kBN - 1), h = tid >> 6;
    for (int k = h; k < n; k += 2) {
      const float2 v = *reinterpret_cast<const float2*>(bhi + k * kStageRow + 2 * c);
      psi[base + (int64_t)k * g.inner + c] = v;
    }
  }

  // ---- norm partials (fixed order) and last-CTA finalize
  for (int r = 0; r < p.nred; ++r) {
    const double t = block_sum128(acc[r], scratch);
    if (tid == 0) blk_red[r] = t;
  }
  __syncthreads();
  if (tid == 0) {
    if (s_fail && tp.error_slot >= 0) p.slots[tp.error_slot] = 1.0;
    for (int r = 0; r < p.nred; ++r) p.partials[(int64_t)r * g.tiles + tile] = blk_red[r];
    __threadfence();
    const unsigned int ticket = atomicAdd(p.counter, 1u);
    s_last = ticket == (unsigned int)(g.tiles - 1);
  }
  __syncthreads();
  if (s_last) {
    __threadfence();
    const int lane = tid & 31;
    for (int r = warp; r < p.nred; r += 4) {
      double v = 0.0;
      for (int64_t b = lane; b < g.tiles; b += 32) v += __ldcg(p.partials + (int64_t)r * g.tiles + b);
#pragma unroll
      for (int o2 = 16; o2 > 0; o2 >>= 1) v += __shfl_down_sync(0xffffffffu, v, o2);
      if (lane == 0) totals[r] = v;
    }
    __syncthreads();
    if (tid == 0) {
      for (int oi = 0; oi < p.nops; ++oi) run_scalar_tc(p, p.ops[oi], totals);
      __threadfence();
      *p.counter = 0u;
    }
  }

  // ---- teardown: outstanding copies (on failure), then tensor memory
  if (tid == 0 && s_fail) {
    // the producer may have copies in flight: wait (bounded) for both stages
    mbar_wait(&full[0], 0u, kWaitLimit);
    mbar_wait(&full[1], 0u, kWaitLimit);
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 0) tmem_dealloc(tmem, 256);
}

__global__ void __launch_bounds__(kThreads, 1) angular_tc_kernel(const __grid_constant__ TcParams tp) {
  tc_tile(tp, blockIdx.x);
}

// Many propagations' lane-matrix passes in one launch: block b runs tile
// (b - offsets[i]) of params[i], offsets[i] <= b < offsets[i + 1].
__global__ void __launch_bounds__(kThreads, 1) angular_tc_kernel_batched(const TcParams* __restrict__ params,
                                                                        const int64_t* __restrict__ offsets,
                                                                        int count) {
  const int64_t b = blockIdx.x;
  int lo = 0, hi = count - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (offsets[mid] <= b)
      lo = mid;
    else
      hi = mid - 1;
  }
  tc_tile(params[lo], b - offsets[lo]);
}

// ------------------------------------------------------------------ host side
size_t angular_tc_smem_bytes(int n) { return tc_layout(n).total; }

size_t tc_params_bytes() { return sizeof(TcParams); }

void make_tc_params(const PassParams& p, const int* mat_op, int nmat, const float* const* images, int error_slot,
                    void* out) {
  TcParams tp{};
  tp.p = p;
  tp.nmat = nmat;
  for (int i = 0; i < nmat; ++i) {
    tp.mat_op[i] = mat_op[i];
    tp.images[i] = images[i];
  }
  tp.error_slot = error_slot;
  std::memcpy(out, &tp, sizeof(TcParams));
}

cudaError_t launch_angular_tc_batched(const void* params_dev, const int64_t* offsets_dev, int count, int64_t blocks,
                                      size_t smem, cudaStream_t s) {
  static bool configured = false;
  if (!configured) {
    cudaError_t e =
        cudaFuncSetAttribute(angular_tc_kernel_batched, cudaFuncAttributeMaxDynamicSharedMemorySize, 220 * 1024);
    if (e != cudaSuccess) return e;
    configured = true;
  }
  if (smem > 220 * 1024) return cudaErrorInvalidValue;
  angular_tc_kernel_batched<<<(unsigned)blocks, kThreads, smem, s>>>(reinterpret_cast<const TcParams*>(params_dev),
                                                                     offsets_dev, count);
  count_launch();
  return cudaGetLastError();
}

bool angular_tc_eligible(const Geometry& g) {
  return (g.n == 32 || g.n == 64 || g.n == 128) && g.inner >= kBN && g.inner % kBN == 0;
}

// Chunk images of one real n x n matrix (row-major FP64) for the 3xTF32 A operand:
// per K chunk of 32, 16 KB of tf32-exact high parts then 16 KB of FP32 remainders,
// each in the K-major core-matrix order (row group stride 1024 B, K core stride 128 B).
void angular_tc_images(const double* m, int n, std::vector<float>& out) {
  const int nk = (n + kChunkK - 1) / kChunkK;
  out.assign((size_t)nk * 2 * (kChunkBytes / 4), 0.0f);
  for (int q = 0; q < nk; ++q) {
    float* hi = out.data() + (size_t)q * 2 * (kChunkBytes / 4);
    float* lo = hi + kChunkBytes / 4;
    for (int r = 0; r < kM; ++r)
      for (int kk = 0; kk < kChunkK; ++kk) {
        const int k = q * kChunkK + kk;
        double v = (r < n && k < n) ? m[(size_t)r * n + k] : 0.0;
        // nearest tf32 (10 explicit mantissa bits) of the FP64 value, then the FP32 remainder
        float f = (float)v;
        uint32_t b;
        std::memcpy(&b, &f, 4);
        b = (b + 0x1000u) & 0xFFFFE000u;
        float h;
        std::memcpy(&h, &b, 4);
        // remainder rounded to tf32 as well (the tensor core would truncate it)
        float l = (float)(v - (double)h);
        std::memcpy(&b, &l, 4);
        b = (b + 0x1000u) & 0xFFFFE000u;
        std::memcpy(&l, &b, 4);
        const size_t off = (size_t)(r >> 3) * 256 + (size_t)(kk >> 2) * 32 + (size_t)(r & 7) * 4 + (kk & 3);
        hi[off] = h;
        lo[off] = l;
      }
  }
}

cudaError_t launch_angular_tc(const PassParams& p, const int* mat_op, int nmat, const float* const* images,
                              int error_slot, cudaStream_t s) {
  TcParams tp{};
  tp.p = p;
  tp.nmat = nmat;
  for (int i = 0; i < nmat; ++i) {
    tp.mat_op[i] = mat_op[i];
    tp.images[i] = images[i];
  }
  tp.error_slot = error_slot;
  const size_t smem = angular_tc_smem_bytes((int)p.g.n);
  static bool configured = false;
  if (!configured) {
    cudaError_t e = cudaFuncSetAttribute(angular_tc_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, 220 * 1024);
    if (e != cudaSuccess) return e;
    configured = true;
  }
  if (smem > 220 * 1024) return cudaErrorInvalidValue;
  angular_tc_kernel<<<(unsigned)p.g.tiles, kThreads, smem, s>>>(tp);
  count_launch();
  return cudaGetLastError();
}

}  // namespace so
