// Angular (lane-matrix) sweep on the 5th-generation tensor cores, FP32 state.
//
// Replaces, fused into one pass, MatrixTransformation::transform /
// inverse_transform (matrix_transformation.rs:60-75) for real matrices -- the
// Legendre transforms of legendre_diagonalization.rs:13-45 -- together with the
// diagonal propagators, border damping and norm folds the step applies between
// and around them (n_dim_propagator.rs:32-36, one_dim_propagator.rs:37-46,
// border_dumping.rs:57-93, wave_function.rs:68-85).
//
// Layout: the state is stored [outer][n][inner] (n = lane axis, e.g. theta; inner =
// radial points).  A CTA owns a tile of BN complex columns of the inner axis for all
// n rows.  Treating (re, im) as two real columns, a lane-matrix product is the real
// GEMM D[M x 2BN] = A[M x n] . B[n x 2BN], A the (zero-padded) matrix, B the tile:
//   n <= 128: M = 128, BN = 64 (N = 128), A chunks of K = 32
//   n = 256 : M = 256 as two 128-row halves, BN = 32 (N = 64), A chunks of K = 16
// 3xTF32: A = A_hi + A_lo (split once from the FP64 matrix on the host), B = B_hi +
// B_lo (split on the fly), both parts tf32-exact, D = A_hi B_hi + A_hi B_lo + A_lo B_hi.
// The tensor core's FP32 accumulation truncates; to keep that bias small each K chunk
// group accumulates in its own TMEM region (up to 4) and the epilogue adds them with
// round-to-nearest FP32 adds.
//
//   prologue  (thread = column): load tile, pre-ops, split -> B_hi/B_lo (smem)
//   GEMM 1    (one thread issues tcgen05.mma; A chunks stream in by bulk TMA)
//   epilogue 1 (thread = row, tcgen05.ld from TMEM): mid-ops, split -> B for GEMM 2
//   GEMM 2
//   epilogue 2: post-ops -> staging -> coalesced store
//   FP64 norm partials folded by the last CTA in a fixed order (as lane_sweep.cu).
// Point-wise ops run on batches of 8-16 values per thread so each thread keeps that
// many table / state loads in flight.
// Every mbarrier wait is bounded (2 s); on a timeout the CTA records an error in a
// slot, waits (bounded) for its own copies, frees its tensor memory and returns.
#include "common.cuh"
#include "tc_common.cuh"

namespace so {

namespace {

constexpr int kChunkBytes = 16384;  // one of hi / lo: 128 rows x 32 K or 256 rows x 16 K
constexpr int kLboB = 144;          // B: core matrices along K (16 B padding vs 128)
constexpr uint64_t kWaitLimit = 2000000000ull;  // 2 s per wait
constexpr int kThreads = 256;

struct TcShape {
  int mh;        // 128-row halves of M
  int bn;        // complex columns per tile
  int nc;        // fp32 columns = MMA N
  int chunk_k;   // K per A chunk
  int nk;        // chunks per matrix
  int ksteps;    // K steps of 8 per matrix
  int reg_cols;  // TMEM columns of one accumulator region (all M halves)
  int nmain;     // regions for the A_hi B_hi products; one more region holds the corrections
  int sbo_a;     // A: row-group stride (bytes)
  int stage_row; // output staging row stride (floats)
  int groups;    // threads per column: 256 / bn
};

// The tensor core truncates its FP32 accumulation, so a region that accumulates t
// products is biased toward zero by about t/2 ulps.  The large A_hi B_hi products are
// spread over up to 7 regions (a couple of K steps each); the corrections A_hi B_lo +
// A_lo B_hi are 2^-11 smaller and share one region.
__host__ __device__ inline TcShape tc_shape(int n) {
  TcShape s{};
  s.mh = n == 256 ? 2 : 1;
  s.bn = 32;
  s.nc = 2 * s.bn;
  s.chunk_k = 32 / s.mh;
  s.nk = n / s.chunk_k;
  s.ksteps = n / 8;
  s.reg_cols = s.nc * s.mh;
  const int nreg = 512 / s.reg_cols;
  s.nmain = s.ksteps < nreg - 1 ? s.ksteps : nreg - 1;
  s.sbo_a = (s.chunk_k / 4) * 128;
  s.stage_row = s.nc + 4;
  s.groups = kThreads / s.bn;
  return s;
}

struct TcSmemLayout {
  uint32_t stage0, stage1, bhi, blo, bars, sbo_b, bbytes, total;
};

__host__ __device__ inline TcSmemLayout tc_layout(int n) {
  const TcShape s = tc_shape(n);
  TcSmemLayout L{};
  L.sbo_b = (uint32_t)(n / 4) * kLboB + 16;
  L.bbytes = (uint32_t)(s.nc / 8) * L.sbo_b;
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

__device__ double block_sum256(double v, double* scratch) {
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) v += __shfl_down_sync(0xffffffffu, v, off);
  if ((threadIdx.x & 31) == 0) scratch[threadIdx.x >> 5] = v;
  __syncthreads();
  double r = 0.0;
  if (threadIdx.x == 0)
    for (int w = 0; w < kThreads / 32; ++w) r += scratch[w];
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

// Per-tile factors of the point-wise ops, built once per tile so that the per-point
// work reads shared memory and does FP32 arithmetic only (FP64 runs on a narrow pipe).
struct TileTabs {
  float colw[kMaxRed][32];   // NORM: product of the FP32 weights of every non-lane axis, per tile column
  float2 colt[kMaxOps][32];  // DIAG1D on a non-lane axis: the table value of each tile column
  float scale[kMaxOps];      // SCALE: sqrt(target / norm)
};

__device__ __forceinline__ void build_tile_tabs(const PassParams& p, TileTabs& T, int64_t o, int64_t i0, int bn) {
  const Geometry& g = p.g;
  for (int idx = threadIdx.x; idx < p.nops * bn; idx += blockDim.x) {
    const int oi = idx / bn, c = idx - oi * bn;
    const DevOp& op = p.ops[oi];
    const int64_t i = i0 + c;
    if (op.kind == OP_NORM) {
      float w = 1.0f;
      for (int a = 0; a < g.ndim; ++a)
        if (a != g.sweep_axis) w *= __ldg(op.wf[a] + coord_of(g, a, o, i));
      T.colw[op.red][c] = w;
    } else if (op.kind == OP_DIAG1D && op.axis != g.sweep_axis) {
      T.colt[oi][c] = __ldg(reinterpret_cast<const float2*>(op.ptr) + coord_of(g, op.axis, o, i));
    } else if (op.kind == OP_SCALE && c == 0) {
      T.scale[oi] = (float)sqrt(__ldcg(p.slots + op.b) / __ldcg(p.slots + op.c));
    }
  }
}

// Point-wise ops [ob, oe) on the NB values of one lane-axis row j, tile columns
// c0 .. c0 + NB - 1 (storage indices ix0 .. ix0 + NB - 1): the epilogue layout.
template <int NB>
__device__ __forceinline__ void apply_row(const PassParams& p, const TileTabs& T, int ob, int oe, float2 (&v)[NB],
                                          int j, int c0, int64_t ix0, double* acc) {
  const Geometry& g = p.g;
  for (int oi = ob; oi < oe; ++oi) {
    const DevOp& op = p.ops[oi];
    switch (op.kind) {
      case OP_DIAG1D: {
        if (op.axis == g.sweep_axis) {
          const float2 t = __ldg(reinterpret_cast<const float2*>(op.ptr) + j);
#pragma unroll
          for (int u = 0; u < NB; ++u) v[u] = cmulf(v[u], t);
        } else {
#pragma unroll
          for (int u = 0; u < NB; ++u) v[u] = cmulf(v[u], T.colt[oi][c0 + u]);
        }
        break;
      }
      case OP_DIAGND: {
        const float2* t = reinterpret_cast<const float2*>(op.ptr) + ix0;
        if ((reinterpret_cast<uintptr_t>(t) & 15u) == 0) {
          float4 tv[NB / 2];
#pragma unroll
          for (int q = 0; q < NB / 2; ++q) tv[q] = __ldg(reinterpret_cast<const float4*>(t) + q);
#pragma unroll
          for (int q = 0; q < NB / 2; ++q) {
            v[2 * q] = cmulf(v[2 * q], make_float2(tv[q].x, tv[q].y));
            v[2 * q + 1] = cmulf(v[2 * q + 1], make_float2(tv[q].z, tv[q].w));
          }
        } else {
          float2 tv[NB];
#pragma unroll
          for (int u = 0; u < NB; ++u) tv[u] = __ldg(t + u);
#pragma unroll
          for (int u = 0; u < NB; ++u) v[u] = cmulf(v[u], tv[u]);
        }
        break;
      }
      case OP_SCALE: {
        const float f = T.scale[oi];
#pragma unroll
        for (int u = 0; u < NB; ++u) v[u] = {v[u].x * f, v[u].y * f};
        break;
      }
      case OP_NORM: {
        float s = 0.0f;
#pragma unroll
        for (int u = 0; u < NB; ++u) s = fmaf(fmaf(v[u].x, v[u].x, v[u].y * v[u].y), T.colw[op.red][c0 + u], s);
        acc[op.red] += (double)(s * __ldg(op.wf[g.sweep_axis] + j));
        break;
      }
      default:
        break;
    }
  }
}

// Point-wise ops [ob, oe) on the NB values of one tile column c, lane-axis rows jr[u]
// (storage indices ix[u]): the prologue layout.
template <int NB>
__device__ __forceinline__ void apply_col(const PassParams& p, const TileTabs& T, int ob, int oe, float2 (&v)[NB],
                                          const int (&jr)[NB], int c, const int64_t (&ix)[NB], double* acc) {
  const Geometry& g = p.g;
  for (int oi = ob; oi < oe; ++oi) {
    const DevOp& op = p.ops[oi];
    switch (op.kind) {
      case OP_DIAG1D: {
        const float2* t = reinterpret_cast<const float2*>(op.ptr);
        if (op.axis == g.sweep_axis) {
          float2 tv[NB];
#pragma unroll
          for (int u = 0; u < NB; ++u) tv[u] = __ldg(t + jr[u]);
#pragma unroll
          for (int u = 0; u < NB; ++u) v[u] = cmulf(v[u], tv[u]);
        } else {
          const float2 tc = T.colt[oi][c];
#pragma unroll
          for (int u = 0; u < NB; ++u) v[u] = cmulf(v[u], tc);
        }
        break;
      }
      case OP_DIAGND: {
        const float2* t = reinterpret_cast<const float2*>(op.ptr);
        float2 tv[NB];
#pragma unroll
        for (int u = 0; u < NB; ++u) tv[u] = __ldg(t + ix[u]);
#pragma unroll
        for (int u = 0; u < NB; ++u) v[u] = cmulf(v[u], tv[u]);
        break;
      }
      case OP_SCALE: {
        const float f = T.scale[oi];
#pragma unroll
        for (int u = 0; u < NB; ++u) v[u] = {v[u].x * f, v[u].y * f};
        break;
      }
      case OP_NORM: {
        const float* wr = op.wf[g.sweep_axis];
        float s = 0.0f;
#pragma unroll
        for (int u = 0; u < NB; ++u) s = fmaf(fmaf(v[u].x, v[u].x, v[u].y * v[u].y), __ldg(wr + jr[u]), s);
        acc[op.red] += (double)(s * T.colw[op.red][c]);
        break;
      }
      default:
        break;
    }
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
  const float* images[2]; // A chunk images per matrix: nk x (hi 16 KB, lo 16 KB)
  int32_t error_slot;
};

__device__ __forceinline__ void tc_tile(const TcParams& gtp, const int64_t tile) {
  using namespace tc;
  extern __shared__ __align__(1024) unsigned char sm[];
  __shared__ __align__(16) TcParams tp;
  __shared__ TileTabs tabs;
  __shared__ uint32_t tmem_base_s;
  __shared__ double scratch[kThreads / 32];
  __shared__ double blk_red[kMaxRed];
  __shared__ double totals[kMaxRed];
  __shared__ int s_last, s_fail;
  static_assert(sizeof(TcParams) % 4 == 0, "TcParams is copied as 32-bit words");
  for (int k = threadIdx.x; k < (int)(sizeof(TcParams) / 4); k += kThreads)
    reinterpret_cast<uint32_t*>(&tp)[k] = reinterpret_cast<const uint32_t*>(&gtp)[k];
  __syncthreads();
  const PassParams& p = tp.p;
  const Geometry& g = p.g;

  const int n = (int)g.n;
  const TcShape S = tc_shape(n);
  const TcSmemLayout L = tc_layout(n);
  unsigned char* stage[2] = {sm + L.stage0, sm + L.stage1};
  float* bhi = reinterpret_cast<float*>(sm + L.bhi);
  float* blo = reinterpret_cast<float*>(sm + L.blo);
  uint64_t* bars = reinterpret_cast<uint64_t*>(sm + L.bars);
  uint64_t* full = bars;       // [2]
  uint64_t* empty = bars + 2;  // [2]
  uint64_t* dbar = bars + 4;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int total_chunks = S.nk * tp.nmat;
  const uint32_t tmem_cols = 512u;

  const int64_t o = tile / g.tiles_per_outer;
  const int64_t i0 = (tile - o * g.tiles_per_outer) * S.bn;
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
  build_tile_tabs(p, tabs, o, i0, S.bn);
  if (warp == 0) tmem_alloc(&tmem_base_s, tmem_cols);
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = tmem_base_s;

  // A producer (thread 0): chunk c of the whole sequence -> stage c & 1
  auto issue_chunk = [&](int c) {
    const int m = c / S.nk, q = c - m * S.nk;
    const int s = c & 1;
    mbar_expect_tx(&full[s], 2u * kChunkBytes);
    bulk_g2s(stage[s], tp.images[m] + (size_t)q * 2 * (kChunkBytes / 4), 2u * kChunkBytes, &full[s]);
  };
  if (tid == 0) {
    issue_chunk(0);
    if (total_chunks > 1) issue_chunk(1);
  }

  double acc[kMaxRed];
#pragma unroll
  for (int r = 0; r < kMaxRed; ++r) acc[r] = 0.0;

  // ---- prologue: thread = complex column c, rows h, h + G, ... (G = groups)
  {
    const int c = tid % S.bn, h = tid / S.bn, G = S.groups;
    // a thread owns n / G rows (a multiple of 4 for every supported n): batches of 4
    for (int kb = h; kb < n; kb += 4 * G) {
      float2 v[4];
      int jr[4];
      int64_t ix[4];
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        jr[u] = kb + u * G;
        ix[u] = base + (int64_t)jr[u] * g.inner + c;
        v[u] = psi[ix[u]];
      }
      apply_col<4>(p, tabs, 0, tp.mat_op[0], v, jr, c, ix, acc);
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        float rh, rl, ih, il;
        split_tf32(v[u].x, rh, rl);
        split_tf32(v[u].y, ih, il);
        const uint32_t a0 = boff(2 * c, jr[u], L.sbo_b) >> 2, a1 = boff(2 * c + 1, jr[u], L.sbo_b) >> 2;
        bhi[a0] = rh;
        blo[a0] = rl;
        bhi[a1] = ih;
        blo[a1] = il;
      }
    }
  }
  fence_proxy_async();
  __syncthreads();

  const uint32_t idesc = idesc_tf32(128, (uint32_t)S.nc);
  // MMA issue for matrix m.  K step t (of ksteps) puts A_hi B_hi into main region
  // t * nmain / ksteps and the two corrections into the last region (nmain).
  auto run_gemm = [&](int m) -> bool {
    const int kpc = S.chunk_k / 8;  // K steps per chunk
    for (int q = 0; q < S.nk; ++q) {
      const int c = m * S.nk + q, s = c & 1;
      if (!mbar_wait(&full[s], (uint32_t)((c >> 1) & 1), kWaitLimit)) return false;
      tc_fence_after();
      for (int ks = 0; ks < kpc; ++ks) {
        const int t = q * kpc + ks;
        const int rm = t * S.nmain / S.ksteps;
        const bool first_main = t == 0 || rm != (t - 1) * S.nmain / S.ksteps;
        const int kg = q * S.chunk_k + ks * 8;
        const uint64_t bh = smem_desc(reinterpret_cast<unsigned char*>(bhi) + (kg >> 2) * kLboB, kLboB, L.sbo_b);
        const uint64_t bl = smem_desc(reinterpret_cast<unsigned char*>(blo) + (kg >> 2) * kLboB, kLboB, L.sbo_b);
        for (int hh = 0; hh < S.mh; ++hh) {
          const uint32_t dm = tmem + (uint32_t)(rm * S.reg_cols + hh * S.nc);
          const uint32_t dc = tmem + (uint32_t)(S.nmain * S.reg_cols + hh * S.nc);
          const int aoff = hh * 16 * S.sbo_a + ks * 256;
          const uint64_t ahi = smem_desc(stage[s] + aoff, 128, (uint32_t)S.sbo_a);
          const uint64_t alo = smem_desc(stage[s] + kChunkBytes + aoff, 128, (uint32_t)S.sbo_a);
          mma_tf32(dm, ahi, bh, idesc, first_main ? 0u : 1u);
          mma_tf32(dc, ahi, bl, idesc, t == 0 ? 0u : 1u);
          mma_tf32(dc, alo, bh, idesc, 1u);
        }
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

  // epilogue mapping: warp w reads TMEM lanes 32 (w & 3) .. +31; upper warps take the
  // second 16-column chunk (n <= 128) or the second 128-row half (n = 256, both chunks)
  const int lg = warp & 3, up = warp >> 2;
  const int j = (S.mh == 2 ? 128 * up : 0) + 32 * lg + lane;  // lane-axis row
  const bool row_ok = j < n;
  float* stg = bhi;  // output staging reuses the B_hi area once the last GEMM is done

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
    for (int cc = 0; cc < S.mh; ++cc) {
      const int ch = S.mh == 1 ? up : cc;  // 16-column chunk of this thread
      const uint32_t col = (uint32_t)((S.mh == 2 ? S.nc * up : 0) + 32 * ch);
      const uint32_t lane_addr = tmem + ((uint32_t)(lg * 32) << 16) + col;
      // main regions in order, then the correction region; round-to-nearest FP32 adds
      float v[32];
      tmem_ld32(lane_addr, v);
      for (int r = 1; r <= S.nmain; ++r) {
        float w2[32];
        tmem_ld32(lane_addr + (uint32_t)(r * S.reg_cols), w2);
#pragma unroll
        for (int e = 0; e < 32; ++e) v[e] += w2[e];
      }
      if (row_ok) {
        const int c0 = 16 * ch;  // complex column of v[0..1]
        float2 x[16];
#pragma unroll
        for (int u = 0; u < 16; ++u) x[u] = {v[2 * u], v[2 * u + 1]};
        apply_row<16>(p, tabs, sb, se, x, j, c0, base + (int64_t)j * g.inner + c0, acc);
        if (last) {
#pragma unroll
          for (int u = 0; u < 16; u += 2)
            *reinterpret_cast<float4*>(stg + j * S.stage_row + 2 * (c0 + u)) =
                make_float4(x[u].x, x[u].y, x[u + 1].x, x[u + 1].y);
        } else {
#pragma unroll
          for (int u = 0; u < 16; ++u) {
            float h0, l0;
            const int q = 2 * (c0 + u);
            split_tf32(x[u].x, h0, l0);
            bhi[boff(q, j, L.sbo_b) >> 2] = h0;
            blo[boff(q, j, L.sbo_b) >> 2] = l0;
            split_tf32(x[u].y, h0, l0);
            bhi[boff(q + 1, j, L.sbo_b) >> 2] = h0;
            blo[boff(q + 1, j, L.sbo_b) >> 2] = l0;
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
    const int c = tid % S.bn, h = tid / S.bn, G = S.groups;
    for (int kb = h; kb < n; kb += 4 * G) {
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        const int k = kb + u * G;
        psi[base + (int64_t)k * g.inner + c] = *reinterpret_cast<const float2*>(stg + k * S.stage_row + 2 * c);
      }
    }
  }

  // ---- norm partials (fixed order) and last-CTA finalize
  for (int r = 0; r < p.nred; ++r) {
    const double t = block_sum256(acc[r], scratch);
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
    for (int r = warp; r < p.nred; r += kThreads / 32) {
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
    mbar_wait(&full[0], 0u, kWaitLimit);
    mbar_wait(&full[1], 0u, kWaitLimit);
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 0) tmem_dealloc(tmem, tmem_cols);
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

int angular_tc_columns(int n) { return tc_shape(n).bn; }

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

// the largest dynamic shared memory any supported lane extent asks for
static size_t tc_max_dynamic_smem() { return tc_layout(256).total; }

static bool configure_once(const void* kern, bool& flag) {
  if (flag) return true;
  if (cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)tc_max_dynamic_smem()) !=
      cudaSuccess)
    return false;
  flag = true;
  return true;
}

cudaError_t launch_angular_tc_batched(const void* params_dev, const int64_t* offsets_dev, int count, int64_t blocks,
                                      size_t smem, cudaStream_t s) {
  static bool configured = false;
  if (!configure_once((const void*)angular_tc_kernel_batched, configured)) return cudaGetLastError();
  if (smem > tc_max_dynamic_smem()) return cudaErrorInvalidValue;
  angular_tc_kernel_batched<<<(unsigned)blocks, kThreads, smem, s>>>(reinterpret_cast<const TcParams*>(params_dev),
                                                                     offsets_dev, count);
  count_launch();
  return cudaGetLastError();
}

bool angular_tc_eligible(const Geometry& g) {
  if (!(g.n == 32 || g.n == 64 || g.n == 128 || g.n == 256)) return false;
  const int bn = tc_shape((int)g.n).bn;
  return g.inner >= bn && g.inner % bn == 0;
}

// Chunk images of one real n x n matrix (row-major FP64) for the 3xTF32 A operand: per
// K chunk, 16 KB of tf32-exact high parts then 16 KB of tf32-exact remainders, each in
// the K-major core-matrix order (row-group stride sbo_a, K core-matrix stride 128 B).
void angular_tc_images(const double* m, int n, std::vector<float>& out) {
  const TcShape S = tc_shape(n);
  const int rows = 128 * S.mh;
  out.assign((size_t)S.nk * 2 * (kChunkBytes / 4), 0.0f);
  auto tf32 = [](float x) {
    uint32_t b;
    std::memcpy(&b, &x, 4);
    b = (b + 0x1000u) & 0xFFFFE000u;
    float r;
    std::memcpy(&r, &b, 4);
    return r;
  };
  for (int q = 0; q < S.nk; ++q) {
    float* hi = out.data() + (size_t)q * 2 * (kChunkBytes / 4);
    float* lo = hi + kChunkBytes / 4;
    for (int r = 0; r < rows; ++r)
      for (int kk = 0; kk < S.chunk_k; ++kk) {
        const int k = q * S.chunk_k + kk;
        const double v = (r < n && k < n) ? m[(size_t)r * n + k] : 0.0;
        const float h = tf32((float)v);
        const float l = tf32((float)(v - (double)h));  // the tensor core would truncate an unrounded remainder
        const size_t off = (size_t)(r >> 3) * (S.sbo_a / 4) + (size_t)(kk >> 2) * 32 + (size_t)(r & 7) * 4 + (kk & 3);
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
  if (!configure_once((const void*)angular_tc_kernel, configured)) return cudaGetLastError();
  if (smem > tc_max_dynamic_smem()) return cudaErrorInvalidValue;
  angular_tc_kernel<<<(unsigned)p.g.tiles, kThreads, smem, s>>>(tp);
  count_launch();
  return cudaGetLastError();
}

}  // namespace so
