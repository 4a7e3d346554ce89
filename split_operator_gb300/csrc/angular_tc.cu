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

constexpr int kChunkBytes = 8192;   // one of hi / lo: 128 rows x 16 K or 256 rows x 8 K
constexpr int kLboB = 144;          // B: core matrices along K (16 B padding vs 128)
constexpr uint64_t kWaitLimit = 2000000000ull;  // 2 s per wait
constexpr int kWorkThreads = 256;            // warps 0-7: loads, point-wise ops, TMEM drains, stores
constexpr int kThreads = kWorkThreads + 32;  // warp 8: A-chunk TMA producer and MMA issuer (one lane)
constexpr uint32_t kTmemCols = 256;  // half of the SM's tensor memory: two CTAs share an SM
constexpr int kRegions = 4;          // 64-column accumulator regions in kTmemCols
constexpr int kFillSteps = 6;        // K steps between two drains of the main regions
constexpr int kColtSlots = 4;        // DIAG1D ops on a non-lane axis per pass

struct TcShape {
  int mh;        // 128-row halves of M
  int bn;        // complex columns per tile
  int nc;        // fp32 columns = MMA N
  int chunk_k;   // K per A chunk
  int nk;        // chunks per matrix
  int ksteps;    // K steps of 8 per matrix
  int reg_cols;  // TMEM columns of one accumulator region (all M halves)
  int nmain;     // regions for the A_hi B_hi products; one more region holds the corrections
  int fills;     // drains of the main regions per matrix
  int sbo_a;     // A: row-group stride (bytes)
  int stage_row; // output staging row stride (floats)
  int groups;    // work threads per column: 256 / bn
};

// The tensor core truncates its FP32 accumulation, so a region that accumulates t
// products is biased toward zero by about t/2 ulps.  The large A_hi B_hi products go
// to three regions, a couple of K steps each; every kFillSteps K steps the regions are
// drained into registers (round-to-nearest adds) and start again from zero.  The
// corrections A_hi B_lo + A_lo B_hi are 2^-11 smaller and share the fourth region.
//   n <= 128: M = 128, BN = 32 (N = 64), A chunks of K = 16
//   n = 256 : M = 256 as two 128-row halves, BN = 16 (N = 32), A chunks of K = 8
__host__ __device__ inline TcShape tc_shape(int n) {
  TcShape s{};
  s.mh = n == 256 ? 2 : 1;
  s.bn = n == 256 ? 16 : 32;
  s.nc = 2 * s.bn;
  s.chunk_k = 16 / s.mh;
  s.nk = n / s.chunk_k;
  s.ksteps = n / 8;
  s.reg_cols = s.nc * s.mh;
  s.nmain = kRegions - 1;
  s.fills = (s.ksteps + kFillSteps - 1) / kFillSteps;
  s.sbo_a = (s.chunk_k / 4) * 128;
  s.stage_row = s.nc + 4;
  s.groups = kWorkThreads / s.bn;
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

// Float-float (hi + lo) arithmetic: about 48 significant bits from FP32 operations
// (Knuth's two-sum), used for the block-level norm folds -- this GPU's FP64 pipe is
// narrow enough that a few FP64 shuffle reductions per tile cost more than the tile.
struct FF {
  float hi, lo;
};

__device__ __forceinline__ FF ff_add(FF a, FF b) {
  const float s = a.hi + b.hi;
  const float bb = s - a.hi;
  const float e = (a.hi - (s - bb)) + (b.hi - bb) + a.lo + b.lo;
  const float hi = s + e;
  return {hi, e - (hi - s)};
}

// fixed-order sum of one float per thread over the whole block, in float-float;
// valid in thread 0
__device__ FF block_sum(float v, FF* scratch) {
  FF a{v, 0.0f};
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) {
    const FF b{__shfl_down_sync(0xffffffffu, a.hi, off), __shfl_down_sync(0xffffffffu, a.lo, off)};
    a = ff_add(a, b);
  }
  if ((threadIdx.x & 31) == 0) scratch[threadIdx.x >> 5] = a;
  __syncthreads();
  FF r{0.0f, 0.0f};
  if (threadIdx.x == 0)
    for (int w = 0; w < kThreads / 32; ++w) r = ff_add(r, scratch[w]);
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
  float2 colt[kColtSlots][32];  // DIAG1D on a non-lane axis: the table value of each tile column
  float scale[kMaxOps];         // SCALE: sqrt(target / norm)
  int8_t slot[kMaxOps];         // DIAG1D on a non-lane axis: its colt row
};

__host__ __device__ inline bool diag1d_across(const DevOp& op, int sweep_axis) {
  return op.kind == OP_DIAG1D && op.axis != sweep_axis;
}

__device__ __forceinline__ void build_tile_tabs(const PassParams& p, TileTabs& T, int64_t o, int64_t i0, int bn) {
  const Geometry& g = p.g;
  if ((int)threadIdx.x < p.nops) {
    int k = 0;
    for (int q = 0; q < (int)threadIdx.x; ++q) k += diag1d_across(p.ops[q], g.sweep_axis);
    T.slot[threadIdx.x] = (int8_t)k;
  }
  __syncthreads();
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
      T.colt[T.slot[oi]][c] = __ldg(reinterpret_cast<const float2*>(op.ptr) + coord_of(g, op.axis, o, i));
    } else if (op.kind == OP_SCALE && c == 0) {
      T.scale[oi] = (float)sqrt(__ldcg(p.slots + op.b) / __ldcg(p.slots + op.c));
    }
  }
}

// Point-wise ops [ob, oe) on the NB values of one lane-axis row j, tile columns
// c0 .. c0 + NB - 1 (storage indices ix0 .. ix0 + NB - 1): the epilogue layout.
// rw_val is this row's weight in the row-weight vector rw_ptr (loaded ahead of time).
template <int NB>
__device__ __forceinline__ void apply_row(const PassParams& p, const TileTabs& T, int ob, int oe, float2 (&v)[NB],
                                          int j, int c0, int64_t ix0, float* acc, const float* rw_ptr,
                                          float rw_val) {
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
          for (int u = 0; u < NB; ++u) v[u] = cmulf(v[u], T.colt[T.slot[oi]][c0 + u]);
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
        const float* wr = op.wf[g.sweep_axis];
        acc[op.red] += s * (wr == rw_ptr ? rw_val : __ldg(wr + j));
        break;
      }
      default:
        break;
    }
  }
}

// Point-wise ops [ob, oe) on the NB values of one tile column c, lane-axis rows
// j0 + u G (storage indices ix0 + u rstride): the prologue layout.
template <int NB>
__device__ __forceinline__ void apply_col(const PassParams& p, const TileTabs& T, int ob, int oe, float2 (&v)[NB],
                                          int j0, int G, int c, int64_t ix0, int64_t rstride, float* acc) {
  const Geometry& g = p.g;
  for (int oi = ob; oi < oe; ++oi) {
    const DevOp& op = p.ops[oi];
    switch (op.kind) {
      case OP_DIAG1D: {
        const float2* t = reinterpret_cast<const float2*>(op.ptr);
        if (op.axis == g.sweep_axis) {
          float2 tv[NB];
#pragma unroll
          for (int u = 0; u < NB; ++u) tv[u] = __ldg(t + j0 + u * G);
#pragma unroll
          for (int u = 0; u < NB; ++u) v[u] = cmulf(v[u], tv[u]);
        } else {
          const float2 tc = T.colt[T.slot[oi]][c];
#pragma unroll
          for (int u = 0; u < NB; ++u) v[u] = cmulf(v[u], tc);
        }
        break;
      }
      case OP_DIAGND: {
        const float2* t = reinterpret_cast<const float2*>(op.ptr);
        float2 tv[NB];
#pragma unroll
        for (int u = 0; u < NB; ++u) tv[u] = __ldg(t + ix0 + u * rstride);
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
        for (int u = 0; u < NB; ++u) s = fmaf(fmaf(v[u].x, v[u].x, v[u].y * v[u].y), __ldg(wr + j0 + u * G), s);
        acc[op.red] += s * T.colw[op.red][c];
        break;
      }
      default:
        break;
    }
  }
}

// Prologue of one thread (tile column c, rows h, h + G, ...): loads, the ops before the
// first lane matrix, and the split into the B_hi / B_lo operand images.
template <int NB>
__device__ __forceinline__ void prologue_rows(const PassParams& p, const TileTabs& T, int oe, const float2* psi,
                                              int64_t base, int c, int h, int G, int n, float* bhi, float* blo,
                                              uint32_t sbo_b, float* acc) {
  const int64_t rstride = (int64_t)G * p.g.inner;
  for (int kb = h; kb < n; kb += NB * G) {
    const int64_t ix0 = base + (int64_t)kb * p.g.inner + c;
    float2 v[NB];
#pragma unroll
    for (int u = 0; u < NB; ++u) v[u] = psi[ix0 + u * rstride];
    apply_col<NB>(p, T, 0, oe, v, kb, G, c, ix0, rstride, acc);
#pragma unroll
    for (int u = 0; u < NB; ++u) {
      const int j = kb + u * G;
      float rh, rl, ih, il;
      tc::split_tf32(v[u].x, rh, rl);
      tc::split_tf32(v[u].y, ih, il);
      const uint32_t a0 = boff(2 * c, j, sbo_b) >> 2, a1 = boff(2 * c + 1, j, sbo_b) >> 2;
      bhi[a0] = rh;
      blo[a0] = rl;
      bhi[a1] = ih;
      blo[a1] = il;
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
  const float* images[2]; // A chunk images per matrix: nk x (hi 8 KB, lo 8 KB)
  int32_t error_slot;
  unsigned long long* trace;  // optional phase timestamps, kTraceSlots per tile (nullptr: off)
};

// Phase timestamps (%globaltimer, ns) of the optional trace, per tile.
enum TraceSlot {
  TR_START, TR_SETUP, TR_PROLOGUE, TR_DRAIN0, TR_MAT0, TR_EPI0, TR_MAT1, TR_EPI1, TR_JOIN, TR_STORE, TR_NORMS,
  TR_TICKET, TR_END, TR_CHUNK0, TR_ISSUE0, TR_ISSUE1,
  TR_TMA4, TR_FULL4, TR_MMA4, TR_DONE4,  // chunk 4: copy issued, landed, MMAs issued, MMAs completed
  kTraceSlots
};
__device__ __forceinline__ void trace_mark(const TcParams& tp, int64_t tile, int slot) {
  if (tp.trace) tp.trace[tile * kTraceSlots + slot] = tc::globaltimer_ns();
}

// The producer / MMA lane.  A chunks (hi 8 KB + lo 8 KB) stream through two stages by bulk
// TMA; for each matrix (once its B operand is written) and each fill it issues the K
// steps of the fill -- step t puts A_hi B_hi into main region (t - t0) nused / span and
// both corrections into the correction region -- and commits the fill to dbar.  Once the
// MMAs of chunk c complete, its stage is refilled with chunk c + 2.
// Every wait is bounded; on a failure it waits (bounded) for the copies and MMAs already
// issued and returns false.  Chunks 0 .. preissued-1 were issued at kernel entry.
__device__ __noinline__ bool mma_producer(const TcShape S, const TcSmemLayout L, uint32_t sm0, const float* img0,
                                          const float* img1, int nmat, uint32_t tmem, unsigned long long* tr,
                                          int preissued) {
  using namespace tc;
  uint64_t* bars = reinterpret_cast<uint64_t*>(sm_ptr(sm0 + L.bars));
  uint64_t* full = bars;
  uint64_t* empty = bars + 2;
  uint64_t* dbar = bars + 4;
  uint64_t* freebar = bars + 5;
  uint64_t* bready = bars + 6;
  uint64_t* quiet = bars + 7;
  const int total_chunks = S.nk * nmat;
  const uint32_t stage_bytes = 2u * kChunkBytes;
  int issued = 0, landed = 0;
  auto issue_chunk = [&](int c) {
    const int m = c / S.nk, q = c - m * S.nk;
    const int s = c & 1;
    if (tr && c == 4) tr[TR_TMA4] = globaltimer_ns();
    mbar_expect_tx(&full[s], stage_bytes);
    bulk_g2s(sm_ptr(sm0 + L.stage0 + (uint32_t)s * stage_bytes), (m == 0 ? img0 : img1) + (size_t)q * 2 * (kChunkBytes / 4),
             stage_bytes, &full[s]);
    issued = c + 1;
  };
  const uint32_t idesc = idesc_tf32(128, (uint32_t)S.nc);
  const uint64_t bbits = smem_desc_bits(kLboB, L.sbo_b), abits = smem_desc_bits(128, (uint32_t)S.sbo_a);
  const int kpc = S.chunk_k / 8;  // K steps per chunk
  bool ok = true;
  issued = preissued;  // chunks 0 and 1 went out at kernel entry
  int nfree = 0;
  for (int m = 0; m < nmat && ok; ++m) {
    ok = mbar_wait(bready, (uint32_t)(m & 1), kWaitLimit);
    tc_fence_after();
    for (int f = 0; f < S.fills && ok; ++f) {
      if (f > 0) {
        ok = mbar_wait(freebar, (uint32_t)(nfree & 1), kWaitLimit);
        ++nfree;
        tc_fence_after();
        if (!ok) break;
      }
      const int t0 = f * S.ksteps / S.fills, t1 = (f + 1) * S.ksteps / S.fills;
      const int span = t1 - t0, nused = span < S.nmain ? span : S.nmain;
      for (int t = t0; t < t1 && ok; ++t) {
        const int q = t / kpc, ks = t - q * kpc;
        const int c = m * S.nk + q, s = c & 1;
        if (ks == 0) {
          ok = mbar_wait(&full[s], (uint32_t)((c >> 1) & 1), kWaitLimit);
          if (!ok) break;
          if (tr && c == 0) tr[TR_CHUNK0] = globaltimer_ns();
          if (tr && c == 4) tr[TR_FULL4] = globaltimer_ns();
          landed = c + 1;
          tc_fence_after();
        }
        const int rm = (t - t0) * nused / span;
        const bool first_main = t == t0 || rm != (t - 1 - t0) * nused / span;
        const uint32_t kb = (uint32_t)(((q * S.chunk_k + ks * 8) >> 2) * kLboB);
        const uint64_t bh = smem_desc_at(bbits, sm0 + L.bhi + kb), bl = smem_desc_at(bbits, sm0 + L.blo + kb);
        const uint32_t st = sm0 + L.stage0 + (uint32_t)s * stage_bytes + (uint32_t)(ks * 256);
        for (int hh = 0; hh < S.mh; ++hh) {
          const uint32_t dm = tmem + (uint32_t)(rm * S.reg_cols + hh * S.nc);
          const uint32_t dc = tmem + (uint32_t)(S.nmain * S.reg_cols + hh * S.nc);
          const uint32_t aoff = st + (uint32_t)(hh * 16 * S.sbo_a);
          mma_tf32(dm, smem_desc_at(abits, aoff), bh, idesc, first_main ? 0u : 1u);
          mma_tf32(dc, smem_desc_at(abits, aoff), bl, idesc, t == 0 ? 0u : 1u);
          mma_tf32(dc, smem_desc_at(abits, aoff + kChunkBytes), bh, idesc, 1u);
        }
        if (ks == kpc - 1) {
          // refill this stage with chunk c + 2 as soon as the MMAs reading it complete, so
          // that both stages always have a copy in flight
          mma_commit(&empty[s]);
          if (tr && c == 4) tr[TR_MMA4] = globaltimer_ns();
          if (c + 2 < total_chunks) {
            ok = mbar_wait(&empty[s], (uint32_t)((c >> 1) & 1), kWaitLimit);
            if (tr && c == 4) tr[TR_DONE4] = globaltimer_ns();
            if (ok) issue_chunk(c + 2);
          }
        }
      }
      if (ok) mma_commit(dbar);
    }
    if (tr && m < 2) tr[TR_ISSUE0 + m] = globaltimer_ns();
  }
  if (!ok) {
    // let every copy and MMA already issued finish before the CTA lets go of its memory
    for (int c = landed; c < issued; ++c) mbar_wait(&full[c & 1], (uint32_t)((c >> 1) & 1), kWaitLimit);
    mma_commit(quiet);
    mbar_wait(quiet, 0u, kWaitLimit);
  }
  return ok;
}

__device__ __forceinline__ void tc_tile(const TcParams& gtp, const int64_t tile) {
  using namespace tc;
  extern __shared__ __align__(1024) unsigned char sm[];
  __shared__ __align__(16) TcParams tp;
  __shared__ TileTabs tabs;
  __shared__ uint32_t tmem_base_s;
  __shared__ FF scratch[kThreads / 32];
  __shared__ double blk_red[kMaxRed];
  __shared__ double totals[kMaxRed];
  __shared__ int s_last;
  __shared__ volatile int s_fail;
  static_assert(sizeof(TcParams) % 4 == 0, "TcParams is copied as 32-bit words");
  // every supported lane extent has nk >= 2 chunks per matrix: chunks 0 and 1 go out here
  if (threadIdx.x == kWorkThreads) {
    // producer lane: barriers, then the first two A chunks, before anything else
    const TcSmemLayout L0 = tc_layout((int)gtp.p.g.n);
    uint64_t* b0 = reinterpret_cast<uint64_t*>(sm + L0.bars);
    for (int k = 0; k < 5; ++k) tc::mbar_init(b0 + k, 1);  // full[2], empty[2], dbar
    tc::mbar_init(b0 + 5, kWorkThreads);                   // freebar
    tc::mbar_init(b0 + 6, kWorkThreads);                   // bready
    tc::mbar_init(b0 + 7, 1);                              // quiet
    tc::fence_mbar_init();
    const float* img0 = gtp.images[0];
    for (int c = 0; c < 2; ++c) {
      tc::mbar_expect_tx(b0 + c, 2u * kChunkBytes);
      tc::bulk_g2s(sm + L0.stage0 + c * 2 * kChunkBytes, img0 + (size_t)c * 2 * (kChunkBytes / 4), 2u * kChunkBytes,
                   b0 + c);
    }
    // the rest of the A sequence toward L2 now: the CTAs of a pass walk it in lock step,
    // and a chunk that is not yet in L2 costs each of them a DRAM round trip
    const int nk = tc_shape((int)gtp.p.g.n).nk;
    for (int m = 0; m < gtp.nmat; ++m)
      for (int q = m == 0 ? 2 : 0; q < nk; ++q)
        tc::prefetch_l2(gtp.images[m] + (size_t)q * 2 * (kChunkBytes / 4), 2u * kChunkBytes);
  }
  for (int k = threadIdx.x; k < (int)(sizeof(TcParams) / 4); k += kThreads)
    reinterpret_cast<uint32_t*>(&tp)[k] = reinterpret_cast<const uint32_t*>(&gtp)[k];
  __syncthreads();
  if (threadIdx.x == 0) trace_mark(tp, tile, TR_START);
  const PassParams& p = tp.p;
  const Geometry& g = p.g;

  const int n = (int)g.n;
  const TcShape S = tc_shape(n);
  const TcSmemLayout L = tc_layout(n);
  float* bhi = reinterpret_cast<float*>(sm + L.bhi);
  float* blo = reinterpret_cast<float*>(sm + L.blo);
  uint64_t* bars = reinterpret_cast<uint64_t*>(sm + L.bars);
  // bars: full[2] (A chunk landed), empty[2] (MMAs reading a stage completed), then:
  uint64_t* dbar = bars + 4;     // MMAs of a fill completed (work warps drain)
  uint64_t* freebar = bars + 5;  // work warps drained a fill (regions free again)
  uint64_t* bready = bars + 6;   // B operand of the next matrix written
  // bars + 7: every MMA issued has completed (producer failure path)
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;

  const int64_t o = tile / g.tiles_per_outer;
  const int64_t i0 = (tile - o * g.tiles_per_outer) * S.bn;
  const int64_t base = o * g.n * g.inner + i0;  // element (row 0, column 0) of the tile
  float2* psi = reinterpret_cast<float2*>(p.psi);

  if (tid == 0) s_fail = 0;
  build_tile_tabs(p, tabs, o, i0, S.bn);
  // full-size tables read after the first lane matrix: start their tile rows toward L2
  // now, so the epilogue loads do not wait for DRAM
  for (int oi = tp.mat_op[0] + 1; oi < p.nops; ++oi) {
    const DevOp& op = p.ops[oi];
    if (op.kind != OP_DIAGND) continue;
    bool seen = false;
    for (int q = tp.mat_op[0] + 1; q < oi; ++q) seen |= p.ops[q].kind == OP_DIAGND && p.ops[q].ptr == op.ptr;
    const float2* t = reinterpret_cast<const float2*>(op.ptr) + base;
    if (!seen && (reinterpret_cast<uintptr_t>(t) & 15u) == 0)
      for (int j = tid; j < n; j += kThreads) prefetch_l2(t + (int64_t)j * g.inner, (uint32_t)(S.bn * sizeof(float2)));
  }
  if (warp == 0) tmem_alloc(&tmem_base_s, kTmemCols);
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = tmem_base_s;
  if (tid == 0) trace_mark(tp, tile, TR_SETUP);

  // per-thread FP32 partial sums of the norms (at most a few dozen terms each); the
  // block folds them in float-float and the last CTA in FP64
  float acc[kMaxRed];
#pragma unroll
  for (int r = 0; r < kMaxRed; ++r) acc[r] = 0.0f;

  if (warp == kWorkThreads / 32) {
    // ================= producer / MMA warp (lane 0)
    if (lane == 0 && !mma_producer(S, L, smem_u32(sm), tp.images[0], tp.images[1], tp.nmat, tmem,
                                   tp.trace ? tp.trace + tile * kTraceSlots : nullptr, 2))
      s_fail = 1;
  } else {
    // ================= work warps
    {
      // prologue: thread = complex column c, rows h, h + G, ... (G = groups); a thread owns
      // n / G rows (4, 8, 16 or 32) and keeps the loads of a batch in flight together
      const int c = tid % S.bn, h = tid / S.bn, G = S.groups;
      if (n / G >= 16)
        prologue_rows<16>(p, tabs, tp.mat_op[0], psi, base, c, h, G, n, bhi, blo, L.sbo_b, acc);
      else if (n / G >= 8)
        prologue_rows<8>(p, tabs, tp.mat_op[0], psi, base, c, h, G, n, bhi, blo, L.sbo_b, acc);
      else
        prologue_rows<4>(p, tabs, tp.mat_op[0], psi, base, c, h, G, n, bhi, blo, L.sbo_b, acc);
      fence_proxy_async();
      mbar_arrive(bready);
      if (tid == 0) trace_mark(tp, tile, TR_PROLOGUE);
    }
    // drain mapping: warp w reads TMEM lanes 32 (w & 3) .. +31 and one 32-column slice:
    // n <= 128: the upper warps take the second slice of N = 64; n = 256: the upper warps
    // take the second 128-row half (N = 32)
    const int lg = warp & 3, up = warp >> 2;
    const int j = (S.mh == 2 ? 128 * up : 0) + 32 * lg + lane;  // lane-axis row
    const bool row_ok = j < n;
    const uint32_t slice = (uint32_t)(S.mh == 2 ? S.nc * up : 32 * up);
    const int c0 = S.mh == 2 ? 0 : 16 * up;  // complex column of v[0..1]
    const uint32_t lane_addr = tmem + ((uint32_t)(lg * 32) << 16) + slice;
    float* stg = bhi;  // output staging reuses the B_hi area once the last GEMM is done
    int drains = 0;    // completed phases of dbar
    // the lane-axis weight of this row for the norms after the first matrix, loaded now
    // (it arrives while the GEMM runs)
    const float* rw_ptr = nullptr;
    float rw_val = 0.0f;
    for (int oi = tp.mat_op[0] + 1; oi < p.nops && rw_ptr == nullptr; ++oi)
      if (p.ops[oi].kind == OP_NORM) rw_ptr = p.ops[oi].wf[g.sweep_axis];
    if (rw_ptr && row_ok) rw_val = __ldg(rw_ptr + j);
    for (int m = 0; m < tp.nmat; ++m) {
      float v[32];
#pragma unroll
      for (int e = 0; e < 32; ++e) v[e] = 0.0f;
      bool ok = true;
      for (int f = 0; f < S.fills; ++f) {
        ok = mbar_wait(dbar, (uint32_t)(drains & 1), kWaitLimit);
        ok = __all_sync(0xffffffffu, ok);  // tcgen05.ld below is warp-collective
        if (!ok) break;
        ++drains;
        tc_fence_after();
        // main regions of this fill, then (after the last fill) the correction region;
        // round-to-nearest FP32 adds in a fixed order
        const int t0 = f * S.ksteps / S.fills, t1 = (f + 1) * S.ksteps / S.fills;
        const int nused = (t1 - t0) < S.nmain ? (t1 - t0) : S.nmain;
        // regions 0 .. nused-1 of the fill, then after the last fill the correction region
        const int nr = nused + (f + 1 == S.fills ? 1 : 0);
#pragma unroll 1
        for (int k = 0; k < nr; ++k) {
          const int r = k < nused ? k : S.nmain;
          float w2[16];
          tmem_ld16(lane_addr + (uint32_t)(r * S.reg_cols), w2);
#pragma unroll
          for (int e = 0; e < 16; ++e) v[e] += w2[e];
          tmem_ld16(lane_addr + (uint32_t)(r * S.reg_cols + 16), w2);
#pragma unroll
          for (int e = 0; e < 16; ++e) v[16 + e] += w2[e];
        }
        tc_fence_before();
        if (f + 1 < S.fills) mbar_arrive(freebar);
        if (tid == 0 && m == 0 && f == 0) trace_mark(tp, tile, TR_DRAIN0);
      }
      if (tid == 0 && m < 2) trace_mark(tp, tile, TR_MAT0 + 2 * m);
      if (!ok) {
        s_fail = 1;
        break;
      }
      const bool last = m + 1 == tp.nmat;
      // ops between this matrix and the next one (or the end of the program)
      const int sb = tp.mat_op[m] + 1, se = last ? p.nops : tp.mat_op[m + 1];
      // two halves of 8 complex columns
#pragma unroll
      for (int hv = 0; hv < 2; ++hv) {
        if (!row_ok) break;
        float2 x[8];
#pragma unroll
        for (int u = 0; u < 8; ++u) x[u] = {v[16 * hv + 2 * u], v[16 * hv + 2 * u + 1]};
        const int cb = c0 + 8 * hv;
        apply_row<8>(p, tabs, sb, se, x, j, cb, base + (int64_t)j * g.inner + cb, acc, rw_ptr, rw_val);
        if (last) {
#pragma unroll
          for (int u = 0; u < 8; u += 2)
            *reinterpret_cast<float4*>(stg + j * S.stage_row + 2 * (cb + u)) =
                make_float4(x[u].x, x[u].y, x[u + 1].x, x[u + 1].y);
        } else {
#pragma unroll
          for (int u = 0; u < 8; ++u) {
            float h0, l0;
            const int q = 2 * (cb + u);
            split_tf32(x[u].x, h0, l0);
            bhi[boff(q, j, L.sbo_b) >> 2] = h0;
            blo[boff(q, j, L.sbo_b) >> 2] = l0;
            split_tf32(x[u].y, h0, l0);
            bhi[boff(q + 1, j, L.sbo_b) >> 2] = h0;
            blo[boff(q + 1, j, L.sbo_b) >> 2] = l0;
          }
        }
      }
      if (!last) {
        fence_proxy_async();
        mbar_arrive(bready);
      }
      if (tid == 0 && m < 2) trace_mark(tp, tile, TR_EPI0 + 2 * m);
    }
  }
  __syncthreads();
  if (tid == 0) trace_mark(tp, tile, TR_JOIN);

  if (!s_fail && tid < kWorkThreads) {
    // coalesced store of the staged tile: thread = complex column
    const int c = tid % S.bn, h = tid / S.bn, G = S.groups;
    for (int kb = h; kb < n; kb += 4 * G) {
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        const int k = kb + u * G;
        psi[base + (int64_t)k * g.inner + c] = *reinterpret_cast<const float2*>(bhi + k * S.stage_row + 2 * c);
      }
    }
  }
  if (tid == 0) trace_mark(tp, tile, TR_STORE);

  // ---- norm partials (fixed order) and last-CTA finalize
  for (int r = 0; r < p.nred; ++r) {
    const FF t = block_sum(acc[r], scratch);
    if (tid == 0) blk_red[r] = (double)t.hi + (double)t.lo;
  }
  __syncthreads();
  if (tid == 0) trace_mark(tp, tile, TR_NORMS);
  if (tid == 0) {
    if (s_fail && tp.error_slot >= 0) p.slots[tp.error_slot] = 1.0;
    for (int r = 0; r < p.nred; ++r) p.partials[(int64_t)r * g.tiles + tile] = blk_red[r];
    __threadfence();
    const unsigned int ticket = atomicAdd(p.counter, 1u);
    s_last = ticket == (unsigned int)(g.tiles - 1);
    trace_mark(tp, tile, TR_TICKET);
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

  // ---- teardown: tensor memory (every MMA has completed: drained, or waited on above)
  tc_fence_before();
  __syncthreads();
  if (tid == 0) trace_mark(tp, tile, TR_END);
  if (warp == 0) tmem_dealloc(tmem, kTmemCols);
}

__global__ void __launch_bounds__(kThreads, 2) angular_tc_kernel(const __grid_constant__ TcParams tp) {
  tc_tile(tp, blockIdx.x);
}

// Many propagations' lane-matrix passes in one launch: block b runs tile
// (b - offsets[i]) of params[i], offsets[i] <= b < offsets[i + 1].
__global__ void __launch_bounds__(kThreads, 2) angular_tc_kernel_batched(const TcParams* __restrict__ params,
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
static size_t tc_max_dynamic_smem() {
  size_t m = 0;
  for (int n = 32; n <= 256; n *= 2) m = tc_layout(n).total > m ? tc_layout(n).total : m;
  return m;
}

// two CTAs per SM: the whole shared-memory carveout, each CTA below half of it
static bool configure_once(const void* kern, bool& flag) {
  if (flag) return true;
  if (cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)tc_max_dynamic_smem()) !=
      cudaSuccess)
    return false;
  if (cudaFuncSetAttribute(kern, cudaFuncAttributePreferredSharedMemoryCarveout, cudaSharedmemCarveoutMaxShared) !=
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

bool angular_tc_ops_fit(const DevOp* ops, int nops, int sweep_axis) {
  int across = 0;
  for (int i = 0; i < nops; ++i) across += diag1d_across(ops[i], sweep_axis);
  return across <= kColtSlots;
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

int angular_tc_trace_slots() { return kTraceSlots; }

cudaError_t launch_angular_tc(const PassParams& p, const int* mat_op, int nmat, const float* const* images,
                              int error_slot, cudaStream_t s, unsigned long long* trace) {
  TcParams tp{};
  tp.trace = trace;
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
