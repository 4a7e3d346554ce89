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
// radial points).  A tile is BN complex columns of the inner axis for all n rows.
// Treating (re, im) as two real columns, a lane-matrix product is the real GEMM
// D[M x 2BN] = A[M x n] . B[n x 2BN], A the (zero-padded) matrix, B the tile:
//   n <= 128: M = 128, BN = 32 (N = 64), A chunks of K = 16
//   n = 256 : M = 256 as two 128-row halves, BN = 16 (N = 32); a
//             parity-structured Legendre pair as two K = 128 GEMMs (see tc_shape)
// 3xTF32: A = A_hi + A_lo (split once from the FP64 matrix on the host), B = B_hi +
// B_lo (split on the fly), both parts tf32-exact, D = A_hi B_hi + A_hi B_lo + A_lo B_hi.
//
// Persistent CTAs, two per SM, each walking its share of the tiles of the launch:
//   warps 0-7  load the tile, run the point-wise ops, split it into the B operand,
//              drain the accumulators, run the ops between / after the matrices,
//              store, and fold the norms (named barrier 1 among themselves)
//   warp 8     streams the A chunks (one MMA K step each) of every tile, in order,
//              through 2-6 shared-memory stages by bulk TMA (it runs ahead across tiles)
//   warp 9     issues tcgen05.mma (one lane) as chunks land and the B operand is ready
// The tensor core truncates its FP32 accumulation, so the A_hi B_hi products go to
// three TMEM regions a couple of K steps each and the work warps drain the
// regions into registers (round-to-nearest adds) every kFillSteps K steps; the
// corrections, 2^-11 smaller, share a fourth region.  FP32 norm partials are folded per tile in
// float-float and across tiles in FP64 by the last tile of the pass, in a fixed order.
// Every mbarrier wait is bounded (2 s); on a timeout the CTA records an error in a
// slot, lets its copies and MMAs finish (bounded), frees its tensor memory and returns.
#include <algorithm>
#include <cmath>
#include <cstring>

#include "common.cuh"
#include "tc_common.cuh"

namespace so {

namespace {

// A chunks: 8 KB per operand slice (128 rows x 32 bf16 / 16 tf32 K values, or 256 rows x
// half that).  The stages share 48 KB: two of 24 KB for split-BF16x6, three of 16 KB for
// the two-slice modes.
constexpr int kChunkBytes = 8192;
constexpr int kStageBudget = 48 * 1024;
constexpr int kLboB = 144;          // B: core matrices along K (16 B padding vs 128)
constexpr uint64_t kWaitLimit = 2000000000ull;  // 2 s per wait
constexpr int kWorkThreads = 256;               // warps 0-7
constexpr int kThreads = kWorkThreads + 64;     // + warp 8 (TMA) + warp 9 (MMA)
constexpr uint32_t kTmemCols = 256;  // half of the SM's tensor memory: two CTAs per SM
constexpr int kRegions = 4;          // 64-column accumulator regions in kTmemCols
constexpr int kFillSteps = 6;        // K steps between two drains of the main regions
constexpr int kVals = 32;            // FP32 accumulator columns a work thread drains
constexpr int kCtasPerSm = 2;        // persistent CTAs per SM (each one's memory latency hides behind the other)
constexpr int kColtSlots = 4;        // DIAG1D ops on a non-lane axis per pass

struct TcShape {
  bool par;      // parity-split lane matrices (two K = n/2 GEMMs, one per M half)
  bool oz;       // split-BF16x6: three fixed-point bf16 slices per operand, exact FP32 sums
  int slices;    // operand slices: 2 (hi, lo) or 3 (split-BF16x6)
  int kc;        // K values per 16-byte core-matrix row (4 tf32, 8 bf16)
  int km;        // K per MMA instruction (8 tf32, 16 bf16)
  int kdim;      // K of each GEMM: n, or n / 2 with par
  int mh;        // 128-row halves of M
  int bn;        // complex columns per tile
  int nc;        // fp32 columns = MMA N
  int chunk_k;   // K per A chunk
  int chunk_bytes;  // bytes of one slice of an A chunk (128 rows x chunk_k per M half)
  int stages;    // A chunk stages in flight
  int nk;        // chunks per matrix
  int ksteps;    // K steps of 8 per matrix
  int reg_cols;  // TMEM columns of one accumulator region (all M halves)
  int nmain;     // regions for the A_hi B_hi products; one more region holds the corrections
  int fills;     // drains of the main regions per matrix
  int sbo_a;     // A: row-group stride (bytes)
  int a_half16;  // A descriptor step to the second 128-row half ((16 row groups x sbo_a) >> 4)
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
// par: the two lane matrices split by parity into two half-size GEMMs (n = 256 only):
// K = n / 2, the 128-row halves of M are the even and odd parts, each with its own B.
// bf: split-BF16x3 operands (2-byte elements, 8 K values per 16-byte core-matrix row,
// K = 16 per instruction) instead of 3xTF32 (4-byte, 4 per row, K = 8); in bytes the
// chunk, core-matrix and descriptor steps are the same.
// oz: split-BF16x6 (bf16 operands in three fixed-point slices, six products, one exact
// accumulation per GEMM: see the comment above oz_quanta); implies bf.
__host__ __device__ inline TcShape tc_shape(int n, bool par = false, bool bf = false, bool oz = false) {
  TcShape s{};
  bf = bf || oz;
  s.oz = oz;
  s.slices = oz ? 3 : 2;
  s.par = par && n == 256;
  s.kc = bf ? 8 : 4;
  s.km = bf ? 16 : 8;
  s.mh = n == 256 ? 2 : 1;
  s.bn = n == 256 ? 16 : 32;
  s.nc = 2 * s.bn;
  s.chunk_k = (bf ? 32 : 16) / s.mh;
  s.chunk_bytes = kChunkBytes;
  s.stages = kStageBudget / (kChunkBytes * s.slices);
  s.kdim = s.par ? n / 2 : n;
  s.nk = s.kdim / s.chunk_k;
  s.ksteps = s.kdim / s.km;
  s.reg_cols = s.nc * s.mh;
  s.nmain = oz ? 3 : kRegions - 1;  // oz: the three product orders R0, R1, R2
  s.fills = oz ? 1 : (s.ksteps + kFillSteps - 1) / kFillSteps;
  s.sbo_a = (s.chunk_k / s.kc) * 128;
  s.a_half16 = (16 * s.sbo_a) >> 4;
  s.stage_row = s.nc + 4;
  s.groups = kWorkThreads / s.bn;
  return s;
}

struct TcSmemLayout {
  uint32_t stage0, stage_bytes, bhi, bmid, blo, bars, sbo_b, bhalf, bbytes, total;
};

// [stages x A stages (slices x chunk_bytes each)][B_hi][B_mid (oz)][B_lo][mbarriers:
// full[stages], empty[stages], dbar, freebar, bready, quiet].  With par each B slice holds two K = n/2
// operands, bhalf bytes apart (the even / odd or sum / difference halves).
__host__ __device__ inline TcSmemLayout tc_layout(int n, bool par = false, bool bf = false, bool oz = false) {
  const TcShape s = tc_shape(n, par, bf, oz);
  TcSmemLayout L{};
  L.sbo_b = (uint32_t)(s.kdim / s.kc) * kLboB + 16;
  L.bhalf = (uint32_t)(s.nc / 8) * L.sbo_b;
  L.bbytes = (s.par ? 2u : 1u) * L.bhalf;
  L.bbytes = (L.bbytes + 127u) & ~127u;
  L.stage0 = 0;
  L.stage_bytes = (uint32_t)(s.slices * s.chunk_bytes);
  L.bhi = (uint32_t)s.stages * L.stage_bytes;
  L.bmid = L.bhi + L.bbytes;  // (oz only)
  L.blo = (s.oz ? L.bmid : L.bhi) + L.bbytes;
  L.bars = L.blo + L.bbytes;
  L.total = L.bars + (2 * s.stages + 4) * 8;
  return L;
}

// byte offset of B operand element (column q, K row k) in the K-major core-matrix layout
template <bool BF>
__device__ __forceinline__ uint32_t boff(int q, int k, uint32_t sbo) {
  constexpr int kc = BF ? 8 : 4, es = BF ? 2 : 4;
  return (uint32_t)(q >> 3) * sbo + (uint32_t)(k / kc) * kLboB + (uint32_t)(q & 7) * 16u + (uint32_t)(k % kc) * es;
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

// barrier among the work warps only (the TMA and MMA warps run their own loops)
__device__ __forceinline__ void work_sync() { asm volatile("bar.sync 1, %0;" ::"n"(kWorkThreads) : "memory"); }

// the same barrier, returning whether v holds in every work thread
__device__ __forceinline__ bool work_all(bool v) {
  uint32_t r;
  asm volatile(
      "{\n\t.reg .pred p, q;\n\t"
      "setp.ne.u32 p, %1, 0;\n\t"
      "bar.red.and.pred q, 1, %2, p;\n\t"
      "selp.u32 %0, 1, 0, q;\n\t}"
      : "=r"(r)
      : "r"((uint32_t)v), "n"(kWorkThreads)
      : "memory");
  return r != 0;
}

// fixed-order sum of one float per work thread, in float-float; valid in thread 0
// The tile's nred float-float block sums together (fixed order): each warp reduces every
// value by the same shuffle tree, lane 0 stores them, one barrier; thread k adds reduction
// k's warp partials 0 .. 7 in order and stores its FP64 value in out[k]; a second barrier
// publishes them.  scratch: kMaxRed x (kWorkThreads / 32) entries.
__device__ __forceinline__ void block_sums(const float (&acc)[kMaxRed], int nred, FF* scratch, double* out) {
  constexpr int kW = kWorkThreads / 32;
#pragma unroll
  for (int k = 0; k < kMaxRed; ++k) {
    if (k >= nred) break;
    FF a{acc[k], 0.0f};
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
      const FF b{__shfl_down_sync(0xffffffffu, a.hi, off), __shfl_down_sync(0xffffffffu, a.lo, off)};
      a = ff_add(a, b);
    }
    if ((threadIdx.x & 31) == 0) scratch[k * kW + (threadIdx.x >> 5)] = a;
  }
  work_sync();
  if ((int)threadIdx.x < nred) {
    FF r{0.0f, 0.0f};
    for (int w = 0; w < kW; ++w) r = ff_add(r, scratch[threadIdx.x * kW + w]);
    out[threadIdx.x] = (double)r.hi + (double)r.lo;
  }
  work_sync();
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

// Per-tile factors of the point-wise ops, built once per tile (by the work warps) so that the per-point
// work reads shared memory and does FP32 arithmetic only (FP64 runs on a narrow pipe).
struct TileTabs {
  float colw[kMaxRed][32];      // NORM: product of the FP32 weights of every non-lane axis, per tile column
  float2 colt[kColtSlots][32];  // DIAG1D on a non-lane axis: the table value of each tile column
  float scale[kMaxOps];         // SCALE: sqrt(target / norm)
  int8_t slot[kMaxOps];         // DIAG1D on a non-lane axis: its colt row
};

__host__ __device__ inline bool diag1d_across(const DevOp& op, int sweep_axis) {
  return op.kind == OP_DIAG1D && op.axis != sweep_axis;
}

// Packed tiles (PK > 1, lane extent n = 128 / PK): PK groups of bn columns side by side,
// 128 tile columns in all.  Their passes (checked on the host) have one non-lane axis, every
// norm with the same weights and every across-lane diagonal with the same table, so the
// tables hold one row of 128 columns each, laid over the first rows of colw / colt.
template <int PK>
__device__ __forceinline__ float tab_w(const TileTabs& T, int red, int col) {
  if constexpr (PK > 1)
    return (&T.colw[0][0])[col];
  else
    return T.colw[red][col];
}
template <int PK>
__device__ __forceinline__ float2 tab_t(const TileTabs& T, int slot, int col) {
  if constexpr (PK > 1)
    return (&T.colt[0][0])[col];
  else
    return T.colt[slot][col];
}

template <int PK>
__device__ __forceinline__ void build_tile_tabs(const PassParams& p, TileTabs& T, int64_t o, int64_t i0, int bn) {
  const Geometry& g = p.g;
  if constexpr (PK > 1) {
    // bn = all PK x 32 tile columns, a single non-lane axis (inner index i0 + c)
    for (int idx = threadIdx.x; idx < p.nops * bn; idx += kWorkThreads) {
      const int oi = idx / bn, c = idx - oi * bn;
      const DevOp& op = p.ops[oi];
      const int64_t i = i0 + c;
      if (op.kind == OP_NORM)
        (&T.colw[0][0])[c] = __ldg(op.wf[g.perm[g.ndim - 1]] + i);
      else if (op.kind == OP_DIAG1D && op.axis != g.sweep_axis)
        (&T.colt[0][0])[c] = __ldg(reinterpret_cast<const float2*>(op.ptr) + i);
      else if (op.kind == OP_SCALE && c == 0)
        T.scale[oi] = (float)sqrt(__ldcg(p.slots + op.b) / __ldcg(p.slots + op.c));
    }
    return;
  }
  if ((int)threadIdx.x < p.nops) {
    int k = 0;
    for (int q = 0; q < (int)threadIdx.x; ++q) k += diag1d_across(p.ops[q], g.sweep_axis);
    T.slot[threadIdx.x] = (int8_t)k;
  }
  work_sync();
  for (int idx = threadIdx.x; idx < p.nops * bn; idx += kWorkThreads) {
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
template <int NB, int PK = 1>
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
          for (int u = 0; u < NB; ++u) v[u] = cmulf(v[u], tab_t<PK>(T, T.slot[oi], c0 + u));
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
        for (int u = 0; u < NB; ++u)
          s = fmaf(fmaf(v[u].x, v[u].x, v[u].y * v[u].y), tab_w<PK>(T, op.red, c0 + u), s);
        const float* wr = op.wf[g.sweep_axis];
        acc[op.red] += s * (wr == rw_ptr ? rw_val : __ldg(wr + j));
        break;
      }
      default:
        break;
    }
  }
}

// The same ops on two rows ja, jb of the same NB columns (the even / odd epilogue holds rows
// i and n-1-i): op by op for both rows, so each table's two row loads are in flight together.
template <int NB>
__device__ __forceinline__ void apply_row2(const PassParams& p, const TileTabs& T, int ob, int oe, float2 (&va)[NB],
                                           float2 (&vb)[NB], int ja, int jb, int c0, int64_t ixa, int64_t ixb,
                                           float* acc, const float* rw_ptr, float rwa, float rwb) {
  const Geometry& g = p.g;
  for (int oi = ob; oi < oe; ++oi) {
    const DevOp& op = p.ops[oi];
    switch (op.kind) {
      case OP_DIAG1D: {
        if (op.axis == g.sweep_axis) {
          const float2 ta = __ldg(reinterpret_cast<const float2*>(op.ptr) + ja);
          const float2 tb = __ldg(reinterpret_cast<const float2*>(op.ptr) + jb);
#pragma unroll
          for (int u = 0; u < NB; ++u) {
            va[u] = cmulf(va[u], ta);
            vb[u] = cmulf(vb[u], tb);
          }
        } else {
#pragma unroll
          for (int u = 0; u < NB; ++u) {
            const float2 t = T.colt[T.slot[oi]][c0 + u];
            va[u] = cmulf(va[u], t);
            vb[u] = cmulf(vb[u], t);
          }
        }
        break;
      }
      case OP_DIAGND: {
        const float2* ta = reinterpret_cast<const float2*>(op.ptr) + ixa;
        const float2* tb = reinterpret_cast<const float2*>(op.ptr) + ixb;
        if (((reinterpret_cast<uintptr_t>(ta) | reinterpret_cast<uintptr_t>(tb)) & 15u) == 0) {
          float4 qa[NB / 2], qb[NB / 2];
#pragma unroll
          for (int q = 0; q < NB / 2; ++q) {
            qa[q] = __ldg(reinterpret_cast<const float4*>(ta) + q);
            qb[q] = __ldg(reinterpret_cast<const float4*>(tb) + q);
          }
#pragma unroll
          for (int q = 0; q < NB / 2; ++q) {
            va[2 * q] = cmulf(va[2 * q], make_float2(qa[q].x, qa[q].y));
            va[2 * q + 1] = cmulf(va[2 * q + 1], make_float2(qa[q].z, qa[q].w));
            vb[2 * q] = cmulf(vb[2 * q], make_float2(qb[q].x, qb[q].y));
            vb[2 * q + 1] = cmulf(vb[2 * q + 1], make_float2(qb[q].z, qb[q].w));
          }
        } else {
#pragma unroll
          for (int u = 0; u < NB; ++u) {
            va[u] = cmulf(va[u], __ldg(ta + u));
            vb[u] = cmulf(vb[u], __ldg(tb + u));
          }
        }
        break;
      }
      case OP_SCALE: {
        const float f = T.scale[oi];
#pragma unroll
        for (int u = 0; u < NB; ++u) {
          va[u] = {va[u].x * f, va[u].y * f};
          vb[u] = {vb[u].x * f, vb[u].y * f};
        }
        break;
      }
      case OP_NORM: {
        float sa = 0.0f, sb = 0.0f;
#pragma unroll
        for (int u = 0; u < NB; ++u) {
          const float w = T.colw[op.red][c0 + u];
          sa = fmaf(fmaf(va[u].x, va[u].x, va[u].y * va[u].y), w, sa);
          sb = fmaf(fmaf(vb[u].x, vb[u].x, vb[u].y * vb[u].y), w, sb);
        }
        const float* wr = op.wf[g.sweep_axis];
        const bool pre = wr == rw_ptr;
        acc[op.red] += sa * (pre ? rwa : __ldg(wr + ja));
        acc[op.red] += sb * (pre ? rwb : __ldg(wr + jb));
        break;
      }
      default:
        break;
    }
  }
}

// Point-wise ops [ob, oe) on the NB values of one tile column c, lane-axis rows
// j0 + u G (storage indices ix0 + u rstride): the prologue layout.
// PK > 1 (packed tile): value u sits at virtual row R = j0 + u G, i.e. lane row R % nl of
// column group R / nl (nl = the real lane extent), storage index base + (R % nl) inner +
// (R / nl) bn + c; ix0 and rstride are then unused.
template <int NB, int PK = 1>
__device__ __forceinline__ void apply_col(const PassParams& p, const TileTabs& T, int ob, int oe, float2 (&v)[NB],
                                          int j0, int G, int c, int64_t ix0, int64_t rstride, float* acc,
                                          int nl = 0, int bn = 0, int64_t base = 0) {
  const Geometry& g = p.g;
  if constexpr (PK > 1) {
    int jl[NB], col[NB];
    int64_t ix[NB];
#pragma unroll
    for (int u = 0; u < NB; ++u) {
      const int R = j0 + u * G;
      jl[u] = R & (nl - 1);
      col[u] = (R / nl) * bn + c;
      ix[u] = base + (int64_t)jl[u] * g.inner + col[u];
    }
    for (int oi = ob; oi < oe; ++oi) {
      const DevOp& op = p.ops[oi];
      switch (op.kind) {
        case OP_DIAG1D: {
          const float2* t = reinterpret_cast<const float2*>(op.ptr);
          if (op.axis == g.sweep_axis) {
            float2 tv[NB];
#pragma unroll
            for (int u = 0; u < NB; ++u) tv[u] = __ldg(t + jl[u]);
#pragma unroll
            for (int u = 0; u < NB; ++u) v[u] = cmulf(v[u], tv[u]);
          } else {
#pragma unroll
            for (int u = 0; u < NB; ++u) v[u] = cmulf(v[u], tab_t<PK>(T, 0, col[u]));
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
          for (int u = 0; u < NB; ++u)
            s = fmaf(fmaf(v[u].x, v[u].x, v[u].y * v[u].y), __ldg(wr + jl[u]) * tab_w<PK>(T, 0, col[u]), s);
          acc[op.red] += s;
          break;
        }
        default:
          break;
      }
    }
    return;
  }
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

// hi / lo operand parts of four consecutive K values of one B column, stored at byte
// offset `off` of the hi and lo images: two 16-byte rows (tf32) or two 8-byte halves of
// rows (bf16)
template <bool BF>
__device__ __forceinline__ void store4(unsigned char* bh, unsigned char* bl, uint32_t off, float a, float b, float c,
                                       float d) {
  if constexpr (BF) {
    uint16_t h[4], l[4];
    tc::split_bf16(a, h[0], l[0]);
    tc::split_bf16(b, h[1], l[1]);
    tc::split_bf16(c, h[2], l[2]);
    tc::split_bf16(d, h[3], l[3]);
    *reinterpret_cast<uint2*>(bh + off) = make_uint2(h[0] | (uint32_t)h[1] << 16, h[2] | (uint32_t)h[3] << 16);
    *reinterpret_cast<uint2*>(bl + off) = make_uint2(l[0] | (uint32_t)l[1] << 16, l[2] | (uint32_t)l[3] << 16);
  } else {
    float4 h, l;
    tc::split_tf32(a, h.x, l.x);
    tc::split_tf32(b, h.y, l.y);
    tc::split_tf32(c, h.z, l.z);
    tc::split_tf32(d, h.w, l.w);
    *reinterpret_cast<float4*>(bh + off) = h;
    *reinterpret_cast<float4*>(bl + off) = l;
  }
}

// ---- split-BF16x6: exact tensor-core sums (the Ozaki scheme with bf16 slices)
// The tensor core truncates when it adds products whose bits spread over more than an FP32
// significand; a sum whose terms are all multiples of one quantum q and stay below 2^24 q in
// magnitude has no such bits, so the core adds it exactly.  Each B column (and, on the host,
// each A row) is cut at the power of two just above its largest magnitude into three
// fixed-point slices of 8 significant bits -- x = s0 + s1 + s2 + O(2^-24 max), s_i a
// multiple of q_i = 2^(e-8-8i) with |s_i / q_i| <= 256 -- which bf16 holds exactly.  A
// product of two slices is then an integer below 2^16 times q_A q_B, and a GEMM of K <= 256
// such products stays below 2^24 of its quantum: the three product orders accumulate
// exactly over all of K in three TMEM regions, R0 = A0 B0, R1 = A0 B1 + A1 B0,
// R2 = A0 B2 + A1 B1 + A2 B0 (the dropped orders are 2^-24 of the leading one), and the
// only rounding is the round-to-nearest R2 + R1 + R0 of the drain -- no truncation bias.
// Reference: K. Ozaki, T. Ogita, S. Oishi, S. M. Rump, "Error-free transformations of
// matrix multiplication by using fast routines of matrix multiplication and its
// applications", Numer. Algorithms 59 (2012).
struct OzQ {
  float s0, s1, s2;  // 1.5 x 2^23 q_i: adding and subtracting one rounds to a multiple of q_i
};

// quanta of a column whose largest magnitude has the FP32 bits `maxbits`: q0 = 2^(E+1-8)
// for max in [2^E, 2^(E+1)); columns below 2^-103 (and empty ones) share the smallest
// quanta whose third slice is still a normal number, columns of 2^111 or more (never a
// finite state's) the largest whose rounding constant is finite
__device__ __forceinline__ OzQ oz_quanta(uint32_t maxbits) {
  uint32_t e = maxbits >> 23;  // biased exponent of the (non-negative) maximum
  e = e < 24u ? 24u : (e > 238u ? 238u : e);
  const uint32_t es = e + 16u;  // biased exponent of 2^23 q0 (q0's is e - 7)
  return {__uint_as_float((es << 23) | 0x400000u), __uint_as_float(((es - 8u) << 23) | 0x400000u),
          __uint_as_float(((es - 16u) << 23) | 0x400000u)};
}

// x -> three bf16 slices (each exact: a bf16 value's FP32 bits end in 16 zero bits).  For
// |x| < 2^22 q, (x + 1.5 2^23 q) - 1.5 2^23 q is x rounded to a multiple of q (to nearest,
// ties to even): the sum stays in the binade whose spacing is q.  Slice i: |x_i| <= 2^8 q_i.
__device__ __forceinline__ void oz_split(float x, const OzQ& q, uint32_t& h0, uint32_t& h1, uint32_t& h2) {
  const float s0 = __fsub_rn(__fadd_rn(x, q.s0), q.s0);
  float r = __fsub_rn(x, s0);
  const float s1 = __fsub_rn(__fadd_rn(r, q.s1), q.s1);
  r = __fsub_rn(r, s1);
  const float s2 = __fsub_rn(__fadd_rn(r, q.s2), q.s2);
  h0 = __float_as_uint(s0) >> 16;
  h1 = __float_as_uint(s1) >> 16;
  h2 = __float_as_uint(s2) >> 16;
}

// four consecutive K values of one B column (one quantum) at byte offset `off` of the three
// slice images: one 8-byte store per slice
__device__ __forceinline__ void store4_oz(unsigned char* b0, unsigned char* b1, unsigned char* b2, uint32_t off,
                                          float a, float b, float c, float d, const OzQ& q) {
  uint32_t x0[4], x1[4], x2[4];
  oz_split(a, q, x0[0], x1[0], x2[0]);
  oz_split(b, q, x0[1], x1[1], x2[1]);
  oz_split(c, q, x0[2], x1[2], x2[2]);
  oz_split(d, q, x0[3], x1[3], x2[3]);
  *reinterpret_cast<uint2*>(b0 + off) = make_uint2(x0[0] | x0[1] << 16, x0[2] | x0[3] << 16);
  *reinterpret_cast<uint2*>(b1 + off) = make_uint2(x1[0] | x1[1] << 16, x1[2] | x1[3] << 16);
  *reinterpret_cast<uint2*>(b2 + off) = make_uint2(x2[0] | x2[1] << 16, x2[2] | x2[3] << 16);
}

__device__ __forceinline__ void store1_oz(unsigned char* b0, unsigned char* b1, unsigned char* b2, uint32_t off,
                                          float x, const OzQ& q) {
  uint32_t h0, h1, h2;
  oz_split(x, q, h0, h1, h2);
  *reinterpret_cast<uint16_t*>(b0 + off) = (uint16_t)h0;
  *reinterpret_cast<uint16_t*>(b1 + off) = (uint16_t)h1;
  *reinterpret_cast<uint16_t*>(b2 + off) = (uint16_t)h2;
}

// per-column maxima in shared memory (FP32 bits of |x|, which order like the values)
__device__ __forceinline__ void colmax_add(uint32_t* cm, int col, float m) {
  atomicMax(cm + col, __float_as_uint(m));
}

// one operand element: hi / lo parts at byte offset `off`
template <bool BF>
__device__ __forceinline__ void store1(unsigned char* bh, unsigned char* bl, uint32_t off, float x) {
  if constexpr (BF) {
    uint16_t h, l;
    tc::split_bf16(x, h, l);
    *reinterpret_cast<uint16_t*>(bh + off) = h;
    *reinterpret_cast<uint16_t*>(bl + off) = l;
  } else {
    float h, l;
    tc::split_tf32(x, h, l);
    *reinterpret_cast<float*>(bh + off) = h;
    *reinterpret_cast<float*>(bl + off) = l;
  }
}

// Prologue with vector operand stores.  Thread (column c, block a) owns the row blocks
// RB (a + G k) .. + RB - 1, k < NK: its loads are coalesced across the warp (consecutive
// columns of one row) and, since K is the contiguous direction of a core-matrix row, four
// consecutive K rows of one B column are one vector store.
//   mode 0: row j -> K row j (RB = 4)
//   mode 2: even / odd halves, row j -> half j & 1, K row j >> 1 (RB = 8)
//   mode 1: sum / difference pairs, rows j < n/2 and n-1-j -> K row j of both halves (RB = 4)
// OZ (split-BF16x6): the operand goes to three slice images (bh, bm, bl) with the quanta of
// each column's largest value, gathered in cm (per-column maxima, zero on entry) first.
// PK > 1: a packed tile (virtual rows: lane row j % nl of column group j / nl, bn columns a group).
template <int NK, int RB, int MODE, bool BF, bool OZ, int PK = 1>
__device__ __forceinline__ void prologue_vec(const PassParams& p, const TileTabs& T, int oe, const float2* psi,
                                             int64_t base, int c, int a, int G, int n, unsigned char* bh,
                                             unsigned char* bm, unsigned char* bl, uint32_t bhalf, uint32_t sbo_b,
                                             float* acc, unsigned long long* loaded_mark, uint32_t* cm, int nl = 0,
                                             int bn = 0) {
  const int64_t inner = p.g.inner;
  const int64_t bstride = (int64_t)RB * G;  // rows between a thread's row blocks
  float2 v[RB][NK];
  float2 w[MODE == 1 ? RB : 1][MODE == 1 ? NK : 1];  // mirrored rows n-1-j (sum / difference)
#pragma unroll
  for (int r = 0; r < RB; ++r)
#pragma unroll
    for (int k = 0; k < NK; ++k) {
      const int64_t j = (int64_t)RB * a + r + bstride * k;
      if constexpr (PK > 1)
        v[r][k] = psi[base + (j & (nl - 1)) * inner + (j / nl) * bn + c];
      else
        v[r][k] = psi[base + j * inner + c];
      if constexpr (MODE == 1) w[r][k] = psi[base + (n - 1 - j) * inner + c];
    }
  if (loaded_mark) {
    // the first value consumed: every load of this thread has returned
    float s = 0.0f;
#pragma unroll
    for (int r = 0; r < RB; ++r)
#pragma unroll
      for (int k = 0; k < NK; ++k) s += v[r][k].x;
    if (s != 12345.678f) *loaded_mark = tc::globaltimer_ns();
  }
#pragma unroll
  for (int r = 0; r < RB; ++r) {
    const int j0 = RB * a + r;
    apply_col<NK, PK>(p, T, 0, oe, v[r], j0, (int)bstride, c, base + (int64_t)j0 * inner + c, bstride * inner, acc,
                      nl, bn, base);
    if constexpr (MODE == 1)
      apply_col<NK>(p, T, 0, oe, w[r], n - 1 - j0, -(int)bstride, c, base + (int64_t)(n - 1 - j0) * inner + c,
                    -bstride * inner, acc);
  }
  if constexpr (OZ && PK > 1) {
    // packed tile: row block k lies in column group (RB a + bstride k) / nl, whose columns
    // carry their own quanta (set g of cm: 64 entries, re and im of its 32 columns)
    OzQ qr[NK], qi[NK];
#pragma unroll
    for (int k = 0; k < NK; ++k) {
      float mr = 0.0f, mi = 0.0f;
#pragma unroll
      for (int r = 0; r < RB; ++r) {
        mr = fmaxf(mr, fabsf(v[r][k].x));
        mi = fmaxf(mi, fabsf(v[r][k].y));
      }
      const int grp = (RB * a + (int)bstride * k) / nl;
      colmax_add(cm + grp * 64, 2 * c, mr);
      colmax_add(cm + grp * 64, 2 * c + 1, mi);
    }
    work_sync();
#pragma unroll
    for (int k = 0; k < NK; ++k) {
      const int grp = (RB * a + (int)bstride * k) / nl;
      qr[k] = oz_quanta(cm[grp * 64 + 2 * c]);
      qi[k] = oz_quanta(cm[grp * 64 + 2 * c + 1]);
    }
#pragma unroll
    for (int k = 0; k < NK; ++k) {
      const int j0 = RB * a + (int)bstride * k;
      const uint32_t orr = boff<true>(2 * c, j0, sbo_b), oim = boff<true>(2 * c + 1, j0, sbo_b);
      store4_oz(bh, bm, bl, orr, v[0][k].x, v[1][k].x, v[2][k].x, v[3][k].x, qr[k]);
      store4_oz(bh, bm, bl, oim, v[0][k].y, v[1][k].y, v[2][k].y, v[3][k].y, qi[k]);
    }
    return;
  }
  if constexpr (OZ) {
    // the column's largest stored magnitude (re and im are separate B columns); for the sum /
    // difference pairs |v| + |w| bounds both |v + w| and |v - w|
    float mr = 0.0f, mi = 0.0f;
#pragma unroll
    for (int r = 0; r < RB; ++r)
#pragma unroll
      for (int k = 0; k < NK; ++k) {
        if constexpr (MODE == 1) {
          mr = fmaxf(mr, fabsf(v[r][k].x) + fabsf(w[r][k].x));
          mi = fmaxf(mi, fabsf(v[r][k].y) + fabsf(w[r][k].y));
        } else {
          mr = fmaxf(mr, fabsf(v[r][k].x));
          mi = fmaxf(mi, fabsf(v[r][k].y));
        }
      }
    colmax_add(cm, 2 * c, mr);
    colmax_add(cm, 2 * c + 1, mi);
    work_sync();
    const OzQ qr = oz_quanta(cm[2 * c]), qi = oz_quanta(cm[2 * c + 1]);
#pragma unroll
    for (int k = 0; k < NK; ++k) {
      const int j0 = RB * a + (int)bstride * k;
      if constexpr (MODE == 0) {
        const uint32_t orr = boff<true>(2 * c, j0, sbo_b), oim = boff<true>(2 * c + 1, j0, sbo_b);
        store4_oz(bh, bm, bl, orr, v[0][k].x, v[1][k].x, v[2][k].x, v[3][k].x, qr);
        store4_oz(bh, bm, bl, oim, v[0][k].y, v[1][k].y, v[2][k].y, v[3][k].y, qi);
      } else if constexpr (MODE == 2) {
#pragma unroll
        for (int hf = 0; hf < 2; ++hf) {
          const uint32_t o = hf * bhalf;
          const uint32_t orr = o + boff<true>(2 * c, j0 >> 1, sbo_b), oim = o + boff<true>(2 * c + 1, j0 >> 1, sbo_b);
          store4_oz(bh, bm, bl, orr, v[hf][k].x, v[2 + hf][k].x, v[4 + hf][k].x, v[6 + hf][k].x, qr);
          store4_oz(bh, bm, bl, oim, v[hf][k].y, v[2 + hf][k].y, v[4 + hf][k].y, v[6 + hf][k].y, qi);
        }
      } else {
        const uint32_t orr = boff<true>(2 * c, j0, sbo_b), oim = boff<true>(2 * c + 1, j0, sbo_b);
#pragma unroll
        for (int hf = 0; hf < 2; ++hf) {
          const float sg = hf ? -1.0f : 1.0f;
          const uint32_t o = hf * bhalf;
          store4_oz(bh, bm, bl, o + orr, v[0][k].x + sg * w[0][k].x, v[1][k].x + sg * w[1][k].x,
                    v[2][k].x + sg * w[2][k].x, v[3][k].x + sg * w[3][k].x, qr);
          store4_oz(bh, bm, bl, o + oim, v[0][k].y + sg * w[0][k].y, v[1][k].y + sg * w[1][k].y,
                    v[2][k].y + sg * w[2][k].y, v[3][k].y + sg * w[3][k].y, qi);
        }
      }
    }
    return;
  }
#pragma unroll
  for (int k = 0; k < NK; ++k) {
    const int j0 = RB * a + (int)bstride * k;  // first row of the block
    if constexpr (MODE == 0) {
      const uint32_t orr = boff<BF>(2 * c, j0, sbo_b), oim = boff<BF>(2 * c + 1, j0, sbo_b);
      store4<BF>(bh, bl, orr, v[0][k].x, v[1][k].x, v[2][k].x, v[3][k].x);
      store4<BF>(bh, bl, oim, v[0][k].y, v[1][k].y, v[2][k].y, v[3][k].y);
    } else if constexpr (MODE == 2) {
#pragma unroll
      for (int hf = 0; hf < 2; ++hf) {
        const uint32_t o = hf * bhalf;
        const uint32_t orr = o + boff<BF>(2 * c, j0 >> 1, sbo_b), oim = o + boff<BF>(2 * c + 1, j0 >> 1, sbo_b);
        store4<BF>(bh, bl, orr, v[hf][k].x, v[2 + hf][k].x, v[4 + hf][k].x, v[6 + hf][k].x);
        store4<BF>(bh, bl, oim, v[hf][k].y, v[2 + hf][k].y, v[4 + hf][k].y, v[6 + hf][k].y);
      }
    } else {
      const uint32_t orr = boff<BF>(2 * c, j0, sbo_b), oim = boff<BF>(2 * c + 1, j0, sbo_b);
#pragma unroll
      for (int hf = 0; hf < 2; ++hf) {
        const float sg = hf ? -1.0f : 1.0f;
        const uint32_t o = hf * bhalf;
        store4<BF>(bh, bl, o + orr, v[0][k].x + sg * w[0][k].x, v[1][k].x + sg * w[1][k].x,
                   v[2][k].x + sg * w[2][k].x, v[3][k].x + sg * w[3][k].x);
        store4<BF>(bh, bl, o + oim, v[0][k].y + sg * w[0][k].y, v[1][k].y + sg * w[1][k].y,
                   v[2][k].y + sg * w[2][k].y, v[3][k].y + sg * w[3][k].y);
      }
    }
  }
}

// B operand row of NV complex values: columns c0 .. c0 + NV - 1 (c0 a multiple of 8) at K
// row k.  Column q = 2 (c0 + u) (+1) sits in core-matrix group c0 / 4 + u / 4, row 2 (u % 4)
// (+1): byte offsets (u / 4) sbo + (u % 4) 32 (+16) from that of q = 2 c0.
template <int NV, bool BF>
__device__ __forceinline__ void write_b_row(const float2 (&x)[NV], int c0, int k, unsigned char* bh,
                                            unsigned char* bl, uint32_t sbo_b) {
  const uint32_t o0 = boff<BF>(2 * c0, k, sbo_b);
#pragma unroll
  for (int u = 0; u < NV; ++u) {
    const uint32_t o = o0 + (uint32_t)(u >> 2) * sbo_b + (uint32_t)(u & 3) * 32u;
    store1<BF>(bh, bl, o, x[u].x);
    store1<BF>(bh, bl, o + 16, x[u].y);
  }
}

// The same row into the three slice images of split-BF16x6, with the quanta of its columns
// (cm: per-column maxima of the whole operand, complete when this runs)
template <int NV>
__device__ __forceinline__ void write_b_row_oz(const float2 (&x)[NV], int c0, int k, unsigned char* b0,
                                               unsigned char* b1, unsigned char* b2, uint32_t sbo_b,
                                               const uint32_t* cm) {
  const uint32_t o0 = boff<true>(2 * c0, k, sbo_b);
#pragma unroll
  for (int u = 0; u < NV; ++u) {
    const uint32_t o = o0 + (uint32_t)(u >> 2) * sbo_b + (uint32_t)(u & 3) * 32u;
    store1_oz(b0, b1, b2, o, x[u].x, oz_quanta(cm[2 * (c0 + u)]));
    store1_oz(b0, b1, b2, o + 16, x[u].y, oz_quanta(cm[2 * (c0 + u) + 1]));
  }
}

// Column maxima of a B operand written row by row: every lane of the warp holds one row of
// the same NV complex columns c0 .. (rows that are not written pass zeros); the warp reduces
// each column and one lane per column adds it to cm.  Called by all 32 lanes.
template <int NV>
__device__ __forceinline__ void colmax_rows(const float2 (&x)[NV], int c0, uint32_t* cm) {
  const int lane = threadIdx.x & 31;
#pragma unroll
  for (int u = 0; u < NV; ++u) {
    const uint32_t mr = __reduce_max_sync(0xffffffffu, __float_as_uint(fabsf(x[u].x)));
    const uint32_t mi = __reduce_max_sync(0xffffffffu, __float_as_uint(fabsf(x[u].y)));
    if (lane == (2 * u) % 32) atomicMax(cm + 2 * (c0 + u), mr);
    if (lane == (2 * u + 1) % 32) atomicMax(cm + 2 * (c0 + u) + 1, mi);
  }
}

// NV complex values of row j, columns c0 .., into the output staging
template <int NV>
__device__ __forceinline__ void stage_row(const float2 (&x)[NV], int c0, int j, float* stg, int stage_row_floats) {
#pragma unroll
  for (int u = 0; u < NV; u += 2)
    *reinterpret_cast<float4*>(stg + j * stage_row_floats + 2 * (c0 + u)) =
        make_float4(x[u].x, x[u].y, x[u + 1].x, x[u + 1].y);
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
  const float* images[2]; // A chunk images per matrix: nk x slices x chunk_bytes
  int32_t error_slot;
  int32_t parity[2];          // per matrix: 0 plain; 1 sum / difference rows; 2 even / odd columns
  unsigned long long* trace;  // optional phase timestamps, kTraceSlots per tile (nullptr: off)
  int32_t pack;               // column groups per tile (1; or 128 / n packed, images block-diagonal)
  int32_t npre;               // distinct full-size tables read after the first matrix (prefetched per tile)
  const void* pre[4];
  int32_t slice_axis[2];      // state matrix: the logical axis whose coordinate picks the image (-1: one image)
  int64_t slice_stride[2];    // floats between two coordinates' images
  // ... the tile's coordinate along it: ((tile mod pre) / div) mod ext (pre 0: no first mod),
  // 32-bit arithmetic worked out on the host (tiles of a pass < 2^32)
  uint32_t slice_pre[2], slice_div[2], slice_ext[2];
};

// Phase timestamps (%globaltimer, ns) of the optional trace, per tile (work thread 0).
enum TraceSlot {
  TR_START, TR_PROLOGUE, TR_MAT0, TR_EPI0, TR_MAT1, TR_EPI1, TR_STORE, TR_END,
  TR_TMA = 8,     // + c: chunk c (< 8) of the tile: copy issued (TMA warp)
  TR_FULL = 16,   // + c: chunk c landed (MMA warp)
  TR_MMA = 24,    // + c: chunk c's MMAs issued and committed (MMA warp)
  TR_TABS = 32,   // per-tile tables built (work warps)
  TR_LOADED = 33, // prologue values in registers (work thread 0)
  TR_STORED = 34, // prologue operand stores issued (work thread 0)
  TR_DRAIN0 = 35, // first matrix: accumulators drained (work thread 0)
  TR_APPLY0 = 36, // first matrix: point-wise ops after it applied (work thread 0)
  TR_SYNC0 = 37,  // first matrix: the next operand's column maxima complete (split-BF16x6)
  kTraceSlots = 38
};
__device__ __forceinline__ void trace_mark(const TcParams& tp, int64_t tile, int slot) {
  if (tp.trace) tp.trace[tile * kTraceSlots + slot] = tc::globaltimer_ns();
}

// K steps [t0, t1) of fill f split into at most nmain regions
struct FillSpan {
  int t0, t1, nused;
};
__device__ __forceinline__ FillSpan fill_span(const TcShape& S, int f) {
  FillSpan r;
  r.t0 = f * S.ksteps / S.fills;
  r.t1 = (f + 1) * S.ksteps / S.fills;
  r.nused = (r.t1 - r.t0) < S.nmain ? (r.t1 - r.t0) : S.nmain;
  return r;
}

// A tile of a launch: its pass description and its index within the pass.
struct TileRef {
  const TcParams* prm;
  int64_t tile;
};

// Warp 8, lane 0: the A chunks of every tile of this CTA, in order, through the stages.
template <typename Resolve>
__device__ __noinline__ void tma_producer(Resolve resolve, int64_t total, const TcShape S, uint32_t sm0,
                                          const TcSmemLayout L, volatile int* fail) {
  using namespace tc;
  uint64_t* full = reinterpret_cast<uint64_t*>(sm_ptr(sm0 + L.bars));
  uint64_t* empty = full + S.stages;
  const uint32_t stage_bytes = L.stage_bytes;
  const int ns = S.stages;
  int64_t cc = 0;  // chunks issued
  int s = 0;       // its stage (cc mod ns) and the use count of that stage (cc / ns)
  uint32_t use = 0;
  bool ok = true;
  for (int64_t gt = blockIdx.x; gt < total && ok && !*fail; gt += gridDim.x) {
    const TileRef r = resolve(gt);
    const int nmat = r.prm->nmat;
    for (int m = 0; m < nmat && ok; ++m) {
      const float* img = r.prm->images[m];
      if (r.prm->slice_axis[m] >= 0) {
        // a state matrix: the image of the tile's coordinate along the slice axis
        uint32_t t = (uint32_t)r.tile;
        if (r.prm->slice_pre[m]) t %= r.prm->slice_pre[m];
        img += (int64_t)((t / r.prm->slice_div[m]) % r.prm->slice_ext[m]) * r.prm->slice_stride[m];
      }
      for (int q = 0; q < S.nk; ++q) {
        if (use > 0 && !mbar_poll(&empty[s], (use - 1) & 1u, kWaitLimit)) {
          ok = false;
          break;
        }
        const int ct = m * S.nk + q;  // chunk within the tile
        if (r.prm->trace && ct < 8) r.prm->trace[r.tile * kTraceSlots + TR_TMA + ct] = globaltimer_ns();
        mbar_expect_tx(&full[s], stage_bytes);
        bulk_g2s(sm_ptr(sm0 + L.stage0 + (uint32_t)s * stage_bytes),
                 img + (size_t)q * S.slices * (S.chunk_bytes / 4), stage_bytes, &full[s]);
        ++cc;
        if (++s == ns) {
          s = 0;
          ++use;
        }
      }
    }
  }
  if (!ok) {
    *fail = 1;
    // let the copies in flight land before the CTA lets go of its shared memory
    for (int64_t c = cc - ns < 0 ? 0 : cc - ns; c < cc; ++c)
      mbar_poll(&full[(int)(c % ns)], (uint32_t)((c / ns) & 1), kWaitLimit);
  }
}

// Warp 9, lane 0: for each tile and matrix (once its B operand is written) and each
// fill, the K steps of the fill -- step t puts A_hi B_hi into main region
// (t - t0) nused / span and both corrections into the correction region -- then a
// commit of the fill to dbar.  Each chunk's MMAs are committed to its stage's empty
// barrier, which the TMA warp waits on before refilling the stage.  (Split-BF16x6 has its
// own issuer, mma_issuer_oz.)
template <bool BF, typename Resolve>
__device__ __noinline__ void mma_issuer(Resolve resolve, int64_t total, const TcShape S, uint32_t sm0,
                                        const TcSmemLayout L, uint32_t tmem, volatile int* fail) {
  using namespace tc;
  uint64_t* full = reinterpret_cast<uint64_t*>(sm_ptr(sm0 + L.bars));
  const int ns = S.stages;
  uint64_t* empty = full + ns;
  uint64_t* dbar = full + 2 * ns;
  uint64_t* freebar = dbar + 1;
  uint64_t* bready = dbar + 2;
  uint64_t* quiet = dbar + 3;
  const uint32_t stage_bytes = L.stage_bytes;
  const uint32_t idesc = BF ? idesc_bf16(128, (uint32_t)S.nc) : idesc_tf32(128, (uint32_t)S.nc);
  const uint64_t bbits = smem_desc_bits(kLboB, L.sbo_b), abits = smem_desc_bits(128, (uint32_t)S.sbo_a);
  const int kpc = S.chunk_k / S.km;  // K steps per chunk
  const uint64_t bstep_half = S.par ? (uint64_t)(L.bhalf >> 4) : 0u;
  int64_t cc = 0;                 // chunks consumed
  int s = 0;                      // stage of the chunk being consumed (cc mod ns)
  uint32_t fphase = 0;            // its full barrier's phase ((cc / ns) & 1)
  uint64_t ahi = 0;               // A_hi descriptor of the current K step (a chunk may span two fills)
  uint32_t nready = 0, nfree = 0;
  bool ok = true;
  for (int64_t gt = blockIdx.x; gt < total && ok; gt += gridDim.x) {
    const TileRef tr = resolve(gt);
    const int nmat = tr.prm->nmat;
    unsigned long long* trace = tr.prm->trace ? tr.prm->trace + tr.tile * kTraceSlots : nullptr;
    const int64_t cc_tile = cc;  // first chunk of this tile
    for (int m = 0; m < nmat && ok; ++m) {
      ok = mbar_poll(bready, nready & 1u, kWaitLimit);
      ++nready;
      tc_fence_after();
      for (int f = 0; f < S.fills && ok; ++f) {
        if (f > 0) {
          ok = mbar_poll(freebar, nfree & 1u, kWaitLimit);
          ++nfree;
          tc_fence_after();
          if (!ok) break;
        }
        const FillSpan fs = fill_span(S, f);
        const int span = fs.t1 - fs.t0;
        // descriptors and TMEM addresses advance by constant steps (no division per step):
        // B by 2 K core matrices (2 x kLboB bytes) per K step, A by 256 bytes per K step
        // within a chunk; the main region index moves when (t - t0) nused crosses span
        uint64_t bh = smem_desc_at(bbits, sm0 + L.bhi + (uint32_t)(fs.t0 * 2 * kLboB));
        uint64_t bl = smem_desc_at(bbits, sm0 + L.blo + (uint32_t)(fs.t0 * 2 * kLboB));
        int rm = 0, racc = 0;
        bool newreg = true;  // this step starts region rm
        uint32_t dm0 = tmem;
        const uint32_t dc0 = tmem + (uint32_t)(S.nmain * S.reg_cols);
        for (int t = fs.t0; t < fs.t1; ++t) {
          const int ks = t & (kpc - 1);  // kpc is 1 or 2
          if (ks == 0) {
            ok = mbar_poll(&full[s], fphase, kWaitLimit);
            if (!ok) break;
            if (trace && (int)(cc - cc_tile) < 8) trace[TR_FULL + (int)(cc - cc_tile)] = globaltimer_ns();
            tc_fence_after();
            ahi = smem_desc_at(abits, sm0 + L.stage0 + (uint32_t)s * stage_bytes);
          }
          const uint32_t first_main = newreg ? 0u : 1u;  // 0: the step starts the region
          const uint32_t first_corr = t == 0 ? 0u : 1u;
          for (int hh = 0; hh < S.mh; ++hh) {
            const uint64_t ah = ahi + (uint64_t)(hh * S.a_half16);
            const uint64_t bo = (uint64_t)hh * bstep_half;  // parity split: each half its own B
            if constexpr (BF) {
              mma_bf16(dm0 + (uint32_t)(hh * S.nc), ah, bh + bo, idesc, first_main);
              mma_bf16(dc0 + (uint32_t)(hh * S.nc), ah, bl + bo, idesc, first_corr);
              mma_bf16(dc0 + (uint32_t)(hh * S.nc), ah + (uint64_t)(S.chunk_bytes >> 4), bh + bo, idesc, 1u);
            } else {
              mma_tf32(dm0 + (uint32_t)(hh * S.nc), ah, bh + bo, idesc, first_main);
              mma_tf32(dc0 + (uint32_t)(hh * S.nc), ah, bl + bo, idesc, first_corr);
              mma_tf32(dc0 + (uint32_t)(hh * S.nc), ah + (uint64_t)(S.chunk_bytes >> 4), bh + bo, idesc, 1u);
            }
          }
          bh += (uint64_t)(2 * kLboB >> 4);
          bl += (uint64_t)(2 * kLboB >> 4);
          ahi += (uint64_t)(256 >> 4);
          racc += fs.nused;
          newreg = racc >= span;
          if (newreg) {
            racc -= span;
            ++rm;
            dm0 = tmem + (uint32_t)(rm * S.reg_cols);
          }
          if (ks == kpc - 1) {
            mma_commit(&empty[s]);
            if (trace && (int)(cc - cc_tile) < 8) trace[TR_MMA + (int)(cc - cc_tile)] = globaltimer_ns();
            ++cc;
            if (++s == ns) {
              s = 0;
              fphase ^= 1u;
            }
          }
        }
        if (ok) mma_commit(dbar);
      }
    }
  }
  if (!ok) {
    *fail = 1;
    // every MMA already issued completes before the tensor memory is released
    mma_commit(quiet);
    mbar_poll(quiet, 0u, kWaitLimit);
  }
}

// Warp 9, lane 0, split-BF16x6: the same schedule as mma_issuer with its invariants in
// registers and the loops over the K steps of a chunk and the M halves unrolled (MH = 1:
// chunks of two K steps; MH = 2: one), so the lane spends its time issuing products rather
// than recomputing descriptors (a probe measured the product issue itself at ~51 cycles).
template <int MH, typename Resolve>
__device__ __noinline__ void mma_issuer_oz(Resolve resolve, int64_t total, const TcShape S, uint32_t sm0,
                                           const TcSmemLayout L, uint32_t tmem, volatile int* fail) {
  using namespace tc;
  constexpr int KPC = MH == 1 ? 2 : 1;  // K steps per chunk
  uint64_t* full = reinterpret_cast<uint64_t*>(sm_ptr(sm0 + L.bars));
  const int ns = S.stages;
  uint64_t* empty = full + ns;
  uint64_t* dbar = full + 2 * ns;
  uint64_t* bready = dbar + 2;
  uint64_t* quiet = dbar + 3;
  const uint32_t idesc = idesc_bf16(128, (uint32_t)S.nc);
  const uint64_t bbits = smem_desc_bits(kLboB, L.sbo_b), abits = smem_desc_bits(128, (uint32_t)S.sbo_a);
  const uint64_t b0 = smem_desc_at(bbits, sm0 + L.bhi), b1 = smem_desc_at(bbits, sm0 + L.bmid),
                 b2 = smem_desc_at(bbits, sm0 + L.blo);
  const uint64_t a_first = smem_desc_at(abits, sm0 + L.stage0), a_stage = (uint64_t)(L.stage_bytes >> 4);
  const uint64_t slice = (uint64_t)(S.chunk_bytes >> 4), ahalf = (uint64_t)S.a_half16;
  const uint64_t bhalf = S.par ? (uint64_t)(L.bhalf >> 4) : 0u;
  constexpr uint64_t kBStep = (uint64_t)(2 * kLboB >> 4), kAStep = (uint64_t)(256 >> 4);
  const uint32_t rc = (uint32_t)S.reg_cols, nch = (uint32_t)S.nc;
  const int ksteps = S.ksteps;
  int64_t cc = 0;
  int s = 0;
  uint32_t fphase = 0, nready = 0;
  bool ok = true;
  for (int64_t gt = blockIdx.x; gt < total && ok; gt += gridDim.x) {
    const TileRef tr = resolve(gt);
    const int nmat = tr.prm->nmat;
    unsigned long long* trace = tr.prm->trace ? tr.prm->trace + tr.tile * kTraceSlots : nullptr;
    const int64_t cc_tile = cc;
    for (int m = 0; m < nmat && ok; ++m) {
      ok = mbar_poll(bready, nready & 1u, kWaitLimit);
      ++nready;
      tc_fence_after();
      uint64_t bh = b0, bm = b1, bl = b2;
      for (int t = 0; t < ksteps && ok; t += KPC) {
        ok = mbar_poll(&full[s], fphase, kWaitLimit);
        if (!ok) break;
        if (trace && (int)(cc - cc_tile) < 8) trace[TR_FULL + (int)(cc - cc_tile)] = globaltimer_ns();
        tc_fence_after();
        uint64_t a = a_first + (uint64_t)s * a_stage;
#pragma unroll
        for (int kk = 0; kk < KPC; ++kk) {
          const uint32_t acc = (t + kk) > 0 ? 1u : 0u;
#pragma unroll
          for (int hh = 0; hh < MH; ++hh) {
            const uint64_t a0 = a + (uint64_t)hh * ahalf, bo = (uint64_t)hh * bhalf;
            const uint32_t r0 = tmem + (uint32_t)hh * nch;
            mma_bf16(r0, a0, bh + bo, idesc, acc);
            mma_bf16(r0 + rc, a0, bm + bo, idesc, acc);
            mma_bf16(r0 + rc, a0 + slice, bh + bo, idesc, 1u);
            mma_bf16(r0 + 2u * rc, a0, bl + bo, idesc, acc);
            mma_bf16(r0 + 2u * rc, a0 + slice, bm + bo, idesc, 1u);
            mma_bf16(r0 + 2u * rc, a0 + 2u * slice, bh + bo, idesc, 1u);
          }
          bh += kBStep;
          bm += kBStep;
          bl += kBStep;
          a += kAStep;
        }
        mma_commit(&empty[s]);
        if (trace && (int)(cc - cc_tile) < 8) trace[TR_MMA + (int)(cc - cc_tile)] = globaltimer_ns();
        ++cc;
        if (++s == ns) {
          s = 0;
          fphase ^= 1u;
        }
      }
      if (ok) mma_commit(dbar);
    }
  }
  if (!ok) {
    *fail = 1;
    // every MMA already issued completes before the tensor memory is released
    mma_commit(quiet);
    mbar_poll(quiet, 0u, kWaitLimit);
  }
}

// The tiles blockIdx.x, blockIdx.x + gridDim.x, ... of a launch (every tile of a launch
// has the same lane extent n).
// PK > 1: packed tiles of lane extent 128 / PK (see tab_w): the tensor core sees one
// 128-row tile whose row R is lane row R % nl of column group R / nl, with the lane matrix
// block-diagonal (PK copies), so no accumulator row and no epilogue thread is idle.
// A finished tile's norm partials, waiting to be published: the work warps of the next tile
// write them and draw the pass ticket while that tile's first GEMM runs (or after the CTA's
// last tile), so the ticket's fence and atomic round trip stay off the tile chain.
struct PendTicket {
  const TcParams* prm;  // nullptr: nothing pending
  double* partials;
  unsigned int* counter;
  int64_t tiles, tile;
  int nred;
  double red[kMaxRed];
};

// Warp 0 (all lanes): publish the pending partials; the CTA that draws a pass's last ticket
// folds all of the pass's partials in FP64 in a fixed order and runs its scalar ops.
__device__ __noinline__ void publish_pending(PendTicket& pd, double* totals, int lane) {
  const TcParams* q = pd.prm;
  if (q == nullptr) return;
  double* const part = pd.partials;
  const int64_t tiles = pd.tiles;
  const int nred = pd.nred;
  unsigned int last = 0u;
  if (lane == 0) {
    for (int k = 0; k < nred; ++k) part[(int64_t)k * tiles + pd.tile] = pd.red[k];
    __threadfence();
    last = atomicAdd(pd.counter, 1u) == (unsigned int)(tiles - 1) ? 1u : 0u;
  }
  last = __shfl_sync(0xffffffffu, last, 0);
  __syncwarp();
  if (lane == 0) pd.prm = nullptr;
  if (!last) return;
  __threadfence();
  for (int k = 0; k < nred; ++k) {
    double a = 0.0;
    for (int64_t b = lane; b < tiles; b += 32) a += __ldcg(part + (int64_t)k * tiles + b);
#pragma unroll
    for (int o2 = 16; o2 > 0; o2 >>= 1) a += __shfl_down_sync(0xffffffffu, a, o2);
    if (lane == 0) totals[k] = a;
  }
  __syncwarp();
  if (lane == 0) {
    const PassParams& p = q->p;
    for (int oi = 0; oi < p.nops; ++oi) run_scalar_tc(p, p.ops[oi], totals);
    __threadfence();
    *p.counter = 0u;
  }
  __syncwarp();
}

template <bool BF, bool OZ, int PK, typename Resolve>
__device__ __forceinline__ void tc_persistent(Resolve resolve, const int64_t total) {
  using namespace tc;
  extern __shared__ __align__(1024) unsigned char sm[];
  __shared__ __align__(16) TcParams tp;  // the pass of the work warps' current tile
  __shared__ TileTabs tabs;
  __shared__ uint32_t tmem_base_s;
  __shared__ FF scratch[kMaxRed * (kWorkThreads / 32)];
  __shared__ double blk_red[kMaxRed];
  __shared__ double totals[kMaxRed];
  __shared__ PendTicket s_pend;
  __shared__ volatile int s_fail;
  // split-BF16x6: column maxima of the two B operands of a tile (re and im of each column; a
  // packed tile keeps one set per column group: its block-diagonal matrix only sums products
  // within a group, so each group's columns carry their own quanta)
  constexpr int kCm = 64 * PK;
  __shared__ uint32_t s_colmax[2][kCm];
  static_assert(sizeof(TcParams) % 4 == 0, "TcParams is copied as 32-bit words");
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  if (blockIdx.x >= total) return;
  const TcParams* first = resolve(blockIdx.x).prm;  // every tile of a launch shares n and parity mode
  const int nl = (int)first->p.g.n;  // the lane extent; n: the tile's rows (nl PK)
  const int n = nl * PK;
  const bool par = first->parity[0] != 0;
  const TcShape S = tc_shape(n, par, BF, OZ);
  const TcSmemLayout L = tc_layout(n, par, BF, OZ);
  uint64_t* bars = reinterpret_cast<uint64_t*>(sm + L.bars);
  uint64_t* dbar = bars + 2 * S.stages;  // MMAs of a fill completed (the work warps drain)
  uint64_t* freebar = dbar + 1;         // the work warps drained a fill (regions free again)
  uint64_t* bready = dbar + 2;          // the B operand of the next matrix is written
  float* bhi = reinterpret_cast<float*>(sm + L.bhi);  // also the FP32 output staging
  unsigned char* bhb = sm + L.bhi;                    // B operand images (hi, lo; mid for OZ)
  unsigned char* bmb = sm + L.bmid;
  unsigned char* blb = sm + L.blo;

  if (tid == 0) {
    for (int k = 0; k < 2 * S.stages; ++k) mbar_init(bars + k, 1);  // full[], empty[]
    mbar_init(dbar, 1);
    mbar_init(freebar, kWorkThreads);
    mbar_init(bready, kWorkThreads);
    mbar_init(dbar + 3, 1);  // quiet
    fence_mbar_init();
    s_fail = 0;
    s_pend.prm = nullptr;
  }
  if (warp == 0) tmem_alloc(&tmem_base_s, kTmemCols);
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = tmem_base_s;
  const uint32_t sm0 = smem_u32(sm);

  if (warp == kWorkThreads / 32) {
    if (lane == 0) tma_producer(resolve, total, S, sm0, L, &s_fail);
  } else if (warp == kWorkThreads / 32 + 1) {
    if (lane == 0) {
      if constexpr (OZ) {
        if (S.mh == 2)
          mma_issuer_oz<2>(resolve, total, S, sm0, L, tmem, &s_fail);
        else
          mma_issuer_oz<1>(resolve, total, S, sm0, L, tmem, &s_fail);
      } else {
        mma_issuer<BF>(resolve, total, S, sm0, L, tmem, &s_fail);
      }
    }
  } else {
    // ================= work warps
    const int lg = warp & 3, up = warp >> 2;
    const int i = 32 * lg + lane;                    // TMEM lane within a 128-row half
    const int j = (S.mh == 2 ? 128 * up : 0) + i;    // lane-axis row of a plain drain
    const bool row_ok = j < n;
    // kVals FP32 columns per thread.  Plain: n <= 128 the upper warps take the second half
    // of N = 64, n = 256 the second 128-row half (its N = 32 columns).  Parity split,
    // sum / difference matrix: as plain, the row of half h lane i being 2 i + h.  Even /
    // odd matrix: columns 16 up .. 16 up + 15 of both halves (E, O), rows i and n-1-i.
    const int c0 = S.mh == 2 ? 0 : (kVals / 2) * up;  // complex column of v[0..1] (plain)
    const uint32_t lane_base = tmem + ((uint32_t)(lg * 32) << 16);
    constexpr int kLd = kVals / 32;  // 16-column loads per half of a thread's columns (even / odd form)
    const uint32_t bhb2 = L.bhalf;  // bytes between the two B halves
    float* stg = bhi;  // output staging reuses the B_hi area once the last GEMM is done
    uint32_t drains = 0;
    const TcParams* cur = nullptr;
    for (int64_t gt = blockIdx.x; gt < total; gt += gridDim.x) {
      const TileRef r = resolve(gt);
      if (r.prm != cur) {
        for (int k = tid; k < (int)(sizeof(TcParams) / 4); k += kWorkThreads)
          reinterpret_cast<uint32_t*>(&tp)[k] = reinterpret_cast<const uint32_t*>(r.prm)[k];
        cur = r.prm;
        work_sync();
      }
      const PassParams& p = tp.p;
      const Geometry& g = p.g;
      const int64_t tile = r.tile;
      const int64_t o = tile / g.tiles_per_outer;
      const int64_t i0 = (tile - o * g.tiles_per_outer) * S.bn * PK;
      const int64_t base = o * g.n * g.inner + i0;  // element (row 0, column 0) of the tile
      float2* psi = reinterpret_cast<float2*>(p.psi);
      if (tid == 0) trace_mark(tp, tile, TR_START);

      // a pass that starts with its matrix needs the tables only after the first GEMM: they
      // are built while it runs (after the prologue) instead of ahead of the prologue
      const bool late_tabs = tp.mat_op[0] == 0;
      if (!late_tabs) build_tile_tabs<PK>(p, tabs, o, i0, S.bn * PK);
      // full-size tables read after the first lane matrix (each distinct table once, listed on
      // the host): start their tile rows toward L2
      for (int q = 0; q < tp.npre; ++q) {
        const float2* t = reinterpret_cast<const float2*>(tp.pre[q]) + base;
        if ((reinterpret_cast<uintptr_t>(t) & 15u) == 0)
          for (int jj = tid; jj < nl; jj += kWorkThreads)
            prefetch_lines_l2(t + (int64_t)jj * g.inner, (uint32_t)(S.bn * PK * sizeof(float2)));
      }
      if constexpr (OZ)
        for (int k = tid; k < 2 * kCm; k += kWorkThreads) s_colmax[k / kCm][k % kCm] = 0u;
      work_sync();  // tabs complete; the previous tile's staging has been stored
      if (tid == 0) trace_mark(tp, tile, TR_TABS);

      // per-thread FP32 partial sums of the norms of this tile
      float acc[kMaxRed];
#pragma unroll
      for (int k = 0; k < kMaxRed; ++k) acc[k] = 0.0f;
      {
        // prologue: thread = complex column c, rows h, h + G, ... (G = groups)
        // rows per thread: n / G = 4, 8 or 16 (n / 2 / G = 8 for the sum / difference pairs)
        const int c = tid % S.bn, h = tid / S.bn, G = S.groups;
        const int k0 = tp.parity[0];
        const int mo = tp.mat_op[0];
        unsigned long long* lm = (tid == 0 && tp.trace) ? tp.trace + tile * kTraceSlots + TR_LOADED : nullptr;
        uint32_t* cm0 = s_colmax[0];
        if (k0 == 1)
          prologue_vec<2, 4, 1, BF, OZ>(p, tabs, mo, psi, base, c, h, G, n, bhb, bmb, blb, bhb2, L.sbo_b, acc, lm, cm0);
        else if (k0 == 2)
          prologue_vec<2, 8, 2, BF, OZ>(p, tabs, mo, psi, base, c, h, G, n, bhb, bmb, blb, bhb2, L.sbo_b, acc, lm, cm0);
        else if (n / G == 16)
          prologue_vec<4, 4, 0, BF, OZ, PK>(p, tabs, mo, psi, base, c, h, G, n, bhb, bmb, blb, 0, L.sbo_b, acc, lm,
                                            cm0, nl, S.bn);
        else if (n / G == 8)
          prologue_vec<2, 4, 0, BF, OZ>(p, tabs, mo, psi, base, c, h, G, n, bhb, bmb, blb, 0, L.sbo_b, acc, lm, cm0);
        else
          prologue_vec<1, 4, 0, BF, OZ>(p, tabs, mo, psi, base, c, h, G, n, bhb, bmb, blb, 0, L.sbo_b, acc, lm, cm0);
        if (tid == 0) trace_mark(tp, tile, TR_STORED);
        fence_proxy_async();
        mbar_arrive(bready);
      }
      if (tid == 0) trace_mark(tp, tile, TR_PROLOGUE);
      // the next tile's state rows toward L2 (its prologue loads then hit L2); issued behind
      // this tile's prologue, since finding the next tile's pass reads its descriptor
      if (gt + gridDim.x < total) {
        const TileRef rn = resolve(gt + gridDim.x);
        const Geometry& gn = rn.prm->p.g;
        const int64_t on = rn.tile / gn.tiles_per_outer;
        const float2* pn = reinterpret_cast<const float2*>(rn.prm->p.psi) + on * gn.n * gn.inner +
                           (rn.tile - on * gn.tiles_per_outer) * S.bn * PK;
        for (int jj = tid; jj < nl; jj += kWorkThreads)
          prefetch_lines_l2(pn + (int64_t)jj * gn.inner, (uint32_t)(S.bn * PK * sizeof(float2)));
      }
      // (the first drain's barrier orders these writes before the epilogue reads them)
      if (late_tabs) build_tile_tabs<PK>(p, tabs, o, i0, S.bn * PK);
      // lane-axis weights of this thread's epilogue rows for the norms after the first
      // matrix, loaded now (they arrive while the GEMM runs)
      const float* rw_ptr = nullptr;
      for (int oi = tp.mat_op[0] + 1; oi < p.nops && rw_ptr == nullptr; ++oi)
        if (p.ops[oi].kind == OP_NORM) rw_ptr = p.ops[oi].wf[g.sweep_axis];
      float rw_plain = 0.0f, rw_sum = 0.0f, rw_a = 0.0f, rw_b = 0.0f;
      if (rw_ptr) {
        if (row_ok) rw_plain = __ldg(rw_ptr + (PK > 1 ? (j & (nl - 1)) : j));
        if (S.par) {
          rw_sum = __ldg(rw_ptr + 2 * i + up);
          rw_a = __ldg(rw_ptr + i);
          rw_b = __ldg(rw_ptr + (n - 1 - i));
        }
      }

      // the previous tile's partials and ticket, while this tile's first GEMM runs
      if (warp == 0) publish_pending(s_pend, totals, lane);

      bool ok = true;
      for (int m = 0; m < tp.nmat && ok; ++m) {
        const int kind = tp.parity[m];
        const bool last = m + 1 == tp.nmat;
        const int next = last ? -1 : tp.parity[m + 1];
        // ops between this matrix and the next one (or the end of the program)
        const int sb = tp.mat_op[m] + 1, se = last ? p.nops : tp.mat_op[m + 1];
        float v[kVals];
#pragma unroll
        for (int e = 0; e < kVals; ++e) v[e] = 0.0f;
        if constexpr (OZ) {
          // one drain per matrix: R2 + R1 + R0, the small orders first (round to nearest)
          ok = work_all(mbar_wait(dbar, drains & 1u, kWaitLimit));
          if (ok) {
            ++drains;
            tc_fence_after();
#pragma unroll
            for (int hv = 0; hv < kVals / 8; ++hv) {
              // 8 columns of each region at a time (registers: the preloaded table row is live)
              const int h16 = hv >> 1;
              const uint32_t col = (kind == 2 ? (uint32_t)((h16 / kLd) * S.nc + (kVals / 2) * up + 16 * (h16 % kLd))
                                              : (uint32_t)(kVals * up + 16 * h16)) + 8u * (uint32_t)(hv & 1);
              float w0[8], w1[8], w2[8];
              tmem_ld8x3(lane_base + col, (uint32_t)S.reg_cols, w0, w1, w2);
#pragma unroll
              for (int e = 0; e < 8; ++e) v[8 * hv + e] = (w2[e] + w1[e]) + w0[e];
            }
            tc_fence_before();
          }
        } else
        for (int f = 0; f < S.fills; ++f) {
          ok = work_all(mbar_wait(dbar, drains & 1u, kWaitLimit));
          if (!ok) break;
          ++drains;
          tc_fence_after();
          const FillSpan fs = fill_span(S, f);
          // regions 0 .. nused-1 of the fill, then after the last fill the correction
          // region; round-to-nearest FP32 adds in a fixed order
          const int nr = fs.nused + (f + 1 == S.fills ? 1 : 0);
#pragma unroll 1
          for (int k = 0; k < nr; ++k) {
            const int rg = k < fs.nused ? k : S.nmain;
#pragma unroll
            for (int hv = 0; hv < kVals / 16; ++hv) {
              const uint32_t col = kind == 2 ? (uint32_t)((hv / kLd) * S.nc + (kVals / 2) * up + 16 * (hv % kLd))
                                             : (uint32_t)(kVals * up + 16 * hv);
              float w2[16];
              tmem_ld16(lane_base + (uint32_t)(rg * S.reg_cols) + col, w2);
#pragma unroll
              for (int e = 0; e < 16; ++e) v[16 * hv + e] += w2[e];
            }
          }
          tc_fence_before();
          if (f + 1 < S.fills) mbar_arrive(freebar);
        }
        if (!ok) break;
        if (tid == 0 && m < 2) trace_mark(tp, tile, TR_MAT0 + 2 * m);
        if (tid == 0 && m == 0) trace_mark(tp, tile, TR_DRAIN0);
        if (kind != 2) {
          const int jr = kind == 1 ? 2 * i + up : j;
          if constexpr (OZ) {
            // every work thread takes part in the column maxima of the next operand (rows past
            // the lane extent pass zeros)
            const bool valid = jr < n;
            float2 x[kVals / 2];
#pragma unroll
            for (int u = 0; u < kVals / 2; ++u) x[u] = valid ? float2{v[2 * u], v[2 * u + 1]} : float2{0.0f, 0.0f};
            if (valid) {
              if constexpr (PK > 1) {
                // packed: lane row jr % nl of column group jr / nl
                const int jl = jr & (nl - 1), cg = (jr / nl) * S.bn + c0;
                apply_row<kVals / 2, PK>(p, tabs, sb, se, x, jl, cg, base + (int64_t)jl * g.inner + cg, acc, rw_ptr,
                                         rw_plain);
              } else {
                apply_row<kVals / 2>(p, tabs, sb, se, x, jr, c0, base + (int64_t)jr * g.inner + c0, acc, rw_ptr,
                                     kind == 1 ? rw_sum : rw_plain);
              }
            }
            if (tid == 0 && m == 0) trace_mark(tp, tile, TR_APPLY0);
            if (last) {
              if (valid) stage_row<kVals / 2>(x, c0, jr, stg, S.stage_row);
            } else {
              // a warp whose rows all lie past the lane extent (n < 128) adds nothing
              // (a packed tile's warp holds rows of one column group: its maxima go to that
              // group's set)
              uint32_t* cm1 = s_colmax[1] + (PK > 1 ? (jr / nl) * 64 : 0);
              if (S.mh == 2 || 32 * lg < n) colmax_rows<kVals / 2>(x, c0, cm1);
              work_sync();
              if (tid == 0 && m == 0) trace_mark(tp, tile, TR_SYNC0);
              if (valid) {
                const uint32_t ho = next == 2 ? (uint32_t)(jr & 1) * bhb2 : 0u;
                write_b_row_oz<kVals / 2>(x, c0, next == 2 ? jr >> 1 : jr, bhb + ho, bmb + ho, blb + ho, L.sbo_b,
                                          cm1);
              }
            }
          } else if (jr < n) {
            // op-major over the thread's 32 complex values: the table loads of an op are all
            // in flight together
            float2 x[kVals / 2];
#pragma unroll
            for (int u = 0; u < kVals / 2; ++u) x[u] = {v[2 * u], v[2 * u + 1]};
            apply_row<kVals / 2>(p, tabs, sb, se, x, jr, c0, base + (int64_t)jr * g.inner + c0, acc, rw_ptr,
                                 kind == 1 ? rw_sum : rw_plain);
            if (last)
              stage_row<kVals / 2>(x, c0, jr, stg, S.stage_row);
            else if (next == 2)
              write_b_row<kVals / 2, BF>(x, c0, jr >> 1, bhb + (jr & 1) * bhb2, blb + (jr & 1) * bhb2, L.sbo_b);
            else
              write_b_row<kVals / 2, BF>(x, c0, jr, bhb, blb, L.sbo_b);
          }
        } else {
          // even / odd matrix: psi_i = E + O, psi_{n-1-i} = E - O
          const int cc0 = (kVals / 4) * up, ja = i, jb = n - 1 - i;
          float2 xa[kVals / 4], xb[kVals / 4];
#pragma unroll
          for (int u = 0; u < kVals / 4; ++u) {
            const float er = v[2 * u], ei = v[2 * u + 1], orr = v[kVals / 2 + 2 * u], oi = v[kVals / 2 + 2 * u + 1];
            xa[u] = {er + orr, ei + oi};
            xb[u] = {er - orr, ei - oi};
          }
          apply_row2<kVals / 4>(p, tabs, sb, se, xa, xb, ja, jb, cc0, base + (int64_t)ja * g.inner + cc0,
                                base + (int64_t)jb * g.inner + cc0, acc, rw_ptr, rw_a, rw_b);
          if (tid == 0 && m == 0) trace_mark(tp, tile, TR_APPLY0);
          if (last) {
            stage_row<kVals / 4>(xa, cc0, ja, stg, S.stage_row);
            stage_row<kVals / 4>(xb, cc0, jb, stg, S.stage_row);
          } else if (OZ && next == 1) {
            float2 sp[kVals / 4], sm2[kVals / 4];
#pragma unroll
            for (int u = 0; u < kVals / 4; ++u) {
              sp[u] = {xa[u].x + xb[u].x, xa[u].y + xb[u].y};
              sm2[u] = {xa[u].x - xb[u].x, xa[u].y - xb[u].y};
            }
            colmax_rows<kVals / 4>(sp, cc0, s_colmax[1]);
            colmax_rows<kVals / 4>(sm2, cc0, s_colmax[1]);
            work_sync();
            if (tid == 0 && m == 0) trace_mark(tp, tile, TR_SYNC0);
            write_b_row_oz<kVals / 4>(sp, cc0, i, bhb, bmb, blb, L.sbo_b, s_colmax[1]);
            write_b_row_oz<kVals / 4>(sm2, cc0, i, bhb + bhb2, bmb + bhb2, blb + bhb2, L.sbo_b, s_colmax[1]);
          } else if (OZ) {
            colmax_rows<kVals / 4>(xa, cc0, s_colmax[1]);
            colmax_rows<kVals / 4>(xb, cc0, s_colmax[1]);
            work_sync();
            if (tid == 0 && m == 0) trace_mark(tp, tile, TR_SYNC0);
            const uint32_t hoa = (uint32_t)(ja & 1) * bhb2, hob = (uint32_t)(jb & 1) * bhb2;
            write_b_row_oz<kVals / 4>(xa, cc0, ja >> 1, bhb + hoa, bmb + hoa, blb + hoa, L.sbo_b, s_colmax[1]);
            write_b_row_oz<kVals / 4>(xb, cc0, jb >> 1, bhb + hob, bmb + hob, blb + hob, L.sbo_b, s_colmax[1]);
          } else if (next == 1) {
            // sum / difference operand of the next matrix, K row i
            float2 sd[kVals / 4];
#pragma unroll
            for (int u = 0; u < kVals / 4; ++u) sd[u] = {xa[u].x + xb[u].x, xa[u].y + xb[u].y};
            write_b_row<kVals / 4, BF>(sd, cc0, i, bhb, blb, L.sbo_b);
#pragma unroll
            for (int u = 0; u < kVals / 4; ++u) sd[u] = {xa[u].x - xb[u].x, xa[u].y - xb[u].y};
            write_b_row<kVals / 4, BF>(sd, cc0, i, bhb + bhb2, blb + bhb2, L.sbo_b);
          } else {
            write_b_row<kVals / 4, BF>(xa, cc0, ja >> 1, bhb + (ja & 1) * bhb2, blb + (ja & 1) * bhb2, L.sbo_b);
            write_b_row<kVals / 4, BF>(xb, cc0, jb >> 1, bhb + (jb & 1) * bhb2, blb + (jb & 1) * bhb2, L.sbo_b);
          }
        }
        if (!last) {
          fence_proxy_async();
          mbar_arrive(bready);
        }
        if (tid == 0 && m < 2) trace_mark(tp, tile, TR_EPI0 + 2 * m);
      }
      if (!ok) {
        if (tid == 0) s_fail = 1;
        break;
      }
      work_sync();  // staging complete

      // norm partials of this tile (float-float, fixed order) and the pass ticket first, so
      // the fence waits for no state store and the ticket's round trip overlaps the store
      block_sums(acc, p.nred, scratch, blk_red);
      if (tid == 0) {
        // published by the next tile (or after the last one): see PendTicket
        s_pend.partials = p.partials;
        s_pend.counter = p.counter;
        s_pend.tiles = g.tiles;
        s_pend.tile = tile;
        s_pend.nred = p.nred;
        for (int k = 0; k < p.nred; ++k) s_pend.red[k] = blk_red[k];
        s_pend.prm = r.prm;
      }

      // coalesced store of the staged tile: thread = complex column
      {
        const int c = tid % S.bn, h = tid / S.bn, G = S.groups;
        for (int kb = h; kb < n; kb += 4 * G) {
#pragma unroll
          for (int u = 0; u < 4; ++u) {
            const int k = kb + u * G;
            const int64_t ix = PK > 1 ? (int64_t)(k & (nl - 1)) * g.inner + (k / nl) * S.bn + c
                                      : (int64_t)k * g.inner + c;
            psi[base + ix] = *reinterpret_cast<const float2*>(stg + k * S.stage_row + 2 * c);
          }
        }
      }
      if (tid == 0) trace_mark(tp, tile, TR_STORE);
      work_sync();  // the staging and the pass copy are free for the next tile
      if (tid == 0) trace_mark(tp, tile, TR_END);
    }
    // the last tile's partials (a CTA that stopped on a failed wait publishes nothing: the
    // pass has recorded its error)
    if (warp == 0 && !s_fail) publish_pending(s_pend, totals, lane);
  }
  __syncthreads();
  if (tid == 0 && s_fail) {
    // the pass of the first tile records the failure
    const TcParams* f0 = resolve(blockIdx.x).prm;
    if (f0->error_slot >= 0) f0->p.slots[f0->error_slot] = 1.0;
  }
  // teardown: every MMA has completed (drained, or waited on by the MMA warp)
  tc_fence_before();
  __syncthreads();
  if (warp == 0) tmem_dealloc(tmem, kTmemCols);
}

// OPM: operand mode, 0 = 3xTF32, 1 = split-BF16x3, 2 = split-BF16x6 (exact sums)
template <int OPM, int PK = 1>
__global__ void __launch_bounds__(kThreads, kCtasPerSm) angular_tc_kernel(const __grid_constant__ TcParams tp) {
  const TcParams* prm = &tp;
  tc_persistent<OPM != 0, OPM == 2, PK>([prm](int64_t t) { return TileRef{prm, t}; }, tp.p.g.tiles);
}

// Many propagations' lane-matrix passes in one launch (all with the same lane extent):
// global tile b is tile (b - offsets[i]) of params[i], offsets[i] <= b < offsets[i + 1];
// offsets[count] is the total.
template <int OPM, int PK = 1>
__global__ void __launch_bounds__(kThreads, kCtasPerSm) angular_tc_kernel_batched(const TcParams* __restrict__ params,
                                                                        const uint2* __restrict__ owners,
                                                                        int64_t total) {
  // owners[b] = (pass index, tile within the pass) of global tile b, built on the host: one
  // load per lookup (every warp looks up every tile it works on, the work warps also the
  // next one; a binary search over the offsets would be a chain of dependent loads)
  auto resolve = [params, owners](int64_t b) {
    const uint2 o = __ldg(owners + b);
    return TileRef{params + o.x, (int64_t)o.y};
  };
  tc_persistent<OPM != 0, OPM == 2, PK>(resolve, total);
}

// ------------------------------------------------------------------ host side
size_t angular_tc_smem_bytes(int n, bool par, int mode) { return tc_layout(n, par, mode != 0, mode == 2).total; }

int angular_tc_columns(int n) { return tc_shape(n).bn; }

size_t tc_params_bytes() { return sizeof(TcParams); }

void make_tc_params(const PassParams& p, const int* mat_op, int nmat, const float* const* images, int error_slot,
                    const int* parity, void* out, int pack, const int* slice_axis, const int64_t* slice_stride) {
  TcParams tp{};
  tp.p = p;
  tp.pack = pack;
  tp.nmat = nmat;
  tp.slice_axis[0] = tp.slice_axis[1] = -1;
  for (int i = 0; i < nmat; ++i) {
    tp.mat_op[i] = mat_op[i];
    tp.images[i] = images[i];
    tp.parity[i] = parity ? parity[i] : 0;
    if (slice_axis && slice_axis[i] >= 0) {
      // the tile's coordinate along the slice axis (storage position q): an outer axis from
      // the tile's outer index o = tile / tiles_per_outer, an inner one from its first column
      // i0 = (tile mod tiles_per_outer) x columns (the axis's stride a multiple of columns)
      const Geometry& g = p.g;
      int q = 0;
      for (int a = 0; a < g.ndim; ++a)
        if (g.perm[a] == slice_axis[i]) q = a;
      int64_t div = 1;
      if (q < g.spos) {
        for (int a = q + 1; a < g.spos; ++a) div *= g.sshape[a];
        tp.slice_pre[i] = 0;
        tp.slice_div[i] = (uint32_t)(div * g.tiles_per_outer);
      } else {
        for (int a = q + 1; a < g.ndim; ++a) div *= g.sshape[a];
        tp.slice_pre[i] = (uint32_t)g.tiles_per_outer;
        tp.slice_div[i] = (uint32_t)(div / g.lanes_per_tile);
      }
      tp.slice_ext[i] = (uint32_t)g.sshape[q];
      tp.slice_axis[i] = slice_axis[i];
      tp.slice_stride[i] = slice_stride[i];
    }
  }
  tp.error_slot = error_slot;
  // the distinct full-size tables after the first matrix (the kernel prefetches their tile rows)
  for (int oi = nmat > 0 ? mat_op[0] + 1 : p.nops; oi < p.nops && tp.npre < 4; ++oi) {
    if (p.ops[oi].kind != OP_DIAGND) continue;
    bool seen = false;
    for (int q = 0; q < tp.npre; ++q) seen = seen || tp.pre[q] == p.ops[oi].ptr;
    if (!seen) tp.pre[tp.npre++] = p.ops[oi].ptr;
  }
  std::memcpy(out, &tp, sizeof(TcParams));
}

void tc_params_set_trace(void* params, unsigned long long* trace) {
  reinterpret_cast<TcParams*>(params)->trace = trace;
}

// the largest dynamic shared memory any supported lane extent asks for
static size_t tc_max_dynamic_smem() {
  size_t m = 0;
  for (int n = 32; n <= 256; n *= 2)
    for (int par = 0; par < 2; ++par)
      for (int mode = 0; mode < 3; ++mode) {
        const size_t t = tc_layout(n, par, mode != 0, mode == 2).total;
        m = t > m ? t : m;
      }
  return m;
}

// persistent CTAs with the whole shared-memory carveout
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

// persistent grid: ctas_per_sm (1 or 2; 0 = kCtasPerSm) CTAs per SM, fewer when there are
// fewer tiles
static unsigned persistent_grid(int64_t tiles, int ctas_per_sm = 0) {
  static int sms = 0;
  if (sms == 0) {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) !=
                                                  cudaSuccess)
      sms = 1;
  }
  const int per = (ctas_per_sm == 1 || ctas_per_sm == 2) ? ctas_per_sm : kCtasPerSm;
  const int64_t slots = (int64_t)sms * per;
  return (unsigned)(tiles < slots ? tiles : slots);
}

int64_t angular_tc_grid(int64_t tiles, int ctas_per_sm) { return (int64_t)persistent_grid(tiles, ctas_per_sm); }

// kernel variants: operand modes 0, 1, 2 unpacked, and split-BF16x6 packed 2 and 4 ways
static int tc_variant(int mode, int pack) {
  if (mode < 0 || mode > 2) return -1;
  if (pack == 1) return mode;
  if (mode == 2 && pack == 2) return 3;
  if (mode == 2 && pack == 4) return 4;
  return -1;
}

cudaError_t launch_angular_tc_batched(const void* params_dev, const void* owners_dev, int64_t blocks, size_t smem,
                                      int mode, cudaStream_t s, int ctas_per_sm, int pack) {
  static bool configured[5] = {false, false, false, false, false};
  const int v = tc_variant(mode, pack);
  if (v < 0) return cudaErrorInvalidValue;
  const void* kerns[5] = {(const void*)angular_tc_kernel_batched<0>, (const void*)angular_tc_kernel_batched<1>,
                          (const void*)angular_tc_kernel_batched<2>, (const void*)angular_tc_kernel_batched<2, 2>,
                          (const void*)angular_tc_kernel_batched<2, 4>};
  if (!configure_once(kerns[v], configured[v])) return cudaGetLastError();
  if (smem > tc_max_dynamic_smem()) return cudaErrorInvalidValue;
  const TcParams* prm = reinterpret_cast<const TcParams*>(params_dev);
  const uint2* own = reinterpret_cast<const uint2*>(owners_dev);
  const unsigned grid = persistent_grid(blocks, ctas_per_sm);
  switch (v) {
    case 4: angular_tc_kernel_batched<2, 4><<<grid, kThreads, smem, s>>>(prm, own, blocks); break;
    case 3: angular_tc_kernel_batched<2, 2><<<grid, kThreads, smem, s>>>(prm, own, blocks); break;
    case 2: angular_tc_kernel_batched<2><<<grid, kThreads, smem, s>>>(prm, own, blocks); break;
    case 1: angular_tc_kernel_batched<1><<<grid, kThreads, smem, s>>>(prm, own, blocks); break;
    default: angular_tc_kernel_batched<0><<<grid, kThreads, smem, s>>>(prm, own, blocks); break;
  }
  count_launch();
  return cudaGetLastError();
}

bool angular_tc_eligible(const Geometry& g) {
  if (!(g.n == 32 || g.n == 64 || g.n == 128 || g.n == 256)) return false;
  const int bn = tc_shape((int)g.n).bn;
  return g.inner >= bn && g.inner % bn == 0;
}

// Column groups a tile of this pass packs (split-BF16x6, lanes of 32 or 64 points): 128 / n
// when the tile's 128 / n groups of 32 columns fit the inner axis and the pass's tables have
// the packed form (two axes, the lane axis outermost; every norm with the same weights and
// every across-lane diagonal with the same table), else 1.
int angular_tc_pack(const Geometry& g, const DevOp* ops, int nops, int mode) {
  if (mode != 2 || !(g.n == 32 || g.n == 64) || g.ndim != 2 || g.spos != 0 || g.outer != 1) return 1;
  const int pk = (int)(128 / g.n), bn = tc_shape((int)g.n).bn;
  if (g.inner % ((int64_t)pk * bn) != 0) return 1;
  const float* w = nullptr;
  const void* t = nullptr;
  const int other = g.perm[1];
  for (int i = 0; i < nops; ++i) {
    const DevOp& o = ops[i];
    if (o.kind == OP_NORM) {
      if (w && w != o.wf[other]) return 1;
      w = o.wf[other];
    } else if (diag1d_across(o, g.sweep_axis)) {
      if (t && t != o.ptr) return 1;
      t = o.ptr;
    } else if (!(o.kind == OP_MAT || o.kind == OP_DIAGND || o.kind == OP_SCALE || o.kind == OP_COPY ||
                 o.kind == OP_LOSS || o.kind == OP_SETC || o.kind == OP_RECORD ||
                 (o.kind == OP_DIAG1D && o.axis == g.sweep_axis))) {
      return 1;
    }
  }
  return pk;
}

bool angular_tc_ops_fit(const DevOp* ops, int nops, int sweep_axis) {
  int across = 0;
  for (int i = 0; i < nops; ++i) across += diag1d_across(ops[i], sweep_axis);
  return across <= kColtSlots;
}

// Chunk images of the A operand: rows x kdim values a(r, k); per K chunk chunk_bytes of
// high parts then chunk_bytes of remainders, both exact in the operand format, each in the K-major
// core-matrix order (row-group stride sbo_a, K core-matrix stride 128 B).  3xTF32: tf32
// values in 4-byte words; split-BF16x3: bf16 values in 2-byte halves of the same buffer.
template <typename F>
static void tc_images(const TcShape& S, bool bf, F a, std::vector<float>& out) {
  const int rows = 128 * S.mh;
  out.assign((size_t)S.nk * 2 * (S.chunk_bytes / 4), 0.0f);
  auto tf32 = [](float x) {
    uint32_t b;
    std::memcpy(&b, &x, 4);
    b = (b + 0x1000u) & 0xFFFFE000u;
    float r;
    std::memcpy(&r, &b, 4);
    return r;
  };
  auto bf16 = [](float x) -> uint16_t {  // round to nearest even (finite inputs)
    uint32_t b;
    std::memcpy(&b, &x, 4);
    b += 0x7FFFu + ((b >> 16) & 1u);
    return (uint16_t)(b >> 16);
  };
  auto bf16_value = [](uint16_t h) {
    const uint32_t b = (uint32_t)h << 16;
    float r;
    std::memcpy(&r, &b, 4);
    return r;
  };
  for (int q = 0; q < S.nk; ++q) {
    unsigned char* hi = reinterpret_cast<unsigned char*>(out.data() + (size_t)q * 2 * (S.chunk_bytes / 4));
    unsigned char* lo = hi + S.chunk_bytes;
    for (int r = 0; r < rows; ++r)
      for (int kk = 0; kk < S.chunk_k; ++kk) {
        const double v = a(r, q * S.chunk_k + kk);
        const size_t off = (size_t)(r >> 3) * S.sbo_a + (size_t)(kk / S.kc) * 128 + (size_t)(r & 7) * 16 +
                           (size_t)(kk % S.kc) * (bf ? 2 : 4);
        if (bf) {
          const uint16_t h = bf16((float)v);
          const uint16_t l = bf16((float)(v - (double)bf16_value(h)));
          std::memcpy(hi + off, &h, 2);
          std::memcpy(lo + off, &l, 2);
        } else {
          const float h = tf32((float)v);
          const float l = tf32((float)(v - (double)h));  // the tensor core would truncate an unrounded remainder
          std::memcpy(hi + off, &h, 4);
          std::memcpy(lo + off, &l, 4);
        }
      }
  }
}

// Split-BF16x6 chunk images: per K chunk three slice images s0, s1, s2 (bf16, the same
// core-matrix order), each row cut at the power of two above its largest magnitude over all
// of K: a = s0 + s1 + s2 + O(2^-24 max), s_i a multiple of 2^(e-8-8i) with |s_i| <= 2^(e-8i)
// (see oz_quanta for the B side and why the sums are then exact).
template <typename F>
static void tc_images_oz(const TcShape& S, F a, std::vector<float>& out) {
  const int rows = 128 * S.mh;
  out.assign((size_t)S.nk * 3 * (S.chunk_bytes / 4), 0.0f);
  std::vector<double> q0(rows, 0.0);
  for (int r = 0; r < rows; ++r) {
    double amax = 0.0;
    for (int k = 0; k < S.kdim; ++k) amax = std::max(amax, std::fabs(a(r, k)));
    int e = 0;
    if (amax > 0.0) std::frexp(amax, &e);  // amax < 2^e
    q0[r] = amax > 0.0 ? std::ldexp(1.0, e - 8) : 0.0;
  }
  auto bf16_bits = [](double s) {  // s is exactly a bf16 value
    const float f = (float)s;
    uint32_t b;
    std::memcpy(&b, &f, 4);
    return (uint16_t)(b >> 16);
  };
  for (int q = 0; q < S.nk; ++q) {
    unsigned char* base = reinterpret_cast<unsigned char*>(out.data() + (size_t)q * 3 * (S.chunk_bytes / 4));
    for (int r = 0; r < rows; ++r) {
      if (q0[r] == 0.0) continue;
      const double qs[3] = {q0[r], std::ldexp(q0[r], -8), std::ldexp(q0[r], -16)};
      for (int kk = 0; kk < S.chunk_k; ++kk) {
        double rem = a(r, q * S.chunk_k + kk);
        const size_t off = (size_t)(r >> 3) * S.sbo_a + (size_t)(kk / S.kc) * 128 + (size_t)(r & 7) * 16 +
                           (size_t)(kk % S.kc) * 2;
        for (int sl = 0; sl < 3; ++sl) {
          const double sv = std::nearbyint(rem / qs[sl]) * qs[sl];
          rem -= sv;
          const uint16_t h = bf16_bits(sv);
          std::memcpy(base + (size_t)sl * S.chunk_bytes + off, &h, 2);
        }
      }
    }
  }
}

// One real n x n matrix (row-major FP64: out[r] = sum_k m[r][k] in[k]), zero-padded to M.
// mode: 0 3xTF32, 1 split-BF16x3, 2 split-BF16x6
void angular_tc_images(const double* m, int n, int mode, std::vector<float>& out) {
  auto a = [&](int r, int k) { return (r < n && k < n) ? m[(size_t)r * n + k] : 0.0; };
  if (mode == 2)
    tc_images_oz(tc_shape(n, false, true, true), a, out);
  else
    tc_images(tc_shape(n, false, mode == 1), mode == 1, a, out);
}

// Parity structure of a lane matrix for the split form (n = 256 only):
//   1  m[l][n-1-j] = (-1)^l m[l][j]  (e.g. the Legendre transform T[l][j] = sqrt(l+1/2) P_l(x_j) w_j
//      on symmetric nodes): out[2a + h] = sum_{j < n/2} m[2a + h][j] (in[j] +- in[n-1-j])
//   2  m[n-1-j][l] = (-1)^l m[j][l]  (its inverse P_l(x_j) sqrt(l+1/2)): with E_j / O_j the
//      sums over even / odd l, out[j] = E_j + O_j and out[n-1-j] = E_j - O_j
//   0  neither (to 1e-12 of the largest entry)
int angular_tc_parity(const double* m, int n) {
  if (n != 256) return 0;
  double amax = 0.0;
  for (int i = 0; i < n * n; ++i) amax = std::max(amax, std::fabs(m[i]));
  const double tol = 1e-12 * amax;
  bool rowp = true, colp = true;
  for (int a = 0; a < n && (rowp || colp); ++a)
    for (int b = 0; b < n; ++b) {
      const double sg = (a & 1) ? -1.0 : 1.0;
      if (rowp && std::fabs(m[(size_t)a * n + (n - 1 - b)] - sg * m[(size_t)a * n + b]) > tol) rowp = false;
      if (colp && std::fabs(m[(size_t)(n - 1 - b) * n + a] - sg * m[(size_t)b * n + a]) > tol) colp = false;
    }
  return rowp ? 1 : (colp ? 2 : 0);
}

// A images of the split form: rows 0..127 the first half (even l, or E), rows 128..255
// the second (odd l, or O), K = n / 2.
void angular_tc_parity_images(const double* m, int n, int kind, int mode, std::vector<float>& out) {
  const int hn = n / 2;
  const bool bf = mode != 0;
  const TcShape S = tc_shape(n, true, bf, mode == 2);
  auto a1 = [&](int r, int k) { return m[(size_t)(2 * (r % hn) + r / hn) * n + k]; };
  auto a2 = [&](int r, int k) { return m[(size_t)(r % hn) * n + 2 * k + r / hn]; };
  if (mode == 2) {
    if (kind == 1)
      tc_images_oz(S, a1, out);
    else
      tc_images_oz(S, a2, out);
  } else if (kind == 1) {
    tc_images(S, bf, a1, out);
  } else {
    tc_images(S, bf, a2, out);
  }
}

int angular_tc_trace_slots() { return kTraceSlots; }

// Self-test of the bounded waits: one CTA waits on an mbarrier that nothing arrives at, with
// both wait forms of the tensor-core kernel (suspend-hinted try_wait and plain polling), and
// reports whether each gave up: out[0], out[1] = 1 when the wait timed out as intended,
// out[2] = elapsed ns.  The barrier is completed afterwards, so nothing is left waiting.
__global__ void bounded_wait_selftest_kernel(uint64_t limit_ns, unsigned long long* out) {
  using namespace tc;
  __shared__ __align__(8) uint64_t bar;
  if (threadIdx.x == 0) {
    mbar_init(&bar, 1);
    fence_mbar_init();
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    const uint64_t t0 = globaltimer_ns();
    const bool a = mbar_wait(&bar, 0u, limit_ns);
    const bool b = mbar_poll(&bar, 0u, limit_ns);
    out[0] = a ? 0ull : 1ull;
    out[1] = b ? 0ull : 1ull;
    out[2] = globaltimer_ns() - t0;
    mbar_arrive(&bar);
  }
  __syncthreads();
}

cudaError_t bounded_wait_selftest(uint64_t limit_ns, unsigned long long* host_out) {
  unsigned long long* d = nullptr;
  cudaError_t e = cudaMalloc(&d, 3 * sizeof(unsigned long long));
  if (e != cudaSuccess) return e;
  bounded_wait_selftest_kernel<<<1, 32>>>(limit_ns, d);
  count_launch();
  e = cudaGetLastError();
  if (e == cudaSuccess) e = cudaMemcpy(host_out, d, 3 * sizeof(unsigned long long), cudaMemcpyDeviceToHost);
  cudaFree(d);
  return e;
}

cudaError_t launch_angular_tc(const PassParams& p, const int* mat_op, int nmat, const float* const* images,
                              int error_slot, const int* parity, int mode, cudaStream_t s,
                              unsigned long long* trace, int ctas_per_sm, int pack, const int* slice_axis,
                              const int64_t* slice_stride) {
  TcParams tp;
  make_tc_params(p, mat_op, nmat, images, error_slot, parity, &tp, pack, slice_axis, slice_stride);
  tp.trace = trace;
  const int v = tc_variant(mode, pack);
  if (v < 0) return cudaErrorInvalidValue;
  const size_t smem = angular_tc_smem_bytes((int)p.g.n * pack, tp.parity[0] != 0, mode);
  static bool configured[5] = {false, false, false, false, false};
  const void* kerns[5] = {(const void*)angular_tc_kernel<0>, (const void*)angular_tc_kernel<1>,
                          (const void*)angular_tc_kernel<2>, (const void*)angular_tc_kernel<2, 2>,
                          (const void*)angular_tc_kernel<2, 4>};
  if (!configure_once(kerns[v], configured[v])) return cudaGetLastError();
  if (smem > tc_max_dynamic_smem()) return cudaErrorInvalidValue;
  const unsigned grid = persistent_grid(p.g.tiles, ctas_per_sm);
  switch (v) {
    case 4: angular_tc_kernel<2, 4><<<grid, kThreads, smem, s>>>(tp); break;
    case 3: angular_tc_kernel<2, 2><<<grid, kThreads, smem, s>>>(tp); break;
    case 2: angular_tc_kernel<2><<<grid, kThreads, smem, s>>>(tp); break;
    case 1: angular_tc_kernel<1><<<grid, kThreads, smem, s>>>(tp); break;
    default: angular_tc_kernel<0><<<grid, kThreads, smem, s>>>(tp); break;
  }
  count_launch();
  return cudaGetLastError();
}

}  // namespace so
