// Multilayer perceptron for learned starting states of imaginary-time relaxation
// (no counterpart in the reference crate).  Hand-written CUDA kernels:
//   forward   Z = X W^T + b, tanh on hidden layers (BF16 weights, FP32 accumulate)
//   backward  dW = dZ^T X, db = column sums of dZ, dX = dZ W
//   Adam      on FP32 master weights, then a BF16 copy for the next forward pass
// The three products run on the tensor cores (tcgen05.mma kind::f16, accumulators in
// TMEM) with FP32 activations and gradients split into two BF16 parts.  Every product and
// sum runs in a fixed order, so training is deterministic.
#include <cmath>
#include <cstring>
#include <memory>
#include <random>
#include <stdexcept>
#include <vector>

#include <cuda_bf16.h>

#include "../../include/split_operator.h"
#include "common.cuh"
#include "tc_common.cuh"

namespace so {

void set_last_error(const char* msg);

namespace {

template <typename T>
__device__ __forceinline__ float to_f(T v);
template <>
__device__ __forceinline__ float to_f<float>(float v) {
  return v;
}
template <>
__device__ __forceinline__ float to_f<__nv_bfloat16>(__nv_bfloat16 v) {
  return __bfloat162float(v);
}

// ---- tensor-core GEMM (tcgen05.mma kind::f16, BF16 operands, FP32 accumulation in TMEM)
// C[m][n] = sum_k A(m, k) B(n, k) over a 128 x 128 tile per CTA, K in chunks of 16.  The
// 128 threads stage each chunk into shared memory in the K-major core-matrix layout (8 rows
// x 16 bytes per core matrix, K core matrices 128 B apart, row groups 256 B apart), which
// also does the transposes the backward products need (A and B are read through strides).
// FP32 operands are split x = bf16(x) + bf16(x - bf16(x)) (16 significant bits together);
// the BF16 weights are exact as they are.  Products: hi hi + lo hi (B exact) or
// hi hi + hi lo + lo hi (both split); the remaining lo lo term is 2^-16 of the result.
// Two shared-memory stages: thread 0 issues a chunk's MMAs and commits them to the stage's
// mbarrier, which the threads wait on (bounded) before they overwrite that stage.
constexpr int kGm = 128, kGn = 128, kGk = 16;
constexpr uint32_t kGStage = 4u * kGm * kGk * 2u;  // A hi, A lo, B hi, B lo: 4 KB each
constexpr uint64_t kGWait = 2000000000ull;         // 2 s

struct GemmOperand {
  const void* p;
  int64_t s_row, s_k;  // element strides: A(m, k) = p[m s_row + k s_k] (B(n, k) likewise)
  int bf16;            // 1: BF16 values (used as they are); 0: FP32 (split into hi + lo)
};

// byte offset of element (row r, k) in a 128 x 16 chunk image
__device__ __forceinline__ uint32_t gemm_off(int r, int k) {
  return (uint32_t)(r >> 3) * 256u + (uint32_t)(k >> 3) * 128u + (uint32_t)(r & 7) * 16u + (uint32_t)(k & 7) * 2u;
}

// row r of a chunk (16 K values) of one operand into its hi / lo images
__device__ __forceinline__ void gemm_stage_row(const GemmOperand& o, int64_t row, int64_t rows, int64_t k0, int K,
                                               int r, unsigned char* hi, unsigned char* lo) {
  uint32_t h[8], l[8];
#pragma unroll
  for (int k = 0; k < kGk; ++k) {
    float x = 0.0f;
    if (row < rows && k0 + k < K) {
      const int64_t e = row * o.s_row + (k0 + k) * o.s_k;
      x = o.bf16 ? __bfloat162float(reinterpret_cast<const __nv_bfloat16*>(o.p)[e])
                 : reinterpret_cast<const float*>(o.p)[e];
    }
    uint16_t xh, xl;
    tc::split_bf16(x, xh, xl);  // exact for a BF16 value: xl = 0
    if (k & 1) {
      h[k >> 1] |= (uint32_t)xh << 16;
      l[k >> 1] |= (uint32_t)xl << 16;
    } else {
      h[k >> 1] = xh;
      l[k >> 1] = xl;
    }
  }
  // two 16-byte core-matrix rows (K 0-7 and 8-15) per image
  *reinterpret_cast<uint4*>(hi + gemm_off(r, 0)) = make_uint4(h[0], h[1], h[2], h[3]);
  *reinterpret_cast<uint4*>(hi + gemm_off(r, 8)) = make_uint4(h[4], h[5], h[6], h[7]);
  *reinterpret_cast<uint4*>(lo + gemm_off(r, 0)) = make_uint4(l[0], l[1], l[2], l[3]);
  *reinterpret_cast<uint4*>(lo + gemm_off(r, 8)) = make_uint4(l[4], l[5], l[6], l[7]);
}

__global__ void __launch_bounds__(128) tc_gemm_kernel(int M, int N, int K, GemmOperand A, GemmOperand B,
                                                      float* __restrict__ C, int64_t ldc, int* err) {
  using namespace tc;
  __shared__ __align__(1024) unsigned char sm[2 * kGStage];
  __shared__ __align__(8) uint64_t done[3];  // per stage: its MMAs completed; [2]: all MMAs
  __shared__ uint32_t tmem_s;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int64_t m0 = (int64_t)blockIdx.y * kGm, n0 = (int64_t)blockIdx.x * kGn;
  if (tid == 0) {
    for (int i = 0; i < 3; ++i) mbar_init(&done[i], 1);
    fence_mbar_init();
  }
  if (warp == 0) tmem_alloc(&tmem_s, kGn);
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = tmem_s;
  const uint32_t idesc = idesc_bf16(kGm, kGn);
  const bool bsplit = !B.bf16, asplit = !A.bf16;
  const int nk = (K + kGk - 1) / kGk;
  bool ok = true;
  for (int c = 0; c < nk; ++c) {
    const int s = c & 1;
    unsigned char* st = sm + (uint32_t)s * kGStage;
    // the MMAs that read this stage two chunks ago have completed
    if (c >= 2) ok = ok && mbar_wait(&done[s], (uint32_t)((c / 2 - 1) & 1), kGWait);
    gemm_stage_row(A, m0 + tid, M, (int64_t)c * kGk, K, tid, st, st + 4096);
    gemm_stage_row(B, n0 + tid, N, (int64_t)c * kGk, K, tid, st + 8192, st + 12288);
    fence_proxy_async();
    __syncthreads();
    if (tid == 0) {
      tc_fence_after();
      const uint32_t a = smem_u32(st);
      const uint64_t ah = smem_desc_at(smem_desc_bits(128, 256), a), al = smem_desc_at(smem_desc_bits(128, 256), a + 4096);
      const uint64_t bh = smem_desc_at(smem_desc_bits(128, 256), a + 8192),
                     bl = smem_desc_at(smem_desc_bits(128, 256), a + 12288);
      mma_bf16(tmem, ah, bh, idesc, c > 0 ? 1u : 0u);
      if (asplit) mma_bf16(tmem, al, bh, idesc, 1u);
      if (bsplit) mma_bf16(tmem, ah, bl, idesc, 1u);
      mma_commit(&done[s]);
    }
  }
  if (tid == 0) mma_commit(&done[2]);
  ok = mbar_wait(&done[2], 0u, kGWait) && ok;
  tc_fence_after();
  if (!__syncthreads_and(ok)) {
    if (tid == 0) atomicExch(err, 1);
  } else {
    // TMEM lane = row m0 + 32 warp + lane, 32 columns per load
    const int64_t m = m0 + 32 * warp + lane;
    for (int cb = 0; cb < kGn; cb += 32) {
      float v[32];
      tmem_ld32(tmem + ((uint32_t)(32 * warp) << 16) + (uint32_t)cb, v);
      if (m < M)
#pragma unroll
        for (int j = 0; j < 32; ++j)
          if (n0 + cb + j < N) C[m * ldc + n0 + cb + j] = v[j];
    }
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 0) tmem_dealloc(tmem, kGn);
}

// C (M x N, row stride ldc) = A B^T through the tensor-core kernel
void tc_gemm(int M, int N, int K, GemmOperand A, GemmOperand B, float* C, int64_t ldc, int* err, cudaStream_t s) {
  dim3 grid((N + kGn - 1) / kGn, (M + kGm - 1) / kGm);
  tc_gemm_kernel<<<grid, 128, 0, s>>>(M, N, K, A, B, C, ldc, err);
  count_launch();
}

__global__ void bias_act_kernel(float* Z, const float* b, int rows, int cols, int act) {
  const int64_t n = (int64_t)rows * cols;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    float v = Z[i] + b[i % cols];
    Z[i] = act ? tanhf(v) : v;
  }
}

// dY = 2 (Y - T) / (rows * cols); loss partials per block (fixed order)
__global__ void mse_grad_kernel(const float* Y, const float* T, float* dY, int rows, int cols, double* partial) {
  __shared__ double sh[256];
  const int64_t n = (int64_t)rows * cols;
  const float sc = 2.0f / (float)n;
  double acc = 0.0;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const float d = Y[i] - T[i];
    dY[i] = sc * d;
    acc += (double)d * d;
  }
  sh[threadIdx.x] = acc;
  __syncthreads();
  for (int s = 128; s > 0; s >>= 1) {
    if ((int)threadIdx.x < s) sh[threadIdx.x] += sh[threadIdx.x + s];
    __syncthreads();
  }
  if (threadIdx.x == 0) partial[blockIdx.x] = sh[0];
}

// dZ = dY * (1 - y^2) for tanh layers (in place)
__global__ void tanh_back_kernel(float* dY, const float* Y, int64_t n) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    dY[i] *= 1.0f - Y[i] * Y[i];
}

// db[c] = sum_r dZ[r][c] (one thread per column, fixed order)
__global__ void colsum_kernel(const float* dZ, float* db, int rows, int cols) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= cols) return;
  float s = 0.f;
  for (int r = 0; r < rows; ++r) s += dZ[(size_t)r * cols + c];
  db[c] = s;
}

__global__ void adam_kernel(float* w, const float* g, float* m, float* v, int64_t n, float lr, float b1, float b2,
                            float eps, float c1, float c2) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const float gi = g[i];
    const float mi = b1 * m[i] + (1.f - b1) * gi;
    const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    w[i] -= lr * (mi / c1) / (sqrtf(vi / c2) + eps);
  }
}

__global__ void to_bf16_kernel(const float* src, __nv_bfloat16* dst, int64_t n) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    dst[i] = __float2bfloat16_rn(src[i]);
}

unsigned grid_for(int64_t n) {
  int64_t b = (n + 255) / 256;
  if (b > 4096) b = 4096;
  return (unsigned)(b < 1 ? 1 : b);
}

void check(cudaError_t e, const char* w) {
  if (e != cudaSuccess) throw std::runtime_error(std::string(w) + ": " + cudaGetErrorString(e));
}

template <typename T>
struct DBuf {
  T* p = nullptr;
  size_t n = 0;
  void alloc(size_t count) {
    if (p) cudaFree(p);
    n = count;
    check(cudaMalloc(&p, std::max<size_t>(1, count) * sizeof(T)), "cudaMalloc");
    check(cudaMemset(p, 0, std::max<size_t>(1, count) * sizeof(T)), "cudaMemset");
  }
  ~DBuf() {
    if (p) cudaFree(p);
  }
};

}  // namespace

struct Mlp {
  std::vector<int> w;  // widths: input, hidden..., output
  struct Layer {
    int in, out;
    DBuf<float> W, b, gW, gb, mW, vW, mb, vb;
    DBuf<__nv_bfloat16> W16;
  };
  std::vector<std::unique_ptr<Layer>> layers;
  std::vector<DBuf<float>> act, grad;  // per layer output (activations) and its gradient
  DBuf<float> x, target;
  DBuf<double> partial;
  DBuf<int> err;  // set by a tensor-core product whose bounded wait gave up
  int cap = 0;
  int64_t t = 0;  // Adam step
  cudaStream_t s = nullptr;

  void ensure(int batch) {
    if (batch <= cap) return;
    cap = batch;
    x.alloc((size_t)batch * w[0]);
    target.alloc((size_t)batch * w.back());
    act.resize(layers.size());
    grad.resize(layers.size());
    for (size_t l = 0; l < layers.size(); ++l) {
      act[l].alloc((size_t)batch * layers[l]->out);
      grad[l].alloc((size_t)batch * layers[l]->out);
    }
    partial.alloc(4096);
    if (!err.p) err.alloc(1);
  }

  // a bounded wait inside a tensor-core product gave up: report it (and clear the flag)
  void check_err() {
    int e = 0;
    check(cudaMemcpyAsync(&e, err.p, sizeof(int), cudaMemcpyDeviceToHost, s), "copy");
    check(cudaStreamSynchronize(s), "sync");
    if (e) {
      check(cudaMemsetAsync(err.p, 0, sizeof(int), s), "memset");
      throw std::runtime_error("a tensor-core product's bounded wait gave up");
    }
  }

  void refresh_bf16() {
    for (auto& L : layers) {
      const int64_t n = (int64_t)L->in * L->out;
      to_bf16_kernel<<<grid_for(n), 256, 0, s>>>(L->W.p, L->W16.p, n);
      count_launch();
    }
  }

  void forward(int batch) {
    const float* in = x.p;
    for (size_t l = 0; l < layers.size(); ++l) {
      Layer& L = *layers[l];
      // Z[b][o] = sum_i X[b][i] W[o][i]
      tc_gemm(batch, L.out, L.in, GemmOperand{in, L.in, 1, 0}, GemmOperand{L.W16.p, L.in, 1, 1}, act[l].p, L.out,
              err.p, s);
      const int hidden = l + 1 < layers.size();
      bias_act_kernel<<<grid_for((int64_t)batch * L.out), 256, 0, s>>>(act[l].p, L.b.p, batch, L.out, hidden);
      count_launch();
      in = act[l].p;
    }
  }

  double backward(int batch) {
    const int nl = (int)layers.size();
    const int64_t nout = (int64_t)batch * w.back();
    const unsigned gb = std::min<unsigned>(grid_for(nout), 4096);
    mse_grad_kernel<<<gb, 256, 0, s>>>(act[nl - 1].p, target.p, grad[nl - 1].p, batch, w.back(), partial.p);
    count_launch();
    for (int l = nl - 1; l >= 0; --l) {
      Layer& L = *layers[l];
      if (l < nl - 1) {
        tanh_back_kernel<<<grid_for((int64_t)batch * L.out), 256, 0, s>>>(grad[l].p, act[l].p,
                                                                          (int64_t)batch * L.out);
        count_launch();
      }
      const float* in = l == 0 ? x.p : act[l - 1].p;
      // dW[o][i] = sum_b dZ[b][o] X[b][i]
      tc_gemm(L.out, L.in, batch, GemmOperand{grad[l].p, 1, L.out, 0}, GemmOperand{in, 1, L.in, 0}, L.gW.p, L.in,
              err.p, s);
      colsum_kernel<<<(L.out + 127) / 128, 128, 0, s>>>(grad[l].p, L.gb.p, batch, L.out);
      count_launch();
      if (l > 0) {
        // dX[b][i] = sum_o dZ[b][o] W[o][i]
        tc_gemm(batch, L.in, L.out, GemmOperand{grad[l].p, L.out, 1, 0}, GemmOperand{L.W16.p, 1, L.in, 1},
                grad[l - 1].p, L.in, err.p, s);
      }
    }
    std::vector<double> h(gb);
    check(cudaMemcpyAsync(h.data(), partial.p, gb * sizeof(double), cudaMemcpyDeviceToHost, s), "copy");
    check(cudaStreamSynchronize(s), "sync");
    check_err();
    double loss = 0.0;
    for (double v : h) loss += v;
    return loss / (double)nout;
  }

  void adam(float lr) {
    ++t;
    const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
    const float c1 = 1.f - std::pow(b1, (float)t), c2 = 1.f - std::pow(b2, (float)t);
    for (auto& L : layers) {
      const int64_t nw = (int64_t)L->in * L->out;
      adam_kernel<<<grid_for(nw), 256, 0, s>>>(L->W.p, L->gW.p, L->mW.p, L->vW.p, nw, lr, b1, b2, eps, c1, c2);
      adam_kernel<<<grid_for(L->out), 256, 0, s>>>(L->b.p, L->gb.p, L->mb.p, L->vb.p, L->out, lr, b1, b2, eps, c1,
                                                   c2);
      count_launch(2);
    }
    refresh_bf16();
  }
};

}  // namespace so

struct so_mlp_t {
  so::Mlp m;
};

namespace {
template <class F>
int mlp_guard(F&& f) {
  try {
    f();
    return SO_OK;
  } catch (const std::exception& e) {
    so::set_last_error(e.what());
    return SO_ERR_CUDA;
  }
}
size_t nparams(const so::Mlp& m) {
  size_t n = 0;
  for (auto& L : m.layers) n += (size_t)L->in * L->out + L->out;
  return n;
}
}  // namespace

extern "C" {

int so_mlp_new(const int* widths, size_t count, uint64_t seed, so_mlp* out) {
  if (!widths || count < 2 || !out) {
    so::set_last_error("so_mlp_new: need at least an input and an output width");
    return SO_ERR_INVALID;
  }
  return mlp_guard([&] {
    auto h = std::make_unique<so_mlp_t>();
    so::Mlp& m = h->m;
    m.w.assign(widths, widths + count);
    std::mt19937_64 rng(seed);
    for (size_t l = 0; l + 1 < count; ++l) {
      auto L = std::make_unique<so::Mlp::Layer>();
      L->in = widths[l];
      L->out = widths[l + 1];
      const size_t nw = (size_t)L->in * L->out;
      for (auto* b : {&L->W, &L->gW, &L->mW, &L->vW}) b->alloc(nw);
      for (auto* b : {&L->b, &L->gb, &L->mb, &L->vb}) b->alloc(L->out);
      L->W16.alloc(nw);
      // Glorot-uniform weights, zero biases
      std::uniform_real_distribution<float> u(-1.f, 1.f);
      const float lim = std::sqrt(6.f / (float)(L->in + L->out));
      std::vector<float> w(nw);
      for (float& v : w) v = lim * u(rng);
      so::check(cudaMemcpy(L->W.p, w.data(), nw * sizeof(float), cudaMemcpyHostToDevice), "copy");
      m.layers.push_back(std::move(L));
    }
    m.refresh_bf16();
    so::check(cudaDeviceSynchronize(), "sync");
    *out = h.release();
  });
}

int so_mlp_num_params(so_mlp m, size_t* out) {
  if (!m || !out) return SO_ERR_INVALID;
  *out = nparams(m->m);
  return SO_OK;
}

// FP32 master parameters, layer by layer: W (out x in, row-major) then b
int so_mlp_get_params(so_mlp h, float* out) {
  return mlp_guard([&] {
    size_t off = 0;
    for (auto& L : h->m.layers) {
      const size_t nw = (size_t)L->in * L->out;
      so::check(cudaMemcpy(out + off, L->W.p, nw * 4, cudaMemcpyDeviceToHost), "copy");
      off += nw;
      so::check(cudaMemcpy(out + off, L->b.p, L->out * 4, cudaMemcpyDeviceToHost), "copy");
      off += L->out;
    }
  });
}

int so_mlp_set_params(so_mlp h, const float* in) {
  return mlp_guard([&] {
    size_t off = 0;
    for (auto& L : h->m.layers) {
      const size_t nw = (size_t)L->in * L->out;
      so::check(cudaMemcpy(L->W.p, in + off, nw * 4, cudaMemcpyHostToDevice), "copy");
      off += nw;
      so::check(cudaMemcpy(L->b.p, in + off, L->out * 4, cudaMemcpyHostToDevice), "copy");
      off += L->out;
    }
    h->m.refresh_bf16();
    so::check(cudaDeviceSynchronize(), "sync");
  });
}

// y = network(x) for `batch` rows (host arrays, FP32)
int so_mlp_forward(so_mlp h, const float* x, size_t batch, float* y) {
  return mlp_guard([&] {
    so::Mlp& m = h->m;
    m.ensure((int)batch);
    so::check(cudaMemcpy(m.x.p, x, batch * m.w[0] * 4, cudaMemcpyHostToDevice), "copy");
    m.forward((int)batch);
    m.check_err();
    so::check(cudaMemcpy(y, m.act.back().p, batch * m.w.back() * 4, cudaMemcpyDeviceToHost), "copy");
  });
}

// Loss (mean squared error) and parameter gradients (same order as so_mlp_get_params)
int so_mlp_gradients(so_mlp h, const float* x, const float* target, size_t batch, double* loss, float* grads) {
  return mlp_guard([&] {
    so::Mlp& m = h->m;
    m.ensure((int)batch);
    so::check(cudaMemcpy(m.x.p, x, batch * m.w[0] * 4, cudaMemcpyHostToDevice), "copy");
    so::check(cudaMemcpy(m.target.p, target, batch * m.w.back() * 4, cudaMemcpyHostToDevice), "copy");
    m.forward((int)batch);
    *loss = m.backward((int)batch);
    size_t off = 0;
    for (auto& L : m.layers) {
      const size_t nw = (size_t)L->in * L->out;
      so::check(cudaMemcpy(grads + off, L->gW.p, nw * 4, cudaMemcpyDeviceToHost), "copy");
      off += nw;
      so::check(cudaMemcpy(grads + off, L->gb.p, L->out * 4, cudaMemcpyDeviceToHost), "copy");
      off += L->out;
    }
  });
}

// `steps` full-batch Adam steps on (x, target); losses[i] = loss before step i
int so_mlp_train(so_mlp h, const float* x, const float* target, size_t batch, size_t steps, float lr,
                 double* losses) {
  return mlp_guard([&] {
    so::Mlp& m = h->m;
    m.ensure((int)batch);
    so::check(cudaMemcpy(m.x.p, x, batch * m.w[0] * 4, cudaMemcpyHostToDevice), "copy");
    so::check(cudaMemcpy(m.target.p, target, batch * m.w.back() * 4, cudaMemcpyHostToDevice), "copy");
    for (size_t i = 0; i < steps; ++i) {
      m.forward((int)batch);
      const double l = m.backward((int)batch);
      if (losses) losses[i] = l;
      m.adam(lr);
    }
    so::check(cudaDeviceSynchronize(), "sync");
  });
}

void so_mlp_free(so_mlp h) { delete h; }

}  // extern "C"
