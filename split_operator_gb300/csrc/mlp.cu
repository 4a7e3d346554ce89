// Multilayer perceptron for learned starting states of imaginary-time relaxation
// (no counterpart in the reference crate).  Hand-written CUDA kernels:
//   forward   Z = X W^T + b, tanh on hidden layers (BF16 weights, FP32 accumulate)
//   backward  dW = dZ^T X, db = column sums of dZ, dX = dZ W  (FP32)
//   Adam      on FP32 master weights, then a BF16 copy for the next forward pass
// Every output element is summed by one thread in a fixed order, so training is
// deterministic for a given launch configuration.
#include <cmath>
#include <cstring>
#include <memory>
#include <random>
#include <stdexcept>
#include <vector>

#include <cuda_bf16.h>

#include "../../include/split_operator.h"
#include "common.cuh"

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

// C[m][n] (+)= sum_k A(m, k) B(k, n); A(m,k) = TA ? A[k*lda+m] : A[m*lda+k], B(k,n) = TB ? B[n*ldb+k] : B[k*ldb+n]
constexpr int kTile = 64, kTk = 16;
template <typename TAt, typename TBt, bool TA, bool TB>
__global__ void __launch_bounds__(256) gemm_kernel(int M, int N, int K, const TAt* __restrict__ A, int lda,
                                                  const TBt* __restrict__ B, int ldb, float* __restrict__ C, int ldc,
                                                  int accumulate) {
  __shared__ float As[kTk][kTile + 1];
  __shared__ float Bs[kTk][kTile + 1];
  const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
  const int m0 = blockIdx.y * kTile, n0 = blockIdx.x * kTile;
  float acc[4][4] = {};
  for (int k0 = 0; k0 < K; k0 += kTk) {
    for (int e = threadIdx.x; e < kTk * kTile; e += 256) {
      const int kk = e / kTile, mm = e % kTile;
      const int m = m0 + mm, k = k0 + kk;
      float a = 0.f;
      if (m < M && k < K) a = to_f(TA ? A[(size_t)k * lda + m] : A[(size_t)m * lda + k]);
      As[kk][mm] = a;
      const int n = n0 + mm;
      float b = 0.f;
      if (n < N && k < K) b = to_f(TB ? B[(size_t)n * ldb + k] : B[(size_t)k * ldb + n]);
      Bs[kk][mm] = b;
    }
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < kTk; ++kk) {
      float a[4], b[4];
#pragma unroll
      for (int i = 0; i < 4; ++i) {
        a[i] = As[kk][ty * 4 + i];
        b[i] = Bs[kk][tx * 4 + i];
      }
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) acc[i][j] = fmaf(a[i], b[j], acc[i][j]);
    }
    __syncthreads();
  }
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const int m = m0 + ty * 4 + i, n = n0 + tx * 4 + j;
      if (m < M && n < N) {
        float* c = C + (size_t)m * ldc + n;
        *c = accumulate ? *c + acc[i][j] : acc[i][j];
      }
    }
}

template <typename TAt, typename TBt, bool TA, bool TB>
void gemm(int M, int N, int K, const TAt* A, int lda, const TBt* B, int ldb, float* C, int ldc, cudaStream_t s) {
  dim3 grid((N + kTile - 1) / kTile, (M + kTile - 1) / kTile);
  gemm_kernel<TAt, TBt, TA, TB><<<grid, 256, 0, s>>>(M, N, K, A, lda, B, ldb, C, ldc, 0);
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
      gemm<float, __nv_bfloat16, false, true>(batch, L.out, L.in, in, L.in, L.W16.p, L.in, act[l].p, L.out, s);
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
      gemm<float, float, true, false>(L.out, L.in, batch, grad[l].p, L.out, in, L.in, L.gW.p, L.in, s);
      colsum_kernel<<<(L.out + 127) / 128, 128, 0, s>>>(grad[l].p, L.gb.p, batch, L.out);
      count_launch();
      if (l > 0) {
        // dX[b][i] = sum_o dZ[b][o] W[o][i]
        gemm<float, __nv_bfloat16, false, false>(batch, L.in, L.out, grad[l].p, L.out, L.W16.p, L.in,
                                                 grad[l - 1].p, L.in, s);
      }
    }
    std::vector<double> h(gb);
    check(cudaMemcpyAsync(h.data(), partial.p, gb * sizeof(double), cudaMemcpyDeviceToHost, s), "copy");
    check(cudaStreamSynchronize(s), "sync");
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
