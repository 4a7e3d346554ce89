// CPU FP64 restatement of the split_operator propagation step (TEST AND
// MEASUREMENT INFRASTRUCTURE ONLY: imported by the test suite and by bench.py's
// CPU-baseline / reference leg, never by the product).
//
// It keeps the reference crate's structure and cost profile, not just its
// results: one full-array pass per operator, lanes copied to a temporary
// before each FFT (fft_transformation.rs:59-68), one dense mat-vec per lane for
// the Legendre transform (matrix_transformation.rs:64-65), single-threaded
// element-wise N-dim multiplies (n_dim_propagator.rs:32-36) and single-threaded
// norm folds (wave_function.rs:78-80), with threads (OpenMP, standing in for
// rayon) exactly where the reference runs lanes in parallel
// (fft_transformation.rs:59,78; matrix_transformation.rs:64,73;
// one_dim_propagator.rs:44).  The norm cache follows change_observer.rs:7-46:
// a norm is recomputed only after an operator touched the array.
//
// The FFT is a radix-2 Stockham transform with FP64 twiddles (the reference uses
// rustfft 6.2.0, which is not available here); both are exact DFTs up to rounding.
#include <cmath>
#include <complex>
#include <cstring>
#include <vector>

#ifdef _OPENMP
#include <omp.h>
#endif

using cd = std::complex<double>;

namespace {

struct Fft {
  int n;
  std::vector<cd> tw;  // exp(-2 pi i k / n)
  explicit Fft(int n_) : n(n_), tw(n_) {
    for (int k = 0; k < n; ++k) {
      const double a = -2.0 * M_PI * (double)k / (double)n;
      tw[k] = cd(std::cos(a), std::sin(a));
    }
  }
  // unnormalised transform, sign -1 forward / +1 inverse (rustfft convention)
  void run(cd* x, cd* work, int sign) const {
    cd* a = x;
    cd* b = work;
    int half = n / 2;
    for (int p = 1; p < n; p *= 2) {
      const int stride = n / (2 * p);
      for (int i = 0; i < half; ++i) {
        const int k = i % p;
        cd w = tw[k * stride];
        if (sign > 0) w = std::conj(w);
        const cd u = a[i], v = a[i + half] * w;
        const int o = (i - k) * 2 + k;
        b[o] = u + v;
        b[o + p] = u - v;
      }
      std::swap(a, b);
    }
    if (a != x) std::memcpy(x, a, sizeof(cd) * n);
  }
};

double norm_fold(const cd* psi, const double* w, size_t n) {
  double acc = 0.0;
  for (size_t i = 0; i < n; ++i) acc += std::norm(psi[i]) * w[i];
  return acc;
}

}  // namespace

extern "C" {

// Stack [Damp(loss), V/2 (n-dim), Legendre (matrix, axis 1), Rot/2 (n-dim), FFT (axis 0), K (axis 0)]
// on psi[nr][nth] (row-major, the reference's layout).  Complex arrays are interleaved doubles.
// cache_norm: the wave function's cached norm on entry (1.0 after normalize(1.0)).
int cpu_port_radial_angular(int nr, int nth, double* psi_io, const double* vhalf, const double* rothalf,
                            const double* kin, const double* mask, const double* t, const double* tinv,
                            const double* w_r, const double* w_th, int steps, int threads, double* loss_io,
                            double* cache_norm_io) {
#ifdef _OPENMP
  if (threads > 0) omp_set_num_threads(threads);
#endif
  const size_t n = (size_t)nr * nth;
  cd* psi = reinterpret_cast<cd*>(psi_io);
  const cd* V = reinterpret_cast<const cd*>(vhalf);
  const cd* Rt = reinterpret_cast<const cd*>(rothalf);
  const cd* K = reinterpret_cast<const cd*>(kin);
  const cd* M = reinterpret_cast<const cd*>(mask);
  const cd* T = reinterpret_cast<const cd*>(t);
  const cd* Ti = reinterpret_cast<const cd*>(tinv);
  std::vector<double> w(n);
  for (int i = 0; i < nr; ++i)
    for (int j = 0; j < nth; ++j) w[(size_t)i * nth + j] = w_r[i] * w_th[j];
  const Fft fft(nr);
  const double inv_sqrt = std::sqrt((double)nr);
  double loss = *loss_io, cache = *cache_norm_io;
  bool dirty = false;
  double cur = 0.0;

  auto norm = [&]() {
    if (dirty) {
      cache = norm_fold(psi, w.data(), n);
      dirty = false;
    }
    return cache;
  };
  auto damp = [&]() {  // border_dumping.rs:62-84 with its LossChecker
    cur = norm();
#pragma omp parallel for schedule(static)
    for (int j = 0; j < nth; ++j)
      for (int i = 0; i < nr; ++i) psi[(size_t)i * nth + j] *= M[i];
    dirty = true;
    const double after = norm();
    loss += cur - after;
    cur = after;
  };
  auto ndim = [&](const cd* op) {
    for (size_t i = 0; i < n; ++i) psi[i] *= op[i];
    dirty = true;
  };
  auto lane_mat = [&](const cd* m) {
#pragma omp parallel
    {
      std::vector<cd> tmp(nth);
#pragma omp for schedule(static)
      for (int i = 0; i < nr; ++i) {
        cd* row = psi + (size_t)i * nth;
        for (int a = 0; a < nth; ++a) {
          cd s(0.0, 0.0);
          for (int b = 0; b < nth; ++b) s += m[(size_t)a * nth + b] * row[b];
          tmp[a] = s;
        }
        std::memcpy(row, tmp.data(), sizeof(cd) * nth);
      }
    }
    dirty = true;
  };
  auto lane_fft = [&](int sign) {
#pragma omp parallel
    {
      std::vector<cd> tmp(nr), work(nr);
#pragma omp for schedule(static)
      for (int j = 0; j < nth; ++j) {
        for (int i = 0; i < nr; ++i) tmp[i] = psi[(size_t)i * nth + j];
        fft.run(tmp.data(), work.data(), sign);
        for (int i = 0; i < nr; ++i) psi[(size_t)i * nth + j] = tmp[i] / inv_sqrt;
      }
    }
    dirty = true;
  };
  auto kinetic = [&]() {
#pragma omp parallel for schedule(static)
    for (int j = 0; j < nth; ++j)
      for (int i = 0; i < nr; ++i) psi[(size_t)i * nth + j] *= K[i];
    dirty = true;
  };
  for (int s = 0; s < steps; ++s) {
    damp();
    ndim(V);
    lane_mat(T);
    ndim(Rt);
    lane_fft(-1);
    kinetic();
    lane_fft(+1);
    ndim(Rt);
    lane_mat(Ti);
    ndim(V);
    damp();
  }
  *loss_io = loss;
  *cache_norm_io = norm();
  return 0;
}

// Stack [LeakControl, V/2 (axis 0), FFT (axis 0), K (axis 0)] on a 1-D psi[n].
int cpu_port_harmonic_1d(int n, double* psi_io, const double* vhalf, const double* kin, const double* w_x,
                         int steps, double* cache_norm_io) {
  cd* psi = reinterpret_cast<cd*>(psi_io);
  const cd* V = reinterpret_cast<const cd*>(vhalf);
  const cd* K = reinterpret_cast<const cd*>(kin);
  const Fft fft(n);
  std::vector<cd> tmp(n), work(n);
  const double sq = std::sqrt((double)n);
  double cache = *cache_norm_io;
  for (int s = 0; s < steps; ++s) {
    const double leak_norm = cache;  // cached: the previous normalize recorded it
    for (int i = 0; i < n; ++i) psi[i] *= V[i];
    std::memcpy(tmp.data(), psi, sizeof(cd) * n);
    fft.run(tmp.data(), work.data(), -1);
    for (int i = 0; i < n; ++i) psi[i] = tmp[i] / sq;
    for (int i = 0; i < n; ++i) psi[i] *= K[i];
    std::memcpy(tmp.data(), psi, sizeof(cd) * n);
    fft.run(tmp.data(), work.data(), +1);
    for (int i = 0; i < n; ++i) psi[i] = tmp[i] / sq;
    for (int i = 0; i < n; ++i) psi[i] *= V[i];
    const double nn = norm_fold(psi, w_x, (size_t)n);
    const double f = std::sqrt(leak_norm / nn);
    for (int i = 0; i < n; ++i) psi[i] *= f;
    cache = leak_norm;
  }
  *cache_norm_io = cache;
  return 0;
}

}  // extern "C"
