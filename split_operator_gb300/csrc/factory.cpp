// Set-up-time tables, built once in FP64 on the host (as the reference does):
// grids, momentum grids, Hamiltonians, Legendre matrices, potentials, FFT
// twiddles and Gauss-Legendre quadrature.
#include <cmath>
#include <stdexcept>

#include "model.hpp"

namespace so {

static const double kPi = 3.14159265358979323846;

static uint64_t g_grid_uid = 1;
uint64_t Grid::next_uid() { return g_grid_uid++; }

// grid.rs:24-48
Grid Grid::linear_continuos(const std::string& name, double start, double end, size_t n, size_t dim) {
  if (n < 2) throw Error(SO_ERR_INVALID, "grid needs at least 2 nodes");
  Grid g;
  g.name = name;
  g.dimension_no = dim;
  const double step = (end - start) / ((double)n - 1.0);
  g.nodes.resize(n);
  for (size_t i = 0; i < n; ++i) g.nodes[i] = start + step * (double)i;
  g.weights.assign(n, 1.0 * step);
  g.weights[0] = 0.5 * step;
  g.weights[n - 1] = 0.5 * step;
  g.uid = next_uid();
  return g;
}

// grid.rs:51-73
Grid Grid::linear_countable(const std::string& name, double start, double end, size_t n, size_t dim) {
  if (n < 2) throw Error(SO_ERR_INVALID, "grid needs at least 2 nodes");
  Grid g;
  g.name = name;
  g.dimension_no = dim;
  const double step = (end - start) / ((double)n - 1.0);
  g.nodes.resize(n);
  for (size_t i = 0; i < n; ++i) g.nodes[i] = start + step * (double)i;
  g.weights.assign(n, 1.0 * step);
  g.uid = next_uid();
  return g;
}

// grid.rs:76-84
Grid Grid::custom(const std::string& name, std::vector<double> nodes, std::vector<double> weights, size_t dim) {
  if (nodes.size() != weights.size()) throw Error(SO_ERR_SHAPE, "nodes and weights differ in length");
  Grid g;
  g.name = name;
  g.dimension_no = dim;
  g.nodes = std::move(nodes);
  g.weights = std::move(weights);
  g.uid = next_uid();
  return g;
}

// momentum step of fft_transformation.rs:28 and kinetic_operator.rs:9
static double momentum_step(const Grid& g) {
  const double n = (double)g.nodes.size();
  return 2.0 * kPi / (g.nodes.back() - g.nodes.front()) * (1.0 - 1.0 / n);
}

std::vector<double> momenta_fft_order(const Grid& g) {
  const int64_t len = (int64_t)g.nodes.size();
  const double dk = momentum_step(g);
  std::vector<double> k;
  k.reserve(len);
  for (int64_t i = 0; i < len / 2; ++i) k.push_back((double)i * dk);
  for (int64_t i = -len / 2; i < 0; ++i) k.push_back((double)i * dk);
  return k;
}

// fft_transformation.rs:28-43
Grid fft_momentum_grid(const Grid& g, const std::string& name) {
  if (g.nodes.size() < 2) throw Error(SO_ERR_INVALID, "FFT grid needs at least 2 nodes");
  std::vector<double> k = momenta_fft_order(g);
  std::vector<double> w(k.size(), momentum_step(g));
  const size_t len = g.nodes.size();
  w[len / 2 - 1] *= 0.5;
  w[len / 2] *= 0.5;
  return Grid::custom(name, k, w, g.dimension_no);
}

// kinetic_operator.rs:8-21
std::vector<double> kinetic_hamiltonian(const Grid& g, double red_mass) {
  std::vector<double> k = momenta_fft_order(g);
  for (double& v : k) v = v * v / (2.0 * red_mass);
  return k;
}

// rotational_operator.rs:7-26 (row-major (radial, polar))
std::vector<double> rotational_hamiltonian(const Grid& radial, const Grid& polar, double red_mass, double b) {
  const size_t nr = radial.nodes.size(), np = polar.nodes.size();
  std::vector<double> h(nr * np);
  for (size_t i = 0; i < nr; ++i) {
    const double r = radial.nodes[i];
    for (size_t j = 0; j < np; ++j) {
      const int64_t l = (int64_t)j;
      h[i * np + j] = (double)(l * (l + 1)) * (b + 1.0 / (2.0 * red_mass * r * r));
    }
  }
  return h;
}

// special_functions.rs:3-14
std::vector<double> legendre_polynomials(size_t j, double x) {
  if (j < 1) throw Error(SO_ERR_INVALID, "legendre_polynomials needs j >= 1");
  std::vector<double> p(j + 1, 0.0);
  p[0] = 1.0;
  p[1] = x;
  for (size_t i = 2; i <= j; ++i)
    p[i] = ((double)(2 * i - 1) / (double)i) * x * p[i - 1] - ((double)(i - 1) / (double)i) * p[i - 2];
  return p;
}

// special_functions.rs:43-55
static double double_factorial(size_t n) {
  if (n >= 100) throw Error(SO_ERR_INVALID, "double_factorial argument too large");
  if (n == 0) return 1.0;
  double value = (double)n;
  for (int64_t k = (int64_t)n - 2; k >= 2; k -= 2) value *= (double)k;
  return value;
}

// special_functions.rs:57-83
static double negate_m(int64_t l, int64_t m) {
  if (m >= 50) throw Error(SO_ERR_INVALID, "m too large");
  if (m > 0) {
    double v = std::pow(-1.0, (double)m);
    for (int64_t k = l - m; k < l + m; ++k) v /= (double)k + 1.0;
    return v;
  }
  if (m < 0) {
    double v = std::pow(-1.0, (double)m);
    for (int64_t k = l + m; k < l - m; ++k) v *= (double)k + 1.0;
    return v;
  }
  return 1.0;
}

// special_functions.rs:85-116
static double normalization(int64_t l, int64_t m) {
  if (m >= 50) throw Error(SO_ERR_INVALID, "m too large");
  double v = 1.0;
  if (m > 0)
    for (int64_t k = l - m; k < l + m; ++k) v /= (double)k + 1.0;
  else if (m < 0)
    for (int64_t k = l + m; k < l - m; ++k) v *= (double)k + 1.0;
  return std::sqrt(v * ((double)l + 0.5));
}

// special_functions.rs:17-41
std::vector<double> associated_legendre_polynomials(size_t j, int64_t m, double x) {
  const size_t mu = (size_t)(m < 0 ? -m : m);
  if (m == 0) return legendre_polynomials(j, x);
  if (mu + 1 > j) throw Error(SO_ERR_INVALID, "associated_legendre_polynomials needs j > |m|");
  std::vector<double> p(j + 1, 0.0);
  p[mu] = std::pow(-1.0, (double)m) * double_factorial(2 * mu - 1) * std::pow(1.0 - x * x, (double)mu / 2.0);
  if (m < 0) {
    p[mu] *= negate_m((int64_t)mu, (int64_t)mu);
    p[mu + 1] = x * p[mu];
  } else {
    p[mu + 1] = x * (2.0 * (double)mu + 1.0) * p[mu];
  }
  for (size_t i = mu + 2; i <= j; ++i) {
    const double l = (double)(i - 1);
    p[i] = ((2.0 * l + 1.0) * x * p[i - 1] - (l + (double)m) * p[i - 2]) / (l - (double)m + 1.0);
  }
  return p;
}

// legendre_diagonalization.rs:13-45 / :48-80 (omega = 0 is the plain Legendre case)
void legendre_matrices(const Grid& polar, int64_t omega, std::vector<cplx>& t, std::vector<cplx>& tinv) {
  const size_t n = polar.nodes.size();
  const size_t lmax = n - 1;
  std::vector<double> m(n * n, 0.0);
  for (size_t j = 0; j < n; ++j) {
    const double x = std::cos(polar.nodes[j]);
    if (omega == 0) {
      std::vector<double> pl = legendre_polynomials(lmax, x);
      for (size_t i = 0; i < n; ++i) m[i * n + j] = std::sqrt((double)i + 0.5) * pl[i];
    } else {
      std::vector<double> pl = associated_legendre_polynomials(lmax, omega, x);
      const size_t mu = (size_t)(omega < 0 ? -omega : omega);
      for (size_t i = mu; i < n; ++i) m[i * n + j] = normalization((int64_t)i, omega) * pl[i];
    }
  }
  t.assign(n * n, cplx(0, 0));
  tinv.assign(n * n, cplx(0, 0));
  for (size_t i = 0; i < n; ++i)
    for (size_t j = 0; j < n; ++j) {
      tinv[j * n + i] = cplx(m[i * n + j], 0.0);
      t[i * n + j] = cplx(m[i * n + j] * polar.weights[j], 0.0);
    }
}

// Gauss-Legendre quadrature by Newton iteration on P_n (nodes ascending).
void gauss_legendre(size_t n, std::vector<double>& x, std::vector<double>& w) {
  if (n < 1) throw Error(SO_ERR_INVALID, "gauss_legendre needs n >= 1");
  x.assign(n, 0.0);
  w.assign(n, 0.0);
  for (size_t i = 0; i < (n + 1) / 2; ++i) {
    double z = std::cos(kPi * ((double)i + 0.75) / ((double)n + 0.5));
    double dp = 1.0;
    for (int it = 0; it < 100; ++it) {
      double p0 = 1.0, p1 = z;
      for (size_t k = 2; k <= n; ++k) {
        const double p2 = ((2.0 * (double)k - 1.0) * z * p1 - ((double)k - 1.0) * p0) / (double)k;
        p0 = p1;
        p1 = p2;
      }
      if (n == 1) {
        p1 = z;
        p0 = 1.0;
      }
      dp = (double)n * (z * p1 - p0) / (z * z - 1.0);
      const double dz = p1 / dp;
      z -= dz;
      if (std::fabs(dz) < 1e-16) {
        // one more evaluation of the derivative at the converged node
        p0 = 1.0;
        p1 = z;
        for (size_t k = 2; k <= n; ++k) {
          const double p2 = ((2.0 * (double)k - 1.0) * z * p1 - ((double)k - 1.0) * p0) / (double)k;
          p0 = p1;
          p1 = p2;
        }
        dp = (double)n * (z * p1 - p0) / (z * z - 1.0);
        break;
      }
    }
    if (n == 1) {
      z = 0.0;
      dp = 1.0;
    }
    const double wi = 2.0 / ((1.0 - z * z) * dp * dp);
    x[i] = -z;
    x[n - 1 - i] = z;
    w[i] = wi;
    w[n - 1 - i] = wi;
  }
  if (n % 2 == 1) x[n / 2] = 0.0;
}

// FFT twiddles exp(-2 pi i j / n) with octant symmetry so quarter and eighth turns are exact.
std::vector<cplx> twiddles(size_t n) {
  std::vector<cplx> tw(n);
  const double h = std::sqrt(0.5);
  for (size_t j = 0; j < n; ++j) {
    const uint64_t k8 = 8ull * j;
    const uint64_t oct = k8 / n;
    const uint64_t rem = k8 - oct * n;
    double c, s;  // cos and sin of theta = 2 pi j / n
    auto phi_sc = [&](uint64_t num, double& sp, double& cp) {
      if (num == 0) {
        sp = 0.0;
        cp = 1.0;
      } else if (num == n) {
        sp = h;
        cp = h;
      } else {
        const double phi = kPi / 4.0 * ((double)num / (double)n);
        sp = std::sin(phi);
        cp = std::cos(phi);
      }
    };
    double s0, c0, s1, c1;
    phi_sc(rem, s0, c0);
    phi_sc(n - rem, s1, c1);
    switch (oct) {
      case 0: c = c0; s = s0; break;
      case 1: c = s1; s = c1; break;
      case 2: c = -s0; s = c0; break;
      case 3: c = -c1; s = s1; break;
      case 4: c = -c0; s = -s0; break;
      case 5: c = -s1; s = -c1; break;
      case 6: c = s0; s = -c0; break;
      default: c = c1; s = -s1; break;
    }
    tw[j] = cplx(c, -s);
  }
  return tw;
}

// analytic_potentials.rs (NaN -> +inf)
static double nan_inf(double v) { return std::isnan(v) ? INFINITY : v; }
double pot_dispersion(double r, int n, double cn) { return nan_inf(cn * std::pow(r, (double)n)); }
double pot_lennard_jones(double r, double d6, double r6) {
  const double rr = std::pow(r6 / r, 6);
  return nan_inf(d6 * rr * (rr - 2.0));
}
double pot_harmonic(double r, double r0, double mass, double omega) {
  return nan_inf(0.5 * mass * omega * omega * (r - r0) * (r - r0));
}
double pot_morse(double r, double d, double a, double re) {
  const double e = std::exp(-a * (r - re));
  return nan_inf(d * (1.0 - e) * (1.0 - e));
}

// wave_function.rs:152-154
cplx gaussian(double x, double x0, double sigma, double p) {
  const double q = (x - x0) / (2.0 * sigma);
  return std::exp(cplx(-q * q, -(x - x0) * p));
}

// border_dumping.rs:14-33
std::vector<cplx> dumping_end(double width, double end, const Grid& g) {
  const double rmax = g.nodes.back();
  std::vector<cplx> m(g.nodes.size());
  for (size_t i = 0; i < g.nodes.size(); ++i) {
    const double x = g.nodes[i];
    if (x < rmax - width)
      m[i] = 1.0;
    else if (x > rmax - end)
      m[i] = 0.0;
    else
      m[i] = std::sin(kPi / 2.0 * (rmax - x) / width);
  }
  return m;
}

// time_grid.rs:22-33 and propagator_factory.rs:10-50: exp(-i H dt)
cplx select_step(int step, const so_time_grid& t) {
  const double ts = step == SO_STEP_FULL ? t.step : t.step / 2.0;
  if (t.im_time) return cplx(0.0, -ts);
  return cplx(ts, 0.0);
}

std::vector<cplx> phase_table(const double* h, size_t n, cplx dt) {
  std::vector<cplx> out(n);
  for (size_t i = 0; i < n; ++i) out[i] = std::exp(cplx(0.0, -1.0) * cplx(h[i], 0.0) * dt);
  return out;
}

std::vector<cplx> phase_table_complex(const cplx* h, size_t n, cplx dt) {
  std::vector<cplx> out(n);
  for (size_t i = 0; i < n; ++i) out[i] = std::exp(cplx(0.0, -1.0) * h[i] * dt);
  return out;
}

}  // namespace so
