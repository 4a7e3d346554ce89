// extern "C" boundary: status codes, handle types, argument validation.
// Each entry point is declared (with its reference citation) in
// include/split_operator.h.
#include <cmath>
#include <cstdio>
#include <cstring>
#include <new>
#include <numeric>

#include "model.hpp"

struct so_grid_t {
  so::Grid g;
};
struct so_wave_function_t {
  std::unique_ptr<so::WaveFunction> wf;
};
struct so_operator_t {
  std::shared_ptr<so::Operator> op;
};
struct so_operation_stack_t {
  std::shared_ptr<so::OperationStack> st;
};
struct so_propagation_t {
  std::shared_ptr<so::Propagation> p;
};
// the batch shares its members (declared first, so they outlive the executor)
struct so_batch_t {
  std::vector<std::shared_ptr<so::Propagation>> members;
  std::unique_ptr<so::Batch> b;
};

namespace {
thread_local std::string g_err;

template <class F>
int guard(F&& f) {
  try {
    f();
    return SO_OK;
  } catch (const so::Error& e) {
    g_err = e.what();
    return e.status;
  } catch (const std::bad_alloc&) {
    g_err = "out of host memory";
    return SO_ERR_INVALID;
  } catch (const std::exception& e) {
    g_err = e.what();
    return SO_ERR_INVALID;
  } catch (...) {
    g_err = "unknown error";
    return SO_ERR_INVALID;
  }
}

void need(bool c, const char* msg, int st = SO_ERR_INVALID) {
  if (!c) throw so::Error(st, msg);
}

std::vector<so::cplx> cvec(const double* p, size_t n) {
  need(p != nullptr || n == 0, "null array");
  std::vector<so::cplx> v(n);
  for (size_t i = 0; i < n; ++i) v[i] = so::cplx(p[2 * i], p[2 * i + 1]);
  return v;
}

void put(double* out, const std::vector<so::cplx>& v) {
  for (size_t i = 0; i < v.size(); ++i) {
    out[2 * i] = v[i].real();
    out[2 * i + 1] = v[i].imag();
  }
}

size_t prod(const size_t* shape, size_t nd) {
  size_t p = 1;
  for (size_t i = 0; i < nd; ++i) p *= shape[i];
  return p;
}

so::LossChecker* checker_of(so::Operator* op) { return op->loss_checker(); }

std::vector<int> ident(size_t n) {
  std::vector<int> p(n);
  std::iota(p.begin(), p.end(), 0);
  return p;
}
template <class T>
T* as(so_operator o) {
  need(o != nullptr, "null operator");
  T* p = dynamic_cast<T*>(o->op.get());
  need(p != nullptr, "operator has a different type");
  return p;
}

}  // namespace

namespace so {
void set_last_error(const char* msg) { g_err = msg; }
}  // namespace so

extern "C" {

const char* so_last_error(void) { return g_err.c_str(); }
int so_version(void) { return 10000; }
int so_launch_count(uint64_t* out) {
  return guard([&] {
    need(out, "null out");
    *out = so::launch_count();
  });
}
int so_selftest_bounded_wait(uint64_t limit_ns, uint64_t* out) {
  return guard([&] {
    need(out, "null out");
    need(limit_ns > 0 && limit_ns <= 1000000000ull, "limit must be in (0, 1 s]");
    unsigned long long r[3] = {0, 0, 0};
    so::cuda_check(so::bounded_wait_selftest(limit_ns, r), "bounded-wait self-test");
    for (int k = 0; k < 3; ++k) out[k] = r[k];
  });
}

// ---------------------------------------------------------------------- grid
int so_grid_new_linear_continuos(const char* name, double start, double end, size_t n, size_t dim, so_grid* out) {
  return guard([&] {
    need(name && out, "null argument");
    *out = new so_grid_t{so::Grid::linear_continuos(name, start, end, n, dim)};
  });
}
int so_grid_new_linear_countable(const char* name, double start, double end, size_t n, size_t dim, so_grid* out) {
  return guard([&] {
    need(name && out, "null argument");
    *out = new so_grid_t{so::Grid::linear_countable(name, start, end, n, dim)};
  });
}
int so_grid_new_custom(const char* name, const double* nodes, const double* weights, size_t n, size_t dim,
                       so_grid* out) {
  return guard([&] {
    need(name && out && nodes && weights, "null argument");
    *out = new so_grid_t{
        so::Grid::custom(name, std::vector<double>(nodes, nodes + n), std::vector<double>(weights, weights + n), dim)};
  });
}
int so_grid_nodes_no(so_grid g, size_t* out) {
  return guard([&] {
    need(g && out, "null argument");
    *out = g->g.size();
  });
}
int so_grid_dimension_no(so_grid g, size_t* out) {
  return guard([&] {
    need(g && out, "null argument");
    *out = g->g.dimension_no;
  });
}
int so_grid_name(so_grid g, char* buf, size_t cap) {
  return guard([&] {
    need(g && buf && cap > 0, "null argument");
    std::snprintf(buf, cap, "%s", g->g.name.c_str());
  });
}
int so_grid_nodes(so_grid g, double* out) {
  return guard([&] {
    need(g && out, "null argument");
    std::memcpy(out, g->g.nodes.data(), g->g.nodes.size() * sizeof(double));
  });
}
int so_grid_weights(so_grid g, double* out) {
  return guard([&] {
    need(g && out, "null argument");
    std::memcpy(out, g->g.weights.data(), g->g.weights.size() * sizeof(double));
  });
}
void so_grid_free(so_grid g) { delete g; }

// ------------------------------------------------------------- wave function
int so_wave_function_new(const double* array, const size_t* shape, size_t ndim, const so_grid* grids,
                         so_wave_function* out) {
  return guard([&] {
    need(array && shape && grids && out, "null argument");
    need(ndim >= 1 && ndim <= 4, "1 to 4 dimensions are supported", SO_ERR_UNSUPPORTED);
    std::vector<size_t> shp(shape, shape + ndim);
    std::vector<so::Grid> gs;
    for (size_t a = 0; a < ndim; ++a) {
      need(grids[a] != nullptr, "null grid");
      gs.push_back(grids[a]->g);
    }
    auto wf = std::make_unique<so::WaveFunction>(shp, gs, ident(ndim), so::kRealF64);
    wf->eng->import_host(array);
    wf->eng->sync();
    *out = new so_wave_function_t{std::move(wf)};
  });
}

int so_wave_function_clone(so_wave_function w, so_wave_function* out) {
  return guard([&] {
    need(w && out, "null argument");
    so::WaveFunction& s = *w->wf;
    auto c = std::make_unique<so::WaveFunction>(s.shape, s.grids, s.eng->perm, s.eng->real);
    c->last_grid_names = s.last_grid_names;
    c->possible_norm_change = s.possible_norm_change;
    c->eng->write_slot(c->cache_slot, s.eng->read_slot(s.cache_slot));
    s.eng->flush();
    so::cuda_check(cudaMemcpy(c->eng->psi.ptr, s.eng->psi.ptr, s.eng->psi.bytes, cudaMemcpyDeviceToDevice),
                   "clone copy");
    *out = new so_wave_function_t{std::move(c)};
  });
}

int so_wave_function_ndim(so_wave_function w, size_t* ndim, size_t* shape) {
  return guard([&] {
    need(w && ndim, "null argument");
    *ndim = w->wf->shape.size();
    if (shape)
      for (size_t i = 0; i < w->wf->shape.size(); ++i) shape[i] = w->wf->shape[i];
  });
}

int so_wave_function_norm(so_wave_function w, double* out) {
  return guard([&] {
    need(w && out, "null argument");
    so::Emitter em{w->wf->eng.get()};
    const int s = so::norm_slot(*w->wf, em);
    *out = w->wf->eng->read_slot(s);
  });
}

int so_wave_function_dot(so_wave_function a, so_wave_function b, double* out) {
  return guard([&] {
    need(a && b && out, "null argument");
    so::WaveFunction& x = *a->wf;
    so::WaveFunction& y = *b->wf;
    need(x.shape == y.shape && x.eng->perm == y.eng->perm && x.eng->real == y.eng->real, "shapes differ",
         SO_ERR_SHAPE);
    for (size_t i = 0; i < x.grids.size(); ++i)
      need(x.grids[i].weights == y.grids[i].weights, "weight arrays differ (wave_function.rs:91)", SO_ERR_STATE);
    so::Emitter ex{x.eng.get()};
    so::Emitter ey{y.eng.get()};
    const double n1 = x.eng->read_slot(so::norm_slot(x, ex));
    const double n2 = y.eng->read_slot(so::norm_slot(y, ey));
    y.eng->sync();
    const int sr = x.eng->alloc_slot(0.0), si = x.eng->alloc_slot(0.0);
    so::Action act{};
    act.op.kind = so::OP_DOT;
    act.op.a = sr;
    act.op.b = si;
    act.op.ptr = y.eng->psi.ptr;
    x.set_weights(act.op);
    x.eng->submit(act);
    const double re = x.eng->read_slot(sr), im = x.eng->read_slot(si);
    x.eng->free_slot(sr);
    x.eng->free_slot(si);
    const double d = std::sqrt(n1 * n2);
    out[0] = re / d;
    out[1] = im / d;
  });
}

int so_wave_function_normalize(so_wave_function w, double new_norm) {
  return guard([&] {
    need(w, "null argument");
    so::Engine& e = *w->wf->eng;
    const int t = e.alloc_slot(new_norm);
    so::Emitter em{&e};
    so::normalize_to_slot(*w->wf, em, t);
    e.sync();
    e.free_slot(t);
  });
}

static void density_impl(so::WaveFunction& wf, double* out, int axis) {
  so::Engine& e = *wf.eng;
  e.flush();
  so::Geometry g{};
  g.ndim = (int)wf.shape.size();
  for (int q = 0; q < g.ndim; ++q) {
    g.perm[q] = e.perm[q];
    g.sshape[q] = (int64_t)wf.shape[e.perm[q]];
  }
  size_t n = axis < 0 ? wf.points() : wf.shape[axis];
  so::DeviceBuffer d(n * sizeof(double));
  if (axis < 0) {
    so::cuda_check(so::launch_density(d.as<double>(), e.psi.ptr, e.real, g, e.stream), "density");
  } else {
    for (size_t a = 0; a < wf.grids.size(); ++a) wf.last_grid_names[a] = wf.grids[a].name;
    std::vector<const double*> w = wf.weight_ptrs();
    so::cuda_check(so::launch_state_density(d.as<double>(), e.psi.ptr, e.real, g, axis, w.data(), nullptr, e.stream),
                   "state density");
  }
  so::cuda_check(cudaMemcpyAsync(out, d.ptr, n * sizeof(double), cudaMemcpyDeviceToHost, e.stream), "copy");
  so::cuda_check(cudaStreamSynchronize(e.stream), "sync");
}

int so_wave_function_density(so_wave_function w, double* out) {
  return guard([&] {
    need(w && out, "null argument");
    density_impl(*w->wf, out, -1);
  });
}

int so_wave_function_state_density(so_wave_function w, size_t axis, double* out) {
  return guard([&] {
    need(w && out, "null argument");
    need(axis < w->wf->shape.size(), "axis out of range");
    density_impl(*w->wf, out, w->wf->shape.size() == 1 ? -1 : (int)axis);
  });
}

int so_wave_function_get_array(so_wave_function w, double* out) {
  return guard([&] {
    need(w && out, "null argument");
    w->wf->eng->export_host(out);
  });
}

int so_wave_function_set_array(so_wave_function w, const double* in) {
  return guard([&] {
    need(w && in, "null argument");
    w->wf->eng->import_host(in);
    w->wf->eng->sync();
    w->wf->possible_norm_change = true;
  });
}

int so_wave_function_grid(so_wave_function w, size_t axis, so_grid* out) {
  return guard([&] {
    need(w && out, "null argument");
    need(axis < w->wf->grids.size(), "axis out of range");
    *out = new so_grid_t{w->wf->grids[axis]};
  });
}

void so_wave_function_free(so_wave_function w) { delete w; }

int so_gaussian_distribution(const double* x, size_t n, double x0, double sigma, double p, double* out) {
  return guard([&] {
    need(x && out, "null argument");
    for (size_t i = 0; i < n; ++i) {
      const so::cplx v = so::gaussian(x[i], x0, sigma, p);
      out[2 * i] = v.real();
      out[2 * i + 1] = v.imag();
    }
  });
}

// ---------------------------------------------------------------- propagators
int so_one_dim_propagator_new(size_t shape, size_t dim, so_operator* out) {
  return guard([&] {
    need(out, "null argument");
    *out = new so_operator_t{std::make_shared<so::OneDimPropagator>(shape, dim)};
  });
}
int so_one_dim_propagator_set_operator(so_operator p, const double* op, size_t n) {
  return guard([&] {
    auto* o = as<so::OneDimPropagator>(p);
    need(n == o->op.size(), "operator length differs (one_dim_propagator.rs:26)", SO_ERR_SHAPE);
    o->op = cvec(op, n);
    o->version++;
  });
}
int so_one_dim_propagator_add_operator(so_operator p, const double* op, size_t n) {
  return guard([&] {
    auto* o = as<so::OneDimPropagator>(p);
    need(n == o->op.size(), "operator length differs (one_dim_propagator.rs:32)", SO_ERR_SHAPE);
    auto v = cvec(op, n);
    for (size_t i = 0; i < n; ++i) o->op[i] *= v[i];
    o->version++;
  });
}
int so_n_dim_propagator_new(so_operator* out) {
  return guard([&] {
    need(out, "null argument");
    *out = new so_operator_t{std::make_shared<so::NDimPropagator>()};
  });
}
int so_n_dim_propagator_set_operator(so_operator p, const double* op, const size_t* shape, size_t nd) {
  return guard([&] {
    auto* o = as<so::NDimPropagator>(p);
    need(shape && nd >= 1, "null shape");
    o->shape.assign(shape, shape + nd);
    o->op = cvec(op, prod(shape, nd));
    o->version++;
  });
}
int so_n_dim_propagator_add_operator(so_operator p, const double* op, const size_t* shape, size_t nd) {
  return guard([&] {
    auto* o = as<so::NDimPropagator>(p);
    need(shape && std::vector<size_t>(shape, shape + nd) == o->shape, "operator shape differs (n_dim_propagator.rs:27)",
         SO_ERR_SHAPE);
    auto v = cvec(op, prod(shape, nd));
    for (size_t i = 0; i < v.size(); ++i) o->op[i] *= v[i];
    o->version++;
  });
}
int so_non_diag_propagator_new(size_t dim, so_operator* out) {
  return guard([&] {
    need(out, "null argument");
    *out = new so_operator_t{std::make_shared<so::NonDiagPropagator>(dim)};
  });
}
int so_non_diag_propagator_set_operators(so_operator p, const double* ops, size_t count, size_t n) {
  return guard([&] {
    auto* o = as<so::NonDiagPropagator>(p);
    o->ops = cvec(ops, count * n * n);
    o->count = count;
    o->n = n;
    o->version++;
  });
}
int so_propagator_set_loss_checked(so_operator p, const char* name) {
  return guard([&] {
    need(p && name, "null argument");
    std::unique_ptr<so::LossChecker> lc = std::make_unique<so::LossChecker>(name);
    if (auto* a = dynamic_cast<so::OneDimPropagator*>(p->op.get()))
      a->lc = std::move(lc);
    else if (auto* b = dynamic_cast<so::NDimPropagator*>(p->op.get()))
      b->lc = std::move(lc);
    else if (auto* c = dynamic_cast<so::NonDiagPropagator*>(p->op.get()))
      c->lc = std::move(lc);
    else
      throw so::Error(SO_ERR_INVALID, "not a propagator");
  });
}
int so_propagator_apply(so_operator p, so_wave_function w) {
  return guard([&] {
    need(p && w, "null argument");
    need(p->op->cls == so::OpClass::Propagator, "not a propagator");
    so::Emitter em{w->wf->eng.get()};
    p->op->apply(*w->wf, em);
    w->wf->eng->flush();
  });
}
int so_propagator_loss(so_operator p, double* out, int* has) {
  return guard([&] {
    need(p && out && has, "null argument");
    so::LossChecker* lc = checker_of(p->op.get());
    *has = lc ? 1 : 0;
    *out = lc ? lc->loss() : 0.0;
  });
}
int so_propagator_loss_reset(so_operator p) {
  return guard([&] {
    need(p, "null argument");
    if (so::LossChecker* lc = checker_of(p->op.get())) lc->reset(nullptr);
  });
}

int so_one_dim_into_propagator(const double* h, so_grid grid, so_time_grid time, int step, so_operator* out) {
  return guard([&] {
    need(h && grid && out, "null argument");
    auto p = std::make_shared<so::OneDimPropagator>(grid->g.size(), grid->g.dimension_no);
    p->op = so::phase_table(h, grid->g.size(), so::select_step(step, time));
    *out = new so_operator_t{p};
  });
}
int so_n_dim_into_propagator(const double* h, const size_t* shape, size_t nd, so_time_grid time, int step,
                             so_operator* out) {
  return guard([&] {
    need(h && shape && out && nd >= 1, "null argument");
    auto p = std::make_shared<so::NDimPropagator>();
    p->shape.assign(shape, shape + nd);
    p->op = so::phase_table(h, prod(shape, nd), so::select_step(step, time));
    *out = new so_operator_t{p};
  });
}
int so_complex_n_dim_into_propagator(const double* h, const size_t* shape, size_t nd, so_time_grid time, int step,
                                     so_operator* out) {
  return guard([&] {
    need(h && shape && out && nd >= 1, "null argument");
    auto p = std::make_shared<so::NDimPropagator>();
    p->shape.assign(shape, shape + nd);
    auto hc = cvec(h, prod(shape, nd));
    p->op = so::phase_table_complex(hc.data(), hc.size(), so::select_step(step, time));
    *out = new so_operator_t{p};
  });
}

// ------------------------------------------------------------ transformations
int so_fft_transformation_new(so_grid grid, const char* name, so_operator* out) {
  return guard([&] {
    need(grid && name && out, "null argument");
    *out = new so_operator_t{std::make_shared<so::FFTTransformation>(grid->g, name)};
  });
}
int so_matrix_transformation_new(so_grid grid, so_grid gt, so_operator* out) {
  return guard([&] {
    need(grid && gt && out, "null argument");
    *out = new so_operator_t{std::make_shared<so::MatrixTransformation>(grid->g, gt->g)};
  });
}
int so_matrix_transformation_set_diagonalization_matrix(so_operator t, const double* m, const double* mi, size_t n) {
  return guard([&] {
    auto* o = as<so::MatrixTransformation>(t);
    need(n == o->dimension_size, "matrix size differs (matrix_transformation.rs:40-47)", SO_ERR_SHAPE);
    o->t = cvec(m, n * n);
    o->tinv = cvec(mi, n * n);
    o->version++;
  });
}
int so_state_matrix_transformation_new(size_t dep, so_grid grid, so_grid gt, so_operator* out) {
  return guard([&] {
    need(grid && gt && out, "null argument");
    *out = new so_operator_t{std::make_shared<so::StateMatrixTransformation>(dep, grid->g, gt->g)};
  });
}
int so_state_matrix_transformation_set_diagonalization_matrices(so_operator t, const double* ms, const double* mis,
                                                                size_t count, size_t n) {
  return guard([&] {
    auto* o = as<so::StateMatrixTransformation>(t);
    need(n == o->n, "matrix size differs", SO_ERR_SHAPE);
    o->ts = cvec(ms, count * n * n);
    o->tinvs = cvec(mis, count * n * n);
    o->count = count;
    o->version++;
  });
}
int so_transformation_transform(so_operator t, so_wave_function w) {
  return guard([&] {
    need(t && w, "null argument");
    so::Emitter em{w->wf->eng.get()};
    t->op->transform(*w->wf, em);
    w->wf->eng->flush();
  });
}
int so_transformation_inverse_transform(so_operator t, so_wave_function w) {
  return guard([&] {
    need(t && w, "null argument");
    so::Emitter em{w->wf->eng.get()};
    t->op->inverse_transform(*w->wf, em);
    w->wf->eng->flush();
  });
}
int so_transformation_grid(so_operator t, so_grid* out) {
  return guard([&] {
    need(t && out, "null argument");
    so::Grid* g = t->op->grid_transformation();
    need(g != nullptr, "not a transformation");
    *out = new so_grid_t{*g};
  });
}

// ------------------------------------------------------------ hamiltonians
int so_kinetic_hamiltonian(so_grid grid, double red_mass, double* out) {
  return guard([&] {
    need(grid && out, "null argument");
    auto k = so::kinetic_hamiltonian(grid->g, red_mass);
    std::memcpy(out, k.data(), k.size() * sizeof(double));
  });
}
int so_rotational_hamiltonian(so_grid radial, so_grid polar, double red_mass, double b, double* out) {
  return guard([&] {
    need(radial && polar && out, "null argument");
    auto h = so::rotational_hamiltonian(radial->g, polar->g, red_mass, b);
    std::memcpy(out, h.data(), h.size() * sizeof(double));
  });
}
int so_two_dim_into_n_dim_operator(const size_t* shape, size_t nd, const double* h, so_grid g1, so_grid g2,
                                   double* out) {
  return guard([&] {
    need(shape && h && g1 && g2 && out && nd >= 2 && nd <= 4, "bad argument");
    const size_t a1 = g1->g.dimension_no, a2 = g2->g.dimension_no;
    need(a1 < nd && a2 < nd && a1 != a2, "grid dimensions out of range");
    need(shape[a1] == g1->g.size() && shape[a2] == g2->g.size(), "grid sizes differ from shape", SO_ERR_SHAPE);
    const size_t total = prod(shape, nd);
    std::vector<size_t> st(nd);
    size_t acc = 1;
    for (size_t a = nd; a-- > 0;) {
      st[a] = acc;
      acc *= shape[a];
    }
    for (size_t i = 0; i < total; ++i) {
      const size_t c1 = (i / st[a1]) % shape[a1], c2 = (i / st[a2]) % shape[a2];
      out[i] = h[c1 * shape[a2] + c2];
    }
  });
}
int so_legendre_diagonalization_operator(so_grid polar, so_operator* out) {
  return so_associated_legendre_diagonalization_operator(polar, 0, out);
}
int so_associated_legendre_diagonalization_operator(so_grid polar, int omega, so_operator* out) {
  return guard([&] {
    need(polar && out, "null argument");
    const size_t n = polar->g.size();
    need(n >= 2, "polar grid needs at least 2 nodes");
    so::Grid lg = so::Grid::linear_countable("angular_momentum", 0.0, (double)(n - 1), n, polar->g.dimension_no);
    auto m = std::make_shared<so::MatrixTransformation>(polar->g, lg);
    so::legendre_matrices(polar->g, omega, m->t, m->tinv);
    *out = new so_operator_t{m};
  });
}
int so_associated_legendre_operator(so_grid polar, so_grid omega_grid, so_operator* out) {
  return guard([&] {
    need(polar && omega_grid && out, "null argument");
    const size_t n = polar->g.size();
    so::Grid lg = so::Grid::linear_countable("angular_momentum", 0.0, (double)(n - 1), n, polar->g.dimension_no);
    auto s = std::make_shared<so::StateMatrixTransformation>(omega_grid->g.dimension_no, polar->g, lg);
    for (double om : omega_grid->g.nodes) {
      std::vector<so::cplx> t, ti;
      so::legendre_matrices(polar->g, (int64_t)om, t, ti);
      s->ts.insert(s->ts.end(), t.begin(), t.end());
      s->tinvs.insert(s->tinvs.end(), ti.begin(), ti.end());
    }
    s->count = omega_grid->g.size();
    *out = new so_operator_t{s};
  });
}
int so_legendre_polynomials(size_t j, double x, double* out) {
  return guard([&] {
    need(out, "null argument");
    auto p = so::legendre_polynomials(j, x);
    std::memcpy(out, p.data(), p.size() * sizeof(double));
  });
}
int so_associated_legendre_polynomials(size_t j, int m, double x, double* out) {
  return guard([&] {
    need(out, "null argument");
    auto p = so::associated_legendre_polynomials(j, m, x);
    std::memcpy(out, p.data(), p.size() * sizeof(double));
  });
}
int so_gauss_legendre(size_t n, double* nodes, double* weights) {
  return guard([&] {
    need(nodes && weights, "null argument");
    std::vector<double> x, w;
    so::gauss_legendre(n, x, w);
    std::memcpy(nodes, x.data(), n * sizeof(double));
    std::memcpy(weights, w.data(), n * sizeof(double));
  });
}
int so_dispersion(const double* r, size_t n, int power, double cn, double* out) {
  return guard([&] {
    need(r && out, "null argument");
    for (size_t i = 0; i < n; ++i) out[i] = so::pot_dispersion(r[i], power, cn);
  });
}
int so_lennard_jones(const double* r, size_t n, double d6, double r6, double* out) {
  return guard([&] {
    need(r && out, "null argument");
    for (size_t i = 0; i < n; ++i) out[i] = so::pot_lennard_jones(r[i], d6, r6);
  });
}
int so_harmonic(const double* r, size_t n, double r0, double mass, double omega, double* out) {
  return guard([&] {
    need(r && out, "null argument");
    for (size_t i = 0; i < n; ++i) out[i] = so::pot_harmonic(r[i], r0, mass, omega);
  });
}
int so_morse(const double* r, size_t n, double d, double a, double re, double* out) {
  return guard([&] {
    need(r && out, "null argument");
    for (size_t i = 0; i < n; ++i) out[i] = so::pot_morse(r[i], d, a, re);
  });
}

// ------------------------------------------------------------------ controls
int so_leak_control_new(so_operator* out) {
  return guard([&] {
    need(out, "null argument");
    *out = new so_operator_t{std::make_shared<so::LeakControl>()};
  });
}
int so_leak_control_add_loss_checker(so_operator c, const char* name) {
  return guard([&] {
    need(name, "null name");
    as<so::LeakControl>(c)->lc = std::make_unique<so::LossChecker>(name);
  });
}
int so_dumping_end(double width, double end, so_grid grid, double* out) {
  return guard([&] {
    need(grid && out, "null argument");
    put(out, so::dumping_end(width, end, grid->g));
  });
}
int so_border_dumping_new(const double* mask, size_t n, so_grid grid, so_operator* out) {
  return guard([&] {
    need(mask && grid && out, "null argument");
    *out = new so_operator_t{std::make_shared<so::BorderDumping>(cvec(mask, n), grid->g)};
  });
}
int so_border_dumping_add_loss_checker(so_operator c, const char* name) {
  return guard([&] {
    need(name, "null name");
    as<so::BorderDumping>(c)->lc = std::make_unique<so::LossChecker>(name);
  });
}
int so_control_first_half(so_operator c, so_wave_function w) {
  return guard([&] {
    need(c && w, "null argument");
    so::Emitter em{w->wf->eng.get()};
    c->op->first_half(*w->wf, em);
    w->wf->eng->flush();
  });
}
int so_control_second_half(so_operator c, so_wave_function w) {
  return guard([&] {
    need(c && w, "null argument");
    so::Emitter em{w->wf->eng.get()};
    c->op->second_half(*w->wf, em);
    w->wf->eng->flush();
  });
}
int so_control_loss(so_operator c, double* out, int* has) { return so_propagator_loss(c, out, has); }

// -------------------------------------------------------------------- savers
int so_state_saver_new(const char* name, so_time_grid time, so_grid state_grid, size_t frames, so_operator* out) {
  return guard([&] {
    need(name && state_grid && out, "null argument");
    *out = new so_operator_t{std::make_shared<so::StateSaver>(name, time, state_grid->g, nullptr, frames)};
  });
}
int so_wave_function_saver_new(const char* name, so_time_grid time, so_grid x, so_grid y, size_t frames,
                               so_operator* out) {
  return guard([&] {
    need(name && x && y && out, "null argument");
    *out = new so_operator_t{std::make_shared<so::StateSaver>(name, time, x->g, &y->g, frames)};
  });
}
int so_saver_frames(so_operator s, double* data, double* times, size_t* taken) {
  return guard([&] {
    auto* o = as<so::StateSaver>(s);
    if (data) std::memcpy(data, o->data.data(), o->data.size() * sizeof(double));
    if (times) std::memcpy(times, o->times.data(), o->times.size() * sizeof(double));
    if (taken) *taken = o->times.size();
  });
}
int so_saver_shape(so_operator s, size_t* points, size_t* frames) {
  return guard([&] {
    auto* o = as<so::StateSaver>(s);
    if (points) *points = o->points;
    if (frames) *frames = o->frames_no;
  });
}

static void write_npy(const std::string& path, const std::vector<double>& data, const std::vector<size_t>& shape) {
  FILE* f = std::fopen(path.c_str(), "wb");
  if (!f) throw so::Error(SO_ERR_IO, "cannot open " + path);
  std::string sh = "(";
  for (size_t i = 0; i < shape.size(); ++i) sh += std::to_string(shape[i]) + (shape.size() == 1 ? "," : (i + 1 < shape.size() ? ", " : ""));
  sh += ")";
  std::string hdr = "{'descr': '<f8', 'fortran_order': False, 'shape': " + sh + ", }";
  while ((10 + hdr.size() + 1) % 64 != 0) hdr += ' ';
  hdr += '\n';
  const unsigned char magic[8] = {0x93, 'N', 'U', 'M', 'P', 'Y', 1, 0};
  const uint16_t hl = (uint16_t)hdr.size();
  bool ok = std::fwrite(magic, 1, 8, f) == 8;
  ok = ok && std::fwrite(&hl, 2, 1, f) == 1;
  ok = ok && std::fwrite(hdr.data(), 1, hdr.size(), f) == hdr.size();
  ok = ok && std::fwrite(data.data(), sizeof(double), data.size(), f) == data.size();
  std::fclose(f);
  if (!ok) throw so::Error(SO_ERR_IO, "failed to write " + path);
}

void so::StateSaver::save() const {
  if (two_d) {
    write_npy(fname + ".npy", data, {grid_a.size(), grid_b.size(), frames_no});
    write_npy(fname + "_x_grid.npy", grid_a.nodes, {grid_a.size()});
    write_npy(fname + "_y_grid.npy", grid_b.nodes, {grid_b.size()});
  } else {
    write_npy(fname + ".npy", data, {grid_a.size(), frames_no});
    write_npy(fname + "_" + grid_a.name + "_grid.npy", grid_a.nodes, {grid_a.size()});
  }
  write_npy(fname + "_time.npy", times, {times.size()});
}

int so_saver_save(so_operator s) {
  return guard([&] { as<so::StateSaver>(s)->save(); });
}
int so_saver_reset(so_operator s) {
  return guard([&] { as<so::StateSaver>(s)->reset(); });
}
int so_saver_monitor(so_operator s, so_wave_function w) {
  return guard([&] {
    need(w, "null argument");
    so::Emitter em{w->wf->eng.get()};
    as<so::StateSaver>(s)->monitor(*w->wf, em);
  });
}

void so_operator_free(so_operator op) { delete op; }

// -------------------------------------------------------------------- stack
int so_operation_stack_new(so_operation_stack* out) {
  return guard([&] {
    need(out, "null argument");
    *out = new so_operation_stack_t{std::make_shared<so::OperationStack>()};
  });
}
static void add(so_operation_stack s, so_operator o, so::OpClass cls, int flag) {
  need(s && o, "null argument");
  need(o->op->cls == cls, "operator kind does not match the stack call");
  s->st->stack.push_back({o->op, flag});
}
int so_operation_stack_add_propagator(so_operation_stack s, so_operator p) {
  return guard([&] { add(s, p, so::OpClass::Propagator, 0); });
}
int so_operation_stack_add_transformation(so_operation_stack s, so_operator t, int order) {
  return guard([&] {
    need(order == SO_ORDER_NORMAL || order == SO_ORDER_INVERSE_FIRST, "bad order");
    add(s, t, so::OpClass::Transformation, order);
  });
}
int so_operation_stack_add_saver(so_operation_stack s, so_operator v, int apply) {
  return guard([&] {
    // propagation.rs:55: apply != FirstHalf & SecondHalf (i.e. not None)
    need(apply >= 1 && apply <= 3, "a saver must apply on at least one half");
    add(s, v, so::OpClass::Saver, apply);
  });
}
int so_operation_stack_add_control(so_operation_stack s, so_operator c, int apply) {
  return guard([&] {
    need(apply >= 0 && apply <= 3, "bad apply flags");
    add(s, c, so::OpClass::Control, apply);
  });
}
int so_operation_stack_len(so_operation_stack s, size_t* out) {
  return guard([&] {
    need(s && out, "null argument");
    *out = s->st->stack.size();
  });
}
void so_operation_stack_free(so_operation_stack s) { delete s; }

// -------------------------------------------------------------- propagation
int so_propagation_new(so_wave_function w, so_time_grid time, so_operation_stack s, int precision,
                       so_propagation* out) {
  return guard([&] {
    need(w && s && out, "null argument");
    *out = new so_propagation_t{std::make_unique<so::Propagation>(*w->wf, time, s->st, precision)};
  });
}
int so_propagation_propagate(so_propagation p) {
  return guard([&] {
    need(p, "null argument");
    p->p->propagate();
  });
}
int so_propagation_steps(so_propagation p, uint64_t steps) {
  return guard([&] {
    need(p, "null argument");
    p->p->steps(steps);
  });
}
int so_propagation_mean_energy(so_propagation p, double* out) {
  return guard([&] {
    need(p && out, "null argument");
    *out = p->p->mean_energy();
  });
}
static void copy_losses(const std::vector<double>& v, double* out, size_t cap, size_t* count) {
  if (count) *count = v.size();
  if (out)
    for (size_t i = 0; i < v.size() && i < cap; ++i) out[i] = v[i];
}
int so_propagation_get_losses(so_propagation p, double* out, size_t cap, size_t* count) {
  return guard([&] {
    need(p, "null argument");
    copy_losses(p->p->losses(false), out, cap, count);
  });
}
int so_propagation_all_losses(so_propagation p, double* out, size_t cap, size_t* count) {
  return guard([&] {
    need(p, "null argument");
    copy_losses(p->p->losses(true), out, cap, count);
  });
}
int so_propagation_reset_losses(so_propagation p) {
  return guard([&] {
    need(p, "null argument");
    p->p->reset_losses();
  });
}
int so_propagation_reset_savers_state(so_propagation p) {
  return guard([&] {
    need(p, "null argument");
    p->p->reset_savers();
  });
}
int so_propagation_savers_save(so_propagation p) {
  return guard([&] {
    need(p, "null argument");
    p->p->savers_save();
  });
}
int so_propagation_wave_function(so_propagation p, so_wave_function* out) {
  return guard([&] {
    need(p && out, "null argument");
    *out = new so_wave_function_t{p->p->snapshot()};
  });
}
int so_propagation_get_array(so_propagation p, double* out) {
  return guard([&] {
    need(p && out, "null argument");
    p->p->get_array(out);
  });
}
int so_propagation_set_array(so_propagation p, const double* in) {
  return guard([&] {
    need(p && in, "null argument");
    p->p->set_array(in);
  });
}
int so_propagation_norm(so_propagation p, double* out) {
  return guard([&] {
    need(p && out, "null argument");
    *out = p->p->norm();
  });
}
int so_propagation_set_stream(so_propagation p, void* stream) {
  return guard([&] {
    need(p, "null argument");
    p->p->synchronize();
    p->p->set_stream((cudaStream_t)stream);
  });
}
int so_propagation_synchronize(so_propagation p) {
  return guard([&] {
    need(p, "null argument");
    p->p->synchronize();
  });
}
int so_propagation_describe(so_propagation p, char* buf, size_t cap) {
  return guard([&] {
    need(p && buf && cap > 0, "null argument");
    std::snprintf(buf, cap, "%s", p->p->describe().c_str());
  });
}
int so_propagation_set_timing(so_propagation p, int enabled) {
  return guard([&] {
    need(p, "null argument");
    p->p->set_timing(enabled != 0);
  });
}
int so_propagation_kernel_times(so_propagation p, char* buf, size_t cap) {
  return guard([&] {
    need(p && buf && cap > 0, "null argument");
    std::snprintf(buf, cap, "%s", p->p->kernel_times().c_str());
  });
}
int so_propagation_checkpoint(so_propagation p, void* buf, size_t cap, size_t* size) {
  return guard([&] {
    need(p && size, "null argument");
    const std::vector<unsigned char> b = p->p->checkpoint();
    *size = b.size();
    if (buf) {
      need(cap >= b.size(), "checkpoint buffer is smaller than the checkpoint");
      std::memcpy(buf, b.data(), b.size());
    }
  });
}
int so_propagation_restore(so_propagation p, const void* buf, size_t size) {
  return guard([&] {
    need(p && buf, "null argument");
    p->p->restore(static_cast<const unsigned char*>(buf), size);
  });
}
int so_propagation_steps_done(so_propagation p, uint64_t* out) {
  return guard([&] {
    need(p && out, "null argument");
    *out = p->p->steps_done();
  });
}
void so_propagation_free(so_propagation p) { delete p; }

int so_batch_new(const so_propagation* props, size_t count, so_batch* out) {
  return guard([&] {
    need(props && out && count > 0, "null argument");
    std::vector<so::Propagation*> ps;
    std::vector<std::shared_ptr<so::Propagation>> members;
    for (size_t i = 0; i < count; ++i) {
      need(props[i] != nullptr, "null propagation");
      ps.push_back(props[i]->p.get());
      members.push_back(props[i]->p);
    }
    auto exec = std::make_unique<so::Batch>(ps);
    *out = new so_batch_t{std::move(members), std::move(exec)};
  });
}
int so_batch_steps(so_batch b, uint64_t steps) {
  return guard([&] {
    need(b, "null argument");
    b->b->steps(steps);
  });
}
int so_batch_set_timing(so_batch b, int enabled) {
  return guard([&] {
    need(b, "null argument");
    b->b->set_timing(enabled != 0);
  });
}
int so_batch_kernel_times(so_batch b, char* buf, size_t cap) {
  return guard([&] {
    need(b && buf && cap > 0, "null argument");
    std::snprintf(buf, cap, "%s", b->b->kernel_times().c_str());
  });
}
int so_batch_launches_per_step(so_batch b, size_t* out) {
  return guard([&] {
    need(b && out, "null argument");
    *out = b->b->launches_per_step();
  });
}
int so_batch_set_arrays(so_batch b, const double* const* in, size_t count) {
  return guard([&] {
    need(b && in, "null argument");
    need(count == b->b->size(), "count differs from the batch size");
    b->b->set_arrays(in);
  });
}
int so_batch_get_arrays(so_batch b, double* const* out, size_t count) {
  return guard([&] {
    need(b && out, "null argument");
    need(count == b->b->size(), "count differs from the batch size");
    b->b->get_arrays(out);
  });
}
int so_batch_steps_host(so_batch b, const double* const* in, double* const* out, size_t count, uint64_t steps) {
  return guard([&] {
    need(b && in && out, "null argument");
    need(count == b->b->size(), "count differs from the batch size");
    b->b->steps_host(in, out, steps);
  });
}
int so_batch_tune(so_batch b, const char* cache_path, int trial_steps, char* report, size_t cap) {
  return guard([&] {
    need(b, "null argument");
    const std::string r = b->b->tune(cache_path ? cache_path : "", trial_steps);
    if (report && cap > 0) std::snprintf(report, cap, "%s", r.c_str());
  });
}
void so_batch_free(so_batch b) { delete b; }

int so_schedules_load(const char* path) {
  return guard([&] {
    need(path, "null argument");
    FILE* f = std::fopen(path, "r");
    need(f != nullptr, "cannot open the schedule cache", SO_ERR_IO);
    std::string text;
    char buf[4096];
    size_t k;
    while ((k = std::fread(buf, 1, sizeof(buf), f)) > 0) text.append(buf, k);
    std::fclose(f);
    need(so::schedules_from_json(text), "the schedule cache is not in the tuner's format");
  });
}
int so_schedules_save(const char* path) {
  return guard([&] {
    need(path, "null argument");
    FILE* f = std::fopen(path, "w");
    need(f != nullptr, "cannot write the schedule cache", SO_ERR_IO);
    const std::string js = so::schedules_json();
    const bool ok = std::fwrite(js.data(), 1, js.size(), f) == js.size();
    need(std::fclose(f) == 0 && ok, "cannot write the schedule cache", SO_ERR_IO);
  });
}
int so_schedules_reset(void) {
  return guard([&] { so::reset_schedules(); });
}

}  // extern "C"
