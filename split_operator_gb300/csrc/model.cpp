// Engine (device state + pass builder) and the host logic of the operators,
// written to follow the Rust crate's control flow operator by operator so the
// norm cache, loss bookkeeping and representation swaps happen exactly where
// the reference does them; every array touch becomes an emitted device op.
#include <algorithm>
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cmath>
#include <cstring>
#include <mutex>
#include <numeric>
#include <tuple>

#include "model.hpp"

#include <cstdio>
#include <cstdlib>

namespace so {

void cuda_check(cudaError_t e, const char* what) {
  if (e != cudaSuccess) throw Error(SO_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}

DeviceBuffer::DeviceBuffer(size_t b) : bytes(b) {
  if (b) cuda_check(cudaMalloc(&ptr, b), "cudaMalloc");
}
DeviceBuffer& DeviceBuffer::operator=(DeviceBuffer&& o) noexcept {
  if (this != &o) {
    if (ptr) cudaFree(ptr);
    ptr = o.ptr;
    bytes = o.bytes;
    o.ptr = nullptr;
    o.bytes = 0;
  }
  return *this;
}
DeviceBuffer::~DeviceBuffer() {
  if (ptr) cudaFree(ptr);
}

// ------------------------------------------------------------------ ScalarState
ScalarState::~ScalarState() {
  if (home) {
    auto& v = home->bound;
    v.erase(std::remove(v.begin(), v.end(), this), v.end());
    for (int s : slots) home->free_slot(s);
  }
}

const std::vector<int>& ScalarState::bind(Engine* e) {
  if (home == e) return slots;
  if (home) unbind();
  slots.clear();
  for (double v : host) slots.push_back(e->alloc_slot(v));
  home = e;
  e->bound.push_back(this);
  return slots;
}

void ScalarState::unbind() {
  if (!home) return;
  for (size_t i = 0; i < slots.size(); ++i) host[i] = home->read_slot(slots[i]);
  for (int s : slots) home->free_slot(s);
  auto& v = home->bound;
  v.erase(std::remove(v.begin(), v.end(), this), v.end());
  home = nullptr;
  slots.clear();
}

double ScalarState::get(size_t i) { return home ? home->read_slot(slots[i]) : host[i]; }

void ScalarState::set(size_t i, double v) {
  if (home)
    home->write_slot(slots[i], v);
  else
    host[i] = v;
}

// ----------------------------------------------------------------------- Engine
const char* op_kind_name(int k);
static bool is_scalar_kind(int k) { return k == OP_COPY || k == OP_LOSS || k == OP_SETC || k == OP_RECORD; }

Engine::Engine(const std::vector<size_t>& shp, const std::vector<int>& prm, int rl)
    : real(rl), fp64(rl != kRealF32), shape(shp), perm(prm) {
  if (real < kRealF32 || real > kRealFF) throw Error(SO_ERR_INVALID, "unknown state precision");
  if (shape.empty() || shape.size() > (size_t)kMaxDims)
    throw Error(SO_ERR_UNSUPPORTED, "wave functions of 1 to 4 dimensions are supported");
  int dev_count = 0;
  if (cudaGetDeviceCount(&dev_count) != cudaSuccess || dev_count == 0) {
    cudaGetLastError();
    throw Error(SO_ERR_CUDA, "no CUDA device available");
  }
  psi = DeviceBuffer(points() * elem_bytes());
  slots_ = DeviceBuffer(kNumSlots * sizeof(double));
  cuda_check(cudaMemset(slots_.ptr, 0, kNumSlots * sizeof(double)), "cudaMemset");
  counter_ = DeviceBuffer(sizeof(unsigned int) * 4);
  cuda_check(cudaMemset(counter_.ptr, 0, sizeof(unsigned int) * 4), "cudaMemset");
  nonfinite_slot = alloc_slot(0.0);
  timeout_slot = alloc_slot(0.0);
  int64_t max_tiles = 1;
  for (size_t a = 0; a < shape.size(); ++a) {
    try {
      Geometry g = geometry((int)a, false);
      max_tiles = std::max<int64_t>(max_tiles, g.tiles);
    } catch (const Error&) {
    }
  }
  partials_cap_ = (size_t)max_tiles;
  partials_ = DeviceBuffer(partials_cap_ * kMaxRed * sizeof(double));
}

Engine::~Engine() {
  try {
    std::vector<ScalarState*> b = bound;
    for (ScalarState* s : b) s->unbind();
    if (stream) cudaStreamSynchronize(stream);
    else cudaDeviceSynchronize();
  } catch (...) {
  }
}

size_t Engine::points() const {
  size_t p = 1;
  for (size_t s : shape) p *= s;
  return p;
}

bool Engine::resident_capable() const {
  const size_t tile_max = fp64 ? 4096 : 8192;
  return shape.size() == 1 && points() <= tile_max && points() >= 2;
}

static int64_t pow2_floor(int64_t v) {
  int64_t p = 1;
  while (p * 2 <= v) p *= 2;
  return p;
}

Geometry Engine::geometry(int sweep_axis, bool resident) const {
  Geometry g{};
  const int nd = (int)shape.size();
  g.ndim = nd;
  g.spos = -1;
  for (int q = 0; q < nd; ++q) {
    g.perm[q] = perm[q];
    g.sshape[q] = (int64_t)shape[perm[q]];
    if (perm[q] == sweep_axis) g.spos = q;
  }
  if (g.spos < 0) throw Error(SO_ERR_INVALID, "sweep axis out of range");
  g.sweep_axis = sweep_axis;
  g.n = g.sshape[g.spos];
  g.inner = 1;
  for (int q = g.spos + 1; q < nd; ++q) g.inner *= g.sshape[q];
  g.outer = 1;
  for (int q = 0; q < g.spos; ++q) g.outer *= g.sshape[q];
  // two tile buffers of at most ~139 KB together; FP64 lanes of 4097..8192 points only in
  // FFT-pair passes (one in-place lane buffer), which Engine::launch checks
  const int64_t tile_max = fp64 ? 4096 : 8192;
  const int64_t lane_max = resident ? tile_max : 8192;
  g.vals = 8;
  if (g.n > lane_max)
    throw Error(SO_ERR_UNSUPPORTED, "lanes longer than " + std::to_string(lane_max) + " points are not supported");
  int64_t L;
  if (resident) {
    if (g.inner == 1)
      L = g.outer;
    else if (g.outer == 1)
      L = g.inner;
    else
      throw Error(SO_ERR_UNSUPPORTED, "resident pass needs a single lane family");
    if (L * g.n > tile_max) throw Error(SO_ERR_UNSUPPORTED, "array too large for a resident pass");
    g.tiles_per_outer = 1;
    g.tiles = 1;
  } else if (g.inner == 1) {
    const int64_t lmax = std::max<int64_t>(1, pow2_floor(std::max<int64_t>(1, tile_max / g.n)));
    int64_t want = pow2_floor(std::max<int64_t>(1, g.outer / 304));
    want = std::max<int64_t>(want, pow2_floor(std::max<int64_t>(1, 1024 / g.n)));
    L = std::min(want, lmax);
    g.tiles_per_outer = 1;
    g.tiles = (g.outer + L - 1) / L;
  } else {
    const int64_t lmax = std::max<int64_t>(1, pow2_floor(std::max<int64_t>(1, tile_max / g.n)));
    L = std::min<int64_t>({lmax, fp64 ? 16 : 32, pow2_floor(g.inner)});
    while (L > 4 && g.outer * ((g.inner + L - 1) / L) < 304) L /= 2;
    g.tiles_per_outer = (int32_t)((g.inner + L - 1) / L);
    g.tiles = g.outer * g.tiles_per_outer;
  }
  g.lanes_per_tile = (int32_t)L;
  int64_t ls = g.n + (g.n >> 4);
  if (ls % 2 == 0) ls += 1;
  g.lane_stride = (int32_t)ls;
  return g;
}

int Engine::alloc_slot(double init) {
  int s;
  if (!free_slots_.empty()) {
    s = free_slots_.back();
    free_slots_.pop_back();
  } else {
    if (next_slot_ >= kNumSlots) throw Error(SO_ERR_UNSUPPORTED, "out of device scalar slots");
    s = next_slot_++;
  }
  // a fresh slot is not referenced by the open pass: initialise it in stream order without closing the pass
  cuda_check(cudaMemcpyAsync(slots() + s, &init, sizeof(double), cudaMemcpyHostToDevice, stream), "slot init");
  return s;
}

void Engine::free_slot(int s) { free_slots_.push_back(s); }

void Engine::write_slot(int s, double v) {
  flush();
  cuda_check(cudaMemcpyAsync(slots() + s, &v, sizeof(double), cudaMemcpyHostToDevice, stream), "slot write");
}

double Engine::read_slot(int s) {
  flush();
  double v = 0.0;
  cuda_check(cudaMemcpyAsync(&v, slots() + s, sizeof(double), cudaMemcpyDeviceToHost, stream), "slot read");
  cuda_check(cudaStreamSynchronize(stream), "stream sync");
  return v;
}

template <typename T>
static void upload(DeviceBuffer& buf, const std::vector<T>& v, cudaStream_t s) {
  const size_t b = v.size() * sizeof(T);
  if (buf.bytes != b) buf = DeviceBuffer(b);
  cuda_check(cudaMemcpyAsync(buf.ptr, v.data(), b, cudaMemcpyHostToDevice, s), "table upload");
  cuda_check(cudaStreamSynchronize(s), "table upload sync");
}

// the float-float pair of d: hi = d rounded to FP32, lo = the (exact) remainder rounded
static void ff_pair(double d, float* out) {
  out[0] = (float)d;
  out[1] = (float)(d - (double)out[0]);
}

static void upload_complex(DeviceBuffer& buf, const std::vector<cplx>& t, int real, cudaStream_t s) {
  if (real == kRealFF) {
    std::vector<float> v(4 * t.size());
    for (size_t i = 0; i < t.size(); ++i) {
      ff_pair(t[i].real(), &v[4 * i]);
      ff_pair(t[i].imag(), &v[4 * i + 2]);
    }
    upload(buf, v, s);
  } else if (real == kRealF64) {
    std::vector<double> v(2 * t.size());
    for (size_t i = 0; i < t.size(); ++i) {
      v[2 * i] = t[i].real();
      v[2 * i + 1] = t[i].imag();
    }
    upload(buf, v, s);
  } else {
    std::vector<float> v(2 * t.size());
    for (size_t i = 0; i < t.size(); ++i) {
      v[2 * i] = (float)t[i].real();
      v[2 * i + 1] = (float)t[i].imag();
    }
    upload(buf, v, s);
  }
}

const void* Engine::table_1d(const void* key, uint64_t version, const std::vector<cplx>& t) {
  auto& c = tables_[{key, 0}];
  if (c.buf.ptr && c.version == version) return c.buf.ptr;
  if (c.buf.ptr) flush();  // replacing a table the open pass may reference (a first upload needs no flush)
  upload_complex(c.buf, t, real, stream);
  c.version = version;
  return c.buf.ptr;
}

const void* Engine::table_nd(const void* key, uint64_t version, const std::vector<cplx>& t) {
  auto& c = tables_[{key, 1}];
  if (c.buf.ptr && c.version == version) return c.buf.ptr;
  if (c.buf.ptr) flush();
  // logical row-major -> storage order
  const int nd = (int)shape.size();
  std::vector<cplx> st(t.size());
  std::vector<size_t> lstride(nd);
  size_t acc = 1;
  for (int a = nd - 1; a >= 0; --a) {
    lstride[a] = acc;
    acc *= shape[a];
  }
  std::vector<size_t> idx(nd, 0);
  for (size_t s = 0; s < t.size(); ++s) {
    size_t li = 0, r = s;
    for (int q = nd - 1; q >= 0; --q) {
      const size_t ext = shape[perm[q]];
      li += (r % ext) * lstride[perm[q]];
      r /= ext;
    }
    st[s] = t[li];
  }
  upload_complex(c.buf, st, real, stream);
  c.version = version;
  return c.buf.ptr;
}

// Parity structure of a real n x n matrix (logical M[a][b] = m[a n + b]) within tol of its
// largest entry: 1 when M[a][n-1-b] = (-1)^a M[a][b] (a Legendre transform with quadrature
// weights), 2 when M[n-1-b][a] = (-1)^a M[b][a] (its inverse), else 0.
static int lane_matrix_parity(const std::vector<cplx>& m, size_t n, double rel_tol) {
  if (n < 16 || n % 2) return 0;
  double amax = 0.0;
  for (const cplx& v : m) amax = std::max(amax, std::fabs(v.real()));
  const double tol = rel_tol * amax;
  bool rowp = true, colp = true;
  for (size_t a = 0; a < n && (rowp || colp); ++a) {
    const double sg = (a & 1) ? -1.0 : 1.0;
    for (size_t b = 0; b < n; ++b) {
      if (rowp && std::fabs(m[a * n + (n - 1 - b)].real() - sg * m[a * n + b].real()) > tol) rowp = false;
      if (colp && std::fabs(m[(n - 1 - b) * n + a].real() - sg * m[b * n + a].real()) > tol) colp = false;
    }
  }
  return rowp ? 1 : (colp ? 2 : 0);
}

const void* Engine::matrices(const void* key, uint64_t version, const std::vector<cplx>& m, size_t n, size_t count,
                             bool& real, int* parity) {
  auto& c = tables_[{key, 2}];
  if (parity) *parity = 0;
  if (c.buf.ptr && c.version == version) {
    real = c.real;
    if (parity && c.parity) {
      *parity = c.parity;
      return c.half_buf.ptr;
    }
    return c.buf.ptr;
  }
  if (c.buf.ptr) flush();
  real = std::all_of(m.begin(), m.end(), [](const cplx& v) { return v.imag() == 0.0; });
  std::vector<cplx> mt(m.size());
  for (size_t b = 0; b < count; ++b)
    for (size_t j = 0; j < n; ++j)
      for (size_t k = 0; k < n; ++k) mt[b * n * n + k * n + j] = m[b * n * n + j * n + k];
  if (real) {
    if (this->real == kRealFF) {
      std::vector<float> v(2 * mt.size());
      for (size_t i = 0; i < mt.size(); ++i) ff_pair(mt[i].real(), &v[2 * i]);
      upload(c.buf, v, stream);
    } else if (fp64) {
      std::vector<double> v(mt.size());
      for (size_t i = 0; i < mt.size(); ++i) v[i] = mt[i].real();
      upload(c.buf, v, stream);
    } else {
      std::vector<float> v(mt.size());
      for (size_t i = 0; i < mt.size(); ++i) v[i] = (float)mt[i].real();
      upload(c.buf, v, stream);
    }
  } else {
    upload_complex(c.buf, mt, this->real, stream);
  }
  c.version = version;
  c.real = real;
  c.parity = 0;
  if (this->real == kRealFF && real && count == 1) {
    // float-float Legendre pairs: the half matrix of the parity form, each entry the mean of
    // the two it stands for (the structure holds to ~1e-14 of the largest entry: the nodes'
    // cosines are symmetric to an ulp), in the layout mat_apply_parity_ff reads
    const int kind = lane_matrix_parity(m, n, 1e-13);
    if (kind) {
      const size_t h = n / 2;
      std::vector<float> v(2 * n * h);
      for (size_t a = 0; a < n; ++a)
        for (size_t b = 0; b < h; ++b) {
          const double sg = (a & 1) ? -1.0 : 1.0;
          if (kind == 1) {  // H[a][b] at b n + a
            ff_pair(0.5 * (m[a * n + b].real() + sg * m[a * n + (n - 1 - b)].real()), &v[2 * (b * n + a)]);
          } else {          // H[b][a] at a h + b
            ff_pair(0.5 * (m[b * n + a].real() + sg * m[(n - 1 - b) * n + a].real()), &v[2 * (a * h + b)]);
          }
        }
      upload(c.half_buf, v, stream);
      c.parity = kind;
      if (parity) {
        *parity = kind;
        return c.half_buf.ptr;
      }
    }
  }
  if (!fp64 && tc_mode() >= 0 && real && count == 1 && (n == 32 || n == 64 || n == 128 || n == 256)) {
    std::vector<double> md(n * n);
    for (size_t i = 0; i < n * n; ++i) md[i] = m[i].real();
    int kind = 0;
    shared_tc_images(md, (int)n, tc_mode(), stream, c.tc_images, c.tc_par_images, kind);
    tc_images_by_matrix_[c.buf.ptr] = c.tc_images->as<float>();
    if (tc_mode() == 2 && (n == 32 || n == 64)) {
      // packed tiles: 128 / n copies of the matrix on the diagonal of a 128 x 128 one
      const size_t pk = 128 / n;
      std::vector<double> bd(128 * 128, 0.0);
      for (size_t b = 0; b < pk; ++b)
        for (size_t r = 0; r < n; ++r)
          for (size_t k = 0; k < n; ++k) bd[(b * n + r) * 128 + b * n + k] = md[r * n + k];
      std::shared_ptr<DeviceBuffer> none;
      int kind_bd = 0;
      shared_tc_images(bd, 128, tc_mode(), stream, c.tc_pack_images, none, kind_bd);
      tc_pack_by_matrix_[c.buf.ptr] = c.tc_pack_images->as<float>();
    }
    // the parity-split form as well, when the matrix has the structure (Legendre pairs)
    if (kind)
      tc_parity_by_matrix_[c.buf.ptr] = {kind, c.tc_par_images->as<float>()};
    else
      tc_parity_by_matrix_.erase(c.buf.ptr);
  }
  if (!fp64 && tc_mode() >= 0 && real && count > 1 && (n == 32 || n == 64 || n == 128 || n == 256)) {
    // state matrices (one per coordinate of a dependent axis): every matrix's images one
    // after another; a tensor-core tile takes the image of its coordinate
    std::vector<float> all, h;
    std::vector<double> md(n * n);
    int64_t stride = 0;
    for (size_t b = 0; b < count; ++b) {
      for (size_t i = 0; i < n * n; ++i) md[i] = m[b * n * n + i].real();
      angular_tc_images(md.data(), (int)n, tc_mode(), h);
      stride = (int64_t)h.size();
      all.insert(all.end(), h.begin(), h.end());
    }
    upload(c.tc_slice_images, all, stream);
    tc_slice_by_matrix_[c.buf.ptr] = {c.tc_slice_images.as<float>(), stride};
  } else {
    tc_slice_by_matrix_.erase(c.buf.ptr);
  }
  return c.buf.ptr;
}

// Process-wide cache of tensor-core A images by matrix value: every propagation on the same
// polar grid has the same Legendre pair, so a batch of hundreds of propagations streams a
// few images (which stay in L2) instead of one copy per propagation.  Entries are held
// weakly: an image lives as long as an engine uses it.
namespace {
struct ImageEntry {
  int device, n, mode, kind;
  std::vector<double> m;
  std::weak_ptr<DeviceBuffer> img, par;
};
std::mutex g_images_mu;
std::vector<ImageEntry> g_images;
}  // namespace

void Engine::shared_tc_images(const std::vector<double>& md, int n, int mode, cudaStream_t s,
                              std::shared_ptr<DeviceBuffer>& img, std::shared_ptr<DeviceBuffer>& par, int& kind) {
  int dev = 0;
  cuda_check(cudaGetDevice(&dev), "cudaGetDevice");
  std::lock_guard<std::mutex> lock(g_images_mu);
  g_images.erase(std::remove_if(g_images.begin(), g_images.end(), [](const ImageEntry& e) { return e.img.expired(); }),
                 g_images.end());
  for (const ImageEntry& e : g_images)
    if (e.device == dev && e.n == n && e.mode == mode && e.m == md) {
      img = e.img.lock();
      par = e.par.lock();
      if (img && (e.kind == 0 || par)) {
        kind = e.kind;
        return;
      }
    }
  std::vector<float> h;
  angular_tc_images(md.data(), n, mode, h);
  img = std::make_shared<DeviceBuffer>();
  upload(*img, h, s);
  kind = angular_tc_parity(md.data(), n);
  par.reset();
  if (kind) {
    angular_tc_parity_images(md.data(), n, kind, mode, h);
    par = std::make_shared<DeviceBuffer>();
    upload(*par, h, s);
  }
  g_images.push_back(ImageEntry{dev, n, mode, kind, md, img, par});
}

bool Engine::try_launch_tc(const std::vector<DevOp>& ops, int axis, PassParams& p) {
  Geometry g = geometry(axis, false);
  if (!angular_tc_eligible(g)) return false;
  int mats[2], nmat = 0;
  const float* images[2] = {nullptr, nullptr};
  int slice_axis[2] = {-1, -1};
  int64_t slice_stride[2] = {0, 0};
  bool sliced = false;
  const int bn0 = angular_tc_columns((int)g.n);
  for (size_t i = 0; i < ops.size(); ++i) {
    const int k = ops[i].kind;
    if (k == OP_FFT || k == OP_MAT_LANE || k == OP_DOT) return false;
    if (k == OP_MAT) {
      if (nmat == 2 || !(ops[i].flags & 1)) return false;
      auto it = tc_images_by_matrix_.find(ops[i].ptr);
      if (it == tc_images_by_matrix_.end()) return false;
      images[nmat] = it->second;
      mats[nmat++] = (int)i;
    } else if (k == OP_MAT_SLICE) {
      // a state matrix: one matrix per coordinate of the dependent axis, which must be
      // constant over every tile (an outer axis, or an inner one whose stride is a multiple
      // of the tile's columns), with a matrix for every coordinate
      if (nmat == 2 || !(ops[i].flags & 1)) return false;
      auto it = tc_slice_by_matrix_.find(ops[i].ptr);
      if (it == tc_slice_by_matrix_.end()) return false;
      const int dep = ops[i].axis;
      int q = -1;
      for (int a = 0; a < g.ndim; ++a)
        if (g.perm[a] == dep) q = a;
      if (q < 0 || q == g.spos || ops[i].count < g.sshape[q]) return false;
      if (q > g.spos) {
        int64_t stride = 1;
        for (int a = q + 1; a < g.ndim; ++a) stride *= g.sshape[a];
        if (stride % bn0 != 0) return false;
      }
      images[nmat] = it->second.first;
      slice_axis[nmat] = dep;
      slice_stride[nmat] = it->second.second;
      sliced = true;
      mats[nmat++] = (int)i;
    }
  }
  if (nmat == 0 || !angular_tc_ops_fit(ops.data(), (int)ops.size(), g.sweep_axis)) return false;
  // parity-split GEMMs when every matrix of the pass has the structure and no sum /
  // difference matrix follows anything but an even / odd one (SO_TC_PARITY=0 turns it off)
  int parity[2] = {0, 0};
  const char* par_env = std::getenv("SO_TC_PARITY");
  bool par = g.n == 256 && !sliced && !(par_env && par_env[0] == '0');
  for (int m = 0; m < nmat && par; ++m) {
    auto it = tc_parity_by_matrix_.find(ops[mats[m]].ptr);
    if (it == tc_parity_by_matrix_.end()) {
      par = false;
      break;
    }
    parity[m] = it->second.first;
    if (m > 0 && parity[m] == 1 && parity[m - 1] != 2) par = false;
  }
  if (par) {
    for (int m = 0; m < nmat; ++m) images[m] = tc_parity_by_matrix_[ops[mats[m]].ptr].second;
  } else {
    parity[0] = parity[1] = 0;
  }
  // packed tiles for short lanes: 128 / n column groups per tile, block-diagonal images
  int pk = par || sliced ? 1 : angular_tc_pack(g, ops.data(), (int)ops.size(), tc_mode());
  if (pk > 1) {
    const float* pim[2] = {nullptr, nullptr};
    for (int m = 0; m < nmat && pk > 1; ++m) {
      auto it = tc_pack_by_matrix_.find(ops[mats[m]].ptr);
      if (it == tc_pack_by_matrix_.end())
        pk = 1;
      else
        pim[m] = it->second;
    }
    if (pk > 1)
      for (int m = 0; m < nmat; ++m) images[m] = pim[m];
  }
  const int bn = angular_tc_columns((int)g.n) * pk;
  g.lanes_per_tile = bn;
  g.tiles_per_outer = (int32_t)(g.inner / bn);
  g.tiles = g.outer * g.tiles_per_outer;
  p.g = g;
  if ((size_t)g.tiles > partials_cap_) {
    partials_cap_ = (size_t)g.tiles;
    partials_ = DeviceBuffer(partials_cap_ * kMaxRed * sizeof(double));
    p.partials = partials_.as<double>();
  }
  static const char* const kTcNames[3] = {"f32 tc3xtf32", "f32 tcbf16x3", "f32 tcbf16x6"};
  std::string name = std::string(kTcNames[tc_mode()]) + (par ? " parity axis" : (pk > 1 ? " packed axis" : " axis")) +
                     std::to_string(axis) + ":";
  for (const DevOp& o : ops) name += std::string(" ") + op_kind_name(o.kind);
  const TcSchedule sched = tc_schedule(g.n, tc_mode());
  if (recording) {
    // threads: the lane extent, the parity mode, the operand format and the schedule (CTAs per
    // SM, tile order): one batched launch serves one of each; the kernel's thread count is fixed
    RecordedPass r{RecordedPass::TensorCore, false, p, std::vector<unsigned char>(tc_params_bytes()),
                   (int)g.n | (par ? 1 << 16 : 0) | (tc_mode() << 17) | ((sched.ctas_per_sm & 3) << 20) |
                       (sched.blocked ? 1 << 22 : 0) | ((pk == 4 ? 2 : pk == 2 ? 1 : 0) << 23),
                   angular_tc_smem_bytes((int)g.n * pk, par, tc_mode()), name, pass_bytes(ops, g)};
    make_tc_params(p, mats, nmat, images, timeout_slot, parity, r.tcp.data(), pk, slice_axis, slice_stride);
    recording->push_back(std::move(r));
    return true;
  }
  if (timing) {
    timed_begin(name);
    timed_.back().bytes = pass_bytes(ops, g);
  }
  // SO_TC_TRACE=<file>: per-tile phase timestamps of every tensor-core pass, appended as text
  static const char* trace_path = std::getenv("SO_TC_TRACE");
  DeviceBuffer trace;
  if (trace_path) {
    trace = DeviceBuffer((size_t)g.tiles * angular_tc_trace_slots() * sizeof(unsigned long long));
    cuda_check(cudaMemsetAsync(trace.ptr, 0, trace.bytes, stream), "trace clear");
  }
  cuda_check(launch_angular_tc(p, mats, nmat, images, timeout_slot, parity, tc_mode(), stream,
                               trace_path ? trace.as<unsigned long long>() : nullptr, sched.ctas_per_sm, pk,
                               slice_axis, slice_stride),
             "tensor-core pass launch");
  if (trace_path) {
    std::vector<unsigned long long> h(trace.bytes / sizeof(unsigned long long));
    cuda_check(cudaMemcpyAsync(h.data(), trace.ptr, trace.bytes, cudaMemcpyDeviceToHost, stream), "trace copy");
    cuda_check(cudaStreamSynchronize(stream), "trace sync");
    if (FILE* f = std::fopen(trace_path, "a")) {
      std::fprintf(f, "pass %s n=%lld tiles=%lld slots=%d\n", name.c_str(), (long long)g.n, (long long)g.tiles,
                   angular_tc_trace_slots());
      for (size_t i = 0; i < h.size(); ++i)
        std::fprintf(f, "%llu%c", h[i], (i + 1) % angular_tc_trace_slots() == 0 ? '\n' : ' ');
      std::fclose(f);
    }
  }
  if (timing) timed_end();
  return true;
}

const double* Engine::weights(const Grid& g) {
  auto it = weights_.find(g.uid);
  if (it != weights_.end()) return it->second.as<double>();
  // n FP64 weights followed by their FP32 roundings (read by the FP32 passes, which
  // keep FP64 arithmetic out of their per-point work)
  const size_t n = g.weights.size();
  std::vector<double> packed(n + (n + 1) / 2, 0.0);
  std::copy(g.weights.begin(), g.weights.end(), packed.begin());
  float* f = reinterpret_cast<float*>(packed.data() + n);
  for (size_t i = 0; i < n; ++i) f[i] = (float)g.weights[i];
  DeviceBuffer b;
  upload(b, packed, stream);
  const double* p = b.as<double>();
  weights_.emplace(g.uid, std::move(b));
  return p;
}

void WaveFunction::set_weights(DevOp& op) {
  for (size_t a = 0; a < grids.size(); ++a) {
    op.w[a] = eng->weights(grids[a]);
    op.wf[a] = reinterpret_cast<const float*>(op.w[a] + grids[a].weights.size());
  }
}

const void* Engine::twiddle(size_t n, int radix) {
  const int rmax = radix ? radix : (fp64 ? 8 : 16);
  auto it = twiddles_.find({n, rmax});
  if (it != twiddles_.end()) return it->second.ptr;
  DeviceBuffer b;
  std::vector<cplx> tw = twiddles(n);
  if (stage_twiddles((int64_t)n)) {
    // the Stockham stages' order (same values, permuted): forward radix order in [0, n),
    // reversed radix order (the FFT pair pass's second transform) in [n, 2n)
    std::vector<cplx> st(2 * n, cplx(0.0, 0.0));
    for (size_t e = 0; e < n; ++e) {
      st[e] = tw[(size_t)stage_twiddle_exponent((int64_t)e, (int64_t)n, rmax, false)];
      st[n + e] = tw[(size_t)stage_twiddle_exponent((int64_t)e, (int64_t)n, rmax, true)];
    }
    tw.swap(st);
  }
  upload_complex(b, tw, real, stream);
  const void* p = b.ptr;
  twiddles_.emplace(std::make_pair(n, rmax), std::move(b));
  return p;
}

void Engine::submit(const Action& a) {
  const int k = a.op.kind;
  if (a.lane_axis >= 0 && cur_axis_ >= 0 && cur_axis_ != a.lane_axis) flush();
  if (k == OP_SCALE) {
    for (int w : cur_written_)
      if (w == a.op.b || w == a.op.c) {
        flush();
        break;
      }
  }
  const int need = k == OP_NORM ? 1 : (k == OP_DOT ? 2 : 0);
  if ((int)cur_.size() >= kMaxOps || cur_red_ + need > kMaxRed) flush();
  if (k == OP_MAT && tc_mode() >= 0) {
    // the tensor-core pass holds at most two lane-matrix products
    int mats = 0;
    for (const DevOp& o : cur_) mats += o.kind == OP_MAT;
    if (mats >= 2) flush();
  }
  if (a.lane_axis >= 0) cur_axis_ = a.lane_axis;
  DevOp op = a.op;
  if (need) {
    op.red = cur_red_;
    cur_red_ += need;
  }
  if (k == OP_NORM || k == OP_COPY || k == OP_LOSS || k == OP_SETC) cur_written_.push_back(op.a);
  if (k == OP_DOT) {
    cur_written_.push_back(op.a);
    cur_written_.push_back(op.b);
  }
  cur_.push_back(op);
}

void Engine::launch(const std::vector<DevOp>& ops, int axis, bool resident, int repeat) {
  PassParams p{};
  const char* name_tag = "";
  p.g = geometry(axis, resident);
  p.psi = psi.ptr;
  p.slots = slots();
  p.partials = partials_.as<double>();
  p.counter = counter_.as<unsigned int>();
  p.record = record_dev;
  p.nops = (int)ops.size();
  p.repeat = repeat;
  p.resident = resident ? 1 : 0;
  p.nonfinite_slot = nonfinite_slot;
  int nred = 0;
  bool fft = false;
  for (size_t i = 0; i < ops.size(); ++i) {
    p.ops[i] = ops[i];
    if (ops[i].kind == OP_NORM) nred = std::max(nred, ops[i].red + 1);
    if (ops[i].kind == OP_DOT) nred = std::max(nred, ops[i].red + 2);
    if (ops[i].kind == OP_FFT) fft = true;
  }
  p.nred = nred;
  if (fft) p.twiddle = twiddle((size_t)p.g.n);
  pass_choose_buffers(p, fp64);
  if (!fp64 && tc_mode() >= 0 && !resident && try_launch_tc(ops, axis, p)) return;
  if ((fft_pair || (fp64 && p.g.n > 4096)) && fft_pair_plan(p, real, resident)) {
    name_tag = p.radix == 8 && !fp64 ? " fftpair r8" : " fftpair";
    if (p.radix != (fp64 ? 8 : 16)) p.twiddle = twiddle((size_t)p.g.n, p.radix);  // the table in its stage order
    p.ct = fft_pair_ct ? fft_pair_ct_lgn(p, fp64) : 0;
    if (p.ct) name_tag = " fftpair ct";
  }
  if (fp64 && p.g.n > 4096 && !p.fused)
    throw Error(SO_ERR_UNSUPPORTED, "FP64 lanes longer than 4096 points are not supported outside FFT-pair passes "
                                    "([FFT] [point-wise] [FFT] [point-wise] on contiguous power-of-two lanes)");
  if (!resident && (size_t)p.g.tiles > partials_cap_) {
    partials_cap_ = (size_t)p.g.tiles;
    partials_ = DeviceBuffer(partials_cap_ * kMaxRed * sizeof(double));
    p.partials = partials_.as<double>();
  }
  std::string name = std::string(real == kRealFF ? "ff" : (fp64 ? "f64" : "f32")) + (resident ? " resident" : " sweep") +
                     name_tag + " axis" +
                     std::to_string(axis) + ":";
  for (const DevOp& o : ops) name += std::string(" ") + op_kind_name(o.kind);
  if (recording) {
    // fused FFT pairs: bit 16 of the thread count (their own launch group and kernel)
    // radix-8 FP32 pairs: bit 19 (their own kernel); fixed-shape FP32 pairs: bit 20
    const int threads = p.fused ? (fft_pair_block(p.g) | (1 << 16) | (p.radix == 8 && !fp64 ? 1 << 19 : 0) |
                                   (p.ct ? 1 << 20 : 0))
                                : pass_threads(p.g);
    RecordedPass r{resident ? RecordedPass::Resident : RecordedPass::Generic, real, p, {},
                   threads, pass_smem_bytes(p, fp64), name, pass_bytes(ops, p.g)};
    recording->push_back(std::move(r));
    return;
  }
  if (timing) {
    timed_begin(name);
    timed_.back().bytes = pass_bytes(ops, p.g);
  }
  cuda_check(real == kRealFF ? launch_pass_ff(p, stream) : (fp64 ? launch_pass_f64(p, stream) : launch_pass_f32(p, stream)),
             "pass launch");
  if (timing) timed_end();
}

cudaEvent_t Engine::take_event() {
  if (!event_pool_.empty()) {
    cudaEvent_t e = event_pool_.back();
    event_pool_.pop_back();
    return e;
  }
  cudaEvent_t e;
  cuda_check(cudaEventCreate(&e), "event create");
  return e;
}

void Engine::timed_begin(const std::string& name) {
  TimedLaunch t{name, take_event(), take_event(), 0.0};
  cuda_check(cudaEventRecord(t.a, stream), "event record");
  timed_.push_back(t);
}

void Engine::timed_end() { cuda_check(cudaEventRecord(timed_.back().b, stream), "event record"); }

double Engine::pass_bytes(const std::vector<DevOp>& ops, const Geometry& g) const {
  // algorithmic bytes: read + write of the state, plus each distinct full-size table the
  // pass streams, once (a table applied twice in one pass -- the V/2 phase at the end of
  // one step and the start of the next -- is read once)
  double pts = 1.0;
  for (int q = 0; q < g.ndim; ++q) pts *= (double)g.sshape[q];
  double b = 2.0 * pts * (double)elem_bytes();
  std::vector<const void*> seen;
  for (const DevOp& o : ops)
    if ((o.kind == OP_DIAGND || o.kind == OP_DOT) && std::find(seen.begin(), seen.end(), o.ptr) == seen.end()) {
      seen.push_back(o.ptr);
      b += pts * (double)elem_bytes();
    }
  return b;
}

std::string Engine::collect_timing() {
  flush();
  cuda_check(cudaStreamSynchronize(stream), "stream sync");
  struct Acc {
    int n = 0;
    double ms = 0.0, bytes = 0.0;
  };
  std::map<std::string, Acc> acc;
  std::vector<std::string> order;
  for (TimedLaunch& t : timed_) {
    float ms = 0.f;
    cuda_check(cudaEventElapsedTime(&ms, t.a, t.b), "event elapsed");
    if (!acc.count(t.name)) order.push_back(t.name);
    Acc& a = acc[t.name];
    a.n += 1;
    a.ms += ms;
    a.bytes += t.bytes;
    event_pool_.push_back(t.a);
    event_pool_.push_back(t.b);
  }
  timed_.clear();
  std::string out;
  for (const std::string& k : order) {
    const Acc& a = acc[k];
    out += k + "\t" + std::to_string(a.n) + "\t" + std::to_string(a.ms) + "\t" + std::to_string(a.bytes) + "\n";
  }
  return out;
}

void Engine::flush() {
  if (cur_.empty()) return;
  std::vector<DevOp> ops;
  ops.swap(cur_);
  const int axis = cur_axis_ >= 0 ? cur_axis_ : perm.back();
  cur_axis_ = -1;
  cur_red_ = 0;
  cur_written_.clear();
  const bool array = std::any_of(ops.begin(), ops.end(), [](const DevOp& o) { return !is_scalar_kind(o.kind); });
  if (!array) {
    PassParams p{};
    p.slots = slots();
    p.record = record_dev;
    p.nops = (int)ops.size();
    for (size_t i = 0; i < ops.size(); ++i) p.ops[i] = ops[i];
    if (recording) {
      recording->push_back(RecordedPass{RecordedPass::Scalar, real, p, {}, 32, 0, "scalar", 0.0});
      return;
    }
    cuda_check(launch_scalar_program(p, stream), "scalar launch");
    return;
  }
  launch(ops, axis, false, 1);
}

void Engine::run_resident(const std::vector<Action>& prog, int repeat) {
  flush();
  if (prog.empty() || repeat <= 0) return;
  std::vector<DevOp> ops;
  int red = 0;
  for (const Action& a : prog) {
    DevOp op = a.op;
    if (op.kind == OP_NORM || op.kind == OP_DOT) op.red = 0;
    ops.push_back(op);
    (void)red;
  }
  const int axis = perm.back();
  if ((int)ops.size() <= kMaxOps) {
    launch(ops, axis, true, repeat);
    return;
  }
  for (int r = 0; r < repeat; ++r)
    for (size_t s = 0; s < ops.size(); s += kMaxOps) {
      std::vector<DevOp> chunk(ops.begin() + s, ops.begin() + std::min(ops.size(), s + (size_t)kMaxOps));
      launch(chunk, axis, true, 1);
    }
}

void Engine::sync() {
  flush();
  cuda_check(cudaStreamSynchronize(stream), "stream sync");
}

void Engine::check_nonfinite() {
  if (read_slot(timeout_slot) != 0.0) {
    write_slot(timeout_slot, 0.0);
    throw Error(SO_ERR_TIMEOUT, "a bounded device-side wait gave up (tensor-core pass)");
  }
  if (read_slot(nonfinite_slot) != 0.0) {
    write_slot(nonfinite_slot, 0.0);
    throw Error(SO_ERR_NONFINITE, "a norm of the wave function is not finite");
  }
}

static Geometry flat_geometry(const Engine& e) {
  Geometry g{};
  g.ndim = (int)e.shape.size();
  for (int q = 0; q < g.ndim; ++q) {
    g.perm[q] = e.perm[q];
    g.sshape[q] = (int64_t)e.shape[e.perm[q]];
  }
  return g;
}

static bool identity_perm(const std::vector<int>& p) {
  for (size_t i = 0; i < p.size(); ++i)
    if (p[i] != (int)i) return false;
  return true;
}

// Device address of a page-locked, mapped host range (nullptr for pageable memory or a
// range that leaves the mapped allocation): kernels read and write such buffers directly
// over the host link, with no staging copy in device memory.
static char* mapped_range(const void* host, size_t bytes) {
  auto dev = [](const void* p) -> char* {
    cudaPointerAttributes at{};
    if (cudaPointerGetAttributes(&at, p) != cudaSuccess) {
      cudaGetLastError();  // clear the error of an unknown pointer
      return nullptr;
    }
    return at.type == cudaMemoryTypeHost ? static_cast<char*>(at.devicePointer) : nullptr;
  };
  if (bytes == 0) return nullptr;
  char* d0 = dev(host);
  char* d1 = d0 ? dev(static_cast<const char*>(host) + bytes - 1) : nullptr;
  return d0 && d1 == d0 + bytes - 1 ? d0 : nullptr;
}

void Engine::import_host(const double* host, bool copy_engine) {
  flush();
  const size_t b = points() * 16;
  const Geometry g = flat_geometry(*this);
  if (real == kRealF64 && identity_perm(perm)) {
    cuda_check(cudaMemcpyAsync(psi.ptr, host, b, cudaMemcpyHostToDevice, stream), "import copy");
    return;
  }
  if (!copy_engine && (identity_perm(perm) || layout_is_transpose2(g))) {
    if (const char* d = mapped_range(host, b)) {
      cuda_check(launch_import(psi.ptr, real, reinterpret_cast<const double*>(d), g, stream), "import");
      return;
    }
  }
  if (staging_.bytes < b) staging_ = DeviceBuffer(b);
  cuda_check(cudaMemcpyAsync(staging_.ptr, host, b, cudaMemcpyHostToDevice, stream), "import copy");
  cuda_check(launch_import(psi.ptr, real, staging_.as<double>(), g, stream), "import");
}

void Engine::export_host(double* host, bool sync, bool copy_engine) {
  flush();
  const size_t b = points() * 16;
  const Geometry g = flat_geometry(*this);
  char* d = nullptr;
  if (real == kRealF64 && identity_perm(perm)) {
    cuda_check(cudaMemcpyAsync(host, psi.ptr, b, cudaMemcpyDeviceToHost, stream), "export copy");
  } else if (!copy_engine && (identity_perm(perm) || layout_is_transpose2(g)) &&
             (d = mapped_range(host, b)) != nullptr) {
    cuda_check(launch_export(reinterpret_cast<double*>(d), psi.ptr, real, g, stream), "export");
  } else {
    if (staging_.bytes < b) staging_ = DeviceBuffer(b);
    cuda_check(launch_export(staging_.as<double>(), psi.ptr, real, g, stream), "export");
    cuda_check(cudaMemcpyAsync(host, staging_.ptr, b, cudaMemcpyDeviceToHost, stream), "export copy");
  }
  if (sync) cuda_check(cudaStreamSynchronize(stream), "export sync");
}

// The two halves of a staged copy-engine import / export, for callers that order the
// copies (copy engines) and the layout kernels (SMs) separately.
void Engine::stage_in(const double* host) {
  flush();
  const size_t b = points() * 16;
  if (real == kRealF64 && identity_perm(perm)) {
    cuda_check(cudaMemcpyAsync(psi.ptr, host, b, cudaMemcpyHostToDevice, stream), "import copy");
    return;
  }
  if (staging_.bytes < b) staging_ = DeviceBuffer(b);
  cuda_check(cudaMemcpyAsync(staging_.ptr, host, b, cudaMemcpyHostToDevice, stream), "import copy");
}

void Engine::unstage_in() {
  if (real == kRealF64 && identity_perm(perm)) return;
  cuda_check(launch_import(psi.ptr, real, staging_.as<double>(), flat_geometry(*this), stream), "import");
}

void Engine::stage_out() {
  flush();
  if (real == kRealF64 && identity_perm(perm)) return;
  const size_t b = points() * 16;
  if (staging_.bytes < b) staging_ = DeviceBuffer(b);
  cuda_check(launch_export(staging_.as<double>(), psi.ptr, real, flat_geometry(*this), stream), "export");
}

void Engine::import_device(const double* dev) {
  flush();
  cuda_check(launch_import(psi.ptr, real, dev, flat_geometry(*this), stream), "import");
}

void Engine::export_device(double* dev) {
  flush();
  cuda_check(launch_export(dev, psi.ptr, real, flat_geometry(*this), stream), "export");
}

void Engine::unstage_out(double* host) {
  const size_t b = points() * 16;
  const void* src = (real == kRealF64 && identity_perm(perm)) ? psi.ptr : staging_.ptr;
  cuda_check(cudaMemcpyAsync(host, src, b, cudaMemcpyDeviceToHost, stream), "export copy");
}

// ----------------------------------------------------------------- WaveFunction
WaveFunction::WaveFunction(const std::vector<size_t>& shp, const std::vector<Grid>& g, const std::vector<int>& perm,
                           int real)
    : shape(shp), grids(g) {
  if (grids.size() != shape.size()) throw Error(SO_ERR_SHAPE, "one grid per axis is required");
  for (size_t a = 0; a < shape.size(); ++a)
    if (grids[a].size() != shape[a]) throw Error(SO_ERR_SHAPE, "grid size differs from the array axis");
  for (const Grid& gr : grids) last_grid_names.push_back(gr.name);
  eng = std::make_unique<Engine>(shape, perm, real);
  cache_slot = eng->alloc_slot(1.0);
}

size_t WaveFunction::points() const { return eng->points(); }

std::vector<const double*> WaveFunction::weight_ptrs() {
  std::vector<const double*> w;
  for (const Grid& g : grids) w.push_back(eng->weights(g));
  return w;
}

void Emitter::host(std::function<void()> f) {
  if (rec) {
    Action a{};
    a.host_call = (int)calls->size();
    calls->push_back(std::move(f));
    rec->push_back(a);
  } else {
    eng->flush();
    f();
  }
}

int norm_slot(WaveFunction& wf, Emitter& em) {
  if (!wf.possible_norm_change) return wf.cache_slot;
  bool changed = false;
  for (size_t a = 0; a < wf.grids.size(); ++a)
    if (wf.last_grid_names[a] != wf.grids[a].name) changed = true;
  if (changed)
    for (size_t a = 0; a < wf.grids.size(); ++a) wf.last_grid_names[a] = wf.grids[a].name;
  Action act{};
  act.op.kind = OP_NORM;
  act.op.a = wf.cache_slot;
  wf.set_weights(act.op);
  em.emit(act);
  wf.possible_norm_change = false;
  return wf.cache_slot;
}

void normalize_to_slot(WaveFunction& wf, Emitter& em, int target) {
  const int n = norm_slot(wf, em);
  Action s{};
  s.op.kind = OP_SCALE;
  s.op.b = target;
  s.op.c = n;
  em.emit(s);
  if (target != wf.cache_slot) {
    Action c{};
    c.op.kind = OP_COPY;
    c.op.a = wf.cache_slot;
    c.op.b = target;
    em.emit(c);
  }
  wf.possible_norm_change = false;
}

static Action scalar_action(int kind, int a, int b = 0, int c = 0, double value = 0.0) {
  Action act{};
  act.op.kind = kind;
  act.op.a = a;
  act.op.b = b;
  act.op.c = c;
  act.op.value = value;
  return act;
}

// -------------------------------------------------------------------- LossChecker
void LossChecker::check_before(WaveFunction& wf, Emitter& em) {
  const int n = norm_slot(wf, em);
  const auto& s = st.bind(wf.eng.get());
  em.emit(scalar_action(OP_COPY, s[1], n));
}

void LossChecker::check_after(WaveFunction& wf, Emitter& em) {
  const int n = norm_slot(wf, em);
  const auto& s = st.bind(wf.eng.get());
  em.emit(scalar_action(OP_LOSS, s[0], s[1], n));
  em.emit(scalar_action(OP_COPY, s[1], n));
}

void LossChecker::reset(Emitter* em) {
  if (em && st.home == em->eng)
    em->emit(scalar_action(OP_SETC, st.slots[0], 0, 0, 0.0));
  else
    st.set(0, 0.0);
}

// -------------------------------------------------------------------- propagators
void OneDimPropagator::apply_unchecked(WaveFunction& wf, Emitter& em) {
  if (dimension_no >= wf.shape.size() || op.size() != wf.shape[dimension_no])
    throw Error(SO_ERR_SHAPE, "one-dimensional operator does not match the wave function axis");
  wf.possible_norm_change = true;
  Action a{};
  a.op.kind = OP_DIAG1D;
  a.op.axis = (int)dimension_no;
  a.op.ptr = wf.eng->table_1d(this, version, op);
  em.emit(a);
}

void OneDimPropagator::apply(WaveFunction& wf, Emitter& em) {
  if (lc) lc->check_before(wf, em);
  apply_unchecked(wf, em);
  if (lc) lc->check_after(wf, em);
}

void NDimPropagator::apply(WaveFunction& wf, Emitter& em) {
  if (shape != wf.shape) throw Error(SO_ERR_SHAPE, "n-dimensional operator shape differs from the wave function");
  if (lc) lc->check_before(wf, em);
  wf.possible_norm_change = true;
  Action a{};
  a.op.kind = OP_DIAGND;
  a.op.ptr = wf.eng->table_nd(this, version, op);
  em.emit(a);
  if (lc) lc->check_after(wf, em);
}

void NonDiagPropagator::apply(WaveFunction& wf, Emitter& em) {
  if (dimension_no >= wf.shape.size() || n != wf.shape[dimension_no])
    throw Error(SO_ERR_SHAPE, "non-diagonal operator size differs from the wave function axis");
  if (lc) lc->check_before(wf, em);
  wf.possible_norm_change = true;
  Action a{};
  bool real = false;
  a.op.kind = OP_MAT_LANE;
  a.op.ptr = wf.eng->matrices(this, version, ops, n, count, real);
  a.op.flags = real ? 1 : 0;
  a.op.count = (int64_t)count;
  a.lane_axis = (int)dimension_no;
  em.emit(a);
  if (lc) lc->check_after(wf, em);
}

// ---------------------------------------------------------------- transformations
FFTTransformation::FFTTransformation(const Grid& g, const std::string& name)
    : Operator(OpClass::Transformation, "FFTTransformation"),
      dimension_no(g.dimension_no),
      dimension_size(g.size()),
      grid_trans(fft_momentum_grid(g, name)) {}

static void swap_grid(WaveFunction& wf, size_t dim, Grid& other) {
  if (dim >= wf.grids.size()) throw Error(SO_ERR_SHAPE, "transformation axis out of range");
  std::swap(wf.grids[dim], other);
  wf.possible_norm_change = true;
}

static void emit_fft(WaveFunction& wf, Emitter& em, size_t dim, size_t n, int dir) {
  if (dim >= wf.shape.size() || wf.shape[dim] != n) throw Error(SO_ERR_SHAPE, "FFT size differs from the axis");
  Action a{};
  a.op.kind = OP_FFT;
  a.op.dir = dir;
  a.lane_axis = (int)dim;
  em.emit(a);
}

void FFTTransformation::transform(WaveFunction& wf, Emitter& em) {
  swap_grid(wf, dimension_no, grid_trans);
  emit_fft(wf, em, dimension_no, dimension_size, -1);
}

void FFTTransformation::inverse_transform(WaveFunction& wf, Emitter& em) {
  swap_grid(wf, dimension_no, grid_trans);
  emit_fft(wf, em, dimension_no, dimension_size, +1);
}

MatrixTransformation::MatrixTransformation(const Grid& g, const Grid& gt)
    : Operator(OpClass::Transformation, "MatrixTransformation"),
      dimension_no(g.dimension_no),
      dimension_size(g.size()),
      t(g.size() * g.size(), cplx(0, 0)),
      tinv(g.size() * g.size(), cplx(0, 0)),
      grid_trans(gt) {}

static void emit_mat(WaveFunction& wf, Emitter& em, const void* key, uint64_t version, const std::vector<cplx>& m,
                     size_t dim, size_t n) {
  if (dim >= wf.shape.size() || wf.shape[dim] != n) throw Error(SO_ERR_SHAPE, "matrix size differs from the axis");
  Action a{};
  bool real = false;
  int parity = 0;
  a.op.kind = OP_MAT;
  a.op.ptr = wf.eng->matrices(key, version, m, n, 1, real, &parity);
  a.op.flags = (real ? 1 : 0) | (parity << 1);
  a.lane_axis = (int)dim;
  em.emit(a);
}

void MatrixTransformation::transform(WaveFunction& wf, Emitter& em) {
  swap_grid(wf, dimension_no, grid_trans);
  emit_mat(wf, em, &t, version, t, dimension_no, dimension_size);
}

void MatrixTransformation::inverse_transform(WaveFunction& wf, Emitter& em) {
  swap_grid(wf, dimension_no, grid_trans);
  emit_mat(wf, em, &tinv, version, tinv, dimension_no, dimension_size);
}

StateMatrixTransformation::StateMatrixTransformation(size_t dep, const Grid& g, const Grid& gt)
    : Operator(OpClass::Transformation, "StateMatrixTransformation"),
      dimension_no(g.dimension_no),
      dependent(dep),
      n(g.size()),
      grid_trans(gt) {
  if (dep <= g.dimension_no) throw Error(SO_ERR_INVALID, "Dependent dimension should have higher dimension index");
}

static void emit_state_mat(WaveFunction& wf, Emitter& em, const void* key, uint64_t version,
                           const std::vector<cplx>& m, size_t count, size_t dim, size_t dep, size_t n) {
  if (dim >= wf.shape.size() || dep >= wf.shape.size() || wf.shape[dim] != n)
    throw Error(SO_ERR_SHAPE, "state matrix size differs from the axis");
  Action a{};
  bool real = false;
  a.op.kind = OP_MAT_SLICE;
  a.op.ptr = count ? wf.eng->matrices(key, version, m, n, count, real) : nullptr;
  a.op.flags = real ? 1 : 0;
  a.op.axis = (int)dep;
  a.op.count = (int64_t)count;
  a.lane_axis = (int)dim;
  em.emit(a);
}

void StateMatrixTransformation::transform(WaveFunction& wf, Emitter& em) {
  swap_grid(wf, dimension_no, grid_trans);
  emit_state_mat(wf, em, &ts, version, ts, count, dimension_no, dependent, n);
}

void StateMatrixTransformation::inverse_transform(WaveFunction& wf, Emitter& em) {
  swap_grid(wf, dimension_no, grid_trans);
  emit_state_mat(wf, em, &tinvs, version, tinvs, count, dimension_no, dependent, n);
}

// ------------------------------------------------------------------------ controls
void LeakControl::first_half(WaveFunction& wf, Emitter& em) {
  const int n = norm_slot(wf, em);
  const auto& s = st.bind(wf.eng.get());
  em.emit(scalar_action(OP_COPY, s[0], n));
  if (lc) lc->check_before(wf, em);
}

void LeakControl::second_half(WaveFunction& wf, Emitter& em) {
  if (lc) lc->check_after(wf, em);
  const auto& s = st.bind(wf.eng.get());
  normalize_to_slot(wf, em, s[0]);
}

BorderDumping::BorderDumping(const std::vector<cplx>& mask, const Grid& g)
    : Operator(OpClass::Control, "BorderDumping"), op(mask.size(), g.dimension_no) {
  op.op = mask;
}

void BorderDumping::half(WaveFunction& wf, Emitter& em) {
  if (lc) lc->check_before(wf, em);
  op.apply(wf, em);
  if (lc) lc->check_after(wf, em);
}

// -------------------------------------------------------------------------- savers
StateSaver::StateSaver(const std::string& name, so_time_grid t, const Grid& a, const Grid* b, size_t frames)
    : Operator(OpClass::Saver, b ? "WaveFunctionSaver" : "StateSaver"),
      two_d(b != nullptr),
      fname(name),
      time(t),
      grid_a(a),
      frames_no(frames) {
  if (b) grid_b = *b;
  if (frames_no == 0 || frames_no > time.step_no)
    throw Error(SO_ERR_INVALID, "frames_no must be between 1 and step_no (the reference divides step_no by it)");
  points = two_d ? grid_a.size() * grid_b.size() : grid_a.size();
  data.assign(points * frames_no, 0.0);
}

void StateSaver::monitor(WaveFunction& wf, Emitter& em) {
  if (two_d && wf.shape.size() != 2) throw Error(SO_ERR_STATE, "Wave function must be 2d for now");
  const size_t freq = time.step_no / frames_no;
  if (current_frame % freq == 0 && current_frame / freq < frames_no) {
    const size_t frame = current_frame / freq;
    times.push_back(time.step * ((double)current_frame + 1.0));
    WaveFunction* w = &wf;
    em.host([this, w, frame]() { record_frame(*w, frame); });
  }
  current_frame += 1;
}

void StateSaver::record_frame(WaveFunction& wf, size_t frame) {
  Engine& e = *wf.eng;
  e.flush();
  Geometry g{};
  g.ndim = (int)wf.shape.size();
  for (int q = 0; q < g.ndim; ++q) {
    g.perm[q] = e.perm[q];
    g.sshape[q] = (int64_t)wf.shape[e.perm[q]];
  }
  if (two_d || wf.shape.size() == 1) {
    if (wf.points() != points) throw Error(SO_ERR_SHAPE, "saver grid sizes differ from the wave function");
    DeviceBuffer d(points * sizeof(double));
    cuda_check(launch_density(d.as<double>(), e.psi.ptr, e.real, g, e.stream), "density");
    std::vector<double> h(points);
    cuda_check(cudaMemcpyAsync(h.data(), d.ptr, points * sizeof(double), cudaMemcpyDeviceToHost, e.stream), "copy");
    cuda_check(cudaStreamSynchronize(e.stream), "sync");
    for (size_t i = 0; i < points; ++i) data[i * frames_no + frame] = h[i];
  } else {
    const size_t axis = grid_a.dimension_no;
    if (axis >= wf.shape.size() || wf.shape[axis] != points)
      throw Error(SO_ERR_SHAPE, "state grid differs from the wave function axis");
    std::vector<const double*> w = wf.weight_ptrs();
    DeviceBuffer d(points * sizeof(double));
    cuda_check(launch_state_density(d.as<double>(), e.psi.ptr, e.real, g, (int)axis, w.data(), nullptr, e.stream),
               "state density");
    std::vector<double> h(points);
    cuda_check(cudaMemcpyAsync(h.data(), d.ptr, points * sizeof(double), cudaMemcpyDeviceToHost, e.stream), "copy");
    cuda_check(cudaStreamSynchronize(e.stream), "sync");
    for (size_t i = 0; i < points; ++i) data[i * frames_no + frame] = h[i];
  }
}

void StateSaver::reset() { data.assign(points * frames_no, 0.0); }

// ------------------------------------------------------------------- Propagation
// Storage order of a propagation's state: the FFT axis innermost (contiguous FFT
// lanes); without an FFT, a lane-matrix axis outermost (strided lanes make the
// matrix product a GEMM over contiguous columns).
static std::vector<int> choose_perm(size_t ndim, const OperationStack& st) {
  int fft_axis = -1, mat_axis = -1;
  for (const auto& e : st.stack) {
    if (auto* f = dynamic_cast<FFTTransformation*>(e.op.get()))
      if (fft_axis < 0) fft_axis = (int)f->dimension_no;
    if (auto* m = dynamic_cast<MatrixTransformation*>(e.op.get()))
      if (mat_axis < 0) mat_axis = (int)m->dimension_no;
  }
  if (fft_axis >= (int)ndim) fft_axis = -1;
  if (mat_axis >= (int)ndim || mat_axis == fft_axis) mat_axis = -1;
  std::vector<int> perm;
  if (fft_axis < 0 && mat_axis >= 0) perm.push_back(mat_axis);
  for (size_t a = 0; a < ndim; ++a)
    if ((int)a != fft_axis && !(fft_axis < 0 && (int)a == mat_axis)) perm.push_back((int)a);
  if (fft_axis >= 0) perm.push_back(fft_axis);
  return perm;
}

Propagation::Propagation(WaveFunction& src, so_time_grid time, std::shared_ptr<OperationStack> stack, int prec)
    : precision(prec), time_(time), stack_(std::move(stack)) {
  if (prec < SO_PRECISION_FP64 || prec > SO_PRECISION_FLOAT_FLOAT) throw Error(SO_ERR_INVALID, "unknown precision");
  const int real = prec == SO_PRECISION_FP64 ? kRealF64 : (prec == SO_PRECISION_FLOAT_FLOAT ? kRealFF : kRealF32);
  wf_ = std::make_unique<WaveFunction>(src.shape, src.grids, choose_perm(src.shape.size(), *stack_), real);
  wf_->eng->tc_tf32 = prec == SO_PRECISION_FP32_TF32X3;
  wf_->eng->tc_bf16 = prec == SO_PRECISION_FP32_BF16X3;
  wf_->eng->tc_bf16x6 = prec == SO_PRECISION_FP32_BF16X6;
  {
    const char* fp = std::getenv("SO_FFT_PAIR");  // "0": FFT pairs run the general pass kernel
    wf_->eng->fft_pair = !(fp && fp[0] == '0');
    const char* ct = std::getenv("SO_FFT_PAIR_CT");  // "0": FFT pairs keep the general-shape kernel
    wf_->eng->fft_pair_ct = !(ct && ct[0] == '0');
  }
  wf_->last_grid_names = src.last_grid_names;
  wf_->possible_norm_change = src.possible_norm_change;
  wf_->eng->write_slot(wf_->cache_slot, src.eng->read_slot(src.cache_slot));
  std::vector<double> host(src.points() * 2);
  src.eng->export_host(host.data());
  wf_->eng->import_host(host.data());
  wf_->eng->sync();
  for (const auto& e : stack_->stack) keep_.push_back(e.op);
}

Propagation::~Propagation() {
  try {
    if (wf_) wf_->eng->sync();
  } catch (...) {
  }
}

void Propagation::step(Emitter& em) {
  WaveFunction& wf = *wf_;
  auto& ops = stack_->stack;
  for (auto& e : ops) {
    Operator& op = *e.op;
    switch (op.cls) {
      case OpClass::Propagator:
        op.apply(wf, em);
        break;
      case OpClass::Transformation:
        if (e.flag == SO_ORDER_NORMAL)
          op.transform(wf, em);
        else
          op.inverse_transform(wf, em);
        break;
      case OpClass::Saver:
        if (e.flag & SO_APPLY_FIRST_HALF) op.monitor(wf, em);
        break;
      case OpClass::Control:
        if (e.flag & SO_APPLY_FIRST_HALF) op.first_half(wf, em);
        break;
    }
  }
  for (size_t i = ops.size(); i-- > 1;) {
    auto& e = ops[i - 1];
    Operator& op = *e.op;
    switch (op.cls) {
      case OpClass::Propagator:
        op.apply(wf, em);
        break;
      case OpClass::Transformation:
        if (e.flag == SO_ORDER_NORMAL)
          op.inverse_transform(wf, em);
        else
          op.transform(wf, em);
        break;
      case OpClass::Saver:
        if (e.flag & SO_APPLY_SECOND_HALF) op.monitor(wf, em);
        break;
      case OpClass::Control:
        if (e.flag & SO_APPLY_SECOND_HALF) op.second_half(wf, em);
        break;
    }
  }
}

static bool same_program(const std::vector<Action>& a, const std::vector<Action>& b) {
  if (a.size() != b.size()) return false;
  for (size_t i = 0; i < a.size(); ++i) {
    if (a[i].lane_axis != b[i].lane_axis || a[i].host_call != b[i].host_call) return false;
    if (std::memcmp(&a[i].op, &b[i].op, sizeof(DevOp)) != 0) return false;
  }
  return true;
}

void Propagation::steps(uint64_t n) {
  Engine& e = *wf_->eng;
  steps_done_ += n;
  if (!e.resident_capable()) {
    Emitter em{&e};
    for (uint64_t i = 0; i < n; ++i) step(em);
    e.flush();
    return;
  }
  // Whole array in one CTA: consecutive identical steps run as one launch.
  std::vector<Action> prev;
  int rep = 0;
  for (uint64_t i = 0; i < n; ++i) {
    std::vector<Action> rec;
    std::vector<std::function<void()>> calls;
    Emitter em{&e, &rec, &calls};
    step(em);
    const bool has_host = std::any_of(rec.begin(), rec.end(), [](const Action& a) { return a.host_call >= 0; });
    if (!has_host && rep > 0 && same_program(rec, prev)) {
      ++rep;
      continue;
    }
    if (rep > 0) e.run_resident(prev, rep);
    rep = 0;
    prev.clear();
    if (has_host) {
      std::vector<Action> seg;
      for (const Action& a : rec) {
        if (a.host_call >= 0) {
          e.run_resident(seg, 1);
          seg.clear();
          calls[a.host_call]();
        } else {
          seg.push_back(a);
        }
      }
      e.run_resident(seg, 1);
    } else {
      prev = std::move(rec);
      rep = 1;
    }
  }
  if (rep > 0) e.run_resident(prev, rep);
}

double Propagation::mean_energy() {
  Engine& e = *wf_->eng;
  Emitter em{&e};
  if (time_.im_time) {
    if (stack_->stack.empty() || stack_->stack[0].op->cls != OpClass::Control ||
        stack_->stack[0].op->name() != "LeakControl")
      throw Error(SO_ERR_STATE, "For imaginary time propagation first control must be LeakControl.");
    LossChecker* lc = stack_->stack[0].op->loss_checker();
    if (!lc) throw Error(SO_ERR_STATE, "Leak control must have loss checker to get mean energy for imaginary time.");
    lc->reset(&em);
    steps(1);
    const int n = norm_slot(*wf_, em);
    const double norm = e.read_slot(n);
    const double decay = lc->loss();
    e.check_nonfinite();
    return -std::log(norm - decay) / time_.step / 2.0;
  }
  e.flush();
  DeviceBuffer before(e.points() * e.elem_bytes());
  cuda_check(cudaMemcpyAsync(before.ptr, e.psi.ptr, before.bytes, cudaMemcpyDeviceToDevice, e.stream), "clone");
  steps(1);
  const int sre = e.alloc_slot(0.0), sim = e.alloc_slot(0.0);
  Action a{};
  a.op.kind = OP_DOT;
  a.op.a = sre;
  a.op.b = sim;
  a.op.ptr = before.ptr;
  wf_->set_weights(a.op);
  e.submit(a);
  const double re = e.read_slot(sre), im = e.read_slot(sim);
  e.free_slot(sre);
  e.free_slot(sim);
  e.sync();
  return -std::atan2(im, re) / time_.step;
}

std::vector<double> Propagation::losses(bool include_controls) {
  std::vector<double> out;
  for (auto& e : stack_->stack) {
    if (e.op->cls == OpClass::Propagator || (include_controls && e.op->cls == OpClass::Control))
      if (LossChecker* lc = e.op->loss_checker()) out.push_back(lc->loss());
  }
  wf_->eng->check_nonfinite();
  return out;
}

void Propagation::reset_losses() {
  Emitter em{wf_->eng.get()};
  for (auto& e : stack_->stack)
    if (e.op->cls == OpClass::Propagator)
      if (LossChecker* lc = e.op->loss_checker()) lc->reset(&em);
  wf_->eng->flush();
}

std::unique_ptr<WaveFunction> Propagation::snapshot() {
  std::vector<int> ident(wf_->shape.size());
  std::iota(ident.begin(), ident.end(), 0);
  auto w = std::make_unique<WaveFunction>(wf_->shape, wf_->grids, ident, kRealF64);
  w->last_grid_names = wf_->last_grid_names;
  w->possible_norm_change = wf_->possible_norm_change;
  w->eng->write_slot(w->cache_slot, wf_->eng->read_slot(wf_->cache_slot));
  std::vector<double> host(wf_->points() * 2);
  wf_->eng->export_host(host.data());
  w->eng->import_host(host.data());
  w->eng->sync();
  return w;
}

// ------------------------------------------------------------ checkpoint / resume
// Byte layout (native endianness; a checkpoint is read back on the same kind of host):
//   "SOCKPT01", precision i32, ndim u64, shape u64 x ndim, steps_done u64,
//   possible_norm_change u8, norm cache f64, per axis: current grid name, last seen name;
//   operator count u64, per operator: type name, scalar count u64, scalars f64 x count,
//   saver flag u8 [current_frame u64, times, data]; then the state as complex128 in the
//   logical row-major order (exact for FP64 and FP32 states: FP32 values are FP64 values);
//   a float-float state adds its device words (storage order, FP32 hi / lo pairs) as a
//   vector of 8-byte words, since hi + lo does not always fit one FP64 value.
namespace {
struct BlobWriter {
  std::vector<unsigned char> b;
  void bytes(const void* p, size_t n) {
    const unsigned char* c = static_cast<const unsigned char*>(p);
    b.insert(b.end(), c, c + n);
  }
  template <class T>
  void put(const T& v) {
    bytes(&v, sizeof(T));
  }
  void str(const std::string& s) {
    put<uint64_t>(s.size());
    bytes(s.data(), s.size());
  }
  void vec(const std::vector<double>& v) {
    put<uint64_t>(v.size());
    bytes(v.data(), v.size() * sizeof(double));
  }
};
struct BlobReader {
  const unsigned char* p;
  size_t n, off = 0;
  void bytes(void* dst, size_t k) {
    if (off + k > n) throw Error(SO_ERR_INVALID, "checkpoint is truncated");
    std::memcpy(dst, p + off, k);
    off += k;
  }
  template <class T>
  T get() {
    T v;
    bytes(&v, sizeof(T));
    return v;
  }
  std::string str() {
    const uint64_t k = get<uint64_t>();
    if (k > n - off) throw Error(SO_ERR_INVALID, "checkpoint is truncated");
    std::string s(reinterpret_cast<const char*>(p + off), (size_t)k);
    off += (size_t)k;
    return s;
  }
  std::vector<double> vec() {
    const uint64_t k = get<uint64_t>();
    if (k > (n - off) / sizeof(double)) throw Error(SO_ERR_INVALID, "checkpoint is truncated");
    std::vector<double> v((size_t)k);
    bytes(v.data(), v.size() * sizeof(double));
    return v;
  }
};
constexpr char kCkptMagic[8] = {'S', 'O', 'C', 'K', 'P', 'T', '0', '1'};
}  // namespace

std::vector<unsigned char> Propagation::checkpoint() {
  Engine& e = *wf_->eng;
  e.flush();
  BlobWriter w;
  w.bytes(kCkptMagic, sizeof(kCkptMagic));
  w.put<int32_t>(precision);
  w.put<uint64_t>(wf_->shape.size());
  for (size_t s : wf_->shape) w.put<uint64_t>(s);
  w.put<uint64_t>(steps_done_);
  w.put<uint8_t>(wf_->possible_norm_change ? 1 : 0);
  w.put<double>(e.read_slot(wf_->cache_slot));
  for (size_t a = 0; a < wf_->shape.size(); ++a) {
    w.str(wf_->grids[a].name);
    w.str(wf_->last_grid_names[a]);
  }
  w.put<uint64_t>(stack_->stack.size());
  for (auto& ent : stack_->stack) {
    Operator& op = *ent.op;
    w.str(op.type);
    const std::vector<ScalarState*> sc = op.scalar_states();
    std::vector<double> vals;
    for (ScalarState* st : sc)
      for (size_t i = 0; i < st->host.size(); ++i) vals.push_back(st->get(i));
    w.vec(vals);
    auto* sv = dynamic_cast<StateSaver*>(&op);
    w.put<uint8_t>(sv ? 1 : 0);
    if (sv) {
      w.put<uint64_t>(sv->current_frame);
      w.vec(sv->times);
      w.vec(sv->data);
    }
  }
  std::vector<double> host(wf_->points() * 2);
  e.export_host(host.data());
  w.vec(host);
  if (e.real == kRealFF) {
    std::vector<double> raw(wf_->points() * 2);
    cuda_check(cudaMemcpyAsync(raw.data(), e.psi.ptr, e.psi.bytes, cudaMemcpyDeviceToHost, e.stream), "state copy");
    cuda_check(cudaStreamSynchronize(e.stream), "state copy sync");
    w.vec(raw);
  }
  e.check_nonfinite();
  return std::move(w.b);
}

void Propagation::restore(const unsigned char* data, size_t size) {
  if (!data) throw Error(SO_ERR_INVALID, "null checkpoint");
  BlobReader r{data, size};
  char magic[sizeof(kCkptMagic)];
  r.bytes(magic, sizeof(magic));
  if (std::memcmp(magic, kCkptMagic, sizeof(magic)) != 0) throw Error(SO_ERR_INVALID, "not a checkpoint");
  // read and check everything before changing anything
  const int32_t prec = r.get<int32_t>();
  if (prec != precision) throw Error(SO_ERR_STATE, "checkpoint was taken at another precision");
  const uint64_t nd = r.get<uint64_t>();
  if (nd != wf_->shape.size()) throw Error(SO_ERR_SHAPE, "checkpoint has another number of axes");
  for (size_t a = 0; a < nd; ++a)
    if (r.get<uint64_t>() != wf_->shape[a]) throw Error(SO_ERR_SHAPE, "checkpoint has another shape");
  const uint64_t done = r.get<uint64_t>();
  const bool pnc = r.get<uint8_t>() != 0;
  const double cached_norm = r.get<double>();
  std::vector<std::string> last(nd);
  for (size_t a = 0; a < nd; ++a) {
    if (r.str() != wf_->grids[a].name)
      throw Error(SO_ERR_STATE, "checkpoint was taken in another representation of axis " + std::to_string(a));
    last[a] = r.str();
  }
  if (r.get<uint64_t>() != stack_->stack.size()) throw Error(SO_ERR_STATE, "checkpoint has another operator stack");
  struct OpState {
    std::vector<double> vals;
    bool saver = false;
    uint64_t frame = 0;
    std::vector<double> times, data;
  };
  std::vector<OpState> ops(stack_->stack.size());
  for (size_t i = 0; i < ops.size(); ++i) {
    Operator& op = *stack_->stack[i].op;
    if (r.str() != op.type) throw Error(SO_ERR_STATE, "checkpoint operator " + std::to_string(i) + " differs");
    ops[i].vals = r.vec();
    size_t want = 0;
    for (ScalarState* st : op.scalar_states()) want += st->host.size();
    if (ops[i].vals.size() != want) throw Error(SO_ERR_STATE, "checkpoint operator " + std::to_string(i) + " differs");
    ops[i].saver = r.get<uint8_t>() != 0;
    auto* sv = dynamic_cast<StateSaver*>(&op);
    if (ops[i].saver != (sv != nullptr)) throw Error(SO_ERR_STATE, "checkpoint saver layout differs");
    if (sv) {
      ops[i].frame = r.get<uint64_t>();
      ops[i].times = r.vec();
      ops[i].data = r.vec();
      if (ops[i].data.size() != sv->data.size()) throw Error(SO_ERR_STATE, "checkpoint saver size differs");
    }
  }
  const std::vector<double> host = r.vec();
  if (host.size() != wf_->points() * 2) throw Error(SO_ERR_SHAPE, "checkpoint state has another size");
  Engine& e = *wf_->eng;
  std::vector<double> raw;
  if (e.real == kRealFF) {
    raw = r.vec();
    if (raw.size() * sizeof(double) != e.psi.bytes) throw Error(SO_ERR_SHAPE, "checkpoint state has another size");
  }
  if (r.off != size) throw Error(SO_ERR_INVALID, "checkpoint has trailing bytes");
  // apply
  if (e.real == kRealFF) {
    e.flush();
    cuda_check(cudaMemcpyAsync(e.psi.ptr, raw.data(), e.psi.bytes, cudaMemcpyHostToDevice, e.stream), "state copy");
    cuda_check(cudaStreamSynchronize(e.stream), "state copy sync");
  } else {
    e.import_host(host.data());
  }
  e.write_slot(wf_->cache_slot, cached_norm);
  wf_->possible_norm_change = pnc;
  wf_->last_grid_names = last;
  for (size_t i = 0; i < ops.size(); ++i) {
    Operator& op = *stack_->stack[i].op;
    size_t k = 0;
    for (ScalarState* st : op.scalar_states()) {
      // bind to this engine so the values land where the next step reads them
      st->bind(&e);
      for (size_t j = 0; j < st->host.size(); ++j) st->set(j, ops[i].vals[k++]);
    }
    if (auto* sv = dynamic_cast<StateSaver*>(&op)) {
      sv->current_frame = (size_t)ops[i].frame;
      sv->times = ops[i].times;
      sv->data = ops[i].data;
    }
  }
  steps_done_ = done;
  e.sync();
}

void Propagation::reset_savers() {
  for (auto& e : stack_->stack)
    if (e.op->cls == OpClass::Saver) e.op->reset();
}

void Propagation::savers_save() {
  wf_->eng->sync();
  for (auto& e : stack_->stack)
    if (auto* s = dynamic_cast<StateSaver*>(e.op.get())) s->save();
}

void Propagation::get_array(double* out, bool sync, bool copy_engine) { wf_->eng->export_host(out, sync, copy_engine); }

void Propagation::set_array(const double* in, bool copy_engine) {
  wf_->eng->import_host(in, copy_engine);
  wf_->possible_norm_change = true;
}

double Propagation::norm() {
  Emitter em{wf_->eng.get()};
  const int s = norm_slot(*wf_, em);
  const double v = wf_->eng->read_slot(s);
  wf_->eng->check_nonfinite();
  return v;
}

void Propagation::synchronize() {
  wf_->eng->sync();
  wf_->eng->check_nonfinite();
}

bool Propagation::has_savers() const {
  for (const auto& e : stack_->stack)
    if (e.op->cls == OpClass::Saver) return true;
  return false;
}

std::vector<RecordedPass> Propagation::record_steps(uint64_t n) {
  Engine& e = *wf_->eng;
  e.flush();
  std::vector<RecordedPass> out;
  e.recording = &out;
  try {
    Emitter em{&e};
    for (uint64_t i = 0; i < n; ++i) step(em);
    e.flush();
  } catch (...) {
    e.recording = nullptr;
    throw;
  }
  e.recording = nullptr;
  return out;
}

// ------------------------------------------------------------------------ Batch
static bool same_params(const RecordedPass& a, const RecordedPass& b) {
  if (a.kind != b.kind) return false;
  if (a.kind == RecordedPass::TensorCore) return a.tcp == b.tcp;
  return std::memcmp(&a.p, &b.p, sizeof(PassParams)) == 0;
}

Batch::Batch(std::vector<Propagation*> props) : props_(std::move(props)) {
  if (props_.empty()) throw Error(SO_ERR_INVALID, "empty batch");
  for (Propagation* p : props_) {
    if (p->has_savers()) throw Error(SO_ERR_UNSUPPORTED, "batched propagations cannot carry savers");
    if (p->engine().resident_capable())
      throw Error(SO_ERR_UNSUPPORTED, "batched propagations need multi-lane (2-D or larger) states");
  }
  stream_ = props_[0]->engine().stream;
  if (stream_ == nullptr) {
    // graph capture needs a stream other than the legacy default stream
    cuda_check(cudaStreamCreateWithFlags(&stream_, cudaStreamNonBlocking), "batch stream");
    own_stream_ = true;
  }
}

Batch::~Batch() {
  if (const char* path = std::getenv("SO_TC_TRACE_BATCH")) {
    cudaStreamSynchronize(stream_);
    if (FILE* f = std::fopen(path, "a")) {
      for (TraceBuf& tb : traces_) {
        std::vector<unsigned long long> h(tb.buf.bytes / sizeof(unsigned long long));
        if (cudaMemcpy(h.data(), tb.buf.ptr, tb.buf.bytes, cudaMemcpyDeviceToHost) != cudaSuccess) break;
        std::fprintf(f, "pass %s tiles=%lld slots=%d\n", tb.name.c_str(), (long long)tb.tiles,
                     angular_tc_trace_slots());
        for (size_t i = 0; i < h.size(); ++i)
          std::fprintf(f, "%llu%c", h[i], (i + 1) % angular_tc_trace_slots() == 0 ? '\n' : ' ');
      }
      std::fclose(f);
    }
  }
  for (Chunk& ch : chunks_) {
    ch.batch.reset();
    cudaStreamSynchronize(ch.stream);
    cudaStreamDestroy(ch.stream);
    cudaEventDestroy(ch.in_done);
    cudaEventDestroy(ch.out_done);
  }
  for (Timed& t : timed_) {
    cudaEventDestroy(t.a);
    cudaEventDestroy(t.b);
  }
  for (size_t k = 0; k < side_.size(); ++k) {
    cudaStreamSynchronize(side_[k]);
    cudaStreamDestroy(side_[k]);
    cudaEventDestroy(joins_[k]);
  }
  if (fork_) cudaEventDestroy(fork_);
  if (own_stream_) {
    cudaStreamSynchronize(stream_);
    cudaStreamDestroy(stream_);
  }
}

std::vector<Batch::Group> Batch::build_groups(const std::vector<std::vector<RecordedPass>>& rec, size_t pos) {
  // group key: kind, precision, threads, shared memory; FFT-pair passes also by lane extent
  // (each extent has its own launch schedule, and the tuner times each extent's launches)
  std::map<std::tuple<int, int, int, size_t, int64_t>, std::vector<const RecordedPass*>> by;
  for (const auto& r : rec) {
    const RecordedPass& rp = r[pos];
    if (rp.kind == RecordedPass::Scalar || rp.kind == RecordedPass::Resident)
      throw Error(SO_ERR_UNSUPPORTED, "pass kind cannot be batched");
    const int64_t ext = (rp.kind == RecordedPass::Generic && rp.p.fused) ? rp.p.g.n : 0;
    by[{(int)rp.kind, rp.real, rp.threads, rp.smem, ext}].push_back(&rp);
  }
  std::vector<Group> out;
  for (auto& kv : by) {
    const auto& v = kv.second;
    Group g{};
    g.kind = v[0]->kind;
    g.real = v[0]->real;
    g.threads = v[0]->threads;
    g.smem = v[0]->smem;
    g.count = (int)v.size();
    g.name = "batched " + std::to_string(v.size()) + "x " + v[0]->name;
    g.n = v[0]->p.g.n;
    if (g.kind == RecordedPass::Generic && ((g.threads >> 20) & 1)) g.ct_lgn = v[0]->p.ct;
    std::vector<int64_t> off(v.size() + 1, 0);
    const size_t pb = g.kind == RecordedPass::TensorCore ? tc_params_bytes() : sizeof(PassParams);
    std::vector<unsigned char> params(pb * v.size());
    // SO_TC_TRACE_BATCH=<file>: per-tile phase timestamps of every member's tensor-core pass
    // (the last launch of each cached group), written when the batch is destroyed
    static const char* trace_path = std::getenv("SO_TC_TRACE_BATCH");
    g.bytes = 0.0;
    g.sweep = true;  // the compact kernel only when every member's pass allows it
    for (size_t i = 0; i < v.size(); ++i) {
      off[i + 1] = off[i] + v[i]->p.g.tiles;
      g.sweep = g.sweep && v[i]->p.sweep;
      if (g.kind == RecordedPass::TensorCore) {
        std::memcpy(params.data() + i * pb, v[i]->tcp.data(), pb);
        if (trace_path) {
          TraceBuf tb;
          tb.tiles = v[i]->p.g.tiles;
          tb.name = v[i]->name + " n=" + std::to_string(v[i]->p.g.n) + " member " + std::to_string(i);
          tb.buf = DeviceBuffer((size_t)tb.tiles * angular_tc_trace_slots() * sizeof(unsigned long long));
          cuda_check(cudaMemset(tb.buf.ptr, 0, tb.buf.bytes), "trace clear");
          tc_params_set_trace(params.data() + i * pb, tb.buf.as<unsigned long long>());
          traces_.push_back(std::move(tb));
        }
      } else {
        std::memcpy(params.data() + i * pb, &v[i]->p, pb);
      }
      g.bytes += v[i]->bytes;
    }
    g.blocks = off.back();
    g.params = DeviceBuffer(params.size());
    g.offsets = DeviceBuffer(off.size() * sizeof(int64_t));
    cuda_check(cudaMemcpy(g.params.ptr, params.data(), params.size(), cudaMemcpyHostToDevice), "batch params");
    cuda_check(cudaMemcpy(g.offsets.ptr, off.data(), off.size() * sizeof(int64_t), cudaMemcpyHostToDevice),
               "batch offsets");
    if (g.kind == RecordedPass::TensorCore) {
      // the tensor-core kernel looks tiles up directly: (pass index, tile within the pass)
      if (g.blocks >= (int64_t)0xffffffff) throw Error(SO_ERR_UNSUPPORTED, "too many tiles in one batched pass");
      std::vector<uint32_t> own((size_t)g.blocks * 2);
      for (size_t i = 0; i + 1 < off.size(); ++i)
        for (int64_t t = off[i]; t < off[i + 1]; ++t) {
          own[(size_t)t * 2] = (uint32_t)i;
          own[(size_t)t * 2 + 1] = (uint32_t)(t - off[i]);
        }
      if ((g.threads >> 22) & 1) {
        // blocked: CTA k (positions k, k + G, k + 2G, ...) takes one run of consecutive tiles,
        // mostly of one member (one pass description, neighbouring columns)
        const int64_t G = angular_tc_grid(g.blocks, (g.threads >> 20) & 3), base = g.blocks / G,
                      rem = g.blocks % G;
        std::vector<uint32_t> blk(own.size());
        for (int64_t b = 0; b < g.blocks; ++b) {
          const int64_t k = b % G, i = b / G;
          const int64_t t = k * base + std::min(k, rem) + i;
          blk[(size_t)b * 2] = own[(size_t)t * 2];
          blk[(size_t)b * 2 + 1] = own[(size_t)t * 2 + 1];
        }
        own.swap(blk);
      }
      g.owners = DeviceBuffer(own.size() * sizeof(uint32_t));
      cuda_check(cudaMemcpy(g.owners.ptr, own.data(), own.size() * sizeof(uint32_t), cudaMemcpyHostToDevice),
                 "batch tile owners");
    }
    out.push_back(std::move(g));
  }
  return out;
}

void Batch::run_groups(std::vector<Group>& gs, bool concurrent) {
  // the members of a position's groups are disjoint, so the groups may run side by side: the
  // largest first on the batch stream, the others on forked streams joined before the next
  // position (the results are those of the sequential order: no member is touched twice)
  // SO_BATCH_SERIAL=1: every group on the batch stream, one after another (for comparison)
  const char* serial = std::getenv("SO_BATCH_SERIAL");
  const bool fork = concurrent && !timing_ && gs.size() > 1 && !(serial && serial[0] == '1');
  std::vector<size_t> order(gs.size());
  for (size_t k = 0; k < gs.size(); ++k) order[k] = k;
  if (fork) {
    std::stable_sort(order.begin(), order.end(), [&](size_t a, size_t b) { return gs[a].bytes > gs[b].bytes; });
    if (fork_ == nullptr) cuda_check(cudaEventCreateWithFlags(&fork_, cudaEventDisableTiming), "fork event");
    while (side_.size() + 1 < gs.size()) {
      cudaStream_t st;
      cudaEvent_t ev;
      cuda_check(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking), "side stream");
      cuda_check(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming), "join event");
      side_.push_back(st);
      joins_.push_back(ev);
    }
    cuda_check(cudaEventRecord(fork_, stream_), "fork record");
    for (size_t k = 1; k < gs.size(); ++k) cuda_check(cudaStreamWaitEvent(side_[k - 1], fork_, 0), "fork wait");
  }
  for (size_t q = 0; q < gs.size(); ++q) {
    Group& g = gs[order[q]];
    cudaStream_t st = fork && q > 0 ? side_[q - 1] : stream_;
    Timed t{};
    if (timing_) {
      t.name = g.name;
      t.bytes = g.bytes;
      if (g.kind == RecordedPass::TensorCore) {
        t.cls_kind = 1;
        t.cls_mode = (g.threads >> 17) & 3;
      } else if ((g.threads >> 16) & 1) {
        t.cls_kind = 0;
        t.cls_mode = g.real != kRealF32 ? 1 : 0;
      }
      t.cls_n = g.n;
      cuda_check(cudaEventCreate(&t.a), "event");
      cuda_check(cudaEventCreate(&t.b), "event");
      cuda_check(cudaEventRecord(t.a, stream_), "event record");
    }
    if (g.kind == RecordedPass::TensorCore)
      cuda_check(launch_angular_tc_batched(g.params.ptr, g.owners.ptr, g.blocks, g.smem, (g.threads >> 17) & 3,
                                           st, (g.threads >> 20) & 3, 1 << ((g.threads >> 23) & 3)),
                 "batched tensor-core pass");
    else
      cuda_check(launch_pass_batched(g.real, g.sweep, (g.threads >> 16) & 1, g.params.as<PassParams>(),
                                     g.offsets.as<int64_t>(), g.count, g.blocks, g.threads & 0xffff, g.smem, st,
                                     ((g.threads >> 19) & 1) ? 8 : 0,
                                     g.ct_lgn),
                 "batched pass");
    if (timing_) {
      cuda_check(cudaEventRecord(t.b, stream_), "event record");
      timed_.push_back(t);
    }
  }
  if (fork)
    for (size_t k = 1; k < gs.size(); ++k) {
      cuda_check(cudaEventRecord(joins_[k - 1], side_[k - 1]), "join record");
      cuda_check(cudaStreamWaitEvent(stream_, joins_[k - 1], 0), "join wait");
    }
}

void Batch::steps(uint64_t n, bool wait, bool sync_members) {
  if (n == 0) return;
  static const bool trace = std::getenv("SO_PIPE_TRACE") != nullptr;
  const auto t0 = std::chrono::steady_clock::now();
  auto ms = [&] { return std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count(); };
  double t_sync = 0.0, t_rec = 0.0, t_groups = 0.0;
  {
    std::vector<cudaStream_t> seen;  // each member's queued work, then one wait per stream
    for (Propagation* p : props_) {
      p->engine().flush();
      if (std::find(seen.begin(), seen.end(), p->engine().stream) == seen.end()) seen.push_back(p->engine().stream);
    }
    // members on the batch's own stream are ordered by the stream itself
    if (sync_members)
      for (cudaStream_t st : seen) cuda_check(cudaStreamSynchronize(st), "stream sync");
    else
      for (cudaStream_t st : seen)
        if (st != stream_) cuda_check(cudaStreamSynchronize(st), "stream sync");
  }
  t_sync = ms();
  // Host logic of two steps per propagation: passes [head, period..., tail] where the
  // period (the middle passes) repeats for every further step.
  std::vector<std::vector<RecordedPass>> rec;
  for (Propagation* p : props_) rec.push_back(p->record_steps(2));
  t_rec = ms();
  const size_t np = rec[0].size();
  for (const auto& r : rec)
    if (r.size() != np || np < 2)
      throw Error(SO_ERR_UNSUPPORTED, "propagations of a batch must share the pass structure of the step");
  // Two recorded steps give either
  //   odd  np = 2m + 1: [head] [period: m passes] [tail: m passes], the last period pass being the
  //        one where a step's end and the next step's start share a pass; tail == period except
  //        for that last pass.  n steps = head, period x (n - 1), tail.
  //   even np = 2m: [step 1: m passes] [step 2: m passes]; n steps = step 1, step 2 x (n - 1).
  const bool merged = np % 2 == 1;
  const size_t m = merged ? (np - 1) / 2 : np / 2;
  const size_t per0 = merged ? 1 : m;  // first pass of the repeated period
  for (const auto& r : rec)
    for (size_t i = 1; i < m; ++i)
      if (!same_params(r[i], r[m + i])) {
        // name the first differing byte of the pass parameters (diagnostic)
        const unsigned char* a = reinterpret_cast<const unsigned char*>(&r[i].p);
        const unsigned char* b = reinterpret_cast<const unsigned char*>(&r[m + i].p);
        size_t off = 0;
        while (off < sizeof(PassParams) && a[off] == b[off]) ++off;
        throw Error(SO_ERR_UNSUPPORTED, "step program is not periodic (pass " + std::to_string(i) + " '" +
                                            r[i].name + "' vs '" + r[m + i].name + "', byte " +
                                            std::to_string(off) + " of " + std::to_string(np) +
                                            " passes); run these propagations one by one");
      }
  // the launch groups (device parameter blocks) of the last call are reused when every
  // recorded pass has the same parameters: consecutive calls of a steady propagation
  bool reuse = cached_rec_.size() == rec.size() && cached_epoch_ == schedule_epoch();
  for (size_t i = 0; reuse && i < rec.size(); ++i) {
    reuse = cached_rec_[i].size() == rec[i].size();
    for (size_t j = 0; reuse && j < rec[i].size(); ++j) reuse = same_params(rec[i][j], cached_rec_[i][j]);
  }
  if (!reuse) {
    cached_pos_.clear();
    cached_pos_.resize(np);
    for (size_t i = 0; i < np; ++i) cached_pos_[i] = build_groups(rec, i);
    cached_rec_ = std::move(rec);
    cached_epoch_ = schedule_epoch();
  }
  std::vector<std::vector<Group>>& pos = cached_pos_;
  t_groups = ms();
  launches_per_step_ = 0;
  for (size_t i = per0; i < per0 + m; ++i) launches_per_step_ += pos[i].size();
  // first step (head)
  for (size_t i = 0; i < (merged ? 1 : m); ++i) run_groups(pos[i], true);
  // the period once per further step, captured once as a CUDA graph when timing is off
  const uint64_t reps = n - 1;
  if (reps > 0) {
    if (!timing_ && reps >= 4) {
      cudaGraph_t graph;
      cudaGraphExec_t exec;
      cuda_check(cudaStreamBeginCapture(stream_, cudaStreamCaptureModeThreadLocal), "begin capture");
      for (size_t i = per0; i < per0 + m; ++i) run_groups(pos[i], true);
      cuda_check(cudaStreamEndCapture(stream_, &graph), "end capture");
      cuda_check(cudaGraphInstantiate(&exec, graph, 0), "graph instantiate");
      for (uint64_t r = 0; r < reps; ++r) cuda_check(cudaGraphLaunch(exec, stream_), "graph launch");
      count_launch(launches_per_step_ * (reps - 1));  // the capture counted the period once
      cuda_check(cudaStreamSynchronize(stream_), "batch sync");  // before the graph is destroyed
      cudaGraphExecDestroy(exec);
      cudaGraphDestroy(graph);
    } else {
      for (uint64_t r = 0; r < reps; ++r)
        for (size_t i = per0; i < per0 + m; ++i) run_groups(pos[i], true);
    }
  }
  // tail: the last step's closing passes (merged form only)
  if (merged)
    for (size_t i = m + 1; i < np; ++i) run_groups(pos[i], true);
  for (Propagation* p : props_) p->count_steps(n);
  if (trace)
    std::fprintf(stderr, "batch steps(%llu) of %zu: sync %.3f record %.3f groups%s %.3f launched %.3f ms\n",
                 (unsigned long long)n, props_.size(), t_sync, t_rec, reuse ? " (reused)" : "", t_groups, ms());
  if (wait) cuda_check(cudaStreamSynchronize(stream_), "batch sync");
}

void Batch::set_arrays(const double* const* in) {
  for (size_t i = 0; i < props_.size(); ++i)
    if (!in[i]) throw Error(SO_ERR_INVALID, "null state array in batch");
  for (size_t i = 0; i < props_.size(); ++i) props_[i]->set_array(in[i]);
}

void Batch::get_arrays(double* const* out) {
  for (size_t i = 0; i < props_.size(); ++i)
    if (!out[i]) throw Error(SO_ERR_INVALID, "null state array in batch");
  // every export is queued first; one wait per distinct stream at the end
  for (size_t i = 0; i < props_.size(); ++i) props_[i]->get_array(out[i], false);
  std::vector<cudaStream_t> done;
  for (Propagation* p : props_) {
    cudaStream_t s = p->engine().stream;
    if (std::find(done.begin(), done.end(), s) != done.end()) continue;
    done.push_back(s);
    cuda_check(cudaStreamSynchronize(s), "batch export sync");
  }
}

// member chunks of the host-to-host pipeline (SO_HOST_CHUNKS overrides, 1..16; the chunks
// are formed at a batch's first steps_host call and kept)
static size_t host_chunks() {
  const char* e = std::getenv("SO_HOST_CHUNKS");
  const long v = e ? std::strtol(e, nullptr, 10) : 16;
  return (size_t)std::min<long>(64, std::max<long>(1, v));
}

void Batch::steps_host(const double* const* in, double* const* out, uint64_t n) {
  const size_t kHostChunks = host_chunks();
  const size_t m = props_.size();
  for (size_t i = 0; i < m; ++i)
    if (!in[i] || !out[i]) throw Error(SO_ERR_INVALID, "null state array in batch");
  if (chunks_.empty()) {
    // chunks of consecutive members with about equal points, each a batch of its own on
    // its own stream
    double total = 0.0;
    for (Propagation* p : props_) total += (double)p->engine().points();
    const size_t k = std::min<size_t>(kHostChunks, m);
    // the first and the last chunk get half the points of the others: the link carries one
    // direction alone while the first chunk comes in and the last goes out (512-instance
    // batch, 16 chunks: 19.2 -> 19.0 ms per step; a third of the others: 19.1 ms)
    const double taper = 0.5;
    std::vector<double> wsum(k + 1, 0.0);
    for (size_t c = 0; c < k; ++c) wsum[c + 1] = wsum[c] + ((k > 2 && (c == 0 || c + 1 == k)) ? taper : 1.0);
    size_t first = 0;
    double acc = 0.0;
    for (size_t c = 0; c < k; ++c) {
      size_t last = first;
      const double goal = total * wsum[c + 1] / wsum[k];
      while (last < m && (c + 1 == k || acc < goal || last == first)) acc += (double)props_[last++]->engine().points();
      if (last == first) break;
      Chunk ch;
      ch.first = first;
      ch.count = last - first;
      cuda_check(cudaStreamCreateWithFlags(&ch.stream, cudaStreamNonBlocking), "chunk stream");
      cuda_check(cudaEventCreateWithFlags(&ch.in_done, cudaEventDisableTiming), "chunk event");
      cuda_check(cudaEventCreateWithFlags(&ch.out_done, cudaEventDisableTiming), "chunk event");
      std::vector<Propagation*> sub(props_.begin() + first, props_.begin() + last);
      std::vector<cudaStream_t> saved;
      for (Propagation* p : sub) {
        saved.push_back(p->engine().stream);
        p->engine().stream = ch.stream;
      }
      ch.batch = std::make_unique<Batch>(sub);  // its launches go to ch.stream
      for (size_t i = 0; i < sub.size(); ++i) sub[i]->engine().stream = saved[i];
      chunks_.push_back(std::move(ch));
      first = last;
    }
  }
  // members' own streams: everything queued there before this call completes first
  std::vector<cudaStream_t> own;
  for (Propagation* p : props_) {
    p->engine().flush();
    own.push_back(p->engine().stream);
  }
  for (size_t i = 0; i < m; ++i)
    if (std::find(own.begin(), own.begin() + i, own[i]) == own.begin() + i)
      cuda_check(cudaStreamSynchronize(own[i]), "stream sync");
  for (Chunk& ch : chunks_)
    for (size_t i = ch.first; i < ch.first + ch.count; ++i) props_[i]->engine().stream = ch.stream;
  // SO_PIPE_TRACE=1: host-side time of each phase of the call on stderr
  static const bool trace = std::getenv("SO_PIPE_TRACE") != nullptr;
  auto now = [] { return std::chrono::steady_clock::now(); };
  std::vector<std::pair<std::string, double>> marks;
  const auto t0 = now();
  auto mark = [&](const std::string& what) {
    if (trace) marks.emplace_back(what, std::chrono::duration<double, std::milli>(now() - t0).count());
  };
  try {
    // Copy engines: every chunk's states in (host link H2D), in chunk order; later each
    // chunk's states out (D2H), in chunk order.  SMs: the chunk's layout kernels in, its
    // steps, its layout kernels out, each chunk as soon as its own states are in (chunks
    // are not ordered among themselves on the SMs, so one chunk's small launches fill the
    // gaps of another's: 20.1 -> 19.3 ms per step for the 512-instance batch).  So chunk c
    // computes while later chunks arrive and earlier ones leave, and the link carries both
    // directions at once.
    // (Interleaved copies would make every chunk arrive only when all had; a layout kernel
    // queued between two copies would hold the copy engine behind the SMs.)
    // A chunk whose members' host arrays lie back to back (in member order) moves them with
    // one copy per direction through the chunk's own staging buffer: each cudaMemcpyAsync
    // costs a few microseconds of its own on the link (measured on the GB300 for the
    // 512-instance batch, 2.8 GB each way: one copy per member 19.8 ms both ways at once,
    // one copy per direction 16.3 ms).
    std::vector<char> in_merged(chunks_.size()), out_merged(chunks_.size());
    std::vector<std::vector<size_t>> offs(chunks_.size());
    for (size_t c = 0; c < chunks_.size(); ++c) {
      Chunk& ch = chunks_[c];
      bool ic = true, oc = true;
      size_t total = 0;
      for (size_t i = ch.first; i < ch.first + ch.count; ++i) {
        offs[c].push_back(total);
        const size_t pts = props_[i]->engine().points();
        if (i > ch.first) {
          const size_t prev = props_[i - 1]->engine().points();
          // addresses compared as integers (the arrays are separate objects to the language)
          const uintptr_t step = 2 * prev * sizeof(double);
          ic = ic && reinterpret_cast<uintptr_t>(in[i]) == reinterpret_cast<uintptr_t>(in[i - 1]) + step;
          oc = oc && reinterpret_cast<uintptr_t>(out[i]) == reinterpret_cast<uintptr_t>(out[i - 1]) + step;
        }
        total += 2 * pts;
      }
      in_merged[c] = ic && ch.count > 1;
      out_merged[c] = oc && ch.count > 1;
      if ((in_merged[c] || out_merged[c]) && ch.stage.bytes < total * sizeof(double))
        ch.stage = DeviceBuffer(total * sizeof(double));
    }
    for (size_t c = 0; c < chunks_.size(); ++c) {
      Chunk& ch = chunks_[c];
      if (c > 0) cuda_check(cudaStreamWaitEvent(ch.stream, chunks_[c - 1].in_done, 0), "chunk order");
      if (in_merged[c]) {
        // adjacent addresses can still be separate allocations, which one copy may not span:
        // the call then refuses (invalid value, nothing queued) and the members go one by one
        const size_t last = ch.first + ch.count - 1;
        const size_t bytes = (offs[c].back() + 2 * props_[last]->engine().points()) * sizeof(double);
        const cudaError_t e = cudaMemcpyAsync(ch.stage.ptr, in[ch.first], bytes, cudaMemcpyHostToDevice, ch.stream);
        if (e == cudaErrorInvalidValue) {
          cudaGetLastError();
          in_merged[c] = 0;
        } else {
          cuda_check(e, "chunk copy in");
        }
      }
      if (!in_merged[c])
        for (size_t i = ch.first; i < ch.first + ch.count; ++i) props_[i]->engine().stage_in(in[i]);
      cuda_check(cudaEventRecord(ch.in_done, ch.stream), "chunk event");
    }
    mark("copies in queued");
    for (size_t c = 0; c < chunks_.size(); ++c) {
      Chunk& ch = chunks_[c];
      for (size_t i = ch.first; i < ch.first + ch.count; ++i) {
        if (in_merged[c])
          props_[i]->engine().import_device(ch.stage.as<double>() + offs[c][i - ch.first]);
        else
          props_[i]->engine().unstage_in();
        props_[i]->state_replaced();
      }
      ch.batch->steps(n, false, false);  // queued behind the chunk's imports; no host wait
      for (size_t i = ch.first; i < ch.first + ch.count; ++i) {
        if (out_merged[c])
          props_[i]->engine().export_device(ch.stage.as<double>() + offs[c][i - ch.first]);
        else
          props_[i]->engine().stage_out();
      }
      mark("chunk steps queued");
      if (c > 0) cuda_check(cudaStreamWaitEvent(ch.stream, chunks_[c - 1].out_done, 0), "chunk order");
      if (out_merged[c]) {
        const size_t last = ch.first + ch.count - 1;
        const size_t bytes = (offs[c].back() + 2 * props_[last]->engine().points()) * sizeof(double);
        const cudaError_t e = cudaMemcpyAsync(out[ch.first], ch.stage.ptr, bytes, cudaMemcpyDeviceToHost, ch.stream);
        if (e == cudaErrorInvalidValue) {
          // separate allocations after all: one copy per member out of the chunk's buffer
          cudaGetLastError();
          for (size_t i = ch.first; i < ch.first + ch.count; ++i)
            cuda_check(cudaMemcpyAsync(out[i], ch.stage.as<double>() + offs[c][i - ch.first],
                                       2 * props_[i]->engine().points() * sizeof(double), cudaMemcpyDeviceToHost,
                                       ch.stream),
                       "chunk copy out");
        } else {
          cuda_check(e, "chunk copy out");
        }
      } else {
        for (size_t i = ch.first; i < ch.first + ch.count; ++i) props_[i]->engine().unstage_out(out[i]);
      }
      cuda_check(cudaEventRecord(ch.out_done, ch.stream), "chunk event");
      mark("chunk copies out queued");
    }
    for (Chunk& ch : chunks_) {
      cuda_check(cudaStreamSynchronize(ch.stream), "chunk sync");
      mark("chunk done");
    }
  } catch (...) {
    for (size_t i = 0; i < m; ++i) props_[i]->engine().stream = own[i];
    throw;
  }
  for (size_t i = 0; i < m; ++i) props_[i]->engine().stream = own[i];
  if (trace) {
    std::string line = "steps_host:";
    for (const auto& mk : marks) line += " " + mk.first + " " + std::to_string(mk.second) + " ms;";
    std::fprintf(stderr, "%s\n", line.c_str());
  }
}

std::string Batch::tune(const std::string& cache_path, int trial_steps) {
  if (trial_steps < 1) throw Error(SO_ERR_INVALID, "tuning needs at least one step per candidate");
  // the schedule classes present: (kind, n, mode) from one recorded step pair of every member
  std::map<std::tuple<int, int64_t, int>, std::vector<std::pair<int, int>>> cands;
  for (Propagation* p : props_)
    for (const RecordedPass& r : p->record_steps(2)) {
      if (r.kind == RecordedPass::TensorCore) {
        const int mode = (r.threads >> 17) & 3;
        // (CTAs per SM, blocked order); the first candidate is the built-in default
        cands[{1, r.p.g.n, mode}] = {{2, 1}, {2, 0}, {1, 1}, {1, 0}};
      } else if (r.kind == RecordedPass::Generic && r.p.fused && r.real == kRealF32) {
        // (threads per CTA, radix); lanes of n points need 16 threads >= n
        std::vector<std::pair<int, int>> v{{fft_pair_threads(r.p.g), 16}};
        for (int t : {128, 256, 512})
          for (int rd : {16, 8})
            if ((int64_t)16 * t >= r.p.g.n && !(t == v[0].first && rd == 16)) v.push_back({t, rd});
        cands[{0, r.p.g.n, 0}] = v;
      }
    }
  if (cands.empty()) throw Error(SO_ERR_UNSUPPORTED, "the batch has no FFT-pair or tensor-core passes to tune");
  size_t trials = 0;
  for (const auto& kv : cands) trials = std::max(trials, kv.second.size());
  // the members' states, restored once the trials are done
  std::vector<std::vector<unsigned char>> saved;
  for (Propagation* p : props_) saved.push_back(p->checkpoint());
  std::map<std::tuple<int, int64_t, int>, std::vector<double>> ms;  // per class, per candidate
  const bool timing_was = timing_;
  auto apply = [&](const std::tuple<int, int64_t, int>& k, std::pair<int, int> c) {
    if (std::get<0>(k) == 1)
      set_tc_schedule(std::get<1>(k), std::get<2>(k), TcSchedule{c.first, c.second});
    else
      set_pair_schedule(std::get<1>(k), false, PairSchedule{c.first, c.second});
  };
  try {
    for (size_t t = 0; t < trials; ++t) {
      for (const auto& kv : cands) apply(kv.first, kv.second[t % kv.second.size()]);
      timing_ = true;
      timed_.clear();
      steps(1);  // the new launch shapes are built and warm
      kernel_times();
      steps((uint64_t)trial_steps);
      cuda_check(cudaStreamSynchronize(stream_), "batch sync");
      std::map<std::tuple<int, int64_t, int>, double> acc;
      for (Timed& tm : timed_) {
        float e = 0.f;
        cuda_check(cudaEventElapsedTime(&e, tm.a, tm.b), "event elapsed");
        if (tm.cls_kind >= 0) acc[{tm.cls_kind, tm.cls_n, tm.cls_mode}] += e;
        cudaEventDestroy(tm.a);
        cudaEventDestroy(tm.b);
      }
      timed_.clear();
      for (const auto& kv : cands)
        if (t < kv.second.size()) ms[kv.first].push_back(acc[kv.first]);
    }
  } catch (...) {
    timing_ = timing_was;
    for (size_t i = 0; i < props_.size(); ++i) props_[i]->restore(saved[i].data(), saved[i].size());
    throw;
  }
  timing_ = timing_was;
  // winners, and the report
  std::string rep = "{\"trial_steps\": " + std::to_string(trial_steps) + ", \"classes\": [";
  double def_total = 0.0, best_total = 0.0;
  bool first = true;
  for (const auto& kv : cands) {
    const std::vector<double>& v = ms[kv.first];
    size_t best = 0;
    for (size_t i = 1; i < v.size(); ++i)
      if (v[i] < v[best]) best = i;
    apply(kv.first, kv.second[best]);
    def_total += v[0];
    best_total += v[best];
    const bool tc = std::get<0>(kv.first) == 1;
    rep += std::string(first ? "" : ", ") + "{\"pass\": \"" + (tc ? "tensor_core" : "fft_pair") +
           "\", \"n\": " + std::to_string(std::get<1>(kv.first)) + ", \"mode\": " +
           std::to_string(std::get<2>(kv.first)) + ", \"candidates\": [";
    for (size_t i = 0; i < v.size(); ++i)
      rep += std::string(i ? ", " : "") + "{\"" + (tc ? "ctas_per_sm" : "threads") + "\": " +
             std::to_string(kv.second[i].first) + ", \"" + (tc ? "blocked" : "radix") + "\": " +
             std::to_string(kv.second[i].second) + ", \"ms\": " + std::to_string(v[i]) + "}";
    rep += "], \"chosen\": " + std::to_string(best) + "}";
    first = false;
  }
  rep += "], \"default_ms\": " + std::to_string(def_total) + ", \"tuned_ms\": " + std::to_string(best_total) +
         ", \"schedules\": " + schedules_json() + "}";
  for (size_t i = 0; i < props_.size(); ++i) props_[i]->restore(saved[i].data(), saved[i].size());
  if (!cache_path.empty()) {
    FILE* f = std::fopen(cache_path.c_str(), "w");
    if (!f) throw Error(SO_ERR_IO, "cannot write the schedule cache " + cache_path);
    const std::string js = schedules_json();
    const bool ok = std::fwrite(js.data(), 1, js.size(), f) == js.size();
    if (std::fclose(f) != 0 || !ok) throw Error(SO_ERR_IO, "cannot write the schedule cache " + cache_path);
  }
  return rep;
}

std::string Batch::kernel_times() {
  cuda_check(cudaStreamSynchronize(stream_), "batch sync");
  std::map<std::string, std::tuple<int, double, double>> acc;
  std::vector<std::string> order;
  for (Timed& t : timed_) {
    float ms = 0.f;
    cuda_check(cudaEventElapsedTime(&ms, t.a, t.b), "event elapsed");
    if (!acc.count(t.name)) order.push_back(t.name);
    auto& a = acc[t.name];
    std::get<0>(a) += 1;
    std::get<1>(a) += ms;
    std::get<2>(a) += t.bytes;
    cudaEventDestroy(t.a);
    cudaEventDestroy(t.b);
  }
  timed_.clear();
  std::string out;
  for (const std::string& k : order) {
    const auto& a = acc[k];
    out += k + "\t" + std::to_string(std::get<0>(a)) + "\t" + std::to_string(std::get<1>(a)) + "\t" +
           std::to_string(std::get<2>(a)) + "\n";
  }
  return out;
}

const char* op_kind_name(int k) {
  switch (k) {
    case OP_DIAG1D: return "diag1d";
    case OP_DIAGND: return "diagnd";
    case OP_FFT: return "fft";
    case OP_MAT: return "mat";
    case OP_MAT_LANE: return "mat_lane";
    case OP_MAT_SLICE: return "mat_slice";
    case OP_NORM: return "norm";
    case OP_COPY: return "copy";
    case OP_LOSS: return "loss";
    case OP_SCALE: return "scale";
    case OP_SETC: return "setc";
    case OP_RECORD: return "record";
    case OP_DOT: return "dot";
  }
  return "?";
}

std::string Propagation::describe() {
  // Record two steps and group them the way Engine::submit would.
  std::vector<Action> rec;
  std::vector<std::function<void()>> calls;
  Emitter em{wf_->eng.get(), &rec, &calls};
  // describe() must not change observable state: run on a copy of the host-side flags only
  const bool pnc = wf_->possible_norm_change;
  const auto names = wf_->last_grid_names;
  const auto grids = wf_->grids;
  std::vector<Grid> trans_grids;
  for (auto& e : stack_->stack)
    if (Grid* g = e.op->grid_transformation()) trans_grids.push_back(*g);
  std::vector<size_t> frames;
  for (auto& e : stack_->stack)
    if (auto* s = dynamic_cast<StateSaver*>(e.op.get())) frames.push_back(s->current_frame);
  std::vector<std::vector<double>> times;
  for (auto& e : stack_->stack)
    if (auto* s = dynamic_cast<StateSaver*>(e.op.get())) times.push_back(s->times);
  step(em);
  step(em);
  wf_->possible_norm_change = pnc;
  wf_->last_grid_names = names;
  wf_->grids = grids;
  size_t ti = 0, fi = 0, tmi = 0;
  for (auto& e : stack_->stack)
    if (Grid* g = e.op->grid_transformation()) *g = trans_grids[ti++];
  for (auto& e : stack_->stack)
    if (auto* s = dynamic_cast<StateSaver*>(e.op.get())) {
      s->current_frame = frames[fi++];
      s->times = times[tmi++];
    }
  std::string out = wf_->eng->resident_capable() ? "resident " : "sweep ";
  out += "perm=";
  for (int p : wf_->eng->perm) out += std::to_string(p);
  out += "\n";
  int axis = -1;
  std::vector<int> written;
  int nops = 0;
  std::string cur;
  auto close = [&]() {
    if (nops) out += "pass axis=" + std::to_string(axis) + ": " + cur + "\n";
    cur.clear();
    nops = 0;
    axis = -1;
    written.clear();
  };
  for (const Action& a : rec) {
    if (a.host_call >= 0) {
      close();
      out += "host\n";
      continue;
    }
    if (!wf_->eng->resident_capable()) {
      if (a.lane_axis >= 0 && axis >= 0 && axis != a.lane_axis) close();
      if (a.op.kind == OP_SCALE)
        for (int w : written)
          if (w == a.op.b || w == a.op.c) {
            close();
            break;
          }
    }
    if (a.lane_axis >= 0) axis = a.lane_axis;
    if (a.op.kind == OP_NORM || a.op.kind == OP_COPY || a.op.kind == OP_LOSS || a.op.kind == OP_SETC)
      written.push_back(a.op.a);
    cur += op_kind_name(a.op.kind);
    if (a.lane_axis >= 0) cur += "@" + std::to_string(a.lane_axis);
    cur += " ";
    ++nops;
  }
  close();
  return out;
}

}  // namespace so
