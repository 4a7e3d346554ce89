// Launch schedules of the two passes of the batched step, per lane extent: the radial
// FFT-pair pass (threads per CTA, which sets the lanes per tile, and the radix of its Stockham
// stages) and the angular tensor-core pass (persistent CTAs per SM, tile order).  The
// autotuner (Batch::tune) measures the candidates on the live workload and writes the winners
// here; a JSON cache file carries them to later processes.  Unset entries mean the built-in
// defaults.  The reference has no counterpart: it runs rustfft / ndarray over rayon lanes
// (fft_transformation.rs:59-68, matrix_transformation.rs:64-65) with no launch shape to pick.
#include <atomic>
#include <cstdio>
#include <cstring>
#include <map>
#include <mutex>
#include <sstream>
#include <string>
#include <tuple>

#include "common.cuh"

namespace so {

namespace {
std::mutex g_mu;
std::map<std::pair<int64_t, int>, PairSchedule> g_pair;           // (n, fp64)
std::map<std::pair<int64_t, int>, TcSchedule> g_tc;               // (n, operand mode)
std::atomic<uint64_t> g_epoch{1};
}  // namespace

PairSchedule pair_schedule(int64_t n, bool fp64) {
  std::lock_guard<std::mutex> l(g_mu);
  auto it = g_pair.find({n, fp64 ? 1 : 0});
  return it == g_pair.end() ? PairSchedule{0, 0} : it->second;
}

TcSchedule tc_schedule(int64_t n, int mode) {
  std::lock_guard<std::mutex> l(g_mu);
  auto it = g_tc.find({n, mode});
  // built in: the default CTAs per SM, blocked tile order (runs of one member's tiles)
  return it == g_tc.end() ? TcSchedule{0, 1} : it->second;
}

void set_pair_schedule(int64_t n, bool fp64, PairSchedule s) {
  std::lock_guard<std::mutex> l(g_mu);
  g_pair[{n, fp64 ? 1 : 0}] = s;
  ++g_epoch;
}

void set_tc_schedule(int64_t n, int mode, TcSchedule s) {
  std::lock_guard<std::mutex> l(g_mu);
  g_tc[{n, mode}] = s;
  ++g_epoch;
}

void reset_schedules() {
  std::lock_guard<std::mutex> l(g_mu);
  g_pair.clear();
  g_tc.clear();
  ++g_epoch;
}

uint64_t schedule_epoch() { return g_epoch.load(); }

std::string schedules_json() {
  std::lock_guard<std::mutex> l(g_mu);
  std::ostringstream o;
  o << "{\"fft_pair\": [";
  bool first = true;
  for (const auto& kv : g_pair) {
    o << (first ? "" : ", ") << "{\"n\": " << kv.first.first << ", \"fp64\": " << kv.first.second
      << ", \"threads\": " << kv.second.threads << ", \"radix\": " << kv.second.radix << "}";
    first = false;
  }
  o << "], \"tensor_core\": [";
  first = true;
  for (const auto& kv : g_tc) {
    o << (first ? "" : ", ") << "{\"n\": " << kv.first.first << ", \"mode\": " << kv.first.second
      << ", \"ctas_per_sm\": " << kv.second.ctas_per_sm << ", \"blocked\": " << kv.second.blocked << "}";
    first = false;
  }
  o << "]}";
  return o.str();
}

// The cache file is the JSON above (written by schedules_json); this reader takes exactly
// that shape: objects of integer fields inside the two arrays.
bool schedules_from_json(const std::string& text) {
  auto section = [&](const char* key) -> std::string {
    const size_t k = text.find(std::string("\"") + key + "\"");
    if (k == std::string::npos) return "";
    const size_t a = text.find('[', k), b = text.find(']', k);
    if (a == std::string::npos || b == std::string::npos || b < a) return "";
    return text.substr(a + 1, b - a - 1);
  };
  auto field = [](const std::string& obj, const char* name, long long& out) {
    const size_t k = obj.find(std::string("\"") + name + "\"");
    if (k == std::string::npos) return false;
    const size_t c = obj.find(':', k);
    if (c == std::string::npos) return false;
    return std::sscanf(obj.c_str() + c + 1, "%lld", &out) == 1;
  };
  auto objects = [](const std::string& s) {
    std::vector<std::string> v;
    size_t p = 0;
    while ((p = s.find('{', p)) != std::string::npos) {
      const size_t q = s.find('}', p);
      if (q == std::string::npos) break;
      v.push_back(s.substr(p, q - p + 1));
      p = q + 1;
    }
    return v;
  };
  std::map<std::pair<int64_t, int>, PairSchedule> pair;
  std::map<std::pair<int64_t, int>, TcSchedule> tc;
  for (const std::string& o : objects(section("fft_pair"))) {
    long long n, f, t, r;
    if (!field(o, "n", n) || !field(o, "fp64", f) || !field(o, "threads", t) || !field(o, "radix", r)) return false;
    pair[{(int64_t)n, (int)f}] = PairSchedule{(int)t, (int)r};
  }
  for (const std::string& o : objects(section("tensor_core"))) {
    long long n, m, c, b;
    if (!field(o, "n", n) || !field(o, "mode", m) || !field(o, "ctas_per_sm", c) || !field(o, "blocked", b))
      return false;
    tc[{(int64_t)n, (int)m}] = TcSchedule{(int)c, (int)b};
  }
  std::lock_guard<std::mutex> l(g_mu);
  for (const auto& kv : pair) g_pair[kv.first] = kv.second;
  for (const auto& kv : tc) g_tc[kv.first] = kv.second;
  ++g_epoch;
  return true;
}

}  // namespace so
