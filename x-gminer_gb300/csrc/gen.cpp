// Seeded synthetic graph generators (host C++).
//
// These produce the raw edge samples that the benchmark workloads are built from:
// R-MAT, Erdos-Renyi G(n,m), Chung-Lu power law and Barabasi-Albert (single and
// batched).  The reference ships no generator for these families
// (scripts/graph_generator.py only wraps NetworkX); its binary CSR format is what
// the counting path consumes (scripts/graph_format_conversion.py:47-80), and
// that format is produced from these samples by the CSR build (symmetrise,
// dedupe, drop self-loops, sort) in csr_build.cu.
//
// Every random draw is a pure function of (seed, stream, counter) through
// splitmix64, and the floating-point steps (Chung-Lu weights, BA batch sizes) avoid
// libm (DetPow), so every generator gives the same samples on x86-64 and aarch64 and
// for any thread count.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <thread>
#include <vector>

#include "../../include/xgm.h"

namespace {

inline uint64_t mix64(uint64_t x) {
  x += 0x9E3779B97F4A7C15ull;
  x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
  x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
  return x ^ (x >> 31);
}

// Counter-based draw: stream separates independent uses of one seed.
inline uint64_t draw(uint64_t seed, uint64_t stream, uint64_t counter) {
  return mix64(mix64(seed ^ (stream * 0xD1B54A32D192ED03ull)) + counter);
}

// Uniform integer in [0, n) for n <= 2^32 (multiply-high on the top 32 bits).
inline uint64_t below(uint64_t x, uint64_t n) { return ((x >> 32) * n) >> 32; }

// Uniform double in [0, 1) with 53 random bits.
inline double unit(uint64_t x) { return double(x >> 11) * (1.0 / 9007199254740992.0); }

template <class F>
void parallel_for(int64_t n, F f, int64_t min_parallel = int64_t(1) << 16) {
  unsigned hw = std::thread::hardware_concurrency();
  int64_t nt = hw ? hw : 1;
  if (nt > 64) nt = 64;
  if (n < min_parallel) nt = 1;
  if (nt == 1) { f(0, n); return; }
  std::vector<std::thread> th;
  int64_t chunk = (n + nt - 1) / nt;
  for (int64_t t = 0; t < nt; ++t) {
    int64_t lo = t * chunk, hi = std::min(n, lo + chunk);
    if (lo >= hi) break;
    th.emplace_back([=] { f(lo, hi); });
  }
  for (auto& x : th) x.join();
}

// pow / exp / log from correctly rounded IEEE operations only (+ - * / sqrt, frexp,
// ldexp, floor): ln from the atanh series of the mantissa, exp from a Taylor series
// after reduction by ln 2.  libm's versions may differ in the last bit between
// platforms; these give the same bits on every host (host code is built without
// floating-point contraction).
struct DetPow {
  static constexpr double kLn2 = 0.693147180559945309417232121458176568;
  double inv[48];
  DetPow() { for (int k = 1; k < 48; ++k) inv[k] = 1.0 / double(k); }
  double log(double x) const {  // x > 0, finite
    int e = 0;
    double m = std::frexp(x, &e);  // m in [0.5, 1)
    if (m < 0.70710678118654752440) { m = m * 2.0; e -= 1; }
    const double s = (m - 1.0) / (m + 1.0), s2 = s * s;
    double term = s, sum = 0.0;
    for (int k = 1; k <= 25; k += 2) { sum = sum + term * inv[k]; term = term * s2; }
    return 2.0 * sum + double(e) * kLn2;
  }
  double exp(double y) const {  // |y| < 700
    const double kf = std::floor(y / kLn2 + 0.5);
    const double r = y - kf * kLn2;
    double term = 1.0, sum = 1.0;
    for (int i = 1; i <= 18; ++i) { term = term * r * inv[i]; sum = sum + term; }
    return std::ldexp(sum, int(kf));
  }
  double pow(double x, double y) const { return exp(y * log(x)); }
};

// Sum of f(i) over [0, n) in 64 fixed index chunks added in order (any thread count).
template <class F>
double det_sum(int64_t n, F f) {
  const int64_t chunks = 64, step = (n + chunks - 1) / chunks;
  std::vector<double> part(chunks, 0.0);
  parallel_for(chunks, [&](int64_t lo, int64_t hi) {
    for (int64_t c = lo; c < hi; ++c) {
      double s = 0.0;
      for (int64_t i = c * step; i < std::min(n, (c + 1) * step); ++i) s = s + f(i);
      part[c] = s;
    }
  }, n >= (int64_t(1) << 16) ? 1 : chunks + 1);
  double s = 0.0;
  for (double p : part) s = s + p;
  return s;
}

}  // namespace

extern "C" {

int64_t xgm_gen_rmat(int scale, int edge_factor, double a, double b, double c,
                     uint64_t seed, int32_t* src, int32_t* dst) {
  if (scale <= 0 || scale > 30 || edge_factor <= 0) return -1;
  if (a < 0 || b < 0 || c < 0 || a + b + c > 1.0) return -1;
  const int64_t m = int64_t(edge_factor) << scale;
  if (!src || !dst) return m;
  // Quadrant thresholds on a 32-bit uniform: exact products of IEEE doubles.
  const uint64_t ta = uint64_t(a * 4294967296.0);
  const uint64_t tb = uint64_t((a + b) * 4294967296.0);
  const uint64_t tc = uint64_t((a + b + c) * 4294967296.0);
  const int words = (scale + 1) / 2;  // two 32-bit levels per 64-bit draw
  parallel_for(m, [&](int64_t lo, int64_t hi) {
    for (int64_t i = lo; i < hi; ++i) {
      uint32_t u = 0, v = 0;
      for (int w = 0; w < words; ++w) {
        uint64_t x = draw(seed, 1, uint64_t(i) * words + w);
        for (int h = 0; h < 2; ++h) {
          int level = 2 * w + h;
          if (level >= scale) break;
          uint64_t r = h ? (x & 0xFFFFFFFFull) : (x >> 32);
          uint32_t bu, bv;
          if (r < ta) { bu = 0; bv = 0; }
          else if (r < tb) { bu = 0; bv = 1; }
          else if (r < tc) { bu = 1; bv = 0; }
          else { bu = 1; bv = 1; }
          u = (u << 1) | bu;
          v = (v << 1) | bv;
        }
      }
      src[i] = int32_t(u);
      dst[i] = int32_t(v);
    }
  });
  return m;
}

int64_t xgm_gen_er(int64_t n, int64_t m, uint64_t seed, int32_t* src, int32_t* dst) {
  if (n <= 1 || n > (int64_t(1) << 31) - 1 || m < 0) return -1;
  if (!src || !dst) return m;
  parallel_for(m, [&](int64_t lo, int64_t hi) {
    for (int64_t i = lo; i < hi; ++i) {
      src[i] = int32_t(below(draw(seed, 2, 2 * uint64_t(i)), uint64_t(n)));
      dst[i] = int32_t(below(draw(seed, 2, 2 * uint64_t(i) + 1), uint64_t(n)));
    }
  });
  return m;
}

// Chung-Lu: expected degree of vertex i is w_i = w_max * ((i + i0) / i0)^(-1/(gamma-1)),
// with i0 chosen so that the mean weight is avg_deg.  m = n*avg_deg/2 endpoint pairs
// are drawn with probability proportional to weight (inverse CDF).  The weights use
// DetPow and det_sum, so the samples are the same on every host.
int64_t xgm_gen_chung_lu(int64_t n, double gamma, double w_max, double avg_deg,
                         uint64_t seed, int32_t* src, int32_t* dst) {
  if (n <= 1 || n > (int64_t(1) << 31) - 1 || gamma <= 1.0 || w_max <= 0 || avg_deg <= 0)
    return -1;
  const int64_t m = int64_t(double(n) * avg_deg / 2.0);
  if (!src || !dst) return m;
  const double beta = 1.0 / (gamma - 1.0);
  const DetPow dp;
  auto weight = [&](int64_t i, double i0) {
    return w_max * dp.pow((double(i) + i0) / i0, -beta);
  };
  // mean weight grows with i0; bisect on log(i0).
  double lo = 1e-3, hi = double(n) * 1e3;
  for (int it = 0; it < 64; ++it) {
    const double mid = std::sqrt(lo * hi);
    const double mean = det_sum(n, [&](int64_t i) { return weight(i, mid); }) / double(n);
    if (mean < avg_deg) lo = mid; else hi = mid;
  }
  const double i0 = std::sqrt(lo * hi);
  std::vector<double> cdf(n);
  parallel_for(n, [&](int64_t a, int64_t b) {
    for (int64_t i = a; i < b; ++i) cdf[i] = weight(i, i0);
  });
  double acc = 0;
  for (int64_t i = 0; i < n; ++i) {
    acc = acc + cdf[i];
    cdf[i] = acc;
  }
  const double total = acc;
  parallel_for(m, [&](int64_t lo2, int64_t hi2) {
    for (int64_t e = lo2; e < hi2; ++e) {
      for (int side = 0; side < 2; ++side) {
        double r = unit(draw(seed, 3, 2 * uint64_t(e) + side)) * total;
        int64_t k = std::upper_bound(cdf.begin(), cdf.end(), r) - cdf.begin();
        if (k >= n) k = n - 1;
        (side ? dst : src)[e] = int32_t(k);
      }
    }
  });
  return m;
}

// Barabasi-Albert preferential attachment: vertices 0..m-1 start unconnected and are
// the first targets; each later vertex attaches to m distinct vertices drawn from the
// list in which every vertex appears once per incident edge (and the initial targets
// once).  Writes m*(n-m) edges with ids offset by `base`.
static int64_t ba_one(int64_t n, int m, uint64_t seed, int64_t base, int32_t* src,
                      int32_t* dst) {
  if (m < 1 || n <= m) return -1;
  const int64_t ne = int64_t(m) * (n - m);
  if (!src || !dst) return ne;
  std::vector<int32_t> rep;
  rep.reserve(size_t(2 * ne + m));
  std::vector<int32_t> targets(m);
  for (int i = 0; i < m; ++i) targets[i] = i;
  uint64_t ctr = 0;
  int64_t out = 0;
  for (int64_t s = m; s < n; ++s) {
    for (int i = 0; i < m; ++i) {
      src[out] = int32_t(base + s);
      dst[out] = int32_t(base + targets[i]);
      ++out;
      rep.push_back(targets[i]);
      rep.push_back(int32_t(s));
    }
    // draw m distinct targets for the next vertex
    int got = 0;
    while (got < m) {
      int32_t t = rep[below(draw(seed, 4, ctr++), rep.size())];
      bool dup = false;
      for (int k = 0; k < got; ++k) dup |= (targets[k] == t);
      if (!dup) targets[got++] = t;
    }
  }
  return ne;
}

int64_t xgm_gen_ba(int64_t n, int m, uint64_t seed, int32_t* src, int32_t* dst) {
  if (n > (int64_t(1) << 31) - 1) return -1;
  return ba_one(n, m, seed, 0, src, dst);
}

// A batch of BA graphs: graph g has n_g = round(exp(U[ln n_lo, ln n_hi])) vertices and
// attaches m_g ~ U{m_lo..m_hi} edges per new vertex.  Vertex ids are global (graph g
// owns [vtx_off[g], vtx_off[g+1])) and edges are written graph after graph
// (graph g owns edge samples [edge_off[g], edge_off[g+1])).  Call with src == NULL to
// get the offsets (both arrays have num_graphs + 1 entries) and the total sample count.
int64_t xgm_gen_ba_batch(int num_graphs, int64_t n_lo, int64_t n_hi, int m_lo, int m_hi,
                         uint64_t seed, int64_t* vtx_off, int64_t* edge_off, int32_t* src,
                         int32_t* dst) {
  if (num_graphs <= 0 || n_lo < 2 || n_hi < n_lo || m_lo < 1 || m_hi < m_lo ||
      n_lo <= m_hi || !vtx_off || !edge_off)
    return -1;
  std::vector<int64_t> ns(num_graphs);
  std::vector<int> ms(num_graphs);
  const DetPow dp;
  const double l0 = dp.log(double(n_lo)), l1 = dp.log(double(n_hi));
  vtx_off[0] = 0;
  edge_off[0] = 0;
  for (int g = 0; g < num_graphs; ++g) {
    double u = unit(draw(seed, 5, 2 * uint64_t(g)));
    int64_t n = int64_t(std::floor(dp.exp(l0 + u * (l1 - l0)) + 0.5));
    n = std::min(std::max(n, n_lo), n_hi);
    int m = m_lo + int(below(draw(seed, 5, 2 * uint64_t(g) + 1), uint64_t(m_hi - m_lo + 1)));
    ns[g] = n;
    ms[g] = m;
    vtx_off[g + 1] = vtx_off[g] + n;
    edge_off[g + 1] = edge_off[g] + int64_t(m) * (n - m);
  }
  if (vtx_off[num_graphs] > (int64_t(1) << 31) - 1) return -1;
  if (!src || !dst) return edge_off[num_graphs];
  std::vector<std::thread> th;
  unsigned hw = std::thread::hardware_concurrency();
  int nt = std::max(1u, std::min(hw ? hw : 1u, 64u));
  for (int t = 0; t < nt; ++t) {
    th.emplace_back([&, t] {
      for (int g = t; g < num_graphs; g += nt)
        ba_one(ns[g], ms[g], draw(seed, 6, uint64_t(g)), vtx_off[g], src + edge_off[g],
               dst + edge_off[g]);
    });
  }
  for (auto& x : th) x.join();
  return edge_off[num_graphs];
}

}  // extern "C"
