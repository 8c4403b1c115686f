/*
 * gen.c - seeded synthetic graph generators for the oracle side.
 *
 * TEST INFRASTRUCTURE ONLY (part of liborc.so).  The tests and the CPU legs of
 * bench.py (cpu_baseline, --impl reference) build their graphs here, so that timing
 * the reference's CPU algorithm never loads the engine's library.  The samples are
 * bit-identical to the engine's host generators (x-gminer_gb300/csrc/gen.cpp); a CPU
 * test compares the two on every family.  The reference itself ships no generator
 * for these families (scripts/graph_generator.py wraps NetworkX).
 *
 * Every draw is a pure function of (seed, stream, counter) through splitmix64, and
 * the floating-point steps use only correctly rounded IEEE operations in a fixed
 * order (this file is built with -ffp-contract=off), so x86-64 and aarch64 hosts and
 * any thread count give the same samples.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

static inline uint64_t g_mix64(uint64_t x) {
  x += 0x9E3779B97F4A7C15ull;
  x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
  x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
  return x ^ (x >> 31);
}
static inline uint64_t g_draw(uint64_t seed, uint64_t stream, uint64_t ctr) {
  return g_mix64(g_mix64(seed ^ (stream * 0xD1B54A32D192ED03ull)) + ctr);
}
static inline uint64_t g_below(uint64_t x, uint64_t n) { return ((x >> 32) * n) >> 32; }
static inline double g_unit(uint64_t x) {
  return (double)(x >> 11) * (1.0 / 9007199254740992.0);
}

/* ln and exp from series (atanh of the mantissa; Taylor after reduction by ln 2). */
static const double G_LN2 = 0.693147180559945309417232121458176568;
static double g_inv[48];
static void g_inv_init(void) {
  for (int k = 1; k < 48; ++k) g_inv[k] = 1.0 / (double)k;
}
static double g_log(double x) {
  int e = 0;
  double m = frexp(x, &e);
  if (m < 0.70710678118654752440) { m = m * 2.0; e -= 1; }
  double s = (m - 1.0) / (m + 1.0), s2 = s * s, term = s, sum = 0.0;
  for (int k = 1; k <= 25; k += 2) { sum = sum + term * g_inv[k]; term = term * s2; }
  return 2.0 * sum + (double)e * G_LN2;
}
static double g_exp(double y) {
  double kf = floor(y / G_LN2 + 0.5);
  double r = y - kf * G_LN2, term = 1.0, sum = 1.0;
  for (int i = 1; i <= 18; ++i) { term = term * r * g_inv[i]; sum = sum + term; }
  return ldexp(sum, (int)kf);
}

int64_t orc_gen_rmat(int scale, int edge_factor, double a, double b, double c, uint64_t seed,
                     int32_t* src, int32_t* dst) {
  if (scale <= 0 || scale > 30 || edge_factor <= 0) return -1;
  if (a < 0 || b < 0 || c < 0 || a + b + c > 1.0) return -1;
  const int64_t m = (int64_t)edge_factor << scale;
  if (!src || !dst) return m;
  const uint64_t ta = (uint64_t)(a * 4294967296.0);
  const uint64_t tb = (uint64_t)((a + b) * 4294967296.0);
  const uint64_t tc = (uint64_t)((a + b + c) * 4294967296.0);
  const int words = (scale + 1) / 2;
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < m; ++i) {
    uint32_t u = 0, v = 0;
    for (int lvl = 0; lvl < scale; ++lvl) {
      uint64_t x = g_draw(seed, 1, (uint64_t)i * words + (uint64_t)(lvl / 2));
      uint64_t r = (lvl & 1) ? (x & 0xFFFFFFFFull) : (x >> 32);
      uint32_t q = r < ta ? 0u : r < tb ? 1u : r < tc ? 2u : 3u; /* quadrant (bu, bv) */
      u = (u << 1) | (q >> 1);
      v = (v << 1) | (q & 1u);
    }
    src[i] = (int32_t)u;
    dst[i] = (int32_t)v;
  }
  return m;
}

int64_t orc_gen_er(int64_t n, int64_t m, uint64_t seed, int32_t* src, int32_t* dst) {
  if (n <= 1 || n > ((int64_t)1 << 31) - 1 || m < 0) return -1;
  if (!src || !dst) return m;
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < m; ++i) {
    src[i] = (int32_t)g_below(g_draw(seed, 2, 2 * (uint64_t)i), (uint64_t)n);
    dst[i] = (int32_t)g_below(g_draw(seed, 2, 2 * (uint64_t)i + 1), (uint64_t)n);
  }
  return m;
}

static double cl_weight(int64_t i, double i0, double w_max, double beta) {
  return w_max * g_exp(-beta * g_log(((double)i + i0) / i0));
}

/* mean of the weights for a given i0: 64 fixed index chunks, added in order */
static double cl_mean(int64_t n, double i0, double w_max, double beta) {
  const int64_t chunks = 64, step = (n + chunks - 1) / chunks;
  double part[64];
#pragma omp parallel for schedule(static)
  for (int64_t c = 0; c < chunks; ++c) {
    double s = 0.0;
    int64_t hi = (c + 1) * step < n ? (c + 1) * step : n;
    for (int64_t i = c * step; i < hi; ++i) s = s + cl_weight(i, i0, w_max, beta);
    part[c] = s;
  }
  double s = 0.0;
  for (int c = 0; c < chunks; ++c) s = s + part[c];
  return s / (double)n;
}

/* Chung-Lu: w_i = w_max ((i + i0) / i0)^(-1/(gamma-1)), i0 bisected (64 geometric
 * steps) so the mean weight is avg_deg; m = n avg_deg / 2 endpoint pairs drawn by
 * inverse CDF over the running sum of the weights. */
int64_t orc_gen_chung_lu(int64_t n, double gamma, double w_max, double avg_deg, uint64_t seed,
                         int32_t* src, int32_t* dst) {
  if (n <= 1 || n > ((int64_t)1 << 31) - 1 || gamma <= 1.0 || w_max <= 0 || avg_deg <= 0)
    return -1;
  const int64_t m = (int64_t)((double)n * avg_deg / 2.0);
  if (!src || !dst) return m;
  g_inv_init();
  const double beta = 1.0 / (gamma - 1.0);
  double lo = 1e-3, hi = (double)n * 1e3;
  for (int it = 0; it < 64; ++it) {
    double mid = sqrt(lo * hi);
    if (cl_mean(n, mid, w_max, beta) < avg_deg) lo = mid; else hi = mid;
  }
  const double i0 = sqrt(lo * hi);
  double* cdf = (double*)malloc(sizeof(double) * (size_t)n);
  if (!cdf) return -1;
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < n; ++i) cdf[i] = cl_weight(i, i0, w_max, beta);
  double acc = 0.0;
  for (int64_t i = 0; i < n; ++i) { acc = acc + cdf[i]; cdf[i] = acc; }
  const double total = acc;
#pragma omp parallel for schedule(static)
  for (int64_t e = 0; e < m; ++e) {
    for (int side = 0; side < 2; ++side) {
      double r = g_unit(g_draw(seed, 3, 2 * (uint64_t)e + (uint64_t)side)) * total;
      int64_t l = 0, h = n; /* first index with cdf > r */
      while (l < h) {
        int64_t mid = l + (h - l) / 2;
        if (cdf[mid] > r) h = mid; else l = mid + 1;
      }
      if (l >= n) l = n - 1;
      (side ? dst : src)[e] = (int32_t)l;
    }
  }
  free(cdf);
  return m;
}

/* Barabasi-Albert: vertices 0..m-1 are the first targets; vertex s (s >= m) links to
 * the current m targets, then m distinct targets for s + 1 are drawn from the list
 * holding both endpoints of every edge so far. */
static int64_t ba_graph(int64_t n, int m, uint64_t seed, int64_t base, int32_t* src,
                        int32_t* dst) {
  if (m < 1 || n <= m) return -1;
  const int64_t ne = (int64_t)m * (n - m);
  if (!src || !dst) return ne;
  int32_t* rep = (int32_t*)malloc(sizeof(int32_t) * (size_t)(2 * ne + 1));
  int32_t* tg = (int32_t*)malloc(sizeof(int32_t) * (size_t)m);
  if (!rep || !tg) { free(rep); free(tg); return -1; }
  for (int i = 0; i < m; ++i) tg[i] = i;
  int64_t nrep = 0, out = 0;
  uint64_t ctr = 0;
  for (int64_t s = m; s < n; ++s) {
    for (int i = 0; i < m; ++i) {
      src[out] = (int32_t)(base + s);
      dst[out] = (int32_t)(base + tg[i]);
      ++out;
      rep[nrep++] = tg[i];
      rep[nrep++] = (int32_t)s;
    }
    int got = 0;
    while (got < m) {
      int32_t t = rep[g_below(g_draw(seed, 4, ctr++), (uint64_t)nrep)];
      int dup = 0;
      for (int k = 0; k < got; ++k) dup |= (tg[k] == t);
      if (!dup) tg[got++] = t;
    }
  }
  free(rep);
  free(tg);
  return ne;
}

int64_t orc_gen_ba(int64_t n, int m, uint64_t seed, int32_t* src, int32_t* dst) {
  if (n > ((int64_t)1 << 31) - 1) return -1;
  return ba_graph(n, m, seed, 0, src, dst);
}

/* Batch: graph g has n_g = round(exp(U[ln n_lo, ln n_hi])) vertices and m_g ~
 * U{m_lo..m_hi}; ids are global, edges graph after graph (offset tables of
 * num_graphs + 1 entries; src == NULL returns the sample count). */
int64_t orc_gen_ba_batch(int num_graphs, int64_t n_lo, int64_t n_hi, int m_lo, int m_hi,
                         uint64_t seed, int64_t* vtx_off, int64_t* edge_off, int32_t* src,
                         int32_t* dst) {
  if (num_graphs <= 0 || n_lo < 2 || n_hi < n_lo || m_lo < 1 || m_hi < m_lo ||
      n_lo <= m_hi || !vtx_off || !edge_off)
    return -1;
  g_inv_init();
  const double l0 = g_log((double)n_lo), l1 = g_log((double)n_hi);
  int64_t* ns = (int64_t*)malloc(sizeof(int64_t) * (size_t)num_graphs);
  int* ms = (int*)malloc(sizeof(int) * (size_t)num_graphs);
  if (!ns || !ms) { free(ns); free(ms); return -1; }
  vtx_off[0] = 0;
  edge_off[0] = 0;
  for (int g = 0; g < num_graphs; ++g) {
    double u = g_unit(g_draw(seed, 5, 2 * (uint64_t)g));
    int64_t nv = (int64_t)floor(g_exp(l0 + u * (l1 - l0)) + 0.5);
    nv = nv < n_lo ? n_lo : nv > n_hi ? n_hi : nv;
    int mm = m_lo + (int)g_below(g_draw(seed, 5, 2 * (uint64_t)g + 1),
                                 (uint64_t)(m_hi - m_lo + 1));
    ns[g] = nv;
    ms[g] = mm;
    vtx_off[g + 1] = vtx_off[g] + nv;
    edge_off[g + 1] = edge_off[g] + (int64_t)mm * (nv - mm);
  }
  int64_t total = edge_off[num_graphs];
  if (vtx_off[num_graphs] > ((int64_t)1 << 31) - 1) total = -1;
  if (total >= 0 && src && dst) {
#pragma omp parallel for schedule(dynamic, 16)
    for (int g = 0; g < num_graphs; ++g)
      ba_graph(ns[g], ms[g], g_draw(seed, 6, (uint64_t)g), vtx_off[g], src + edge_off[g],
               dst + edge_off[g]);
  }
  free(ns);
  free(ms);
  return total;
}
