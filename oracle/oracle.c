/*
 * oracle.c - CPU restatement of X-GMiner's (G2Miner's) OpenMP counting path.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the checker for the GPU engine: the tests,
 * the smoke check and the CPU-baseline leg of bench.py load it.  The engine itself
 * never links, loads or calls it, and nothing here is a fallback for the engine.
 *
 * Every function restates one function of the reference (cited file:line, paths
 * inside the zlwu92/X-GMiner tree).  Parity of this restatement is pinned two ways
 * by the tests: against the reference's published known answers on citeseer
 * (codes/GraphMiner/src/triangle/README.md:53, src/motif/README.md:57,
 * src/count/README.md:41) and against the reference's own OpenMP binaries built
 * from source by oracle/build_ref.sh, run on the same graph files.
 *
 * Types follow codes/GraphMiner/include/common.h:36-40: vidType = int32,
 * eidType = int64, counts uint64.
 */
#include <limits.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

typedef int32_t vid_t;
typedef int64_t eid_t;

/* ---------------------------------------------------------------- threads */
int orc_max_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}
void orc_set_threads(int n) {
#ifdef _OPENMP
  if (n > 0) omp_set_num_threads(n);
#else
  (void)n;
#endif
}
int orc_has_openmp(void) {
#ifdef _OPENMP
  return 1;
#else
  return 0;
#endif
}
void orc_free(void* p) { free(p); }

/* ------------------------------------------------------- set primitives */
/* VertexSet::get_intersect_num, codes/GraphMiner/include/VertexSet.h:65-75 (merge). */
static inline uint64_t isect_num(const vid_t* a, eid_t na, const vid_t* b, eid_t nb) {
  uint64_t num = 0;
  eid_t l = 0, r = 0;
  while (l < na && r < nb) {
    vid_t x = a[l], y = b[r];
    if (x <= y) l++;
    if (y <= x) r++;
    if (x == y) num++;
  }
  return num;
}
/* VertexSet::intersect_ns (bounded count of common ids < up), VertexSet.h:110-123. */
static inline uint64_t isect_num_bound(const vid_t* a, eid_t na, const vid_t* b, eid_t nb,
                                       vid_t up) {
  uint64_t num = 0;
  eid_t l = 0, r = 0;
  while (l < na && r < nb) {
    vid_t x = a[l], y = b[r];
    if (x >= up || y >= up) break;
    if (x <= y) l++;
    if (y <= x) r++;
    if (x == y) num++;
  }
  return num;
}
/* VertexSet::operator& (set-producing merge), VertexSet.h:53-64. */
static inline eid_t isect_set(const vid_t* a, eid_t na, const vid_t* b, eid_t nb, vid_t* out) {
  eid_t n = 0, l = 0, r = 0;
  while (l < na && r < nb) {
    vid_t x = a[l], y = b[r];
    if (x <= y) l++;
    if (y <= x) r++;
    if (x == y) out[n++] = x;
  }
  return n;
}

/* ------------------------------------------------------------ CSR build */
/* LSD radix sort of 64-bit keys (16-bit digits) over the low `bits` bits. */
static void radix_sort_u64(uint64_t* keys, eid_t n, int bits) {
  uint64_t* tmp = (uint64_t*)malloc(sizeof(uint64_t) * (size_t)(n > 0 ? n : 1));
  eid_t* cnt = (eid_t*)malloc(sizeof(eid_t) * 65536);
  uint64_t *a = keys, *b = tmp;
  for (int shift = 0; shift < bits; shift += 16) {
    memset(cnt, 0, sizeof(eid_t) * 65536);
    for (eid_t i = 0; i < n; i++) cnt[(a[i] >> shift) & 0xFFFF]++;
    eid_t s = 0;
    for (int d = 0; d < 65536; d++) { eid_t c = cnt[d]; cnt[d] = s; s += c; }
    for (eid_t i = 0; i < n; i++) b[cnt[(a[i] >> shift) & 0xFFFF]++] = a[i];
    uint64_t* t = a; a = b; b = t;
  }
  if (a != keys) memcpy(keys, a, sizeof(uint64_t) * (size_t)n);
  free(tmp);
  free(cnt);
}

/* Symmetrise + sort (scripts/graph_format_conversion.py:20-44), plus dedupe and
 * self-loop removal (flags bit 2 / bit 4 as in xgm.h); bit 1 adds reverse edges.
 * Returns 0 on success; *rowptr (nv+1) and *col are malloc'd. */
int orc_build_csr(int64_t nv, const int32_t* src, const int32_t* dst, int64_t m, int flags,
                  int64_t** rowptr_out, int32_t** col_out, int64_t* ne_out) {
  const int sym = flags & 1, dedup = flags & 2, noself = flags & 4;
  eid_t cap = sym ? 2 * m : m;
  uint64_t* keys = (uint64_t*)malloc(sizeof(uint64_t) * (size_t)(cap > 0 ? cap : 1));
  if (!keys) return 3;
  eid_t n = 0;
  for (eid_t i = 0; i < m; i++) {
    uint32_t u = (uint32_t)src[i], v = (uint32_t)dst[i];
    if ((int64_t)u >= nv || (int64_t)v >= nv) { free(keys); return 1; }
    if (noself && u == v) continue;
    keys[n++] = ((uint64_t)u << 32) | v;
    if (sym) keys[n++] = ((uint64_t)v << 32) | u;
  }
  int vb = 1;
  while (((int64_t)1 << vb) < nv) vb++;
  /* the key (u<<32|v) sorts by u then v; sort on the used bits of both halves */
  for (eid_t i = 0; i < n; i++) keys[i] = ((keys[i] >> 32) << vb) | (keys[i] & 0xFFFFFFFFull);
  radix_sort_u64(keys, n, 2 * vb);
  eid_t w = 0;
  for (eid_t i = 0; i < n; i++) {
    if (dedup && w > 0 && keys[w - 1] == keys[i]) continue;
    keys[w++] = keys[i];
  }
  int64_t* rowptr = (int64_t*)calloc((size_t)nv + 1, sizeof(int64_t));
  int32_t* col = (int32_t*)malloc(sizeof(int32_t) * (size_t)(w > 0 ? w : 1));
  const uint64_t vmask = (((uint64_t)1) << vb) - 1;
  for (eid_t i = 0; i < w; i++) {
    rowptr[(keys[i] >> vb) + 1]++;
    col[i] = (int32_t)(keys[i] & vmask);
  }
  for (int64_t v = 0; v < nv; v++) rowptr[v + 1] += rowptr[v];
  free(keys);
  *rowptr_out = rowptr;
  *col_out = col;
  *ne_out = w;
  return 0;
}

/* Graph::orientation, codes/GraphMiner/src/common/graph.cc:233-275 (identical to
 * xgminer/src/graph_v2.cpp:243-289): keep src->dst iff deg(dst) > deg(src), or the
 * degrees tie and dst > src; order within each row is preserved. */
int orc_orient(int64_t nv, const int64_t* rowptr, const int32_t* col, int64_t** dag_rowptr_out,
               int32_t** dag_col_out, int64_t* dag_ne_out) {
  int64_t* nd = (int64_t*)calloc((size_t)nv + 1, sizeof(int64_t));
  if (!nd) return 3;
#pragma omp parallel for schedule(static)
  for (int64_t s = 0; s < nv; s++) {
    int64_t ds = rowptr[s + 1] - rowptr[s], c = 0;
    for (int64_t e = rowptr[s]; e < rowptr[s + 1]; e++) {
      int32_t d = col[e];
      int64_t dd = rowptr[d + 1] - rowptr[d];
      if (dd > ds || (dd == ds && d > s)) c++;
    }
    nd[s + 1] = c;
  }
  for (int64_t v = 0; v < nv; v++) nd[v + 1] += nd[v];
  int32_t* dc = (int32_t*)malloc(sizeof(int32_t) * (size_t)(nd[nv] > 0 ? nd[nv] : 1));
#pragma omp parallel for schedule(static)
  for (int64_t s = 0; s < nv; s++) {
    int64_t ds = rowptr[s + 1] - rowptr[s], o = nd[s];
    for (int64_t e = rowptr[s]; e < rowptr[s + 1]; e++) {
      int32_t d = col[e];
      int64_t dd = rowptr[d + 1] - rowptr[d];
      if (dd > ds || (dd == ds && d > s)) dc[o++] = d;
    }
  }
  *dag_rowptr_out = nd;
  *dag_col_out = dc;
  *dag_ne_out = nd[nv];
  return 0;
}

/* ------------------------------------------------------------- counting */
/* All counting functions take the outer-loop range [lo, hi) with `stride`, so the
 * CPU baseline can time a bounded sample; (0, V, 1) is the full count.  With a sample
 * list set (orc_set_sample), the triangle and clique functions instead take their
 * top-level vertices from sample[lo..hi) with `stride` (a seeded uniform random
 * vertex sample for the CPU baseline). */
#define ROW(v) (col + rowptr[(v)]), (rowptr[(v) + 1] - rowptr[(v)])

static const int64_t* g_sample = NULL;
static int64_t g_sample_n = 0;
void orc_set_sample(const int64_t* verts, int64_t n) {
  g_sample = n > 0 ? verts : NULL;
  g_sample_n = n > 0 ? n : 0;
}
#define TOP(i) (g_sample ? g_sample[(i)] : (i))

/* TCSolver, codes/GraphMiner/src/triangle/omp_base.cc:5-26 (on the DAG). */
uint64_t orc_tc(int64_t nv, const int64_t* rowptr, const int32_t* col, int64_t lo, int64_t hi,
                int64_t stride) {
  (void)nv;
  uint64_t counter = 0;
#pragma omp parallel for reduction(+ : counter) schedule(dynamic, 1)
  for (int64_t i = lo; i < hi; i += stride) {
    const int64_t u = TOP(i);
    for (int64_t e = rowptr[u]; e < rowptr[u + 1]; e++) {
      int32_t v = col[e];
      counter += isect_num(ROW(u), ROW(v));
    }
  }
  return counter;
}

/* automine_4clique, codes/GraphMiner/src/clique/cpu_kernels/clique_base.h:53-68. */
uint64_t orc_clique4(int64_t nv, const int64_t* rowptr, const int32_t* col, int64_t max_deg,
                     int64_t lo, int64_t hi, int64_t stride) {
  (void)nv;
  uint64_t counter = 0;
#pragma omp parallel reduction(+ : counter)
  {
    vid_t* y0y1 = (vid_t*)malloc(sizeof(vid_t) * (size_t)(max_deg + 1));
#pragma omp for schedule(dynamic, 1)
    for (int64_t i = lo; i < hi; i += stride) {
      const int64_t v0 = TOP(i);
      uint64_t local = 0;
      for (int64_t e = rowptr[v0]; e < rowptr[v0 + 1]; e++) {
        int32_t v1 = col[e];
        eid_t n = isect_set(ROW(v0), ROW(v1), y0y1);
        for (eid_t i = 0; i < n; i++) local += isect_num(y0y1, n, ROW(y0y1[i]));
      }
      counter += local;
    }
    free(y0y1);
  }
  return counter;
}

/* automine_5clique, codes/GraphMiner/src/clique/cpu_kernels/automine_omp.h:138-157. */
uint64_t orc_clique5(int64_t nv, const int64_t* rowptr, const int32_t* col, int64_t max_deg,
                     int64_t lo, int64_t hi, int64_t stride) {
  (void)nv;
  uint64_t counter = 0;
#pragma omp parallel reduction(+ : counter)
  {
    vid_t* y1y2 = (vid_t*)malloc(sizeof(vid_t) * (size_t)(max_deg + 1));
    vid_t* y1y2y3 = (vid_t*)malloc(sizeof(vid_t) * (size_t)(max_deg + 1));
#pragma omp for schedule(dynamic, 1)
    for (int64_t i = lo; i < hi; i += stride) {
      const int64_t v1 = TOP(i);
      uint64_t local = 0;
      for (int64_t e = rowptr[v1]; e < rowptr[v1 + 1]; e++) {
        int32_t v2 = col[e];
        eid_t n12 = isect_set(ROW(v1), ROW(v2), y1y2);
        for (eid_t i = 0; i < n12; i++) {
          eid_t n123 = isect_set(y1y2, n12, ROW(y1y2[i]), y1y2y3);
          for (eid_t j = 0; j < n123; j++) local += isect_num(y1y2y3, n123, ROW(y1y2y3[j]));
        }
      }
      counter += local;
    }
    free(y1y2);
    free(y1y2y3);
  }
  return counter;
}

/* k-clique listing on the DAG for any k >= 3: the candidate-set recursion of
 * automine_4clique / automine_5clique (clique_base.h:53-68, automine_omp.h:138-157)
 * carried to depth k - 1, as GLUMIN's 6- and 7-clique kernels do on the GPU
 * (codes/GLUMIN/src/G2Miner/gpu_GM_LUT_kernels/GM_kernels/clique6_warp_edge.cuh,
 * clique7_warp_edge.cuh): candidates of the next level = candidates & N+(u).  `need`
 * more members are to be picked from cand[0..n); buf holds one level per member. */
static uint64_t kclique_rec(const int64_t* rowptr, const int32_t* col, const vid_t* cand,
                            eid_t n, int need, vid_t* buf, size_t level) {
  if (need == 1) return (uint64_t)n;
  uint64_t total = 0;
  for (eid_t i = 0; i < n; i++) {
    const eid_t m = isect_set(cand, n, ROW(cand[i]), buf);
    if (m >= need - 1) total += kclique_rec(rowptr, col, buf, m, need - 1, buf + level, level);
  }
  return total;
}

uint64_t orc_clique_k(int k, int64_t nv, const int64_t* rowptr, const int32_t* col,
                      int64_t max_deg, int64_t lo, int64_t hi, int64_t stride) {
  (void)nv;
  uint64_t counter = 0;
  if (k < 3) return 0;
  const size_t level = (size_t)(max_deg + 1);
#pragma omp parallel reduction(+ : counter)
  {
    vid_t* buf = (vid_t*)malloc(sizeof(vid_t) * level * (size_t)k);
#pragma omp for schedule(dynamic, 1)
    for (int64_t i = lo; i < hi; i += stride) {
      const int64_t v0 = TOP(i);
      counter += kclique_rec(rowptr, col, col + rowptr[v0], rowptr[v0 + 1] - rowptr[v0], k - 1,
                             buf, level);
    }
    free(buf);
  }
  return counter;
}

/* Edge-induced diamond, codes/GraphMiner/src/count/cpu_kernels/diamond.h:1-8
 * (undirected graph): sum over edges v1 < v0 of C(|N(v0) & N(v1)|, 2). */
uint64_t orc_diamond(int64_t nv, const int64_t* rowptr, const int32_t* col, int64_t lo,
                     int64_t hi, int64_t stride) {
  (void)nv;
  uint64_t counter = 0;
#pragma omp parallel for schedule(dynamic, 1) reduction(+ : counter)
  for (int64_t v0 = lo; v0 < hi; v0 += stride) {
    for (int64_t e = rowptr[v0]; e < rowptr[v0 + 1]; e++) {
      int32_t v1 = col[e];
      if (v1 >= v0) break;
      uint64_t n = isect_num(ROW(v0), ROW(v1));
      if (n > 1) counter += n * (n - 1) / 2;
    }
  }
  return counter;
}

/* Edge-induced 4-cycle, codes/GraphMiner/src/count/cpu_kernels/rectangle.h:1-46:
 * for each v0, wedges v0-v1-v2 with v1 < v0 and v2 < v0 are grouped by v2 and every
 * group of n wedges closes C(n,2) cycles.  The reference groups by sorting the wedge
 * list; this restatement groups with a dense per-thread counter (same groups). */
uint64_t orc_cycle4(int64_t nv, const int64_t* rowptr, const int32_t* col, int64_t lo,
                    int64_t hi, int64_t stride) {
  uint64_t counter = 0;
#pragma omp parallel reduction(+ : counter)
  {
    uint32_t* cnt = (uint32_t*)calloc((size_t)nv, sizeof(uint32_t));
    vid_t* touched = (vid_t*)malloc(sizeof(vid_t) * (size_t)(nv > 0 ? nv : 1));
#pragma omp for schedule(dynamic, 1)
    for (int64_t v0 = lo; v0 < hi; v0 += stride) {
      int64_t nt = 0;
      for (int64_t e = rowptr[v0]; e < rowptr[v0 + 1]; e++) {
        int32_t v1 = col[e];
        if (v1 >= v0) break;
        for (int64_t f = rowptr[v1]; f < rowptr[v1 + 1]; f++) {
          int32_t v2 = col[f];
          if (v2 >= v0) break;
          if (cnt[v2]++ == 0) touched[nt++] = v2;
        }
      }
      for (int64_t t = 0; t < nt; t++) {
        uint64_t n = cnt[touched[t]];
        counter += n * (n - 1) / 2;
        cnt[touched[t]] = 0;
      }
    }
    free(cnt);
    free(touched);
  }
  return counter;
}

/* Edge-induced tailed triangle, codes/GraphMiner/src/count/cpu_kernels/tailedtriangle.h:1-12:
 * for each v0 of degree > 2, t(v0) = sum over v1 in N(v0) of |N(v0) & N(v1)| bounded
 * by v1, and the count grows by t(v0) * (deg(v0) - 2). */
uint64_t orc_tailed_triangle(int64_t nv, const int64_t* rowptr, const int32_t* col, int64_t lo,
                             int64_t hi, int64_t stride) {
  (void)nv;
  uint64_t counter = 0;
#pragma omp parallel for schedule(dynamic, 1) reduction(+ : counter)
  for (int64_t v0 = lo; v0 < hi; v0 += stride) {
    int64_t deg = rowptr[v0 + 1] - rowptr[v0];
    if (deg > 2) {
      uint64_t tri = 0;
      for (int64_t e = rowptr[v0]; e < rowptr[v0 + 1]; e++) {
        int32_t v1 = col[e];
        tri += isect_num_bound(ROW(v0), ROW(v1), v1);
      }
      counter += tri * (uint64_t)(deg - 2);
    }
  }
  return counter;
}

/* Ordered-set difference a \ b, elements below `up`, skipping `skip` (the vertex whose
 * neighbourhood b is): VertexSet::difference_buf, codes/GraphMiner/src/common/
 * VertexSet.cc:21-67 (unbounded form: up = INT32_MAX). */
static inline eid_t diff_set(const vid_t* a, eid_t na, const vid_t* b, eid_t nb, vid_t up,
                             vid_t skip, vid_t* out) {
  eid_t n = 0, l = 0, r = 0;
  while (l < na && a[l] < up) {
    vid_t x = a[l];
    while (r < nb && b[r] < x) r++;
    if ((r >= nb || b[r] != x) && x != skip) out[n++] = x;
    l++;
  }
  return n;
}

/* Vertex-induced k-motif census (k = 3, 4) on the undirected graph:
 * automine_3motif / automine_4motif, codes/GraphMiner/src/motif/cpu_kernels/
 * automine_formula.h:2-57, followed by the formula post-processing of MotifSolver,
 * src/motif/omp_formula.cc:38-48.  Output order as the reference prints it
 * (main.cc:28-29): k = 3 [wedges, triangles]; k = 4 [3-stars, 4-paths, tailed
 * triangles, 4-cycles, diamonds, 4-cliques].  Returns 0, or -1 for another k. */
int orc_motif(int k, int64_t nv, const int64_t* rowptr, const int32_t* col, int64_t max_deg,
              uint64_t* out) {
  uint64_t c[6] = {0, 0, 0, 0, 0, 0};
  if (k == 3) {
    uint64_t c0 = 0, c1 = 0;
#pragma omp parallel for schedule(dynamic, 64) reduction(+ : c0, c1)
    for (int64_t v0 = 0; v0 < nv; v0++) {
      uint64_t n = (uint64_t)(rowptr[v0 + 1] - rowptr[v0]);
      c0 += n * (n - (n > 0));
      for (int64_t e = rowptr[v0]; e < rowptr[v0 + 1]; e++) {
        int32_t v1 = col[e];
        if (v1 >= v0) break;
        c1 += isect_num_bound(ROW(v0), ROW(v1), v1);
      }
    }
    out[0] = c0 / 2 - 3 * c1;
    out[1] = c1;
    return 0;
  }
  if (k != 4) return -1;
  uint64_t c0 = 0, c1 = 0, c2 = 0, c3 = 0, c4 = 0, c5 = 0;
#pragma omp parallel reduction(+ : c0, c1, c2, c3, c4, c5)
  {
    const size_t cap = (size_t)(max_deg + 1);
    vid_t* y01 = (vid_t*)malloc(sizeof(vid_t) * cap);    /* y0f0y1f1 */
    vid_t* n01 = (vid_t*)malloc(sizeof(vid_t) * cap);    /* n0f0y1 = N(v1) \ N(v0) */
    vid_t* y0n1 = (vid_t*)malloc(sizeof(vid_t) * cap);   /* y0f0n1f1 */
#pragma omp for schedule(dynamic, 1)
    for (int64_t v0 = 0; v0 < nv; v0++) {
      const vid_t* y0 = col + rowptr[v0];
      const eid_t d0 = rowptr[v0 + 1] - rowptr[v0];
      eid_t nf0 = 0; /* |N(v0) below v0| */
      while (nf0 < d0 && y0[nf0] < v0) nf0++;
      for (eid_t i1 = 0; i1 < nf0; i1++) {
        const int32_t v1 = y0[i1];
        const vid_t* y1 = col + rowptr[v1];
        const eid_t d1 = rowptr[v1 + 1] - rowptr[v1];
        const uint64_t tri = isect_num(y0, d0, y1, d1);
        const uint64_t su = (uint64_t)d0 - tri - 1, sv = (uint64_t)d1 - tri - 1;
        c4 += tri * (tri - (tri > 0));
        c2 += tri * (su + sv);
        c1 += su * sv;
        c0 += su * (su - (su > 0)) + sv * (sv - (sv > 0));
        /* y0f0 & N(v1) below v1 */
        eid_t n = 0;
        {
          eid_t l = 0, r = 0;
          while (l < nf0 && r < d1) {
            vid_t x = y0[l], y = y1[r];
            if (x >= v1 || y >= v1) break;
            if (x <= y) l++;
            if (y <= x) r++;
            if (x == y) y01[n++] = x;
          }
        }
        const eid_t nn = diff_set(y1, d1, y0, d0, INT32_MAX, (vid_t)v0, n01);
        const eid_t nd = diff_set(y0, nf0, y1, d1, v1, v1, y0n1);
        for (eid_t i2 = 0; i2 < n; i2++) {
          const int32_t v2 = y01[i2];
          c5 += isect_num_bound(y01, n, ROW(v2), v2);
        }
        for (eid_t i2 = 0; i2 < nd; i2++) {
          const int32_t v2 = y0n1[i2];
          c3 += isect_num_bound(n01, nn, ROW(v2), (vid_t)v0);
        }
      }
    }
    free(y01);
    free(n01);
    free(y0n1);
  }
  c[4] = c4 / 2 - c5 * 6;
  c[2] = c2 / 2 - c[4] * 2;
  c[1] = c1 - c3 * 4;
  c[0] = c0 / 6 - c[2] / 3;
  out[0] = c[0];
  out[1] = c[1];
  out[2] = c[2];
  out[3] = c3;
  out[4] = c[4];
  out[5] = c5;
  return 0;
}

/* ----------------------------------------------------- algorithmic bytes */
/* Bytes of graph-resident adjacency data each plan reads: 4 B per int32 list element
 * plus 8 B per task record.  The engine reports the same quantity as its roofline
 * numerator; these loops are the checker for it.  kind: 3 = TC, 4 = 4-clique,
 * 5 = 5-clique on the DAG; 6 = diamond, 7 = 4-cycle, 8 = tailed triangle on the
 * undirected graph. */
uint64_t orc_algo_bytes(int kind, int64_t nv, const int64_t* rowptr, const int32_t* col,
                        int64_t max_deg) {
  uint64_t bytes = 0;
#define DEG(v) ((uint64_t)(rowptr[(v) + 1] - rowptr[(v)]))
#pragma omp parallel reduction(+ : bytes)
  {
    vid_t* w = (vid_t*)malloc(sizeof(vid_t) * (size_t)(max_deg + 1));
    vid_t* w2 = (vid_t*)malloc(sizeof(vid_t) * (size_t)(max_deg + 1));
    const int64_t ntop = g_sample ? g_sample_n : nv;
#pragma omp for schedule(dynamic, 64)
    for (int64_t i = 0; i < ntop; i++) {
      const int64_t v0 = TOP(i);
      if (kind == 8) {
        if (DEG(v0) > 2)
          for (int64_t e = rowptr[v0]; e < rowptr[v0 + 1]; e++) bytes += 4 * (DEG(v0) + DEG(col[e]));
        continue;
      }
      if (kind == 7) {
        bytes += 4 * DEG(v0);
        for (int64_t e = rowptr[v0]; e < rowptr[v0 + 1]; e++) {
          int32_t v1 = col[e];
          if (v1 >= v0) break;
          for (int64_t f = rowptr[v1]; f < rowptr[v1 + 1]; f++) {
            if (col[f] >= v0) break;
            bytes += 4;
          }
        }
        continue;
      }
      for (int64_t e = rowptr[v0]; e < rowptr[v0 + 1]; e++) {
        int32_t v1 = col[e];
        if (kind == 6 && v1 >= v0) break;
        bytes += 8 + 4 * (DEG(v0) + DEG(v1));
        if (kind == 4 || kind == 5) {
          eid_t n = isect_set(ROW(v0), ROW(v1), w);
          for (eid_t i = 0; i < n; i++) {
            bytes += 4 * DEG(w[i]);
            if (kind == 5) {
              eid_t n2 = isect_set(w, n, ROW(w[i]), w2);
              for (eid_t j = 0; j < n2; j++) bytes += 4 * DEG(w2[j]);
            }
          }
        }
      }
    }
    free(w);
    free(w2);
  }
#undef DEG
  return bytes;
}

/* ------------------------------------------------ GLUMIN 5-vertex plans (P6-P22)
 * GLUMIN's generated pattern kernels, codes/GLUMIN/src/G2Miner/gpu_GM_LUT_kernels/
 * GM_kernels/P<id>-GM.yml.cuh, restated as CPU loops.  A task is every directed
 * entry (v0, v1) of the undirected CSR (init_edgelist without symmetry breaking,
 * codes/GLUMIN/src/common/graph.cc:296-340).  The set operations are GLUMIN's
 * (codegen/include/gpu_kernels/codegen_utils.cuh:256-300, set_intersect.cuh,
 * set_difference.cuh:44-86,176-232): the elements of the first sorted list below
 * `up` that are (intersect) or are not (difference) in the second.  Nothing skips
 * an already matched vertex, so a difference can hand one back (N(v1) \ N(v0) holds
 * v0); the reference counts those embeddings and so does this restatement. */
#define NOB INT32_MAX
static eid_t g_isect(const vid_t* a, eid_t na, const vid_t* b, eid_t nb, vid_t up, vid_t* out) {
  eid_t n = 0, r = 0;
  for (eid_t l = 0; l < na && a[l] < up; l++) {
    while (r < nb && b[r] < a[l]) r++;
    if (r < nb && b[r] == a[l]) out[n++] = a[l];
  }
  return n;
}
static eid_t g_diff(const vid_t* a, eid_t na, const vid_t* b, eid_t nb, vid_t up, vid_t* out) {
  eid_t n = 0, r = 0;
  for (eid_t l = 0; l < na && a[l] < up; l++) {
    while (r < nb && b[r] < a[l]) r++;
    if (r >= nb || b[r] != a[l]) out[n++] = a[l];
  }
  return n;
}
static uint64_t g_isect_n(const vid_t* a, eid_t na, const vid_t* b, eid_t nb, vid_t up) {
  uint64_t n = 0;
  eid_t r = 0;
  for (eid_t l = 0; l < na && a[l] < up; l++) {
    while (r < nb && b[r] < a[l]) r++;
    if (r < nb && b[r] == a[l]) n++;
  }
  return n;
}
static uint64_t g_diff_n(const vid_t* a, eid_t na, const vid_t* b, eid_t nb, vid_t up) {
  uint64_t n = 0;
  eid_t r = 0;
  for (eid_t l = 0; l < na && a[l] < up; l++) {
    while (r < nb && b[r] < a[l]) r++;
    if (r >= nb || b[r] != a[l]) n++;
  }
  return n;
}

#define NB(v) (col + rowptr[v]), (rowptr[(v) + 1] - rowptr[v])
#define SL(i) s[i], n[i]

/* One task (v0, v1) of plan P<pid>; s[0..4] are slot buffers of max-degree size. */
static uint64_t glumin5_task(int pid, const int64_t* rowptr, const int32_t* col, vid_t v0,
                             vid_t v1, vid_t** s) {
  eid_t n[5] = {0, 0, 0, 0, 0};
  uint64_t c = 0;
  switch (pid) {
    case 6: /* P6-GM.yml.cuh */
      n[0] = g_isect(NB(v0), NB(v1), v1, s[0]);
      n[1] = g_diff(NB(v0), NB(v1), NOB, s[1]);
      for (eid_t i = 0; i < n[0]; i++) {
        vid_t v2 = s[0][i];
        n[2] = g_diff(SL(1), NB(v2), v1, s[2]);
        for (eid_t j = 0; j < n[2]; j++) c += g_isect_n(SL(2), NB(s[2][j]), s[2][j]);
      }
      break;
    case 7: /* P7-GM.yml.cuh */
    case 8: /* P8-GM.yml.cuh */
      n[0] = g_diff(NB(v1), NB(v0), NOB, s[0]);
      n[1] = g_isect(NB(v0), NB(v1), NOB, s[1]);
      n[2] = g_diff(NB(v0), NB(v1), NOB, s[2]);
      for (eid_t i = 0; i < n[0]; i++) {
        vid_t v2 = s[0][i];
        n[3] = g_diff(SL(1), NB(v2), NOB, s[3]);
        n[4] = pid == 7 ? g_diff(SL(2), NB(v2), NOB, s[4]) : g_isect(SL(2), NB(v2), NOB, s[4]);
        for (eid_t j = 0; j < n[3]; j++) c += g_diff_n(SL(4), NB(s[3][j]), NOB);
      }
      break;
    case 9: /* P9-GM.yml.cuh */
    case 13: /* P13-GM.yml.cuh */
      n[0] = g_isect(NB(v0), NB(v1), NOB, s[0]);
      for (eid_t i = 0; i < n[0]; i++) {
        n[1] = g_diff(SL(0), NB(s[0][i]), NOB, s[1]);
        for (eid_t j = 0; j < n[1]; j++) {
          vid_t v3 = s[1][j];
          c += pid == 9 ? g_isect_n(SL(1), NB(v3), v3) : g_diff_n(SL(1), NB(v3), NOB);
        }
      }
      break;
    case 10: /* P10-GM.yml.cuh */
      n[0] = g_diff(NB(v0), NB(v1), v1, s[0]);
      for (eid_t i = 0; i < n[0]; i++) {
        vid_t v2 = s[0][i];
        n[1] = g_diff(SL(0), NB(v2), v2, s[1]);
        for (eid_t j = 0; j < n[1]; j++) c += g_diff_n(SL(1), NB(s[1][j]), s[1][j]);
      }
      break;
    case 11: /* P11-GM.yml.cuh */
      n[0] = g_diff(NB(v1), NB(v0), NOB, s[0]);
      n[1] = g_diff(NB(v0), NB(v1), NOB, s[1]);
      for (eid_t i = 0; i < n[0]; i++) {
        vid_t v2 = s[0][i];
        n[2] = g_diff(SL(1), NB(v2), NOB, s[2]);
        n[3] = g_isect(SL(1), NB(v2), NOB, s[3]);
        for (eid_t j = 0; j < n[2]; j++) c += g_diff_n(SL(3), NB(s[2][j]), v1);
      }
      break;
    case 12: /* P12-GM.yml.cuh */
      n[0] = g_diff(NB(v1), NB(v0), v0, s[0]);
      n[1] = g_diff(NB(v0), NB(v1), NOB, s[1]);
      for (eid_t i = 0; i < n[0]; i++) {
        n[2] = g_isect(SL(1), NB(s[0][i]), NOB, s[2]);
        for (eid_t j = 0; j < n[2]; j++) c += g_diff_n(SL(2), NB(s[2][j]), NOB);
      }
      break;
    case 14: /* P14-GM.yml.cuh */
    case 20: /* P20-GM.yml.cuh */
    case 17: /* P17-GM.yml.cuh */
      n[0] = g_isect(NB(v0), NB(v1), NOB, s[0]);
      n[1] = g_diff(NB(v0), NB(v1), NOB, s[1]);
      for (eid_t i = 0; i < n[0]; i++) {
        vid_t v2 = s[0][i];
        if (pid == 14) {
          n[2] = g_isect(SL(0), NB(v2), v1, s[2]);
          n[3] = g_diff(SL(1), NB(v2), NOB, s[3]);
        } else if (pid == 20) {
          n[2] = g_isect(SL(1), NB(v2), v1, s[2]);
          n[3] = g_diff(SL(1), NB(v2), NOB, s[3]);
        } else {
          n[2] = g_isect(SL(1), NB(v2), NOB, s[2]);
          n[3] = g_diff(SL(0), NB(v2), NOB, s[3]);
        }
        for (eid_t j = 0; j < n[2]; j++) c += g_diff_n(SL(3), NB(s[2][j]), NOB);
      }
      break;
    case 15: /* P15-GM.yml.cuh */
    case 21: /* P21-GM.yml.cuh */
      n[0] = g_diff(NB(v1), NB(v0), NOB, s[0]);
      n[1] = g_diff(NB(v0), NB(v1), NOB, s[1]);
      for (eid_t i = 0; i < n[0]; i++) {
        n[2] = g_diff(SL(1), NB(s[0][i]), NOB, s[2]);
        for (eid_t j = 0; j < n[2]; j++) {
          vid_t v3 = s[2][j];
          c += pid == 15 ? g_diff_n(SL(2), NB(v3), v3) : g_isect_n(SL(2), NB(v3), v3);
        }
      }
      break;
    case 16: /* P16-GM.yml.cuh */
      n[0] = g_diff(NB(v1), NB(v0), NOB, s[0]);
      n[1] = g_diff(NB(v0), NB(v1), NOB, s[1]);
      n[2] = g_isect(NB(v0), NB(v1), NOB, s[2]);
      for (eid_t i = 0; i < n[0]; i++) {
        vid_t v2 = s[0][i];
        n[3] = g_diff(SL(1), NB(v2), NOB, s[3]);
        n[4] = g_isect(SL(2), NB(v2), NOB, s[4]);
        for (eid_t j = 0; j < n[3]; j++) c += g_diff_n(SL(4), NB(s[3][j]), v1);
      }
      break;
    case 18: /* P18-GM.yml.cuh */
      n[0] = g_isect(NB(v0), NB(v1), v1, s[0]);
      n[1] = g_diff(NB(v0), NB(v1), NOB, s[1]);
      for (eid_t i = 0; i < n[0]; i++) {
        n[2] = g_diff(SL(1), NB(s[0][i]), NOB, s[2]);
        for (eid_t j = 0; j < n[2]; j++) c += g_diff_n(SL(2), NB(s[2][j]), s[2][j]);
      }
      break;
    case 19: /* P19-GM.yml.cuh */
      n[0] = g_isect(NB(v0), NB(v1), v1, s[0]);
      n[1] = g_diff(NB(v0), NB(v1), NOB, s[1]);
      for (eid_t i = 0; i < n[0]; i++) {
        vid_t v2 = s[0][i];
        n[2] = g_isect(SL(1), NB(v2), v2, s[2]);
        n[3] = g_diff(SL(0), NB(v2), NOB, s[3]);
        for (eid_t j = 0; j < n[2]; j++) c += g_isect_n(SL(3), NB(s[2][j]), s[2][j]);
      }
      break;
    case 22: /* P22-GM.yml.cuh (its v1 == v0 skip never fires on a loop-free CSR) */
      n[0] = g_isect(NB(v0), NB(v1), NOB, s[0]);
      for (eid_t i = 0; i < n[0]; i++) {
        n[1] = g_isect(SL(0), NB(s[0][i]), NOB, s[1]);
        for (eid_t j = 0; j < n[1]; j++) c += g_diff_n(SL(1), NB(s[1][j]), NOB);
      }
      break;
    default:
      break;
  }
  return c;
}

/* P<pid> count (6 <= pid <= 22); returns 0, or -1 for another id. */
int orc_glumin5(int pid, int64_t nv, const int64_t* rowptr, const int32_t* col, int64_t max_deg,
                uint64_t* out) {
  if (pid < 6 || pid > 22) return -1;
  uint64_t total = 0;
  const int64_t md = max_deg > 0 ? max_deg : 1;
#pragma omp parallel reduction(+ : total)
  {
    vid_t* buf = (vid_t*)malloc(sizeof(vid_t) * 5 * (size_t)md);
    vid_t* s[5];
    for (int i = 0; i < 5; i++) s[i] = buf + (size_t)i * md;
#pragma omp for schedule(dynamic, 16)
    for (int64_t v0 = 0; v0 < nv; v0++)
      for (int64_t e = rowptr[v0]; e < rowptr[v0 + 1]; e++)
        total += glumin5_task(pid, rowptr, col, (vid_t)v0, col[e], s);
    free(buf);
  }
  *out = total;
  return 0;
}

/* ------------------------------------------------------ set-operation programs
 * Interpreter for the engine's program words (see include/xgm.h,
 * xgm_plan_program): tasks are the directed CSR entries (v0, v1), only v1 < v0 when
 * the program says so; level l runs after v_0..v_{l+1} are matched; v_{l+2} then runs
 * over its candidate operand; the last level ends with the counted operation.
 * Operand >= 16 is N(v_(operand-16)), below it a slot. */
typedef struct {
  int k, nslots, flat, v1lt, nops[4], cand[6];
  int op[4][6][6];
  int fin[6];
} prog_t;

typedef struct {
  const prog_t* p;
  const int64_t* rowptr;
  const int32_t* col;
  vid_t v[6];
  vid_t* slot[16];
  eid_t slen[16];
} pstate_t;

static void p_operand(pstate_t* st, int code, const vid_t** a, eid_t* n) {
  if (code >= 16) {
    vid_t v = st->v[code - 16];
    *a = st->col + st->rowptr[v];
    *n = st->rowptr[v + 1] - st->rowptr[v];
  } else {
    *a = st->slot[code];
    *n = st->slen[code];
  }
}

static int p_member(const vid_t* b, eid_t nb, vid_t x) {
  eid_t lo = 0, hi = nb;
  while (lo < hi) {
    eid_t m = (lo + hi) / 2;
    if (b[m] < x) lo = m + 1;
    else hi = m;
  }
  return lo < nb && b[lo] == x;
}

/* Runs one operation; writes its slot, or returns the count when out == NULL. */
static uint64_t p_apply(pstate_t* st, const int* o, vid_t* out, eid_t* nout) {
  const vid_t *a, *b = NULL;
  eid_t na, nb = 0;
  p_operand(st, o[2], &a, &na);
  if (o[1] != 2) p_operand(st, o[3], &b, &nb);
  vid_t up = INT32_MAX;
  for (int j = 0; j < 6; j++)
    if ((o[4] >> j) & 1)
      if (st->v[j] < up) up = st->v[j];
  uint64_t c = 0;
  eid_t n = 0;
  for (eid_t i = 0; i < na && a[i] < up; i++) {
    vid_t x = a[i];
    int skip = 0;
    for (int j = 0; j < 6; j++)
      if (((o[5] >> j) & 1) && x == st->v[j]) skip = 1;
    if (skip) continue;
    if (o[1] != 2 && p_member(b, nb, x) != (o[1] == 0)) continue;
    if (out) out[n++] = x;
    else c++;
  }
  if (nout) *nout = n;
  return c;
}

static uint64_t p_level(pstate_t* st, int l) {
  const prog_t* p = st->p;
  for (int i = 0; i < p->nops[l]; i++) {
    const int* o = p->op[l][i];
    p_apply(st, o, st->slot[o[0]], &st->slen[o[0]]);
  }
  if (l == p->k - 3) return p_apply(st, p->fin, NULL, NULL);
  const vid_t* c;
  eid_t nc;
  p_operand(st, p->cand[l + 2], &c, &nc);
  uint64_t t = 0;
  for (eid_t i = 0; i < nc; i++) {
    st->v[l + 2] = c[i];
    t += p_level(st, l + 1);
  }
  return t;
}

/* Runs a program over every directed CSR entry; returns 0, or -1 for malformed words. */
int orc_setprog(const int32_t* w, int nw, int64_t nv, const int64_t* rowptr, const int32_t* col,
                int64_t max_deg, uint64_t* out) {
  if (nw < 162 || w[0] != 2) return -1;  /* format version 2 */
  prog_t p;
  memset(&p, 0, sizeof(p));
  p.k = w[1];
  p.nslots = w[2];
  p.flat = w[3];
  p.v1lt = w[4];
  for (int l = 0; l < 4; l++) p.nops[l] = w[5 + l];
  for (int i = 2; i < 5; i++) p.cand[i] = w[9 + i - 2];
  if (p.k < 3 || p.k > 6 || p.nslots < 0 || p.nslots > 16) return -1;
  const int32_t* o = w + 12;
  for (int l = 0; l < 4; l++)
    for (int i = 0; i < 6; i++, o += 6) memcpy(p.op[l][i], o, sizeof(int) * 6);
  memcpy(p.fin, o, sizeof(int) * 6);
  uint64_t total = 0;
  const int64_t md = max_deg > 0 ? max_deg : 1;
#pragma omp parallel reduction(+ : total)
  {
    pstate_t st;
    memset(&st, 0, sizeof(st));
    st.p = &p;
    st.rowptr = rowptr;
    st.col = col;
    vid_t* buf = (vid_t*)malloc(sizeof(vid_t) * 16 * (size_t)md);
    for (int i = 0; i < 16; i++) st.slot[i] = buf + (size_t)i * md;
#pragma omp for schedule(dynamic, 16)
    for (int64_t v0 = 0; v0 < nv; v0++)
      for (int64_t e = rowptr[v0]; e < rowptr[v0 + 1]; e++) {
        if (p.v1lt && col[e] >= v0) continue;
        st.v[0] = (vid_t)v0;
        st.v[1] = col[e];
        total += p_level(&st, 0);
      }
    free(buf);
  }
  *out = total;
  return 0;
}

/* ---------------------------------------------------- brute-force occurrences
 * Occurrences of a connected pattern (k <= 6 vertices, adjacency adj[k*k]),
 * vertex-induced or edge-induced: injective maps that keep every pattern edge (and,
 * induced, every non-edge), counted by depth-first search in a BFS order of the
 * pattern and divided by the pattern's automorphism count.  Independent of the
 * engine's program compiler; for small graphs. */
typedef struct {
  int k, induced;
  const uint8_t* adj;
  int order[6], parent[6];
  const int64_t* rowptr;
  const int32_t* col;
  vid_t m[6];
} emb_t;

static int e_adj(const emb_t* e, vid_t a, vid_t b) {
  return p_member(e->col + e->rowptr[a], e->rowptr[a + 1] - e->rowptr[a], b);
}

static uint64_t e_dfs(emb_t* e, int i) {
  if (i == e->k) return 1;
  const int t = e->order[i];
  const vid_t pv = e->m[e->parent[i]];
  uint64_t c = 0;
  for (int64_t x = e->rowptr[pv]; x < e->rowptr[pv + 1]; x++) {
    vid_t y = e->col[x];
    int ok = 1;
    for (int j = 0; j < i && ok; j++) {
      const int u = e->order[j];
      if (e->m[u] == y) ok = 0;
      else if (e->adj[t * e->k + u]) ok = e_adj(e, y, e->m[u]);
      else if (e->induced) ok = !e_adj(e, y, e->m[u]);
    }
    if (!ok) continue;
    e->m[t] = y;
    c += e_dfs(e, i + 1);
  }
  return c;
}

/* Returns 0, or -1 when the pattern is not connected or k is out of range. */
int orc_occurrences(int k, const uint8_t* adj, int induced, int64_t nv, const int64_t* rowptr,
                    const int32_t* col, uint64_t* out) {
  if (k < 2 || k > 6) return -1;
  emb_t e0;
  memset(&e0, 0, sizeof(e0));
  e0.k = k;
  e0.induced = induced;
  e0.adj = adj;
  e0.rowptr = rowptr;
  e0.col = col;
  int seen[6] = {1, 0, 0, 0, 0, 0}, n = 1;
  e0.order[0] = 0;
  for (int h = 0; h < n; h++)
    for (int u = 0; u < k; u++)
      if (!seen[u] && adj[e0.order[h] * k + u]) {
        seen[u] = 1;
        e0.parent[n] = e0.order[h];
        e0.order[n++] = u;
      }
  if (n != k) return -1;
  /* automorphisms */
  int perm[6], c[6] = {0};
  for (int i = 0; i < k; i++) perm[i] = i;
  uint64_t aut = 0;
  for (int i = 0;;) { /* Heap's algorithm over all k! permutations */
    int ok = 1;
    for (int a = 0; a < k && ok; a++)
      for (int b = 0; b < k && ok; b++) ok = adj[perm[a] * k + perm[b]] == adj[a * k + b];
    aut += ok;
    while (i < k && c[i] >= i) c[i++] = 0;
    if (i >= k) break;
    int j = (i % 2) ? c[i] : 0, t = perm[j];
    perm[j] = perm[i];
    perm[i] = t;
    c[i]++;
    i = 1;
  }
  uint64_t total = 0;
#pragma omp parallel for schedule(dynamic, 16) reduction(+ : total)
  for (int64_t v = 0; v < nv; v++) {
    emb_t e = e0;
    e.m[0] = (vid_t)v;
    total += e_dfs(&e, 1);
  }
  *out = total / aut;
  return 0;
}
