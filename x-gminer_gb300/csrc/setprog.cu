// Interpreter for set-operation programs (setprog.cuh) on the undirected CSR in
// original ids.  Tasks are the directed CSR entries (v0, v1), as GLUMIN's
// edge-parallel kernels walk the full edge list (G2Miner/gpu_GM_LUT.cu:78-95,
// GM_kernels/P*-GM.yml.cuh: `for eid ... g.get_src(eid), g.get_dst(eid)`).  Three
// forms, chosen per task by the degree of v0:
//
// - List form (k_setprog, any degree): one warp per task.  A set operation streams
//   its first list through the warp (coalesced, 32 elements a step), tests each
//   element against the second list by binary search, and compacts the survivors with
//   a ballot into the warp's slot; a bound stops the stream at the first element at
//   or above it (the lists are sorted).  The last vertex is never enumerated: the
//   final count runs flat over every (v_{k-2}, x) pair, or, when the counted operand
//   is long, searches the short neighbour lists of the candidates in it.
// - Bitmap form for d(v0) <= 32 (k_setlut): GLUMIN's LUT idea, one warp per v0 with
//   its adjacency rows in shared memory and one lane per task on 32-bit masks.
// - Warp-wide bitmap form for 32 < d(v0) <= 1024 (run_task_bits inside k_setprog):
//   the graph's stored rows, one word of N(v0) index space per lane.
//
// The bitmap forms need a program whose operands live in N(v0) (prog_lut); others
// run in the list form throughout.  Warps claim chunks of entries from an atomic head
// (the row of a chunk's first entry by binary search over rowptr, then entry by
// entry).  A task whose estimated work passes kSplitWork queues its v2 candidates as
// split records of about kSplitWork each, run by a second k_setprog launch (each
// record recomputes the level-0 slots, a few percent of its work).  Launches per
// count: k_setlut (and its stream-record pass), k_setprog tasks, k_setprog splits.
//
// List slots live in a per-warp global scratch area ((slot count + 1) x max degree
// ints), which stays in L1/L2: a slot is written once per level and read by every
// later step.
#include <algorithm>
#include <climits>
#include <cstdlib>
#include <cstring>

#include "api_internal.h"
#include "graph.cuh"
#include "prim.cuh"
#include "setprog.cuh"

namespace xgm {

namespace {

constexpr int kThreads = 256;
constexpr int kWarps = kThreads / 32;
constexpr int kChunk = 8;       // CSR entries claimed per queue step
// Work of a task in lane-steps (one binary search of one lane): a task above kSplitWork
// queues its v2 candidates as records of about kSplitWork each (about a millisecond
// of one warp).
constexpr long long kSplitWork = 4096;
constexpr int64_t kSplitCap = int64_t(1) << 22;  // records (64 MB)
// Long streams of the bitmap form: records of (v0, v1 index, N(v1) entry range) after
// the split records in the same buffer.
constexpr int64_t kStreamCap = int64_t(1) << 20;
constexpr int kStreamChunk = 256;  // N(v1) entries per record

struct SplitRec {
  int32_t e_lo, e_hi;  // CSR entry
  int32_t lo, hi;      // v2 candidate range
};

struct ProgArgs {
  const int64_t* rowptr;
  const int32_t* col;
  int64_t nv, ne;
  int32_t* scratch;
  int64_t slot_cap;   // ints per slot
  int nslots;
  // [0] entry head, [1] split tail, [2] split head, [3] v0 head (bitmap form), [4] stream
  // record tail, [5] stream record head
  unsigned long long* heads;
  SplitRec* split;
  int64_t split_cap;   // split records (then the stream records at split + split_cap)
  int64_t stream_cap;  // stream records of the bitmap form
  unsigned long long* total;
  int split_mode;
  int lut_ok;      // the bitmap kernel takes the tasks with small v0 (ProgLut)
  int lut_stream;  // its stream operation, or -1
  int lut_phase;   // k_setlut: 0 vertices, 1 stream records
  const uint32_t* lut_rows;  // stored rows of v0 with degree 33..1024 (or null)
  const int64_t* lut_off;
};

// Bitmap form: every task of a v0 of degree up to kLutDeg runs in k_setlut, one lane
// per (v0, v1) task, except the stream tasks with d(v1) > kLutStream, which become
// stream records (kStreamChunk entries of N(v1) each) for a second k_setlut pass.
constexpr int kLutDeg = 32;
constexpr int kLutStream = 32;
// A v0 of degree kLutDeg < d0 <= kLutMed runs its tasks in the warp-wide bitmap form
// (one word of N(v0) index space per lane) on the graph's stored rows.
constexpr int kLutMed = 1024;
constexpr int64_t kLutBudget = int64_t(4) << 30;  // bytes of stored rows at most

__device__ __forceinline__ bool lut_task_taken(const ProgArgs& a, int d0) {
  return a.lut_ok && d0 <= kLutDeg;
}

struct WarpState {
  int v[kProgMaxK];
  int vl[kProgMaxK];
  long long vb[kProgMaxK];
  int slen[kProgMaxSlots];
  // warp-wide bitmap form: index in N(v0) (or -1), elements of N(v0) below v_j, the
  // slots (one word per lane) and the row of a v2 outside N(v0)
  int idx[kProgMaxK];
  int pre[kProgMaxK];
  uint32_t bits[kLutSlots][32];
  uint32_t rowbuf[32];
  uint32_t fk[32];  // bits_flat_fin: the counted operand with the v3-independent masks
};

__device__ __forceinline__ unsigned lanemask_lt() {
  unsigned m;
  asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
  return m;
}

// Binary search for x in the sorted list b[0, len).
__device__ __forceinline__ bool member(const int32_t* b, int len, int x) {
  int lo = 0, n = len;
  while (n > 0) {
    const int h = n >> 1;
    if (__ldg(b + lo + h) < x) {
      lo += h + 1;
      n -= h + 1;
    } else {
      n = h;
    }
  }
  return lo < len && __ldg(b + lo) == x;
}

struct Operand {
  const int32_t* p;
  int n;
};

__device__ __forceinline__ Operand operand(const WarpState& w, int code, const ProgArgs& a,
                                           const int32_t* slots) {
  if (code >= kOpList) {
    const int j = code - kOpList;
    return Operand{a.col + w.vb[j], w.vl[j]};
  }
  return Operand{slots + (int64_t)code * a.slot_cap, w.slen[code]};
}

// The bound and exclusion masks of a program for K vertices name only v0..v_{K-2}
// (prog_check), so the loops over matched vertices run over K - 1 entries.
template <int K>
__device__ __forceinline__ int bound_of(const WarpState& w, unsigned mask) {
  int b = INT_MAX;
#pragma unroll
  for (int j = 0; j < K - 1; ++j)
    if ((mask >> j) & 1u) b = min(b, w.v[j]);
  return b;
}

template <int K>
struct Excl {
  int e[K - 1];
  __device__ __forceinline__ bool hit(int x) const {
    bool h = false;
#pragma unroll
    for (int j = 0; j < K - 1; ++j) h |= x == e[j];
    return h;
  }
};

template <int K>
__device__ __forceinline__ Excl<K> excl_of(const WarpState& w, unsigned mask) {
  Excl<K> r;
#pragma unroll
  for (int j = 0; j < K - 1; ++j) r.e[j] = ((mask >> j) & 1u) ? w.v[j] : -1;
  return r;
}

__device__ __forceinline__ void set_vertex(WarpState& w, int j, int x, const ProgArgs& a, int lane) {
  if (lane == 0) {
    const long long b = a.rowptr[x];
    w.v[j] = x;
    w.vb[j] = b;
    w.vl[j] = (int)(a.rowptr[x + 1] - b);
  }
  __syncwarp();
}

// out slot <- op(a, b); warp-wide.
template <int K>
__device__ void run_op(const ProgOp& o, WarpState& w, const ProgArgs& a, int32_t* slots, int lane) {
  const Operand A = operand(w, o.a, a, slots);
  const Operand B = o.kind == OP_FILTER ? Operand{nullptr, 0} : operand(w, o.b, a, slots);
  const int bnd = bound_of<K>(w, o.bound);
  const Excl<K> ex = excl_of<K>(w, o.excl);
  int32_t* out = slots + (int64_t)o.out * a.slot_cap;
  int written = 0;
  for (int base = 0; base < A.n; base += 32) {
    const int i = base + lane;
    const bool in = i < A.n;
    const int x = in ? A.p[i] : INT_MAX;
    const bool below = in && x < bnd;
    bool keep = below && !ex.hit(x);
    if (keep && o.kind != OP_FILTER) keep = member(B.p, B.n, x) == (o.kind == OP_INTERSECT);
    const unsigned m = __ballot_sync(0xffffffffu, keep);
    if (keep) out[written + __popc(m & lanemask_lt())] = x;
    written += __popc(m);
    if (__ballot_sync(0xffffffffu, in && !below)) break;
  }
  if (lane == 0) w.slen[o.out] = written;
  __syncwarp();
}

// |op(a, b)| for the counted vertex; per-lane partial.
template <int K>
__device__ unsigned long long count_op(const ProgOp& o, const WarpState& w, const ProgArgs& a,
                                       const int32_t* slots, int lane) {
  const Operand A = operand(w, o.a, a, slots);
  const Operand B = o.kind == OP_FILTER ? Operand{nullptr, 0} : operand(w, o.b, a, slots);
  const int bnd = bound_of<K>(w, o.bound);
  const Excl<K> ex = excl_of<K>(w, o.excl);
  unsigned long long c = 0;
  for (int base = 0; base < A.n; base += 32) {
    const int i = base + lane;
    const bool in = i < A.n;
    const int x = in ? A.p[i] : INT_MAX;
    const bool below = in && x < bnd;
    bool keep = below && !ex.hit(x);
    if (keep && o.kind != OP_FILTER) keep = member(B.p, B.n, x) == (o.kind == OP_INTERSECT);
    c += keep ? 1 : 0;
    if (__ballot_sync(0xffffffffu, in && !below)) break;
  }
  return c;
}

// First index of sorted A[0, n) at or above x.
__device__ __forceinline__ int lower_index(const int32_t* A, int n, int x) {
  int lo = 0;
  while (n > 0) {
    const int h = n >> 1;
    if (A[lo + h] < x) {
      lo += h + 1;
      n -= h + 1;
    } else {
      n = h;
    }
  }
  return lo;
}

// One lane's count for a candidate u whose list N(u) (du entries from rb) is short
// next to A: each y in N(u) is searched in A instead of each x of A in N(u).  The
// difference count is the number of A's elements that pass the bound and the
// exclusions, minus the intersection.
template <int K>
__device__ unsigned long long count_short(const Operand& A, int u, long long rb, int du, int sbnd,
                                          bool ubnd, const Excl<K>& ex, bool uex, bool want,
                                          const int32_t* col) {
  const int bnd = ubnd ? min(sbnd, u) : sbnd;
  const int m = lower_index(A.p, A.n, bnd);
  unsigned long long inter = 0;
  for (int i = 0; i < du; ++i) {
    const int y = col[rb + i];
    if (y >= bnd) break;
    if (ex.hit(y)) continue;  // y == u cannot occur: no self-loops
    inter += member(A.p, m, y) ? 1 : 0;
  }
  if (want) return inter;
  long long pass = m;
#pragma unroll
  for (int j = 0; j < K - 1; ++j) {
    bool dup = false;
#pragma unroll
    for (int i = 0; i < j; ++i) dup |= ex.e[i] == ex.e[j];
    if (ex.e[j] >= 0 && !dup && member(A.p, m, ex.e[j])) --pass;
  }
  if (uex && !ex.hit(u) && member(A.p, m, u)) --pass;
  return (unsigned long long)(pass - (long long)inter);
}

// Final count merged with the loop over v_iv (iv = k-2) running over C[lo, hi):
// one item per (candidate u, element x of the counted operand).  When the second
// operand is N(u) and A is long, candidates with short lists are counted one per lane
// by count_short, and only the others (gathered into `big`) take the item walk.
template <int K>
__device__ unsigned long long count_flat(const ProgOp& o, const WarpState& w, int iv, Operand C,
                                         int lo, int hi, const ProgArgs& a, const int32_t* slots,
                                         int32_t* big, int lane) {
  const Operand A = operand(w, o.a, a, slots);
  const unsigned ivbit = 1u << iv;
  const int sbnd = bound_of<K>(w, o.bound & ~ivbit);
  const bool ubnd = (o.bound & ivbit) != 0;
  const Excl<K> ex = excl_of<K>(w, o.excl & ~ivbit);
  const bool uex = (o.excl & ivbit) != 0;
  const bool filter = o.kind == OP_FILTER;
  const bool b_u = !filter && o.b == kOpList + iv;
  const Operand Bf = (filter || b_u) ? Operand{nullptr, 0} : operand(w, o.b, a, slots);
  const bool want = o.kind == OP_INTERSECT;
  int n = hi - lo;
  unsigned long long c = 0;
  if (A.n == 0 || n <= 0) return 0;
  if (b_u && A.n >= 64) {
    int nbig = 0;
    for (int base = 0; base < n; base += 32) {
      const int ci = base + lane;
      const bool in = ci < n;
      const int u = in ? C.p[lo + ci] : 0;
      const long long rb = in ? a.rowptr[u] : 0;
      const int du = in ? (int)(a.rowptr[u + 1] - rb) : 0;
      const bool small = in && 4 * du <= A.n;
      if (small) c += count_short<K>(A, u, rb, du, sbnd, ubnd, ex, uex, want, a.col);
      const unsigned mb = __ballot_sync(0xffffffffu, in && !small);
      if (in && !small) big[nbig + __popc(mb & lanemask_lt())] = u;
      nbig += __popc(mb);
    }
    __syncwarp();
    C = Operand{big, nbig};
    lo = 0;
    n = nbig;
    if (n == 0) return c;
  }
  int ci = lane / A.n, ai = lane - ci * A.n;
  while (ci < n) {
    const int u = C.p[lo + ci];
    const int x = A.p[ai];
    const int bnd = ubnd ? min(sbnd, u) : sbnd;
    if (x < bnd && !ex.hit(x) && !(uex && x == u)) {
      if (filter) {
        ++c;
      } else if (b_u) {
        const long long rb = a.rowptr[u];
        c += member(a.col + rb, (int)(a.rowptr[u + 1] - rb), x) == want ? 1 : 0;
      } else {
        c += member(Bf.p, Bf.n, x) == want ? 1 : 0;
      }
    }
    ai += 32;
    while (ai >= A.n) {
      ai -= A.n;
      ++ci;
    }
  }
  return c;
}

// Operands whose lengths bound the work of one v2 step: the level-0 slots (bit = slot)
// and the lists N(v0), N(v1) (bits 16, 17) that every operand read after level 0
// descends from.
__device__ unsigned step_roots(const Prog& p) {
  bool deep[kProgMaxSlots] = {};
  int8_t from[kProgMaxSlots] = {};
  for (int l = 1; l < kProgLevels; ++l)
    for (int i = 0; i < p.nops[l]; ++i) {
      deep[p.ops[l][i].out] = true;
      from[p.ops[l][i].out] = p.ops[l][i].a;
    }
  unsigned m = 0;
  auto add = [&](int c) {
    while (c < kOpList && deep[c]) c = from[c];  // operands are defined before use
    if (c < kOpList) m |= 1u << c;
    else if (c - kOpList <= 1) m |= 1u << (16 + c - kOpList);
  };
  for (int l = 1; l < kProgLevels; ++l)
    for (int i = 0; i < p.nops[l]; ++i) add(p.ops[l][i].a);
  add(p.fin.a);
  if (p.k >= 5) add(p.cand[3]);
  if (p.k == 6) add(p.cand[4]);
  return m;
}

template <int K>
__device__ unsigned long long run_task(const Prog& p, unsigned roots, WarpState& w,
                                       const ProgArgs& a, int32_t* slots, int v0, int v1,
                                       long long e, int lo, int hi, bool may_split, int lane) {
  int32_t* big = slots + (int64_t)a.nslots * a.slot_cap;  // count_flat's long-list candidates
  set_vertex(w, 0, v0, a, lane);
  set_vertex(w, 1, v1, a, lane);
  for (int i = 0; i < p.nops[0]; ++i) run_op<K>(p.ops[0][i], w, a, slots, lane);
  if constexpr (K == 3) return count_op<K>(p.fin, w, a, slots, lane);
  const Operand C2 = operand(w, p.cand[2], a, slots);
  if (hi < 0 || hi > C2.n) hi = C2.n;
  if (may_split && C2.n > 1) {
    // lane-steps of one v2 step: the streams of the level-1 operations, then the
    // final count over (v3, x) pairs (5 vertices), over x (4 vertices), or a v3 loop
    // of such counts (6 vertices)
    int len = 0;
    for (int j = 0; j < kProgMaxSlots; ++j)
      if ((roots >> j) & 1u) len = max(len, w.slen[j]);
    if ((roots >> 16) & 1u) len = max(len, w.vl[0]);
    if ((roots >> 17) & 1u) len = max(len, w.vl[1]);
    const long long step = 1 + len / 32 + (K >= 5 ? (long long)len * len / 64 : 0) *
                                                (K == 6 ? 1 + len / 32 : 1);
    if ((long long)C2.n * step > kSplitWork) {
      // every candidate goes to the records, so a warp that claims a chunk of heavy
      // tasks only builds their level-0 slots
      const int per = (int)max(1LL, min((long long)C2.n, kSplitWork / step));
      const int nrec = (C2.n + per - 1) / per;
      unsigned long long base = 0;
      if (lane == 0) base = atomicAdd(a.heads + 1, (unsigned long long)nrec);
      base = __shfl_sync(0xffffffffu, base, 0);
      const bool fits = base + nrec <= (unsigned long long)a.split_cap;
      for (int r = lane; r < nrec; r += 32) {
        // a claim that crosses the capacity leaves empty records below it; the task
        // then runs all of its candidates itself
        if (base + r >= (unsigned long long)a.split_cap) break;
        const int rlo = per * r;
        a.split[base + r] = fits ? SplitRec{(int32_t)(e & 0xffffffffLL), (int32_t)(e >> 32), rlo,
                                            min(rlo + per, C2.n)}
                                 : SplitRec{0, 0, 0, 0};
      }
      if (fits) return 0;
    }
  }
  unsigned long long c = 0;
  if constexpr (K == 4) {
    if (p.flat) return count_flat<K>(p.fin, w, 2, C2, lo, hi, a, slots, big, lane);
    for (int i2 = lo; i2 < hi; ++i2) {
      set_vertex(w, 2, C2.p[i2], a, lane);
      for (int i = 0; i < p.nops[1]; ++i) run_op<K>(p.ops[1][i], w, a, slots, lane);
      c += count_op<K>(p.fin, w, a, slots, lane);
    }
    return c;
  } else if constexpr (K == 5) {
    for (int i2 = lo; i2 < hi; ++i2) {
      set_vertex(w, 2, C2.p[i2], a, lane);
      for (int i = 0; i < p.nops[1]; ++i) run_op<K>(p.ops[1][i], w, a, slots, lane);
      const Operand C3 = operand(w, p.cand[3], a, slots);
      if (p.flat) {
        c += count_flat<K>(p.fin, w, 3, C3, 0, C3.n, a, slots, big, lane);
      } else {
        for (int i3 = 0; i3 < C3.n; ++i3) {
          set_vertex(w, 3, C3.p[i3], a, lane);
          for (int i = 0; i < p.nops[2]; ++i) run_op<K>(p.ops[2][i], w, a, slots, lane);
          c += count_op<K>(p.fin, w, a, slots, lane);
        }
      }
    }
    return c;
  } else {  // 6 vertices: one more enumerated level (v3), then as 5 vertices with v4
    for (int i2 = lo; i2 < hi; ++i2) {
      set_vertex(w, 2, C2.p[i2], a, lane);
      for (int i = 0; i < p.nops[1]; ++i) run_op<K>(p.ops[1][i], w, a, slots, lane);
      const Operand C3 = operand(w, p.cand[3], a, slots);
      for (int i3 = 0; i3 < C3.n; ++i3) {
        set_vertex(w, 3, C3.p[i3], a, lane);
        for (int i = 0; i < p.nops[2]; ++i) run_op<K>(p.ops[2][i], w, a, slots, lane);
        const Operand C4 = operand(w, p.cand[4], a, slots);
        if (p.flat) {
          c += count_flat<K>(p.fin, w, 4, C4, 0, C4.n, a, slots, big, lane);
        } else {
          for (int i4 = 0; i4 < C4.n; ++i4) {
            set_vertex(w, 4, C4.p[i4], a, lane);
            for (int i = 0; i < p.nops[3]; ++i) run_op<K>(p.ops[3][i], w, a, slots, lane);
            c += count_op<K>(p.fin, w, a, slots, lane);
          }
        }
      }
    }
    return c;
  }
}

__device__ __forceinline__ int row_of(const int64_t* rowptr, int64_t nv, long long e) {
  int64_t lo = 0, n = nv + 1;  // first index with rowptr[idx] > e, minus one
  while (n > 0) {
    const int64_t h = n >> 1;
    if (rowptr[lo + h] <= e) {
      lo += h + 1;
      n -= h + 1;
    } else {
      n = h;
    }
  }
  return (int)(lo - 1);
}

// ------------------------------------------------------- warp-wide bitmap form
// For a v0 of degree 33..1024 the tasks of a bitmap-eligible program run on the
// graph's stored rows (row i = the N(v0) indices adjacent to N(v0)[i], W = d0/32
// words): lane w owns word w of every N(v0)-space slot, an operation is one AND /
// AND-NOT per lane, and the final count one AND + popc per lane per v3 instead of
// binary searches.  A v2 from the stream N(v1) \ N(v0) gets its row built into
// `rowbuf` (each lane searches its share of N(v2) in N(v0)).

__device__ __forceinline__ bool bits_task(const ProgArgs& a, int d0) {
  return a.lut_ok && a.lut_rows && d0 > kLutDeg && d0 <= kLutMed;
}

struct BitsCtx {
  const int32_t* n0;    // N(v0)
  const uint32_t* row;  // stored rows of v0
  int d0, W;
  uint32_t valid;       // this lane's word of [0, d0)
  bool act;             // lane < W
};

__device__ __forceinline__ uint32_t bits_row(const WarpState& w, const BitsCtx& B, int code,
                                             int lane) {
  const int j = code - kOpList;
  if (j == 0) return B.valid;
  const int i = w.idx[j];
  if (i >= 0) return B.act ? B.row[(int64_t)i * B.W + lane] : 0u;
  return w.rowbuf[lane];
}

template <int K>
__device__ __forceinline__ uint32_t bits_keep(const WarpState& w, const BitsCtx& B, const ProgOp& o,
                                              int lane) {
  int pb = INT_MAX;
#pragma unroll
  for (int j = 0; j < K - 1; ++j)
    if ((o.bound >> j) & 1u) pb = min(pb, w.pre[j]);
  const int lo = 32 * lane;
  uint32_t m = pb >= lo + 32 ? 0xffffffffu : (pb <= lo ? 0u : ((1u << (pb - lo)) - 1u));
#pragma unroll
  for (int j = 0; j < K - 1; ++j)
    if (((o.excl >> j) & 1u) && w.idx[j] >= lo && w.idx[j] < lo + 32) m &= ~(1u << (w.idx[j] - lo));
  return m & B.valid;
}

__device__ __forceinline__ uint32_t bits_operand(const WarpState& w, const BitsCtx& B, int code,
                                                 int lane) {
  if (code == kOpList) return B.valid;                  // N(v0)
  if (code == kOpList + 1) return bits_row(w, B, code, lane);  // N(v1) n N(v0)
  return w.bits[code][lane];
}

template <int K>
__device__ __forceinline__ uint32_t bits_apply(const WarpState& w, const BitsCtx& B, const ProgOp& o,
                                               uint32_t A, int lane) {
  if (o.kind == OP_INTERSECT) A &= bits_row(w, B, o.b, lane);
  else if (o.kind == OP_DIFFERENCE) A &= ~bits_row(w, B, o.b, lane);
  return A & bits_keep<K>(w, B, o, lane);
}

template <int K>
__device__ __forceinline__ void bits_level(const Prog& p, int l, WarpState& w, const BitsCtx& B,
                                           int lane) {
  for (int i = 0; i < p.nops[l]; ++i) {
    const ProgOp& o = p.ops[l][i];
    w.bits[o.out][lane] = bits_apply<K>(w, B, o, bits_operand(w, B, o.a, lane), lane);
  }
}

__device__ __forceinline__ void bits_set(WarpState& w, int j, int x, int i, int pre, int lane) {
  if (lane == 0) {
    w.v[j] = x;
    w.idx[j] = i;
    w.pre[j] = pre;
  }
  __syncwarp();
}

// The final count with the v3 loop spread over lanes: the v3 candidates (bits of c3w,
// one word per lane) are compacted into `list`, then each lane counts one v3 over the
// W words.  Everything that does not depend on v3 (the counted operand, the valid
// range, the bound and exclusions of v0..v2, and the row of the second operand when it
// is not v3's) is folded into fk[] once; per v3 and word that leaves one AND (with v3's
// row) and a popc, plus v3's own bound / exclusion in its word.  For the programs whose
// last level is the count alone.
template <int K>
__device__ unsigned long long bits_flat_fin(const Prog& p, WarpState& w, const BitsCtx& B,
                                            uint32_t c3w, int32_t* list, int lane) {
  const ProgOp& o = p.fin;
  const bool ub = (o.bound >> 3) & 1u, ux = (o.excl >> 3) & 1u;
  const int jb = o.kind == OP_FILTER ? -1 : o.b - kOpList;
  const bool per_v3 = jb == 3;  // the second operand is N(v3)
  {
    ProgOp o2 = o;  // fold v0..v2's masks (and a row that is not v3's) into fk
    o2.bound &= 0x7u;
    o2.excl &= 0x7u;
    if (per_v3) o2.kind = OP_FILTER;
    w.fk[lane] = bits_apply<K>(w, B, o2, bits_operand(w, B, o.a, lane), lane);
  }
  const int cnt = __popc(c3w);
  int incl = cnt;
#pragma unroll
  for (int k = 1; k < 32; k <<= 1) {
    const int y = __shfl_up_sync(0xffffffffu, incl, k);
    if (lane >= k) incl += y;
  }
  const int n3 = __shfl_sync(0xffffffffu, incl, 31);
  int pos = incl - cnt;
  for (uint32_t m = c3w; m; m &= m - 1) list[pos++] = lane * 32 + __ffs(m) - 1;
  __syncwarp();
  const bool isect = o.kind == OP_INTERSECT;
  unsigned long long c = 0;
  for (int t = lane; t < n3; t += 32) {
    const int b3 = list[t];
    const int bw = b3 >> 5;
    const uint32_t below = (1u << (b3 & 31)) - 1u;
    const int lim = ub ? bw + 1 : B.W;
    const uint32_t* r3 = B.row + (int64_t)b3 * B.W;
    for (int wi = 0; wi < lim; ++wi) {
      uint32_t x = w.fk[wi];
      if (wi == bw) {
        if (ub) x &= below;
        if (ux) x &= ~(1u << (b3 & 31));
      }
      if (per_v3) x = isect ? (x & r3[wi]) : (x & ~r3[wi]);
      c += __popc(x);
    }
  }
  __syncwarp();
  return c;
}

// v2 fixed: the level-1 operations, then the v3 loop (5 vertices) or the count.
template <int K>
__device__ unsigned long long bits_step2(const Prog& p, WarpState& w, const BitsCtx& B,
                                         int32_t* list, int lane) {
  bits_level<K>(p, 1, w, B, lane);
  if (K == 4) return (unsigned long long)__popc(bits_apply<K>(w, B, p.fin, bits_operand(w, B, p.fin.a, lane), lane));
  __syncwarp();  // the level-1 slots are read across lanes below
  const uint32_t c3 = bits_operand(w, B, p.cand[3], lane);
  if (p.nops[2] == 0) return bits_flat_fin<K>(p, w, B, c3, list, lane);
  unsigned long long c = 0;
  for (int wi = 0; wi < B.W; ++wi) {
    for (uint32_t m = __shfl_sync(0xffffffffu, c3, wi); m; m &= m - 1) {
      const int b = wi * 32 + __ffs(m) - 1;
      bits_set(w, 3, B.n0[b], b, b, lane);
      bits_level<K>(p, 2, w, B, lane);
      c += __popc(bits_apply<K>(w, B, p.fin, bits_operand(w, B, p.fin.a, lane), lane));
    }
  }
  return c;
}

template <int K>
__device__ unsigned long long run_task_bits(const Prog& p, WarpState& w, const ProgArgs& a,
                                            int32_t* slots, int v0, int v1, long long e, int lo,
                                            int hi, bool may_split, int lane) {
  set_vertex(w, 0, v0, a, lane);
  set_vertex(w, 1, v1, a, lane);
  int32_t* list = slots + (int64_t)a.nslots * a.slot_cap;  // v3 candidates (bits_flat_fin)
  BitsCtx B;
  B.d0 = w.vl[0];
  B.W = (B.d0 + 31) >> 5;
  B.n0 = a.col + w.vb[0];
  B.row = a.lut_rows + a.lut_off[v0];
  B.act = lane < B.W;
  B.valid = !B.act ? 0u
                   : ((lane < B.W - 1 || (B.d0 & 31) == 0) ? 0xffffffffu
                                                           : ((1u << (B.d0 & 31)) - 1u));
  const int i1 = lower_index(B.n0, B.d0, v1);
  if (lane == 0) {
    w.idx[0] = -1;
    w.pre[0] = lower_index(B.n0, B.d0, v0);
    w.idx[1] = i1;
    w.pre[1] = i1;
  }
  __syncwarp();
  for (int i = 0; i < p.nops[0]; ++i) {
    const ProgOp& o = p.ops[0][i];
    if (i == a.lut_stream) run_op<K>(o, w, a, slots, lane);  // the v2 list N(v1) \ N(v0)
    else w.bits[o.out][lane] = bits_apply<K>(w, B, o, bits_operand(w, B, o.a, lane), lane);
  }
  __syncwarp();
  const bool stream = a.lut_stream >= 0;
  const Operand C2 = stream ? operand(w, p.cand[2], a, slots) : Operand{nullptr, 0};
  const uint32_t c2w = stream ? 0u : bits_operand(w, B, p.cand[2], lane);
  int n2 = stream ? C2.n : __popc(c2w);
  if (!stream) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) n2 += __shfl_xor_sync(0xffffffffu, n2, o);
  }
  if (hi < 0 || hi > n2) hi = n2;
  if (may_split && n2 > 1) {
    const long long step = 4 + (K == 5 ? B.d0 : 0);
    if ((long long)n2 * step > kSplitWork) {
      const int per = (int)max(1LL, min((long long)n2, kSplitWork / step));
      const int nrec = (n2 + per - 1) / per;
      unsigned long long base = 0;
      if (lane == 0) base = atomicAdd(a.heads + 1, (unsigned long long)nrec);
      base = __shfl_sync(0xffffffffu, base, 0);
      const bool fits = base + nrec <= (unsigned long long)a.split_cap;
      for (int r = lane; r < nrec; r += 32) {
        if (base + r >= (unsigned long long)a.split_cap) break;
        const int rlo = per * r;
        a.split[base + r] = fits ? SplitRec{(int32_t)(e & 0xffffffffLL), (int32_t)(e >> 32), rlo,
                                            min(rlo + per, n2)}
                                 : SplitRec{0, 0, 0, 0};
      }
      if (fits) return 0;
    }
  }
  unsigned long long c = 0;
  if (stream) {
    for (int i2 = lo; i2 < hi; ++i2) {
      // y's list bounds and its rank in N(v0) into registers (independent loads that
      // overlap), then into the warp state once every lane is done with the last v2
      const int y = C2.p[i2];
      const long long rby = a.rowptr[y];
      const int dy = (int)(a.rowptr[y + 1] - rby);
      const int pre = lower_index(B.n0, B.d0, y);
      __syncwarp();
      if (lane == 0) {
        w.v[2] = y;
        w.vb[2] = rby;
        w.vl[2] = dy;
        w.idx[2] = -1;
        w.pre[2] = pre;
      }
      w.rowbuf[lane] = 0u;
      __syncwarp();
      if (dy > B.d0) {
        // N(y) the longer list: each lane tests entries of N(v0) against N(y), and a
        // ballot gives each word of the row
        const int32_t* ny = a.col + rby;
        for (int base = 0; base < B.d0; base += 32) {
          const int i = base + lane;
          const unsigned word = __ballot_sync(0xffffffffu, i < B.d0 && member(ny, dy, B.n0[i]));
          if (lane == 0) w.rowbuf[base >> 5] = word;
        }
      } else {
        for (int t = lane; t < dy; t += 32) {
          const int z = a.col[rby + t];
          const int k = lower_index(B.n0, B.d0, z);
          if (k < B.d0 && B.n0[k] == z) atomicOr(&w.rowbuf[k >> 5], 1u << (k & 31));
        }
      }
      __syncwarp();
      c += bits_step2<K>(p, w, B, list, lane);
    }
  } else {
    int rank = 0;
    for (int wi = 0; wi < B.W && rank < hi; ++wi) {
      uint32_t m = __shfl_sync(0xffffffffu, c2w, wi);
      const int pc = __popc(m);
      if (rank + pc <= lo) {
        rank += pc;
        continue;
      }
      for (; m && rank < hi; m &= m - 1, ++rank) {
        if (rank < lo) continue;
        const int b = wi * 32 + __ffs(m) - 1;
        bits_set(w, 2, B.n0[b], b, b, lane);
        c += bits_step2<K>(p, w, B, list, lane);
      }
    }
  }
  return c;
}

// Stored rows: per v of degree 33..1024, d(v) rows of ceil(d(v)/32) words.
__global__ void k_lut_sizes(const int64_t* rowptr, int64_t nv, int64_t* sz) {
  for (int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; v < nv;
       v += (int64_t)gridDim.x * blockDim.x) {
    const int d = (int)(rowptr[v + 1] - rowptr[v]);
    sz[v] = (d > kLutDeg && d <= kLutMed) ? (int64_t)d * ((d + 31) / 32) : 0;
  }
}

// One warp per vertex v, one lane per row: the row of u = N(v)[i] scans N(u) into N(v)
// when that is cheaper, else searches every N(v) element in N(u).
__global__ void __launch_bounds__(kThreads) k_lut_rows(const int64_t* rowptr, const int32_t* col,
                                                       int64_t nv, const int64_t* off,
                                                       uint32_t* rows) {
  __shared__ uint32_t buf[kWarps][32][33];
  const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
  const int64_t nw = (int64_t)gridDim.x * kWarps;
  for (int64_t v = (int64_t)blockIdx.x * kWarps + wib; v < nv; v += nw) {
    const int64_t rb = rowptr[v];
    const int d = (int)(rowptr[v + 1] - rb);
    if (d <= kLutDeg || d > kLutMed) continue;
    const int W = (d + 31) >> 5;
    const int32_t* n0 = col + rb;
    uint32_t* out = rows + off[v];
    uint32_t* r = buf[wib][lane];
    const int lgd = 32 - __clz(d);
    for (int i = lane; i < d; i += 32) {
      for (int k = 0; k < W; ++k) r[k] = 0u;
      const int u = n0[i];
      const int64_t ru = rowptr[u];
      const int du = (int)(rowptr[u + 1] - ru);
      if ((int64_t)du * lgd <= (int64_t)d * (32 - __clz(du | 1))) {
        for (int t = 0; t < du; ++t) {
          const int y = col[ru + t];
          const int k = lower_index(n0, d, y);
          if (k < d && n0[k] == y) r[k >> 5] |= 1u << (k & 31);
        }
      } else {
        for (int k = 0; k < d; ++k)
          if (member(col + ru, du, n0[k])) r[k >> 5] |= 1u << (k & 31);
      }
      for (int k = 0; k < W; ++k) out[(int64_t)i * W + k] = r[k];
    }
  }
}

template <int K>
__global__ void __launch_bounds__(kThreads, 4) k_setprog(Prog prog, ProgArgs a) {
  __shared__ Prog p;
  __shared__ unsigned roots;
  __shared__ WarpState ws[kWarps];
  if (threadIdx.x == 0) {
    p = prog;
    roots = step_roots(prog);
  }
  __syncthreads();
  const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
  WarpState& w = ws[wib];
  int32_t* slots = a.scratch + ((int64_t)blockIdx.x * kWarps + wib) * (a.nslots + 1) * a.slot_cap;
  unsigned long long c = 0;
  if (!a.split_mode) {
    for (;;) {
      unsigned long long e0 = 0;
      if (lane == 0) e0 = atomicAdd(a.heads, (unsigned long long)kChunk);
      e0 = __shfl_sync(0xffffffffu, e0, 0);
      if ((long long)e0 >= a.ne) break;
      const long long e1 = min((long long)e0 + kChunk, (long long)a.ne);
      int v0 = 0;
      if (lane == 0) v0 = row_of(a.rowptr, a.nv, (long long)e0);
      v0 = __shfl_sync(0xffffffffu, v0, 0);
      for (long long e = (long long)e0; e < e1; ++e) {
        while (a.rowptr[v0 + 1] <= e) ++v0;
        const int v1 = a.col[e];
        if (p.v1lt && v1 >= v0) continue;
        const int d0 = (int)(a.rowptr[v0 + 1] - a.rowptr[v0]);
        if (lut_task_taken(a, d0)) continue;
        if (K >= 4 && bits_task(a, d0))
          c += run_task_bits<K>(p, w, a, slots, v0, v1, e, 0, -1, true, lane);
        else
          c += run_task<K>(p, roots, w, a, slots, v0, v1, e, 0, -1, true, lane);
      }
    }
  } else {
    const unsigned long long nrec = min(*(volatile unsigned long long*)(a.heads + 1),
                                        (unsigned long long)a.split_cap);
    for (;;) {
      unsigned long long r = 0;
      if (lane == 0) r = atomicAdd(a.heads + 2, 1ull);
      r = __shfl_sync(0xffffffffu, r, 0);
      if (r >= nrec) break;
      const SplitRec rec = a.split[r];
      if (rec.lo >= rec.hi) continue;
      const long long e = (long long)(uint32_t)rec.e_lo | ((long long)rec.e_hi << 32);
      int v0 = 0;
      if (lane == 0) v0 = row_of(a.rowptr, a.nv, e);
      v0 = __shfl_sync(0xffffffffu, v0, 0);
      const int d0 = (int)(a.rowptr[v0 + 1] - a.rowptr[v0]);
      if (K >= 4 && bits_task(a, d0))
        c += run_task_bits<K>(p, w, a, slots, v0, a.col[e], e, rec.lo, rec.hi, false, lane);
      else
        c += run_task<K>(p, roots, w, a, slots, v0, a.col[e], e, rec.lo, rec.hi, false, lane);
    }
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) c += __shfl_xor_sync(0xffffffffu, c, o);
  if (lane == 0 && c) atomicAdd(a.total, c);
}

// ------------------------------------------------------------------ bitmap form
// GLUMIN's LUT kernels (GM_LUT_kernels/P*.yml.cuh, codegen_LUT.cuh) keep the adjacency
// among N(v0) as bit rows and run the plan on them.  Here a warp takes one v0 of
// degree <= 32: N(v0) and its 32-bit rows (row i = the N(v0) indices adjacent to
// N(v0)[i]) sit in shared memory, and each lane runs one task (v0, v1) on 32-bit masks
// in N(v0) index space: an intersection is an AND with a row, a difference an AND with
// its complement, a bound (x < v_j) a prefix mask (N(v0) is sorted), an exclusion one
// cleared bit, and the count a popc.  The row of v0 is all of N(v0); a v2 from the
// stream N(v1) \ N(v0) is not in that space and gets its row built on the fly.

// Bits of N(v0) (n0[0, d0), sorted) adjacent to y: a merge when N(y) is short, else a
// binary search of each N(v0) element in N(y).
__device__ uint32_t row_over(const int32_t* n0, int d0, int y, const ProgArgs& a) {
  const long long rb = a.rowptr[y];
  const int dy = (int)(a.rowptr[y + 1] - rb);
  uint32_t r = 0;
  if (dy <= 8 * d0) {
    int i = 0;
    for (int j = 0; j < dy && i < d0; ++j) {
      const int z = a.col[rb + j];
      while (i < d0 && n0[i] < z) ++i;
      if (i < d0 && n0[i] == z) r |= 1u << i;
    }
  } else {
    for (int i = 0; i < d0; ++i)
      if (member(a.col + rb, dy, n0[i])) r |= 1u << i;
  }
  return r;
}

// Two-hop rows of a small v0 (stream programs): for every y adjacent to some N(v0)[i],
// the bits i with y in N(N(v0)[i]) — which is y's row over N(v0) (the graph is
// symmetric).  Built once per v0 by streaming the N(v0) members' lists into an
// open-addressing map in shared memory, so a streamed v2's row is one probe instead of
// a walk over N(v2).  Skipped (rows built on the fly) when the lists would fill more
// than half the map.
constexpr int kMapSlots = 512;

__device__ __forceinline__ uint32_t map_hash(int y) { return ((uint32_t)y * 2654435761u) >> 23; }

// Returns whether the map was built (all lanes agree).
__device__ bool map_build(int32_t* hkey, uint32_t* hval, const int32_t* n0, int d0,
                          const ProgArgs& a, int lane) {
  long long tot = 0;
  if (lane < d0) tot = a.rowptr[n0[lane] + 1] - a.rowptr[n0[lane]];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) tot += __shfl_xor_sync(0xffffffffu, tot, o);
  if (tot > kMapSlots / 2) return false;
  for (int k = lane; k < kMapSlots; k += 32) hkey[k] = -1, hval[k] = 0u;
  __syncwarp();
  for (int i = 0; i < d0; ++i) {
    const long long rb = a.rowptr[n0[i]];
    const int du = (int)(a.rowptr[n0[i] + 1] - rb);
    for (int t = lane; t < du; t += 32) {
      const int y = a.col[rb + t];
      uint32_t h = map_hash(y);
      for (int probe = 0; probe < kMapSlots; ++probe, h = (h + 1) & (kMapSlots - 1)) {
        const int prev = atomicCAS(&hkey[h], -1, y);
        if (prev == -1 || prev == y) {
          atomicOr(&hval[h], 1u << i);
          break;
        }
      }
    }
  }
  __syncwarp();
  return true;
}

__device__ __forceinline__ uint32_t map_row(const int32_t* hkey, const uint32_t* hval, int y) {
  uint32_t h = map_hash(y);
  for (int probe = 0; probe < kMapSlots; ++probe, h = (h + 1) & (kMapSlots - 1)) {
    const int k = hkey[h];
    if (k == y) return hval[h];
    if (k == -1) break;
  }
  return 0u;
}

struct LutLane {
  int v[kProgMaxK];    // matched ids
  int idx[kProgMaxK];  // index in N(v0), or -1
  int pre[kProgMaxK];  // elements of N(v0) below v_j
  uint32_t row[kProgMaxK];
};

template <int K>
__device__ __forceinline__ uint32_t row_of_code(const LutLane& L, int code) {
  uint32_t r = 0;
#pragma unroll
  for (int j = 0; j < K - 1; ++j)
    if (code == kOpList + j) r = L.row[j];
  return r;
}

// prefix mask of the bound (x < min v_j) and the exclusion mask, over matched vertices
template <int K>
__device__ __forceinline__ uint32_t keep_mask(const LutLane& L, const ProgOp& o, uint32_t valid) {
  int pb = 32;
  uint32_t ex = 0;
#pragma unroll
  for (int j = 0; j < K - 1; ++j) {
    if ((o.bound >> j) & 1u) pb = min(pb, L.pre[j]);
    if (((o.excl >> j) & 1u) && L.idx[j] >= 0) ex |= 1u << L.idx[j];
  }
  const uint32_t pm = pb >= 32 ? 0xffffffffu : ((1u << pb) - 1u);
  return valid & pm & ~ex;
}

template <int K>
__device__ __forceinline__ uint32_t lut_apply(const LutLane& L, const ProgOp& o, uint32_t A,
                                              uint32_t valid) {
  uint32_t r = A;
  if (o.kind == OP_INTERSECT) r &= row_of_code<K>(L, o.b);
  else if (o.kind == OP_DIFFERENCE) r &= ~row_of_code<K>(L, o.b);
  return r & keep_mask<K>(L, o, valid);
}

// Slot columns of a bitmap task (stride 32 words): the slots of level 0 are read from
// the column of the lane that ran the task's level-0 operations (`head`), the slots of
// the later levels live in the running lane's own column.  A slot is defined once, so
// the two sets of indices are disjoint.
struct LutSlots {
  uint32_t* own;
  const uint32_t* head;
  unsigned l0;  // slots defined at level 0
  __device__ __forceinline__ uint32_t get(int code) const {
    return ((l0 >> code) & 1u) ? head[code * 32] : own[code * 32];
  }
};

__device__ __forceinline__ uint32_t lut_operand(const LutLane& L, int code, const LutSlots& S,
                                                uint32_t valid) {
  if (code == kOpList) return valid;               // N(v0)
  if (code == kOpList + 1) return L.row[1];        // N(v1) n N(v0), the only use of N(v1)
  return S.get(code);
}

__device__ __forceinline__ void lut_set(LutLane& L, int j, int x, int i, const int32_t* n0, int d0) {
  L.v[j] = x;
  L.idx[j] = i;
  L.pre[j] = i >= 0 ? i : lower_index(n0, d0, x);
}

template <int K>
__device__ unsigned long long lut_level(const Prog& p, int l, LutLane& L, const LutSlots& S,
                                        uint32_t valid) {
  for (int i = 0; i < p.nops[l]; ++i) {
    const ProgOp& o = p.ops[l][i];
    S.own[o.out * 32] = lut_apply<K>(L, o, lut_operand(L, o.a, S, valid), valid);
  }
  if (l == K - 3) return (unsigned long long)__popc(lut_apply<K>(L, p.fin, lut_operand(L, p.fin.a, S, valid), valid));
  return 0;
}

// v0, v1, v2 matched (and the level-0 slots written): the level-1 operations, then the
// count (4 vertices) or the v3 loop (5 vertices).  When the last level is the count
// alone, everything that does not depend on v3 (operand, valid range, bounds /
// exclusions of v0..v2, a row that is not v3's) is folded once per v2, then per v3 its
// own bound, exclusion and row, and a popc.
template <int K>
__device__ unsigned long long lut_step2(const Prog& p, LutLane& L, const LutSlots& S,
                                        uint32_t valid, const int32_t* n0, int d0,
                                        const uint32_t* lut) {
  if (K == 4) return lut_level<K>(p, 1, L, S, valid);
  lut_level<K>(p, 1, L, S, valid);
  const uint32_t c3 = lut_operand(L, p.cand[3], S, valid);
  const ProgOp& fo = p.fin;
  unsigned long long c = 0;
  if (K == 5 && p.nops[2] == 0) {
    const bool f_ub = (fo.bound >> 3) & 1u, f_ux = (fo.excl >> 3) & 1u;
    const bool f_v3 = fo.kind != OP_FILTER && fo.b == kOpList + 3;
    const bool f_is = fo.kind == OP_INTERSECT;
    ProgOp o2 = fo;
    o2.bound &= 0x7u;
    o2.excl &= 0x7u;
    if (f_v3) o2.kind = OP_FILTER;
    const uint32_t fk = lut_apply<K>(L, o2, lut_operand(L, fo.a, S, valid), valid);
    for (uint32_t m = c3; m; m &= m - 1) {
      const int b = __ffs(m) - 1;
      uint32_t x = fk;
      if (f_ub) x &= (1u << b) - 1u;
      if (f_ux) x &= ~(1u << b);
      if (f_v3) x = f_is ? (x & lut[b]) : (x & ~lut[b]);
      c += (unsigned long long)__popc(x);
    }
    return c;
  }
  for (uint32_t m = c3; m; m &= m - 1) {
    const int b = __ffs(m) - 1;
    lut_set(L, 3, n0[b], b, n0, d0);
    L.row[3] = lut[b];
    c += lut_level<K>(p, 2, L, S, valid);
  }
  return c;
}

// One (v0, v1) task on masks; sl = this lane's slots (stride 32).  A stream program's
// v2 candidates are the entries t0, t0 + ts, ... of N(v1) within [s_lo, s_hi) (ts = 1:
// this lane runs the whole task; ts = 32: the warp's lanes share it).
template <int K>
__device__ unsigned long long lut_task(const Prog& p, const ProgArgs& a, int v0, int i1, int d0,
                                       const int32_t* n0, const uint32_t* lut, uint32_t* sl,
                                       int t0, int ts, int s_lo = 0, int s_hi = 1 << 30,
                                       const int32_t* hkey = nullptr,
                                       const uint32_t* hval = nullptr) {
  const int v1 = n0[i1];
  if (p.v1lt && v1 >= v0) return 0;
  const long long rb1 = a.rowptr[v1];
  const int d1 = (int)(a.rowptr[v1 + 1] - rb1);
  const uint32_t valid = d0 >= 32 ? 0xffffffffu : ((1u << d0) - 1u);
  LutLane L;
#pragma unroll
  for (int j = 0; j < kProgMaxK; ++j) L.v[j] = -1, L.idx[j] = -1, L.pre[j] = 0, L.row[j] = 0;
  lut_set(L, 0, v0, -1, n0, d0);
  L.row[0] = valid;
  lut_set(L, 1, v1, i1, n0, d0);
  L.row[1] = lut[i1];
  const LutSlots S{sl, sl, 0u};
  for (int i = 0; i < p.nops[0]; ++i) {
    if (i == a.lut_stream) continue;
    const ProgOp& o = p.ops[0][i];
    sl[o.out * 32] = lut_apply<K>(L, o, lut_operand(L, o.a, S, valid), valid);
  }
  unsigned long long c = 0;
  if (a.lut_stream >= 0) {
    // v2 over N(v1) \ N(v0), below the operation's bound, minus its exclusions
    const ProgOp& o = p.ops[0][a.lut_stream];
    int ub = INT_MAX;
#pragma unroll
    for (int j = 0; j < 2; ++j)
      if ((o.bound >> j) & 1u) ub = min(ub, L.v[j]);
    const int tend = min(d1, s_hi);
    for (int t = max(t0, s_lo); t < tend; t += ts) {
      const int y = a.col[rb1 + t];
      if (y >= ub) break;
      const int i = lower_index(n0, d0, y);
      if (i < d0 && n0[i] == y) continue;
      if ((((o.excl >> 0) & 1u) && y == v0) || (((o.excl >> 1) & 1u) && y == v1)) continue;
      lut_set(L, 2, y, -1, n0, d0);
      L.row[2] = hkey ? map_row(hkey, hval, y) : row_over(n0, d0, y, a);
      c += lut_step2<K>(p, L, S, valid, n0, d0, lut);
    }
  } else {
    for (uint32_t m = lut_operand(L, p.cand[2], S, valid); m; m &= m - 1) {
      const int b = __ffs(m) - 1;
      lut_set(L, 2, n0[b], b, n0, d0);
      L.row[2] = lut[b];
      c += lut_step2<K>(p, L, S, valid, n0, d0, lut);
    }
  }
  return c;
}

// Phase 0 of a stream program for one v0 (d0 <= 32), as a warp: lane i runs the
// level-0 operations of task (v0, N(v0)[i]) when `mine` (d(v1) within the bitmap
// range, v1 allowed); then the (task, v2) pairs of all those tasks (v2 over the part of
// N(v1) below the stream's bound) are dealt out to the lanes in turn, so that a lane's
// work no longer follows the length of its own task's stream.  A pair reads its task's
// level-0 slots from the task's lane (`sw` = the warp's slot columns, written before
// the call).  All lanes call this.
template <int K>
__device__ unsigned long long lut_stream_pairs(const Prog& p, const ProgArgs& a, int v0, int d0,
                                               const int32_t* n0, const uint32_t* lut,
                                               uint32_t* sw, unsigned l0, bool mine,
                                               const int32_t* hkey, const uint32_t* hval,
                                               int lane) {
  const uint32_t valid = d0 >= 32 ? 0xffffffffu : ((1u << d0) - 1u);
  const int pre0 = lower_index(n0, d0, v0);
  const ProgOp& so = p.ops[0][a.lut_stream];
  LutLane L;
#pragma unroll
  for (int j = 0; j < kProgMaxK; ++j) L.v[j] = -1, L.idx[j] = -1, L.pre[j] = 0, L.row[j] = 0;
  L.v[0] = v0;
  L.pre[0] = pre0;
  L.row[0] = valid;
  long long rb1 = 0;
  int n = 0;
  if (mine) {
    const int v1 = n0[lane];
    if (!(p.v1lt && v1 >= v0)) {
      lut_set(L, 1, v1, lane, n0, d0);
      L.row[1] = lut[lane];
      const LutSlots S{sw + lane, sw + lane, 0u};
      for (int i = 0; i < p.nops[0]; ++i) {
        if (i == a.lut_stream) continue;
        const ProgOp& o = p.ops[0][i];
        sw[o.out * 32 + lane] = lut_apply<K>(L, o, lut_operand(L, o.a, S, valid), valid);
      }
      int ub = INT_MAX;
      if (so.bound & 1u) ub = min(ub, v0);
      if ((so.bound >> 1) & 1u) ub = min(ub, v1);
      rb1 = a.rowptr[v1];
      n = lower_index(a.col + rb1, (int)(a.rowptr[v1 + 1] - rb1), ub);
    }
  }
  __syncwarp();  // the level-0 slots are read by other lanes below
  int incl = n;
#pragma unroll
  for (int k = 1; k < 32; k <<= 1) {
    const int y = __shfl_up_sync(0xffffffffu, incl, k);
    if (lane >= k) incl += y;
  }
  const int total = __shfl_sync(0xffffffffu, incl, 31);
  const bool ex0 = so.excl & 1u, ex1 = (so.excl >> 1) & 1u;
  unsigned long long c = 0;
  for (int base = 0; base < total; base += 32) {
    const int item = base + lane;
    // the task of this item: the first lane whose inclusive count passes it
    int t = 0;
#pragma unroll
    for (int s = 16; s > 0; s >>= 1) {
      const int v = __shfl_sync(0xffffffffu, incl, t + s - 1);
      if (v <= item) t += s;
    }
    const int first = __shfl_sync(0xffffffffu, incl - n, t);
    const long long rbt = __shfl_sync(0xffffffffu, rb1, t);
    if (item >= total) continue;
    const int v1 = n0[t];
    const int y = a.col[rbt + (item - first)];
    const int i = lower_index(n0, d0, y);
    if (i < d0 && n0[i] == y) continue;  // in N(v0): not a stream vertex
    if ((ex0 && y == v0) || (ex1 && y == v1)) continue;
    L.v[1] = v1;
    L.idx[1] = t;
    L.pre[1] = t;
    L.row[1] = lut[t];
    L.v[2] = y;
    L.idx[2] = -1;
    L.pre[2] = i;
    L.row[2] = hkey ? map_row(hkey, hval, y) : row_over(n0, d0, y, a);
    const LutSlots S{sw + lane, sw + t, l0};
    c += lut_step2<K>(p, L, S, valid, n0, d0, lut);
  }
  __syncwarp();
  return c;
}

// N(v0) and its rows into the warp's shared memory (lanes < d0).
__device__ __forceinline__ void lut_load(int32_t* n0, uint32_t* lut, long long rb, int d0,
                                         const ProgArgs& a, int lane) {
  if (lane < d0) n0[lane] = a.col[rb + lane];
  __syncwarp();
  if (lane < d0) lut[lane] = row_over(n0, d0, n0[lane], a);
  __syncwarp();
}

template <int K>
__global__ void __launch_bounds__(kThreads, 4) k_setlut(Prog prog, ProgArgs a) {
  __shared__ Prog p;
  __shared__ int32_t n0s[kWarps][32];
  __shared__ uint32_t luts[kWarps][32];
  __shared__ uint32_t sls[kWarps][kLutSlots * 32];
  __shared__ int32_t hkeys[kWarps][kMapSlots];
  __shared__ uint32_t hvals[kWarps][kMapSlots];
  if (threadIdx.x == 0) p = prog;
  __syncthreads();
  const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
  SplitRec* srec = a.split + a.split_cap;  // stream records
  unsigned l0 = 0;  // slots written by the level-0 operations
  for (int i = 0; i < p.nops[0]; ++i)
    if (i != a.lut_stream) l0 |= 1u << p.ops[0][i].out;
  int32_t* hk = hkeys[wib];
  uint32_t* hv = hvals[wib];
  unsigned long long c = 0;
  if (a.lut_phase == 0) {
    for (;;) {
      unsigned long long v0 = 0;
      if (lane == 0) v0 = atomicAdd(a.heads + 3, 1ull);
      v0 = __shfl_sync(0xffffffffu, v0, 0);
      if ((long long)v0 >= a.nv) break;
      const long long rb = a.rowptr[v0];
      const int d0 = (int)(a.rowptr[v0 + 1] - rb);
      if (d0 == 0 || d0 > kLutDeg) continue;
      lut_load(n0s[wib], luts[wib], rb, d0, a, lane);
      const bool mapped = a.lut_stream >= 0 && map_build(hk, hv, n0s[wib], d0, a, lane);
      // one lane per task (stream programs: one lane per (task, v2) pair); stream tasks
      // with a long N(v1) become stream records
      int d1 = 0;
      if (lane < d0) {
        const int v1 = n0s[wib][lane];
        d1 = (int)(a.rowptr[v1 + 1] - a.rowptr[v1]);
        if (a.lut_stream < 0)
          c += lut_task<K>(p, a, (int)v0, lane, d0, n0s[wib], luts[wib], &sls[wib][lane], 0, 1,
                           0, 1 << 30, nullptr, hv);
      }
      __syncwarp();
      if (a.lut_stream >= 0)
        c += lut_stream_pairs<K>(p, a, (int)v0, d0, n0s[wib], luts[wib], sls[wib], l0,
                                 lane < d0 && d1 <= kLutStream, mapped ? hk : nullptr, hv, lane);
      if (a.lut_stream >= 0) {
        const bool lng = lane < d0 && d1 > kLutStream;
        const int nrec = lng ? (d1 + kStreamChunk - 1) / kStreamChunk : 0;
        const unsigned long long base = nrec ? atomicAdd(a.heads + 4, (unsigned long long)nrec) : 0;
        const bool fits = base + nrec <= (unsigned long long)a.stream_cap;
        for (int r = 0; r < nrec; ++r)
          if (base + r < (unsigned long long)a.stream_cap)
            srec[base + r] = fits ? SplitRec{(int32_t)v0, lane, r * kStreamChunk,
                                            min((r + 1) * kStreamChunk, d1)}
                                  : SplitRec{0, 0, 0, 0};
        // no room: the warp runs the task itself, lanes striding over N(v1)
        unsigned todo = __ballot_sync(0xffffffffu, lng && !fits);
        for (; todo; todo &= todo - 1) {
          const int i1 = __ffs(todo) - 1;
          c += lut_task<K>(p, a, (int)v0, i1, d0, n0s[wib], luts[wib], &sls[wib][lane], lane, 32,
                           0, 1 << 30, mapped ? hk : nullptr, hv);
        }
        __syncwarp();
      }
    }
  } else {
    const unsigned long long nrec = min(*(volatile unsigned long long*)(a.heads + 4),
                                        (unsigned long long)a.stream_cap);
    for (;;) {
      unsigned long long r = 0;
      if (lane == 0) r = atomicAdd(a.heads + 5, 1ull);
      r = __shfl_sync(0xffffffffu, r, 0);
      if (r >= nrec) break;
      const SplitRec rec = srec[r];
      if (rec.lo >= rec.hi) continue;
      const int v0 = rec.e_lo;
      const long long rb = a.rowptr[v0];
      const int d0 = (int)(a.rowptr[v0 + 1] - rb);
      lut_load(n0s[wib], luts[wib], rb, d0, a, lane);
      const bool mapped = map_build(hk, hv, n0s[wib], d0, a, lane);
      c += lut_task<K>(p, a, v0, rec.e_hi, d0, n0s[wib], luts[wib], &sls[wib][lane], rec.lo + lane,
                       32, rec.lo, rec.hi, mapped ? hk : nullptr, hv);
      __syncwarp();
    }
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) c += __shfl_xor_sync(0xffffffffu, c, o);
  if (lane == 0 && c) atomicAdd(a.total, c);
}

template <int K>
cudaError_t launch_k(const Prog& p, const ProgArgs& a, int grid, cudaStream_t s) {
  ProgArgs b = a;
  b.split_mode = 0;
  if (K >= 4 && a.lut_ok) {
    b.lut_phase = 0;
    k_setlut<K><<<grid, kThreads, 0, s>>>(p, b);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    if (a.lut_stream >= 0) {
      b.lut_phase = 1;
      k_setlut<K><<<grid, kThreads, 0, s>>>(p, b);
      e = cudaGetLastError();
      if (e != cudaSuccess) return e;
    }
  }
  k_setprog<K><<<grid, kThreads, 0, s>>>(p, b);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess || K == 3) return e;
  b.split_mode = 1;
  k_setprog<K><<<grid, kThreads, 0, s>>>(p, b);
  return cudaGetLastError();
}

int occupancy(int k) {
  int n = 0;
  cudaError_t e = k == 3   ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_setprog<3>, kThreads, 0)
                  : k == 4 ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_setprog<4>, kThreads, 0)
                  : k == 5 ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_setprog<5>, kThreads, 0)
                           : cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_setprog<6>, kThreads, 0);
  return (e == cudaSuccess && n > 0) ? n : 1;
}

}  // namespace

// Stored rows for the warp-wide bitmap form, built once per graph (kept while they
// fit kLutBudget; otherwise those tasks stay on the list form).
cudaError_t ensure_lut_rows(const DevGraph& g, cudaStream_t s) {
  if (g.lut_state != 0) return cudaSuccess;
  if (g.nv == 0) {
    g.lut_state = -1;
    return cudaSuccess;
  }
  int64_t* off = nullptr;
  cudaError_t e = cudaMallocAsync((void**)&off, sizeof(int64_t) * (g.nv + 1), s);
  if (e == cudaErrorMemoryAllocation) {  // no room: those tasks stay on the list form
    cudaGetLastError();
    g.lut_state = -1;
    return cudaSuccess;
  }
  if (e != cudaSuccess) return e;
  const int blocks = (int)std::min<int64_t>((g.nv + kThreads - 1) / kThreads, 65536);
  k_lut_sizes<<<blocks, kThreads, 0, s>>>(g.rowptr_o, g.nv, off);
  e = cudaGetLastError();
  if (e == cudaSuccess) e = scan_excl(off, off, g.nv, off + g.nv, s);
  int64_t total = 0;
  if (e == cudaSuccess) e = cudaMemcpyAsync(&total, off + g.nv, sizeof(int64_t), cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess || total == 0 || total * (int64_t)sizeof(uint32_t) > kLutBudget) {
    cudaFreeAsync(off, s);
    if (e == cudaSuccess) g.lut_state = -1;
    return e;
  }
  uint32_t* rows = nullptr;
  e = cudaMallocAsync((void**)&rows, sizeof(uint32_t) * total, s);
  if (e != cudaSuccess) {
    cudaFreeAsync(off, s);
    if (e != cudaErrorMemoryAllocation) return e;
    cudaGetLastError();
    g.lut_state = -1;
    return cudaSuccess;
  }
  const int wblocks = (int)std::min<int64_t>((g.nv + kWarps - 1) / kWarps, 65536);
  k_lut_rows<<<wblocks, kThreads, 0, s>>>(g.rowptr_o, g.col_o, g.nv, off, rows);
  e = cudaGetLastError();
  if (e != cudaSuccess) {
    cudaFreeAsync(rows, s);
    cudaFreeAsync(off, s);
    return e;
  }
  g.lut_rows = rows;
  g.lut_off = off;
  g.lut_state = 1;
  return cudaSuccess;
}

xgm_status count_program(xgm_ctx* ctx, const DevGraph& g, const Prog& p, uint64_t* out,
                         xgm_stats& st) {
  std::string why;
  if (!prog_check(p, &why)) {
    set_thread_error("invalid set-operation program: " + why);
    return XGM_ERR_INVALID;
  }
  cudaStream_t s = ctx->stream;
  XGM_CUDA_TRY(cudaSetDevice(ctx->device));
  XGM_CUDA_TRY(cudaMemsetAsync(ctx->d_sc, 0, sizeof(Scalars), s));
  XGM_CUDA_TRY(cudaEventRecord(ctx->ev[0], s));
  const int nslots = p.nslots > 0 ? p.nslots : 1;
  const int64_t slot_cap = g.max_deg > 0 ? g.max_deg : 1;
  // resident warps, fewer when the scratch would pass 8 GB
  int grid = ctx->num_sms * occupancy(p.k);
  // per warp: the program's slots and one list of candidates for count_flat
  const int64_t per_block = (int64_t)kWarps * (nslots + 1) * slot_cap * (int64_t)sizeof(int32_t);
  const int64_t budget = int64_t(8) << 30;
  if ((int64_t)grid * per_block > budget)
    grid = (int)std::max<int64_t>(ctx->num_sms, budget / per_block);
  const int64_t need = (int64_t)grid * kWarps * (nslots + 1) * slot_cap;
  if (need > ctx->prog_scratch_cap) {
    if (ctx->prog_scratch) XGM_CUDA_TRY(cudaFreeAsync(ctx->prog_scratch, s));
    ctx->prog_scratch = nullptr;
    ctx->prog_scratch_cap = 0;
    XGM_CUDA_TRY(cudaMallocAsync((void**)&ctx->prog_scratch, sizeof(int32_t) * need, s));
    ctx->prog_scratch_cap = need;
  }
  if (!ctx->prog_split) {
    XGM_CUDA_TRY(cudaMallocAsync((void**)&ctx->prog_split,
                                 sizeof(SplitRec) * (kSplitCap + kStreamCap), s));
    XGM_CUDA_TRY(cudaMallocAsync((void**)&ctx->prog_heads, sizeof(unsigned long long) * 8, s));
  }
  XGM_CUDA_TRY(cudaMemsetAsync(ctx->prog_heads, 0, sizeof(unsigned long long) * 8, s));
  ProgLut lut;
  const bool lut_ok = prog_lut(p, &lut);
  if (lut_ok && p.k >= 4) XGM_CUDA_TRY(ensure_lut_rows(g, s));  // once per graph
  XGM_CUDA_TRY(cudaEventRecord(ctx->ev[1], s));
  ProgArgs a;
  a.rowptr = g.rowptr_o;
  a.col = g.col_o;
  a.nv = g.nv;
  a.ne = g.ne;
  a.scratch = ctx->prog_scratch;
  a.slot_cap = slot_cap;
  a.nslots = nslots;
  a.heads = (unsigned long long*)ctx->prog_heads;
  a.split = (SplitRec*)ctx->prog_split;
  a.split_cap = kSplitCap;
  a.stream_cap = kStreamCap;
  // test hook: XGM_PROG_RECORD_CAP lowers both record capacities, so the overflow
  // paths (a task that cannot queue its records runs them itself) can be exercised
  if (const char* cap = std::getenv("XGM_PROG_RECORD_CAP")) {
    const long long c = std::atoll(cap);
    if (c >= 0) {
      a.split_cap = std::min<int64_t>(a.split_cap, c);
      a.stream_cap = std::min<int64_t>(a.stream_cap, c);
    }
  }
  a.total = &ctx->d_sc->count;
  a.split_mode = 0;
  a.lut_ok = lut_ok ? 1 : 0;
  a.lut_stream = lut.stream;
  a.lut_phase = 0;
  a.lut_rows = (lut_ok && g.lut_state == 1) ? g.lut_rows : nullptr;
  a.lut_off = (lut_ok && g.lut_state == 1) ? g.lut_off : nullptr;
  int launches = 0;
  if (g.ne > 0) {
    cudaError_t e = p.k == 3   ? launch_k<3>(p, a, grid, s)
                    : p.k == 4 ? launch_k<4>(p, a, grid, s)
                    : p.k == 5 ? launch_k<5>(p, a, grid, s)
                               : launch_k<6>(p, a, grid, s);
    if (e != cudaSuccess) return cuda_fail(e, "k_setprog", __FILE__, __LINE__);
    launches = p.k == 3 ? 1 : (a.lut_ok ? (a.lut_stream >= 0 ? 4 : 3) : 2);
  }
  XGM_CUDA_TRY(cudaEventRecord(ctx->ev[2], s));
  XGM_CUDA_TRY(cudaMemcpyAsync(ctx->d_sc->n, ctx->prog_heads + 1, sizeof(int64_t),
                               cudaMemcpyDeviceToDevice, s));
  xgm_status r = ctx_sync_scalars(ctx);
  if (r != XGM_OK) return r;
  float prep = 0, kern = 0;
  cudaEventElapsedTime(&prep, ctx->ev[0], ctx->ev[1]);
  cudaEventElapsedTime(&kern, ctx->ev[1], ctx->ev[2]);
  std::memset(&st, 0, sizeof(st));
  st.prep_ms = prep;
  st.kernel_ms = kern;
  st.launches = launches;
  st.tasks = g.ne;
  st.variant_tasks[XGM_VAR_SPLIT] = std::min<int64_t>(ctx->h_sc->n[0], a.split_cap);
  *out = ctx->h_sc->count;
  return XGM_OK;
}

void program_buffers_free(xgm_ctx* ctx) {
  cudaStream_t s = ctx->stream;
  if (ctx->prog_scratch) cudaFreeAsync(ctx->prog_scratch, s);
  if (ctx->prog_split) cudaFreeAsync(ctx->prog_split, s);
  if (ctx->prog_heads) cudaFreeAsync(ctx->prog_heads, s);
  ctx->prog_scratch = nullptr;
  ctx->prog_split = nullptr;
  ctx->prog_heads = nullptr;
  ctx->prog_scratch_cap = 0;
}

}  // namespace xgm
