// Triangle and k-clique counting on the degree-oriented DAG, hand-written for sm_103a.
//
// Reference kernels this replaces (same counts, different schedule):
//  - warp_edge (TC): codes/GraphMiner/src/triangle/gpu_kernels/bs_warp_edge.cuh:1-20
//  - clique4_warp_edge / clique5_warp_edge:
//      xgminer/src/gpu_kernels/glumin/gpu_GM_LUT_kernels/GM_kernels/clique{4,5}_warp_edge.cuh
//  - LUT forms clique4_warp_vertex_subgraph / clique5_warp_edge_subgraph
//      (GM_LUT_kernels/clique4_warp_vertex_subgraph.cuh:3-42,
//       clique5_warp_edge_subgraph.cuh:3-51), which build a per-warp bitmap of the
//      candidate set in global memory (BinaryEncode, binary_encode.h:8-515).
//  - persistent atomic edge queue: clique5_warp_edge_taskallocate.cuh:76-79.
//
// Scheme.  Vertices are degree ranks, so N+(v) is sorted and every member is > v.  A
// vertex task v0 takes its local set S = N+(v0) (|S| = s) and builds in shared memory
// the bitmap adjacency of the DAG induced on S: row i holds bit j iff S[j] in N+(S[i]),
// which implies j > i, so row i keeps only words floor(i/32)..W-1 (triangular layout).
// Row construction streams each N+(S[i]) once, coalesced, and looks members up in an
// open-addressing hash of S.  Then a k-clique rooted at v0 is a (k-1)-clique of the
// local DAG:
//    k = 3: number of local edges (no bitmap needed)
//    k = 4: sum_i sum_{j in row i} popc(row_i & row_j)
//    k = 5: sum_i sum_{j in row i} sum_{l in row_i & row_j} popc(row_i & row_j & row_l)
//    k = 6, 7: the same walk one or two levels deeper
// Hub vertices (s above the CTA capacity) are split into edge sub-tasks (v0, v1) whose
// local set is N+(v0) & N+(v1) and which count (k-2)-cliques of it the same way.
// One persistent kernel runs seven queues in order, each fed by an atomic head: hub
// edge sub-tasks, CTA tasks, wide-warp tasks (s <= 128), binary-search warp tasks,
// eight-lane group tasks (s <= 8, four per warp), bucket-filtered search tasks, and
// streaming warp tasks (s <= 32).
#include <atomic>
#include <cstddef>
#include <type_traits>
#include "clique.cuh"

namespace xgm {

namespace {

// ---------------------------------------------------------------- CTA shapes
// A CTA task holds its local set S in shared memory.  Layout (bytes):
//   lb[cap] i64 | S[cap + 4] i32 | pre[cap + 8] i32 | hkey[hash] i32 | hval[hash] u16 |
//   [cnt[cap] u32] | rows[tri_words(cap)] u32 | bloom[512] u32 | misc[32] i64
// cnt (per-member participation counters) exists in the participation and multi modes
// only; the count modes keep each list's length in lb's top bits instead.  A row's word
// offset is computed (tri_row_off), not stored.  (Without cnt and the offsets two
// count-mode CTAs fit the 196 KB shared-memory configuration, 60 KB of L1: measured no
// faster, the launch is issue-bound; the space went to a 4096-slot hash instead, load
// factor <= 1/4: R-MAT s22 4-clique 84.5 -> 83.1 ms.)
// S has four words of slack: a bulk copy lands a list at its own 16-byte phase.
// CtaMain is the persistent counting kernel's CTA (512 threads, 2 CTAs per SM, local
// sets of up to 1024); CtaHub is the hub kernel's (1024 threads, 1 CTA per SM, up to
// 1536: hub vertices just above the main CTA's capacity run whole instead of split).
constexpr int tri_words_c(int s) {
  return s * ((s + 31) >> 5) - (16 * (s >> 5) * ((s >> 5) - 1) + (s & 31) * (s >> 5));
}
template <int NT, int CAP, int HBITS, bool CNT = false>
struct CtaShape {
  static constexpr int kThreads = NT, kWarps = NT / 32, kCap = CAP;
  static constexpr int kHashBits = HBITS, kHash = 1 << HBITS;
  static constexpr int kBloomWords = 512;  // 16 Kbit membership pre-filter of the local set
  static constexpr int kRowsWords = tri_words_c(CAP);
  static constexpr int kOffLb = 0;
  static constexpr int kOffS = kOffLb + 8 * CAP;
  static constexpr int kOffPre = kOffS + 4 * (CAP + 4);
  static constexpr int kOffHkey = kOffPre + 4 * (CAP + 8);
  static constexpr int kOffHval = kOffHkey + 4 * kHash;
  static constexpr int kOffCnt = kOffHval + 2 * kHash;
  static constexpr int kOffRows = kOffCnt + (CNT ? 4 * CAP : 0);
  static constexpr int kOffBloom = kOffRows + 4 * kRowsWords;
  static constexpr int kOffMisc = kOffBloom + 4 * kBloomWords;
  static constexpr int kOffBar = kOffMisc + 8 * 31;  // mbarrier of the bulk copies
  static constexpr int kSmem = kOffMisc + 8 * 32;
  static_assert(2 * NT >= CAP, "the length scan gives each thread two members");
  static_assert(kHash >= 2 * CAP, "hash load factor at most one half");
  static_assert(kOffS % 16 == 0 && kOffMisc % 8 == 0 && 4 * kWarps <= 8 * 31,
                "aligned regions; warp totals below the barrier");
};
using CtaMain = CtaShape<kCtaThreads, kCtaCap, 12>;           // count modes
using CtaMainCnt = CtaShape<kCtaThreads, kCtaCap, 12, true>;  // participation / multi
using CtaHub = CtaShape<kHubThreads, kHubCap, 12>;
static_assert(CtaMain::kRowsWords == 16896, "main CTA shape");
static_assert(2 * (CtaMain::kSmem + 1024) <= 228 * 1024, "two count-mode CTAs per SM");
static_assert(CtaMain::kOffS == CtaMainCnt::kOffS && CtaMain::kOffMisc + 4096 == CtaMainCnt::kOffMisc,
              "the shapes differ only by cnt");
constexpr int kOffS = CtaMain::kOffS;
constexpr int kCtaSmem = CtaMain::kSmem;
constexpr int kCtaSmemCnt = CtaMainCnt::kSmem;
constexpr int kHubSmem = CtaHub::kSmem;
static_assert(kHubSmem <= 227 * 1024, "hub CTA fits one SM's shared memory");
constexpr int kWalkUnits = 4;   // 16-byte units per lane in flight in the CTA walk
constexpr int kWideUnits = 2;   // the same in the wide-warp walk
constexpr int kClipMin = 96;    // lists longer than this are clipped at max(S)
constexpr int kClipLoMin = 8;   // lists longer than this start at the next member of S

// First position in the sorted col[lo, hi) holding a value >= x.
__device__ __forceinline__ long long lower_pos(const int32_t* col, long long lo, long long hi,
                                               int32_t x) {
  while (lo < hi) {
    const long long mid = (lo + hi) >> 1;
    if (ldg_i32(col + mid) < x) lo = mid + 1; else hi = mid;
  }
  return lo;
}

// Wide-warp region (one warp, s <= kWideCap, 4-word rows), aliased over the CTA region
// once the CTA queues drain; the warp regions follow all wide regions so a warp in the
// last phase never overlaps a warp still in the wide phase.
constexpr int kWideBloomWords = 64;  // 2048-bit filter: ~6 % false positives at s = 128
constexpr int kWarpBloomWords = 32;  // 1024-bit filter: ~3 % false positives at s = 32

struct WideSmem {
  uint32_t bloom[kWideBloomWords];  // membership pre-filter of S
  long long lb[kWideCap];
  int32_t S[kWideCap];
  int32_t pre[kWideCap + 4];
  uint32_t rows[kWideCap * kWideWords];  // full rows, word w of row i at [i*4 + w]
  uint32_t cnt[kWideCap];
};
static_assert(offsetof(WideSmem, rows) % 16 == 0 && sizeof(WideSmem) % 16 == 0,
              "wide rows are read as uint4");
constexpr int kOffWarpRegion = kCtaWarps * (int)sizeof(WideSmem);

// Warp region: one per warp (s <= 32, one-word rows).
struct WarpSmem {
  uint32_t bloom[kWarpBloomWords];  // membership pre-filter of S
  long long lb[kWarpCap];
  int32_t S[kWarpCap];
  int32_t pre[kWarpCap + 2];
  uint32_t rows[kWarpCap];
  uint32_t cnt[kWarpCap];
};
static_assert(kOffWarpRegion + sizeof(WarpSmem) * kCtaWarps <= kCtaSmem, "warp regions fit");
static_assert(sizeof(WideSmem) % 16 == 0, "wide regions stay 16-byte aligned");
static_assert(kWarpBloomWords == 32 && kWideBloomWords == 64, "filters are cleared lane-wise");

template <class Sh = CtaMain>
__device__ __forceinline__ uint32_t hash_slot(int32_t x) {
  return ((uint32_t)x * 2654435761u) >> (32 - Sh::kHashBits);
}

// Bloom bit of x (independent of hash_slot's multiplier): 14 bits for the CTA filter,
// the top 11 / 10 of them for the wide / warp filters.
__device__ __forceinline__ uint32_t bloom_bit(int32_t x) {
  return ((uint32_t)x * 0x85EBCA6Bu) >> 18;
}

template <class Sh = CtaMain>
__device__ __forceinline__ int hash_find(const int32_t* hkey, const uint16_t* hval, int32_t x) {
  uint32_t slot = hash_slot<Sh>(x);
#pragma unroll 1
  for (int probe = 0; probe < Sh::kHash; ++probe) {
    int32_t k = hkey[slot];
    if (k == x) return hval[slot];
    if (k == -1) return -1;
    slot = (slot + 1) & (Sh::kHash - 1);
  }
  return -1;
}

// Block-wide exclusive scan of values v[i], i < n <= Sh::kCap, into pre[0..n]; CTA-wide.
template <class Sh = CtaMain>
__device__ void cta_scan_lengths(int32_t* pre, int n, int32_t* warp_tot) {
  // each thread owns items [tid*2, tid*2+1] (Sh::kCap <= 2 * Sh::kThreads)
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  int a = 2 * tid < n ? pre[2 * tid] : 0;
  int b = 2 * tid + 1 < n ? pre[2 * tid + 1] : 0;
  int s = a + b, inc = s;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    int y = __shfl_up_sync(kFull, inc, o);
    if (lane >= o) inc += y;
  }
  if (lane == 31) warp_tot[warp] = inc;
  __syncthreads();
  if (warp == 0) {
    int w = lane < Sh::kWarps ? warp_tot[lane] : 0, wi = w;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      int y = __shfl_up_sync(kFull, wi, o);
      if (lane >= o) wi += y;
    }
    if (lane < Sh::kWarps) warp_tot[lane] = wi - w;
  }
  __syncthreads();
  int ex = warp_tot[warp] + inc - s;
  if (2 * tid < n) pre[2 * tid] = ex;
  if (2 * tid + 1 < n) pre[2 * tid + 1] = ex + a;
  if (2 * tid + 1 == n - 1 || 2 * tid == n - 1) pre[n] = ex + s;
  __syncthreads();
}

// Kernel modes: plain count; triangle participation (per-vertex / per-edge triangle
// counts for the motif plans); count weighted by the out-degree of each clique's
// highest-ranked vertex (the plan's algorithmic-bytes term).
// kModeMulti (K == 4, batched graphs) counts triangles and 4-cliques of every task in
// one pass and credits triangle participation too.
enum { kModeCount = 0, kModePart = 1, kModeWeight = 2, kModeMulti = 3 };

// Count of (q)-cliques in the local DAG held by the CTA (q >= 3 uses the bitmap).  WGT
// (Q == 3 only) weights each clique by d+ of its top member, d+(S[l]) = pre[l+1]-pre[l].
// rows [0, n) are walked; W (default: from n) is the word count of the whole set.
//
// Every member j of one bitmap word lies in the same block qj = j / 32, so its row starts
// at tri_row_off(32 qj, W) + (j % 32)(W - qj): the walk takes one base pointer per word
// and reaches row j's word w with one multiply-add (no per-member offset load), and adds
// the word's popcounts in 32 bits.
template <int Q, bool WGT, class Sh = CtaMain>
__device__ __forceinline__ uint64_t cta_count_rows(const uint32_t* rows, int n, const int32_t* pre,
                                                   int W = 0) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int s = n;
  if (W == 0) W = (n + 31) >> 5;
  uint64_t acc = 0;
  for (int i = warp; i < s; i += Sh::kWarps) {
    const int qi = i >> 5, nwi = W - qi;
    const uint32_t wi = lane < nwi ? rows[tri_row_off(i, W) + lane] : 0u;
    const int w = qi + lane;
    unsigned nz = __ballot_sync(kFull, wi != 0u);
    while (nz) {
      const int src = __ffs(nz) - 1;
      nz &= nz - 1;
      uint32_t bits = __shfl_sync(kFull, wi, src);
      const int qj = qi + src;
      const bool on = lane < nwi && w >= qj;
      const uint32_t* Bj = rows + tri_row_off(qj << 5, W) + (w - qj);  // + b (W - qj)
      const int sj = W - qj;
      if constexpr (Q == 3 && !WGT) {
        uint32_t part = 0;
        while (bits) {  // four members per pass: independent load / AND / popc chains
          int b[4];
          bool h[4];
#pragma unroll
          for (int u = 0; u < 4; ++u) {
            h[u] = bits != 0u;
            b[u] = h[u] ? __ffs(bits) - 1 : 0;
            bits &= bits - 1;
          }
          if (on) {
            uint32_t x[4];
#pragma unroll
            for (int u = 0; u < 4; ++u) x[u] = Bj[b[u] * sj];
#pragma unroll
            for (int u = 0; u < 4; ++u) part += h[u] ? __popc(wi & x[u]) : 0u;
          }
        }
        acc += part;
      } else if constexpr (Q == 3) {
        while (bits) {
          const int b = __ffs(bits) - 1;
          bits &= bits - 1;
          uint32_t b3 = on ? (wi & Bj[b * sj]) : 0u;
          while (b3) {
            const int l = (w << 5) + __ffs(b3) - 1;
            b3 &= b3 - 1;
            acc += (uint64_t)(pre[l + 1] - pre[l]);
          }
        }
      } else {
        // Q == 4: m = R_i & R_j, lane w holding word w; each member l of m is a lane of
        // its own: for every nonzero word ql of m, lane b takes l = 32 ql + b when bit b
        // is set, and adds popc(m & R_l) over the nonzero words of m from ql on (m's bits
        // cluster in a few words: at R-MAT scale 19, 36 members in 2.8 words per pair)
        while (bits) {
          const int b = __ffs(bits) - 1;
          bits &= bits - 1;
          const uint32_t m = on ? (wi & Bj[b * sj]) : 0u;
          unsigned nz2 = __ballot_sync(kFull, m != 0u);
          uint32_t part = 0;
          while (nz2) {
            const int src2 = __ffs(nz2) - 1;
            const uint32_t bq = __shfl_sync(kFull, m, src2);
            const int ql = qi + src2;
            const bool act = (bq >> lane) & 1u;
            // row l = 32 ql + lane, its word w2 at Rl[w2 - qi]
            const uint32_t* Rl = rows + tri_row_off(ql << 5, W) + lane * (W - ql) + (qi - ql);
            unsigned rest = nz2;
            nz2 &= nz2 - 1;
            while (rest) {
              const int s3 = __ffs(rest) - 1;
              rest &= rest - 1;
              const uint32_t mw = __shfl_sync(kFull, m, s3);
              if (act) part += __popc(mw & Rl[s3]);
            }
          }
          acc += part;
        }
      }
    }
  }
  return acc;
}

// Rows [row_lo, row_hi) of the local DAG whose rows span at most G words, G lanes per
// row (32 / G rows per warp): lane sub of a group holds word qi + sub of its row, every
// ballot / shuffle stays inside the group, and the loops run while any group of the
// warp has work (__any_sync), so all 32 lanes meet at every warp-synchronous call.
// Row offsets of the members of one word come from one base pointer, as in
// cta_count_rows.
template <int Q, int G, class Sh = CtaMain>
__device__ uint64_t count_rows_grouped(const uint32_t* rows, int W, int row_lo, int row_hi) {
  static_assert(Q == 3 || Q == 4, "grouped rows cover the 4- and 5-clique count phases");
  constexpr unsigned kGMask = G == 32 ? 0xffffffffu : ((1u << G) - 1u);
  constexpr int kGroups = 32 / G;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int sub = lane % G, gbase = lane - sub;
  uint64_t acc = 0;
  for (int i0 = row_lo + warp * kGroups; i0 < row_hi; i0 += Sh::kWarps * kGroups) {
    const int i = i0 + lane / G;
    const bool live = i < row_hi;
    const int qi = live ? (i >> 5) : 0, nwi = W - qi;
    const uint32_t wi = (live && sub < nwi) ? rows[tri_row_off(i, W) + sub] : 0u;
    const int w = qi + sub;
    unsigned nz = (__ballot_sync(kFull, wi != 0u) >> gbase) & kGMask;
    while (__any_sync(kFull, nz != 0u)) {
      const bool had = nz != 0u;
      const int src = had ? __ffs(nz) - 1 : 0;
      if (had) nz &= nz - 1;
      uint32_t bits = __shfl_sync(kFull, wi, gbase + src);
      if (!had) bits = 0u;
      const int qj = qi + src;
      const bool on = sub < nwi && w >= qj;
      const uint32_t* Bj = rows + tri_row_off(qj << 5, W) + (w - qj);
      const int sj = W - qj;
      uint32_t part = 0;
      if constexpr (Q == 3) {
        while (__any_sync(kFull, bits != 0u)) {  // four members per pass
          int b[4];
          bool h[4];
#pragma unroll
          for (int u = 0; u < 4; ++u) {
            h[u] = bits != 0u;
            b[u] = h[u] ? __ffs(bits) - 1 : 0;
            bits &= bits - 1;
          }
          if (h[0] && on) {
            uint32_t x[4];
#pragma unroll
            for (int u = 0; u < 4; ++u) x[u] = Bj[b[u] * sj];
#pragma unroll
            for (int u = 0; u < 4; ++u) part += h[u] ? __popc(wi & x[u]) : 0u;
          }
        }
        acc += part;
        continue;
      }
      while (__any_sync(kFull, bits != 0u)) {
        const bool hb = bits != 0u;
        const int b = hb ? __ffs(bits) - 1 : 0;
        if (hb) bits &= bits - 1;
        const uint32_t m = (hb && on) ? (wi & Bj[b * sj]) : 0u;
        if (Q == 3) {
          part += __popc(m);
        } else {
          unsigned nz2 = (__ballot_sync(kFull, m != 0u) >> gbase) & kGMask;
          while (__any_sync(kFull, nz2 != 0u)) {
            const bool had2 = nz2 != 0u;
            const int src2 = had2 ? __ffs(nz2) - 1 : 0;
            if (had2) nz2 &= nz2 - 1;
            uint32_t bits2 = __shfl_sync(kFull, m, gbase + src2);
            if (!had2) bits2 = 0u;
            const int ql = qi + src2;
            const bool on2 = m != 0u && w >= ql;
            const uint32_t* Bl = rows + tri_row_off(ql << 5, W) + (w - ql);
            const int sl = W - ql;
            while (__any_sync(kFull, bits2 != 0u)) {  // four members per pass
              int b[4];
              bool h[4];
#pragma unroll
              for (int u = 0; u < 4; ++u) {
                h[u] = bits2 != 0u;
                b[u] = h[u] ? __ffs(bits2) - 1 : 0;
                bits2 &= bits2 - 1;
              }
              if (h[0] && on2) {
                uint32_t x[4];
#pragma unroll
                for (int u = 0; u < 4; ++u) x[u] = Bl[b[u] * sl];
#pragma unroll
                for (int u = 0; u < 4; ++u) part += h[u] ? __popc(m & x[u]) : 0u;
              }
            }
          }
        }
      }
      acc += part;
    }
  }
  return acc;
}

// cta_count_rows (unweighted, Q = 3 or 4) for rows spanning up to 64 words (local sets
// above 1024, the hub CTA): lane holds words qi + lane and qi + lane + 32 of row i, and
// each enumeration runs over the two halves in turn.
template <int Q, class Sh>
__device__ uint64_t cta_count_rows2(const uint32_t* rows, int nrows, int W) {
  static_assert(Q == 3 || Q == 4, "two-word rows cover the 4- and 5-clique count phases");
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  uint64_t acc = 0;
  for (int i = warp; i < nrows; i += Sh::kWarps) {
    const int qi = i >> 5, nwi = W - qi;
    const int ri = tri_row_off(i, W);
    const uint32_t wa = lane < nwi ? rows[ri + lane] : 0u;
    const uint32_t wb = lane + 32 < nwi ? rows[ri + lane + 32] : 0u;
    const int wA = qi + lane, wB = wA + 32;
#pragma unroll 1
    for (int half = 0; half < 2; ++half) {
      unsigned nz = __ballot_sync(kFull, (half ? wb : wa) != 0u);
      while (nz) {
        const int src = __ffs(nz) - 1;
        nz &= nz - 1;
        uint32_t bits = __shfl_sync(kFull, half ? wb : wa, src);
        const int qj = qi + src + 32 * half;
        const bool onA = lane < nwi && wA >= qj, onB = lane + 32 < nwi && wB >= qj;
        const uint32_t* Bj = rows + tri_row_off(qj << 5, W);  // + b (W - qj) + (w - qj)
        const int sj = W - qj;
        while (bits) {
          const int b = __ffs(bits) - 1;
          bits &= bits - 1;
          const uint32_t ma = onA ? (wa & Bj[b * sj + (wA - qj)]) : 0u;
          const uint32_t mb = onB ? (wb & Bj[b * sj + (wB - qj)]) : 0u;
          if constexpr (Q == 3) {
            acc += (uint32_t)(__popc(ma) + __popc(mb));
          } else {
            uint32_t part = 0;
#pragma unroll 1
            for (int h2 = 0; h2 < 2; ++h2) {
              unsigned nz2 = __ballot_sync(kFull, (h2 ? mb : ma) != 0u);
              while (nz2) {
                const int src2 = __ffs(nz2) - 1;
                nz2 &= nz2 - 1;
                uint32_t bits2 = __shfl_sync(kFull, h2 ? mb : ma, src2);
                const int ql = qi + src2 + 32 * h2;
                const bool onA2 = ma != 0u && wA >= ql, onB2 = mb != 0u && wB >= ql;
                const uint32_t* Bl = rows + tri_row_off(ql << 5, W);
                const int sl = W - ql;
                while (bits2) {
                  const int b2 = __ffs(bits2) - 1;
                  bits2 &= bits2 - 1;
                  if (onA2) part += __popc(ma & Bl[b2 * sl + (wA - ql)]);
                  if (onB2) part += __popc(mb & Bl[b2 * sl + (wB - ql)]);
                }
              }
            }
            acc += part;
          }
        }
      }
    }
  }
  return acc;
}

// The 4- and 5-clique count phases (unweighted) with the rows split into tiers by how
// many words they span (row i spans W - floor(i/32)): rows spanning more than 16 words
// keep the full-warp walk of cta_count_rows, the others run 2, 4 or 8 to a warp
// (count_rows_grouped) so no lane idles on words past its row's end.
template <int Q, class Sh = CtaMain>
__device__ uint64_t cta_count_rows_tiered(const uint32_t* rows, int s, const int32_t* pre) {
  const int W = (s + 31) >> 5;
  // first row spanning at most t words: 32 * (W - t), clamped to [0, s]
  auto first = [&](int t) { const int r = 32 * (W - t); return r < 0 ? 0 : (r > s ? s : r); };
  const int r16 = first(16), r8 = first(8), r4 = first(4);
  uint64_t acc = 0;
  if constexpr (Q == 4 && Sh::kCap <= 1024) {
    // the 5-clique count runs lane per member of m (cta_count_rows): no word tiers
    return cta_count_rows<4, false, Sh>(rows, s, pre, W);
  }
  if constexpr (Sh::kCap > 1024) {  // rows may span more than 32 words
    if (r16 > 0) acc += cta_count_rows2<Q, Sh>(rows, r16, W);
  } else {
    if (r16 > 0) acc += cta_count_rows<Q, false, Sh>(rows, r16, pre, W);
  }
  acc += count_rows_grouped<Q, 16, Sh>(rows, W, r16, r8);
  acc += count_rows_grouped<Q, 8, Sh>(rows, W, r8, r4);
  acc += count_rows_grouped<Q, 4, Sh>(rows, W, r4, s);
  return acc;
}

// D-cliques of the local DAG inside a candidate set, for the 6- and 7-clique plans
// (local clique depth 5 and 6).  The set is warp-distributed: this lane holds word w;
// every candidate l > i, so the walk of cta_count_rows carries over level by level:
// the next level's set is this level's set & R_l.
template <int D>
__device__ uint64_t rows_deep(const uint32_t* rows, int W, uint32_t m, int w, int qi) {
  if constexpr (D == 1) {
    return (uint64_t)__popc(m);
  } else {
    uint64_t acc = 0;
    unsigned nz = __ballot_sync(kFull, m != 0u);
    while (nz) {
      const int src = __ffs(nz) - 1;
      nz &= nz - 1;
      uint32_t bits = __shfl_sync(kFull, m, src);
      const int ql = qi + src;  // block of every l of this word: row l = base + b (W - ql)
      const bool on = m != 0u && w >= ql;
      const uint32_t* Bl = rows + tri_row_off(ql << 5, W) + (w - ql);
      const int sl = W - ql;
      while (bits) {
        const int b = __ffs(bits) - 1;
        bits &= bits - 1;
        const uint32_t m2 = on ? (m & Bl[b * sl]) : 0u;
        acc += rows_deep<D - 1>(rows, W, m2, w, qi);
      }
    }
    return acc;
  }
}

// rows_deep with G lanes per candidate set (32 / G sets per warp, one per group): group
// ballots and shuffles, loops while any group has work.
template <int D, int G>
__device__ uint64_t rows_deep_grouped(const uint32_t* rows, int W, uint32_t m, int w, int qi,
                                      int gbase) {
  if constexpr (D == 1) {
    return (uint64_t)__popc(m);
  } else {
    constexpr unsigned kGMask = (1u << G) - 1u;
    uint64_t acc = 0;
    unsigned nz = (__ballot_sync(kFull, m != 0u) >> gbase) & kGMask;
    while (__any_sync(kFull, nz != 0u)) {
      const bool had = nz != 0u;
      const int src = had ? __ffs(nz) - 1 : 0;
      if (had) nz &= nz - 1;
      uint32_t bits = __shfl_sync(kFull, m, gbase + src);
      if (!had) bits = 0u;
      const int ql = qi + src;
      const bool on = m != 0u && w >= ql;
      const uint32_t* Bl = rows + tri_row_off(ql << 5, W) + (w - ql);
      const int sl = W - ql;
      while (__any_sync(kFull, bits != 0u)) {
        const bool hb = bits != 0u;
        const int b = hb ? __ffs(bits) - 1 : 0;
        if (hb) bits &= bits - 1;
        const uint32_t m2 = (hb && on) ? (m & Bl[b * sl]) : 0u;
        acc += rows_deep_grouped<D - 1, G>(rows, W, m2, w, qi, gbase);
      }
    }
    return acc;
  }
}

template <int Q, int G, class Sh = CtaMain>
__device__ uint64_t count_deep_grouped(const uint32_t* rows, int W, int row_lo, int row_hi) {
  constexpr int kGroups = 32 / G;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int sub = lane % G, gbase = lane - sub;
  uint64_t acc = 0;
  for (int i0 = row_lo + warp * kGroups; i0 < row_hi; i0 += Sh::kWarps * kGroups) {
    const int i = i0 + lane / G;
    const bool live = i < row_hi;
    const int qi = live ? (i >> 5) : 0, nwi = W - qi;
    const uint32_t wi = (live && sub < nwi) ? rows[tri_row_off(i, W) + sub] : 0u;
    acc += rows_deep_grouped<Q - 1, G>(rows, W, wi, qi + sub, qi, gbase);
  }
  return acc;
}

// Q-cliques for Q >= 5, rows tiered by the words they span as in cta_count_rows_tiered.
template <int Q, class Sh = CtaMain>
__device__ uint64_t cta_count_deep(const uint32_t* rows, int s) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int W = (s + 31) >> 5;
  auto first = [&](int t) { const int r = 32 * (W - t); return r < 0 ? 0 : (r > s ? s : r); };
  const int r16 = first(16), r8 = first(8), r4 = first(4);
  uint64_t acc = 0;
  for (int i = warp; i < r16; i += Sh::kWarps) {
    const int qi = i >> 5, nwi = W - qi;
    const uint32_t wi = lane < nwi ? rows[tri_row_off(i, W) + lane] : 0u;
    acc += rows_deep<Q - 1>(rows, W, wi, qi + lane, qi);
  }
  acc += count_deep_grouped<Q, 16, Sh>(rows, W, r16, r8);
  acc += count_deep_grouped<Q, 8, Sh>(rows, W, r8, r4);
  acc += count_deep_grouped<Q, 4, Sh>(rows, W, r4, s);
  return acc;
}

// The same for one-word rows (local sets of up to 32, one lane per row).
template <int D>
__device__ uint64_t word_deep(const uint32_t* rows, uint32_t m) {
  if constexpr (D == 1) {
    return (uint64_t)__popc(m);
  } else {
    uint64_t acc = 0;
    while (m) {
      const int l = __ffs(m) - 1;
      m &= m - 1;
      acc += word_deep<D - 1>(rows, m & rows[l]);
    }
    return acc;
  }
}

// And for the wide tier's 4-word rows (row l at rows + l * 4; one lane per row).
template <int D>
__device__ uint64_t wide_deep(const uint32_t* rows, const uint32_t (&m)[4]) {
  if constexpr (D == 1) {
    return (uint64_t)(__popc(m[0]) + __popc(m[1]) + __popc(m[2]) + __popc(m[3]));
  } else {
    uint64_t acc = 0;
#pragma unroll 1
    for (int x = 0; x < 4; ++x) {
      uint32_t bits = m[x];
      while (bits) {
        const int l = (x << 5) + __ffs(bits) - 1;
        bits &= bits - 1;
        const uint32_t* Rl = rows + l * 4;
        uint32_t m2[4];
#pragma unroll
        for (int y = 0; y < 4; ++y) m2[y] = y >= x ? (m[y] & Rl[y]) : 0u;
        acc += wide_deep<D - 1>(rows, m2);
      }
    }
    return acc;
  }
}

// Participation counters of the triangle-participation mode.
struct Part {
  unsigned long long* v;  // per vertex (rank ids)
  unsigned* e;            // per rank-space col entry
};

// The CTA has S[0..s) (sorted, local set) in shared memory.  Counts the Q-cliques of the
// DAG induced on S, Q = 1..6.  PART (Q == 2 only, S = N+(root) starting at col entry
// sbase): every local edge (i, j) is the triangle (root, S[i], S[j]); it is credited to
// vertices S[i], S[j] and edges (root,S[i]), (root,S[j]), (S[i],S[j]).  The root's own
// credit is the returned count.  span_ok = false keeps the Bloom filter + hash membership
// test even where the span bitmap fits (XGM_SCHED_HASH_ONLY).
template <int Q, int MODE, class Sh = CtaMain>
__device__ uint64_t cta_local(const GView& g, char* sm, int s, Part part, long long sbase,
                              uint64_t* q2out = nullptr, int s_off = 0, bool span_ok = true) {
  constexpr bool MULTI = MODE == kModeMulti;  // Q == 3: also local edges + participation
  constexpr bool PART = MODE == kModePart || MULTI;
  constexpr bool WGT = MODE == kModeWeight;
  // 128-bit loads of the lists (all but the weighted mode, whose weights are the lists'
  // element counts in pre[])
  constexpr bool kVec = !WGT;
  int32_t* S = (int32_t*)(sm + Sh::kOffS) + s_off;
  if (Q == 1) {
    if (!WGT) return (uint64_t)s;  // same value in every thread
    uint64_t a = 0;                // per-thread partial sums
    for (int i = threadIdx.x; i < s; i += Sh::kThreads) {
      const longlong2 d = ldg_ll2(g.dptr + S[i]);
      a += (uint64_t)(d.y - d.x);
    }
    return a;
  }
  long long* lb = (long long*)(sm + Sh::kOffLb);
  int32_t* pre = (int32_t*)(sm + Sh::kOffPre);
  int32_t* hkey = (int32_t*)(sm + Sh::kOffHkey);
  uint16_t* hval = (uint16_t*)(sm + Sh::kOffHval);
  uint32_t* cnt = (uint32_t*)(sm + Sh::kOffCnt);  // participation / multi shapes only
  static_assert(!PART || Sh::kOffRows > Sh::kOffCnt, "participation needs the cnt region");
  uint32_t* rows = (uint32_t*)(sm + Sh::kOffRows);
  int32_t* wtot = (int32_t*)(sm + Sh::kOffMisc);
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int W = (s + 31) >> 5;

  uint32_t* bloom = (uint32_t*)(sm + Sh::kOffBloom);
  // Dense span: S is sorted, so when max(S) - S[0] < 32 * kHash (R-MAT's CTA tasks: their
  // members are the top-ranked vertices) membership is a bitmap over [S[0], max(S)] in
  // the hash-key region and a member's index is the per-word prefix (in the hash-value
  // region) plus a popcount: no Bloom filter, no probes.  Else the hash table.
  const int32_t sb0 = S[0];
  const uint32_t span = (uint32_t)(S[s - 1] - sb0) + 1u;
  const bool dense = span_ok && span <= 32u * (uint32_t)Sh::kHash;  // same in every thread
  uint32_t* bm = (uint32_t*)hkey;
  uint16_t* bpre = hval;
  if (dense) {
    for (int h = tid; h < (int)((span + 31) >> 5); h += Sh::kThreads) bm[h] = 0u;
  } else {
    for (int h = tid; h < Sh::kHash; h += Sh::kThreads) hkey[h] = -1;
    for (int h = tid; h < Sh::kBloomWords; h += Sh::kThreads) bloom[h] = 0u;
  }
  if (Q >= 3)
    for (int x = tid; x < tri_words(s); x += Sh::kThreads) rows[x] = 0u;
  if (PART)
    for (int i = tid; i < s; i += Sh::kThreads) cnt[i] = 0u;
  // Row i's list is streamed whole: only members S[i+1] .. max(S) can hit, but clipping
  // it to that range (two binary searches in the global row) removes 1.2 % of the CTA
  // tasks' 16.8 G elements at R-MAT scale 22 and cost more in the setup than it saved
  // (4-clique 73.2 -> 69.1 ms without it); the membership test rejects the rest.  The
  // last member has no later member to hit (not in weighted mode: its weights are the
  // full out-degrees pre[j+1] - pre[j]).
  for (int i = tid; i < s; i += Sh::kThreads) {
    const longlong2 d = ldg_ll2(g.dptr + S[i]);
    long long lo = d.x;
    const long long hi = d.y;
    if (!WGT && i + 1 == s) lo = hi;
    if constexpr (kVec) {  // 16-byte units from the aligned start
      // lb = aligned start (bits 0-39) | phase (40-41) | length (42-63): graphs hold
      // fewer than 2^40 entries and a degree-oriented out-list fewer than sqrt(2E) < 2^21
      const long long a = lo & ~3ll;
      lb[i] = a | ((lo - a) << 40) | ((hi - lo) << 42);
      pre[i] = hi > lo ? (int32_t)((hi - a + 3) >> 2) : 0;
    } else {
      lb[i] = lo;
      pre[i] = (int32_t)(hi - lo);
    }
  }
  __syncthreads();
  for (int i = tid; i < s; i += Sh::kThreads) {
    const int32_t x = S[i];
    if (dense) {
      // bit of x, and bpre[w] = members in words below w for the words since the
      // previous member's (the last member's word is the last one queried)
      const uint32_t off = (uint32_t)(x - sb0);
      atomicOr(&bm[off >> 5], 1u << (off & 31));
      const int w0 = i == 0 ? 0 : (int)(((uint32_t)(S[i - 1] - sb0) >> 5) + 1);
      for (int w = w0; w <= (int)(off >> 5); ++w) bpre[w] = (uint16_t)i;
      continue;
    }
    uint32_t slot = hash_slot<Sh>(x);
    // s <= Sh::kCap < Sh::kHash members: an empty slot always exists
    for (int probe = 0; probe < Sh::kHash && atomicCAS(&hkey[slot], -1, x) != -1; ++probe)
      slot = (slot + 1) & (Sh::kHash - 1);
    hval[slot] = (uint16_t)i;
    const uint32_t b = bloom_bit(x);
    atomicOr(&bloom[b >> 5], 1u << (b & 31));
  }
  cta_scan_lengths<Sh>(pre, s, wtot);  // ends with __syncthreads
  const int total = pre[s];
  const int32_t smax = S[s - 1];
  uint64_t acc = 0, q2 = 0;
  // All but the weighted mode: flattened walk over 16-byte units of the rows' lists
  // (pre[] counts units; lb[i] = the list's aligned start | its phase | its length):
  // warp chunks of 32 kWalkUnits units, one 128-bit load per lane and unit, all loads of
  // a lane in flight before use (kWalkUnits 2 -> 4: s22 4-clique 69.1 -> 67.3 ms).
  // Elements of a unit outside the list (the other rows' entries next to it) are masked
  // by position.  Then the membership test as below.
  if constexpr (kVec) {
    // the membership test is chosen once per task (DENSE: span bitmap, else Bloom + hash)
    auto walk = [&](auto dense_c) {
      constexpr bool DENSE = decltype(dense_c)::value;
      constexpr int kNU = kWalkUnits, kChunk = 32 * kNU;
      for (int c = warp; c * kChunk < total; c += Sh::kWarps) {
        const int kb = c * kChunk + lane;
        int i;
        {  // segment of the chunk start, as in the scalar walk below
          constexpr int kR1 = Sh::kCap <= 1024 ? 32 : 64;
          constexpr int kR2 = kR1 / 32;
          const int k0 = c * kChunk;
          const int c1 = lane * kR1;
          const unsigned b1 = __ballot_sync(kFull, c1 < s && pre[c1] <= k0);
          const int r1 = 31 - __clz(b1);
          const int c2 = r1 * kR1 + lane * kR2;
          const unsigned b2 = __ballot_sync(kFull, c2 < s && pre[c2] <= k0);
          i = r1 * kR1 + (31 - __clz(b2)) * kR2;
          while (i + 1 < s && pre[i + 1] <= kb) ++i;
        }
        int4 v[kNU];
        int iv[kNU], rel[kNU], len[kNU];
        long long pb[kNU];  // participation: col position of the unit's first word
#pragma unroll
        for (int h = 0; h < kNU; ++h) {
          const int k = kb + 32 * h;
          iv[h] = i;
          rel[h] = 0;
          len[h] = 0;
          pb[h] = 0;
          v[h] = make_int4(0, 0, 0, 0);
          if (k < total) {
            while (k >= pre[i + 1]) ++i;
            const unsigned long long L = (unsigned long long)lb[i];
            const int u = k - pre[i];
            iv[h] = i;
            rel[h] = 4 * u - (int)((L >> 40) & 3);  // element index of the unit's first word
            len[h] = (int)(L >> 42);
            pb[h] = (long long)(L & ((1ull << 40) - 1)) + 4 * u;
            v[h] = __ldg((const int4*)(g.col + (long long)(L & ((1ull << 40) - 1))) + u);
          }
        }
#pragma unroll
        for (int h = 0; h < kNU; ++h) {
          const int32_t xs4[4] = {v[h].x, v[h].y, v[h].z, v[h].w};
#pragma unroll
          for (int t = 0; t < 4; ++t) {
            const int e = rel[h] + t;
            const int32_t x = xs4[t];
            if ((unsigned)e >= (unsigned)len[h]) continue;
            int j;
            if constexpr (DENSE) {
              const uint32_t off = (uint32_t)(x - sb0);
              if (off >= span) continue;
              const uint32_t wv = bm[off >> 5], bit = 1u << (off & 31);
              if (!(wv & bit)) continue;
              j = bpre[off >> 5] + __popc(wv & (bit - 1u));
            } else {
              if (x > smax) continue;
              const uint32_t b = bloom_bit(x);
              if (!((bloom[b >> 5] >> (b & 31)) & 1u)) continue;
              j = hash_find<Sh>(hkey, hval, x);
              if (j < 0) continue;
            }
            const int ii = iv[h];
            if (Q == 2) {
              acc += 1;
            } else {
              atomicOr(&rows[tri_row_off(ii, W) + (j >> 5) - (ii >> 5)], 1u << (j & 31));
              if (MULTI) q2 += 1;
            }
            if (PART) {
              atomicAdd(&cnt[ii], 1u);
              atomicAdd(&cnt[j], 1u);
              atomicAdd(&part.e[pb[h] + t], 1u);
            }
          }
        }
      }
    };
    if (dense) walk(std::true_type{});
    else walk(std::false_type{});
  } else {
    // Flattened walk over all (i, element) pairs: warp chunks of 256 consecutive
    // elements, lanes contiguous within a chunk so row reads are coalesced.  Each lane
    // keeps its segment's base in registers, issues four loads before using them, and
    // rejects most non-members with one membership probe (span bitmap, or Bloom filter
    // before the hash lookup).
    auto walk = [&](auto dense_c) {
      constexpr bool DENSE = decltype(dense_c)::value;
      for (int c = warp; c * 256 < total; c += Sh::kWarps) {
        const int kb = c * 256 + lane;
        int i;
        {  // segment of the chunk start (largest i < s with pre[i] <= c * 256): a two-round
           // 32-way search by the warp (strides kR1 then kR1 / 32), then each lane steps to
           // its own segment
          constexpr int kR1 = Sh::kCap <= 1024 ? 32 : 64;
          static_assert(32 * kR1 >= Sh::kCap, "two search rounds cover the local set");
          constexpr int kR2 = kR1 / 32;
          const int k0 = c * 256;
          const int c1 = lane * kR1;
          const unsigned b1 = __ballot_sync(kFull, c1 < s && pre[c1] <= k0);
          const int r1 = 31 - __clz(b1);  // b1 has bit 0: pre[0] = 0 <= k0
          const int c2 = r1 * kR1 + lane * kR2;
          const unsigned b2 = __ballot_sync(kFull, c2 < s && pre[c2] <= k0);
          i = r1 * kR1 + (31 - __clz(b2)) * kR2;
          while (i + 1 < s && pre[i + 1] <= kb) ++i;  // stays below s past the end
        }
        int seg_end = pre[i + 1];
        long long seg_base = lb[i] - pre[i];
#pragma unroll
        for (int h = 0; h < 2; ++h) {
          int32_t xv[4];
          int iv[4];
          long long pv[4];
#pragma unroll
          for (int t = 0; t < 4; ++t) {
            const int k = kb + 32 * (4 * h + t);
            xv[t] = 0x7FFFFFFF;  // above every id: rejected below
            iv[t] = i;
            pv[t] = 0;
            if (k < total) {
              while (k >= seg_end) {
                ++i;
                seg_end = pre[i + 1];
                seg_base = lb[i] - pre[i];
              }
              pv[t] = seg_base + k;
              iv[t] = i;
              xv[t] = ldg_i32(g.col + pv[t]);
            }
          }
#pragma unroll
          for (int t = 0; t < 4; ++t) {
            const int32_t x = xv[t];
            int j;
            if constexpr (DENSE) {
              const uint32_t off = (uint32_t)(x - sb0);
              if (off >= span) continue;
              const uint32_t wv = bm[off >> 5], bit = 1u << (off & 31);
              if (!(wv & bit)) continue;
              j = bpre[off >> 5] + __popc(wv & (bit - 1u));
            } else {
              if (x > smax) continue;
              const uint32_t b = bloom_bit(x);
              if (!((bloom[b >> 5] >> (b & 31)) & 1u)) continue;
              j = hash_find<Sh>(hkey, hval, x);
              if (j < 0) continue;
            }
            const int ii = iv[t];
            if (Q == 2) {
              acc += WGT ? (uint64_t)(pre[j + 1] - pre[j]) : 1;
              if (PART) {
                atomicAdd(&cnt[ii], 1u);
                atomicAdd(&cnt[j], 1u);
                atomicAdd(&part.e[pv[t]], 1u);
              }
            } else {
              atomicOr(&rows[tri_row_off(ii, W) + (j >> 5) - (ii >> 5)], 1u << (j & 31));
              if (MULTI) {
                q2 += 1;
                atomicAdd(&cnt[ii], 1u);
                atomicAdd(&cnt[j], 1u);
                atomicAdd(&part.e[pv[t]], 1u);
              }
            }
          }
        }
      }
    };
    if (dense) walk(std::true_type{});
    else walk(std::false_type{});
  }
  if (MULTI) *q2out = q2;
  __syncthreads();
  if (PART) {
    for (int i = tid; i < s; i += Sh::kThreads)
      if (cnt[i]) {
        atomicAdd(&part.v[S[i]], (unsigned long long)cnt[i]);
        atomicAdd(&part.e[sbase + i], cnt[i]);
      }
  }
  if (Q == 3) acc = WGT ? cta_count_rows<3, true, Sh>(rows, s, pre)
                        : cta_count_rows_tiered<3, Sh>(rows, s, pre);
  if (Q == 4) acc = cta_count_rows_tiered<4, Sh>(rows, s, pre);
  if constexpr (Q >= 5) acc = cta_count_deep<Q, Sh>(rows, s);
  return acc;
}

// CTA-wide ordered intersection N+(v0) & N+(v1) into S; returns its size or -1 when it
// exceeds kCtaCap.  Members of N+(v1) are binary-searched in N+(v0) (global, sorted).
// PART credits the triangles (v0, v1, w): edges (v1, w) and (v0, w) and vertex w.
// Without STORE only the size is produced (no capacity limit); WSUM adds d+(w) of every
// member to *wsum (per thread).
template <bool PART, bool STORE, bool WSUM = false, class Sh = CtaMain>
__device__ int cta_intersect_into_S(const GView& g, char* sm, int32_t v0, int32_t v1, Part part,
                                    uint64_t* wsum = nullptr) {
  int32_t* S = (int32_t*)(sm + kOffS);
  int32_t* wtot = (int32_t*)(sm + Sh::kOffMisc);
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const longlong2 a = ldg_ll2(g.dptr + v0), b = ldg_ll2(g.dptr + v1);
  int n = 0;
  for (long long base = b.x; base < b.y; base += kCtaThreads) {
    const long long e = base + tid;
    bool found = false;
    int32_t y = 0;
    if (e < b.y) {
      y = ldg_i32(g.col + e);
      long long lo = a.x, hi = a.y;
      while (lo < hi) {
        long long mid = (lo + hi) >> 1;
        if (ldg_i32(g.col + mid) < y) lo = mid + 1; else hi = mid;
      }
      found = lo < a.y && ldg_i32(g.col + lo) == y;
      if (PART && found) {
        atomicAdd(&part.e[e], 1u);
        atomicAdd(&part.e[lo], 1u);
        atomicAdd(&part.v[y], 1ull);
      }
      if (WSUM && found) {
        const longlong2 dy = ldg_ll2(g.dptr + y);
        *wsum += (uint64_t)(dy.y - dy.x);
      }
    }
    const unsigned bal = __ballot_sync(kFull, found);
    if (lane == 0) wtot[warp] = __popc(bal);
    __syncthreads();
    int off = n;
    for (int w = 0; w < warp; ++w) off += wtot[w];
    int tot = 0;
    for (int w = 0; w < kCtaWarps; ++w) tot += wtot[w];
    const int pos = off + __popc(bal & lanemask_lt());
    if (STORE && found && pos < kCtaCap) S[pos] = y;
    n += tot;
    __syncthreads();
  }
  return (!STORE || n <= kCtaCap) ? n : -1;
}

// --------------------------------------------------------------- warp tier
__device__ __forceinline__ int warp_bsearch(const int32_t* S, int s, int32_t x) {
  int lo = 0, hi = s;
  while (lo < hi) {
    int mid = (lo + hi) >> 1;
    if (S[mid] < x) lo = mid + 1; else hi = mid;
  }
  return (lo < s && S[lo] == x) ? lo : -1;
}

// One warp, local set S = N+(v0) with s <= 32: Q-cliques of the local DAG.
template <int Q, int MODE>
__device__ uint64_t warp_vertex_task(const GView& g, WarpSmem& w, int32_t v0, Part part,
                                     uint64_t* q2out = nullptr) {
  static_assert(Q >= 2, "warp tasks count at least local edges");
  constexpr bool MULTI = MODE == kModeMulti;
  constexpr bool PART = MODE == kModePart || MULTI;
  constexpr bool WGT = MODE == kModeWeight;
  const int lane = threadIdx.x & 31;
  const longlong2 d0 = ldg_ll2(g.dptr + v0);
  const int s = (int)(d0.y - d0.x);
  int len = 0;
  int32_t xs = 0;
  longlong2 dx = make_longlong2(0, 0);
  if (lane < s) {
    xs = ldg_i32(g.col + d0.x + lane);
    w.S[lane] = xs;
    dx = ldg_ll2(g.dptr + xs);
    w.lb[lane] = dx.x;
    len = (int)(dx.y - dx.x);
  }
  const int32_t smax = __shfl_sync(kFull, xs, s - 1);
  const int32_t next = __shfl_down_sync(kFull, xs, 1);
  // clip row lane to [S[lane+1], max(S)] (other members cannot hit; the CTA tier streams
  // whole lists, whose clipping cost more than it saved there)
  if (!WGT && lane < s) {
    long long lo = dx.x, hi = dx.y;
    if (lane + 1 == s) lo = hi;
    else if (hi - lo > kClipLoMin) lo = lower_pos(g.col, lo, hi, next);
    if (hi - lo > kClipMin && ldg_i32(g.col + hi - 1) > smax) hi = lower_pos(g.col, lo, hi, smax + 1);
    w.lb[lane] = lo;
    len = (int)(hi - lo);
  }
  int inc = len;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    int y = __shfl_up_sync(kFull, inc, o);
    if (lane >= o) inc += y;
  }
  w.pre[lane] = inc - len;
  if (lane == 31) w.pre[32] = inc;
  w.rows[lane] = 0u;
  w.cnt[lane] = 0u;
  w.bloom[lane] = 0u;  // kWarpBloomWords == 32
  __syncwarp();
  if (lane < s) {
    const uint32_t b = bloom_bit(xs) >> 4;  // 10 bits
    atomicOr(&w.bloom[b >> 5], 1u << (b & 31));
  }
  __syncwarp();  // pre[s] is the total: lanes >= s contributed length 0
  const int total = w.pre[s];
  uint64_t acc = 0, q2 = 0;
  int i = 0;
  int seg_end = w.pre[1];
  long long seg_base = w.lb[0];
  for (int kb = lane; kb < total; kb += 128) {
    int32_t xv[4];
    int iv[4];
    long long pv[4];
#pragma unroll
    for (int t = 0; t < 4; ++t) {
      const int k = kb + 32 * t;
      xv[t] = 0x7FFFFFFF;
      iv[t] = i;
      pv[t] = 0;
      if (k < total) {
        while (k >= seg_end) {
          ++i;
          seg_end = w.pre[i + 1];
          seg_base = w.lb[i] - w.pre[i];
        }
        pv[t] = seg_base + k;
        iv[t] = i;
        xv[t] = ldg_i32(g.col + pv[t]);
      }
    }
#pragma unroll
    for (int t = 0; t < 4; ++t) {
      const int32_t x = xv[t];
      if (x > smax) continue;
      const uint32_t b = bloom_bit(x) >> 4;
      if (!((w.bloom[b >> 5] >> (b & 31)) & 1u)) continue;
      const int j = warp_bsearch(w.S, s, x);
      if (j < 0) continue;
      const int ii = iv[t];
      if (Q == 2) {
        acc += WGT ? (uint64_t)(w.pre[j + 1] - w.pre[j]) : 1;
        if (PART) {
          atomicAdd(&w.cnt[ii], 1u);
          atomicAdd(&w.cnt[j], 1u);
          atomicAdd(&part.e[pv[t]], 1u);
        }
      } else {
        atomicOr(&w.rows[ii], 1u << j);
        if (MULTI) {
          q2 += 1;
          atomicAdd(&w.cnt[ii], 1u);
          atomicAdd(&w.cnt[j], 1u);
          atomicAdd(&part.e[pv[t]], 1u);
        }
      }
    }
  }
  if (MULTI) *q2out = q2;
  __syncwarp();
  if (PART && lane < s && w.cnt[lane]) {
    atomicAdd(&part.v[w.S[lane]], (unsigned long long)w.cnt[lane]);
    atomicAdd(&part.e[d0.x + lane], w.cnt[lane]);
  }
  if (Q >= 3 && Q <= 4 && lane < s) {
    const uint32_t r = w.rows[lane];
    uint32_t bits = r;
    while (bits) {
      const int j = __ffs(bits) - 1;
      bits &= bits - 1;
      const uint32_t m = r & w.rows[j];
      if (Q == 3) {
        if (WGT) {
          uint32_t b3 = m;
          while (b3) {
            const int l = __ffs(b3) - 1;
            b3 &= b3 - 1;
            acc += (uint64_t)(w.pre[l + 1] - w.pre[l]);
          }
        } else {
          acc += __popc(m);
        }
      } else {
        uint32_t b2 = m;
        while (b2) {
          const int l = __ffs(b2) - 1;
          b2 &= b2 - 1;
          acc += __popc(m & w.rows[l]);
        }
      }
    }
  }
  if constexpr (Q >= 5) {
    if (lane < s) acc += word_deep<Q - 1>(w.rows, w.rows[lane]);
  }
  __syncwarp();
  return acc;
}

// One warp, local set S = N+(v0) with s <= 32, rows built by binary search instead of
// streaming: for row i, lane j-i-1 looks S[j] (j > i) up in the sorted N+(S[i]) (clipped
// at max(S) outside the weighted mode) and a ballot gives the row.  Work per task is
// ~ s^2/2 * log2(list length) dependent loads instead of the sum of the list lengths, so
// it wins for small local sets with long neighbour lists (the merge-vs-binary-search
// choice of the reference's intersection primitives, operations.cuh:106-114).
template <int Q, int MODE>
__device__ uint64_t warp_search_task(const GView& g, WarpSmem& w, int32_t v0, Part part,
                                     uint64_t* q2out = nullptr) {
  static_assert(Q >= 2, "search tasks count at least local edges");
  constexpr bool MULTI = MODE == kModeMulti;
  constexpr bool PART = MODE == kModePart || MULTI;
  constexpr bool WGT = MODE == kModeWeight;
  const int lane = threadIdx.x & 31;
  const longlong2 d0 = ldg_ll2(g.dptr + v0);
  const int s = (int)(d0.y - d0.x);
  int32_t xs = 0;
  longlong2 dx = make_longlong2(0, 0);
  if (lane < s) {
    xs = ldg_i32(g.col + d0.x + lane);
    w.S[lane] = xs;
    dx = ldg_ll2(g.dptr + xs);
    w.lb[lane] = dx.x;
  }
  const int32_t smax = __shfl_sync(kFull, xs, s - 1);
  long long hi_end = dx.y;
  if (!WGT && lane < s && dx.y - dx.x > kClipMin && ldg_i32(g.col + dx.y - 1) > smax) {
    long long lo = dx.x, hi = dx.y;
    while (lo < hi) {
      const long long mid = (lo + hi) >> 1;
      if (ldg_i32(g.col + mid) <= smax) lo = mid + 1; else hi = mid;
    }
    hi_end = lo;
  }
  w.pre[lane] = (int32_t)(dx.y - dx.x);  // full out-degree (the weighted mode's weights)
  w.rows[lane] = 0u;
  w.cnt[lane] = 0u;
  __syncwarp();
  uint64_t acc = 0, q2 = 0;
  for (int i = 0; i + 1 < s; ++i) {
    const long long a = __shfl_sync(kFull, dx.x, i), b = __shfl_sync(kFull, hi_end, i);
    const int j = i + 1 + lane;
    bool found = false;
    long long at = 0;
    if (j < s) {
      const int32_t y = w.S[j];
      long long lo = a, hi = b;
      while (lo < hi) {
        const long long mid = (lo + hi) >> 1;
        if (ldg_i32(g.col + mid) < y) lo = mid + 1; else hi = mid;
      }
      found = lo < b && ldg_i32(g.col + lo) == y;
      at = lo;
    }
    const unsigned bal = __ballot_sync(kFull, found);
    if (Q == 2) {
      if (found) acc += WGT ? (uint64_t)w.pre[j] : 1;
    } else if (lane == 0) {
      w.rows[i] = bal << (i + 1);
    }
    if (PART && found) {
      atomicAdd(&w.cnt[j], 1u);
      atomicAdd(&part.e[at], 1u);
    }
    if (lane == 0 && PART && bal) atomicAdd(&w.cnt[i], (unsigned)__popc(bal));
    if (MULTI && found) q2 += 1;
  }
  if (MULTI) *q2out = q2;
  __syncwarp();
  if (PART && lane < s && w.cnt[lane]) {
    atomicAdd(&part.v[w.S[lane]], (unsigned long long)w.cnt[lane]);
    atomicAdd(&part.e[d0.x + lane], w.cnt[lane]);
  }
  if (Q >= 3 && Q <= 4 && lane < s) {
    const uint32_t r = w.rows[lane];
    uint32_t bits = r;
    while (bits) {
      const int j = __ffs(bits) - 1;
      bits &= bits - 1;
      const uint32_t m = r & w.rows[j];
      if (Q == 3) {
        if (WGT) {
          uint32_t b3 = m;
          while (b3) {
            const int l = __ffs(b3) - 1;
            b3 &= b3 - 1;
            acc += (uint64_t)w.pre[l];
          }
        } else {
          acc += __popc(m);
        }
      } else {
        uint32_t b2 = m;
        while (b2) {
          const int l = __ffs(b2) - 1;
          b2 &= b2 - 1;
          acc += __popc(m & w.rows[l]);
        }
      }
    }
  }
  if constexpr (Q >= 5) {
    if (lane < s) acc += word_deep<Q - 1>(w.rows, w.rows[lane]);
  }
  __syncwarp();
  return acc;
}

// One warp, local set S = N+(v0) with s <= 32, rows by binary search behind X-GMiner's
// bucket-bitmap pre-filter (xgminer/include/xgminer_bitmap.cuh:161-278): for row i,
// lane j-i-1 tests bucket b = S[j] & 15 against the bucket bitmap of N+(S[i]) and
// searches only that bucket of the bucket-grouped list (about 1/16 of it).  Plain
// counting only (the participation and weighted modes run these tasks as SEARCH).
template <int Q>
__device__ uint64_t warp_bucket_task(const GView& g, WarpSmem& w, int32_t v0) {
  static_assert(Q >= 2, "bucket tasks count at least local edges");
  const int lane = threadIdx.x & 31;
  const longlong2 d0 = ldg_ll2(g.dptr + v0);
  const int s = (int)(d0.y - d0.x);
  int32_t xs = 0, deg = 0;
  long long base = 0;
  uint32_t msk = 0u;
  if (lane < s) {
    xs = ldg_i32(g.col + d0.x + lane);
    w.S[lane] = xs;
    const longlong2 dx = ldg_ll2(g.dptr + xs);
    base = dx.x;
    deg = (int32_t)(dx.y - dx.x);
    msk = g.bmask[xs];
  }
  w.rows[lane] = 0u;
  __syncwarp();
  uint64_t acc = 0;
  for (int i = 0; i + 1 < s; ++i) {
    const int32_t u = __shfl_sync(kFull, xs, i);
    const long long bu = __shfl_sync(kFull, base, i);
    const uint32_t mu = __shfl_sync(kFull, msk, i);
    const int32_t du = __shfl_sync(kFull, deg, i);
    const int j = i + 1 + lane;
    bool found = false;
    if (j < s) {
      const int32_t y = w.S[j];
      const int b = y & (kBuckets - 1);
      if ((mu >> b) & 1u) {
        const uint32_t* off = g.boff + (int64_t)u * kBuckets;
        long long lo = bu + off[b];
        const long long end = bu + (b + 1 < kBuckets ? (long long)off[b + 1] : (long long)du);
        long long hi = end;
        while (lo < hi) {
          const long long mid = (lo + hi) >> 1;
          if (ldg_i32(g.bcol + mid) < y) lo = mid + 1; else hi = mid;
        }
        found = lo < end && ldg_i32(g.bcol + lo) == y;
      }
    }
    const unsigned bal = __ballot_sync(kFull, found);
    if (Q == 2) {
      acc += found ? 1u : 0u;
    } else if (lane == 0) {
      w.rows[i] = bal << (i + 1);
    }
  }
  __syncwarp();
  if (Q >= 3 && lane < s) acc += word_deep<Q - 1>(w.rows, w.rows[lane]);
  __syncwarp();
  return acc;
}

// Eight lanes per task, four tasks per warp, local set S = N+(v0) with s <= 8: rows by
// binary search as in the SEARCH tier, each group of eight lanes its own task (the
// per-task granularity the reference fixes at one warp, glumin_GM_solver.cu:324-346).
// rows / cnt are the group's 8-entry slices of the warp's region.  Returns this lane's
// partial count (the caller sums the group); *q2out gets its local-edge partial.
template <int Q, int MODE>
__device__ uint64_t group_task(const GView& g, uint32_t* rows, uint32_t* cnt, int32_t v0, bool ok,
                               Part part, uint64_t* q2out) {
  static_assert(Q >= 2, "group tasks count at least local edges");
  constexpr bool MULTI = MODE == kModeMulti;
  constexpr bool PART = MODE == kModePart || MULTI;
  const int lane = threadIdx.x & 31, gl = lane & 7, gbase = lane & ~7;
  longlong2 d0 = make_longlong2(0, 0);
  if (ok) d0 = ldg_ll2(g.dptr + v0);
  const int s = ok ? (int)(d0.y - d0.x) : 0;
  int32_t xs = 0;
  longlong2 dx = make_longlong2(0, 0);
  if (gl < s) {
    xs = ldg_i32(g.col + d0.x + gl);
    dx = ldg_ll2(g.dptr + xs);
  }
  cnt[gl] = 0u;
  __syncwarp();
  uint32_t myrow = 0u;
  uint64_t acc = 0, q2 = 0;
  for (int i = 0; i < kGroupCap - 1; ++i) {  // uniform trip count: every group shuffles alike
    const long long a = __shfl_sync(kFull, dx.x, gbase + i), b = __shfl_sync(kFull, dx.y, gbase + i);
    const int j = i + 1 + gl;
    const int32_t y = __shfl_sync(kFull, xs, gbase + (j < kGroupCap ? j : kGroupCap - 1));
    bool found = false;
    long long at = 0;
    if (j < s) {
      long long lo = a, hi = b;
      while (lo < hi) {
        const long long mid = (lo + hi) >> 1;
        if (ldg_i32(g.col + mid) < y) lo = mid + 1; else hi = mid;
      }
      found = lo < b && ldg_i32(g.col + lo) == y;
      at = lo;
    }
    const uint32_t bits = (__ballot_sync(kFull, found) >> gbase) & 0xFFu;
    if (gl == i) myrow = bits << (i + 1);
    if (Q == 2 && found) acc += 1;
    if (PART) {
      if (found) {
        atomicAdd(&cnt[j], 1u);
        atomicAdd(&part.e[at], 1u);
      }
      if (gl == 0 && bits) atomicAdd(&cnt[i], (unsigned)__popc(bits));
    }
    if (MULTI && found) q2 += 1;
  }
  rows[gl] = myrow;
  __syncwarp();
  if (PART && gl < s && cnt[gl]) {
    atomicAdd(&part.v[xs], (unsigned long long)cnt[gl]);
    atomicAdd(&part.e[d0.x + gl], cnt[gl]);
  }
  if (Q >= 3 && gl < s) acc += word_deep<Q - 1>(rows, myrow);
  __syncwarp();
  if (MULTI) *q2out = q2;
  return acc;
}

__device__ __forceinline__ uint64_t group_sum_u64(uint64_t v) {
#pragma unroll
  for (int o = 4; o > 0; o >>= 1) v += __shfl_xor_sync(kFull, v, o);
  return v;
}

// One warp, local set S = N+(v0) with s <= 128 (rows of 4 words): Q-cliques of the
// local DAG.  Same walk as the CTA tier (segment registers, four loads in flight, Bloom
// pre-filter) with binary search in S; counting gives each lane whole rows.
template <int Q, int MODE>
__device__ uint64_t warp_wide_task(const GView& g, WideSmem& w, int32_t v0, Part part,
                                   uint64_t* q2out = nullptr) {
  static_assert(Q >= 2, "wide tasks count at least local edges");
  constexpr bool MULTI = MODE == kModeMulti;
  constexpr bool PART = MODE == kModePart || MULTI;
  constexpr bool WGT = MODE == kModeWeight;
  constexpr bool kVec = !PART && !WGT;  // 128-bit loads of the lists, as in cta_local
  const int lane = threadIdx.x & 31;
  const longlong2 d0 = ldg_ll2(g.dptr + v0);
  const int s = (int)(d0.y - d0.x);
  // lane owns items 4*lane .. 4*lane+3 (contiguous, for the scan)
  int len[4];
  long long lbv[4];
  int32_t xs[4];
#pragma unroll
  for (int t = 0; t < 4; ++t) {
    const int i = 4 * lane + t;
    len[t] = 0;
    lbv[t] = 0;
    xs[t] = 0;
    if (i < s) {
      xs[t] = ldg_i32(g.col + d0.x + i);
      w.S[i] = xs[t];
      const longlong2 d = ldg_ll2(g.dptr + xs[t]);
      lbv[t] = d.x;
      len[t] = (int)(d.y - d.x);
    }
  }
  __syncwarp();
  const int32_t smax = w.S[s - 1];
  const int32_t next0 = __shfl_down_sync(kFull, xs[0], 1);  // item 4 * lane + 4
  if (!WGT) {  // clip row i to [S[i+1], max(S)] (neutral here, unlike the CTA tier)
#pragma unroll
    for (int t = 0; t < 4; ++t) {
      const int i = 4 * lane + t;
      if (i >= s) continue;
      long long lo = lbv[t], hi = lbv[t] + len[t];
      if (i + 1 == s) lo = hi;
      else if (hi - lo > kClipLoMin) lo = lower_pos(g.col, lo, hi, t < 3 ? xs[t + 1] : next0);
      if (hi - lo > kClipMin && ldg_i32(g.col + hi - 1) > smax)
        hi = lower_pos(g.col, lo, hi, smax + 1);
      lbv[t] = lo;
      len[t] = (int)(hi - lo);
    }
  }
  int units[4];  // kVec: 16-byte units of each list from its aligned start
#pragma unroll
  for (int t = 0; t < 4; ++t) {
    const long long a = lbv[t] & ~3ll;
    units[t] = kVec ? (len[t] > 0 ? (int)((lbv[t] + len[t] - a + 3) >> 2) : 0) : len[t];
  }
  const int mine = units[0] + units[1] + units[2] + units[3];
  int inc = mine;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int y = __shfl_up_sync(kFull, inc, o);
    if (lane >= o) inc += y;
  }
  int ex = inc - mine;
  if (PART)
    for (int x = lane; x < kWideCap; x += 32) w.cnt[x] = 0u;
#pragma unroll
  for (int t = 0; t < 4; ++t) {
    const int i = 4 * lane + t;
    if (i <= s) w.pre[i] = ex;  // pre[s] = total (items >= s have length 0)
    if (i < s) {
      if (kVec) {  // aligned start | phase; the list's length in cnt
        const long long a = lbv[t] & ~3ll;
        w.lb[i] = a | (lbv[t] - a);
        w.cnt[i] = (uint32_t)len[t];
      } else {
        w.lb[i] = lbv[t];
      }
    }
    ex += units[t];
  }
  if (lane == 31) w.pre[kWideCap] = inc;  // total when s == kWideCap
  for (int x = lane; x < kWideCap * kWideWords; x += 32) w.rows[x] = 0u;
  w.bloom[lane] = 0u;  // kWideBloomWords == 64
  w.bloom[lane + 32] = 0u;
  __syncwarp();
#pragma unroll
  for (int t = 0; t < 4; ++t)
    if (4 * lane + t < s) {
      const uint32_t b = bloom_bit(xs[t]) >> 3;  // 11 bits
      atomicOr(&w.bloom[b >> 5], 1u << (b & 31));
    }
  __syncwarp();
  const int total = w.pre[s];
  uint64_t acc = 0, q2 = 0;
  int i = 0;
  if constexpr (kVec) {  // kWideUnits 16-byte units per lane in flight, then their elements
    constexpr int kNU = kWideUnits;
    for (int kb = lane; kb < total; kb += 32 * kNU) {
      int4 v[kNU];
      int iv[kNU], rel[kNU], ln[kNU];
#pragma unroll
      for (int h = 0; h < kNU; ++h) {
        const int k = kb + 32 * h;
        iv[h] = i;
        rel[h] = 0;
        ln[h] = 0;
        v[h] = make_int4(0, 0, 0, 0);
        if (k < total) {
          while (k >= w.pre[i + 1]) ++i;
          const long long L = w.lb[i];
          const int u = k - w.pre[i];
          iv[h] = i;
          rel[h] = 4 * u - (int)(L & 3);
          ln[h] = (int)w.cnt[i];
          v[h] = __ldg((const int4*)(g.col + (L & ~3ll)) + u);
        }
      }
#pragma unroll
      for (int h = 0; h < kNU; ++h) {
        const int32_t xs4[4] = {v[h].x, v[h].y, v[h].z, v[h].w};
#pragma unroll
        for (int t = 0; t < 4; ++t) {
          const int e = rel[h] + t;
          const int32_t x = xs4[t];
          if (e < 0 || e >= ln[h] || x > smax) continue;
          const uint32_t b = bloom_bit(x) >> 3;
          if (!((w.bloom[b >> 5] >> (b & 31)) & 1u)) continue;
          const int j = warp_bsearch(w.S, s, x);
          if (j < 0) continue;
          const int ii = iv[h];
          if (Q == 2) acc += 1;
          else atomicOr(&w.rows[ii * kWideWords + (j >> 5)], 1u << (j & 31));
        }
      }
    }
  } else {
  int seg_end = w.pre[1];
  long long seg_base = w.lb[0];
  for (int kb = lane; kb < total; kb += 128) {
    int32_t xv[4];
    int iv[4];
    long long pv[4];
#pragma unroll
    for (int t = 0; t < 4; ++t) {
      const int k = kb + 32 * t;
      xv[t] = 0x7FFFFFFF;
      iv[t] = i;
      pv[t] = 0;
      if (k < total) {
        while (k >= seg_end) {
          ++i;
          seg_end = w.pre[i + 1];
          seg_base = w.lb[i] - w.pre[i];
        }
        pv[t] = seg_base + k;
        iv[t] = i;
        xv[t] = ldg_i32(g.col + pv[t]);
      }
    }
#pragma unroll
    for (int t = 0; t < 4; ++t) {
      const int32_t x = xv[t];
      if (x > smax) continue;
      const uint32_t b = bloom_bit(x) >> 3;
      if (!((w.bloom[b >> 5] >> (b & 31)) & 1u)) continue;
      const int j = warp_bsearch(w.S, s, x);
      if (j < 0) continue;
      const int ii = iv[t];
      if (Q == 2) {
        acc += WGT ? (uint64_t)(w.pre[j + 1] - w.pre[j]) : 1;
        if (PART) {
          atomicAdd(&w.cnt[ii], 1u);
          atomicAdd(&w.cnt[j], 1u);
          atomicAdd(&part.e[pv[t]], 1u);
        }
      } else {
        atomicOr(&w.rows[ii * kWideWords + (j >> 5)], 1u << (j & 31));
        if (MULTI) {
          q2 += 1;
          atomicAdd(&w.cnt[ii], 1u);
          atomicAdd(&w.cnt[j], 1u);
          atomicAdd(&part.e[pv[t]], 1u);
        }
      }
    }
  }
  }
  if (MULTI) *q2out = q2;
  __syncwarp();
  if (PART)
    for (int r = lane; r < s; r += 32)
      if (w.cnt[r]) {
        atomicAdd(&part.v[w.S[r]], (unsigned long long)w.cnt[r]);
        atomicAdd(&part.e[d0.x + r], w.cnt[r]);
      }
  if constexpr ((Q == 3 && !WGT) || Q == 4) {
    // lane per row, its four words in registers; a member's row is one 128-bit load
    // (rows are 16-byte aligned; words below a member's block are zero, so the full
    // four-word AND needs no per-word branch)
    static_assert(kWideWords == 4, "wide rows are one uint4");
    const uint4* R4 = reinterpret_cast<const uint4*>(w.rows);
    for (int r = lane; r < s; r += 32) {
      const uint4 rr = R4[r];
      const uint32_t rw[4] = {rr.x, rr.y, rr.z, rr.w};
#pragma unroll
      for (int wj = 0; wj < 4; ++wj) {
        uint32_t bits = rw[wj];
        while (bits) {
          const int j = (wj << 5) + __ffs(bits) - 1;
          bits &= bits - 1;
          const uint4 rj = R4[j];
          const uint32_t m0 = rr.x & rj.x, m1 = rr.y & rj.y, m2 = rr.z & rj.z, m3 = rr.w & rj.w;
          if constexpr (Q == 3) {
            acc += (uint32_t)(__popc(m0) + __popc(m1) + __popc(m2) + __popc(m3));
          } else {
            const uint32_t mw[4] = {m0, m1, m2, m3};
            uint32_t part = 0;
#pragma unroll
            for (int wl = 0; wl < 4; ++wl) {
              uint32_t b3 = mw[wl];
              while (b3) {
                const int l = (wl << 5) + __ffs(b3) - 1;
                b3 &= b3 - 1;
                const uint4 rl = R4[l];
                part += __popc(m0 & rl.x) + __popc(m1 & rl.y) + __popc(m2 & rl.z) +
                        __popc(m3 & rl.w);
              }
            }
            acc += part;
          }
        }
      }
    }
  } else if (Q == 3) {  // weighted: each clique by d+ of its top member
    for (int r = lane; r < s; r += 32) {
      const uint32_t* Rr = w.rows + r * kWideWords;
      for (int wj = r >> 5; wj < kWideWords; ++wj) {
        uint32_t bits = Rr[wj];
        while (bits) {
          const int j = (wj << 5) + __ffs(bits) - 1;
          bits &= bits - 1;
          const uint32_t* Rj = w.rows + j * kWideWords;
          for (int ww = j >> 5; ww < kWideWords; ++ww) {
            const uint32_t m = Rr[ww] & Rj[ww];
            if (!m) continue;
            if (Q == 3) {
              if (WGT) {
                uint32_t b3 = m;
                while (b3) {
                  const int l = (ww << 5) + __ffs(b3) - 1;
                  b3 &= b3 - 1;
                  acc += (uint64_t)(w.pre[l + 1] - w.pre[l]);
                }
              } else {
                acc += __popc(m);
              }
            } else {
              uint32_t b3 = m;
              while (b3) {
                const int l = (ww << 5) + __ffs(b3) - 1;
                b3 &= b3 - 1;
                const uint32_t* Rl = w.rows + l * kWideWords;
                for (int wl = l >> 5; wl < kWideWords; ++wl) {
                  // m restricted to word wl is Rr[wl] & Rj[wl]
                  acc += __popc(Rr[wl] & Rj[wl] & Rl[wl]);
                }
              }
            }
          }
        }
      }
    }
  }
  if constexpr (Q >= 5) {
    for (int r = lane; r < s; r += 32) {
      uint32_t m[4];
#pragma unroll
      for (int y = 0; y < 4; ++y) m[y] = w.rows[r * kWideWords + y];
      acc += wide_deep<Q - 1>(w.rows, m);
    }
  }
  __syncwarp();
  return acc;
}

// ------------------------------------------------------------ persistent kernel
// Emission by one lane that holds a task's totals (grouped tasks).
__device__ __forceinline__ void emit_one(const GOut& o, int32_t v0, uint64_t a, uint64_t b,
                                         uint64_t& acc) {
  if (o.gid) {
    const long long base = (long long)o.gid[v0] * o.stride;
    if (a && o.slot >= 0) atomicAdd(&o.out[base + o.slot], (unsigned long long)a);
    if (b && o.slot2 >= 0) atomicAdd(&o.out[base + o.slot2], (unsigned long long)b);
  } else {
    acc += a;
  }
}

// Per-task emission: one global total (gid == null) or per-graph totals
// out[gid[v0] * stride + slot] (batched graphs).  Called by all 32 lanes of a warp.
__device__ __forceinline__ void emit(const GOut& o, int32_t v0, uint64_t r, uint64_t r2,
                                     uint64_t& acc) {
  if (o.gid) {
    const uint64_t a = warp_sum_u64(r), b = warp_sum_u64(r2);
    if ((threadIdx.x & 31) == 0) {
      const long long base = (long long)o.gid[v0] * o.stride;
      if (a && o.slot >= 0) atomicAdd(&o.out[base + o.slot], (unsigned long long)a);
      if (b && o.slot2 >= 0) atomicAdd(&o.out[base + o.slot2], (unsigned long long)b);
    }
  } else {
    acc += r;
  }
}

// K = clique size (3..7).  MODE kModePart (K == 3) credits triangle participation to
// `part` instead of counting; kModeWeight (K <= 4) weights each clique by the out-degree
// of its highest-ranked vertex; kModeMulti (K == 4) emits triangles to o.slot and
// 4-cliques to o.slot2 and credits participation.
// CTA shape of a kernel mode: the participation and multi modes keep per-member counters.
template <int MODE>
using CtaShapeOf = std::conditional_t<MODE == kModePart || MODE == kModeMulti, CtaMainCnt, CtaMain>;

template <int K, int MODE>
__global__ void __launch_bounds__(kCtaThreads, 2)
    k_clique(GView g, TaskLists t, QueueHeads* q, unsigned long long* count, uint32_t* err,
             Part part, GOut o) {
  constexpr bool MULTI = MODE == kModeMulti;
  constexpr bool PART = MODE == kModePart || MULTI;
  constexpr int kMinS = MULTI ? 2 : K - 1;  // smallest out-degree that can contribute
  static_assert(!MULTI || K == 4, "multi mode runs the 4-clique machinery");
  using ShK = CtaShapeOf<MODE>;
  extern __shared__ __align__(16) char sm[];
  __shared__ long long task_s;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const long long n_split = t.n[0], n_cta = t.n[1], n_warp = t.n[2], n_hubs = t.n[3];
  const long long n_wide = t.n[4], n_search = t.n[5], n_bucket = t.n[6], n_group = t.n[7];
  uint64_t acc = 0;

  // 1) hub edge sub-tasks: local set N+(v0) & N+(v1), (K-2)-cliques of it
  for (;;) {
    if (tid == 0) task_s = (long long)atomicAdd(&q->split, 1ull);
    __syncthreads();
    const long long ti = task_s;
    __syncthreads();
    if (ti >= n_split) break;
    const long long c0 = t.log_split ? clock64() : 0;
    long long lo = 0, hi = n_hubs;  // hub h with split_off[h] <= ti < split_off[h+1]
    while (hi - lo > 1) {
      long long mid = (lo + hi) >> 1;
      if (t.split_off[mid] <= ti) lo = mid; else hi = mid;
    }
    const int32_t v0 = t.split_v[lo];
    const longlong2 d0 = ldg_ll2(g.dptr + v0);
    const long long e01 = d0.x + (ti - t.split_off[lo]);
    const int32_t v1 = ldg_i32(g.col + e01);
    // the local set is stored only when (K-2)-cliques of it have to be counted
    constexpr bool kStore = MULTI || (MODE != kModePart && K - 2 >= 2);
    constexpr bool kWsum = MODE == kModeWeight && K == 3;
    uint64_t wsum = 0;
    const int n = cta_intersect_into_S<PART, kStore, kWsum, ShK>(g, sm, v0, v1, part, &wsum);
    if (n < 0) {
      if (tid == 0) atomicOr(err, ERR_CAPACITY);
    } else {
      if (PART && tid == 0 && n > 0) {
        // triangles (v0, v1, w) for every w of the intersection
        atomicAdd(&part.v[v0], (unsigned long long)n);
        atomicAdd(&part.v[v1], (unsigned long long)n);
        atomicAdd(&part.e[e01], (unsigned)n);
      }
      if (MULTI) {
        const uint64_t k4 =
            n >= 2 ? cta_local<2, kModeCount, ShK>(g, sm, n, part, -1, nullptr, 0, !t.hash_only)
                   : 0;
        emit(o, v0, tid == 0 ? (uint64_t)n : 0, k4, acc);
      } else if (!PART && n > 0) {
        uint64_t r;
        if (K - 2 == 1) r = kWsum ? wsum : (tid == 0 ? (uint64_t)n : 0);  // |L| once per CTA
        else r = cta_local<K - 2, MODE, ShK>(g, sm, n, part, -1, nullptr, 0, !t.hash_only);
        if (MODE == kModeWeight) acc += r; else emit(o, v0, r, 0, acc);
      }
    }
    __syncthreads();
    if (t.log_split && tid == 0) t.log_split[ti] = clock64() - c0;
  }
  // 2) CTA vertex tasks: local set N+(v0)
  for (;;) {
    if (tid == 0) task_s = (long long)atomicAdd(&q->cta, 1ull);
    __syncthreads();
    const long long ti = task_s;
    __syncthreads();
    if (ti >= n_cta) break;
    const long long c0 = t.log_cta ? clock64() : 0;
    const int32_t v0 = t.cta[ti];
    const longlong2 d0 = ldg_ll2(g.dptr + v0);
    const int s = (int)(d0.y - d0.x);
    if (s > kCtaCap) {
      if (tid == 0) atomicOr(err, ERR_CAPACITY);
    } else if (s >= kMinS) {
      int32_t* S = (int32_t*)(sm + kOffS);
      for (int i = tid; i < s; i += kCtaThreads) S[i] = ldg_i32(g.col + d0.x + i);
      __syncthreads();
      uint64_t q2 = 0;
      const uint64_t r = cta_local<K - 1, MODE, ShK>(g, sm, s, part, d0.x, &q2, 0, !t.hash_only);
      if (PART) {
        // every local edge is a triangle containing v0
        const uint64_t tot = warp_sum_u64(MULTI ? q2 : r);
        if (lane == 0 && tot) atomicAdd(&part.v[v0], (unsigned long long)tot);
      }
      if (MULTI) emit(o, v0, q2, r, acc);
      else if (MODE == kModeWeight) acc += r;
      else if (!PART) emit(o, v0, r, 0, acc);
    }
    __syncthreads();
    if (t.log_cta && tid == 0) t.log_cta[ti] = clock64() - c0;
  }
  // 3) wide-warp vertex tasks (s <= 128); the CTA region is reused per warp
  {
    WideSmem& wd = ((WideSmem*)sm)[warp];
    for (;;) {
      long long ti = 0;
      if (lane == 0) ti = (long long)atomicAdd(&q->wide, 1ull);
      ti = __shfl_sync(kFull, ti, 0);
      if (ti >= n_wide) break;
      const long long c0 = t.log_wide ? clock64() : 0;
      const int32_t v0 = t.wide[ti];
      const longlong2 d0 = ldg_ll2(g.dptr + v0);
      const int s = (int)(d0.y - d0.x);
      if (s > kWideCap) {
        if (lane == 0) atomicOr(err, ERR_CAPACITY);
      } else if (s >= kMinS) {
        uint64_t q2 = 0;
        const uint64_t r = warp_wide_task<K - 1, MODE>(g, wd, v0, part, &q2);
        if (PART) {
          const uint64_t tot = warp_sum_u64(MULTI ? q2 : r);
          if (lane == 0 && tot) atomicAdd(&part.v[v0], (unsigned long long)tot);
        }
        if (MULTI) emit(o, v0, q2, r, acc);
        else if (MODE == kModeWeight) acc += r;
        else if (!PART) emit(o, v0, r, 0, acc);
      }
      if (t.log_wide && lane == 0) t.log_wide[ti] = clock64() - c0;
    }
  }
  // 4) warp vertex tasks (s <= 32), in a region disjoint from every wide region: first
  //    those built by binary search, then those built by streaming
  WarpSmem& ws = ((WarpSmem*)(sm + kOffWarpRegion))[warp];
  for (;;) {
    long long ti = 0;
    if (lane == 0) ti = (long long)atomicAdd(&q->search, 1ull);
    ti = __shfl_sync(kFull, ti, 0);
    if (ti >= n_search) break;
    const long long c0 = t.log_search ? clock64() : 0;
    const int32_t v0 = t.search[ti];
    const longlong2 d0 = ldg_ll2(g.dptr + v0);
    const int s = (int)(d0.y - d0.x);
    if (s > kWarpCap) {
      if (lane == 0) atomicOr(err, ERR_CAPACITY);
    } else if (s >= kMinS) {
      uint64_t q2 = 0;
      const uint64_t r = warp_search_task<K - 1, MODE>(g, ws, v0, part, &q2);
      if (PART) {
        const uint64_t tot = warp_sum_u64(MULTI ? q2 : r);
        if (lane == 0 && tot) atomicAdd(&part.v[v0], (unsigned long long)tot);
      }
      if (MULTI) emit(o, v0, q2, r, acc);
      else if (MODE == kModeWeight) acc += r;
      else if (!PART) emit(o, v0, r, 0, acc);
    }
    if (t.log_search && lane == 0) t.log_search[ti] = clock64() - c0;
  }
  // grouped tasks: four per warp, eight lanes each (weighted mode: one task at a time)
  for (;;) {
    long long base = 0;
    if (lane == 0) base = (long long)atomicAdd(&q->group, (unsigned long long)kGroupsPerWarp);
    base = __shfl_sync(kFull, base, 0);
    if (base >= n_group) break;
    if constexpr (MODE == kModeWeight) {
      for (int x = 0; x < kGroupsPerWarp && base + x < n_group; ++x) {
        const int32_t v0 = t.group[base + x];
        const longlong2 d0 = ldg_ll2(g.dptr + v0);
        const int s = (int)(d0.y - d0.x);
        if (s > kGroupCap) {
          if (lane == 0) atomicOr(err, ERR_CAPACITY);
        } else if (s >= kMinS) {
          acc += warp_search_task<K - 1, MODE>(g, ws, v0, part, nullptr);
        }
      }
    } else {
      const int gi = lane >> 3;
      const long long ti = base + gi;
      const bool live = ti < n_group;
      const long long c0 = t.log_group ? clock64() : 0;
      const int32_t v0 = live ? t.group[ti] : 0;
      int s = 0;
      if (live) {
        const longlong2 d0 = ldg_ll2(g.dptr + v0);
        s = (int)(d0.y - d0.x);
        if (s > kGroupCap && (lane & 7) == 0) atomicOr(err, ERR_CAPACITY);
      }
      const bool ok = live && s >= kMinS && s <= kGroupCap;
      uint64_t q2 = 0;
      const uint64_t r = group_sum_u64(
          group_task<K - 1, MODE>(g, ws.rows + 8 * gi, ws.cnt + 8 * gi, v0, ok, part, &q2));
      q2 = group_sum_u64(q2);
      if (ok && (lane & 7) == 0) {
        if (PART) {
          const uint64_t tot = MULTI ? q2 : r;
          if (tot) atomicAdd(&part.v[v0], (unsigned long long)tot);
        }
        if (MULTI) emit_one(o, v0, q2, r, acc);
        else if (!PART) emit_one(o, v0, r, 0, acc);
      }
      if (t.log_group && live && (lane & 7) == 0) t.log_group[ti] = clock64() - c0;
    }
  }
  for (;;) {  // bucket-filtered search tasks (run as SEARCH outside plain counting)
    long long ti = 0;
    if (lane == 0) ti = (long long)atomicAdd(&q->bucket, 1ull);
    ti = __shfl_sync(kFull, ti, 0);
    if (ti >= n_bucket) break;
    const long long c0 = t.log_bucket ? clock64() : 0;
    const int32_t v0 = t.bucket[ti];
    const longlong2 d0 = ldg_ll2(g.dptr + v0);
    const int s = (int)(d0.y - d0.x);
    if (s > kWarpCap) {
      if (lane == 0) atomicOr(err, ERR_CAPACITY);
    } else if (s >= kMinS) {
      uint64_t q2 = 0, r;
      if (MODE == kModeCount && g.bcol) r = warp_bucket_task<K - 1>(g, ws, v0);
      else r = warp_search_task<K - 1, MODE>(g, ws, v0, part, &q2);
      if (PART) {
        const uint64_t tot = warp_sum_u64(MULTI ? q2 : r);
        if (lane == 0 && tot) atomicAdd(&part.v[v0], (unsigned long long)tot);
      }
      if (MULTI) emit(o, v0, q2, r, acc);
      else if (MODE == kModeWeight) acc += r;
      else if (!PART) emit(o, v0, r, 0, acc);
    }
    if (t.log_bucket && lane == 0) t.log_bucket[ti] = clock64() - c0;
  }
  for (;;) {
    long long ti = 0;
    if (lane == 0) ti = (long long)atomicAdd(&q->warp, 1ull);
    ti = __shfl_sync(kFull, ti, 0);
    if (ti >= n_warp) break;
    const long long c0 = t.log_warp ? clock64() : 0;
    const int32_t v0 = t.warp[ti];
    const longlong2 d0 = ldg_ll2(g.dptr + v0);
    const int s = (int)(d0.y - d0.x);
    if (s > kWarpCap) {
      if (lane == 0) atomicOr(err, ERR_CAPACITY);
    } else if (s >= kMinS) {
      uint64_t q2 = 0;
      const uint64_t r = warp_vertex_task<K - 1, MODE>(g, ws, v0, part, &q2);
      if (PART) {
        const uint64_t tot = warp_sum_u64(MULTI ? q2 : r);
        if (lane == 0 && tot) atomicAdd(&part.v[v0], (unsigned long long)tot);
      }
      if (MULTI) emit(o, v0, q2, r, acc);
      else if (MODE == kModeWeight) acc += r;
      else if (!PART) emit(o, v0, r, 0, acc);
    }
    if (t.log_warp && lane == 0) t.log_warp[ti] = clock64() - c0;
  }
  if (!PART && count) {
    acc = warp_sum_u64(acc);
    if (lane == 0 && acc) atomicAdd(count, (unsigned long long)acc);
  }
}

// ------------------------------------------------------------------ hub kernel
// Bulk copy (TMA, cp.async.bulk) global -> this CTA's shared memory, completing on an
// mbarrier; both addresses and the size are multiples of 16 bytes.
__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint32_t bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes)
               : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint32_t bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
      " selp.u32 %0, 1, 0, p;\n}"
      : "=r"(ok)
      : "r"(bar), "r"(parity)
      : "memory");
  return ok != 0;
}
__device__ __forceinline__ void bulk_g2s(uint32_t dst, const void* src, uint32_t bytes,
                                         uint32_t bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
      ::"r"(dst), "l"(src), "r"(bytes), "r"(bar)
      : "memory");
}
// Bounded wait for the phase `parity` of the barrier (try_wait suspends the thread for
// a while each call): false when the limit ran out.
constexpr int kBarSpin = 1 << 22;
__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity) {
  for (int it = 0; it < kBarSpin; ++it)
    if (mbar_try_wait(bar, parity)) return true;
  return false;
}

// Hub vertices just above the main CTA's capacity (kCtaCap < s <= t.hub_max <= kHubCap)
// run whole: one 1024-thread CTA per SM holds N+(v0) and the bitmap of the DAG induced
// on it (cta_local on the CtaHub layout, ~209 KB of shared memory) instead of splitting
// the hub into s edge sub-tasks that each intersect two global lists (the role of
// GLUMIN's per-hub LUT, glumin_GM_solver.cu:490-503, codegen_bitmap.cuh:884-968).  The
// hub's list is staged by one bulk copy (TMA) from its 16-byte-aligned start; the first
// member sits `off` words in.  Count mode, k <= 5 only (otherwise every hub is split).
template <int K>
__global__ void __launch_bounds__(kHubThreads, 1)
    k_clique_hub(GView g, TaskLists t, QueueHeads* q, unsigned long long* count, uint32_t* err,
                 GOut o) {
  static_assert(K >= 3 && K <= 5, "the hub CTA counts up to 5-cliques (rows of <= 64 words)");
  extern __shared__ __align__(128) char sm[];
  __shared__ long long task_s;
  const int tid = threadIdx.x, lane = tid & 31;
  const uint32_t bar = (uint32_t)__cvta_generic_to_shared(sm + CtaHub::kOffBar);
  const uint32_t sdst = (uint32_t)__cvta_generic_to_shared(sm + CtaHub::kOffS);
  if (tid == 0) {
    mbar_init(bar, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncthreads();
  uint32_t phase = 0;
  uint64_t acc = 0;
  const long long n_hubs = t.n[3];
  for (;;) {
    if (tid == 0) task_s = (long long)atomicAdd(&q->hub, 1ull);
    __syncthreads();
    const long long ti = task_s;
    __syncthreads();
    if (ti >= n_hubs) break;
    const int32_t v0 = t.split_v[ti];
    const longlong2 d0 = ldg_ll2(g.dptr + v0);
    const int s = (int)(d0.y - d0.x);
    // hubs with sub-tasks run split in the main kernel; those without run here
    if (s <= kCtaCap || s > t.hub_max || t.split_off[ti + 1] != t.split_off[ti]) continue;
    const long long a0 = d0.x & ~3ll;
    const int off = (int)(d0.x - a0);
    const uint32_t bytes = (uint32_t)(((off + s) * 4 + 15) & ~15);  // <= 4 (kHubCap + 4)
    if (tid == 0) {
      // the previous task's generic-proxy accesses to S come before this async write
      asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
      mbar_expect_tx(bar, bytes);
      bulk_g2s(sdst, g.col + a0, bytes, bar);  // col has 16 bytes of slack at its end
    }
    const bool ok = mbar_wait(bar, phase);
    phase ^= 1u;
    if (!__syncthreads_and(ok)) {  // the copy did not land: report it, stop this CTA
      if (tid == 0) {
        atomicOr(err, ERR_TIMEOUT);
        mbar_wait(bar, phase ^ 1u);  // bounded: let a late copy finish before exit
      }
      break;
    }
    const uint64_t r = cta_local<K - 1, kModeCount, CtaHub>(g, sm, s, Part{nullptr, nullptr}, -1,
                                                            nullptr, off, !t.hash_only);
    emit(o, v0, r, 0, acc);
    __syncthreads();
  }
  if (count) {
    acc = warp_sum_u64(acc);
    if (lane == 0 && acc) atomicAdd(count, (unsigned long long)acc);
  }
}

// Sets the dynamic shared-memory opt-in of `fn` once per device (bit d of `mask`;
// devices >= 64 set it on every launch).
template <class F>
cudaError_t smem_optin(F fn, int bytes, std::atomic<unsigned long long>& mask,
                       int carveout_pct = -1) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  const unsigned long long bit = dev < 64 ? (1ull << dev) : 0ull;
  if (!bit || !(mask.load(std::memory_order_acquire) & bit)) {
    e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
    if (e != cudaSuccess) return e;
    if (carveout_pct >= 0) {  // preferred shared-memory share of the unified L1
      e = cudaFuncSetAttribute(fn, cudaFuncAttributePreferredSharedMemoryCarveout, carveout_pct);
      if (e != cudaSuccess) return e;
    }
    mask.fetch_or(bit, std::memory_order_acq_rel);
  }
  return cudaSuccess;
}

template <int K>
cudaError_t launch_hub(const GView& g, const TaskLists& t, QueueHeads* q,
                       unsigned long long* count, uint32_t* err, cudaStream_t s, const GOut& o) {
  static std::atomic<unsigned long long> attr_devices{0};
  cudaError_t e = smem_optin(k_clique_hub<K>, kHubSmem, attr_devices);
  if (e != cudaSuccess) return e;
  int dev = 0, sms = 0;
  e = cudaGetDevice(&dev);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  if (e != cudaSuccess) return e;
  k_clique_hub<K><<<sms, kHubThreads, kHubSmem, s>>>(g, t, q, count, err, o);
  return cudaGetLastError();
}

template <int K, int MODE>
cudaError_t launch_k(const GView& g, const TaskLists& t, QueueHeads* q, unsigned long long* count,
                     uint32_t* err, Part part, int grid, cudaStream_t s, GOut o = GOut{}) {
  // The shared-memory opt-in is a per-device function attribute.
  static std::atomic<unsigned long long> attr_devices{0};
  constexpr int kSmem = CtaShapeOf<MODE>::kSmem;
  cudaError_t e = smem_optin(k_clique<K, MODE>, kSmem, attr_devices,
                             -1);
  if (e != cudaSuccess) return e;
  k_clique<K, MODE><<<grid, kCtaThreads, kSmem, s>>>(g, t, q, count, err, part, o);
  return cudaGetLastError();
}

}  // namespace

size_t clique_smem_bytes() { return kCtaSmem; }

cudaError_t clique_occupancy(int* per_sm) {
  cudaError_t e = cudaFuncSetAttribute(k_clique<4, kModeCount>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, kCtaSmem);
  if (e != cudaSuccess) return e;
  return cudaOccupancyMaxActiveBlocksPerMultiprocessor(per_sm, k_clique<4, kModeCount>,
                                                       kCtaThreads, kCtaSmem);
}

int clique_grid(int num_sms) { return 2 * num_sms; }

cudaError_t launch_clique(int k, const GView& g, const TaskLists& t, QueueHeads* q,
                          unsigned long long* count, uint32_t* err, int grid, cudaStream_t s,
                          const GOut& o) {
  const Part none{nullptr, nullptr};
  cudaError_t e;
  switch (k) {
    case 3: e = launch_k<3, kModeCount>(g, t, q, count, err, none, grid, s, o); break;
    case 4: e = launch_k<4, kModeCount>(g, t, q, count, err, none, grid, s, o); break;
    case 5: e = launch_k<5, kModeCount>(g, t, q, count, err, none, grid, s, o); break;
    case 6: e = launch_k<6, kModeCount>(g, t, q, count, err, none, grid, s, o); break;
    case 7: e = launch_k<7, kModeCount>(g, t, q, count, err, none, grid, s, o); break;
    default: return cudaErrorInvalidValue;
  }
  if (e != cudaSuccess || t.hub_max <= kCtaCap) return e;
  switch (k) {
    case 3: return launch_hub<3>(g, t, q, count, err, s, o);
    case 4: return launch_hub<4>(g, t, q, count, err, s, o);
    case 5: return launch_hub<5>(g, t, q, count, err, s, o);
    default: return cudaErrorInvalidValue;  // schedule_into leaves hub_max at 0 for k > 5
  }
}

cudaError_t launch_multi(const GView& g, const TaskLists& t, QueueHeads* q,
                         unsigned long long* vpart, unsigned* epart, uint32_t* err, int grid,
                         cudaStream_t s, const GOut& o) {
  return launch_k<4, kModeMulti>(g, t, q, nullptr, err, Part{vpart, epart}, grid, s, o);
}

cudaError_t launch_clique_weighted(int k, const GView& g, const TaskLists& t, QueueHeads* q,
                                   unsigned long long* sum, uint32_t* err, int grid,
                                   cudaStream_t s) {
  const Part none{nullptr, nullptr};
  switch (k) {
    case 3: return launch_k<3, kModeWeight>(g, t, q, sum, err, none, grid, s);
    case 4: return launch_k<4, kModeWeight>(g, t, q, sum, err, none, grid, s);
    default: return cudaErrorInvalidValue;
  }
}

cudaError_t launch_triangle_participation(const GView& g, const TaskLists& t, QueueHeads* q,
                                          unsigned long long* vpart, unsigned* epart,
                                          uint32_t* err, int grid, cudaStream_t s) {
  return launch_k<3, kModePart>(g, t, q, nullptr, err, Part{vpart, epart}, grid, s);
}

}  // namespace xgm
