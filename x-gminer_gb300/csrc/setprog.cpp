// Set-operation programs (setprog.cuh): GLUMIN's P6-P22 tables, the pattern
// compiler and the word form.
#include "setprog.cuh"

#include <algorithm>
#include <cstring>
#include <vector>

namespace xgm {

namespace {

constexpr int8_t G(int j) { return (int8_t)(kOpList + j); }
constexpr uint8_t V(int j) { return (uint8_t)(1u << j); }

ProgOp op(int out, int kind, int a, int b, int bound = 0, int excl = 0) {
  return ProgOp{(int8_t)out, (int8_t)kind, (int8_t)a, (int8_t)b, (uint8_t)bound, (uint8_t)excl};
}

void fail(std::string* why, const char* msg) {
  if (why) *why = msg;
}

}  // namespace

// GLUMIN's generated 5-vertex plans, one row per GM_kernels/P<id>-GM.yml.cuh body
// (codes/GLUMIN/src/G2Miner/gpu_GM_LUT_kernels/GM_kernels/): the level-0 slots from
// N(v0) and N(v1), the slot v2 runs over, the level-1 slots refined with N(v2), the
// slot v3 runs over and the counted operation.  The set semantics are GLUMIN's: a
// difference keeps every element of its first list that is absent from the second,
// so a matched vertex can reappear (N(v1) \ N(v0) holds v0); P12, P13, P19 and P22
// count such repeated-vertex embeddings, as the reference does.
bool prog_glumin(int pid, Prog* p) {
  Prog q;
  q.k = 5;
  q.flat = 1;
  q.cand[2] = 0;
  const int I = OP_INTERSECT, D = OP_DIFFERENCE;
  auto set = [&](std::initializer_list<ProgOp> l0, std::initializer_list<ProgOp> l1, int c3,
                 ProgOp fin) {
    int n = 0, hi = -1;
    for (const ProgOp& o : l0) q.ops[0][n++] = o, hi = std::max(hi, (int)o.out);
    q.nops[0] = (int8_t)n;
    n = 0;
    for (const ProgOp& o : l1) q.ops[1][n++] = o, hi = std::max(hi, (int)o.out);
    q.nops[1] = (int8_t)n;
    q.cand[3] = (int8_t)c3;
    q.fin = fin;
    q.nslots = (int8_t)(hi + 1);
  };
  switch (pid) {
    case 6:  // P6-GM.yml.cuh:38-56
      set({op(0, I, G(0), G(1), V(1)), op(1, D, G(0), G(1))}, {op(2, D, 1, G(2), V(1))}, 2,
          op(-1, I, 2, G(3), V(3)));
      break;
    case 7:  // P7-GM.yml.cuh
      set({op(0, D, G(1), G(0)), op(1, I, G(0), G(1)), op(2, D, G(0), G(1))},
          {op(3, D, 1, G(2)), op(4, D, 2, G(2))}, 3, op(-1, D, 4, G(3)));
      break;
    case 8:  // P8-GM.yml.cuh
      set({op(0, D, G(1), G(0)), op(1, I, G(0), G(1)), op(2, D, G(0), G(1))},
          {op(3, D, 1, G(2)), op(4, I, 2, G(2))}, 3, op(-1, D, 4, G(3)));
      break;
    case 9:  // P9-GM.yml.cuh
      set({op(0, I, G(0), G(1))}, {op(1, D, 0, G(2))}, 1, op(-1, I, 1, G(3), V(3)));
      break;
    case 10:  // P10-GM.yml.cuh
      set({op(0, D, G(0), G(1), V(1))}, {op(1, D, 0, G(2), V(2))}, 1, op(-1, D, 1, G(3), V(3)));
      break;
    case 11:  // P11-GM.yml.cuh
      set({op(0, D, G(1), G(0)), op(1, D, G(0), G(1))}, {op(2, D, 1, G(2)), op(3, I, 1, G(2))}, 2,
          op(-1, D, 3, G(3), V(1)));
      break;
    case 12:  // P12-GM.yml.cuh
      set({op(0, D, G(1), G(0), V(0)), op(1, D, G(0), G(1))}, {op(2, I, 1, G(2))}, 2,
          op(-1, D, 2, G(3)));
      break;
    case 13:  // P13-GM.yml.cuh
      set({op(0, I, G(0), G(1))}, {op(1, D, 0, G(2))}, 1, op(-1, D, 1, G(3)));
      break;
    case 14:  // P14-GM.yml.cuh
      set({op(0, I, G(0), G(1)), op(1, D, G(0), G(1))}, {op(2, I, 0, G(2), V(1)), op(3, D, 1, G(2))},
          2, op(-1, D, 3, G(3)));
      break;
    case 15:  // P15-GM.yml.cuh
      set({op(0, D, G(1), G(0)), op(1, D, G(0), G(1))}, {op(2, D, 1, G(2))}, 2,
          op(-1, D, 2, G(3), V(3)));
      break;
    case 16:  // P16-GM.yml.cuh
      set({op(0, D, G(1), G(0)), op(1, D, G(0), G(1)), op(2, I, G(0), G(1))},
          {op(3, D, 1, G(2)), op(4, I, 2, G(2))}, 3, op(-1, D, 4, G(3), V(1)));
      break;
    case 17:  // P17-GM.yml.cuh
      set({op(0, I, G(0), G(1)), op(1, D, G(0), G(1))}, {op(2, I, 1, G(2)), op(3, D, 0, G(2))}, 2,
          op(-1, D, 3, G(3)));
      break;
    case 18:  // P18-GM.yml.cuh
      set({op(0, I, G(0), G(1), V(1)), op(1, D, G(0), G(1))}, {op(2, D, 1, G(2))}, 2,
          op(-1, D, 2, G(3), V(3)));
      break;
    case 19:  // P19-GM.yml.cuh
      set({op(0, I, G(0), G(1), V(1)), op(1, D, G(0), G(1))},
          {op(2, I, 1, G(2), V(2)), op(3, D, 0, G(2))}, 2, op(-1, I, 3, G(3), V(3)));
      break;
    case 20:  // P20-GM.yml.cuh
      set({op(0, I, G(0), G(1)), op(1, D, G(0), G(1))}, {op(2, I, 1, G(2), V(1)), op(3, D, 1, G(2))},
          2, op(-1, D, 3, G(3)));
      break;
    case 21:  // P21-GM.yml.cuh
      set({op(0, D, G(1), G(0)), op(1, D, G(0), G(1))}, {op(2, D, 1, G(2))}, 2,
          op(-1, I, 2, G(3), V(3)));
      break;
    case 22:  // P22-GM.yml.cuh (its `v1 == v0` skip never fires on a loop-free CSR)
      set({op(0, I, G(0), G(1))}, {op(1, I, 0, G(2))}, 1, op(-1, D, 1, G(3)));
      break;
    default:
      return false;
  }
  *p = q;
  return true;
}

// Compiler.  Matching order: the vertex of highest degree, its highest-degree
// neighbour, then greedily the vertex with most matched neighbours (ties: degree,
// then index), so every vertex after the first edge touches a matched one.
// Symmetry breaking: stabiliser chain of the automorphism group in matching order
// (Grochow & Kellis, RECOMB 2007); for each vertex i the other members w of its
// orbit get x_w < x_i, which keeps exactly one image of every occurrence and only
// bounds later vertices by earlier ones.  Candidates of vertex t are the
// intersection of N(v_m) over matched neighbours m, minus N(v_m) over matched
// non-neighbours when vertex-induced, with matched non-neighbours excluded
// explicitly (a difference does not remove v_m itself).
bool prog_compile(int k, const uint8_t adj[8][8], bool induced, Prog* out, std::string* why) {
  if (k < 3 || k > kProgMaxK) return fail(why, "programs cover patterns of 3 to 6 vertices"), false;
  int deg[8] = {};
  for (int i = 0; i < k; ++i)
    for (int j = 0; j < k; ++j) {
      if ((adj[i][j] != 0) != (adj[j][i] != 0) || (i == j && adj[i][j]))
        return fail(why, "pattern adjacency is not symmetric and loop-free"), false;
      deg[i] += adj[i][j] ? 1 : 0;
    }
  int order[kProgMaxK];
  bool used[8] = {};
  order[0] = 0;
  for (int v = 1; v < k; ++v)
    if (deg[v] > deg[order[0]]) order[0] = v;
  used[order[0]] = true;
  for (int i = 1; i < k; ++i) {
    int best = -1, bc = 0;
    for (int v = 0; v < k; ++v) {
      if (used[v]) continue;
      int c = 0;
      for (int j = 0; j < i; ++j) c += adj[v][order[j]] ? 1 : 0;
      if (c == 0) continue;
      if (best < 0 || c > bc || (c == bc && deg[v] > deg[best])) best = v, bc = c;
    }
    if (best < 0) return fail(why, "pattern is not connected"), false;
    order[i] = best;
    used[best] = true;
  }
  uint8_t a[kProgMaxK][kProgMaxK];
  for (int i = 0; i < k; ++i)
    for (int j = 0; j < k; ++j) a[i][j] = adj[order[i]][order[j]] ? 1 : 0;

  // automorphisms of the relabelled pattern
  std::vector<std::vector<int>> H;
  std::vector<int> perm(k);
  for (int i = 0; i < k; ++i) perm[i] = i;
  do {
    bool ok = true;
    for (int i = 0; i < k && ok; ++i)
      for (int j = 0; j < k && ok; ++j) ok = a[perm[i]][perm[j]] == a[i][j];
    if (ok) H.push_back(perm);
  } while (std::next_permutation(perm.begin(), perm.end()));
  uint8_t bound[kProgMaxK] = {};
  for (int i = 0; i < k; ++i) {
    for (const auto& p : H)
      if (p[i] != i) {
        if (p[i] < i) return fail(why, "symmetry breaking failed"), false;
        bound[p[i]] |= V(i);
      }
    std::vector<std::vector<int>> keep;
    for (const auto& p : H)
      if (p[i] == i) keep.push_back(p);
    H.swap(keep);
  }

  Prog q;
  q.k = (int8_t)k;
  int state[kProgMaxK];
  uint8_t applied[kProgMaxK] = {};
  for (int t = 0; t < k; ++t) state[t] = -1;
  int nslots = 0;
  for (int l = 0; l <= k - 3; ++l) {
    const int last = l + 1;  // v_0 .. v_last are matched
    const uint8_t M = (uint8_t)((1u << (last + 1)) - 1);
    for (int t = l + 2; t < k; ++t) {
      const bool final = t == l + 2;
      if (state[t] < 0) {
        int root = -1;
        for (int m = 0; m <= last && root < 0; ++m)
          if (a[t][m]) root = m;
        if (root < 0) continue;
        state[t] = G(root);
        applied[t] = V(root);
      }
      std::vector<std::pair<int, int>> todo;  // (kind, m): intersections first
      for (int m = 0; m <= last; ++m)
        if (!(applied[t] & V(m)) && a[t][m]) todo.push_back({OP_INTERSECT, m});
      for (int m = 0; m <= last; ++m)
        if (!(applied[t] & V(m)) && !a[t][m] && induced) todo.push_back({OP_DIFFERENCE, m});
      applied[t] |= M;
      uint8_t ex = 0;
      for (int m = 0; m <= last; ++m)
        if (!a[t][m]) ex |= V(m);
      const uint8_t bnd = bound[t] & M;
      const bool counted = final && t == k - 1;
      auto emit = [&](int kind, int b) -> bool {
        if (q.nops[l] >= kProgMaxOps || nslots >= kProgMaxSlots) return false;
        q.ops[l][q.nops[l]++] = op(nslots, kind, state[t], b, bnd, ex);
        state[t] = nslots++;
        return true;
      };
      const size_t n_ops = counted ? (todo.empty() ? 0 : todo.size() - 1) : todo.size();
      for (size_t i = 0; i < n_ops; ++i)
        if (!emit(todo[i].first, G(todo[i].second))) return fail(why, "program too large"), false;
      if (counted) {
        q.fin = todo.empty() ? op(-1, OP_FILTER, state[t], 0, bnd, ex)
                             : op(-1, todo.back().first, state[t], G(todo.back().second), bnd, ex);
      } else if (final) {
        if (todo.empty() && (bnd | ex))
          if (!emit(OP_FILTER, 0)) return fail(why, "program too large"), false;
        q.cand[t] = (int8_t)state[t];
      }
    }
  }
  q.nslots = (int8_t)nslots;
  q.v1lt = (bound[1] & V(0)) ? 1 : 0;  // the only condition v1 can carry
  q.flat = (k >= 4 && q.nops[k - 3] == 0 && q.fin.a != G(k - 2)) ? 1 : 0;
  std::string w;
  if (!prog_check(q, &w)) return fail(why, ("compiled program is inconsistent: " + w).c_str()), false;
  *out = q;
  return true;
}

// GLUMIN's LUT kernels (GM_LUT_kernels/P*.yml.cuh with codegen_LUT.cuh) run the
// same plans on a bitmap of the adjacency among N(v0); this decides whether a program
// has that shape.
bool prog_lut(const Prog& p, ProgLut* out) {
  ProgLut r;
  if (p.k < 4 || p.k > 5 || p.nslots > kLutSlots) return *out = r, false;
  // space of each slot: 1 = subset of N(v0) (bitmap), 2 = the N(v1) \ N(v0) stream
  int8_t space[kProgMaxSlots] = {};
  auto n0 = [&](int code) { return code == G(0) || (code < kOpList && space[code] == 1); };
  for (int i = 0; i < p.nops[0]; ++i) {
    const ProgOp& o = p.ops[0][i];
    if (n0(o.a) || (o.a == G(1) && o.b == G(0) && o.kind == OP_INTERSECT)) {
      space[o.out] = 1;
    } else if (o.a == G(1) && o.b == G(0) && o.kind == OP_DIFFERENCE && o.out == p.cand[2] &&
               r.stream < 0) {
      space[o.out] = 2;
      r.stream = (int8_t)i;
    } else {
      return *out = ProgLut{}, false;
    }
  }
  // the stream feeds the v2 loop only
  auto uses = [&](int code) {
    for (int l = 1; l < kProgLevels; ++l)
      for (int i = 0; i < p.nops[l]; ++i)
        if (p.ops[l][i].a == code) return true;
    return p.fin.a == code || (p.k == 5 && p.cand[3] == code);
  };
  if (r.stream >= 0 && uses(p.ops[0][r.stream].out)) return *out = ProgLut{}, false;
  if (!(n0(p.cand[2]) || (p.cand[2] < kOpList && space[p.cand[2]] == 2)))
    return *out = ProgLut{}, false;
  for (int l = 1; l <= p.k - 3; ++l)
    for (int i = 0; i < p.nops[l]; ++i) {
      const ProgOp& o = p.ops[l][i];
      if (!n0(o.a)) return *out = ProgLut{}, false;
      space[o.out] = 1;
    }
  if (p.k == 5 && !n0(p.cand[3])) return *out = ProgLut{}, false;
  if (!n0(p.fin.a)) return *out = ProgLut{}, false;
  r.ok = 1;
  *out = r;
  return true;
}

bool prog_check(const Prog& p, std::string* why) {
  if (p.k < 3 || p.k > kProgMaxK) return fail(why, "k out of range"), false;
  if (p.nslots < 0 || p.nslots > kProgMaxSlots) return fail(why, "slot count out of range"), false;
  if (p.v1lt != 0 && p.v1lt != 1) return fail(why, "v1lt is a flag"), false;
  bool defined[kProgMaxSlots] = {};
  auto operand_ok = [&](int code, int last, bool list_only) {
    if (code >= kOpList) return code - kOpList <= last;
    return !list_only && code >= 0 && code < p.nslots && defined[code];
  };
  auto op_ok = [&](const ProgOp& o, int last, bool counted) {
    if (o.kind < OP_INTERSECT || o.kind > OP_FILTER) return false;
    if (!operand_ok(o.a, last, false)) return false;
    if (o.kind != OP_FILTER && !operand_ok(o.b, last, true)) return false;
    const unsigned matched = (1u << (last + 1)) - 1;
    if ((o.bound & ~matched) || (o.excl & ~matched)) return false;
    if (!counted && (o.out < 0 || o.out >= p.nslots || defined[o.out])) return false;
    return true;
  };
  for (int l = 0; l <= p.k - 3; ++l) {
    if (p.nops[l] < 0 || p.nops[l] > kProgMaxOps) return fail(why, "op count out of range"), false;
    for (int i = 0; i < p.nops[l]; ++i) {
      if (!op_ok(p.ops[l][i], l + 1, false)) return fail(why, "malformed operation"), false;
      defined[p.ops[l][i].out] = true;
    }
    if (l < p.k - 3 && !operand_ok(p.cand[l + 2], l + 1, false))
      return fail(why, "candidate operand undefined"), false;
  }
  for (int l = p.k - 2; l < kProgLevels; ++l)
    if (p.nops[l] != 0) return fail(why, "operations beyond the last level"), false;
  if (!op_ok(p.fin, p.k - 2, true)) return fail(why, "malformed final count"), false;
  if (p.flat && (p.k < 4 || p.nops[p.k - 3] != 0 || p.fin.a == G(p.k - 2)))
    return fail(why, "flat count not applicable"), false;
  return true;
}

void prog_to_words(const Prog& p, int32_t* w) {
  std::memset(w, 0, sizeof(int32_t) * kProgWords);
  w[0] = kProgVersion;
  w[1] = p.k;
  w[2] = p.nslots;
  w[3] = p.flat;
  w[4] = p.v1lt;
  for (int l = 0; l < kProgLevels; ++l) w[5 + l] = p.nops[l];
  for (int i = 2; i < kProgMaxK - 1; ++i) w[9 + i - 2] = p.cand[i];
  int32_t* o = w + kProgHeader;
  auto put = [&](const ProgOp& x) {
    o[0] = x.out, o[1] = x.kind, o[2] = x.a, o[3] = x.b, o[4] = x.bound, o[5] = x.excl;
    o += 6;
  };
  for (int l = 0; l < kProgLevels; ++l)
    for (int i = 0; i < kProgMaxOps; ++i) put(p.ops[l][i]);
  put(p.fin);
}

bool prog_from_words(const int32_t* w, int n, Prog* p, std::string* why) {
  if (n < kProgWords || w[0] != kProgVersion) return fail(why, "not a program (version word)"), false;
  Prog q;
  q.k = (int8_t)w[1];
  q.nslots = (int8_t)w[2];
  q.flat = (int8_t)w[3];
  q.v1lt = (int8_t)w[4];
  for (int l = 0; l < kProgLevels; ++l) q.nops[l] = (int8_t)w[5 + l];
  for (int i = 2; i < kProgMaxK - 1; ++i) q.cand[i] = (int8_t)w[9 + i - 2];
  const int32_t* o = w + kProgHeader;
  auto get = [&](ProgOp& x) {
    x = op(o[0], o[1], o[2], o[3], o[4], o[5]);
    o += 6;
  };
  for (int l = 0; l < kProgLevels; ++l)
    for (int i = 0; i < kProgMaxOps; ++i) get(q.ops[l][i]);
  get(q.fin);
  if (!prog_check(q, why)) return false;
  *p = q;
  return true;
}

}  // namespace xgm
