// Set-operation programs: pattern plans written as chains of sorted-list
// intersections and differences over the undirected CSR, run by one interpreter
// kernel (setprog.cu).
//
// GLUMIN generates one kernel per pattern from a plan of this shape
// (codes/GLUMIN/codegen/codegen/codegen.py:901-933; the generated bodies are
// G2Miner/gpu_GM_LUT_kernels/GM_kernels/P*-GM.yml.cuh): every directed edge (v0, v1)
// of the CSR is a task; slots are filled from N(v0) and N(v1); v2 runs over one slot
// and further slots are refined with N(v2); v3 runs over another, and the last vertex
// is counted, not enumerated (__intersect_num / __difference_num,
// codegen/include/gpu_kernels/codegen_utils.cuh:256-300).  A bound keeps only
// elements below a matched vertex's id (set_difference.cuh:44-86, 176-232).
//
// Here a plan is data, not code: the programs for GLUMIN's P6-P22 are tables
// (setprog.cpp), and a compiler turns any other connected pattern of up to six
// vertices into a program with exact symmetry breaking and explicit exclusion of the
// vertices already matched.
#pragma once
#include <stdint.h>

#include <string>

namespace xgm {

constexpr int kProgMaxK = 6;
constexpr int kProgLevels = kProgMaxK - 2;  // level l runs after v_{l+1} is matched
constexpr int kProgMaxOps = 6;              // per level
constexpr int kProgMaxSlots = 16;
constexpr int kOpList = 16;                 // operand kOpList + j: N(v_j); below: a slot

enum ProgOpKind : int8_t { OP_INTERSECT = 0, OP_DIFFERENCE = 1, OP_FILTER = 2 };

// out = { x in a : x < min(v_j : bound bit j), x != v_j for excl bit j, and
//         (x in b) for INTERSECT, (x not in b) for DIFFERENCE; b unused by FILTER }.
// a and b are sorted; out keeps a's order.
struct ProgOp {
  int8_t out;    // slot written (the final count writes none)
  int8_t kind;   // ProgOpKind
  int8_t a;      // slot or kOpList + j
  int8_t b;      // kOpList + j
  uint8_t bound;
  uint8_t excl;
};

struct Prog {
  int8_t k = 0;                  // pattern vertices, 3..6
  int8_t nslots = 0;
  int8_t flat = 0;               // last vertex loop merged with the final count
  int8_t v1lt = 0;               // tasks keep v1 < v0 only (v0, v1 interchangeable)
  int8_t nops[kProgLevels] = {};
  int8_t cand[kProgMaxK] = {};   // cand[i], 2 <= i <= k-2: operand v_i runs over
  ProgOp ops[kProgLevels][kProgMaxOps] = {};
  ProgOp fin = {};               // counted at level k-3
};

// Flat word form shared with the C-ABI (xgm_plan_program) and the oracle:
// [2 (format version), k, nslots, flat, v1lt, nops[0..3], cand[2..4], then
// 4 x kProgMaxOps ops and fin, six words each: out, kind, a, b, bound, excl].
constexpr int kProgVersion = 2;
constexpr int kProgHeader = 12;
constexpr int kProgWords = kProgHeader + (kProgLevels * kProgMaxOps + 1) * 6;
void prog_to_words(const Prog& p, int32_t* w);
bool prog_from_words(const int32_t* w, int n, Prog* p, std::string* why);
// Operands defined before use, slots in range, bounds and exclusions only on matched
// vertices.
bool prog_check(const Prog& p, std::string* why);

// Bitmap (LUT) form: whether the program runs in the index space of N(v0) — every
// operand read after level 0, the v3 candidates and the counted operand descend from
// N(v0); the v2 candidates may instead be the stream N(v1) \ N(v0) (one level-0
// difference, `stream`), whose vertices get their rows built on the fly.  The bitmap
// kernels hold kLutSlots slots per task (4- and 5-vertex programs use at most 5).
constexpr int kLutSlots = 8;
struct ProgLut {
  int8_t ok = 0;
  int8_t stream = -1;  // index of the level-0 operation giving cand[2] from N(v1), or -1
};
bool prog_lut(const Prog& p, ProgLut* out);

// GLUMIN's P6..P22 (vertex-induced 5-vertex plans), exactly as generated.
bool prog_glumin(int pid, Prog* p);
// A program counting each occurrence of the pattern (k <= 6 vertices, symmetric 0/1
// adjacency, connected) once: vertex-induced or edge-induced.
bool prog_compile(int k, const uint8_t adj[8][8], bool induced, Prog* p, std::string* why);

}  // namespace xgm
