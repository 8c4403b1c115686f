// xgm_count_cli — command-line front end over the C ABI (include/xgm.h) with the
// flags of xgminer's own binary (xgminer/main.cpp:19-60, include/cmd_option.h:30-159):
//
//   xgm_count_cli --graph <prefix> --algorithm glumin_g2miner --patternID 20
//   xgm_count_cli --graph <prefix> --pattern-name diamond --vert-induced 1
//   xgm_count_cli --graph <prefix> --pattern-size 3 --pattern-adj-mat 011101110
//
// <prefix> names the reference's binary graph files (<prefix>.meta.txt / .vertex.bin /
// .edge.bin).  --patternID follows xgminer's numbering (include/common.h:185-208 and
// glumin.h:34-39): 1 triangle, 2 rectangle, 3 diamond, and the GraphPi shapes of
// src/pattern_graphpi.cpp:60-146 by their names there — 10 QG3 (K4 minus an edge),
// 11 pentagon, 13 house, 14 hourglass (two triangles joined by a perfect matching),
// 15 Cycle_6_Tri — counted edge-induced as GraphPi does unless --vert-induced; 17..40
// GLUMIN P1..P24 (patternID - 16).  Every GPU algorithm name of
// xgminer selects this engine (it picks its own kernels per task); cpu_baseline is the
// reference's CPU path and is not part of this engine.  Prints the count the way the
// reference's solvers do ("Pattern P<k> count: N") and the device time.
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>

#include "xgm.h"

namespace {

struct Options {
  std::string graph, algorithm = "glumin_g2miner", pattern_name, adj;
  int pattern_id = 0, pattern_size = 0, induced = 0, repeat = 1, device = 0;
  bool help = false;
};

void usage(const char* prog) {
  std::printf(
      "usage: %s --graph <prefix> [--algorithm <name>] (--patternID N | --pattern-name <name> |\n"
      "          --pattern-size K --pattern-adj-mat <K*K 0/1 digits>) [--vert-induced 0|1]\n"
      "          [--repeat N] [--device D]\n"
      "  algorithms: glumin_g2miner, glumin_g2miner_lut, glumin_gf, glumin_gf_lut,\n"
      "              glumin_automine, glumin_automine_lut, glumin_cliques, glumin_cliques_lut,\n"
      "              bitmap_bigset_opt (all run this engine)\n"
      "  patternID:  1 triangle, 2 rectangle, 3 diamond, 10 QG3, 11 pentagon, 13 house,\n"
      "              14 hourglass, 15 Cycle_6_Tri, 17..40 GLUMIN P1..P24\n",
      prog);
}

bool parse(int argc, char** argv, Options* o) {
  for (int i = 1; i < argc; ++i) {
    const std::string a = argv[i];
    auto val = [&](const char* name) -> const char* {
      if (i + 1 >= argc) {
        std::fprintf(stderr, "missing value for %s\n", name);
        std::exit(2);
      }
      return argv[++i];
    };
    if (a == "-h" || a == "--help") o->help = true;
    else if (a == "-g" || a == "--graph") o->graph = val("--graph");
    else if (a == "--algorithm") o->algorithm = val("--algorithm");
    else if (a == "--patternID") o->pattern_id = std::atoi(val("--patternID"));
    else if (a == "--pattern-name") o->pattern_name = val("--pattern-name");
    else if (a == "--pattern-adj-mat") o->adj = val("--pattern-adj-mat");
    else if (a == "--pattern-size") o->pattern_size = std::atoi(val("--pattern-size"));
    else if (a == "--vert-induced") o->induced = std::atoi(val("--vert-induced"));
    else if (a == "--repeat") o->repeat = std::atoi(val("--repeat"));
    else if (a == "--device") o->device = std::atoi(val("--device"));
    else if (a == "-d" || a == "--dataname" || a == "--run-xgminer" || a == "--do-validation")
      (void)val(a.c_str());  // accepted for compatibility; no effect here
    else {
      std::fprintf(stderr, "unknown option %s\n", a.c_str());
      return false;
    }
  }
  return true;
}

bool known_algorithm(const std::string& a) {
  static const char* kGpu[] = {"glumin_g2miner",   "glumin_g2miner_lut", "glumin_gf",
                               "glumin_gf_lut",    "glumin_automine",    "glumin_automine_lut",
                               "glumin_cliques",   "glumin_cliques_lut", "bitmap_bigset_opt"};
  for (const char* k : kGpu)
    if (a == k) return true;
  return false;
}

// xgminer pattern id -> plan name (edge-induced unless --vert-induced for the count-app
// shapes; GLUMIN P ids carry their own convention)
const char* id_name(int id) {
  static char buf[8];
  switch (id) {
    case 1: return "triangle";
    case 2: return "rectangle";
    case 3: return "diamond";
    case 10: return "diamond";  // GraphPi QG3: edges 01 02 03 12 13
    case 11: return "5-cycle";  // GraphPi Pentagon
    case 13: return "5-house";  // GraphPi House
    default: break;
  }
  if (id >= 17 && id <= 40) {
    std::snprintf(buf, sizeof(buf), "P%d", id - 16);
    return buf;
  }
  return nullptr;
}

// The 6-vertex GraphPi shapes (src/pattern_graphpi.cpp:104-132) as adjacency strings.
const char* id_adj(int id) {
  switch (id) {
    case 14:  // Hourglass: 01 02 04 12 15 23 34 35 45
      return "011010"
             "101001"
             "110100"
             "001011"
             "100101"
             "010110";
    case 15:  // Cycle_6_Tri: 01 02 12 13 14 23 25 04 05
      return "011011"
             "101110"
             "110101"
             "011000"
             "110000"
             "101000";
    default:
      return nullptr;
  }
}

int fail(xgm_ctx* ctx, xgm_status st, const char* what) {
  const char* msg = xgm_last_error(ctx);
  std::fprintf(stderr, "%s: %s (%s)\n", what, xgm_status_string(st), msg ? msg : "");
  return 1;
}

}  // namespace

int main(int argc, char** argv) {
  Options o;
  if (!parse(argc, argv, &o) || o.help) {
    usage(argv[0]);
    return o.help ? 0 : 2;
  }
  if (o.algorithm == "cpu_baseline") {
    std::fprintf(stderr, "cpu_baseline is the reference's CPU path; this engine runs on the GPU\n");
    return 2;
  }
  if (!known_algorithm(o.algorithm)) {
    std::fprintf(stderr, "Unsupported algorithm: %s\n", o.algorithm.c_str());
    return 2;
  }
  if (o.graph.empty()) {
    usage(argv[0]);
    return 2;
  }
  if (o.adj.empty() && o.pattern_size == 0 && o.pattern_name.empty() && id_adj(o.pattern_id)) {
    o.adj = id_adj(o.pattern_id);
    o.pattern_size = 6;
  }
  const bool by_adj = !o.adj.empty() || o.pattern_size > 0;
  if (!by_adj && o.pattern_name.empty() && !id_name(o.pattern_id)) {
    std::fprintf(stderr, "patternID %d is not a supported plan\n", o.pattern_id);
    return 2;
  }
  xgm_config cfg{o.device, 0};
  xgm_ctx* ctx = nullptr;
  xgm_status st = xgm_create(&ctx, &cfg);
  if (st != XGM_OK) return fail(nullptr, st, "xgm_create");
  int rc = 0;
  xgm_graph* g = nullptr;
  xgm_plan* plan = nullptr;
  std::string label;
  do {
    st = xgm_graph_load(ctx, o.graph.c_str(), 0, &g);
    if (st != XGM_OK) {
      rc = fail(ctx, st, "xgm_graph_load");
      break;
    }
    if (by_adj) {
      const int k = o.pattern_size;
      if (k < 2 || k > 8 || (int)o.adj.size() != k * k) {
        std::fprintf(stderr, "--pattern-adj-mat needs --pattern-size K and K*K digits\n");
        rc = 2;
        break;
      }
      xgm_plan_desc d;
      std::memset(&d, 0, sizeof(d));
      d.num_vertices = k;
      d.induced = o.induced;
      for (int i = 0; i < k; ++i)
        for (int j = 0; j < k; ++j) d.adj[i][j] = o.adj[i * k + j] == '1' ? 1 : 0;
      st = xgm_plan_compile(ctx, &d, &plan);
      label = "pattern " + o.adj;
    } else {
      std::string name = o.pattern_name;
      if (name.empty()) name = id_name(o.pattern_id);
      const bool glumin_id = name.size() > 1 && name[0] == 'P' && name[1] >= '0' && name[1] <= '9';
      if (o.induced && !glumin_id) {
        // the count-app and .yml names are edge-induced: rebuild as vertex-induced
        xgm_plan* by_name = nullptr;
        st = xgm_plan_from_name(ctx, name.c_str(), &by_name);
        if (st == XGM_OK) {
          xgm_plan_desc d;
          std::memset(&d, 0, sizeof(d));
          d.builtin = xgm_plan_pattern(by_name);
          d.induced = 1;
          if (d.builtin == XGM_PATTERN_PROGRAM) {
            std::fprintf(stderr, "--vert-induced with a 5-vertex name: use --pattern-adj-mat\n");
            xgm_plan_destroy(by_name);
            rc = 2;
            break;
          }
          st = xgm_plan_compile(ctx, &d, &plan);
          xgm_plan_destroy(by_name);
        }
      } else {
        st = xgm_plan_from_name(ctx, name.c_str(), &plan);
      }
      label = glumin_id ? "Pattern " + name : name;
    }
    if (st != XGM_OK) {
      rc = fail(ctx, st, "plan");
      break;
    }
    xgm_graph_info info;
    xgm_graph_info_get(g, &info);
    std::printf("graph %s: |V| %lld, |E| %lld, max degree %lld\n", o.graph.c_str(),
                (long long)info.num_vertices, (long long)info.num_edges,
                (long long)info.max_degree);
    uint64_t count = 0;
    xgm_stats stats;
    double best = 0;
    for (int r = 0; r < (o.repeat > 0 ? o.repeat : 1); ++r) {
      st = xgm_count(ctx, g, plan, nullptr, &count, &stats);
      if (st != XGM_OK) break;
      const double ms = stats.kernel_ms + stats.prep_ms;
      if (r == 0 || ms < best) best = ms;
    }
    if (st != XGM_OK) {
      rc = fail(ctx, st, "xgm_count");
      break;
    }
    std::printf("%s count: %llu\n", label.c_str(), (unsigned long long)count);
    std::printf("runtime [gpu] = %.6f sec\n", best / 1e3);
  } while (false);
  if (plan) xgm_plan_destroy(plan);
  if (g) xgm_graph_destroy(g);
  xgm_destroy(ctx);
  return rc;
}
