// Host file I/O in the reference's binary CSR layout.
//
// <prefix>.meta.txt : V, E, "4 8 1 2" (sizeof vid, eid, vlabel, elabel), max degree,
//                     feature length, #vertex classes, #edge classes
// <prefix>.vertex.bin: int64[V+1] row pointers
// <prefix>.edge.bin  : int32[E] column indices
// Reader: xgminer/src/graph_v2.cpp:5-134 / codes/GraphMiner/src/common/graph.cc:4-45;
// writer: scripts/graph_format_conversion.py:47-80.
#include <cstdio>
#include <fstream>
#include <string>
#include <vector>

#include "io.h"

namespace xgm {

xgm_status read_graph_files(const std::string& prefix, std::vector<int64_t>& rowptr,
                            std::vector<int32_t>& col, std::string& msg) {
  std::ifstream meta(prefix + ".meta.txt");
  if (!meta) {
    msg = "cannot open " + prefix + ".meta.txt";
    return XGM_ERR_IO;
  }
  int64_t nv = 0, ne = 0;
  int vid = 0, eid = 0, vl = 0, el = 0;
  int64_t maxd = 0;
  meta >> nv >> ne >> vid >> eid >> vl >> el >> maxd;
  if (!meta || nv <= 0 || ne < 0 || vid != 4 || eid != 8) {
    msg = "malformed meta file " + prefix + ".meta.txt (expects V E 4 8 ...)";
    return XGM_ERR_IO;
  }
  rowptr.resize(size_t(nv) + 1);
  col.resize(size_t(ne));
  FILE* fv = std::fopen((prefix + ".vertex.bin").c_str(), "rb");
  FILE* fe = std::fopen((prefix + ".edge.bin").c_str(), "rb");
  bool ok = fv && fe;
  if (ok) ok = std::fread(rowptr.data(), sizeof(int64_t), rowptr.size(), fv) == rowptr.size();
  if (ok && ne > 0) ok = std::fread(col.data(), sizeof(int32_t), col.size(), fe) == col.size();
  if (fv) std::fclose(fv);
  if (fe) std::fclose(fe);
  if (!ok) {
    msg = "cannot read " + prefix + ".vertex.bin / .edge.bin";
    return XGM_ERR_IO;
  }
  if (rowptr[0] != 0 || rowptr[size_t(nv)] != ne) {
    msg = "row pointers of " + prefix + " do not span the edge file";
    return XGM_ERR_GRAPH;
  }
  return XGM_OK;
}

}  // namespace xgm

extern "C" xgm_status xgm_graph_write_files(const char* prefix, const xgm_csr_host* csr) {
  if (!prefix || !csr || csr->num_vertices <= 0 || !csr->rowptr ||
      (csr->num_edges > 0 && !csr->colidx))
    return XGM_ERR_INVALID;
  const std::string p(prefix);
  int64_t maxd = 0;
  for (int64_t v = 0; v < csr->num_vertices; ++v) {
    int64_t d = csr->rowptr[v + 1] - csr->rowptr[v];
    if (d > maxd) maxd = d;
  }
  std::ofstream meta(p + ".meta.txt");
  if (!meta) return XGM_ERR_IO;
  meta << csr->num_vertices << "\n" << csr->num_edges << "\n4 8 1 2\n" << maxd << "\n0\n0\n0\n";
  meta.close();
  FILE* fv = std::fopen((p + ".vertex.bin").c_str(), "wb");
  FILE* fe = std::fopen((p + ".edge.bin").c_str(), "wb");
  bool ok = fv && fe;
  if (ok)
    ok = std::fwrite(csr->rowptr, sizeof(int64_t), size_t(csr->num_vertices) + 1, fv) ==
         size_t(csr->num_vertices) + 1;
  if (ok && csr->num_edges > 0)
    ok = std::fwrite(csr->colidx, sizeof(int32_t), size_t(csr->num_edges), fe) ==
         size_t(csr->num_edges);
  if (fv) std::fclose(fv);
  if (fe) std::fclose(fe);
  return ok ? XGM_OK : XGM_ERR_IO;
}
