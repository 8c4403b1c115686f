// Host file I/O in the reference's binary CSR layout (io.cpp).
#pragma once
#include <stdint.h>

#include <string>
#include <vector>

#include "../../include/xgm.h"

namespace xgm {
xgm_status read_graph_files(const std::string& prefix, std::vector<int64_t>& rowptr,
                            std::vector<int32_t>& col, std::string& msg);
}  // namespace xgm
