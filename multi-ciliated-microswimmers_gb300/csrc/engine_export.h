// Host copy of everything a single-box engine holds, for moving a box into a
// replica batch (mpcd_batch_add_engine).
#pragma once
#include <vector>

#include "../../include/mpcd_gpu.h"

namespace mpcd {

struct EngineExport {
  mpcd_params p{};
  double a[3] = {0.5, 0.5, 0.5};
  double globalt = 0.0;
  long long steps = 0;
  long nf = 0;
  std::vector<double> fpos, fvel;
  long nb = 0;
  std::vector<double> bpos, bvel;
  std::vector<int> bmoves;
  std::vector<int> sp_t, sp_o, sp_k, sp_r;
  std::vector<double> sp_rest, sp_kk;
  std::vector<mpcd_cilium> cil;
  std::vector<double> newlen, oldlen;
};

// 0 on success (MPCD_* code otherwise; the engine's last error says why)
int engine_export(mpcd_engine* h, EngineExport& out);

}  // namespace mpcd
