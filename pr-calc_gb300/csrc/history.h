// history.h — constants and the skewer plan of the history-correction chain
// (allvars_d2z.h:1-17 of pr-calc), shared by history.cpp and d2z_capi.cu.
#pragma once
#include <vector>

#include "../../include/prc_d2z.h"

#define HISTORY_INITIAL 49.9
#define HISTORY_FINAL 0.01
#define CHISTORY_INITIAL 49.9
#define CHISTORY_FINAL 0.01
#define X_MFP_INITIAL 0.01
#define X_MFP_FINAL 0.999
#define NMFP PRC_NMFP
#define MFP_INITIAL_CELL 1
#define MFP_FINAL_BOX 1.0

namespace prc_hist {

// Skewer starts, fractions and grid constants of GetBubbleMFP for one zreion grid.
struct MfpPlan {
  int N = 0, nx = 0, ns = 0;
  float box = 0, cell = 0, mfp_initial = 0, mfp_final = 0, dmfp = 0, dxmfp = 0;
  std::vector<float> zcur;   // per x value
  std::vector<int> start;    // (i, j, k) per skewer, x-major
  std::vector<float> frac;   // (y, z) per skewer
};

int mfp_plan(const prc_mfp_setup* s, const float* zreion_host, const float* history, MfpPlan* plan);
void mfp_finish(const MfpPlan& p, const int* steps, float* mfp, float* mfp_x, float* dfdmfp);

}  // namespace prc_hist
