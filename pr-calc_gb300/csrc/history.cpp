// history.cpp — host side of the reionization-history correction chain of
// pr-calc's delta2zreion (the steps after the hot loop, main_d2z.C:76-101):
//
//   prc_f2f_*            Float2FloatTable            tables.C:9-38
//   prc_fcoll / deltac   PS collapsed fraction        cosmology.C:141-172,311-324
//   prc_mfp_*            GetBubbleMFP                 bubblehistory_d2z.C:82-252
//   prc_chistory         GetCHistory + BubbleMFP      bubblehistory_d2z.C:45-80,254-276
//   prc_zvz              CorrectHistory's z -> z map  bubblehistory_d2z.C:278-326
//
// float/double conversions follow the reference operation by operation
// (compile with -ffp-contract=off).  The skewer starts use glibc's random_r
// with the state rand() has when nothing seeded it (srand(1)), so at one rank
// the sequence of accepted cells and fractions is the reference's; the walks
// themselves run on the GPU (prc_d2z_bubble_mfp in d2z_capi.cu).
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <vector>

#include "../../include/prc_d2z.h"
#include "errors.h"
#include "history.h"

extern "C" {

// ---------------------------------------------------------------- tables.C:9-38
int prc_f2f_load(const char* path, prc_f2f_table* t) {
  if (!path || !t) return prc_fail(PRC_ERR_INVALID, "prc_f2f_load: null argument");
  memset(t, 0, sizeof(*t));
  FILE* fd = fopen(path, "rb");
  if (!fd) return prc_fail(PRC_ERR_IO, "prc_f2f_load: cannot open %s", path);
  float mn, mx;
  int n;
  if (fread(&mn, 4, 1, fd) != 1 || fread(&mx, 4, 1, fd) != 1 || fread(&n, 4, 1, fd) != 1 || n < 2 ||
      n > (1 << 26)) {
    fclose(fd);
    return prc_fail(PRC_ERR_IO, "prc_f2f_load: bad header in %s", path);
  }
  float* tab = (float*)malloc(sizeof(float) * (size_t)n);
  if (!tab || fread(tab, 4, (size_t)n, fd) != (size_t)n) {
    free(tab);
    fclose(fd);
    return prc_fail(PRC_ERR_IO, "prc_f2f_load: short table in %s", path);
  }
  fclose(fd);
  t->minval = mn;
  t->maxval = mx;
  t->n = n;
  t->delta = (mx - mn) / n;  // tables.C:17 (spacing (max-min)/n, as the reference reads it)
  t->table = tab;
  return PRC_OK;
}

float prc_f2f_eval(const prc_f2f_table* t, float inval) {
  if (inval <= t->minval) return t->table[0];
  if (inval >= t->maxval) return t->table[t->n - 1];
  const int bin = int((inval - t->minval) / t->delta);
  if (bin >= t->n - 1) return t->table[t->n - 1];  // the reference would read table[n] here
  const float f = (inval - (t->minval + bin * t->delta)) / t->delta;
  return (1 - f) * t->table[bin] + f * t->table[bin + 1];
}

void prc_f2f_free(prc_f2f_table* t) {
  if (!t) return;
  free(t->table);
  t->table = nullptr;
  t->n = 0;
}

// ---------------------------------------------------------------- cosmology.C:141-172
float prc_deltac(float z, float omegam, float omegal, float w, float* dcoll) {
  const float pi = 3.14159265358979f;
  const float x = 1 + z;
  const float x2 = x * x;
  const float x3 = x * x * x;
  const float omega = omegam * x3 / (omegam * x3 + (1 - omegam - omegal) * x2 + omegal);
  // pow with an integer exponent is the double function (C++ overload rules)
  const float a = 2 / omega - 1;
  const float eta = (float)log((double)a + sqrt(pow((double)a, 2) - 1));
  float dc, dcl;
  if ((omegam < 1) && (omegal == 0)) {
    const float sh = sinhf(eta), ch = coshf(eta);
    dc = (float)(1.5 * ((double)(3 * sh * (sh - eta)) / pow((double)(ch - 1), 2) - 2) *
                 (1 + pow((double)(2 * pi / (sh - eta)), 2. / 3.)));
    dcl = (float)((double)(4 * pi * pi) * pow((double)(ch - 1), 3) / pow((double)(sh - eta), 2));
  } else {
    dc = (float)(3 * pow((12 * pi), 2. / 3.) / 20 * (1 + 0.0123 * (double)log10f(omega)));
    dcl = (float)(18 * pi * pi * (1 + 0.4093 * pow((1 / omega - 1), 0.9052)));
  }
  if (dcoll) *dcoll = dcl;
  dc /= prc_growth(z, omegam, omegal, w);
  return dc;
}

// cosmology.C:311-324
float prc_fcoll(float z, float zInit, float omegam, float omegal, float w, float sigma_min) {
  (void)zInit;
  float dcoll;
  const float arg = (float)((double)prc_deltac(z, omegam, omegal, w, &dcoll) / sqrt(2.) / (double)sigma_min);
  return erfcf(arg);
}

}  // extern "C"

// ---------------------------------------------------------------- GetBubbleMFP
namespace prc_hist {

int mfp_plan(const prc_mfp_setup* s, const float* zreion_host, const float* history, MfpPlan* plan) {
  const int N = s->N;
  const int NX = s->n_x, NS = s->n_skewers;
  if (N < 3 || NX < 2 || NS < 1) return prc_fail(PRC_ERR_INVALID, "bubble mfp: bad sizes");
  plan->N = N;
  plan->nx = NX;
  plan->ns = NS;
  plan->box = s->box_mpc;
  plan->cell = s->box_mpc / N;                                   // :97
  plan->mfp_final = (float)log(MFP_FINAL_BOX * (double)s->box_mpc);  // :99
  plan->mfp_initial = logf(MFP_INITIAL_CELL * plan->cell);        // :100
  plan->dmfp = (plan->mfp_final - plan->mfp_initial) / (NMFP);     // :102
  plan->dxmfp = (float)((X_MFP_FINAL - X_MFP_INITIAL) / (NX - 1));  // :103
  const float dzh = (float)((HISTORY_FINAL - HISTORY_INITIAL) / (PRC_NHISTORY - 1));
  plan->zcur.assign(NX, 0.f);
  plan->start.assign((size_t)NX * NS * 3, 0);
  plan->frac.assign((size_t)NX * NS * 2, 0.f);
  // unseeded rand(): glibc's generator in the state srand(1) leaves
  char state[128];
  random_data rd;
  memset(&rd, 0, sizeof(rd));
  if (initstate_r(1, state, sizeof(state), &rd) != 0) return prc_fail(PRC_ERR_NUMERIC, "bubble mfp: initstate_r");
  auto draw = [&]() {
    int32_t r;
    random_r(&rd, &r);
    return (float)r / RAND_MAX;
  };
  float zcur = 0.f;
  for (int ix = 0; ix < NX; ix++) {
    const float xcur = (float)(X_MFP_INITIAL + ix * plan->dxmfp);
    // :113-124 redshift of this ionised fraction (zcur keeps its value on an exact tie)
    if (xcur < history[0]) {
      zcur = (float)HISTORY_INITIAL;
    } else if (xcur > history[PRC_NHISTORY - 1]) {
      zcur = (float)HISTORY_FINAL;
    } else {
      for (int i = 0; i < PRC_NHISTORY - 1; i++)
        if (xcur > history[i] && xcur < history[i + 1]) {
          const float fint = (xcur - history[i]) / (history[i + 1] - history[i]);
          zcur = (float)((1 - fint) * (HISTORY_INITIAL + i * dzh) + fint * (HISTORY_INITIAL + (i + 1) * dzh));
          break;
        }
    }
    plan->zcur[ix] = zcur;
    // is any cell above zcur with j, k < N-2?  (otherwise the reference never stops drawing)
    for (int is = 0; is < NS; is++) {
      int istart = 0, jstart = 0, kstart = 0;
      long long tries = 0;
      for (;;) {
        const float sx = draw(), sy = draw(), sz = draw();
        istart = (int)(sx * (float)N);
        jstart = (int)(sy * N);
        kstart = (int)(sz * N);
        if (istart >= N) istart -= N;
        if (jstart >= N) jstart -= N;
        if (kstart >= N) kstart -= N;
        const long long idx = ((long long)istart * N + jstart) * N + kstart;
        if (zreion_host[idx] > zcur && jstart < N - 2 && kstart < N - 2) break;
        if (++tries > 100000000LL)
          return prc_fail(PRC_ERR_NUMERIC, "bubble mfp: no ionised cell found for x=%g (z=%g)", (double)xcur,
                          (double)zcur);
      }
      int* st = &plan->start[((size_t)ix * NS + is) * 3];
      st[0] = istart;
      st[1] = jstart;
      st[2] = kstart;
      plan->frac[((size_t)ix * NS + is) * 2 + 0] = draw();  // :185 after the y walk
      plan->frac[((size_t)ix * NS + is) * 2 + 1] = draw();  // :223 after the z walk
    }
  }
  return PRC_OK;
}

// :186-195 / :224-233 for one walk of m steps
static inline void account(const MfpPlan& p, int ix, int m, float frac, float* mean_l, float* dfdmfpl) {
  float clow = (float)log(m - 0.5);
  if (m > 1) clow = (float)log(m - 1.);
  const float chigh = (float)log(m * 1.0);
  const float current_distance = expf(clow + (chigh - clow) * frac) * p.cell;
  *mean_l += current_distance;
  const float lcd = logf(current_distance);
  const int imfp = (int)((lcd - p.mfp_initial) / p.dmfp);
  const int bin = ix * NMFP + imfp;
  if (imfp >= 0 && imfp < NMFP && lcd < p.mfp_final && lcd > p.mfp_initial) dfdmfpl[bin]++;
}

void mfp_finish(const MfpPlan& p, const int* steps /*nx*ns*2*/, float* mfp, float* mfp_x, float* dfdmfp) {
  memset(dfdmfp, 0, sizeof(float) * (size_t)NMFP * p.nx);
  for (int ix = 0; ix < p.nx; ix++) {
    float mean_l = 0;
    for (int is = 0; is < p.ns; is++) {
      const size_t s = (size_t)ix * p.ns + is;
      account(p, ix, steps[2 * s + 0], p.frac[2 * s + 0], &mean_l, dfdmfp);
      account(p, ix, steps[2 * s + 1], p.frac[2 * s + 1], &mean_l, dfdmfp);
    }
    mfp[ix] = (float)(mean_l / (2. * p.ns));  // :237-241 with nproc = 1
  }
  mfp_x[0] = (float)X_MFP_INITIAL;  // the reference leaves mfp_x[0] unset (:245)
  for (int i = 1; i < p.nx; i++) mfp_x[i] = (float)(X_MFP_INITIAL + i * p.dxmfp);
}

}  // namespace prc_hist

extern "C" {

// ---------------------------------------------------------------- GetCHistory
int prc_chistory(const prc_f2f_table* fcoll, const float* mfp, int n_x, float rmfp, float zeta, float* chistory) {
  if (!fcoll || !fcoll->table || !mfp || !chistory || n_x < 2)
    return prc_fail(PRC_ERR_INVALID, "prc_chistory: bad argument");
  const float dzch = (float)((CHISTORY_FINAL - CHISTORY_INITIAL) / (PRC_NCHISTORY - 1));  // :50
  const float dxmfp = (float)((X_MFP_FINAL - X_MFP_INITIAL) / (n_x - 1));
  auto bubble_mfp = [&](float x) {  // :254-276
    const int itab = (int)((x - X_MFP_INITIAL) / dxmfp);
    const float f = (float)((x - itab * dxmfp - X_MFP_INITIAL) / dxmfp);
    if (itab < 0) return mfp[0];
    if (itab >= n_x - 1) return mfp[n_x - 1];
    return (1 - f) * mfp[itab] + f * mfp[itab + 1];
  };
  chistory[0] = 0.;
  for (int i = 1; i < PRC_NCHISTORY; i++) {
    const float x1 = chistory[i - 1];
    const float z1 = (float)(CHISTORY_INITIAL + i * dzch);
    const float z2 = (float)(CHISTORY_INITIAL + (i + 1) * dzch);
    const float f1 = prc_f2f_eval(fcoll, z1);
    const float f2 = prc_f2f_eval(fcoll, z2);
    const float df = f2 - f1;
    const float rb = bubble_mfp(x1);
    chistory[i] = chistory[i - 1] + df / (1 + rb / rmfp) * zeta;
    if (chistory[i] >= 1) chistory[i] = 1;
  }
  return PRC_OK;
}

// ---------------------------------------------------------------- CorrectHistory's map
// zvz[i] = zreioncorrect(history[i]) for history[i] != 0, holes filled from
// above (bubblehistory_d2z.C:314-326).  zreioncorrect's first-match linear scan
// (:290-299) becomes a forward sweep: history is non-decreasing, so the first
// bracket of each x never lies before the previous one's.
int prc_zvz(const float* history, const float* chistory, float* zvz) {
  if (!history || !chistory || !zvz) return prc_fail(PRC_ERR_INVALID, "prc_zvz: null argument");
  const float dzch = (float)((CHISTORY_FINAL - CHISTORY_INITIAL) / (PRC_NCHISTORY - 1));
  for (int i = 0; i < PRC_NHISTORY; i++) zvz[i] = -1;
  bool mono = true;  // the forward sweep needs a non-decreasing chistory
  for (int j = 1; j < PRC_NCHISTORY; j++)
    if (chistory[j] < chistory[j - 1]) mono = false;
  int j0 = 0;
  float xprev = -1;
  for (int i = 1; i < PRC_NHISTORY; i++) {
    const float x = history[i];
    if (x == 0) continue;
    float z;
    if (x < chistory[0]) {
      z = (float)CHISTORY_INITIAL;
    } else if (x > chistory[PRC_NCHISTORY - 1]) {
      z = (float)CHISTORY_FINAL;
    } else {
      if (!mono || x < xprev) j0 = 0;  // not monotone: scan from the start
      int j = j0;
      while (j < PRC_NCHISTORY - 1 && !(x >= chistory[j] && x <= chistory[j + 1])) j++;
      if (j >= PRC_NCHISTORY - 1)
        return prc_fail(PRC_ERR_NUMERIC, "prc_zvz: no bracket for x=%g (the reference exits here)", (double)x);
      j0 = j;
      const float f = (x - chistory[j]) / (chistory[j + 1] - chistory[j]);
      z = (float)((1 - f) * (CHISTORY_INITIAL + j * dzch) + f * (CHISTORY_INITIAL + (j + 1) * dzch));
    }
    xprev = x;
    zvz[i] = z;
  }
  for (int i = PRC_NHISTORY - 2; i >= 0; i--)
    if (zvz[i] < 0) zvz[i] = zvz[i + 1];
  return PRC_OK;
}

}  // extern "C"
