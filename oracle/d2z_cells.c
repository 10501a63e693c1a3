/*
 * d2z_cells.c -- TEST INFRASTRUCTURE (the oracle).  CPU restatement of the
 * per-cell and per-mode loops of pr-calc's delta2zreion step, with the
 * reference's float/double conversions kept operation by operation.  Only the
 * tests, __graft_entry__.smoke() and bench.py's CPU-baseline / reference arm
 * load this library, and only to check results against it; the product never
 * does.
 *
 * Parity is unpinned: the reference (c++/src) needs MPI, FFTW 3.3.3 and GSL,
 * none of which are installed where this code is built and run, and it ships no test vectors.  These
 * loops follow its source line by line instead:
 *   orc_window_faithful  delta2zreion_d2z.C:41-43,58-89  (float kx, ky, kz,
 *                        sqrtf of the float sum, W = 3.*(sinf-x*cosf)/pow(x,3)
 *                        in double, stored as float; k = 0 -> 0)
 *   orc_barrier_update   delta2zreion_d2z.C:105-146 with d2z :206-216
 *                        (A in float, bracket in double, strict >)
 *   orc_hist             bubblehistory_d2z.C:17-28
 * Threads: OpenMP over the outer loop (each thread owns disjoint cells).
 * Build: gcc -O2 -fPIC -shared -fopenmp -ffp-contract=off (see oracle/build.py).
 */
#include <math.h>
#include <stdint.h>
#include <string.h>

#ifdef _OPENMP
#include <omp.h>
#endif

int orc_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

void orc_set_threads(int n) {
#ifdef _OPENMP
  if (n > 0) omp_set_num_threads(n);
#else
  (void)n;
#endif
}

/* W for every mode of the half spectrum, shape (N, N, N/2+1), reference float
 * arithmetic.  dk = 2*M_PI/BoxSize computed as the reference does (float),
 * passed in; R is the float radius in Mpc. */
void orc_window_faithful(int N, float dk, float R, float* W) {
  const float kmax = dk * N;
  const int H1 = N / 2 + 1;
#pragma omp parallel for schedule(static)
  for (int i = 0; i < N; i++) {
    float kx = i * dk;
    if (i >= N / 2) kx = kx - kmax;
    const float kx2 = kx * kx;
    for (int j = 0; j < N; j++) {
      float ky = j * dk;
      if (j >= N / 2) ky = ky - kmax;
      const float ky2 = ky * ky;
      float* row = W + ((long)i * N + j) * H1;
      for (int k = 0; k <= N / 2; k++) {
        float kz = k * dk;
        if (k >= N / 2) kz = kz - kmax;
        const float kz2 = kz * kz;
        const float rk = sqrtf(kx2 + ky2 + kz2);
        const float rkR = rk * R;
        const float num = sinf(rkR) - rkR * cosf(rkR);
        const float w = (float)(3. * (double)num / pow((double)rkR, 3.0));
        row[k] = (rk != 0) ? w : 0.0f;
      }
    }
  }
}

/* spec (complex64, interleaved) *= W, in place. */
void orc_apply_window_c64(long n, float* spec, const float* W) {
#pragma omp parallel for schedule(static)
  for (long i = 0; i < n; i++) {
    spec[2 * i] *= W[i];
    spec[2 * i + 1] *= W[i];
  }
}

/* z = (float)((double)A * ((double)d + B) - 1); if (z > zreion) update.
 * B = sqrt(2.*(double)(float)(smin^2 - s^2)) * (double)erfizeta, precomputed.
 * argmax (nullable) receives r.  sum2 (nullable) receives sum of d^2 in
 * double (GetMeanSigma, arrayoperations.C:4-35). */
void orc_barrier_update(long n, const float* d, float A, double B, int r, float* zreion, uint8_t* argmax,
                        double* sum2) {
  double s2 = 0;
#pragma omp parallel for schedule(static) reduction(+ : s2)
  for (long i = 0; i < n; i++) {
    const float dcur = d[i];
    const float zcur = (float)((double)A * ((double)dcur + B) - 1);
    if (zcur > zreion[i]) {
      zreion[i] = zcur;
      if (argmax) argmax[i] = (uint8_t)r;
    }
    s2 += (double)dcur * (double)dcur;
  }
  if (sum2) *sum2 = s2;
}

/* GetHistory binning: counts[bin]++ for bin = (int)((z - 49.9)/dz) in [0, nh). */
void orc_hist(long n, const float* z, float dzf, int nh, uint32_t* counts) {
  memset(counts, 0, sizeof(uint32_t) * (size_t)nh);
  for (long i = 0; i < n; i++) {
    const int bin = (int)(((double)z[i] - 49.9) / (double)dzf);
    if (bin >= 0 && bin < nh) counts[bin]++;
  }
}
