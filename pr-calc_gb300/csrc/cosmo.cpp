// cosmo.cpp — host tables of the delta2zreion step, in FP64 where the reference
// works in double and in FP32 where it stores floats.
//
// Restates, with the reference's float/double conversions kept operation by
// operation (pr-calc c++/src, C++ overload rules: sqrt/log/log10/pow of float
// arguments are the float functions; pow with an integer or double argument is
// the double one):
//   growth      cosmology.C:174-212   (Carroll-Press-Turner g, Ma et al. w term)
//   transeh     cosmology.C:290-309   (Eisenstein-Hu no-wiggle transfer function)
//   sgm2k       cosmology.C:274-288   (integrand of sigma^2 in ln k)
//   normalize   cosmology.C:246-272,  cdmehint cosmology.C:214-244
//   inverse_erfc math.C:23-61         (bracketing root finder, returns x_lo)
//   tau         cosmology.C:52-83
//   set-up of delta2zreion_d2z.C:14-38,55,97-100 and main_d2z.C:57-64
// The two third-party algorithms the reference takes from GSL are written here
// from their published descriptions, not from GSL:
//   * adaptive Gauss-Kronrod (7-15 point, Kronrod 1965 nodes; global adaptive
//     bisection of the interval with the largest error estimate, Piessens et al.,
//     QUADPACK 1983) for gsl_integration_qags(epsabs 0, epsrel 1e-7, limit 1000);
//   * Brent's method (Brent 1973, "Algorithms for minimization without
//     derivatives", ch. 4) for gsl_root_fsolver_brent stopped by an interval
//     test |hi - lo| < 1e-4 * min(|lo|, |hi|), returning the lower end.
// Compile with -ffp-contract=off so that float expressions round per operation.
#include <math.h>
#include <stdio.h>
#include <string.h>

#include <vector>

#include "../../include/prc_d2z.h"
#include "errors.h"

namespace {

struct Cosmo {
  double omega0, baryon0, hubble0, an0, pnorm0;
};

// ---------------------------------------------------------------- transfer
double transeh(const Cosmo& c, double k) {
  const double om = c.omega0, ob = c.baryon0, hh = c.hubble0;
  const double alpha = 1 - 0.328 * log(431 * om * hh * hh) * (ob / om) +
                       0.38 * log(22.3 * om * hh * hh) * pow(ob / om, 2);
  const double sound = 44.5 * log(9.83 / (om * hh * hh)) / sqrt(1 + 10 * pow(ob * hh * hh, 3. / 4.));
  const double shape = om * hh * (alpha + (1 - alpha) / (1 + pow(0.43 * k * sound, 4)));
  const double q = (k / hh) * pow(2.728 / 2.7, 2) / shape;
  const double L = log(2 * exp(1.0) + 1.8 * q);
  return L / (L + (14.2 + 731 / (1 + 62.5 * q)) * q * q);
}

double sgm2k(const Cosmo& c, double lk, double R) {
  const double k = exp(lk);
  const double kR = k * R;
  const double Pin = pow(k, 3 + c.an0);
  const double T = transeh(c, k);
  const double W = 3 * (sin(kR) - kR * cos(kR)) / pow(kR, 3);
  return Pin * T * T * pow(W, 2) * pow(c.pnorm0, 2);
}

// ---------------------------------------------------------------- quadrature
// 15-point Kronrod / 7-point Gauss rule on [a,b]: returns K15, error |K15-G7|.
struct Seg {
  double a, b, r, e;
};

template <class F>
void gk15(F&& f, double a, double b, double* res, double* err) {
  // Kronrod nodes (positive half, descending) and weights; Gauss weights at the
  // even-indexed Kronrod nodes.
  static const double xk[8] = {0.991455371120812639206854697526329, 0.949107912342758524526189684047851,
                               0.864864423359769072789712788640926, 0.741531185599394439863864773280788,
                               0.586087235467691130294144845693013, 0.405845151377397166906606412076961,
                               0.207784955007898467600689403773245, 0.000000000000000000000000000000000};
  static const double wk[8] = {0.022935322010529224963732008058970, 0.063092092629978553290700663189204,
                               0.104790010322250183839876322541518, 0.140653259715525918745189590510238,
                               0.169004726639267902826583426598550, 0.190350578064785409913256402421014,
                               0.204432940075298892414161999234649, 0.209482141084727828012999174891714};
  static const double wg[4] = {0.129484966168869693270611432679082, 0.279705391489276667901467771423780,
                               0.381830050505118944950369775488975, 0.417959183673469387755102040816327};
  const double c = 0.5 * (a + b), h = 0.5 * (b - a);
  const double fc = f(c);
  double rk = fc * wk[7], rg = fc * wg[3];
  for (int j = 0; j < 7; ++j) {
    const double dx = h * xk[j];
    const double f1 = f(c - dx), f2 = f(c + dx);
    rk += wk[j] * (f1 + f2);
    if (j & 1) rg += wg[j / 2] * (f1 + f2);
  }
  *res = rk * h;
  *err = fabs((rk - rg) * h);
}

template <class F>
int integrate(F&& f, double a, double b, double epsrel, int limit, double* out) {
  std::vector<Seg> segs;
  segs.reserve(limit);
  Seg s0{a, b, 0, 0};
  gk15(f, a, b, &s0.r, &s0.e);
  segs.push_back(s0);
  double tot = s0.r, err = s0.e;
  while (err > epsrel * fabs(tot)) {
    if ((int)segs.size() >= limit) {
      *out = tot;
      return PRC_ERR_NUMERIC;
    }
    size_t w = 0;
    for (size_t i = 1; i < segs.size(); ++i)
      if (segs[i].e > segs[w].e) w = i;
    Seg s = segs[w];
    const double m = 0.5 * (s.a + s.b);
    Seg l{s.a, m, 0, 0}, r{m, s.b, 0, 0};
    gk15(f, l.a, l.b, &l.r, &l.e);
    gk15(f, r.a, r.b, &r.r, &r.e);
    segs[w] = l;
    segs.push_back(r);
    tot = 0;
    err = 0;
    for (const Seg& q : segs) {
      tot += q.r;
      err += q.e;
    }
  }
  *out = tot;
  return PRC_OK;
}

int sigma2_of_R(const Cosmo& c, double R, double* out) {
  auto f = [&](double lk) { return sgm2k(c, lk, R); };
  return integrate(f, log(1e-5 / R), log(1e5 / R), 1e-7, 1000, out);
}

// ---------------------------------------------------------------- Brent
// Root of f on [lo, hi] (f(lo), f(hi) of opposite sign).  After every step the
// bracket is [min(b,c), max(b,c)]; iterate until |hi - lo| < rel * min(|lo|,|hi|)
// (or 100 steps) and return lo, as math.C:60 does.
template <class F>
int brent_lower(F&& f, double lo, double hi, double rel, int max_iter, double* out) {
  double a = lo, b = hi, fa = f(a), fb = f(b);
  if ((fa > 0 && fb > 0) || (fa < 0 && fb < 0)) return PRC_ERR_NUMERIC;
  double c = b, fc = fb, d = b - a, e = b - a;
  double xlo = lo, xhi = hi;
  for (int it = 0; it < max_iter; ++it) {
    if ((fb < 0 && fc < 0) || (fb > 0 && fc > 0)) {
      c = a;
      fc = fa;
      d = e = b - a;
    }
    if (fabs(fc) < fabs(fb)) {
      a = b; b = c; c = a;
      fa = fb; fb = fc; fc = fa;
    }
    const double tol = 0.5 * 2.220446049250313e-16 * fabs(b);
    const double m = 0.5 * (c - b);
    if (fb == 0 || fabs(m) <= tol) {
      xlo = xhi = b;
      break;
    }
    if (fabs(e) < tol || fabs(fa) <= fabs(fb)) {
      d = e = m;  // bisection
    } else {
      double p, q, r;
      const double s = fb / fa;
      if (a == c) {  // secant
        p = 2 * m * s;
        q = 1 - s;
      } else {  // inverse quadratic interpolation
        q = fa / fc;
        r = fb / fc;
        p = s * (2 * m * q * (q - r) - (b - a) * (r - 1));
        q = (q - 1) * (r - 1) * (s - 1);
      }
      if (p > 0) q = -q; else p = -p;
      const double lim1 = 3 * m * q - fabs(tol * q), lim2 = fabs(e * q);
      if (2 * p < (lim1 < lim2 ? lim1 : lim2)) {
        e = d;
        d = p / q;
      } else {
        d = e = m;
      }
    }
    a = b;
    fa = fb;
    b += (fabs(d) > tol) ? d : (m > 0 ? tol : -tol);
    fb = f(b);
    xlo = b < c ? b : c;
    xhi = b < c ? c : b;
    const double mn = fabs(xlo) < fabs(xhi) ? fabs(xlo) : fabs(xhi);
    if ((xlo > 0 && xhi > 0) || (xlo < 0 && xhi < 0)) {
      if (fabs(xhi - xlo) < rel * mn) break;
    }
  }
  *out = xlo;
  return PRC_OK;
}

// ---------------------------------------------------------------- reference set-up
int normalize_(float omega, float baryon, float hubble, float an, float sigma8, float* pnorm) {
  Cosmo c{omega, baryon, hubble, an, 1.0};
  const double R = (double)(8 / hubble);  // int / float
  double s2;
  int st = sigma2_of_R(c, R, &s2);
  *pnorm = (float)(sigma8 / sqrt(s2));
  return st;
}

int cdmehint_(float omega, float baryon, float hubble, float an, float pnorm, float mass, float* sgm2) {
  const float rhoc = 2.775e11f;
  const float pi = 3.141592654f, fourpi = 4 * pi;
  Cosmo c{omega, baryon, hubble, an, pnorm};
  const double dens = (double)(omega * rhoc * hubble * hubble);
  const float num = (3 * mass) / fourpi;
  const double R = pow((double)num / dens, 1. / 3.);
  double s2;
  int st = sigma2_of_R(c, R, &s2);
  *sgm2 = (float)s2;
  return st;
}

}  // namespace

extern "C" {

float prc_growth(float z, float omegam, float omegal, float w) {
  const float x = 1 + z;
  const float x2 = x * x;
  const float x3 = x * x * x;
  const float x3w = powf(x3, w);
  const float omega = omegam * x3 / (omegam * x3 + (1 - omegam - omegal) * x2 + omegal);
  const float lambda = omegal * x3 * x3w / (omegam * x3 + (1 - omegam - omegal) * x2 + omegal * x3 * x3w);
  float g = (float)(2.5 * (double)omega /
                    (pow((double)omega, 4. / 7.) - (double)lambda +
                     (double)((1 + omega / 2) * (1 + lambda / 70))));
  float g0 = (float)(2.5 * (double)omegam /
                     (pow((double)omegam, 4. / 7.) - (double)omegal +
                      (double)((1 + omegam / 2) * (1 + omegal / 70))));
  const double wd = (double)w;
  const float t = (float)(-(0.255 + 0.305 * wd + 0.0027 / wd) * (double)(1 - omega) -
                          (0.366 + 0.266 * wd - 0.0700 / wd) * (double)logf(omega));
  const float t0 = (float)(-(0.255 + 0.305 * wd + 0.0027 / wd) * (double)(1 - omegam) -
                           (0.366 + 0.266 * wd - 0.0700 / wd) * (double)logf(omegam));
  g *= powf(-w, t);
  g0 *= powf(-w, t0);
  return (g / x) / g0;
}

int prc_sigma2(float omegam, float omegab, float h, float ns, float pnorm, float mass, float* sgm2) {
  if (!sgm2) return prc_fail(PRC_ERR_INVALID, "prc_sigma2: null output");
  int st = cdmehint_(omegam, omegab, h, ns, pnorm, mass, sgm2);
  if (st != PRC_OK) return prc_fail(st, "sigma^2 quadrature did not reach epsrel 1e-7 in 1000 intervals");
  return PRC_OK;
}

int prc_inverse_erfc(float x, float* out) {
  if (!out) return prc_fail(PRC_ERR_INVALID, "prc_inverse_erfc: null output");
  const double a = (double)x;
  auto f = [a](double v) { return erfc(v) - a; };
  double r;
  int st = brent_lower(f, 0.0, 100.0, 1e-4, 100, &r);
  if (st != PRC_OK) return prc_fail(st, "inverse_erfc: root not bracketed on [0,100] (x=%g)", (double)x);
  *out = (float)r;
  return PRC_OK;
}

float prc_tau(const float* za, const float* xa, int nz, float omegam, float omegab, float h) {
  const float thompson = 6.65e-25f;
  const float YHe = 0.25f;
  const float hubble0 = (float)(100. / 3.086e19 * (double)h);
  const float ne0 = (float)((double)(omegab * h * h) * 1.88e-29 / 1.67e-24);
  const float c = 3e10f;
  const float dtau0 = thompson * ne0 * c / hubble0;
  float tau = 0;
  for (int i = 1; i < nz - 1; i++) {
    const float z = za[i];
    const float x = xa[i];
    const float dz = fabsf(za[i + 1] - za[i]);
    const float NHe = (z < 3) ? 2.f : 1.f;
    const double num = (double)(x * dtau0) * pow((double)(1 + z), 2.0);
    const double den = sqrt((double)omegam * pow((double)(1 + z), 3.0) + 1 - (double)omegam);
    const float dtau = (float)(num / den * (double)(1 - YHe + NHe * YHe / 4) * (double)dz);
    tau += dtau;
  }
  return tau;
}

int prc_compute_tables(const prc_params* p, prc_tables* out) {
  if (!p || !out) return prc_fail(PRC_ERR_INVALID, "prc_compute_tables: null argument");
  if (p->N < 2 || p->Nscales < 2 || p->Nscales > PRC_MAX_RADII)
    return prc_fail(PRC_ERR_INVALID, "prc_compute_tables: need N >= 2 and 2 <= Nscales <= %d", PRC_MAX_RADII);
  if (!(p->zeta > 1)) return prc_fail(PRC_ERR_INVALID, "prc_compute_tables: zeta must exceed 1");
  int st;
  // main_d2z.C:29 (BoxSize/=h), :57-64
  const float box = p->BoxSize / p->h;
  out->DInit = prc_growth(p->zInit, p->Omegam, p->Omegal, p->w);
  out->zHigh = 20.0f;
  out->DHigh = prc_growth(out->zHigh, p->Omegam, p->Omegal, p->w);
  // delta2zreion_d2z.C:14-26
  const float rho0 = (float)(2.775e11 * (double)p->Omegam * (double)p->h * (double)p->h);
  float pnorm;
  if ((st = normalize_(p->Omegam, p->Omegab, p->h, p->ns, p->sigma8, &pnorm)) != PRC_OK)
    return prc_fail(st, "normalize: sigma_8 quadrature did not converge");
  out->pnorm = pnorm;
  float erfizeta;
  if ((st = prc_inverse_erfc((float)(1. / (double)p->zeta), &erfizeta)) != PRC_OK) return st;
  out->erfizeta = erfizeta;
  float sgm2;
  if ((st = prc_sigma2(p->Omegam, p->Omegab, p->h, p->ns, pnorm, p->M_min, &sgm2)) != PRC_OK) return st;
  const float sigma_min = sqrtf(sgm2);
  out->sigma_min = sigma_min;
  // delta2zreion_d2z.C:29-38
  const int N = p->N, Nscales = p->Nscales;
  const float Rinitial = box * p->Rmin / N;
  const float Rfinal = p->Rmax / p->h;
  const float dScale = (log10f(Rfinal) - log10f(Rinitial)) / (Nscales - 1);
  // d2z (delta2zreion_d2z.C:206-216): A in float, the bracket in double
  const float deltac = 1.686f;
  const float A = (1 + out->zHigh) * out->DHigh / deltac;
  out->barrier_a = (double)A;
  for (int r = 0; r < Nscales; r++) {
    const float R = (float)pow(10.0, (double)(log10f(Rinitial) + r * dScale));  // :55
    const float mass = (float)(4 * M_PI / 3 * (double)rho0 * R * R * R);         // :97
    float s2;
    if ((st = prc_sigma2(p->Omegam, p->Omegab, p->h, p->ns, pnorm, mass, &s2)) != PRC_OK) return st;
    const float sigma = sqrtf(s2);  // :100
    if (out->radii_mpc) out->radii_mpc[r] = (double)R;
    if (out->sigma_r) out->sigma_r[r] = sigma;
    const float dvar = sigma_min * sigma_min - sigma * sigma;
    if (out->barrier_b) out->barrier_b[r] = sqrt(2. * (double)dvar) * (double)erfizeta;
  }
  return PRC_OK;
}

}  // extern "C"
