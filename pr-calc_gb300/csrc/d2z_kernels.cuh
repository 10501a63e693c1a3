// d2z_kernels.cuh — the delta2zreion hot path as sm_103a kernels.
//
// Device layout of one box (N = grid side, H = N/2, NN = N*N), in float2 units:
//   spectrum  : main S[ix][iy][kz] (kz < H, NN*H entries) followed by the
//               kz = H (Nyquist) plane Q[ix][iy] (NN entries)
//   slot b    : same size; main U_b[ix][iy][kz], Nyquist plane transposed
//               Qt_b[iy][ix] so that its y pass is a strided-column pass too
// A "column pass" transforms along ix or iy: a group of G threads owns two
// adjacent columns (one 16-byte access per row) and all N rows; adjacent
// groups own adjacent columns, so a CTA touches whole 128-byte row segments.
// A "line pass" transforms along z: a group owns one contiguous line and uses
// the half-length complex FFT of a real sequence (even samples in .x, odd in .y).
//
// Reference steps fused here (pr-calc c++/src):
//   k_r2c_z + k_col(fwd, y) + k_col(fwd, x) : main_d2z.C:57-59 (delta /= DInit)
//                                            and the R2C at main_d2z.C:67
//   k_win_x   : window loop delta2zreion_d2z.C:57-89 + first axis of the C2R (:92)
//   k_col(inv): second axis of the C2R
//   k_c2r_z   : last axis of the C2R, NormalizeArray (:93), GetMeanSigma (:94),
//               barrier d2z (:206-216) and the running max (:105-146)
//   k_hist    : GetHistory binning (bubblehistory_d2z.C:17-28)
#pragma once
#include "fft.cuh"

namespace prc {

constexpr int kMaxBatch = 16;
constexpr int kNHistory = 100000;

// ------------------------------------------------------------ per-N plans
// Column plan: Plan<E, radices...> of length N; line plan: length N/2.
template <int N> struct Cfg;
template <> struct Cfg<8> { using Col = Plan<8, 8>; using Line = Plan<4, 4>; };
template <> struct Cfg<12> { using Col = Plan<12, 4, 3>; using Line = Plan<6, 3, 2>; };
template <> struct Cfg<16> { using Col = Plan<16, 16>; using Line = Plan<8, 8>; };
template <> struct Cfg<24> { using Col = Plan<12, 4, 3, 2>; using Line = Plan<12, 4, 3>; };
template <> struct Cfg<32> { using Col = Plan<16, 16, 2>; using Line = Plan<16, 16>; };
template <> struct Cfg<48> { using Col = Plan<12, 4, 4, 3>; using Line = Plan<12, 4, 3, 2>; };
template <> struct Cfg<64> { using Col = Plan<16, 16, 4>; using Line = Plan<8, 8, 4>; };
template <> struct Cfg<96> { using Col = Plan<24, 8, 4, 3>; using Line = Plan<12, 4, 4, 3>; };
template <> struct Cfg<128> { using Col = Plan<16, 16, 8>; using Line = Plan<8, 8, 8>; };
template <> struct Cfg<192> { using Col = Plan<24, 8, 8, 3>; using Line = Plan<24, 8, 4, 3>; };
template <> struct Cfg<256> { using Col = Plan<16, 16, 16>; using Line = Plan<16, 16, 8>; };
template <> struct Cfg<512> { using Col = Plan<16, 8, 8, 8>; using Line = Plan<8, 8, 8, 4>; };
template <> struct Cfg<1024> { using Col = Plan<16, 16, 16, 4>; using Line = Plan<16, 16, 16, 2>; };


template <int N> struct K {
  static constexpr int H = N / 2;
  using ColP = typename Cfg<N>::Col;
  using LineP = typename Cfg<N>::Line;
  static constexpr int CE = ColP::E;
  static constexpr int CG = N / CE;
  static constexpr int LE = LineP::E;
  static constexpr int LG = H / LE;
  static_assert(PlanRun<ColP>::L == N, "column plan length");
  static_assert(PlanRun<LineP>::L == H, "line plan length");
  static constexpr int COL_THREADS = 256;
  static constexpr int LINE_THREADS = 256;
  static constexpr int CNG = COL_THREADS / CG;   // column groups per CTA
  static constexpr int LNG = LINE_THREADS / LG;  // line groups per CTA
  static constexpr int col_smem_f2 = N + CNG * GroupBuf<N, 2>::size;
  static constexpr int line_smem_f2 = N + LNG * GroupBuf<H, 1>::size;
};

// ------------------------------------------------------------ kernel args
struct ColSeg {
  const float2* in;
  float2* out;
  int row_stride;    // float2 between FFT rows
  int outer_stride;  // float2 between outer indices
  int n_outer;
  int n_cp;          // column pairs per outer index
  int transpose;     // 1: out[(col)*N + row] (a square N x N plane)
};

struct ColArgs {
  ColSeg seg[2];            // main + Nyquist plane
  long long slot_stride;    // float2 between slots (blockIdx.y)
  const float2* tw;         // N-entry table e^{+2 pi i k/N}
};

struct SweepArgs {
  const float2* spec;   // spectrum (k_win_x input)
  float2* slots;        // slot 0 base
  long long slot_stride;
  const float2* tw;
  float* zreion;        // N^3
  uint8_t* argmax;      // N^3 or null
  double* sig_acc;      // per-radius sum of x^2 (raw C2R units) or null
  int nb;               // radii in this sweep
  int r0;               // global index of the first radius
  int first;            // first sweep: zreion/argmax not read
  float as;             // A / N^3
  float kr[kMaxBatch];  // dk * R_b
  float cb[kMaxBatch];  // A*B_b - 1 (NaN: never wins)
};

// ------------------------------------------------------------ helpers
__device__ __forceinline__ int fsq(int f, int n) {
  const int a = (f <= (n >> 1)) ? f : n - f;
  return a * a;
}

// Top-hat window W(x) = 3 (sin x - x cos x) / x^3 (delta2zreion_d2z.C:77),
// evaluated without the cancellation of the closed form for x < 1 by its
// Taylor series  sum_m 3 (-1)^m (2m+2) x^{2m} / (2m+3)!.
__device__ __forceinline__ float tophat(float x) {
  if (x < 1.0f) {
    const float x2 = x * x;
    float p = 3.2118087673643226e-11f;
    p = fmaf(p, x2, -5.7812557812557812e-09f);
    p = fmaf(p, x2, 7.5156325156325156e-07f);
    p = fmaf(p, x2, -6.6137566137566138e-05f);
    p = fmaf(p, x2, 3.5714285714285714e-03f);
    p = fmaf(p, x2, -0.1f);
    p = fmaf(p, x2, 1.0f);
    return p;
  }
  float s, c;
  sincosf(x, &s, &c);
  const float r = 1.0f / x;
  return 3.0f * fmaf(-x, c, s) * (r * r * r);
}

__device__ __forceinline__ void load_tw(float2* tw_s, const float2* tw, int n) {
  for (int i = threadIdx.x; i < n; i += blockDim.x) tw_s[i] = tw[i];
  __syncthreads();
}

// ============================================================ column pass
// Generic strided pass without window: F2/F3 (forward) and P2 (inverse).
template <int N, bool INV>
__global__ void __launch_bounds__(K<N>::COL_THREADS, 2) k_col(ColArgs a) {
  using KK = K<N>;
  constexpr int E = KK::CE, G = KK::CG, NG = KK::CNG;
  extern __shared__ float4 smem4[];
  float2* tw = reinterpret_cast<float2*>(smem4);
  load_tw(tw, a.tw, N);
  const int g = threadIdx.x / G, t = threadIdx.x % G;
  float2* gbuf = tw + N + g * GroupBuf<N, 2>::size;
  GroupSync<G> sync(g);
  const long long soff = (long long)blockIdx.y * a.slot_stride;
  const int items0 = a.seg[0].n_outer * a.seg[0].n_cp;
  const int items = items0 + a.seg[1].n_outer * a.seg[1].n_cp;
  for (int s = blockIdx.x; s * NG < items; s += gridDim.x) {
    const int item = s * NG + g;
    const bool valid = item < items;
    const bool si = item >= items0;
    // field-wise select keeps the segment descriptors in the parameter bank
    const int n_cp = si ? a.seg[1].n_cp : a.seg[0].n_cp;
    const int row_stride = si ? a.seg[1].row_stride : a.seg[0].row_stride;
    const int outer_stride = si ? a.seg[1].outer_stride : a.seg[0].outer_stride;
    const int transpose = si ? a.seg[1].transpose : a.seg[0].transpose;
    const float2* sin_ = si ? a.seg[1].in : a.seg[0].in;
    float2* sout = si ? a.seg[1].out : a.seg[0].out;
    const int it = valid ? (si ? item - items0 : item) : 0;
    const int outer = it / n_cp;
    const int cpi = it - outer * n_cp;
    const float2* in = sin_ + soff + (long long)outer * outer_stride + 2 * cpi;
    float2 v[2][E];
#pragma unroll
    for (int m = 0; m < E; ++m) {
      const int row = t + G * m;
      float4 q = valid ? __ldg(reinterpret_cast<const float4*>(in + (long long)row * row_stride))
                       : make_float4(0.f, 0.f, 0.f, 0.f);
      v[0][m] = make_float2(q.x, q.y);
      v[1][m] = make_float2(q.z, q.w);
    }
    PlanRun<typename KK::ColP>::template run<2, INV, 1>(v, gbuf, t, tw, sync);
    if (valid) {
      float2* out = sout + soff;
      if (!transpose) {
        out += (long long)outer * outer_stride + 2 * cpi;
#pragma unroll
        for (int m = 0; m < E; ++m) {
          const int row = t + G * m;
          reinterpret_cast<float4*>(out + (long long)row * row_stride)[0] =
              make_float4(v[0][m].x, v[0][m].y, v[1][m].x, v[1][m].y);
        }
      } else {
#pragma unroll
        for (int m = 0; m < E; ++m) {
          const int row = t + G * m;
          out[(2 * cpi) * N + row] = v[0][m];
          out[(2 * cpi + 1) * N + row] = v[1][m];
        }
      }
    }
  }
}

// ============================================================ window + x pass
// For each radius of the sweep: delta_hat * W(|k| R_b) (k = 0 -> 0), inverse
// FFT along x, into slot b.  The spectrum tile is re-read per radius (L1/L2).
template <int N>
__global__ void __launch_bounds__(K<N>::COL_THREADS, 2) k_win_x(SweepArgs a) {
  using KK = K<N>;
  constexpr int H = N / 2, E = KK::CE, G = KK::CG, NG = KK::CNG;
  constexpr long long NN = (long long)N * N;
  extern __shared__ float4 smem4[];
  float2* tw = reinterpret_cast<float2*>(smem4);
  load_tw(tw, a.tw, N);
  const int g = threadIdx.x / G, t = threadIdx.x % G;
  float2* gbuf = tw + N + g * GroupBuf<N, 2>::size;
  GroupSync<G> sync(g);
  const int items0 = N * (H / 2);
  const int items = items0 + N / 2;
  for (int s = blockIdx.x; s * NG < items; s += gridDim.x) {
    const int item = s * NG + g;
    const bool valid = item < items;
    const bool nyq = item >= items0;
    // source pointer, row stride, and squared frequency of the two columns
    const float2* in;
    int row_stride, syz0, syz1, c0;
    if (!nyq) {
      const int it = valid ? item : 0;
      const int iy = it / (H / 2), cp = it % (H / 2);
      in = a.spec + (long long)iy * H + 2 * cp;
      row_stride = N * H;
      const int fy2 = fsq(iy, N);
      syz0 = fy2 + (2 * cp) * (2 * cp);
      syz1 = fy2 + (2 * cp + 1) * (2 * cp + 1);
      c0 = 2 * cp;
    } else {
      const int cp = item - items0;
      in = a.spec + NN * H + 2 * cp;
      row_stride = N;
      syz0 = fsq(2 * cp, N) + H * H;
      syz1 = fsq(2 * cp + 1, N) + H * H;
      c0 = 2 * cp;
    }
    int sx[E];
#pragma unroll
    for (int m = 0; m < E; ++m) sx[m] = fsq(t + G * m, N);
    for (int b = 0; b < a.nb; ++b) {
      const float kr = a.kr[b];
      float2 v[2][E];
#pragma unroll
      for (int m = 0; m < E; ++m) {
        const int row = t + G * m;
        float4 q = valid ? __ldg(reinterpret_cast<const float4*>(in + (long long)row * row_stride))
                         : make_float4(0.f, 0.f, 0.f, 0.f);
        v[0][m] = make_float2(q.x, q.y);
        v[1][m] = make_float2(q.z, q.w);
      }
      // window: rows ix and N-ix share |k|, so each pair is evaluated once
#pragma unroll
      for (int c = 0; c < 2; ++c) {
        const int syz = c ? syz1 : syz0;
        float w[E];
        constexpr int EH = E / 2;
        constexpr bool share = (G <= 32);
#pragma unroll
        for (int m = 0; m < E; ++m) {
          if (!share || m <= EH) {
            const int m2 = sx[m] + syz;
            w[m] = (m2 == 0) ? 0.f : tophat(sqrtf((float)m2) * kr);
          }
        }
        if constexpr (share) {
#pragma unroll
          for (int m = EH + 1; m < E; ++m) {
            const float o = __shfl_sync(0xffffffffu, w[E - 1 - m], (G - t) & (G - 1), G);
            w[m] = (t == 0) ? w[E - m] : o;
          }
          // m == EH: for t > 0 the directly computed value equals the mirror's
        }
#pragma unroll
        for (int m = 0; m < E; ++m) v[c][m] = cscale(v[c][m], w[m]);
      }
      PlanRun<typename KK::ColP>::template run<2, true, 1>(v, gbuf, t, tw, sync);
      if (valid) {
        float2* out = a.slots + (long long)b * a.slot_stride;
        if (!nyq) {
          const int iy = item / (H / 2), cp = item % (H / 2);
          out += (long long)iy * H + 2 * cp;
#pragma unroll
          for (int m = 0; m < E; ++m) {
            const int row = t + G * m;
            reinterpret_cast<float4*>(out + (long long)row * (N * H))[0] =
                make_float4(v[0][m].x, v[0][m].y, v[1][m].x, v[1][m].y);
          }
        } else {
          out += NN * H;
#pragma unroll
          for (int m = 0; m < E; ++m) {
            const int row = t + G * m;
            out[(long long)c0 * N + row] = v[0][m];
            out[(long long)(c0 + 1) * N + row] = v[1][m];
          }
        }
      }
    }
  }
}

// ============================================================ line helpers
// Forward real-to-half-complex along a line.  In: v[m] = (x[2p], x[2p+1]) at
// p = t + G*m.  Out: v[m] = X[k] at k = t + G*m (k < H); returns X[H] (real) in
// lane t == 0.  Z = DFT_H(x_even + i x_odd); X[k] = Ze[k] + e^{-2 pi i k/N} Zo[k].
template <int N, class Sync>
__device__ __forceinline__ float line_r2c(float2 (&v)[1][K<N>::LE], float2* gbuf, int t,
                                          const float2* tw, const Sync& sync) {
  constexpr int H = N / 2, E = K<N>::LE, G = K<N>::LG;
  PlanRun<typename K<N>::LineP>::template run<1, false, 2>(v, gbuf, t, tw, sync);
#pragma unroll
  for (int m = 0; m < E; ++m) gbuf[Swz<H, 1>::f(t + G * m)] = v[0][m];
  sync();
  float2 p[E];
#pragma unroll
  for (int m = 0; m < E; ++m) p[m] = gbuf[Swz<H, 1>::f((H - (t + G * m)) % H)];
  sync();
  float xh = 0.f;
#pragma unroll
  for (int m = 0; m < E; ++m) {
    const int k = t + G * m;
    const float2 z = v[0][m], zc = cconj(p[m]);
    const float2 ze = cscale(cadd(z, zc), 0.5f);
    const float2 d = csub(z, zc);
    const float2 zo = make_float2(0.5f * d.y, -0.5f * d.x);  // d / (2i)
    v[0][m] = cadd(ze, cmul(cconj(tw[k]), zo));
    if (m == 0) xh = ze.x - zo.x;
  }
  return xh;
}

// Inverse half-complex-to-real along a line (FFTW c2r semantics: the imaginary
// parts of X[0] and X[H] are ignored).  In: v[m] = X[k] at k = t + G*m, xh =
// X[H] (read by lane t == 0 only).  Out: v[m] = (x[2p], x[2p+1]) at p = t + G*m,
// unnormalised.
template <int N, class Sync>
__device__ __forceinline__ void line_c2r(float2 (&v)[1][K<N>::LE], float2 xh, float2* gbuf, int t,
                                         const float2* tw, const Sync& sync) {
  constexpr int H = N / 2, E = K<N>::LE, G = K<N>::LG;
#pragma unroll
  for (int m = 0; m < E; ++m) gbuf[Swz<H, 1>::f(t + G * m)] = v[0][m];
  sync();
  float2 p[E];
#pragma unroll
  for (int m = 0; m < E; ++m) p[m] = gbuf[Swz<H, 1>::f((H - (t + G * m)) % H)];
  sync();
#pragma unroll
  for (int m = 0; m < E; ++m) {
    const int k = t + G * m;
    float2 x = v[0][m], xp = p[m];
    if (k == 0) {
      x = make_float2(x.x, 0.f);
      xp = make_float2(xh.x, 0.f);
    }
    const float2 xc = cconj(xp);
    const float2 xe = cadd(x, xc);
    const float2 xo = cmul(csub(x, xc), tw[k]);
    v[0][m] = make_float2(xe.x - xo.y, xe.y + xo.x);  // xe + i*xo
  }
  PlanRun<typename K<N>::LineP>::template run<1, true, 2>(v, gbuf, t, tw, sync);
}

// ============================================================ forward z pass
// Real line (N samples, scaled by 1/DInit) -> X[0..H-1] into S and X[H] into
// the transposed Nyquist plane Qt[iy][ix].
template <int N>
__global__ void __launch_bounds__(K<N>::LINE_THREADS) k_r2c_z(const float* __restrict__ delta,
                                                               float dinit, float2* S, float2* Qt,
                                                               const float2* twg) {
  using KK = K<N>;
  constexpr int H = N / 2, E = KK::LE, G = KK::LG, NG = KK::LNG;
  extern __shared__ float4 smem4[];
  float2* tw = reinterpret_cast<float2*>(smem4);
  load_tw(tw, twg, N);
  const int g = threadIdx.x / G, t = threadIdx.x % G;
  float2* gbuf = tw + N + g * GroupBuf<H, 1>::size;
  GroupSync<G> sync(g);
  const int lines = N * N;
  for (int s = blockIdx.x; s * NG < lines; s += gridDim.x) {
    const int l = s * NG + g;
    const bool valid = l < lines;
    float2 v[1][E];
    const float2* src = reinterpret_cast<const float2*>(delta + (long long)(valid ? l : 0) * N);
#pragma unroll
    for (int m = 0; m < E; ++m) {
      float2 q = valid ? __ldg(src + t + G * m) : make_float2(0.f, 0.f);
      v[0][m] = make_float2(__fdiv_rn(q.x, dinit), __fdiv_rn(q.y, dinit));
    }
    const float xh = line_r2c<N>(v, gbuf, t, tw, sync);
    if (valid) {
      float2* dst = S + (long long)l * H;
#pragma unroll
      for (int m = 0; m < E; ++m) dst[t + G * m] = v[0][m];
      if (t == 0) {
        const int ix = l / N, iy = l - (l / N) * N;
        Qt[(long long)iy * N + ix] = make_float2(xh, 0.f);
      }
    }
  }
}

// ============================================================ inverse z pass
// For each radius of the sweep: X[0..H] -> real line, z = A/N^3 * x + (A B_b - 1),
// running max / argmax in registers, optional sum of x^2; one zreion RMW per sweep.
template <int N>
__global__ void __launch_bounds__(K<N>::LINE_THREADS) k_c2r_z(SweepArgs a) {
  using KK = K<N>;
  constexpr int H = N / 2, E = KK::LE, G = KK::LG, NG = KK::LNG;
  constexpr long long NN = (long long)N * N;
  extern __shared__ float4 smem4[];
  float2* tw = reinterpret_cast<float2*>(smem4);
  load_tw(tw, a.tw, N);
  __shared__ double red[kMaxBatch];
  if (threadIdx.x < kMaxBatch) red[threadIdx.x] = 0.0;
  __syncthreads();
  const int g = threadIdx.x / G, t = threadIdx.x % G;
  float2* gbuf = tw + N + g * GroupBuf<H, 1>::size;
  GroupSync<G> sync(g);
  const int lines = N * N;
  const bool want_sig = a.sig_acc != nullptr;
  float sig[kMaxBatch];
#pragma unroll
  for (int b = 0; b < kMaxBatch; ++b) sig[b] = 0.f;
  for (int s = blockIdx.x; s * NG < lines; s += gridDim.x) {
    const int l = s * NG + g;
    const bool valid = l < lines;
    const int lv = valid ? l : 0;
    const int ix = lv / N, iy = lv % N;
    float zr[2 * E];
    uint8_t am[2 * E];
    float* zline = a.zreion + (long long)lv * N;
    uint8_t* aline = a.argmax ? a.argmax + (long long)lv * N : nullptr;
    if (a.first || !valid) {
#pragma unroll
      for (int i = 0; i < 2 * E; ++i) { zr[i] = 0.f; am[i] = 255; }
    } else {
#pragma unroll
      for (int m = 0; m < E; ++m) {
        const int p = t + G * m;
        float2 q = reinterpret_cast<const float2*>(zline)[p];
        zr[2 * m] = q.x;
        zr[2 * m + 1] = q.y;
        if (aline) {
          uchar2 u = reinterpret_cast<const uchar2*>(aline)[p];
          am[2 * m] = u.x;
          am[2 * m + 1] = u.y;
        } else {
          am[2 * m] = am[2 * m + 1] = 255;
        }
      }
    }
    for (int b = 0; b < a.nb; ++b) {
      const float2* slot = a.slots + (long long)b * a.slot_stride;
      const float2* src = slot + (long long)lv * H;
      float2 v[1][E];
#pragma unroll
      for (int m = 0; m < E; ++m) v[0][m] = valid ? __ldg(src + t + G * m) : make_float2(0.f, 0.f);
      float2 xn = make_float2(0.f, 0.f);
      if (t == 0 && valid) xn = __ldg(slot + NN * H + (long long)iy * N + ix);
      line_c2r<N>(v, xn, gbuf, t, tw, sync);
      const float cb = a.cb[b];
      const uint8_t rid = (uint8_t)(a.r0 + b);
      float ss = 0.f;
#pragma unroll
      for (int m = 0; m < E; ++m) {
        const float x0 = v[0][m].x, x1 = v[0][m].y;
        const float z0 = fmaf(a.as, x0, cb), z1 = fmaf(a.as, x1, cb);
        if (z0 > zr[2 * m]) { zr[2 * m] = z0; am[2 * m] = rid; }
        if (z1 > zr[2 * m + 1]) { zr[2 * m + 1] = z1; am[2 * m + 1] = rid; }
        ss = fmaf(x0, x0, fmaf(x1, x1, ss));
      }
      if (want_sig && valid) {
#pragma unroll
        for (int bb = 0; bb < kMaxBatch; ++bb)
          if (bb == b) sig[bb] += ss;
      }
    }
    if (valid) {
#pragma unroll
      for (int m = 0; m < E; ++m) {
        const int p = t + G * m;
        reinterpret_cast<float2*>(zline)[p] = make_float2(zr[2 * m], zr[2 * m + 1]);
        if (aline) reinterpret_cast<uchar2*>(aline)[p] = make_uchar2(am[2 * m], am[2 * m + 1]);
      }
    }
  }
  if (want_sig) {
#pragma unroll
    for (int b = 0; b < kMaxBatch; ++b) {
      if (b < a.nb) {
        float s = sig[b];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
        if ((threadIdx.x & 31) == 0) atomicAdd(&red[b], (double)s);
      }
    }
    __syncthreads();
    if (threadIdx.x < a.nb) atomicAdd(&a.sig_acc[a.r0 + threadIdx.x], red[threadIdx.x]);
  }
}

}  // namespace prc
