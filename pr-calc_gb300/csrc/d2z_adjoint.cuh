// d2z_adjoint.cuh — adjoint (vector-Jacobian product) of the forward path.
//
// The reference has no gradient; this is new.  z_c = A (delta_{r*(c),c} + B_{r*})
// - 1 where r*(c) is the winning radius (argmax), and 0 for cells never updated.
// The barrier is linear in delta_R, so dz_c/d delta_R = A for R = r*(c) and the
// adjoint needs neither delta_R nor a recompute of it.  Each smoothing operator
// L_R = (1/(N^3 D_init)) IDFT diag(W_R) DFT is a real, even circulant convolution,
// hence self-adjoint, and
//   dL/d delta_lin = (1/(N^3 D_init)) IDFT( sum_R W_R * DFT(h_R) ),
//   h_R(c) = A * g_c * [r*(c) == R],      dL/dB_R = A * sum_{c: r*(c)=R} g_c.
// Kernels: k_adj_z builds h_R for a sweep of radii and runs the real-to-half-
// complex z pass; a forward column y pass follows (k_col); k_adj_x runs the x
// pass and accumulates W_R * (.) into the spectrum accumulator; after the last
// sweep the accumulator goes back through the inverse column passes and
// k_c2r_plain.
#pragma once
#include "d2z_kernels.cuh"

namespace prc {

struct AdjArgs {
  const float* g;        // dL/dz, N^3
  const uint8_t* am;     // argmax, N^3
  float A;
  float2* slots;         // slot 0 base
  long long slot_stride;
  float2* acc;           // spectrum-layout accumulator
  const float2* tw;
  double* dB;            // n_radii, or null
  int nb, r0, first;
  float kr[kMaxBatch];
  float* out;            // k_c2r_plain output (N^3)
  float scale;           // k_c2r_plain scale
};

// h_R along z -> half spectrum: main into slot b, X[H] into the slot's
// transposed Nyquist scratch (offset NN*(H+1)).
template <int N>
__global__ void __launch_bounds__(K<N>::LINE_THREADS) k_adj_z(AdjArgs a) {
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
  float sb[kMaxBatch];
#pragma unroll
  for (int b = 0; b < kMaxBatch; ++b) sb[b] = 0.f;
  for (int s = blockIdx.x; s * NG < lines; s += gridDim.x) {
    const int l = s * NG + g;
    const bool valid = l < lines;
    const int lv = valid ? l : 0;
    const float2* gl = reinterpret_cast<const float2*>(a.g + (long long)lv * N);
    const uchar2* al = reinterpret_cast<const uchar2*>(a.am + (long long)lv * N);
    for (int b = 0; b < a.nb; ++b) {
      const uint8_t rid = (uint8_t)(a.r0 + b);
      float2 v[1][E];
      float part = 0.f;
#pragma unroll
      for (int m = 0; m < E; ++m) {
        const int p = t + G * m;
        float2 gv = valid ? __ldg(gl + p) : make_float2(0.f, 0.f);
        uchar2 u = valid ? al[p] : make_uchar2(255, 255);
        const float h0 = (u.x == rid) ? gv.x : 0.f;
        const float h1 = (u.y == rid) ? gv.y : 0.f;
        part += h0 + h1;
        v[0][m] = make_float2(a.A * h0, a.A * h1);
      }
#pragma unroll
      for (int bb = 0; bb < kMaxBatch; ++bb)
        if (bb == b) sb[bb] += part;
      const float xh = line_r2c<N>(v, gbuf, t, tw, sync);
      if (valid) {
        float2* slot = a.slots + (long long)b * a.slot_stride;
        float2* dst = slot + (long long)l * H;
#pragma unroll
        for (int m = 0; m < E; ++m) dst[t + G * m] = v[0][m];
        if (t == 0) {
          const int ix = l / N, iy = l - (l / N) * N;
          slot[NN * (H + 1) + (long long)iy * N + ix] = make_float2(xh, 0.f);
        }
      }
    }
  }
  if (a.dB) {
#pragma unroll
    for (int b = 0; b < kMaxBatch; ++b) {
      if (b < a.nb) {
        float s = sb[b];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
        if ((threadIdx.x & 31) == 0) atomicAdd(&red[b], (double)s);
      }
    }
    __syncthreads();
    if (threadIdx.x < a.nb) atomicAdd(&a.dB[a.r0 + threadIdx.x], (double)a.A * red[threadIdx.x]);
  }
}

// Forward x pass of each slot, then acc += W_b * result (acc zeroed by the
// first sweep).  Slot main rows ix at stride N*H; slot Nyquist plane Q_b[ix][iy]
// (written by the preceding y pass) rows ix at stride N.
template <int N>
__global__ void __launch_bounds__(K<N>::COL_THREADS, 2) k_adj_x(AdjArgs a) {
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
    long long off;
    int row_stride, syz0, syz1;
    if (!nyq) {
      const int it = valid ? item : 0;
      const int iy = it / (H / 2), cp = it % (H / 2);
      off = (long long)iy * H + 2 * cp;
      row_stride = N * H;
      const int fy2 = fsq(iy, N);
      syz0 = fy2 + (2 * cp) * (2 * cp);
      syz1 = fy2 + (2 * cp + 1) * (2 * cp + 1);
    } else {
      const int cp = item - items0;
      off = NN * H + 2 * cp;
      row_stride = N;
      syz0 = fsq(2 * cp, N) + H * H;
      syz1 = fsq(2 * cp + 1, N) + H * H;
    }
    int sx[E];
#pragma unroll
    for (int m = 0; m < E; ++m) sx[m] = fsq(t + G * m, N);
    for (int b = 0; b < a.nb; ++b) {
      const float2* in = a.slots + (long long)b * a.slot_stride + off;
      float2 v[2][E];
#pragma unroll
      for (int m = 0; m < E; ++m) {
        const int row = t + G * m;
        float4 q = valid ? __ldg(reinterpret_cast<const float4*>(in + (long long)row * row_stride))
                         : make_float4(0.f, 0.f, 0.f, 0.f);
        v[0][m] = make_float2(q.x, q.y);
        v[1][m] = make_float2(q.z, q.w);
      }
      PlanRun<typename KK::ColP>::template run<2, false, 1>(v, gbuf, t, tw, sync);
      const float kr = a.kr[b];
      const bool zero_acc = a.first && b == 0;
      if (valid) {
        float2* accp = a.acc + off;
#pragma unroll
        for (int m = 0; m < E; ++m) {
          const int row = t + G * m;
          float4* ap = reinterpret_cast<float4*>(accp + (long long)row * row_stride);
          float4 q = zero_acc ? make_float4(0.f, 0.f, 0.f, 0.f) : *ap;
          const int m20 = sx[m] + syz0, m21 = sx[m] + syz1;
          const float w0 = (m20 == 0) ? 0.f : tophat(sqrtf((float)m20) * kr);
          const float w1 = (m21 == 0) ? 0.f : tophat(sqrtf((float)m21) * kr);
          q.x = fmaf(w0, v[0][m].x, q.x);
          q.y = fmaf(w0, v[0][m].y, q.y);
          q.z = fmaf(w1, v[1][m].x, q.z);
          q.w = fmaf(w1, v[1][m].y, q.w);
          *ap = q;
        }
      }
    }
  }
}

// Plain inverse z pass: slot 0 (main + transposed Nyquist) -> out = scale * x.
template <int N>
__global__ void __launch_bounds__(K<N>::LINE_THREADS) k_c2r_plain(AdjArgs a) {
  using KK = K<N>;
  constexpr int H = N / 2, E = KK::LE, G = KK::LG, NG = KK::LNG;
  constexpr long long NN = (long long)N * N;
  extern __shared__ float4 smem4[];
  float2* tw = reinterpret_cast<float2*>(smem4);
  load_tw(tw, a.tw, N);
  const int g = threadIdx.x / G, t = threadIdx.x % G;
  float2* gbuf = tw + N + g * GroupBuf<H, 1>::size;
  GroupSync<G> sync(g);
  const int lines = N * N;
  for (int s = blockIdx.x; s * NG < lines; s += gridDim.x) {
    const int l = s * NG + g;
    const bool valid = l < lines;
    const int lv = valid ? l : 0;
    const int ix = lv / N, iy = lv % N;
    const float2* src = a.slots + (long long)lv * H;
    float2 v[1][E];
#pragma unroll
    for (int m = 0; m < E; ++m) v[0][m] = valid ? __ldg(src + t + G * m) : make_float2(0.f, 0.f);
    float2 xn = make_float2(0.f, 0.f);
    if (t == 0 && valid) xn = __ldg(a.slots + NN * H + (long long)iy * N + ix);
    line_c2r<N>(v, xn, gbuf, t, tw, sync);
    if (valid) {
      float2* dst = reinterpret_cast<float2*>(a.out + (long long)l * N);
#pragma unroll
      for (int m = 0; m < E; ++m) dst[t + G * m] = make_float2(a.scale * v[0][m].x, a.scale * v[0][m].y);
    }
  }
}

}  // namespace prc
