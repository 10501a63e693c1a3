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
// complex z pass; a forward column y pass follows (k_tile<TM_FWD>); the x pass
// k_tile<TM_ACC> accumulates W_R * (.) into the spectrum accumulator; after the
// last sweep the accumulator goes back through the inverse column passes and
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
  const float2* tw;
  double* dB;            // n_radii, or null
  int nb, r0;
  float* out;            // k_c2r_plain output (N^3)
  float scale;           // k_c2r_plain scale
};

// h_R along z -> half spectrum: main into slot b, X[H] into the slot's
// transposed Nyquist scratch (offset NN*(H+1)).
template <int N>
__global__ void __launch_bounds__(LK<N>::THREADS, LK<N>::MINB) k_adj_z(AdjArgs a) {
  using KK = LK<N>;
  constexpr int H = N / 2, E = KK::E, G = KK::G, NG = KK::NG;
  constexpr long long NN = (long long)N * N;
  extern __shared__ float4 smem4[];
  float2* tw = reinterpret_cast<float2*>(smem4);
  float2* tws = tw + N;
  load_tw(tw, a.tw, N);
  PlanRun<typename KK::P>::template fill<2>(tws, a.tw);
  __syncthreads();
  __shared__ double red[kMaxBatch];
  if (threadIdx.x < kMaxBatch) red[threadIdx.x] = 0.0;
  __syncthreads();
  const int g = threadIdx.x / G, t = threadIdx.x % G;
  float2* gbuf = tws + KK::TW + g * KK::gsize;
  GroupSync<G> sync(g);
  const int lines = N * N;
  const bool want_db = a.dB != nullptr;
  for (int s = blockIdx.x; s * NG < lines; s += gridDim.x) {
    const int l = s * NG + g;
    const bool valid = l < lines;
    const int lv = valid ? l : 0;
    const float2* gl = reinterpret_cast<const float2*>(a.g + (long long)lv * N);
    const uchar2* al = reinterpret_cast<const uchar2*>(a.am + (long long)lv * N);
    for (int b = 0; b < a.nb; ++b) {
      const uint8_t rid = (uint8_t)(a.r0 + b);
      float2 v[E];
      float part = 0.f;
#pragma unroll
      for (int m = 0; m < E; ++m) {
        const int p = t + G * m;
        float2 gv = valid ? __ldg(gl + p) : make_float2(0.f, 0.f);
        uchar2 u = valid ? al[p] : make_uchar2(255, 255);
        const float h0 = (u.x == rid) ? gv.x : 0.f;
        const float h1 = (u.y == rid) ? gv.y : 0.f;
        part += h0 + h1;
        v[m] = make_float2(a.A * h0, a.A * h1);
      }
      if (want_db) {
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) part += __shfl_xor_sync(0xffffffffu, part, o);
        if ((threadIdx.x & 31) == 0) atomicAdd(&red[b], (double)part);
      }
      const float xh = line_r2c<N>(v, gbuf, t, tw, tws, sync);
      if (valid) {
        float2* slot = a.slots + (long long)b * a.slot_stride;
        float2* dst = slot + (long long)l * H;
#pragma unroll
        for (int m = 0; m < E; ++m) dst[t + G * m] = v[m];
        if (t == 0) {
          const int ix = l / N, iy = l - (l / N) * N;
          slot[NN * (H + 1) + (long long)iy * N + ix] = make_float2(xh, 0.f);
        }
      }
    }
  }
  if (want_db) {
    __syncthreads();
    if (threadIdx.x < a.nb) atomicAdd(&a.dB[a.r0 + threadIdx.x], (double)a.A * red[threadIdx.x]);
  }
}

// Plain inverse z pass: slot 0 (main + transposed Nyquist) -> out = scale * x.
template <int N>
__global__ void __launch_bounds__(LK<N>::THREADS, LK<N>::MINB) k_c2r_plain(AdjArgs a) {
  using KK = LK<N>;
  constexpr int H = N / 2, E = KK::E, G = KK::G, NG = KK::NG;
  constexpr long long NN = (long long)N * N;
  extern __shared__ float4 smem4[];
  float2* tw = reinterpret_cast<float2*>(smem4);
  float2* tws = tw + N;
  load_tw(tw, a.tw, N);
  PlanRun<typename KK::P>::template fill<2>(tws, a.tw);
  __syncthreads();
  const int g = threadIdx.x / G, t = threadIdx.x % G;
  float2* gbuf = tws + KK::TW + g * KK::gsize;
  GroupSync<G> sync(g);
  const int lines = N * N;
  for (int s = blockIdx.x; s * NG < lines; s += gridDim.x) {
    const int l = s * NG + g;
    const bool valid = l < lines;
    const int lv = valid ? l : 0;
    const int ix = lv / N, iy = lv % N;
    const float2* src = a.slots + (long long)lv * H;
    float2 v[E];
#pragma unroll
    for (int m = 0; m < E; ++m) v[m] = valid ? __ldg(src + t + G * m) : make_float2(0.f, 0.f);
    float2 xn = make_float2(0.f, 0.f);
    if (t == 0 && valid) xn = __ldg(a.slots + NN * H + (long long)iy * N + ix);
    line_c2r<N>(v, xn, gbuf, t, tw, tws, sync);
    if (valid) {
      float2* dst = reinterpret_cast<float2*>(a.out + (long long)l * N);
#pragma unroll
      for (int m = 0; m < E; ++m) dst[t + G * m] = make_float2(a.scale * v[m].x, a.scale * v[m].y);
    }
  }
}

}  // namespace prc
