// fft.cuh — register/shared-memory Stockham FFT building blocks for sm_103a.
//
// One FFT of length L is carried by a *group* of G = L/E threads; thread t of
// the group holds the E elements at positions t + G*m (m = 0..E-1) for C
// independent columns (C = 2 lets one 16-byte access fetch two adjacent
// pencils).  A mixed-radix Stockham autosort (Govindaraju et al., "High
// performance discrete Fourier transforms on graphics processors", SC 2008)
// runs stage by stage: with span Ns and radix R, virtual butterfly j reads
// positions j + r*L/R and writes (j/Ns)*Ns*R + j%Ns + r*Ns.  Both the input
// positions of every stage and the output positions of the last stage are
// t + G*m, so the data enter and leave in registers in natural order and only
// the (#stages - 1) inner exchanges touch shared memory.
//
// Sign convention: INV = true is FFTW's backward transform (e^{+2 pi i nk/L}),
// INV = false the forward one (e^{-2 pi i nk/L}); neither is normalised.
// Twiddles come from a table tw[i] = e^{+2 pi i i/NT} (NT = table length,
// built in FP64 on the host, rounded to FP32); an L-point FFT reads it with
// stride NT/L.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace prc {

// ---------------------------------------------------------------- complex
__device__ __forceinline__ float2 cadd(float2 a, float2 b) { return make_float2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ float2 csub(float2 a, float2 b) { return make_float2(a.x - b.x, a.y - b.y); }
__device__ __forceinline__ float2 cscale(float2 a, float s) { return make_float2(a.x * s, a.y * s); }
__device__ __forceinline__ float2 cconj(float2 a) { return make_float2(a.x, -a.y); }
__device__ __forceinline__ float2 cmul(float2 a, float2 b) {
  return make_float2(fmaf(a.x, b.x, -a.y * b.y), fmaf(a.x, b.y, a.y * b.x));
}
// multiply by s*i, s = +1 (INV) or -1
template <bool INV> __device__ __forceinline__ float2 mul_si(float2 a) {
  return INV ? make_float2(-a.y, a.x) : make_float2(a.y, -a.x);
}
// twiddle from the +sign table, conjugated for the forward direction
template <bool INV> __device__ __forceinline__ float2 twid(float2 w) {
  return INV ? w : make_float2(w.x, -w.y);
}

// constants (from their closed forms)
#define PRC_SQRT1_2 0.70710678118654752440f
#define PRC_SQRT3_2 0.86602540378443864676f
#define PRC_COS_PI8 0.92387953251128675613f
#define PRC_SIN_PI8 0.38268343236508977173f

// ---------------------------------------------------------------- small DFTs
template <int R, bool INV> struct Dft;

template <bool INV> struct Dft<2, INV> {
  static __device__ __forceinline__ void run(float2* a) {
    float2 t = a[1];
    a[1] = csub(a[0], t);
    a[0] = cadd(a[0], t);
  }
};

template <bool INV> struct Dft<3, INV> {
  static __device__ __forceinline__ void run(float2* a) {
    float2 t1 = cadd(a[1], a[2]);
    float2 t2 = make_float2(fmaf(-0.5f, t1.x, a[0].x), fmaf(-0.5f, t1.y, a[0].y));
    float2 d = csub(a[1], a[2]);
    float2 t3 = mul_si<INV>(cscale(d, PRC_SQRT3_2));
    a[0] = cadd(a[0], t1);
    a[1] = cadd(t2, t3);
    a[2] = csub(t2, t3);
  }
};

template <bool INV> struct Dft<4, INV> {
  static __device__ __forceinline__ void run(float2* a) {
    float2 t0 = cadd(a[0], a[2]);
    float2 t1 = csub(a[0], a[2]);
    float2 t2 = cadd(a[1], a[3]);
    float2 t3 = mul_si<INV>(csub(a[1], a[3]));
    a[0] = cadd(t0, t2);
    a[2] = csub(t0, t2);
    a[1] = cadd(t1, t3);
    a[3] = csub(t1, t3);
  }
};

// w8^k for k = 1,2,3 applied in place
template <bool INV> __device__ __forceinline__ float2 mul_w8_1(float2 a) {
  // (1 + s i)/sqrt2
  float2 b = mul_si<INV>(a);
  return make_float2((a.x + b.x) * PRC_SQRT1_2, (a.y + b.y) * PRC_SQRT1_2);
}
template <bool INV> __device__ __forceinline__ float2 mul_w8_3(float2 a) {
  // (-1 + s i)/sqrt2
  float2 b = mul_si<INV>(a);
  return make_float2((b.x - a.x) * PRC_SQRT1_2, (b.y - a.y) * PRC_SQRT1_2);
}

template <bool INV> struct Dft<8, INV> {
  static __device__ __forceinline__ void run(float2* a) {
    float2 e[4] = {a[0], a[2], a[4], a[6]};
    float2 o[4] = {a[1], a[3], a[5], a[7]};
    Dft<4, INV>::run(e);
    Dft<4, INV>::run(o);
    o[1] = mul_w8_1<INV>(o[1]);
    o[2] = mul_si<INV>(o[2]);
    o[3] = mul_w8_3<INV>(o[3]);
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      a[k] = cadd(e[k], o[k]);
      a[k + 4] = csub(e[k], o[k]);
    }
  }
};

template <bool INV> struct Dft<16, INV> {
  static __device__ __forceinline__ void run(float2* a) {
    float2 e[8], o[8];
#pragma unroll
    for (int k = 0; k < 8; ++k) { e[k] = a[2 * k]; o[k] = a[2 * k + 1]; }
    Dft<8, INV>::run(e);
    Dft<8, INV>::run(o);
    // o[k] *= w16^k,  w16 = e^{s i pi/8}
    const float s = INV ? 1.f : -1.f;
    o[1] = cmul(o[1], make_float2(PRC_COS_PI8, s * PRC_SIN_PI8));
    o[2] = mul_w8_1<INV>(o[2]);
    o[3] = cmul(o[3], make_float2(PRC_SIN_PI8, s * PRC_COS_PI8));
    o[4] = mul_si<INV>(o[4]);
    o[5] = cmul(o[5], make_float2(-PRC_SIN_PI8, s * PRC_COS_PI8));
    o[6] = mul_w8_3<INV>(o[6]);
    o[7] = cmul(o[7], make_float2(-PRC_COS_PI8, s * PRC_SIN_PI8));
#pragma unroll
    for (int k = 0; k < 8; ++k) {
      a[k] = cadd(e[k], o[k]);
      a[k + 8] = csub(e[k], o[k]);
    }
  }
};

// ---------------------------------------------------------------- plans
template <int E_, int... R> struct Plan {
  static constexpr int E = E_;
};

template <int... R> struct Prod;
template <> struct Prod<> { static constexpr int v = 1; };
template <int R0, int... R> struct Prod<R0, R...> { static constexpr int v = R0 * Prod<R...>::v; };

template <int... R> struct NumStages { static constexpr int v = sizeof...(R); };

// ---------------------------------------------------------------- group sync
// G <= 32: the group lives inside one warp (several groups may share it; all
// groups of a warp always run the same stages, so a full-warp sync is safe).
// G == 64: two warps, synchronised by a named barrier id 1 + group index.
template <int G> struct GroupSync {
  __device__ __forceinline__ explicit GroupSync(int /*group_in_cta*/) {}
  __device__ __forceinline__ void operator()() const { __syncwarp(); }
};
template <> struct GroupSync<64> {
  int id;
  __device__ __forceinline__ explicit GroupSync(int g) : id(1 + g) {}
  __device__ __forceinline__ void operator()() const {
    asm volatile("bar.sync %0, 64;" ::"r"(id) : "memory");
  }
};

// ---------------------------------------------------------------- smem layout
// Group buffer of L positions x C columns.  Positions are swizzled inside
// blocks of 8 (C=2, 16-byte units) or 16 (C=1, 8-byte units) so that the
// stride-R stores of the early stages do not pile onto one bank.
template <int L, int C> struct Swz {
  static constexpr int B = (C == 2) ? 8 : 16;
  static constexpr bool on = (L % B) == 0;
  static __device__ __forceinline__ int f(int p) { return on ? (p ^ ((p / B) & (B - 1))) : p; }
};
template <int L, int C> struct GroupBuf {
  // float2 elements per group buffer, padded so neighbouring groups start on
  // different banks
  static constexpr int size = L * C + 4 * C;
};

template <int L, int C>
__device__ __forceinline__ void sm_put(float2* sm, int pos, const float2 (&a)[C]) {
  int p = Swz<L, C>::f(pos);
  if constexpr (C == 2) {
    reinterpret_cast<float4*>(sm)[p] = make_float4(a[0].x, a[0].y, a[1].x, a[1].y);
  } else {
    sm[p] = a[0];
  }
}
template <int L, int C>
__device__ __forceinline__ void sm_get(const float2* sm, int pos, float2 (&a)[C]) {
  int p = Swz<L, C>::f(pos);
  if constexpr (C == 2) {
    float4 q = reinterpret_cast<const float4*>(sm)[p];
    a[0] = make_float2(q.x, q.y);
    a[1] = make_float2(q.z, q.w);
  } else {
    a[0] = sm[p];
  }
}

// ---------------------------------------------------------------- Stockham
// TWS = table stride (table length / L).
template <int L, int E, int C, bool INV, int TWS, int Ns, int... Rs> struct Stages;

template <int L, int E, int C, bool INV, int TWS, int Ns> struct Stages<L, E, C, INV, TWS, Ns> {
  template <class Sync>
  static __device__ __forceinline__ void run(float2 (&)[C][E], float2*, int, const float2*, const Sync&) {}
};

template <int L, int E, int C, bool INV, int TWS, int Ns, int R, int... Rest>
struct Stages<L, E, C, INV, TWS, Ns, R, Rest...> {
  template <class Sync>
  static __device__ __forceinline__ void run(float2 (&v)[C][E], float2* sm, int t,
                                             const float2* tw, const Sync& sync) {
    constexpr int G = L / E;
    constexpr int Q = E / R;
    static_assert(E % R == 0, "radix must divide the per-thread element count");
    constexpr bool last = (Ns * R == L);
    constexpr int TSTEP = (L / (Ns * R)) * TWS;  // table step per unit of r*k
#pragma unroll
    for (int q = 0; q < Q; ++q) {
      const int j = t + G * q;
      const int k = (Ns == 1) ? 0 : (j % Ns);
      float2 a[C][R];
#pragma unroll
      for (int r = 0; r < R; ++r)
#pragma unroll
        for (int c = 0; c < C; ++c) a[c][r] = v[c][q + r * Q];
      if constexpr (Ns > 1) {
#pragma unroll
        for (int r = 1; r < R; ++r) {
          const float2 w = twid<INV>(tw[r * k * TSTEP]);
#pragma unroll
          for (int c = 0; c < C; ++c) a[c][r] = cmul(a[c][r], w);
        }
      }
#pragma unroll
      for (int c = 0; c < C; ++c) Dft<R, INV>::run(a[c]);
      if constexpr (last) {
#pragma unroll
        for (int r = 0; r < R; ++r)
#pragma unroll
          for (int c = 0; c < C; ++c) v[c][q + r * Q] = a[c][r];
      } else {
        const int base = (j / Ns) * Ns * R + k;
#pragma unroll
        for (int r = 0; r < R; ++r) {
          float2 o[C];
#pragma unroll
          for (int c = 0; c < C; ++c) o[c] = a[c][r];
          sm_put<L, C>(sm, base + r * Ns, o);
        }
      }
    }
    if constexpr (!last) {
      sync();
#pragma unroll
      for (int m = 0; m < E; ++m) {
        float2 o[C];
        sm_get<L, C>(sm, t + G * m, o);
#pragma unroll
        for (int c = 0; c < C; ++c) v[c][m] = o[c];
      }
      sync();
      Stages<L, E, C, INV, TWS, Ns * R, Rest...>::run(v, sm, t, tw, sync);
    }
  }
};

template <class P> struct PlanRun;
template <int E, int... R> struct PlanRun<Plan<E, R...>> {
  static constexpr int L = Prod<R...>::v;
  template <int C, bool INV, int TWS, class Sync>
  static __device__ __forceinline__ void run(float2 (&v)[C][E], float2* sm, int t,
                                             const float2* tw, const Sync& sync) {
    Stages<L, E, C, INV, TWS, 1, R...>::run(v, sm, t, tw, sync);
  }
};

}  // namespace prc
