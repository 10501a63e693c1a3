// fft.cuh — register/shared-memory Stockham FFT building blocks for sm_103a.
//
// One FFT of length L is carried by a *group* of G = L/E threads; thread t of
// the group holds the E elements at positions t + G*m (m = 0..E-1).  A mixed-radix Stockham autosort (Govindaraju et al., "High
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
// built in FP64 on the host, rounded to FP32), re-laid out per stage in shared
// memory (TwFill) so that a warp's twiddle reads hit distinct banks.
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

// Radix 12 by the Good-Thomas prime-factor map (12 = 3 x 4, coprime): input
// n = (4 n1 + 3 n2) mod 12, output k = (4 k1 + 9 k2) mod 12, so that
// w12^{nk} = w3^{n1 k1} w4^{n2 k2} and the 12-point DFT is four 3-point DFTs
// followed by three 4-point DFTs with no twiddles between them (8 FP
// instructions a point against about 10 for a radix-3 and a radix-4 stage
// with the stage twiddles between them, and one shared-memory exchange less).
template <bool INV> struct Dft<12, INV> {
  static __device__ __forceinline__ void run(float2* a) {
    float2 y[4][3];
#pragma unroll
    for (int n2 = 0; n2 < 4; ++n2) {
      float2 b[3] = {a[(3 * n2) % 12], a[(4 + 3 * n2) % 12], a[(8 + 3 * n2) % 12]};
      Dft<3, INV>::run(b);
#pragma unroll
      for (int k1 = 0; k1 < 3; ++k1) y[n2][k1] = b[k1];
    }
#pragma unroll
    for (int k1 = 0; k1 < 3; ++k1) {
      float2 c[4] = {y[0][k1], y[1][k1], y[2][k1], y[3][k1]};
      Dft<4, INV>::run(c);
#pragma unroll
      for (int k2 = 0; k2 < 4; ++k2) a[(4 * k1 + 9 * k2) % 12] = c[k2];
    }
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
  unsigned mask;
  __device__ __forceinline__ explicit GroupSync(int /*group_in_cta*/, unsigned lanes = 0xffffffffu)
      : mask(lanes) {}
  __device__ __forceinline__ void operator()() const { __syncwarp(mask); }
};
template <> struct GroupSync<64> {
  int id;
  __device__ __forceinline__ explicit GroupSync(int g, unsigned = 0xffffffffu) : id(1 + g) {}
  __device__ __forceinline__ void operator()() const {
    asm volatile("bar.sync %0, 64;" ::"r"(id) : "memory");
  }
};

// ---------------------------------------------------------------- smem layout
template <int L, int G = 32> struct GroupBuf {
  // float2 elements per group buffer; groups narrower than one shared-memory
  // wavefront (16 lanes x 8 B) are padded by one group access width so that
  // the groups sharing a wavefront start on other banks
  static constexpr int pad = G < 16 ? G : 0;
  static constexpr int size = L + pad;
};

// A group's exchange buffer of L positions (one column, 8-byte elements).
// Positions are XOR-swizzled inside blocks of 16 (p ^ ((p >> 4) & 15)) when L
// is a multiple of 16.  Because the swizzle is linear over GF(2), a position
// tp | cp made of disjoint thread bits tp and compile-time bits cp maps to
// X(tp) ^ X(cp): the thread part is computed once (thread()) and every access
// costs one XOR with a constant.
template <int L> struct LineBuf {
  float2* sm;
  static constexpr bool on = (L % 16) == 0;
  static __device__ __forceinline__ constexpr int sw(int p) { return on ? (p ^ ((p >> 4) & 15)) : p; }
  __device__ __forceinline__ int thread(int tp) const { return sw(tp); }
  __device__ __forceinline__ float2 get(int h, int cp) const { return sm[h ^ sw(cp)]; }
  __device__ __forceinline__ void put(int h, int cp, float2 v) const { sm[h ^ sw(cp)] = v; }
  __device__ __forceinline__ float2 get_pos(int p) const { return sm[sw(p)]; }
  __device__ __forceinline__ void put_pos(int p, float2 v) const { sm[sw(p)] = v; }
};

template <int X> struct IsPow2 { static constexpr bool v = X > 0 && (X & (X - 1)) == 0; };
template <int... R> struct AllPow2;
template <> struct AllPow2<> { static constexpr bool v = true; };
template <int R0, int... R> struct AllPow2<R0, R...> {
  static constexpr bool v = IsPow2<R0>::v && AllPow2<R...>::v;
};

// ---------------------------------------------------------------- twiddles
// Per-stage twiddle tables.  The stage with span Ns > 1 and radix R reads
// w^{r k}, w = e^{+2 pi i/(Ns R)}, for r = 1..R-1 and k = j mod Ns; it is stored
// as tab[(r-1)*Ns + k] so that the lanes of a warp (consecutive k) read
// consecutive words.  Stage tables follow each other in one array.
template <int L, int Ns, int... Rs> struct TwSize;
template <int L, int Ns> struct TwSize<L, Ns> { static constexpr int v = 0; };
template <int L, int Ns, int R, int... Rest> struct TwSize<L, Ns, R, Rest...> {
  static constexpr int v = (Ns > 1 ? (R - 1) * Ns : 0) + TwSize<L, Ns * R, Rest...>::v;
};

// Fills the stage tables from the N-entry table e^{+2 pi i k/NT}; TWS = NT/L.
template <int L, int TWS, int Ns, int OFF, int... Rs> struct TwFill;
template <int L, int TWS, int Ns, int OFF> struct TwFill<L, TWS, Ns, OFF> {
  static __device__ __forceinline__ void run(float2*, const float2*) {}
};
template <int L, int TWS, int Ns, int OFF, int R, int... Rest> struct TwFill<L, TWS, Ns, OFF, R, Rest...> {
  static __device__ __forceinline__ void run(float2* tab, const float2* tabN) {
    if constexpr (Ns > 1) {
      constexpr int STEP = (L / (Ns * R)) * TWS;
      for (int i = threadIdx.x; i < (R - 1) * Ns; i += blockDim.x) {
        const int r = i / Ns + 1, k = i - (i / Ns) * Ns;
        tab[OFF + i] = tabN[r * k * STEP];
      }
    }
    TwFill<L, TWS, Ns * R, OFF + (Ns > 1 ? (R - 1) * Ns : 0), Rest...>::run(tab, tabN);
  }
};

// ---------------------------------------------------------------- Stockham
// Buf provides thread(tp) / get(h, cp) / put(h, cp, v) for split positions and
// get_pos / put_pos for general ones; SPLIT (power-of-two G and radices)
// selects the former.  tws: the stage twiddle tables, OFF this stage's offset.
// PP (ping-pong): Buf holds two exchange buffers and flip() swaps them after
// each exchange, so one barrier per exchange suffices (the next exchange
// writes the other buffer, which every thread finished reading before the
// barrier it has just passed).
template <int L, int E, bool INV, bool SPLIT, bool PP, int Ns, int OFF, int... Rs> struct Stages;

template <int L, int E, bool INV, bool SPLIT, bool PP, int Ns, int OFF> struct Stages<L, E, INV, SPLIT, PP, Ns, OFF> {
  template <class Buf, class Sync>
  static __device__ __forceinline__ void run(float2 (&)[E], Buf&, int, const float2*, const Sync&) {}
};

template <int L, int E, bool INV, bool SPLIT, bool PP, int Ns, int OFF, int R, int... Rest>
struct Stages<L, E, INV, SPLIT, PP, Ns, OFF, R, Rest...> {
  template <class Buf, class Sync>
  static __device__ __forceinline__ void run(float2 (&v)[E], Buf& buf, int t, const float2* tws,
                                             const Sync& sync) {
    constexpr int G = L / E;
    constexpr int Q = E / R;
    static_assert(E % R == 0, "radix must divide the per-thread element count");
    constexpr bool last = (Ns * R == L);
    constexpr int NG = (Ns > G) ? Ns / G : 1;
    // Store positions split into thread bits and constant bits: with Ns <= G,
    // (t/Ns)*Ns*R + t%Ns  |  q*G*R + r*Ns; with Ns > G, t  |  (q/NG)*Ns*R +
    // G*(q%NG) + r*Ns.
    int hw = 0;
    if constexpr (SPLIT && !last) hw = buf.thread(Ns <= G ? (t / Ns) * Ns * R + (t % Ns) : t);
#pragma unroll
    for (int q = 0; q < Q; ++q) {
      const int j = t + G * q;
      const int k = (Ns == 1) ? 0 : (j % Ns);
      float2 a[R];
#pragma unroll
      for (int r = 0; r < R; ++r) a[r] = v[q + r * Q];
      if constexpr (Ns > 1) {
#pragma unroll
        for (int r = 1; r < R; ++r) a[r] = cmul(a[r], twid<INV>(tws[OFF + (r - 1) * Ns + k]));
      }
      Dft<R, INV>::run(a);
      if constexpr (last) {
#pragma unroll
        for (int r = 0; r < R; ++r) v[q + r * Q] = a[r];
      } else if constexpr (SPLIT) {
#pragma unroll
        for (int r = 0; r < R; ++r)
          buf.put(hw, (Ns <= G) ? (q * G * R + r * Ns) : ((q / NG) * Ns * R + G * (q % NG) + r * Ns), a[r]);
      } else {
        const int base = (j / Ns) * Ns * R + k;
#pragma unroll
        for (int r = 0; r < R; ++r) buf.put_pos(base + r * Ns, a[r]);
      }
    }
    if constexpr (!last) {
      sync();
      if constexpr (SPLIT) {
        const int hr = buf.thread(t);
#pragma unroll
        for (int m = 0; m < E; ++m) v[m] = buf.get(hr, G * m);
      } else {
#pragma unroll
        for (int m = 0; m < E; ++m) v[m] = buf.get_pos(t + G * m);
      }
      if constexpr (PP) buf.flip();
      else sync();
      Stages<L, E, INV, SPLIT, PP, Ns * R, OFF + (Ns > 1 ? (R - 1) * Ns : 0), Rest...>::run(v, buf, t, tws, sync);
    }
  }
};

template <class P> struct PlanRun;
template <int E, int... R> struct PlanRun<Plan<E, R...>> {
  static constexpr int L = Prod<R...>::v;
  static constexpr int G = L / E;
  static constexpr bool SPLIT = IsPow2<G>::v && AllPow2<R...>::v;
  static constexpr int TW = TwSize<L, 1, R...>::v;  // stage-table entries
  // stage tables from an NT-entry table (TWS = NT / L)
  template <int TWS>
  static __device__ __forceinline__ void fill(float2* tws, const float2* tabN) {
    TwFill<L, TWS, 1, 0, R...>::run(tws, tabN);
  }
  template <bool INV, bool PP = false, class Buf, class Sync>
  static __device__ __forceinline__ void run(float2 (&v)[E], Buf& buf, int t, const float2* tws,
                                             const Sync& sync) {
    Stages<L, E, INV, SPLIT, PP, 1, 0, R...>::run(v, buf, t, tws, sync);
  }
};

}  // namespace prc
