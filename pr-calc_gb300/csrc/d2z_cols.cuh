// d2z_cols.cuh — column passes with one lane per column (grids with N >= 32
// and H a multiple of the tile width).
//
// A tile is T adjacent columns x N rows (T = 16; 8 in the window pass at
// N = 512 and in every pass at N = 768 and 1024).  Thread
// (t, c) of a CTA of T*G threads holds rows t + G*m (m < E) of column c in
// registers: T lanes of a warp are the T columns of one row, so every global
// load and store is a whole row segment (128 or 64 bytes) and the data go
// straight from HBM into the FFT registers and back, with no shared-memory
// staging of the tile.  Only the Stockham exchanges touch shared memory: row
// p of column c lives at p*T + c (T = 8: with a row swizzle), so a half-warp
// touches 16 words in distinct banks, and the CTA alternates between two
// exchange buffers so that each exchange costs one barrier.  A warp holds FFT
// lanes t and G - t together; their rows ix and N - ix have the same |k|, so
// the window is evaluated once per mirror pair and handed over with one
// shuffle.
//
// Modes as in k_tile: TM_FWD / TM_INV plain transforms (blockIdx.y selects a
// slot; the next tile is loaded into registers while the current one is
// transformed), TM_WIN (spectrum tile read once, then per radius: window,
// inverse transform, store to the radius slot; the next tile's load is issued
// during the last radius), TM_ACC (per radius: forward transform of the slot
// tile, accumulate W_b times it; one read-modify-write of the output).
#pragma once
#include <type_traits>

#include "d2z_kernels.cuh"

namespace prc {

// Plan and tile width T (columns).  T = 16: the half-warps are the two FFT
// lanes t, G - t of a mirror pair.  T = 8 (G = 32 or 64): a half-warp holds
// lanes t and t + G/4 (8 columns each), its partner half-warp the mirrors
// G - t and G - t - G/4; rows of 64 bytes are swizzled (PPCol::swz) so that the
// two rows of a half-warp always sit in opposite bank halves.  The window pass
// at N = 512 uses T = 8: two 256-thread CTAs per SM instead of one of 512, so
// one CTA issues while the other waits at a barrier.
// TWIN / PWIN: tile width and plan of the window pass (default T / P).  (At
// N = 512 an 8-element window plan, <8,8,8> with 64-lane groups in two
// 512-thread CTAs of 64 registers, measured 7% slower than <16,16,2>.)
template <int N> struct CCfg { static constexpr bool on = false; };
template <class C, class = void> struct WinPlan { using type = typename C::P; };
template <class C> struct WinPlan<C, decltype(void(sizeof(typename C::PWIN)))> { using type = typename C::PWIN; };
template <class P> struct FirstRadix;
template <int E, int R0, int... R> struct FirstRadix<Plan<E, R0, R...>> { static constexpr int v = R0; };
constexpr int ilog2(int x) { return x <= 1 ? 0 : 1 + ilog2(x / 2); }
template <> struct CCfg<32> { static constexpr bool on = true; using P = Plan<16, 16, 2>; static constexpr int T = 16, TWIN = 16; };
template <> struct CCfg<64> { static constexpr bool on = true; using P = Plan<16, 16, 4>; static constexpr int T = 16, TWIN = 16; };
template <> struct CCfg<96> { static constexpr bool on = true; using P = Plan<12, 12, 4, 2>; static constexpr int T = 16, TWIN = 16; };
template <> struct CCfg<128> { static constexpr bool on = true; using P = Plan<16, 16, 8>; static constexpr int T = 16, TWIN = 16; };
template <> struct CCfg<192> { static constexpr bool on = true; using P = Plan<12, 12, 4, 4>; static constexpr int T = 16, TWIN = 16; };
template <> struct CCfg<256> { static constexpr bool on = true; using P = Plan<16, 16, 16>; static constexpr int T = 16, TWIN = 16; };
template <> struct CCfg<384> { static constexpr bool on = true; using P = Plan<12, 12, 4, 4, 2>; static constexpr int T = 16, TWIN = 16; };
template <> struct CCfg<512> { static constexpr bool on = true; using P = Plan<16, 16, 16, 2>; static constexpr int T = 16, TWIN = 8; };
// N = 768: 64 lanes x 8 columns, as at 1024.
template <> struct CCfg<768> { static constexpr bool on = true; using P = Plan<12, 4, 4, 4, 12>; static constexpr int T = 8, TWIN = 8; };
// N = 1024: 64 lanes x 8 columns in every pass.  (Measured no faster: plain
// passes on 32 lanes x 16 columns with 32 elements a lane, and on 64 lanes x 16
// columns in 1024-thread CTAs of 64 registers -- both 128-byte rows, one
// exchange buffer, no register prefetch -- 1-2% slower over the whole step.)
template <> struct CCfg<1024> { static constexpr bool on = true; using P = Plan<16, 16, 16, 4>; static constexpr int T = 8, TWIN = 8; };

// PPF: -1 two exchange buffers when they fit, 0 one; MINB_: resident CTAs per
// SM the registers are sized for (0: by the CTA size).
template <int N, int T_ = CCfg<N>::T, class P_ = typename CCfg<N>::P, int PPF = -1, int MINB_ = 0> struct CK {
  using P = P_;
  static constexpr int H = N / 2, T = T_, E = P::E, G = N / E, THREADS = T * G;
  static_assert(PlanRun<P>::L == N, "column plan length");
  static_assert(G % 2 == 0 && H % T == 0, "column tile shape");
  static_assert(T == 16 || (T == 8 && (G == 64 || G == 32)), "lane layouts: T = 16, or T = 8 with G = 32 or 64");
  static constexpr int EH = E / 2;
  static constexpr int TW = (PlanRun<P>::TW + 1) & ~1;  // stage twiddles, even for alignment
  static constexpr int BUF = N * T;                     // one exchange buffer
  // two exchange buffers (one barrier per exchange) when they fit in shared
  // memory, else one (two barriers per exchange: 1024 rows x 16 columns)
  static constexpr bool PP = PPF >= 0 ? PPF == 1 : (TW + 2 * BUF) * 8 <= 200 * 1024;
  static constexpr int smem_f2 = TW + (PP ? 2 : 1) * BUF;
  // resident CTAs per SM the register budget is sized for (E = 8: two 512-thread CTAs)
  static constexpr int MINB = MINB_ > 0 ? MINB_ : THREADS >= 512 ? (E <= 8 ? 2 : 1) : (THREADS >= 256 ? 2 : 4);
};

// Two exchange buffers, column c: row p at (p ^ swz(p))*T + c.  swz is linear
// over GF(2), so rows split as tp | cp (disjoint bits) address as
// thread(tp) ^ ((cp ^ swz(cp))*T): one XOR per access.  T = 8 flips the row
// parity by bits q and q + 4 of p, q = log2(G/4) (checked for every read and
// store pattern of the N = 512 and N = 1024 plans: one wavefront per
// half-warp access); q + 4 is q + log2(first radix) in general.
template <int T, int G, int R0> struct PPCol {
  float2* b;
  int other;  // offset to the other buffer
  static constexpr int LQ = ilog2(G / 4);      // the bit that tells the two lanes of a half-warp apart
  static constexpr int LS = LQ + ilog2(R0);    // where the first stage's stores move that bit
  static __device__ __forceinline__ constexpr int swz(int p) {
    return T == 8 ? (((p >> LQ) ^ (p >> LS)) & 1) : 0;
  }
  __device__ __forceinline__ int thread(int tp) const { return (tp ^ swz(tp)) * T; }
  __device__ __forceinline__ float2 get(int h, int cp) const { return b[h ^ ((cp ^ swz(cp)) * T)]; }
  __device__ __forceinline__ void put(int h, int cp, float2 v) const { b[h ^ ((cp ^ swz(cp)) * T)] = v; }
  __device__ __forceinline__ float2 get_pos(int p) const { return b[(p ^ swz(p)) * T]; }
  __device__ __forceinline__ void put_pos(int p, float2 v) const { b[(p ^ swz(p)) * T] = v; }
  __device__ __forceinline__ void flip() {
    b += other;
    other = -other;
  }
};

struct CtaSync {
  __device__ __forceinline__ void operator()() const { __syncthreads(); }
};

// Window-pass variants (tile width, plan) the autotuner chooses among.
// Variant 0 is the default (TWIN / PWIN); up to kWinVariants per grid size.
// PPF / MINB as in CK.  (At N = 512, 8-column tiles re-read from L1 for every
// radius instead of held in registers, in three 256-thread CTAs per SM with
// one or two exchange buffers, measured 9.3-9.8 ms per 32-radius launch
// against 5.05 ms for the register-held tile: at 80 registers the transform
// spills, and the re-reads wait in its critical path.)
constexpr int kWinVariants = 3;
// (A variant that reads W(|k| R_b) from a per-sweep table over the integer
// |m|^2, filled with the same arithmetic so the results were bit-identical,
// was measured at N = 256 and 512 and left out: the table reads are gathers
// that miss L1, 8.9 against 5.2 ms per 32-radius launch at 512.)
struct WinDef { static constexpr int PPF = -1, MINB = 0; };
template <int N, int V> struct WinVar : WinDef { static constexpr bool on = false; static constexpr int T = 16; using P = void; };
template <int N> struct WinVar<N, 0> : WinDef {
  static constexpr bool on = CCfg<N>::on;
  static constexpr int T = CCfg<N>::TWIN;
  using P = typename WinPlan<CCfg<N>>::type;
};
template <> struct WinVar<128, 1> : WinDef { static constexpr bool on = true; static constexpr int T = 16; using P = Plan<8, 8, 4, 4>; };
template <> struct WinVar<256, 1> : WinDef { static constexpr bool on = true; static constexpr int T = 16; using P = Plan<8, 8, 8, 4>; };
template <> struct WinVar<256, 2> : WinDef { static constexpr bool on = true; static constexpr int T = 8; using P = Plan<8, 8, 8, 4>; };
template <> struct WinVar<512, 1> : WinDef { static constexpr bool on = true; static constexpr int T = 16; using P = Plan<16, 16, 16, 2>; };
template <> struct WinVar<512, 2> : WinDef { static constexpr bool on = true; static constexpr int T = 8; using P = Plan<8, 8, 8, 8>; };
// The faithful float window (PRC_FLAG_FAITHFUL_WINDOW) on variant 0's tiles
// and plan: a launch code beside the variants, never chosen by the autotuner.
constexpr int kWinFaithful = 7;
template <int N> struct WinVar<N, kWinFaithful> : WinVar<N, 0> {};

// Grid sizes whose window pass may split a sweep's radii over blockIdx.y
// (radius_range): up to 128, where the tiles do not fill two waves of CTAs.
// Larger grids keep the plain loop (at 512 the split's extra live register
// would make the window pass spill).
template <int N> constexpr bool kWinRadiusSplit = N <= 128;

// Tile width and plan of a mode: the window pass uses its variant V, and the
// accumulate mode uses variant 0 of the window pass when the plain plan holds
// more than 16 elements a lane (its accumulator would not fit beside them).
template <int N, int MODE> struct ColUsesWin {
  static constexpr bool v =
      MODE == TM_WIN || (MODE == TM_ACC && (CCfg<N>::P::E > 16 || CCfg<N>::T * (N / CCfg<N>::P::E) > 512));
};
template <int N, int MODE, int V> struct ColK {
  static constexpr int VV = MODE == TM_WIN ? V : 0;
  using type = typename std::conditional<ColUsesWin<N, MODE>::v,
                                         CK<N, WinVar<N, VV>::T, typename WinVar<N, VV>::P, WinVar<N, VV>::PPF,
                                            WinVar<N, VV>::MINB>,
                                         CK<N, CCfg<N>::T, typename CCfg<N>::P>>::type;
};

// MB (grouped launch): the tiles of a.nbox boxes of this grid size, box i's
// segment pointers, radius count and dk * R_b from a.box[i]; tile ti is tile
// ti mod (tiles of one box) of box ti / (tiles of one box).  The inverse y
// pass takes slot blockIdx.y of the first a.nvb[blockIdx.y] boxes (those with
// more than blockIdx.y slots: the boxes are sorted by nb, largest first).
template <int N, int MODE, int V = 0, bool MB = false>
__global__ void __launch_bounds__(ColK<N, MODE, V>::type::THREADS, ColK<N, MODE, V>::type::MINB) k_col(TileArgs a) {
  using KK = typename ColK<N, MODE, V>::type;
  using P = typename KK::P;
  constexpr int H = N / 2, E = KK::E, G = KK::G, T = KK::T, EH = KK::EH;
  constexpr bool INV = (MODE == TM_INV || MODE == TM_WIN);
  extern __shared__ float4 smem4[];
  float2* tws = reinterpret_cast<float2*>(smem4);
  __shared__ float s_kr[kMaxBatch];
  if constexpr (MODE == TM_WIN || MODE == TM_ACC) stage_params(s_kr, a.kr);
  PlanRun<P>::template fill<1>(tws, a.tw);
  __syncthreads();
  const int lane = threadIdx.x & 31, wp = threadIdx.x >> 5, c = lane & (T - 1);
  int t;
  if constexpr (T == 16) {
    t = (lane < 16) ? wp : (wp == 0 ? G / 2 : G - wp);
  } else {
    // half-warp 0: lanes w, w + G/4; half-warp 1: their mirrors G - w, G - G/4 - w
    constexpr int Q = G / 4;
    const int sl = (lane >> 3) & 1;
    t = (lane < 16) ? (sl ? wp + Q : wp) : (sl ? G - Q - wp : (wp ? G - wp : G / 2));
  }
  PPCol<T, G, FirstRadix<P>::v> buf{tws + KK::TW + c, KK::BUF};
  const CtaSync sync;
  static_assert(!MB || MODE != TM_ACC, "no grouped adjoint pass");
  const long long yoff = (MODE == TM_FWD || MODE == TM_INV) ? (long long)blockIdx.y * a.slot_stride : 0;
  const int tiles0 = a.seg[0].n_outer * a.seg[0].tpo;
  const int tpb = tiles0 + a.seg[1].n_outer * a.seg[1].tpo;  // tiles of one box
  const int tiles = !MB ? tpb : tpb * (MODE == TM_INV ? a.nvb[blockIdx.y] : a.nbox);

  // A tile: its segment (0 main, 1 Nyquist plane), outer index, column
  // block and offset; the segment's fields are read from the kernel
  // parameters when used (selected, never indexed, so they stay in the
  // parameter bank) rather than held in registers across the radii.
  struct WhereS {
    int sn, outer, tc;
    long long off;
  };
  struct WhereM : WhereS {
    int bx;  // the tile's box (grouped launches)
  };
  using Where = typename std::conditional<MB, WhereM, WhereS>::type;
  auto where = [&](int ti) {
    Where w;
    if constexpr (MB) {
      w.bx = ti / tpb;
      ti -= w.bx * tpb;
    }
    w.sn = ti >= tiles0;
    const int tl = w.sn ? ti - tiles0 : ti;
    const int tpo = w.sn ? a.seg[1].tpo : a.seg[0].tpo;
    w.outer = tl / tpo;
    w.tc = tl - w.outer * tpo;
    w.off = (long long)w.outer * (w.sn ? a.seg[1].outer_stride : a.seg[0].outer_stride) + (long long)w.tc * T;
    return w;
  };
  auto sg_in = [&](const Where& w) -> const float2* {
    if constexpr (MB) {
      const BoxCol* bc = a.box + w.bx;
      return w.sn ? bc->in1 : bc->in0;
    } else {
      return w.sn ? a.seg[1].in : a.seg[0].in;
    }
  };
  auto sg_out = [&](const Where& w) -> float2* {
    if constexpr (MB) {
      const BoxCol* bc = a.box + w.bx;
      return w.sn ? bc->out1 : bc->out0;
    } else {
      return w.sn ? a.seg[1].out : a.seg[0].out;
    }
  };
  auto sg_rs = [&](const Where& w) { return w.sn ? a.seg[1].row_stride : a.seg[0].row_stride; };
  auto sg_nyq = [&](const Where& w) { return w.sn ? a.seg[1].nyq : a.seg[0].nyq; };
  auto gload = [&](const float2* base, int rs, float2 (&v)[E]) {
    const float2* p = base + (long long)t * rs + c;
    const long long step = (long long)G * rs;
#pragma unroll
    for (int m = 0; m < E; ++m) v[m] = __ldg(p + m * step);
  };
  auto gstore = [&](const Where& w, float2* dst, const float2 (&v)[E]) {
    if (w.sn ? a.seg[1].transpose : a.seg[0].transpose) {
      float2* q = dst + (long long)w.outer * (w.sn ? a.seg[1].outer_stride : a.seg[0].outer_stride) +
                  (long long)(w.tc * T + c) * N + t;
#pragma unroll
      for (int m = 0; m < E; ++m) q[G * m] = v[m];
    } else {
      const int rs = sg_rs(w);
      float2* q = dst + w.off + (long long)t * rs + c;
      const long long step = (long long)G * rs;
#pragma unroll
      for (int m = 0; m < E; ++m) q[m * step] = v[m];
    }
  };
  // |k| of rows t + G*m, m <= E/2, of this thread's column (-1: k = 0)
  auto kmag = [&](const Where& w, float (&kq)[EH + 1]) {
    const int col = w.tc * T + c;
    const int syz = sg_nyq(w) ? fsq(col, N) + H * H : fsq(w.outer, N) + col * col;
#pragma unroll
    for (int m = 0; m <= EH; ++m) {
      const int m2 = fsq(t + G * m, N) + syz;
      kq[m] = (m2 == 0) ? -1.f : sqrtf((float)m2);
    }
  };
  // rows m > E/2 mirror rows of the partner lane (lane ^ 16, FFT lane G - t,
  // register E-1-m) or of this lane (t = 0: E-m; t = G/2: E-1-m)
  auto mirror = [&](float (&wv)[E]) {
#pragma unroll
    for (int m = EH + 1; m < E; ++m) {
      const float o = __shfl_xor_sync(0xffffffffu, wv[E - 1 - m], 16);
      wv[m] = (t == 0) ? wv[E - m] : (t == G / 2 ? wv[E - 1 - m] : o);
    }
  };
  // the smallest kq of the warp
  auto warp_kmin = [&](const float (&kq)[EH + 1]) {
    float k = kq[0];
#pragma unroll
    for (int m = 1; m <= EH; ++m) k = fminf(k, kq[m]);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) k = fminf(k, __shfl_xor_sync(0xffffffffu, k, o));
    return k;
  };
  // W(|k| R_b) of all E rows.  The Taylor branch runs only in warps where
  // some lane needs it: where kmin kr < 1, kmin the warp's smallest kq (-1
  // where the warp holds k = 0, which then always takes it, as a per-lane
  // test would; the result is the same, row by row).
  // zero_in_taylor: k = 0 (kq = -1) makes kmin negative, so its warp always
  // takes the Taylor branch, and W(0) = 0 is set there; otherwise after it,
  // row by row (the accumulate pass keeps that form: it holds fewer registers)
  auto wvals = [&](const float (&kq)[EH + 1], float kmin, float kr, float (&wv)[E], bool zero_in_taylor) {
#pragma unroll
    for (int m = 0; m <= EH; ++m) wv[m] = tophat_big(kq[m] * kr);
    if (kmin * kr < 1.0f) {
#pragma unroll
      for (int m = 0; m <= EH; ++m) {
        const float x = kq[m] * kr;
        if (x < 1.0f) wv[m] = (zero_in_taylor && kq[m] < 0.f) ? 0.f : tophat_small(x);
      }
    }
    if (!zero_in_taylor) {
#pragma unroll
      for (int m = 0; m <= EH; ++m)
        if (kq[m] < 0.f) wv[m] = 0.f;
    }
    mirror(wv);
  };

  if constexpr ((MODE == TM_FWD || MODE == TM_INV) && E <= 16 && KK::THREADS <= 512) {
    float2 v[E], nx[E];
    int ti = blockIdx.x;
    if (ti < tiles) {
      const Where w = where(ti);
      gload(sg_in(w) + w.off + yoff, sg_rs(w), v);
    }
    for (; ti < tiles; ti += gridDim.x) {
      const Where w = where(ti);
      const int tn = ti + gridDim.x;
      if (tn < tiles) {
        const Where wn = where(tn);
        gload(sg_in(wn) + wn.off + yoff, sg_rs(wn), nx);
      }
      PlanRun<P>::template run<INV, KK::PP>(v, buf, t, tws, sync);
      gstore(w, sg_out(w) + yoff, v);
#pragma unroll
      for (int m = 0; m < E; ++m) v[m] = nx[m];
    }
  } else if constexpr (MODE == TM_FWD || MODE == TM_INV) {
    // 32 elements a lane, or 1024-thread CTAs with 64 registers: no room for a
    // prefetch; the independent loads of every lane keep enough bytes in flight
    for (int ti = blockIdx.x; ti < tiles; ti += gridDim.x) {
      const Where w = where(ti);
      float2 v[E];
      gload(sg_in(w) + w.off + yoff, sg_rs(w), v);
      PlanRun<P>::template run<INV, KK::PP>(v, buf, t, tws, sync);
      gstore(w, sg_out(w) + yoff, v);
    }
  } else if constexpr (MODE == TM_WIN) {
    // FW: the reference's float window, every row evaluated on its own
    constexpr bool FW = (V == kWinFaithful);
    float2 raw[E];
    int ti = blockIdx.x;
    if (ti < tiles) {
      const Where w = where(ti);
      gload(sg_in(w) + w.off, sg_rs(w), raw);
    }
    for (; ti < tiles; ti += gridDim.x) {
      const Where w = where(ti);
      float kq[FW ? E : EH + 1];
      float kmin = 0.f;
      if constexpr (FW) {
        const int col = w.tc * T + c;
        const int iy = sg_nyq(w) ? col : w.outer, iz = sg_nyq(w) ? H : col;
#pragma unroll
        for (int m = 0; m < E; ++m) kq[m] = rk_faithful(t + G * m, iy, iz, N, a.dk, a.kmax);
      } else {
        kmag(w, kq);
        kmin = warp_kmin(kq);
      }
      auto radius = [&](int b, bool last) {
        float wv[E];
        float krb;
        if constexpr (MB) krb = __ldg(&a.box[w.bx].kr[b]);
        else krb = s_kr[b];
        if constexpr (FW) {
#pragma unroll
          for (int m = 0; m < E; ++m) wv[m] = window_faithful(kq[m], krb);
        } else {
          // (at N = 1024 the folded form costs 8 bytes of spills: keep the other)
          wvals(kq, kmin, krb, wv, N != 1024);
        }
        float2 v[E];
#pragma unroll
        for (int m = 0; m < E; ++m) v[m] = cscale(raw[m], wv[m]);
        if (last) {
          // raw and kq are dead: the next tile's loads overlap this radius
          const int tn = ti + gridDim.x;
          if (tn < tiles) {
            const Where wn = where(tn);
            gload(sg_in(wn) + wn.off, sg_rs(wn), raw);
          }
        }
        PlanRun<P>::template run<true, KK::PP>(v, buf, t, tws, sync);
        gstore(w, sg_out(w) + (long long)b * a.slot_stride, v);
      };
      // the last radius is peeled so that kq's and raw's live ranges end before it
      int b0 = 0, b1;
      if constexpr (MB) b1 = __ldg(&a.box[w.bx].nb);
      else if constexpr (kWinRadiusSplit<N>) radius_range(a.nb, b0, b1);
      else b1 = a.nb;
      for (int b = b0; b < b1 - 1; ++b) radius(b, false);
      radius(b1 - 1, true);
    }
  } else {  // TM_ACC (output never transposed)
    for (int ti = blockIdx.x; ti < tiles; ti += gridDim.x) {
      const Where w = where(ti);
      float kq[EH + 1];
      kmag(w, kq);
      const float kmin = warp_kmin(kq);
      float2 acc[E];
#pragma unroll
      for (int m = 0; m < E; ++m) acc[m] = make_float2(0.f, 0.f);
      for (int b = 0; b < a.nb; ++b) {
        float2 v[E];
        gload(sg_in(w) + w.off + (long long)b * a.slot_stride, sg_rs(w), v);
        PlanRun<P>::template run<false, KK::PP>(v, buf, t, tws, sync);
        float wv[E];
        wvals(kq, kmin, s_kr[b], wv, false);
#pragma unroll
        for (int m = 0; m < E; ++m) {
          acc[m].x = fmaf(wv[m], v[m].x, acc[m].x);
          acc[m].y = fmaf(wv[m], v[m].y, acc[m].y);
        }
      }
      const int rs = sg_rs(w);
      float2* q = sg_out(w) + w.off + (long long)t * rs + c;
      const long long step = (long long)G * rs;
#pragma unroll
      for (int m = 0; m < E; ++m) {
        float2 o = a.first ? make_float2(0.f, 0.f) : q[m * step];
        q[m * step] = make_float2(o.x + acc[m].x, o.y + acc[m].y);
      }
    }
  }
}

}  // namespace prc
