// d2z_kernels.cuh — the delta2zreion hot path as sm_103a kernels.
//
// Device layout of one box (N = grid side, H = N/2, NN = N*N), in float2 units,
// "slot" size NN*(H+2):
//   main      [0, NN*H)         X[ix][iy][kz], kz < H
//   Nyquist   [NN*H, NN*(H+1))  the kz = H plane; Q[ix][iy] in the spectrum,
//                               transposed Qt[iy][ix] in the radius slots
//   scratch   [NN*(H+1), NN*(H+2)) a transposed copy for the forward y pass
// Column passes (along ix or iy) run on tiles of T adjacent columns x N rows:
// the CTA loads the tile with coalesced 16-byte accesses (a warp covers whole
// 128-byte row segments) into an XOR-swizzled shared-memory tile, one group of
// G threads transforms each column in place, and the CTA writes the tile back
// the same way.  Line passes (along z) give each group one contiguous line and
// use the half-length complex FFT of a real sequence (even samples in .x,
// odd in .y).
//
// Reference steps fused here (pr-calc c++/src):
//   k_r2c_z + k_tile<FWD> (y, x)  main_d2z.C:57-59 (delta /= DInit) and the R2C (:67)
//   k_tile<WIN>   window loop delta2zreion_d2z.C:57-89 + first axis of the C2R (:92)
//   k_tile<INV>   second axis of the C2R
//   k_c2r_z       last axis of the C2R, NormalizeArray (:93), GetMeanSigma (:94),
//                 barrier d2z (:206-216) and the running max (:105-146)
#pragma once
#include "fft.cuh"

namespace prc {

constexpr int kMaxBatch = 64;  // radii per sweep at most
constexpr int kNHistory = 100000;

// ------------------------------------------------------------ per-N plans
// Line plan (length N/2): Plan<E, radices...>.
template <int N> struct LCfg;
template <> struct LCfg<8> { using P = Plan<4, 4>; };
template <> struct LCfg<12> { using P = Plan<6, 3, 2>; };
template <> struct LCfg<16> { using P = Plan<8, 8>; };
template <> struct LCfg<24> { using P = Plan<12, 4, 3>; };
template <> struct LCfg<32> { using P = Plan<8, 8, 2>; };
template <> struct LCfg<48> { using P = Plan<12, 4, 3, 2>; };
template <> struct LCfg<64> { using P = Plan<8, 8, 4>; };
template <> struct LCfg<96> { using P = Plan<12, 12, 4>; };
template <> struct LCfg<128> { using P = Plan<8, 8, 8>; };
template <> struct LCfg<192> { using P = Plan<12, 12, 4, 2>; };
template <> struct LCfg<256> { using P = Plan<8, 8, 4, 4>; };
template <> struct LCfg<384> { using P = Plan<12, 12, 4, 4>; };
template <> struct LCfg<512> { using P = Plan<8, 8, 8, 4>; };
template <> struct LCfg<768> { using P = Plan<12, 12, 4, 4, 2>; };
template <> struct LCfg<1024> { using P = Plan<8, 8, 8, 8>; };

// Tile plan (length N), tile width T (columns; T divides N/2 and N) and the
// two shifts (SA, SB) of the tile swizzle (chosen by simulating the bank
// pattern of every shared-memory access of the plan; SB = 0: unused).
template <int N> struct TCfg;
template <> struct TCfg<8> { using P = Plan<8, 8>; static constexpr int T = 4, SA = 1, SB = 0; };
template <> struct TCfg<12> { using P = Plan<12, 4, 3>; static constexpr int T = 6, SA = 1, SB = 0; };
template <> struct TCfg<16> { using P = Plan<8, 8, 2>; static constexpr int T = 8, SA = 1, SB = 0; };
template <> struct TCfg<24> { using P = Plan<12, 4, 3, 2>; static constexpr int T = 12, SA = 1, SB = 0; };
template <> struct TCfg<32> { using P = Plan<16, 16, 2>; static constexpr int T = 16, SA = 1, SB = 0; };
template <> struct TCfg<48> { using P = Plan<12, 4, 4, 3>; static constexpr int T = 8, SA = 1, SB = 0; };
template <> struct TCfg<64> { using P = Plan<8, 8, 8>; static constexpr int T = 16, SA = 1, SB = 2; };
template <> struct TCfg<96> { using P = Plan<12, 4, 4, 2, 3>; static constexpr int T = 16, SA = 1, SB = 0; };
template <> struct TCfg<128> { using P = Plan<8, 8, 4, 4>; static constexpr int T = 16, SA = 2, SB = 3; };
template <> struct TCfg<192> { using P = Plan<12, 4, 4, 4, 3>; static constexpr int T = 16, SA = 1, SB = 2; };
template <> struct TCfg<256> { using P = Plan<16, 16, 16>; static constexpr int T = 16, SA = 1, SB = 4; };
template <> struct TCfg<512> { using P = Plan<16, 8, 8, 8>; static constexpr int T = 8, SA = 1, SB = 3; };
template <> struct TCfg<1024> { using P = Plan<16, 16, 16, 4>; static constexpr int T = 4, SA = 1, SB = 2; };

template <int N> struct LK {
  static constexpr int H = N / 2;
  using P = typename LCfg<N>::P;
  static constexpr int E = P::E;
  static constexpr int G = H / E;
  static_assert(PlanRun<P>::L == H, "line plan length");
  static constexpr int THREADS = 256;
  static constexpr int MINB = E <= 8 ? 3 : 2;  // resident CTAs per SM the register budget is sized for
  static constexpr int NG = THREADS / G;
  static constexpr int gsize = GroupBuf<H, G>::size;
  static constexpr int TW = (PlanRun<P>::TW + 1) & ~1;  // stage twiddles, even for alignment
  static constexpr int smem_f2 = N + TW + NG * gsize;   // N-table, stage twiddles, group buffers
};

template <int N> struct TK {
  static constexpr int H = N / 2;
  using P = typename TCfg<N>::P;
  static constexpr int T = TCfg<N>::T;
  static constexpr int E = P::E;
  static constexpr int G = N / E;
  static_assert(PlanRun<P>::L == N, "tile plan length");
  static_assert(H % T == 0 && N % T == 0 && T % 2 == 0, "tile width");
  static constexpr int THREADS = T * G;
  static constexpr int TW = (PlanRun<P>::TW + 1) & ~1;  // stage twiddles, even for alignment
  static constexpr int smem_f2 = TW + N * T;            // twiddles + one tile
  static constexpr int smem2_f2 = TW + 2 * N * T;       // twiddles + two tiles (TM_WIN)
  // resident CTAs per SM the register budget is sized for; the accumulate
  // mode keeps E more complex values per thread
  static constexpr int MINB = THREADS >= 512 ? 2 : (THREADS >= 256 ? 3 : 4);
  static constexpr int MINB_ACC = MINB > 1 ? MINB - 1 : 1;
};

// ------------------------------------------------------------ kernel args
struct TileSeg {
  const float2* in;
  float2* out;
  int row_stride;    // float2 between rows (the transform axis)
  int outer_stride;  // float2 between outer indices
  int n_outer;
  int tpo;           // tiles per outer index
  int transpose;     // 1: out[(column)*N + row] (N x N plane)
  int nyq;           // 1: the kz = H plane (window frequencies: fy = column, fz = H)
};

// One box of a grouped column pass (several boxes of one grid size in one
// launch): its segment pointers, radii or slots of this sweep and dk * R_b.
struct BoxCol {
  const float2* in0;
  float2* out0;
  const float2* in1;
  float2* out1;
  int nb;
  float kr[kMaxBatch];
};

struct TileArgs {
  TileSeg seg[2];          // main array, Nyquist plane (grouped: geometry only)
  long long slot_stride;   // plain: per blockIdx.y; WIN: per radius (out); ACC: per radius (in)
  const float2* tw;        // N-entry table e^{+2 pi i k/N}
  int nb, first;
  int win_var;             // window-pass variant (host-side launch choice)
  int faithful;            // window pass: the reference's float window (kr holds R_b)
  float dk, kmax;          // faithful window: dk = 2 pi / box and kmax = dk * N, in float
  float kr[kMaxBatch];     // dk * R_b (faithful window: R_b)
  // grouped launches: the boxes (sorted by nb, largest first), their count,
  // and per slot y of the inverse y pass the number of boxes with nb > y
  const BoxCol* box;
  int nbox;
  int nvb[kMaxBatch];
};

// One box of a grouped inverse z pass.
struct BoxLine {
  float2* slots;
  float* zreion;
  uint8_t* argmax;
  float* zreion_out;
  uint8_t* argmax_out;
  int nb, r0, first;
  float as;
  float cb[kMaxBatch];
};

// One box of a grouped forward z pass.
struct BoxR2c {
  const float* delta;
  float2* S;
  float2* Qt;
  float dinit;
};

struct SweepArgs {
  float2* slots;        // slot 0 base
  long long slot_stride;
  const float2* tw;
  float* zreion;        // N^3: running max read at the start of the sweep
  uint8_t* argmax;      // N^3 or null
  float* zreion_out;    // where the sweep writes it (may be mapped host memory)
  uint8_t* argmax_out;  // likewise for the argmax (null when argmax is null)
  double* sig_acc;      // per-radius sum of x^2 (raw C2R units) or null
  int* err;             // set to 1 when a copy wait ran out (null: not reported)
  int withhold;         // test hook: CTA 0 never issues its first staging copy, so
                        // that its bounded wait runs out (then after kWithheldPolls)
  int nb;               // radii in this sweep
  int r0;               // global index of the first radius
  int first;            // first sweep: zreion/argmax not read
  float as;             // A / N^3
  float cb[kMaxBatch];  // A*B_b - 1 (NaN: never wins)
  // grouped launches: the boxes, whose entries stand in for slots, zreion,
  // argmax, zreion_out, argmax_out, nb, r0, first, as and cb above
  const BoxLine* box;
  int nbox;
};

enum TileMode { TM_FWD = 0, TM_INV = 1, TM_WIN = 2, TM_ACC = 3 };

// ------------------------------------------------------------ helpers
__device__ __forceinline__ int fsq(int f, int n) {
  const int a = (f <= (n >> 1)) ? f : n - f;
  return a * a;
}

// Top-hat window W(x) = 3 (sin x - x cos x) / x^3 (delta2zreion_d2z.C:77).
// x < 1 (tophat_small): the Taylor series sum_m 3 (-1)^m (2m+2) x^{2m} /
// (2m+3)! (no cancellation).  x >= 1 (tophat_big): Cody-Waite reduction of x
// by 2 pi = C1 + C2 (C1 the float nearest 2 pi; the first FMA is exact for
// x < 2^10 * 2 pi) to [-pi, pi], then the SFU sine/cosine (absolute error
// < 2^-21 there) and the SFU reciprocal (relative error ~2^-23).
__device__ __forceinline__ float tophat_small(float x) {
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
__device__ __forceinline__ float rcp_approx(float x) {
  float r;
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
  return r;
}
__device__ __forceinline__ float tophat_big(float x) {
  const float k = rintf(x * 0.159154943091895336f);
  float r = fmaf(-k, 6.28318548202514648f, x);
  r = fmaf(-k, -1.74845560e-07f, r);
  const float s = __sinf(r), c = __cosf(r);
  const float ix = rcp_approx(x);
  return 3.0f * fmaf(-x, c, s) * (ix * ix * ix);
}
__device__ __forceinline__ float tophat(float x) { return x < 1.0f ? tophat_small(x) : tophat_big(x); }

__device__ __forceinline__ float window_of(int m2, float kr) {
  return (m2 == 0) ? 0.f : tophat(sqrtf((float)m2) * kr);
}

// The reference's own float window, operation by operation
// (delta2zreion_d2z.C:41-43,59-82), for parity runs (PRC_FLAG_FAITHFUL_WINDOW):
// k = i*dk, minus kmax = dk*N for i >= N/2 (the Nyquist index too); |k| =
// sqrt((kx^2 + ky^2) + kz^2) in float; W = 3.*(sin(kR) - kR*cos(kR))/pow(kR, 3)
// with float sine and cosine, the quotient in double (pow(kR, 3) is the
// correctly rounded double product, as kR*kR is exact), rounded to float.
// Every step is rounded as written (no contraction into FMAs), so the
// cancellation of sin x - x cos x at small x is the reference's.  The float
// sine and cosine are the correctly rounded ones (the double functions
// rounded to float): the reference takes them from its C library, whose
// sinf/cosf may differ from those by an ulp (glibc 2.39: about 1% of
// arguments), so there is no bit-exact target; the cancellation amplifies such
// an ulp by about 3/x^2.
__device__ __forceinline__ float kfaithful(int i, int n, float dk, float kmax) {
  const float k = __fmul_rn((float)i, dk);
  return (i >= n / 2) ? __fsub_rn(k, kmax) : k;
}
__device__ __forceinline__ float rk_faithful(int ix, int iy, int iz, int n, float dk, float kmax) {
  const float kx = kfaithful(ix, n, dk, kmax), ky = kfaithful(iy, n, dk, kmax), kz = kfaithful(iz, n, dk, kmax);
  return __fsqrt_rn(__fadd_rn(__fadd_rn(__fmul_rn(kx, kx), __fmul_rn(ky, ky)), __fmul_rn(kz, kz)));
}
__device__ __forceinline__ float window_faithful(float rk, float R) {
  if (rk == 0.f) return 0.f;
  const float x = __fmul_rn(rk, R);
  const double xd = (double)x;
  const float sx = __double2float_rn(sin(xd)), cx = __double2float_rn(cos(xd));
  const float num = __fsub_rn(sx, __fmul_rn(x, cx));
  return __double2float_rn(__ddiv_rn(__dmul_rn(3.0, (double)num), __dmul_rn(__dmul_rn(xd, xd), xd)));
}

__device__ __forceinline__ void load_tw(float2* tw_s, const float2* tw, int n) {
  for (int i = threadIdx.x; i < n; i += blockDim.x) tw_s[i] = tw[i];
}

// Copies a per-radius parameter array into shared memory with compile-time
// indices (a runtime index into kernel parameters would force a local copy);
// thread 0 does it, so it works for CTAs of any size.
__device__ __forceinline__ void stage_params(float* dst, const float (&src)[kMaxBatch]) {
  if (threadIdx.x == 0) {
#pragma unroll
    for (int i = 0; i < kMaxBatch; ++i) dst[i] = src[i];
  }
}

// Radii [b0, b1) of this CTA in a window pass: the sweep's nb radii split
// evenly over gridDim.y (gridDim.y <= nb, so no range is empty).  Small grids
// have fewer tiles than the GPU holds CTAs; splitting the radii gives every SM
// work (each radius of a tile is computed the same way in any split).
__device__ __forceinline__ void radius_range(int nb, int& b0, int& b1) {
  b0 = (int)((long long)blockIdx.y * nb / gridDim.y);
  b1 = (int)((long long)(blockIdx.y + 1) * nb / gridDim.y);
}

// ------------------------------------------------------------ tiles
// A T-column tile is cut into 128-byte lines of 16 float2 words (16/T rows
// each); word w of line l is stored at l*16 + (w ^ f(l)),
// f(l) = (l ^ (l >> SA) ^ (l >> SB)) & 15.  With the per-N shifts of TCfg no
// access of the plan (group column reads, every Stockham store, the
// cooperative row loads) puts two lanes of a half-warp on one bank pair.
// Tiles whose width is not a power of two are not swizzled.
template <int N> struct TileSw {
  static constexpr int T = TCfg<N>::T, SA = TCfg<N>::SA, SB = TCfg<N>::SB;
  static constexpr bool on = IsPow2<T>::v && T <= 16;
  static constexpr int RPL = on ? 16 / T : 1;  // rows per line
  static __device__ __forceinline__ constexpr int f(int l) {
    return (l ^ (l >> SA) ^ (SB ? (l >> SB) : 0)) & 15;
  }
  static __device__ __forceinline__ int idx(int p, int c) {
    if constexpr (!on) {
      return p * T + c;
    } else {
      const int l = p / RPL;
      return l * 16 + (((p % RPL) * T + c) ^ f(l));
    }
  }
};

// One column of a tile.  The swizzle is linear over GF(2), so for a row
// tp | cp (disjoint thread bits tp and compile-time bits cp) the index is
// (h ^ D(cp)) + 16 * (cp / RPL), h = thread(tp): one XOR per access.
template <int N> struct TileCol {
  using S = TileSw<N>;
  float2* tile;
  int col;
  __device__ __forceinline__ int thread(int tp) const {
    if constexpr (S::on)
      return 16 * (tp / S::RPL) | (col ^ ((tp % S::RPL) * S::T) ^ S::f(tp / S::RPL));
    else
      return tp * S::T + col;
  }
  static __device__ __forceinline__ int off(int h, int cp) {
    if constexpr (S::on)
      return (h ^ (((cp % S::RPL) * S::T) ^ S::f(cp / S::RPL))) + 16 * (cp / S::RPL);
    else
      return h + cp * S::T;
  }
  __device__ __forceinline__ float2 get(int h, int cp) const { return tile[off(h, cp)]; }
  __device__ __forceinline__ void put(int h, int cp, float2 v) const { tile[off(h, cp)] = v; }
  __device__ __forceinline__ float2 get_pos(int p) const { return tile[S::idx(p, col)]; }
  __device__ __forceinline__ void put_pos(int p, float2 v) const { tile[S::idx(p, col)] = v; }
};

// Asynchronous 8-byte global -> shared copies (cp.async), so that the next
// tile streams in while the current one is transformed.
__device__ __forceinline__ void cp_async8(float2* smem, const float2* gmem) {
  const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
  asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(s), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int K> __device__ __forceinline__ void cp_async_wait() {
  asm volatile("cp.async.wait_group %0;\n" ::"n"(K) : "memory");
}

// Cooperative tile traffic, one 8-byte word per thread per row step: thread
// (tp, c) = (tid / T, tid % T) moves column c of rows tp + G*i (i < E), so a
// warp covers whole row segments; it is the transpose of the FFT mapping
// (group = column, lane t = rows t + G*m).
template <int N> struct TileIO {
  static constexpr int T = TCfg<N>::T, G = TK<N>::G, E = TK<N>::E;
  const int tp, c;
  int h;
  __device__ __forceinline__ TileIO(float2* tile) : tp(threadIdx.x / T), c(threadIdx.x % T) {
    h = TileCol<N>{tile, c}.thread(tp);
  }
  __device__ __forceinline__ void load_async(float2* tile, const float2* base, int row_stride) const {
    const float2* src = base + (long long)tp * row_stride + c;
    const long long step = (long long)G * row_stride;
#pragma unroll
    for (int i = 0; i < E; ++i) cp_async8(tile + TileCol<N>::off(h, i * G), src + i * step);
  }
  __device__ __forceinline__ void store(const float2* tile, float2* base, int row_stride) const {
    float2* dst = base + (long long)tp * row_stride + c;
    const long long step = (long long)G * row_stride;
#pragma unroll
    for (int i = 0; i < E; ++i) dst[i * step] = tile[TileCol<N>::off(h, i * G)];
  }
  // base += tile (base = 0 first if zero)
  __device__ __forceinline__ void accumulate(const float2* tile, float2* base, int row_stride, bool zero) const {
    float2* dst = base + (long long)tp * row_stride + c;
    const long long step = (long long)G * row_stride;
#pragma unroll
    for (int i = 0; i < E; ++i) {
      const float2 a = tile[TileCol<N>::off(h, i * G)];
      float2 o = zero ? make_float2(0.f, 0.f) : dst[i * step];
      dst[i * step] = make_float2(o.x + a.x, o.y + a.y);
    }
  }
};

// Synchronous cooperative tile traffic in 16-byte chunks (two columns):
// consecutive threads along a row, thread rows tp = tid / CPR, iteration i
// adding the constant row i * RPI.  Fewer, wider instructions than TileIO;
// used by the passes that do not prefetch.
template <int N, int THREADS> struct TileIO16 {
  static constexpr int T = TCfg<N>::T, CPR = T / 2, RPI = THREADS / CPR, ITER = N / RPI;
  static_assert(THREADS % CPR == 0 && N % RPI == 0, "tile io shape");
  const int tp, cc;
  int h0, h1;
  __device__ __forceinline__ TileIO16() : tp(threadIdx.x / CPR), cc(threadIdx.x % CPR) {
    h0 = TileCol<N>{nullptr, 2 * cc}.thread(tp);
    h1 = TileCol<N>{nullptr, 2 * cc + 1}.thread(tp);
  }
  __device__ __forceinline__ void load(float2* tile, const float2* base, int row_stride) const {
    const float2* src = base + (long long)tp * row_stride + 2 * cc;
    const long long step = (long long)RPI * row_stride;
#pragma unroll
    for (int i = 0; i < ITER; ++i) {
      const float4 v = __ldg(reinterpret_cast<const float4*>(src + i * step));
      tile[TileCol<N>::off(h0, i * RPI)] = make_float2(v.x, v.y);
      tile[TileCol<N>::off(h1, i * RPI)] = make_float2(v.z, v.w);
    }
  }
  __device__ __forceinline__ void store(const float2* tile, float2* base, int row_stride) const {
    float2* dst = base + (long long)tp * row_stride + 2 * cc;
    const long long step = (long long)RPI * row_stride;
#pragma unroll
    for (int i = 0; i < ITER; ++i) {
      const float2 a = tile[TileCol<N>::off(h0, i * RPI)], b = tile[TileCol<N>::off(h1, i * RPI)];
      *reinterpret_cast<float4*>(dst + i * step) = make_float4(a.x, a.y, b.x, b.y);
    }
  }
  __device__ __forceinline__ void accumulate(const float2* tile, float2* base, int row_stride, bool zero) const {
    float2* dst = base + (long long)tp * row_stride + 2 * cc;
    const long long step = (long long)RPI * row_stride;
#pragma unroll
    for (int i = 0; i < ITER; ++i) {
      const float2 a = tile[TileCol<N>::off(h0, i * RPI)], b = tile[TileCol<N>::off(h1, i * RPI)];
      float4* d = reinterpret_cast<float4*>(dst + i * step);
      float4 o = zero ? make_float4(0.f, 0.f, 0.f, 0.f) : *d;
      o.x += a.x;
      o.y += a.y;
      o.z += b.x;
      o.w += b.y;
      *d = o;
    }
  }
};

// Transposed store of an N x N plane tile: column c -> out[(c0 + c)*N + row].
template <int N, int T, int THREADS>
__device__ __forceinline__ void tile_store_t(const float2* tile, float2* out, int c0) {
  constexpr int CPC = N / 2;  // chunks per column
  for (int q = threadIdx.x; q < T * CPC; q += THREADS) {
    const int c = q / CPC, pp = q - (q / CPC) * CPC;
    const float2 a = tile[TileSw<N>::idx(2 * pp, c)], b = tile[TileSw<N>::idx(2 * pp + 1, c)];
    *reinterpret_cast<float4*>(out + (long long)(c0 + c) * N + 2 * pp) = make_float4(a.x, a.y, b.x, b.y);
  }
}

// ============================================================ column pass
// One kernel for every column pass:
//   TM_FWD / TM_INV  plain forward / inverse transform, in -> out (blockIdx.y
//                    selects a slot), same layout or transposed; two tile
//                    buffers, the next tile prefetched with cp.async;
//   TM_WIN           spectrum tile loaded once (raw buffer, next one
//                    prefetched during the last radius), then per radius b:
//                    raw * W_b (k = 0 -> 0), inverse transform in the work
//                    buffer, -> slot b;
//   TM_ACC           per radius b: forward transform of slot b, acc += W_b * (.).
// Rows ix and N-ix share |k|, so in the window modes each pair of rows is
// evaluated once and handed to the mirror lane by a shuffle.
template <int N, int MODE>
__global__ void __launch_bounds__(TK<N>::THREADS, MODE == TM_ACC ? TK<N>::MINB_ACC : TK<N>::MINB)
    k_tile(TileArgs a) {
  using KK = TK<N>;
  constexpr int H = N / 2, E = KK::E, G = KK::G, T = KK::T, TH = KK::THREADS;
  constexpr bool INV = (MODE == TM_INV || MODE == TM_WIN);
  constexpr bool WIN = (MODE == TM_WIN || MODE == TM_ACC);
  constexpr bool SPLIT = PlanRun<typename KK::P>::SPLIT;
  extern __shared__ float4 smem4[];
  float2* tws = reinterpret_cast<float2*>(smem4);  // stage twiddles
  float2* buf0 = tws + KK::TW;
  float2* buf1 = buf0 + N * T;
  __shared__ float s_kr[kMaxBatch];
  if constexpr (WIN) stage_params(s_kr, a.kr);
  PlanRun<typename KK::P>::template fill<1>(tws, a.tw);
  const int g = threadIdx.x / G, t = threadIdx.x - (threadIdx.x / G) * G;
  // CTAs smaller than a warp (the smallest grids) name only their own lanes
  constexpr unsigned LANES = TH >= 32 ? 0xffffffffu : ((1u << TH) - 1u);
  GroupSync<G> sync(g, LANES);
  const TileIO<N> io(buf0);
  const int hrow = TileCol<N>{buf0, g}.thread(t);  // rows t + G*m of this group's column (same in both buffers)
  const long long yoff = (MODE == TM_FWD || MODE == TM_INV) ? (long long)blockIdx.y * a.slot_stride : 0;
  const int tiles0 = a.seg[0].n_outer * a.seg[0].tpo;
  const int tiles = tiles0 + a.seg[1].n_outer * a.seg[1].tpo;

  struct Where {
    TileSeg sg;
    int outer, tc;
    long long off;
  };
  auto where = [&](int ti) {
    Where w;
    const bool sn = ti >= tiles0;
    w.sg = sn ? a.seg[1] : a.seg[0];
    const int tl = sn ? ti - tiles0 : ti;
    w.outer = tl / w.sg.tpo;
    w.tc = tl - w.outer * w.sg.tpo;
    w.off = (long long)w.outer * w.sg.outer_stride + (long long)w.tc * T;
    return w;
  };
  auto col_read = [&](const float2* tile, float2 (&v)[E]) {
    const TileCol<N> col{const_cast<float2*>(tile), g};
#pragma unroll
    for (int m = 0; m < E; ++m) v[m] = SPLIT ? col.get(hrow, G * m) : col.get_pos(t + G * m);
  };
  auto col_write = [&](float2* tile, const float2 (&v)[E]) {
    const TileCol<N> col{tile, g};
#pragma unroll
    for (int m = 0; m < E; ++m) {
      if constexpr (SPLIT) col.put(hrow, G * m, v[m]);
      else col.put_pos(t + G * m, v[m]);
    }
  };
  auto window = [&](const Where& w, int b, float (&wv)[E]) {
    const float kr = s_kr[b];
    const int c = w.tc * T + g;
    const int syz = w.sg.nyq ? fsq(c, N) + H * H : fsq(w.outer, N) + c * c;
    constexpr int EH = E / 2;
    constexpr bool share = (G <= 32);
#pragma unroll
    for (int m = 0; m < E; ++m)
      if (!share || m <= EH) wv[m] = window_of(fsq(t + G * m, N) + syz, kr);
    if constexpr (share) {
#pragma unroll
      for (int m = EH + 1; m < E; ++m) {
        const float o = __shfl_sync(LANES, wv[E - 1 - m], (G - t) & (G - 1), G);
        wv[m] = (t == 0) ? wv[E - m] : o;
      }
    }
  };
  // v *= W_b in place; only the E/2+1 directly evaluated values stay live
  auto apply_window = [&](int ti, int b, float2 (&v)[E]) {
    const Where w = where(ti);
    const float kr = s_kr[b];
    const int c = w.tc * T + g;
    const int syz = w.sg.nyq ? fsq(c, N) + H * H : fsq(w.outer, N) + c * c;
    constexpr int EH = E / 2;
    if (a.faithful) {
      // every row on its own: rows ix and N - ix need not round alike here
      const int iy = w.sg.nyq ? c : w.outer, iz = w.sg.nyq ? H : c;
#pragma unroll
      for (int m = 0; m < E; ++m)
        v[m] = cscale(v[m], window_faithful(rk_faithful(t + G * m, iy, iz, N, a.dk, a.kmax), kr));
    } else if constexpr (G <= 32) {
      float wv[EH + 1];
#pragma unroll
      for (int m = 0; m <= EH; ++m) {
        wv[m] = window_of(fsq(t + G * m, N) + syz, kr);
        v[m] = cscale(v[m], wv[m]);
      }
#pragma unroll
      for (int m = EH + 1; m < E; ++m) {
        const float o = __shfl_sync(LANES, wv[E - 1 - m], (G - t) & (G - 1), G);
        v[m] = cscale(v[m], (t == 0) ? wv[E - m] : o);
      }
    } else {
#pragma unroll
      for (int m = 0; m < E; ++m) v[m] = cscale(v[m], window_of(fsq(t + G * m, N) + syz, kr));
    }
  };
  auto store_tile = [&](const Where& w, const float2* tile, float2* dst) {
    if (w.sg.transpose)
      tile_store_t<N, T, TH>(tile, dst + (long long)w.outer * w.sg.outer_stride, w.tc * T);
    else
      io.store(tile, dst + w.off, w.sg.row_stride);
  };

  if constexpr (MODE == TM_FWD || MODE == TM_INV) {
    const TileIO16<N, TH> io16;
    for (int ti = blockIdx.x; ti < tiles; ti += gridDim.x) {
      const Where w = where(ti);
      io16.load(buf0, w.sg.in + w.off + yoff, w.sg.row_stride);
      __syncthreads();
      float2 v[E];
      col_read(buf0, v);
      // the column is also the exchange buffer: every lane of the group must
      // have read it before the first stage writes it (a group of 64 lanes
      // spans two warps)
      sync();
      const TileCol<N> col{buf0, g};
      PlanRun<typename KK::P>::template run<INV>(v, col, t, tws, sync);
      col_write(buf0, v);
      __syncthreads();
      if (w.sg.transpose)
        tile_store_t<N, T, TH>(buf0, w.sg.out + yoff + (long long)w.outer * w.sg.outer_stride, w.tc * T);
      else
        io16.store(buf0, w.sg.out + yoff + w.off, w.sg.row_stride);
      __syncthreads();
    }
  } else if constexpr (MODE == TM_WIN) {
    float2* raw = buf0;
    float2* work = buf1;
    int ti = blockIdx.x;
    if (ti < tiles) {
      const Where w0 = where(ti);
      io.load_async(raw, w0.sg.in + w0.off, w0.sg.row_stride);
    }
    cp_async_commit();
    int b0, b1;
    radius_range(a.nb, b0, b1);
    for (; ti < tiles; ti += gridDim.x) {
      cp_async_wait<0>();
      __syncthreads();
      for (int b = b0; b < b1; ++b) {
        float2 v[E];
        col_read(raw, v);
        if (b == b1 - 1) {
          // every group has its raw column: stream the next spectrum tile in
          __syncthreads();
          const int tn = ti + gridDim.x;
          if (tn < tiles) {
            const Where wn = where(tn);
            io.load_async(raw, wn.sg.in + wn.off, wn.sg.row_stride);
          }
          cp_async_commit();
        }
        apply_window(ti, b, v);
        const TileCol<N> col{work, g};
        PlanRun<typename KK::P>::template run<true>(v, col, t, tws, sync);
        col_write(work, v);
        __syncthreads();
        const Where w = where(ti);
        store_tile(w, work, w.sg.out + (long long)b * a.slot_stride);
        __syncthreads();
      }
    }
    cp_async_wait<0>();
  } else {  // TM_ACC
    const TileIO16<N, TH> io16;
    float2* tile = buf0;
    for (int ti = blockIdx.x; ti < tiles; ti += gridDim.x) {
      const Where w = where(ti);
      float2 acc[E];
#pragma unroll
      for (int m = 0; m < E; ++m) acc[m] = make_float2(0.f, 0.f);
      for (int b = 0; b < a.nb; ++b) {
        io16.load(tile, w.sg.in + w.off + (long long)b * a.slot_stride, w.sg.row_stride);
        __syncthreads();
        float2 v[E];
        col_read(tile, v);
        sync();  // as above: the column is the exchange buffer
        float wv[E];
        window(w, b, wv);
        const TileCol<N> col{tile, g};
        PlanRun<typename KK::P>::template run<false>(v, col, t, tws, sync);
#pragma unroll
        for (int m = 0; m < E; ++m) {
          acc[m].x = fmaf(wv[m], v[m].x, acc[m].x);
          acc[m].y = fmaf(wv[m], v[m].y, acc[m].y);
        }
        __syncthreads();  // the next radius reloads the tile
      }
      col_write(tile, acc);
      __syncthreads();
      io16.accumulate(tile, w.sg.out + w.off, w.sg.row_stride, a.first != 0);
      __syncthreads();
    }
  }
}

// ============================================================ line helpers
// Forward real-to-half-complex along a line.  In: v[m] = (x[2p], x[2p+1]) at
// p = t + G*m.  Out: v[m] = X[k] at k = t + G*m (k < H); returns X[H] (real) in
// lane t == 0.  Z = DFT_H(x_even + i x_odd); X[k] = Ze[k] + e^{-2 pi i k/N} Zo[k].
template <int N, class Sync>
__device__ __forceinline__ float line_r2c(float2 (&v)[LK<N>::E], float2* gbuf, int t, const float2* tw,
                                          const float2* tws, const Sync& sync) {
  constexpr int H = N / 2, E = LK<N>::E, G = LK<N>::G;
  using P = typename LK<N>::P;
  const LineBuf<H> buf{gbuf};
  PlanRun<P>::template run<false>(v, buf, t, tws, sync);
  const int h = buf.thread(t);
#pragma unroll
  for (int m = 0; m < E; ++m) {
    if constexpr (PlanRun<P>::SPLIT) buf.put(h, G * m, v[m]);
    else buf.put_pos(t + G * m, v[m]);
  }
  sync();
  float2 p[E];
#pragma unroll
  for (int m = 0; m < E; ++m) p[m] = buf.get_pos((H - (t + G * m)) % H);
  sync();
  float xh = 0.f;
#pragma unroll
  for (int m = 0; m < E; ++m) {
    const int k = t + G * m;
    const float2 z = v[m], zc = cconj(p[m]);
    const float2 ze = cscale(cadd(z, zc), 0.5f);
    const float2 d = csub(z, zc);
    const float2 zo = make_float2(0.5f * d.y, -0.5f * d.x);  // d / (2i)
    v[m] = cadd(ze, cmul(cconj(tw[k]), zo));
    if (m == 0) xh = ze.x - zo.x;
  }
  return xh;
}

// Inverse half-complex-to-real along a line (FFTW c2r semantics: the imaginary
// parts of X[0] and X[H] are ignored).  In: v[m] = X[k] at k = t + G*m, xh =
// X[H] (read by lane t == 0 only).  Out: v[m] = (x[2p], x[2p+1]) at p = t + G*m,
// unnormalised.
template <int N, class Sync>
__device__ __forceinline__ void line_c2r(float2 (&v)[LK<N>::E], float2 xh, float2* gbuf, int t,
                                         const float2* tw, const float2* tws, const Sync& sync) {
  constexpr int H = N / 2, E = LK<N>::E, G = LK<N>::G;
  using P = typename LK<N>::P;
  const LineBuf<H> buf{gbuf};
  const int h = buf.thread(t);
#pragma unroll
  for (int m = 0; m < E; ++m) {
    if constexpr (PlanRun<P>::SPLIT) buf.put(h, G * m, v[m]);
    else buf.put_pos(t + G * m, v[m]);
  }
  sync();
  float2 p[E];
#pragma unroll
  for (int m = 0; m < E; ++m) p[m] = buf.get_pos((H - (t + G * m)) % H);
  sync();
#pragma unroll
  for (int m = 0; m < E; ++m) {
    const int k = t + G * m;
    float2 x = v[m], xp = p[m];
    if (k == 0) {
      x = make_float2(x.x, 0.f);
      xp = make_float2(xh.x, 0.f);
    }
    const float2 xc = cconj(xp);
    const float2 xe = cadd(x, xc);
    const float2 xo = cmul(csub(x, xc), tw[k]);
    v[m] = make_float2(xe.x - xo.y, xe.y + xo.x);  // xe + i*xo
  }
  PlanRun<P>::template run<true>(v, buf, t, tws, sync);
}

// ============================================================ forward z pass
// Real line (N samples, divided by DInit) -> X[0..H-1] into S and X[H] into
// the transposed Nyquist scratch Qt[iy][ix].
// MB (grouped launch): the lines of nbox boxes of this grid size, line l of
// box l / N^2 with box i's input, spectrum and divisor from box[i].
template <int N, bool MB = false>
__global__ void __launch_bounds__(LK<N>::THREADS, LK<N>::MINB) k_r2c_z(const float* __restrict__ delta, float dinit,
                                                             float2* S, float2* Qt, const float2* twg,
                                                             const BoxR2c* box, int nbox) {
  using KK = LK<N>;
  constexpr int H = N / 2, E = KK::E, G = KK::G, NG = KK::NG;
  extern __shared__ float4 smem4[];
  float2* tw = reinterpret_cast<float2*>(smem4);
  float2* tws = tw + N;
  load_tw(tw, twg, N);
  PlanRun<typename KK::P>::template fill<2>(tws, twg);
  __syncthreads();
  const int g = threadIdx.x / G, t = threadIdx.x % G;
  float2* gbuf = tws + KK::TW + g * KK::gsize;
  GroupSync<G> sync(g);
  constexpr int lpb = N * N;  // lines of one box
  static_assert(!MB || lpb % NG == 0, "a CTA step never spans two boxes");
  const int lines = MB ? lpb * nbox : lpb;
  for (int s = blockIdx.x; s * NG < lines; s += gridDim.x) {
    int l = s * NG + g;
    const bool valid = l < lines;
    const float* dsrc = delta;
    float dv = dinit;
    float2 *Sb = S, *Qb = Qt;
    if constexpr (MB) {
      const int bx = (s * NG) / lpb;  // the same box for the whole step
      const BoxR2c* bp = box + bx;
      dsrc = bp->delta;
      dv = bp->dinit;
      Sb = bp->S;
      Qb = bp->Qt;
      l -= bx * lpb;
    }
    float2 v[E];
    const float2* src = reinterpret_cast<const float2*>(dsrc + (long long)(valid ? l : 0) * N);
#pragma unroll
    for (int m = 0; m < E; ++m) {
      float2 q = valid ? __ldg(src + t + G * m) : make_float2(0.f, 0.f);
      v[m] = make_float2(__fdiv_rn(q.x, dv), __fdiv_rn(q.y, dv));
    }
    const float xh = line_r2c<N>(v, gbuf, t, tw, tws, sync);
    if (valid) {
      float2* dst = Sb + (long long)l * H;
#pragma unroll
      for (int m = 0; m < E; ++m) dst[t + G * m] = v[m];
      if (t == 0) {
        const int ix = l / N, iy = l - (l / N) * N;
        Qb[(long long)iy * N + ix] = make_float2(xh, 0.f);
      }
    }
  }
}

// ============================================================ inverse z pass
// For each radius of the sweep: X[0..H] -> real line, z = A/N^3 * x + (A B_b - 1),
// running max / argmax in registers, optional sum of x^2; one zreion RMW per sweep.
template <int N>
__global__ void __launch_bounds__(LK<N>::THREADS, LK<N>::MINB) k_c2r_z(SweepArgs a) {
  using KK = LK<N>;
  constexpr int H = N / 2, E = KK::E, G = KK::G, NG = KK::NG;
  constexpr long long NN = (long long)N * N;
  extern __shared__ float4 smem4[];
  float2* tw = reinterpret_cast<float2*>(smem4);
  float2* tws = tw + N;
  load_tw(tw, a.tw, N);
  PlanRun<typename KK::P>::template fill<2>(tws, a.tw);
  __shared__ double red[kMaxBatch];
  __shared__ float s_cb[kMaxBatch];
  stage_params(s_cb, a.cb);
  if (threadIdx.x < kMaxBatch) red[threadIdx.x] = 0.0;
  __syncthreads();
  const int g = threadIdx.x / G, t = threadIdx.x % G;
  float2* gbuf = tws + KK::TW + g * KK::gsize;
  GroupSync<G> sync(g);
  const int lines = N * N;
  const bool want_sig = a.sig_acc != nullptr;
  for (int s = blockIdx.x; s * NG < lines; s += gridDim.x) {
    const int l = s * NG + g;
    const bool valid = l < lines;
    const int lv = valid ? l : 0;
    const int ix = lv / N, iy = lv - (lv / N) * N;
    float2 zr[E];
    uint32_t am[E];  // the two argmax bytes of each element
    float* zline = a.zreion + (long long)lv * N;
    uint8_t* aline = a.argmax ? a.argmax + (long long)lv * N : nullptr;
    if (a.first || !valid) {
#pragma unroll
      for (int m = 0; m < E; ++m) {
        zr[m] = make_float2(0.f, 0.f);
        am[m] = 0xFFFFu;
      }
    } else {
#pragma unroll
      for (int m = 0; m < E; ++m) {
        const int p = t + G * m;
        zr[m] = reinterpret_cast<const float2*>(zline)[p];
        am[m] = aline ? (uint32_t)reinterpret_cast<const uint16_t*>(aline)[p] : 0xFFFFu;
      }
    }
    for (int b = 0; b < a.nb; ++b) {
      const float2* slot = a.slots + (long long)b * a.slot_stride;
      const float2* src = slot + (long long)lv * H;
      float2 v[E];
#pragma unroll
      for (int m = 0; m < E; ++m) v[m] = valid ? __ldg(src + t + G * m) : make_float2(0.f, 0.f);
      float2 xn = make_float2(0.f, 0.f);
      if (t == 0 && valid) xn = __ldg(slot + NN * H + (long long)iy * N + ix);
      line_c2r<N>(v, xn, gbuf, t, tw, tws, sync);
      const float cb = s_cb[b];
      const uint32_t rid = (uint32_t)(a.r0 + b);
      float ss = 0.f;
#pragma unroll
      for (int m = 0; m < E; ++m) {
        const float x0 = v[m].x, x1 = v[m].y;
        const float z0 = fmaf(a.as, x0, cb), z1 = fmaf(a.as, x1, cb);
        if (z0 > zr[m].x) { zr[m].x = z0; am[m] = (am[m] & 0xFF00u) | rid; }
        if (z1 > zr[m].y) { zr[m].y = z1; am[m] = (am[m] & 0x00FFu) | (rid << 8); }
        ss = fmaf(x0, x0, fmaf(x1, x1, ss));
      }
      if (want_sig) {
        if (!valid) ss = 0.f;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) ss += __shfl_xor_sync(0xffffffffu, ss, o);
        if ((threadIdx.x & 31) == 0) atomicAdd(&red[b], (double)ss);
      }
    }
    if (valid) {
      float* zo = a.zreion_out + (long long)lv * N;
      uint8_t* ao = a.argmax_out ? a.argmax_out + (long long)lv * N : nullptr;
#pragma unroll
      for (int m = 0; m < E; ++m) {
        const int p = t + G * m;
        reinterpret_cast<float2*>(zo)[p] = zr[m];
        if (ao) reinterpret_cast<uint16_t*>(ao)[p] = (uint16_t)am[m];
      }
    }
  }
  if (want_sig) {
    __syncthreads();
    if (threadIdx.x < a.nb) atomicAdd(&a.sig_acc[a.r0 + threadIdx.x], red[threadIdx.x]);
  }
}

}  // namespace prc
