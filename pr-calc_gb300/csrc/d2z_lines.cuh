// d2z_lines.cuh — the inverse z pass with mirror pairs held by one lane.
//
// The half-complex-to-real transform of a z line needs, for every k, both
// X[k] and X[H-k].  Here lane t of a group of G = H/E lanes loads the pairs
// (X[k], X[H-k]) for k = t + G*m, m < E/2, straight from the slot, computes
// both packed values Z[k] and Z[H-k] from the one pair, keeps Z[k] and hands
// Z[H-k] to lane G-t (which owns position H-k) with one shuffle.  The packed
// sequence then goes through the half-length inverse complex FFT (E = 16: one
// shared-memory exchange for H = 256), so the only shared-memory traffic of
// the kernel is that exchange.
//
// Packing (FFTW c2r semantics, imaginary parts of X[0] and X[H] ignored):
//   xe = X[k] + conj X[H-k],  xo = (X[k] - conj X[H-k]) e^{+2 pi i k/N},
//   Z[k] = xe + i xo,  Z[H-k] = conj(xe) + i conj(xo)
// (the second because e^{+2 pi i (H-k)/N} = -conj e^{+2 pi i k/N}); the
// inverse FFT of Z gives (x[2p], x[2p+1]) at p.  Lane 0 pairs k = G*m with
// G*(E-m): its k = 0 partner is X[H] (the Nyquist plane), its k = H/2 value is
// its own mirror, and its received values sit one register low, which a
// final shift corrects.
//
// Then, per radius of the sweep, the barrier crossing of delta2zreion_d2z.C
// :206-216 (z = A/N^3 x + (A B_b - 1)) and the running max of :105-146 with
// strict >, in registers; one zreion / argmax read-modify-write per sweep.
#pragma once
#include "d2z_kernels.cuh"

namespace prc {

// Plan of the half-length line transform; THREADS / MINB: CTA size and
// resident CTAs per SM.  Smaller CTAs wait at fewer-warp barriers and drift
// out of phase with one another: 128-thread CTAs (four per SM; three at 1024,
// where shared memory holds no more) run the pass 7% faster than 256-thread
// ones at N = 512 (the same 16 warps per SM), 10% at 256 and 3.5% at 1024;
// 64-thread CTAs (seven per SM at 512) are 9% slower again.
template <int N> struct PCfg { static constexpr bool on = false; };
struct PDef { static constexpr int THREADS = 128, MINB = 4; };
template <> struct PCfg<32> : PDef { static constexpr bool on = true; using P = Plan<8, 8, 2>; };
// 64 and 128 (lines of 32 and 64): eight elements a lane instead of sixteen,
// so twice the lanes, twice the line groups (a 64^3 box: 128 CTAs instead of
// 64) and about 80 registers (five CTAs per SM), which a single small box
// needs to fill the GPU: the pass took 76 instead of 115 us at 64^3 x 64
// radii and 99 instead of 107 us at 128^3 x 32.
template <> struct PCfg<64> { static constexpr bool on = true; using P = Plan<8, 8, 4>; static constexpr int THREADS = 128, MINB = 5; };
template <> struct PCfg<96> : PDef { static constexpr bool on = true; using P = Plan<12, 12, 4>; };
template <> struct PCfg<128> { static constexpr bool on = true; using P = Plan<8, 8, 8>; static constexpr int THREADS = 128, MINB = 5; };
template <> struct PCfg<192> : PDef { static constexpr bool on = true; using P = Plan<12, 12, 4, 2>; };
template <> struct PCfg<256> : PDef { static constexpr bool on = true; using P = Plan<16, 16, 8>; };
template <> struct PCfg<384> : PDef { static constexpr bool on = true; using P = Plan<12, 12, 4, 4>; };
template <> struct PCfg<512> : PDef { static constexpr bool on = true; using P = Plan<16, 16, 16>; };
template <> struct PCfg<768> : PDef { static constexpr bool on = true; using P = Plan<12, 12, 4, 4, 2>; };
template <> struct PCfg<1024> {
  static constexpr bool on = true;
  using P = Plan<16, 16, 16, 2>;
  static constexpr int THREADS = 128, MINB = 3;
};

template <int N> struct PK {
  using P = typename PCfg<N>::P;
  static constexpr int H = N / 2, E = P::E, G = H / E;
  static_assert(PlanRun<P>::L == H, "line plan length");
  static_assert(E % 2 == 0 && G >= 2 && G <= 32 && 32 % G == 0, "paired line shape");
  static constexpr int THREADS = PCfg<N>::THREADS;
  static constexpr int NG = THREADS / G;                // lines per CTA step
  static constexpr int MINB = PCfg<N>::MINB;
  static_assert(THREADS >= kMaxBatch && THREADS % G == 0, "per-radius sums need a thread per radius");
  static constexpr int gsize = GroupBuf<H, G>::size;
  static constexpr int TW = (PlanRun<P>::TW + 1) & ~1;
  static constexpr int STG = NG * H;                    // one staged step: NG whole lines (float2)
  static_assert((STG * 8) % (16 * THREADS) == 0, "16-byte copies per thread");
  // N-table, stage twiddles, group buffers, two staged steps, two Nyquist rows
  static constexpr int smem_f2 = N + TW + NG * gsize + 2 * STG + 2 * NG;
};

// TMA bulk copies (cp.async.bulk) completing on an mbarrier.
__device__ __forceinline__ void mbar_init(uint64_t* bar, unsigned count) {
  const unsigned s = (unsigned)__cvta_generic_to_shared(bar);
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;\n" ::"r"(s), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_init_fence() {
  asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
}
// one arrival that also announces `bytes` of transactions, then the copy
__device__ __forceinline__ void bulk_load(void* smem_dst, const void* gmem_src, unsigned bytes, uint64_t* bar) {
  const unsigned d = (unsigned)__cvta_generic_to_shared(smem_dst);
  const unsigned b = (unsigned)__cvta_generic_to_shared(bar);
  asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(b), "r"(bytes) : "memory");
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];\n"
               ::"r"(d), "l"(gmem_src), "r"(bytes), "r"(b)
               : "memory");
}
// waits for phase `parity` of the barrier; false after `limit` polls
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, unsigned parity, int limit) {
  const unsigned b = (unsigned)__cvta_generic_to_shared(bar);
  for (int i = 0; i < limit; ++i) {
    unsigned ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(ok)
        : "r"(b), "r"(parity)
        : "memory");
    if (ok) return true;
  }
  return false;
}
constexpr int kWaitPolls = 1 << 22;  // each poll may suspend; far beyond any copy
constexpr int kWithheldPolls = 256;  // wait limit of a CTA whose copy the test hook withheld

// Steps (line group s, radius b) run in order; the input of the next step is
// copied into the other staging buffer while the current one is transformed:
// the NG lines of a step are one contiguous block of the slot, fetched by one
// TMA bulk copy (cp.async.bulk) issued by thread 0 and completing on that
// buffer's mbarrier; the NG Nyquist values come with 8-byte cp.async.  A wait
// that runs out of polls stops the whole CTA and sets *a.err; before the CTA
// exits, thread 0 (which issued the copy) waits once more, again bounded, for
// that copy to land, so that no bulk copy is left writing into the shared
// memory of a CTA that has gone (the 8-byte copies end at cp_async_wait).
// a.withhold (a test hook) makes CTA 0 skip its first bulk copy, so that its
// first wait runs out for real, with nothing in flight.
// AM: argmax wanted (a.argmax != null); its bytes are packed four to a register.
// SIG: per-radius sums of x^2 wanted (a.sig_acc != null).
// MB (grouped launch): the line groups of a.nbox boxes of this grid size, box
// i's slots, outputs, radius count and barrier constants from a.box[i]; line
// group q is line group q mod (N^2 / NG) of box q / (N^2 / NG).
template <int N, bool AM, bool SIG, bool MB = false>
__global__ void __launch_bounds__(PK<N>::THREADS, PK<N>::MINB) k_c2r_zp(SweepArgs a) {
  static_assert(!(MB && SIG), "no per-radius sums in grouped launches");
  using KK = PK<N>;
  using P = typename KK::P;
  constexpr int H = N / 2, E = KK::E, G = KK::G, NG = KK::NG, EH = E / 2, STG = KK::STG;
  constexpr long long NN = (long long)N * N;
  static_assert((NN % NG) == 0, "whole line groups");
  extern __shared__ float4 smem4[];
  float2* tw = reinterpret_cast<float2*>(smem4);
  float2* tws = tw + N;
  float2* gb = tws + KK::TW;
  float2* stage = gb + NG * KK::gsize;  // 16-byte aligned: N, TW, gsize are even
  float2* nyq = stage + 2 * STG;
  load_tw(tw, a.tw, N);
  PlanRun<P>::template fill<2>(tws, a.tw);
  __shared__ double red[kMaxBatch];
  __shared__ float s_cb[kMaxBatch];
  stage_params(s_cb, a.cb);
  if (threadIdx.x < kMaxBatch) red[threadIdx.x] = 0.0;
  const int g = threadIdx.x / G, t = threadIdx.x % G;
  const LineBuf<H> buf{gb + g * KK::gsize};
  GroupSync<G> sync(g);
  const int partner = (G - t) & (G - 1);
  constexpr long long lgpb = NN / NG;  // line groups of one box
  const long long lg_all = MB ? lgpb * a.nbox : lgpb;
  const int nsteps_l = (int)((lg_all - blockIdx.x + gridDim.x - 1) / gridDim.x);  // line groups of this CTA
  // line group lg of this CTA: its box and its first line within that box
  auto box_of = [&](int lg) { return MB ? (int)(((long long)blockIdx.x + (long long)lg * gridDim.x) / lgpb) : 0; };
  auto line0 = [&](int lg, int bx) {
    return ((long long)blockIdx.x + (long long)lg * gridDim.x - (long long)bx * lgpb) * NG;
  };

  __shared__ __align__(8) uint64_t s_bar[2];
  if (threadIdx.x == 0) {
    mbar_init(&s_bar[0], 1);
    mbar_init(&s_bar[1], 1);
    mbar_init_fence();
  }
  __syncthreads();

  // copies of step (line group lg of this CTA, radius b) into staging buffer bi
  const bool withheld = a.withhold && blockIdx.x == 0;
  auto issue = [&](int lg, int b, int bi) {
    if (lg < nsteps_l) {
      const int bx = box_of(lg);
      const long long l0 = line0(lg, bx);
      const float2* slot = (MB ? a.box[bx].slots : a.slots) + (long long)b * a.slot_stride;
      if (threadIdx.x == 0 && !(withheld && lg == 0 && b == 0))
        bulk_load(stage + bi * STG, slot + l0 * H, STG * 8, &s_bar[bi]);
      if (t == 0) {
        const long long l = l0 + g;
        const int ix = (int)(l / N), iy = (int)(l - (l / N) * N);
        cp_async8(nyq + bi * NG + g, slot + NN * H + (long long)iy * N + ix);
      }
    }
    cp_async_commit();
  };

  issue(0, 0, 0);
  float2 zr[E];
  uint32_t am[AM ? EH : 1];  // argmax bytes of cells 2p, 2p+1 of elements 2j (low half) and 2j+1
  int lg = 0, b = 0;         // current step; steps run radius-fastest
  for (int i = 0; lg < nsteps_l; ++i) {
    const int bi = i & 1;
    const int bx = box_of(lg);
    const BoxLine* bp = MB ? a.box + bx : nullptr;
    const int nb = MB ? bp->nb : a.nb;
    const int nb_next = (b + 1 < nb) ? b + 1 : 0;
    const int lg_next = (b + 1 < nb) ? lg : lg + 1;
    const long long l = line0(lg, bx) + g;
    float* zline = (MB ? bp->zreion : a.zreion) + l * N;
    uint16_t* aline = AM ? reinterpret_cast<uint16_t*>((MB ? bp->argmax : a.argmax) + l * N) : nullptr;
    float* zout = (MB ? bp->zreion_out : a.zreion_out) + l * N;
    uint16_t* aout = AM ? reinterpret_cast<uint16_t*>((MB ? bp->argmax_out : a.argmax_out) + l * N) : nullptr;
    if (b == 0) {
      if (MB ? bp->first : a.first) {
#pragma unroll
        for (int m = 0; m < E; ++m) zr[m] = make_float2(0.f, 0.f);
        if constexpr (AM) {
#pragma unroll
          for (int j = 0; j < EH; ++j) am[j] = 0xFFFFFFFFu;
        }
      } else {
#pragma unroll
        for (int m = 0; m < E; ++m) zr[m] = reinterpret_cast<const float2*>(zline)[t + G * m];
        if constexpr (AM) {
#pragma unroll
          for (int j = 0; j < EH; ++j)
            am[j] = (uint32_t)aline[t + G * (2 * j)] | ((uint32_t)aline[t + G * (2 * j + 1)] << 16);
        }
      }
    }
    // step i uses buffer bi for the (i >> 1)-th time: barrier phase (i >> 1) & 1
    const unsigned phase = (unsigned)((i >> 1) & 1);
    const bool late = !mbar_wait(&s_bar[bi], phase, (withheld && i == 0) ? kWithheldPolls : kWaitPolls);
    cp_async_wait<0>();
    // step i staged for everyone; everyone is done reading buffer (i+1) & 1
    if (__syncthreads_or(late)) {
      if (threadIdx.x == 0) {
        if (a.err) *reinterpret_cast<volatile int*>(a.err) = 1;  // may be mapped host memory
        // the copy this step waited for may still be landing: wait for it
        // (bounded) before the CTA's shared memory is released
        if (!(withheld && i == 0)) mbar_wait(&s_bar[bi], phase, kWaitPolls);
      }
      break;
    }
    issue(lg_next, nb_next, bi ^ 1);
    const float2* src = stage + bi * STG + g * H;
    float2 v[E];
    float2 mir[EH];
#pragma unroll
    for (int m = 0; m < EH; ++m) {
      float2 x = src[t + G * m];
      float2 xp = (m == 0 && t == 0) ? nyq[bi * NG + g] : src[H - t - G * m];
      if (m == 0 && t == 0) {
        x.y = 0.f;
        xp.y = 0.f;
      }
      const float2 xc = cconj(xp);
      const float2 xe = cadd(x, xc);
      const float2 xo = cmul(csub(x, xc), tw[t + G * m]);
      v[m] = make_float2(xe.x - xo.y, xe.y + xo.x);
      mir[m] = make_float2(xe.x + xo.y, xo.x - xe.y);
    }
    const float2 xm = src[H / 2];
    // Z[H-k] to the lane that owns it (lane G-t, register E-1-m)
#pragma unroll
    for (int m = 0; m < EH; ++m) {
      v[E - 1 - m].x = __shfl_sync(0xffffffffu, mir[m].x, partner, G);
      v[E - 1 - m].y = __shfl_sync(0xffffffffu, mir[m].y, partner, G);
    }
    if (t == 0) {
      // lane 0 received its own mirrors Z[G*(E-m)] one register low
#pragma unroll
      for (int j = E - 1; j > EH; --j) v[j] = v[j - 1];
      const float2 xc = cconj(xm);
      const float2 xe = cadd(xm, xc);
      const float2 xo = cmul(csub(xm, xc), tw[H / 2]);
      v[EH] = make_float2(xe.x - xo.y, xe.y + xo.x);
    }
    PlanRun<P>::template run<true>(v, buf, t, tws, sync);
    const float cb = MB ? __ldg(&bp->cb[b]) : s_cb[b];
    const float as = MB ? bp->as : a.as;
    const uint32_t rid = (uint32_t)((MB ? bp->r0 : a.r0) + b);
    float ss = 0.f;
#pragma unroll
    for (int m = 0; m < E; ++m) {
      const float x0 = v[m].x, x1 = v[m].y;
      const float z0 = fmaf(as, x0, cb), z1 = fmaf(as, x1, cb);
      if constexpr (AM) {
        const int sh = 16 * (m & 1);
        if (z0 > zr[m].x) {
          zr[m].x = z0;
          am[m >> 1] = (am[m >> 1] & ~(0xFFu << sh)) | (rid << sh);
        }
        if (z1 > zr[m].y) {
          zr[m].y = z1;
          am[m >> 1] = (am[m >> 1] & ~(0xFF00u << sh)) | (rid << (sh + 8));
        }
      } else {
        // without the argmax the strict update is a max: fmaxf keeps zr when
        // z is NaN (the barrier of a radius that never wins) and equal values
        // are the same number
        zr[m].x = fmaxf(zr[m].x, z0);
        zr[m].y = fmaxf(zr[m].y, z1);
      }
      if constexpr (SIG) ss = fmaf(x0, x0, fmaf(x1, x1, ss));
    }
    if constexpr (SIG) {
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) ss += __shfl_xor_sync(0xffffffffu, ss, o);
      if ((threadIdx.x & 31) == 0) atomicAdd(&red[b], (double)ss);
    }
    if (b == nb - 1) {
#pragma unroll
      for (int m = 0; m < E; ++m) {
        const int p = t + G * m;
        reinterpret_cast<float2*>(zout)[p] = zr[m];
        if constexpr (AM) aout[p] = (uint16_t)(am[m >> 1] >> (16 * (m & 1)));
      }
    }
    lg = lg_next;
    b = nb_next;
  }
  cp_async_wait<0>();
  if constexpr (SIG) {
    __syncthreads();
    if (threadIdx.x < a.nb) atomicAdd(&a.sig_acc[a.r0 + threadIdx.x], red[threadIdx.x]);
  }
}

}  // namespace prc
