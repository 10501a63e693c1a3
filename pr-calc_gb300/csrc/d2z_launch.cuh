// d2z_launch.cuh — host launchers for one grid size; included by inst_*.cu.
#pragma once
#include "d2z_adjoint.cuh"
#include "d2z_cols.cuh"
#include "d2z_dispatch.h"
#include "d2z_kernels.cuh"
#include "d2z_lines.cuh"

namespace prc {

static_assert(kWinVariants == kMaxWinVariants, "window variant table size");

// Column passes: k_col (one lane per column) where CCfg<N> has a plan, else
// k_tile (shared-memory staged tiles).
template <int N, bool COL = CCfg<N>::on> struct ColLaunch;

template <int N> struct ColLaunch<N, false> {
  using TT = TK<N>;
  static constexpr int THREADS = TT::THREADS, T = TT::T;
  static constexpr size_t TS = (size_t)TT::smem_f2 * sizeof(float2);    // one tile
  static constexpr size_t TS2 = (size_t)TT::smem2_f2 * sizeof(float2);  // two tiles (TM_WIN)
  template <int MODE> static void* fn() { return reinterpret_cast<void*>(&k_tile<N, MODE>); }
  static void* faithful_fn() { return reinterpret_cast<void*>(&k_tile<N, TM_WIN>); }
  static constexpr size_t FS = TS2;
  static constexpr int FTHREADS = THREADS;
  static size_t bytes(int mode) { return mode == TM_WIN ? TS2 : TS; }
  static int threads(int) { return THREADS; }
  static constexpr int T_ACC = T;
  // one window variant: the staged tile kernel
  static int win(int v, void** f = nullptr, int* thr = nullptr, size_t* by = nullptr, int* tw = nullptr) {
    if (v == 0) {
      if (f) *f = reinterpret_cast<void*>(&k_tile<N, TM_WIN>);
      if (thr) *thr = THREADS;
      if (by) *by = TS2;
      if (tw) *tw = T;
    }
    return 1;
  }
  static constexpr bool GROUPED = false;
  static void launch(int mode, dim3 grid, cudaStream_t st, const TileArgs& a) {
    switch (mode) {
      case TM_FWD: k_tile<N, TM_FWD><<<grid, THREADS, TS, st>>>(a); break;
      case TM_INV: k_tile<N, TM_INV><<<grid, THREADS, TS, st>>>(a); break;
      case TM_WIN: k_tile<N, TM_WIN><<<grid, THREADS, TS2, st>>>(a); break;
      default: k_tile<N, TM_ACC><<<grid, THREADS, TS, st>>>(a); break;
    }
  }
};

template <int N> struct ColLaunch<N, true> {
  using CC = typename ColK<N, TM_INV, 0>::type;
  using CA = typename ColK<N, TM_ACC, 0>::type;
  static constexpr int THREADS = CC::THREADS, T = CC::T;
  static constexpr int T_ACC = CA::T;
  static constexpr size_t CS = (size_t)CC::smem_f2 * sizeof(float2);
  static constexpr size_t CSA = (size_t)CA::smem_f2 * sizeof(float2);
  // window-pass variant v (when compiled for this N)
  template <int V> struct Win {
    static constexpr bool on = WinVar<N, V>::on;
    using K = typename ColK<N, TM_WIN, V>::type;
  };
  template <int MODE> static void* fn() { return reinterpret_cast<void*>(&k_col<N, MODE>); }
  static size_t bytes(int mode) { return mode == TM_ACC ? CSA : CS; }
  static int threads(int mode) { return mode == TM_ACC ? CA::THREADS : THREADS; }
  template <int V> static void win_info(int v, int* n, void** f, int* thr, size_t* by, int* tw) {
    if constexpr (V < kWinVariants) {
      if constexpr (Win<V>::on) {
        if (v == V) {
          *f = reinterpret_cast<void*>(&k_col<N, TM_WIN, V>);
          *thr = Win<V>::K::THREADS;
          *by = (size_t)Win<V>::K::smem_f2 * sizeof(float2);
          *tw = Win<V>::K::T;
        }
        *n = V + 1;
      }
      win_info<V + 1>(v, n, f, thr, by, tw);
    }
  }
  // number of window variants and, for variant v, its kernel, threads, bytes, tile width
  static int win(int v, void** f = nullptr, int* thr = nullptr, size_t* by = nullptr, int* tw = nullptr) {
    int n = 0, t0 = 0, w0 = 0;
    void* f0 = nullptr;
    size_t b0 = 0;
    win_info<0>(v, &n, f ? f : &f0, thr ? thr : &t0, by ? by : &b0, tw ? tw : &w0);
    return n;
  }
  using WF = typename ColK<N, TM_WIN, kWinFaithful>::type;
  static void* faithful_fn() { return reinterpret_cast<void*>(&k_col<N, TM_WIN, kWinFaithful>); }
  static constexpr size_t FS = (size_t)WF::smem_f2 * sizeof(float2);
  static constexpr int FTHREADS = WF::THREADS;
  template <int V> static void launch_win(int v, dim3 grid, cudaStream_t st, const TileArgs& a) {
    if (V == 0 && a.faithful) {
      k_col<N, TM_WIN, kWinFaithful><<<grid, FTHREADS, FS, st>>>(a);
      return;
    }
    if constexpr (V < kWinVariants) {
      if constexpr (Win<V>::on) {
        if (v == V) {
          k_col<N, TM_WIN, V><<<grid, Win<V>::K::THREADS, (size_t)Win<V>::K::smem_f2 * sizeof(float2), st>>>(a);
          return;
        }
      }
      launch_win<V + 1>(v, grid, st, a);
    }
  }
  static void launch(int mode, dim3 grid, cudaStream_t st, const TileArgs& a) {
    switch (mode) {
      case TM_FWD: k_col<N, TM_FWD><<<grid, THREADS, CS, st>>>(a); break;
      case TM_INV: k_col<N, TM_INV><<<grid, THREADS, CS, st>>>(a); break;
      case TM_WIN: launch_win<0>(a.win_var, grid, st, a); break;
      default: k_col<N, TM_ACC><<<grid, CA::THREADS, CSA, st>>>(a); break;
    }
  }
  // grouped launches (several boxes of this size per launch; window variant 0)
  static constexpr bool GROUPED = N <= 256 && PCfg<N>::on;
  using W0 = typename Win<0>::K;
  static constexpr size_t WS0 = (size_t)W0::smem_f2 * sizeof(float2);
  template <int MODE> static void* fn_mb() { return reinterpret_cast<void*>(&k_col<N, MODE, 0, true>); }
  static void launch_mb(int mode, dim3 grid, cudaStream_t st, const TileArgs& a) {
    if constexpr (GROUPED) {
      switch (mode) {
        case TM_FWD: k_col<N, TM_FWD, 0, true><<<grid, THREADS, CS, st>>>(a); break;
        case TM_INV: k_col<N, TM_INV, 0, true><<<grid, THREADS, CS, st>>>(a); break;
        default: k_col<N, TM_WIN, 0, true><<<grid, W0::THREADS, WS0, st>>>(a); break;
      }
    }
  }
};

// Inverse z pass: k_c2r_zp (mirror pairs in one lane) where PCfg<N> has a
// plan, else k_c2r_z.
template <int N, bool PAIR = PCfg<N>::on> struct C2rLaunch {
  static constexpr int THREADS = LK<N>::THREADS, NG = LK<N>::NG;
  static constexpr size_t BYTES = (size_t)LK<N>::smem_f2 * sizeof(float2);
  static constexpr int NFN = 1;
  static void* fn(int) { return reinterpret_cast<void*>(&k_c2r_z<N>); }
  static void launch(int grid, cudaStream_t st, const SweepArgs& a) { k_c2r_z<N><<<grid, THREADS, BYTES, st>>>(a); }
  static void launch_mb(int, cudaStream_t, const SweepArgs&) {}
};
template <int N> struct C2rLaunch<N, true> {
  static constexpr int THREADS = PK<N>::THREADS, NG = PK<N>::NG;
  static constexpr size_t BYTES = (size_t)PK<N>::smem_f2 * sizeof(float2);
  template <bool AM, bool SIG> static void* f() { return reinterpret_cast<void*>(&k_c2r_zp<N, AM, SIG>); }
  static constexpr int NFN = 4;
  static void* fn(int i) { return i == 0 ? f<false, false>() : i == 1 ? f<true, false>() : i == 2 ? f<false, true>() : f<true, true>(); }
  static void launch(int grid, cudaStream_t st, const SweepArgs& a) {
    if (a.sig_acc) {
      if (a.argmax) k_c2r_zp<N, true, true><<<grid, THREADS, BYTES, st>>>(a);
      else k_c2r_zp<N, false, true><<<grid, THREADS, BYTES, st>>>(a);
    } else {
      if (a.argmax) k_c2r_zp<N, true, false><<<grid, THREADS, BYTES, st>>>(a);
      else k_c2r_zp<N, false, false><<<grid, THREADS, BYTES, st>>>(a);
    }
  }
  // grouped: a.argmax != null means every box of the launch records its argmax
  template <bool AM> static void* f_mb() { return reinterpret_cast<void*>(&k_c2r_zp<N, AM, false, true>); }
  static void launch_mb(int grid, cudaStream_t st, const SweepArgs& a) {
    if (a.argmax) k_c2r_zp<N, true, false, true><<<grid, THREADS, BYTES, st>>>(a);
    else k_c2r_zp<N, false, false, true><<<grid, THREADS, BYTES, st>>>(a);
  }
};

template <int N> struct Launchers {
  using CL = ColLaunch<N>;
  using CR = C2rLaunch<N>;
  using LL = LK<N>;
  static constexpr size_t LS = (size_t)LL::smem_f2 * sizeof(float2);

  template <class F> static cudaError_t smem(F fn, size_t bytes) {
    return cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
  }
  template <class F> static cudaError_t occ(int* dst, F fn, int threads, size_t bytes) {
    cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(dst, fn, threads, bytes);
    if (*dst < 1) *dst = 1;
    return e;
  }
  static cudaError_t init(KernelSet* ks) {
    void* tf = CL::template fn<TM_FWD>();
    void* ti = CL::template fn<TM_INV>();
    void* ta = CL::template fn<TM_ACC>();
    cudaError_t e;
    if ((e = smem(tf, CL::bytes(TM_FWD))) != cudaSuccess) return e;
    if ((e = smem(ti, CL::bytes(TM_INV))) != cudaSuccess) return e;
    if ((e = smem(ta, CL::bytes(TM_ACC))) != cudaSuccess) return e;
    // window-pass variants
    ks->n_win_var = CL::win(0);
    for (int v = 0; v < ks->n_win_var; ++v) {
      void* f = nullptr;
      int thr = 0, tw = 0;
      size_t by = 0;
      CL::win(v, &f, &thr, &by, &tw);
      if ((e = smem(f, by)) != cudaSuccess) return e;
      if ((e = occ(&ks->occ_winv[v], f, thr, by)) != cudaSuccess) return e;
      ks->tile_w_winv[v] = tw;
    }
    ks->occ_tile_win = ks->occ_winv[0];
    ks->tile_w_win = ks->tile_w_winv[0];
    if constexpr (CL::GROUPED) {
      void* fm = CL::template fn_mb<TM_FWD>();
      void* im = CL::template fn_mb<TM_INV>();
      void* wm = CL::template fn_mb<TM_WIN>();
      if ((e = smem(fm, CL::CS)) != cudaSuccess) return e;
      if ((e = smem(im, CL::CS)) != cudaSuccess) return e;
      if ((e = smem(wm, CL::WS0)) != cudaSuccess) return e;
      if ((e = smem(CR::template f_mb<false>(), CR::BYTES)) != cudaSuccess) return e;
      if ((e = smem(CR::template f_mb<true>(), CR::BYTES)) != cudaSuccess) return e;
      if ((e = smem(&k_r2c_z<N, true>, LS)) != cudaSuccess) return e;
      if ((e = occ(&ks->occ_mb_tile, im, CL::THREADS, CL::CS)) != cudaSuccess) return e;
      if ((e = occ(&ks->occ_mb_win, wm, CL::W0::THREADS, CL::WS0)) != cudaSuccess) return e;
      if ((e = occ(&ks->occ_mb_c2r, CR::template f_mb<true>(), CR::THREADS, CR::BYTES)) != cudaSuccess) return e;
      if ((e = occ(&ks->occ_mb_r2c, &k_r2c_z<N, true>, LL::THREADS, LS)) != cudaSuccess) return e;
    }
    if ((e = smem(CL::faithful_fn(), CL::FS)) != cudaSuccess) return e;
    if ((e = occ(&ks->occ_win_faithful, CL::faithful_fn(), CL::FTHREADS, CL::FS)) != cudaSuccess) return e;
    if ((e = smem(&k_r2c_z<N>, LS)) != cudaSuccess) return e;
    for (int i = 0; i < CR::NFN; ++i)
      if ((e = smem(CR::fn(i), CR::BYTES)) != cudaSuccess) return e;
    if ((e = smem(&k_adj_z<N>, LS)) != cudaSuccess) return e;
    if ((e = smem(&k_c2r_plain<N>, LS)) != cudaSuccess) return e;
    if ((e = occ(&ks->occ_tile, ti, CL::THREADS, CL::bytes(TM_INV))) != cudaSuccess) return e;
    if ((e = occ(&ks->occ_tile_acc, ta, CL::threads(TM_ACC), CL::bytes(TM_ACC))) != cudaSuccess) return e;
    if ((e = occ(&ks->occ_r2c, &k_r2c_z<N>, LL::THREADS, LS)) != cudaSuccess) return e;
    if ((e = occ(&ks->occ_c2r, CR::fn(0), CR::THREADS, CR::BYTES)) != cudaSuccess) return e;
    if ((e = occ(&ks->occ_c2r_plain, &k_c2r_plain<N>, LL::THREADS, LS)) != cudaSuccess) return e;
    if ((e = occ(&ks->occ_adj_z, &k_adj_z<N>, LL::THREADS, LS)) != cudaSuccess) return e;
    return cudaSuccess;
  }
  static void r2c_z(const KernelSet&, int grid, cudaStream_t st, const float* d, float dinit, float2* S,
                    float2* Qt, const float2* tw) {
    k_r2c_z<N><<<grid, LL::THREADS, LS, st>>>(d, dinit, S, Qt, tw, nullptr, 0);
  }
  static void r2c_z_mb(const KernelSet&, int grid, cudaStream_t st, const BoxR2c* box, int nbox, const float2* tw) {
    if constexpr (CL::GROUPED) k_r2c_z<N, true><<<grid, LL::THREADS, LS, st>>>(nullptr, 1.f, nullptr, nullptr, tw, box, nbox);
  }
  static void tile_mb(const KernelSet&, int mode, dim3 grid, cudaStream_t st, const TileArgs& a) {
    CL::launch_mb(mode, grid, st, a);
  }
  static void c2r_z_mb(const KernelSet&, int grid, cudaStream_t st, const SweepArgs& a) {
    if constexpr (CL::GROUPED) CR::launch_mb(grid, st, a);
  }
  static void tile(const KernelSet&, int mode, dim3 grid, cudaStream_t st, const TileArgs& a) {
    CL::launch(mode, grid, st, a);
  }
  static void c2r_z(const KernelSet&, int grid, cudaStream_t st, const SweepArgs& a) { CR::launch(grid, st, a); }
  static void adj_z(const KernelSet&, int grid, cudaStream_t st, const AdjArgs& a) {
    k_adj_z<N><<<grid, LL::THREADS, LS, st>>>(a);
  }
  static void c2r_plain(const KernelSet&, int grid, cudaStream_t st, const AdjArgs& a) {
    k_c2r_plain<N><<<grid, LL::THREADS, LS, st>>>(a);
  }
  static KernelSet make() {
    KernelSet ks{};
    ks.N = N;
    ks.tile_threads = CL::THREADS;
    ks.tile_w = CL::T;
    ks.tile_w_acc = CL::T_ACC;
    ks.n_win_var = CL::win(0);
    ks.line_threads = LL::THREADS;
    ks.line_groups = LL::NG;
    ks.c2r_lines = CR::NG;
    ks.tile_smem = CL::bytes(TM_INV);
    ks.line_smem = LS;
    ks.init = &init;
    ks.r2c_z = &r2c_z;
    ks.tile = &tile;
    ks.c2r_z = &c2r_z;
    ks.adj_z = &adj_z;
    ks.c2r_plain = &c2r_plain;
    if constexpr (CL::GROUPED) {
      ks.grouped = 1;
      ks.tile_w_mb_win = CL::W0::T;
      ks.r2c_z_mb = &r2c_z_mb;
      ks.tile_mb = &tile_mb;
      ks.c2r_z_mb = &c2r_z_mb;
    }
    return ks;
  }
};

}  // namespace prc

#define PRC_INSTANTIATE(NV)                      \
  namespace prc {                                \
  const KernelSet* kernel_set_##NV() {           \
    static KernelSet ks = Launchers<NV>::make(); \
    return &ks;                                  \
  }                                              \
  }
