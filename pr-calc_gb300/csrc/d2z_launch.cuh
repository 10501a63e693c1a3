// d2z_launch.cuh — host launchers for one grid size; included by inst_*.cu.
#pragma once
#include "d2z_dispatch.h"
#include "d2z_kernels.cuh"
#include "d2z_adjoint.cuh"

namespace prc {

template <int N> struct Launchers {
  using KK = K<N>;
  static constexpr size_t CS = (size_t)KK::col_smem_f2 * sizeof(float2);
  static constexpr size_t LS = (size_t)KK::line_smem_f2 * sizeof(float2);

  template <class F> static cudaError_t smem(F fn, size_t bytes) {
    return cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
  }
  template <class F> static cudaError_t occ(int* dst, F fn, int threads, size_t bytes) {
    cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(dst, fn, threads, bytes);
    if (*dst < 1) *dst = 1;
    return e;
  }
  static cudaError_t init(KernelSet* ks) {
    void (*col_inv)(ColArgs) = &k_col<N, true>;
    void (*col_fwd)(ColArgs) = &k_col<N, false>;
    cudaError_t e;
    if ((e = smem(col_inv, CS)) != cudaSuccess) return e;
    if ((e = smem(col_fwd, CS)) != cudaSuccess) return e;
    if ((e = smem(&k_win_x<N>, CS)) != cudaSuccess) return e;
    if ((e = smem(&k_r2c_z<N>, LS)) != cudaSuccess) return e;
    if ((e = smem(&k_c2r_z<N>, LS)) != cudaSuccess) return e;
    if ((e = smem(&k_adj_z<N>, LS)) != cudaSuccess) return e;
    if ((e = smem(&k_adj_x<N>, CS)) != cudaSuccess) return e;
    if ((e = smem(&k_c2r_plain<N>, LS)) != cudaSuccess) return e;
    if ((e = occ(&ks->occ_col, col_inv, KK::COL_THREADS, CS)) != cudaSuccess) return e;
    if ((e = occ(&ks->occ_win, &k_win_x<N>, KK::COL_THREADS, CS)) != cudaSuccess) return e;
    if ((e = occ(&ks->occ_r2c, &k_r2c_z<N>, KK::LINE_THREADS, LS)) != cudaSuccess) return e;
    if ((e = occ(&ks->occ_c2r, &k_c2r_z<N>, KK::LINE_THREADS, LS)) != cudaSuccess) return e;
    if ((e = occ(&ks->occ_adj_z, &k_adj_z<N>, KK::LINE_THREADS, LS)) != cudaSuccess) return e;
    if ((e = occ(&ks->occ_adj_x, &k_adj_x<N>, KK::COL_THREADS, CS)) != cudaSuccess) return e;
    return cudaSuccess;
  }
  static void r2c_z(const KernelSet&, int grid, cudaStream_t st, const float* d, float dinit,
                    float2* S, float2* Qt, const float2* tw) {
    k_r2c_z<N><<<grid, KK::LINE_THREADS, LS, st>>>(d, dinit, S, Qt, tw);
  }
  static void col(const KernelSet&, bool inv, dim3 grid, cudaStream_t st, const ColArgs& a) {
    if (inv)
      k_col<N, true><<<grid, KK::COL_THREADS, CS, st>>>(a);
    else
      k_col<N, false><<<grid, KK::COL_THREADS, CS, st>>>(a);
  }
  static void win_x(const KernelSet&, int grid, cudaStream_t st, const SweepArgs& a) {
    k_win_x<N><<<grid, KK::COL_THREADS, CS, st>>>(a);
  }
  static void c2r_z(const KernelSet&, int grid, cudaStream_t st, const SweepArgs& a) {
    k_c2r_z<N><<<grid, KK::LINE_THREADS, LS, st>>>(a);
  }
  static void adj_z(const KernelSet&, int grid, cudaStream_t st, const AdjArgs& a) {
    k_adj_z<N><<<grid, KK::LINE_THREADS, LS, st>>>(a);
  }
  static void adj_x(const KernelSet&, int grid, cudaStream_t st, const AdjArgs& a) {
    k_adj_x<N><<<grid, KK::COL_THREADS, CS, st>>>(a);
  }
  static void c2r_plain(const KernelSet&, int grid, cudaStream_t st, const AdjArgs& a) {
    k_c2r_plain<N><<<grid, KK::LINE_THREADS, LS, st>>>(a);
  }
  static KernelSet make() {
    KernelSet ks{};
    ks.N = N;
    ks.col_threads = KK::COL_THREADS;
    ks.line_threads = KK::LINE_THREADS;
    ks.col_groups = KK::CNG;
    ks.line_groups = KK::LNG;
    ks.col_smem = CS;
    ks.line_smem = LS;
    ks.init = &init;
    ks.r2c_z = &r2c_z;
    ks.col = &col;
    ks.win_x = &win_x;
    ks.c2r_z = &c2r_z;
    ks.adj_z = &adj_z;
    ks.adj_x = &adj_x;
    ks.c2r_plain = &c2r_plain;
    return ks;
  }
};

}  // namespace prc

#define PRC_INSTANTIATE(NV)                                        \
  namespace prc {                                                  \
  const KernelSet* kernel_set_##NV() {                             \
    static KernelSet ks = Launchers<NV>::make();                   \
    return &ks;                                                    \
  }                                                                \
  }
