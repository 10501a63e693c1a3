// d2z_dispatch.h — per-grid-size kernel table.  Each supported N is compiled in
// its own translation unit (inst_*.cu) and registers one KernelSet.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace prc {

struct ColArgs;
struct SweepArgs;
struct AdjArgs;

struct KernelSet {
  int N;
  int col_threads, line_threads;
  int col_groups, line_groups;  // FFT groups per CTA (items a CTA step covers)
  size_t col_smem, line_smem;  // dynamic shared memory bytes
  // resident CTAs per SM (filled by init)
  int occ_col, occ_win, occ_r2c, occ_c2r, occ_adj_z, occ_adj_x;
  cudaError_t (*init)(KernelSet*);
  void (*r2c_z)(const KernelSet&, int grid, cudaStream_t, const float* delta, float dinit,
                float2* S, float2* Qt, const float2* tw);
  void (*col)(const KernelSet&, bool inv, dim3 grid, cudaStream_t, const ColArgs&);
  void (*win_x)(const KernelSet&, int grid, cudaStream_t, const SweepArgs&);
  void (*c2r_z)(const KernelSet&, int grid, cudaStream_t, const SweepArgs&);
  // adjoint: per-radius source R2C along z and the final window-accumulate x pass
  void (*adj_z)(const KernelSet&, int grid, cudaStream_t, const AdjArgs&);
  void (*adj_x)(const KernelSet&, int grid, cudaStream_t, const AdjArgs&);
  void (*c2r_plain)(const KernelSet&, int grid, cudaStream_t, const AdjArgs&);
};

// nullptr when N has no compiled plan
const KernelSet* kernel_set(int N);

}  // namespace prc
