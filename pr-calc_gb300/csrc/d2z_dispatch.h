// d2z_dispatch.h — per-grid-size kernel table.  Each supported N is compiled in
// a translation unit inst_*.cu and registers one KernelSet.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace prc {

constexpr int kMaxWinVariants = 3;  // window-pass variants per grid size (autotuned)

struct TileArgs;
struct SweepArgs;
struct AdjArgs;
struct BoxR2c;

struct KernelSet {
  int N;
  int tile_threads, tile_w;     // threads per column-pass CTA, columns per tile
  int tile_w_win;               // columns per tile of the window pass (variant 0)
  int n_win_var;                // window-pass variants compiled for this N
  int tile_w_winv[kMaxWinVariants], occ_winv[kMaxWinVariants];  // per variant
  int tile_w_acc;               // columns per tile of the accumulate pass (adjoint)
  int line_threads, line_groups;  // threads per line-pass CTA, lines per CTA step
  int c2r_lines;                  // lines per CTA step of the inverse z pass
  size_t tile_smem, line_smem;  // dynamic shared memory bytes
  // resident CTAs per SM (filled by init)
  int occ_tile, occ_tile_win, occ_tile_acc, occ_r2c, occ_c2r, occ_c2r_plain, occ_adj_z;
  int occ_win_faithful;         // the window pass with the reference's float window
  cudaError_t (*init)(KernelSet*);
  void (*r2c_z)(const KernelSet&, int grid, cudaStream_t, const float* delta, float dinit,
                float2* S, float2* Qt, const float2* tw);
  // mode: TM_FWD, TM_INV, TM_WIN, TM_ACC
  void (*tile)(const KernelSet&, int mode, dim3 grid, cudaStream_t, const TileArgs&);
  void (*c2r_z)(const KernelSet&, int grid, cudaStream_t, const SweepArgs&);
  void (*adj_z)(const KernelSet&, int grid, cudaStream_t, const AdjArgs&);
  void (*c2r_plain)(const KernelSet&, int grid, cudaStream_t, const AdjArgs&);
  // grouped launches (several boxes of this size per launch), when compiled
  // for this size (grouped = 1): forward z pass, column passes (TM_FWD,
  // TM_INV, TM_WIN with window variant 0), inverse z pass
  int grouped;
  int tile_w_mb_win;
  int occ_mb_tile, occ_mb_win, occ_mb_c2r, occ_mb_r2c;
  void (*r2c_z_mb)(const KernelSet&, int grid, cudaStream_t, const BoxR2c* box, int nbox, const float2* tw);
  void (*tile_mb)(const KernelSet&, int mode, dim3 grid, cudaStream_t, const TileArgs&);
  void (*c2r_z_mb)(const KernelSet&, int grid, cudaStream_t, const SweepArgs&);
};

// nullptr when N has no compiled plan
const KernelSet* kernel_set(int N);

// true (and one fewer pending) when prc_d2z_test_withhold_copy asked for a
// withheld staging copy in the next forward call
bool take_withhold();

}  // namespace prc
