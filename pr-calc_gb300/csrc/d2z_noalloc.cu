// d2z_noalloc.cu — prc_d2z_forward_static: the forward path for small boxes
// without any device allocation.
//
// Some callers cannot allocate device memory at the moment they need a
// result: a host framework that owns every byte of device memory through its
// own pool and forbids outside cudaMalloc calls, or a latency-critical
// pipeline stage that must not pay for cudaMalloc/cudaFree, which can
// synchronise the whole device.  For them this entry point keeps its whole
// workspace (the half spectrum, one radius slot and the twiddle table) in the
// file-scope array below, which every GPU that loads the library holds until
// the process exits.  The caller passes device pointers for the input and the
// outputs; nothing else is allocated, by this code or by any library it calls.
//
// Limits and sharing: the array is sized for grids up to N = 64 (about
// 2.2 MB).  All calls share it and it keeps the last call's contents, so two
// calls whose work overlaps on the GPU (different streams, or different host
// threads on one device) race on it; serialise them.  The twiddle tables of
// every supported N are written once per device, at the first call; the
// spectrum and the slot need not start at zero (every call writes them before
// reading them, and the first radius writes zreion and argmax without reading
// them).  The one word that must start at zero, the kernels' error word (a
// second file-scope array), is cleared on the stream at the start of every
// call and read back after the call's synchronisation.
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>
#include <string.h>

#include <mutex>

#include "../../include/prc_d2z.h"
#include "d2z_dispatch.h"
#include "d2z_kernels.cuh"
#include "errors.h"

namespace {

constexpr int kStaticMaxN = 64;
constexpr long long kStaticSlotF2 = (long long)kStaticMaxN * kStaticMaxN * (kStaticMaxN / 2 + 2);
constexpr int kSmallN[7] = {8, 12, 16, 24, 32, 48, 64};
constexpr int kTwAll = 8 + 12 + 16 + 24 + 32 + 48 + 64;  // one twiddle table per supported N
// spectrum + one radius slot + the twiddle tables, in float2
constexpr long long kStaticF2 = 2 * kStaticSlotF2 + kTwAll;

static __device__ __align__(256) float2 g_static_scratch[kStaticF2];
static __device__ __align__(256) int g_static_err[1];  // set by a z-pass CTA whose copy wait ran out

constexpr int kMaxDevices = 64;
std::mutex g_setup_mu;
float2* g_scratch_ptr[kMaxDevices] = {};      // device address of g_static_scratch, per device
int* g_err_ptr[kMaxDevices] = {};             // device address of g_static_err, per device
prc::KernelSet g_ks[kMaxDevices][7];          // per device, per supported small N
bool g_ready[kMaxDevices] = {};

// offset of grid side N's twiddle table after the spectrum and the slot
int tw_offset(int si) {
  int o = 0;
  for (int i = 0; i < si; ++i) o += kSmallN[i];
  return o;
}

// Per-device set-up, with that device current: the device addresses of the
// two arrays (their host-side names are only stand-ins), every small N's
// twiddle table e^{+2 pi i k/N} (built in FP64, one synchronous copy) and the
// kernels' shared-memory limits.
int setup_device(int dev) {
  using namespace prc;
  void* p = nullptr;
  cudaError_t e = cudaGetSymbolAddress(&p, g_static_scratch);
  if (e != cudaSuccess || !p)
    return prc_fail(PRC_ERR_CUDA, "prc_d2z_forward_static: cudaGetSymbolAddress: %s", cudaGetErrorString(e));
  void* q = nullptr;
  e = cudaGetSymbolAddress(&q, g_static_err);
  if (e != cudaSuccess || !q)
    return prc_fail(PRC_ERR_CUDA, "prc_d2z_forward_static: cudaGetSymbolAddress: %s", cudaGetErrorString(e));
  float2 htw[kTwAll];
  for (int si = 0; si < 7; ++si) {
    const int N = kSmallN[si];
    for (int k = 0; k < N; ++k) {
      const double ang = 2.0 * M_PI * (double)k / (double)N;
      htw[tw_offset(si) + k] = make_float2((float)cos(ang), (float)sin(ang));
    }
  }
  float2* tw = static_cast<float2*>(p) + 2 * kStaticSlotF2;
  e = cudaMemcpy(tw, htw, sizeof(htw), cudaMemcpyHostToDevice);
  if (e != cudaSuccess)
    return prc_fail(PRC_ERR_CUDA, "prc_d2z_forward_static: twiddle tables: %s", cudaGetErrorString(e));
  for (int si = 0; si < 7; ++si) {
    const KernelSet* ks = kernel_set(kSmallN[si]);
    if (!ks) return prc_fail(PRC_ERR_UNSUPPORTED, "prc_d2z_forward_static: no FFT plan for N=%d", kSmallN[si]);
    g_ks[dev][si] = *ks;
    e = ks->init(&g_ks[dev][si]);
    if (e != cudaSuccess)
      return prc_fail(PRC_ERR_CUDA, "prc_d2z_forward_static: kernel set-up: %s", cudaGetErrorString(e));
  }
  g_scratch_ptr[dev] = static_cast<float2*>(p);
  g_err_ptr[dev] = static_cast<int*>(q);
  g_ready[dev] = true;
  return PRC_OK;
}

int small_index(int N) {
  switch (N) {
    case 8: return 0;
    case 12: return 1;
    case 16: return 2;
    case 24: return 3;
    case 32: return 4;
    case 48: return 5;
    case 64: return 6;
    default: return -1;
  }
}

int grid_of(int items, int occ, int sms) {
  const long long cap = (long long)occ * sms;
  return (int)(items < cap ? (items < 1 ? 1 : items) : cap);
}

}  // namespace

extern "C" int prc_d2z_forward_static(int N, int n_radii, double box_mpc, const double* radii_mpc,
                                      const double* barrier_b, double barrier_a, double growth_init,
                                      const float* d_delta, float* d_zreion, uint8_t* d_argmax,
                                      void* stream) {
  using namespace prc;
  const int si = small_index(N);
  if (si < 0)
    return prc_fail(PRC_ERR_INVALID,
                    "prc_d2z_forward_static: grid side N=%d is not one of 8,12,16,24,32,48,64 "
                    "(the static workspace holds boxes up to N=%d)", N, kStaticMaxN);
  if (n_radii < 1 || n_radii > PRC_MAX_RADII)
    return prc_fail(PRC_ERR_INVALID, "prc_d2z_forward_static: n_radii=%d outside 1..%d", n_radii, PRC_MAX_RADII);
  if (!radii_mpc || !barrier_b || !d_delta || !d_zreion)
    return prc_fail(PRC_ERR_INVALID, "prc_d2z_forward_static: null argument");
  if (!(box_mpc > 0) || !(growth_init > 0) || !(barrier_a > 0))
    return prc_fail(PRC_ERR_INVALID, "prc_d2z_forward_static: box, growth and barrier_a must be > 0");
  for (int r = 0; r < n_radii; ++r)
    if (!(radii_mpc[r] > 0)) return prc_fail(PRC_ERR_INVALID, "prc_d2z_forward_static: radius %d not > 0", r);

  int dev = 0, sms = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e == cudaSuccess && (dev < 0 || dev >= kMaxDevices)) e = cudaErrorInvalidDevice;
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  if (e != cudaSuccess) return prc_fail(PRC_ERR_CUDA, "prc_d2z_forward_static: device query: %s", cudaGetErrorString(e));
  // Set-up, once per device, with that device current (setup_device).  It
  // happens inside the first call on a device, so make that first call before
  // any stream capture begins.
  {
    std::lock_guard<std::mutex> lk(g_setup_mu);
    if (!g_ready[dev]) {
      const int st = setup_device(dev);
      if (st != PRC_OK) return st;
    }
  }
  const KernelSet& ks = g_ks[dev][si];
  cudaStream_t st = (cudaStream_t)stream;
  const int H = N / 2;
  const long long NN = (long long)N * N, slot_f2 = NN * (H + 2);
  float2* spec = g_scratch_ptr[dev];
  float2* slot = spec + slot_f2;
  const float2* tw = spec + 2 * kStaticSlotF2 + tw_offset(si);
  int* d_err = g_err_ptr[dev];
  e = cudaMemsetAsync(d_err, 0, sizeof(int), st);
  if (e != cudaSuccess) return prc_fail(PRC_ERR_CUDA, "prc_d2z_forward_static: clear error word: %s", cudaGetErrorString(e));
  const bool withhold = take_withhold();

  auto mseg = [&](const float2* in, float2* out, bool xpass) {
    TileSeg s;
    s.in = in;
    s.out = out;
    s.row_stride = xpass ? N * H : H;
    s.outer_stride = xpass ? H : N * H;
    s.n_outer = N;
    s.tpo = H / ks.tile_w;
    s.transpose = 0;
    s.nyq = 0;
    return s;
  };
  auto qseg = [&](const float2* in, float2* out, bool transpose) {
    TileSeg s;
    s.in = in;
    s.out = out;
    s.row_stride = N;
    s.outer_stride = 0;
    s.n_outer = 1;
    s.tpo = N / ks.tile_w;
    s.transpose = transpose ? 1 : 0;
    s.nyq = 1;
    return s;
  };
  auto tile = [&](int mode, TileSeg s0, TileSeg s1, int r) {
    if (mode == TM_WIN) {
      s0.tpo = (s0.nyq ? N : H) / ks.tile_w_win;
      s1.tpo = (s1.nyq ? N : H) / ks.tile_w_win;
    }
    TileArgs a;
    memset(&a, 0, sizeof(a));
    a.seg[0] = s0;
    a.seg[1] = s1;
    a.slot_stride = slot_f2;
    a.tw = tw;
    a.nb = 1;
    if (mode == TM_WIN) a.kr[0] = (float)(2.0 * M_PI / box_mpc * radii_mpc[r]);
    const int tiles = s0.n_outer * s0.tpo + s1.n_outer * s1.tpo;
    ks.tile(ks, mode, dim3(grid_of(tiles, mode == TM_WIN ? ks.occ_tile_win : ks.occ_tile, sms), 1, 1), st, a);
  };
  // forward R2C: z lines, then y and x column passes (Nyquist plane via the
  // transposed scratch after it in the spectrum region)
  float2* S = spec;
  float2* Q = spec + NN * H;
  float2* Qt = spec + NN * (H + 1);
  ks.r2c_z(ks, grid_of((N * N + ks.line_groups - 1) / ks.line_groups, ks.occ_r2c, sms), st, d_delta,
           (float)growth_init, S, Qt, tw);
  tile(TM_FWD, mseg(S, S, false), qseg(Qt, Q, true), 0);
  tile(TM_FWD, mseg(S, S, true), qseg(Q, Q, false), 0);
  // one radius per sweep through the single slot
  const double n3 = (double)NN * N;
  for (int r = 0; r < n_radii; ++r) {
    tile(TM_WIN, mseg(spec, slot, true), qseg(spec + NN * H, slot + NN * H, true), r);
    tile(TM_INV, mseg(slot, slot, false), qseg(slot + NN * H, slot + NN * H, false), 0);
    SweepArgs sa;
    memset(&sa, 0, sizeof(sa));
    sa.slots = slot;
    sa.slot_stride = slot_f2;
    sa.tw = tw;
    sa.zreion = d_zreion;
    sa.argmax = d_argmax;
    sa.zreion_out = d_zreion;
    sa.argmax_out = d_argmax;
    sa.sig_acc = nullptr;
    sa.err = d_err;
    sa.withhold = (withhold && r == 0) ? 1 : 0;
    sa.nb = 1;
    sa.r0 = r;
    sa.first = (r == 0);
    sa.as = (float)(barrier_a / n3);
    sa.cb[0] = (float)(barrier_a * barrier_b[r] - 1.0);
    ks.c2r_z(ks, grid_of((N * N + ks.c2r_lines - 1) / ks.c2r_lines, ks.occ_c2r, sms), st, sa);
  }
  int h_err = 0;
  e = cudaGetLastError();
  if (e == cudaSuccess) e = cudaMemcpyAsync(&h_err, d_err, sizeof(int), cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) return prc_fail(PRC_ERR_CUDA, "prc_d2z_forward_static: %s", cudaGetErrorString(e));
  if (h_err)
    return prc_fail(PRC_ERR_CUDA, "prc_d2z_forward_static: a staging copy did not complete within the wait limit");
  return PRC_OK;
}
