// d2z_capi.cu — C ABI of the GB300 delta2zreion path (include/prc_d2z.h).
//
// Owns the per-box device workspace and sequences the kernels of
// d2z_kernels.cuh / d2z_adjoint.cuh on the caller's stream:
//   forward : R2C (z line pass, y and x column passes), then per sweep of up to
//             B radii: window + x pass -> y pass -> z line pass with barrier/max.
//   backward: per sweep: source R2C along z -> y pass -> x pass with window
//             accumulate; then the inverse column passes and a plain z C2R.
// Replaces AllocateArrays (allocate_d2z.C:5-44), the FFTW plans and executes
// (main_d2z.C:32-48,67; delta2zreion_d2z.C:92) and the delta2zreion loop.
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>
#include <string.h>

#include <algorithm>
#include <atomic>
#include <vector>

#include "../../include/prc_d2z.h"
#include "d2z_adjoint.cuh"
#include "d2z_dispatch.h"
#include "errors.h"
#include "history.h"

namespace prc {
#define PRC_DECL(NV) const KernelSet* kernel_set_##NV();
PRC_DECL(8) PRC_DECL(12) PRC_DECL(16) PRC_DECL(24) PRC_DECL(32) PRC_DECL(48) PRC_DECL(64)
PRC_DECL(96) PRC_DECL(128) PRC_DECL(192) PRC_DECL(256) PRC_DECL(384) PRC_DECL(512) PRC_DECL(768)
PRC_DECL(1024)
#undef PRC_DECL

// Test hook (prc_d2z_test_withhold_copy): how many forward calls still run
// their first sweep with one staging copy withheld.
std::atomic<int> g_withhold{0};

bool take_withhold() {
  int v = g_withhold.load();
  while (v > 0 && !g_withhold.compare_exchange_weak(v, v - 1)) {
  }
  return v > 0;
}

const KernelSet* kernel_set(int N) {
  switch (N) {
    case 8: return kernel_set_8();
    case 12: return kernel_set_12();
    case 16: return kernel_set_16();
    case 24: return kernel_set_24();
    case 32: return kernel_set_32();
    case 48: return kernel_set_48();
    case 64: return kernel_set_64();
    case 96: return kernel_set_96();
    case 128: return kernel_set_128();
    case 192: return kernel_set_192();
    case 256: return kernel_set_256();
    case 384: return kernel_set_384();
    case 512: return kernel_set_512();
    case 768: return kernel_set_768();
    case 1024: return kernel_set_1024();
    default: return nullptr;
  }
}

// ------------------------------------------------------------ history binning
// bin = (int)((z - 49.9) / dz), dz = float((0.01 - 49.9)/(1e5 - 1)), evaluated
// in double exactly as bubblehistory_d2z.C:23 does; a float estimate decides
// every cell that is not within 0.05 of a bin edge.
__global__ void k_hist(const float* __restrict__ z, long long n, uint32_t* counts, double dzd) {
  const float inv = (float)(1.0 / dzd);
  const long long stride = (long long)gridDim.x * blockDim.x;
  const long long base = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const long long iters = (n + stride - 1) / stride;
  for (long long it = 0; it < iters; ++it) {
    const long long i = base + it * stride;
    const bool valid = i < n;
    const float zc = valid ? z[i] : 0.f;
    const float qf = (zc - 49.9f) * inv;
    int bin = -1;
    if (fabsf(qf) < 1e9f) {
      const float r = rintf(qf);
      if (fabsf(qf - r) < 0.05f)
        bin = (int)(((double)zc - 49.9) / dzd);
      else
        bin = (int)qf;
    }
    const bool ok = valid && bin >= 0 && bin < kNHistory;
    const int key = ok ? bin : -1;
    const unsigned peers = __match_any_sync(0xffffffffu, key);
    const int leader = __ffs(peers) - 1;
    if (ok && (int)(threadIdx.x & 31) == leader) atomicAdd(&counts[bin], (uint32_t)__popc(peers));
  }
}

// ------------------------------------------------------------ skewer walks
// GetBubbleMFP's walks (bubblehistory_d2z.C:159-183 and :197-221): from each
// start cell step along +y (then +z), periodically, until the first cell with
// zreion < zcur or back at the start; steps = number of moves.  At most N
// moves per walk.
__global__ void k_walks(const float* __restrict__ z, int N, const int* __restrict__ start,
                        const float* __restrict__ zcur, int ns, long long total, int* steps) {
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long s = (long long)blockIdx.x * blockDim.x + threadIdx.x; s < total; s += stride) {
    const float zc = zcur[s / ns];
    const int i = start[3 * s], j0 = start[3 * s + 1], k0 = start[3 * s + 2];
    const float* plane = z + (long long)i * N * N;
    int j = j0, m = 0;
    for (;;) {
      if (++j >= N) j -= N;
      ++m;
      if (plane[(long long)j * N + k0] < zc || j == j0) break;
    }
    steps[2 * s] = m;
    const float* line = plane + (long long)j0 * N;
    int k = k0;
    m = 0;
    for (;;) {
      if (++k >= N) k -= N;
      ++m;
      if (line[k] < zc || k == k0) break;
    }
    steps[2 * s + 1] = m;
  }
}

// CorrectHistory's per-cell map (bubblehistory_d2z.C:328-341) with the bin of
// k_hist; bins outside the table leave the cell unchanged.
__global__ void k_remap(float* __restrict__ z, long long n, const float* __restrict__ zvz, double dzd) {
  const float inv = (float)(1.0 / dzd);
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
    const float zc = z[i];
    const float qf = (zc - 49.9f) * inv;
    if (!(fabsf(qf) < 1e9f)) continue;
    const float r = rintf(qf);
    const int bin = (fabsf(qf - r) < 0.05f) ? (int)(((double)zc - 49.9) / dzd) : (int)qf;
    if (bin >= 0 && bin < kNHistory) z[i] = __ldg(zvz + bin);
  }
}

// ---------------------------------------------------------------- field generator
// Unit Gaussian white noise per cell: Philox4x32-10 (Salmon et al., SC 2011)
// with counter (cell & 0xffffffff, cell >> 32, 0, 0) and key (seed, 0), then
// Box-Muller in FP64 on words 0 and 1: sqrt(-2 ln u1) cos(2 pi u2),
// u = (word + 1/2) / 2^32.  Rounded to float32.
__global__ void k_white_noise(float* __restrict__ out, long long n, uint32_t seed) {
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
    uint32_t c0 = (uint32_t)(i & 0xffffffffll), c1 = (uint32_t)(i >> 32), c2 = 0u, c3 = 0u;
    uint32_t k0 = seed, k1 = 0u;
#pragma unroll
    for (int r = 0; r < 10; ++r) {
      if (r) {
        k0 += 0x9E3779B9u;
        k1 += 0xBB67AE85u;
      }
      const uint32_t hi0 = __umulhi(c0, 0xD2511F53u), lo0 = c0 * 0xD2511F53u;
      const uint32_t hi1 = __umulhi(c2, 0xCD9E8D57u), lo1 = c2 * 0xCD9E8D57u;
      const uint32_t n0 = hi1 ^ c1 ^ k0, n2 = hi0 ^ c3 ^ k1;
      c0 = n0;
      c1 = lo1;
      c2 = n2;
      c3 = lo0;
    }
    const double u1 = ((double)c0 + 0.5) / 4294967296.0;
    const double u2 = ((double)c1 + 0.5) / 4294967296.0;
    out[i] = (float)(sqrt(-2.0 * log(u1)) * cos(2.0 * M_PI * u2));
  }
}

// Half spectrum (main X[ix][iy][kz<H] and the Nyquist plane Q[ix][iy]) times
// amp[|m|^2], |m|^2 = fx^2 + fy^2 + kz^2 with f folded to |f| <= N/2.
__global__ void k_grf_amp(float2* __restrict__ spec, int N, const float* __restrict__ amp) {
  const int H = N / 2;
  const long long NN = (long long)N * N, total = NN * (H + 1);
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < total; i += stride) {
    int ix, iy, kz;
    if (i < NN * H) {
      kz = (int)(i % H);
      const long long l = i / H;
      ix = (int)(l / N);
      iy = (int)(l % N);
    } else {
      const long long q = i - NN * H;
      ix = (int)(q / N);
      iy = (int)(q % N);
      kz = H;
    }
    const int fx = ix <= H ? ix : N - ix, fy = iy <= H ? iy : N - iy;
    const float a = amp[fx * fx + fy * fy + kz * kz];
    const float2 v = spec[i];
    spec[i] = make_float2(v.x * a, v.y * a);
  }
}

}  // namespace prc

using namespace prc;

struct prc_d2z_ctx {
  int N = 0, H = 0, nr = 0, B = 0, flags = 0, dev = 0, sms = 0;
  int win_var = 0;   // window-pass variant (prc_d2z_tune)
  int slots_b = 0;   // radius slots allocated
  long long NN = 0, slot_f2 = 0;
  double box = 0, A = 0, dinit = 1;
  std::vector<double> R, Bb;
  std::vector<float> kr, cb;
  float as = 0;
  cudaStream_t st = nullptr;
  const KernelSet* ks = nullptr;
  KernelSet ksl{};
  float2* spec = nullptr;
  float2* slots = nullptr;
  float2* tw = nullptr;
  float* zre = nullptr;
  uint8_t* am = nullptr;
  double* sig = nullptr;
  double* dB = nullptr;
  uint32_t* counts = nullptr;
  float* gstage = nullptr;
  uint8_t* amstage = nullptr;
  float* grf_amp = nullptr;       // field generator: amplitude by |m|^2
  // set by a kernel whose copy wait ran out: one word of pinned host memory
  // mapped into the device (err its device address, err_h the host's), so
  // that the host reads it after the stream synchronisation without a copy
  int* err = nullptr;
  int* err_h = nullptr;
  // prc_d2z_forward_many: two device copies of a box's input and outputs and
  // two copy streams (in, out), so that the copies of neighbouring boxes run
  // on the copy engines while this box's kernels run
  float* m_delta[2] = {nullptr, nullptr};
  float* m_z[2] = {nullptr, nullptr};
  uint8_t* m_am[2] = {nullptr, nullptr};
  cudaStream_t m_copy[2] = {nullptr, nullptr};
  cudaEvent_t m_in[2] = {nullptr, nullptr};    // input copied
  cudaEvent_t m_read[2] = {nullptr, nullptr};  // input consumed (forward R2C done)
  cudaEvent_t m_done[2] = {nullptr, nullptr};  // outputs final
  cudaEvent_t m_out[2] = {nullptr, nullptr};   // outputs copied out
  cudaEvent_t ev[4] = {nullptr, nullptr, nullptr, nullptr};
  float last_ms[3] = {0, 0, 0};
  int have_timing = 0;
  int launches = 0;
  // per-kernel-kind event timing (prc_d2z_profile)
  int prof = 0;
  std::vector<cudaEvent_t> pev;   // pairs
  std::vector<int> pkind;         // kind of each pair
  size_t pused = 0;
  double kind_ms[PRC_NKINDS] = {0};
  long long kind_n[PRC_NKINDS] = {0};
};

namespace {

// Brackets one launch with a pair of events when profiling is on.
struct Prof {
  prc_d2z_ctx* c;
  size_t i = (size_t)-1;
  Prof(prc_d2z_ctx* c_, int kind) : c(c_) {
    if (!c->prof) return;
    if (c->pused * 2 + 2 > c->pev.size()) {
      cudaEvent_t a, b;
      if (cudaEventCreate(&a) != cudaSuccess || cudaEventCreate(&b) != cudaSuccess) return;
      c->pev.push_back(a);
      c->pev.push_back(b);
      c->pkind.push_back(0);
    }
    i = c->pused++;
    c->pkind[i] = kind;
    cudaEventRecord(c->pev[2 * i], c->st);
  }
  ~Prof() {
    if (i != (size_t)-1) cudaEventRecord(c->pev[2 * i + 1], c->st);
  }
};

// after a stream sync: fold the recorded pairs into the per-kind totals
void prof_collect(prc_d2z_ctx* c) {
  for (size_t i = 0; i < c->pused; ++i) {
    float ms = 0;
    if (cudaEventElapsedTime(&ms, c->pev[2 * i], c->pev[2 * i + 1]) == cudaSuccess) {
      c->kind_ms[c->pkind[i]] += ms;
      c->kind_n[c->pkind[i]] += 1;
    }
  }
  c->pused = 0;
}

int cuda_fail(cudaError_t e, const char* what) {
  return prc_fail(PRC_ERR_CUDA, "%s: %s", what, cudaGetErrorString(e));
}
#define PRC_CU(call, what)                           \
  do {                                               \
    cudaError_t e_ = (call);                         \
    if (e_ != cudaSuccess) return cuda_fail(e_, what); \
  } while (0)

int grid_for(int items, int per_cta, int occ, int sms) {
  long long need = (items + per_cta - 1) / per_cta;
  long long cap = (long long)occ * sms;
  if (need < 1) need = 1;
  return (int)(need < cap ? need : cap);
}

template <class T> int dalloc(T** p, size_t count, const char* what) {
  cudaError_t e = cudaMalloc((void**)p, count * sizeof(T));
  if (e != cudaSuccess) {
    *p = nullptr;
    cudaGetLastError();
    return prc_fail(PRC_ERR_ALLOC, "cudaMalloc %s (%zu bytes): %s", what, count * sizeof(T),
                    cudaGetErrorString(e));
  }
  return PRC_OK;
}

void free_all(prc_d2z_ctx* c) {
  cudaFree(c->spec);
  cudaFree(c->slots);
  cudaFree(c->tw);
  cudaFree(c->zre);
  cudaFree(c->am);
  cudaFree(c->sig);
  cudaFree(c->dB);
  cudaFree(c->counts);
  cudaFree(c->gstage);
  cudaFree(c->amstage);
  cudaFree(c->grf_amp);
  if (c->err_h) cudaFreeHost(c->err_h);
  for (auto& e : c->ev)
    if (e) cudaEventDestroy(e);
  for (int k = 0; k < 2; ++k) {
    cudaFree(c->m_delta[k]);
    cudaFree(c->m_z[k]);
    cudaFree(c->m_am[k]);
    if (c->m_copy[k]) cudaStreamDestroy(c->m_copy[k]);
    for (cudaEvent_t e : {c->m_in[k], c->m_read[k], c->m_done[k], c->m_out[k]})
      if (e) cudaEventDestroy(e);
  }
  for (auto& e : c->pev) cudaEventDestroy(e);
  c->pev.clear();
}

// main-array segment of a column pass along x (rows ix) or y (rows iy)
TileSeg mseg(const prc_d2z_ctx* c, const float2* in, float2* out, bool xpass) {
  TileSeg s;
  s.in = in;
  s.out = out;
  s.row_stride = xpass ? c->N * c->H : c->H;
  s.outer_stride = xpass ? c->H : c->N * c->H;
  s.n_outer = c->N;
  s.tpo = c->H / c->ksl.tile_w;
  s.transpose = 0;
  s.nyq = 0;
  return s;
}

// Nyquist-plane segment: rows at stride N, columns contiguous; optionally
// written transposed
TileSeg qseg(const prc_d2z_ctx* c, const float2* in, float2* out, bool transpose) {
  TileSeg s;
  s.in = in;
  s.out = out;
  s.row_stride = c->N;
  s.outer_stride = 0;
  s.n_outer = 1;
  s.tpo = c->N / c->ksl.tile_w;
  s.transpose = transpose ? 1 : 0;
  s.nyq = 1;
  return s;
}

// one column pass over the main array and the Nyquist plane
void run_tile(prc_d2z_ctx* c, int mode, TileSeg s0, TileSeg s1, int gy, int nb = 1, int r0 = 0, int first = 0) {
  TileArgs a;
  memset(&a, 0, sizeof(a));
  const bool faithful = mode == TM_WIN && (c->flags & PRC_FLAG_FAITHFUL_WINDOW);
  const int wv = faithful ? 0 : c->win_var;  // the faithful window runs on variant 0's tiles
  if (mode == TM_WIN || mode == TM_ACC) {  // these passes may use narrower tiles
    const int tw = mode == TM_WIN ? c->ksl.tile_w_winv[wv] : c->ksl.tile_w_acc;
    s0.tpo = (s0.nyq ? c->N : c->H) / tw;
    s1.tpo = (s1.nyq ? c->N : c->H) / tw;
  }
  a.seg[0] = s0;
  a.seg[1] = s1;
  a.slot_stride = c->slot_f2;
  a.tw = c->tw;
  a.nb = nb;
  a.first = first;
  a.win_var = wv;
  if (faithful) {
    // delta2zreion_d2z.C:41,43: dk = 2.*M_PI/BoxSize and kmax = dk*N in float;
    // the window then takes the float radius itself
    a.faithful = 1;
    a.dk = (float)(2.0 * M_PI / (double)(float)c->box);
    a.kmax = a.dk * (float)c->N;
    for (int b = 0; b < nb; ++b) a.kr[b] = (float)c->R[r0 + b];
  } else if (mode == TM_WIN || mode == TM_ACC) {
    for (int b = 0; b < nb; ++b) a.kr[b] = c->kr[r0 + b];
  }
  const int tiles = s0.n_outer * s0.tpo + s1.n_outer * s1.tpo;
  const int occ = (mode == TM_ACC) ? c->ksl.occ_tile_acc
                : faithful         ? c->ksl.occ_win_faithful
                : (mode == TM_WIN) ? c->ksl.occ_winv[wv] : c->ksl.occ_tile;
  dim3 grid(grid_for(tiles, 1, occ, c->sms), gy, 1);
  if (mode == TM_WIN && c->N <= 128) {
    // fewer tiles than two waves of resident CTAs: the sweep's radii are
    // split over blockIdx.y as well (the kernels of grids up to 128 read
    // their radius range from it)
    const long long want = 2LL * occ * c->sms;
    if (tiles < want) grid.y = (unsigned)std::min<long long>(nb, (want + tiles - 1) / tiles);
  }
  const int kind = mode == TM_FWD ? PRC_KIND_COL_FWD
                 : mode == TM_INV ? PRC_KIND_COL_INV
                 : mode == TM_WIN ? PRC_KIND_WIN_X : PRC_KIND_ADJ_X;
  {
    Prof pf(c, kind);
    c->ks->tile(c->ksl, mode, grid, c->st, a);
  }
  c->launches++;
}

int check_ctx(prc_d2z_ctx* c) {
  if (!c || !c->ks) return prc_fail(PRC_ERR_INVALID, "null or destroyed context");
  return PRC_OK;
}

int set_device(prc_d2z_ctx* c) {
  int cur = -1;
  PRC_CU(cudaGetDevice(&cur), "cudaGetDevice");
  if (cur != c->dev) PRC_CU(cudaSetDevice(c->dev), "cudaSetDevice");
  return PRC_OK;
}

// R2C of delta_lin / divisor (device) into c->spec.
void forward_r2c(prc_d2z_ctx* c, const float* d_delta, double divisor) {
  const int N = c->N, H = c->H;
  const long long NN = c->NN;
  float2* S = c->spec;
  float2* Q = c->spec + NN * H;
  float2* Qt = c->spec + NN * (H + 1);  // scratch after the Nyquist plane
  {
    Prof pf(c, PRC_KIND_R2C_Z);
    c->ks->r2c_z(c->ksl, grid_for(N * N, c->ksl.line_groups, c->ksl.occ_r2c, c->sms), c->st, d_delta,
                 (float)divisor, S, Qt, c->tw);
  }
  c->launches++;
  // y pass: main in place; Nyquist Qt[iy][ix] -> Q[ix][ky]
  run_tile(c, TM_FWD, mseg(c, S, S, false), qseg(c, Qt, Q, true), 1);
  // x pass: main in place; Nyquist Q in place
  run_tile(c, TM_FWD, mseg(c, S, S, true), qseg(c, Q, Q, false), 1);
}

// All radius sweeps of a forward call, kernels only (no copies, events or
// synchronisation), so that the same sequence can be captured into a graph.
// The running max lives in d_z / d_am; the last sweep writes the final values
// to z_out / am_out (default: d_z / d_am), which may be mapped host memory.
void enqueue_sweeps(prc_d2z_ctx* c, float* d_z, uint8_t* d_am, double* sig, float* z_out = nullptr,
                    uint8_t* am_out = nullptr, bool withhold = false) {
  const int N = c->N, H = c->H;
  const long long NN = c->NN;
  for (int r0 = 0; r0 < c->nr; r0 += c->B) {
    const int nb = (c->nr - r0 < c->B) ? c->nr - r0 : c->B;
    SweepArgs sa;
    memset(&sa, 0, sizeof(sa));
    sa.slots = c->slots;
    sa.slot_stride = c->slot_f2;
    sa.tw = c->tw;
    const bool last = (r0 + nb >= c->nr);
    sa.zreion = d_z;
    sa.argmax = d_am;
    sa.zreion_out = (last && z_out) ? z_out : d_z;
    sa.argmax_out = d_am ? ((last && am_out) ? am_out : d_am) : nullptr;
    sa.sig_acc = sig;
    sa.err = c->err;
    sa.withhold = (withhold && r0 == 0) ? 1 : 0;
    sa.nb = nb;
    sa.r0 = r0;
    sa.first = (r0 == 0);
    sa.as = c->as;
    for (int b = 0; b < nb; ++b) sa.cb[b] = c->cb[r0 + b];
    float2* U = c->slots;
    // window + inverse x pass: spectrum -> slots (Nyquist plane transposed)
    run_tile(c, TM_WIN, mseg(c, c->spec, U, true), qseg(c, c->spec + NN * H, U + NN * H, true), 1, nb, r0);
    // inverse y pass of every slot, in place
    run_tile(c, TM_INV, mseg(c, U, U, false), qseg(c, U + NN * H, U + NN * H, false), nb);
    {
      Prof pf(c, PRC_KIND_C2R_Z);
      c->ks->c2r_z(c->ksl, grid_for(N * N, c->ksl.c2r_lines, c->ksl.occ_c2r, c->sms), c->st, sa);
    }
    c->launches++;
  }
}

}  // namespace

// ------------------------------------------------------------ batches
// Many boxes of (possibly) different sizes: one context per box, boxes spread
// round-robin over a few streams, optionally all captured into one CUDA graph
// and replayed with a single launch.
// Grouped launches (PRC_BATCH_GROUPED): the boxes of one grid size form a
// group, and every pass of the step runs as one launch over all boxes of the
// group -- persistent CTAs (a grid of resident CTAs) walking the list of
// (box, tile) or (box, line group) items of that pass -- instead of one launch
// per box.  Each group has its own stream; the groups run side by side.  The
// per-box pointers and constants sit in device tables, rewritten before each
// forward (they carry the caller's input and output pointers), so the
// captured graph of a grouped batch never needs capturing again.  The groups
// share out the batch's n_streams streams, largest grid size first.
struct BatchGroup {
  int N = 0, nsweeps = 0;
  std::vector<int> boxes;        // batch indices
  cudaStream_t st = nullptr;    // one of the batch's streams (groups round-robin, largest first)
  // table offsets (bytes) in the batch's table buffer
  size_t o_r2c = 0, o_fy = 0, o_fx = 0;
  std::vector<size_t> o_win, o_inv, o_line;
  // sweep s: the boxes that have one (each box sweeps its own radius batch),
  // most radii in that sweep first, and their radii in it
  std::vector<std::vector<int>> sw_box, sw_nb;
};

struct prc_d2z_batch {
  int n = 0, dev = 0;
  std::vector<prc_d2z_ctx*> ctx;
  std::vector<cudaStream_t> streams;
  cudaStream_t origin = nullptr;
  std::vector<cudaEvent_t> ev;  // fork + one join per stream
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  std::vector<const void*> key;  // pointers the graph was captured with
  int exec_mode = -1;            // batch mode the graph was captured in
  // grouped launches
  std::vector<BatchGroup> groups;
  std::vector<cudaEvent_t> gev;  // one join event per group
  char* h_tab = nullptr;         // host image of the tables (pinned: the copy is asynchronous)
  size_t tab_bytes = 0;
  char* d_tab = nullptr;
  int launches = 0;              // launches of the last grouped forward
};

namespace {

void batch_free(prc_d2z_batch* b) {
  if (b->exec) cudaGraphExecDestroy(b->exec);
  if (b->graph) cudaGraphDestroy(b->graph);
  for (auto e : b->gev) cudaEventDestroy(e);
  cudaFree(b->d_tab);
  if (b->h_tab) cudaFreeHost(b->h_tab);
  for (auto* c : b->ctx) prc_d2z_destroy(c);
  for (auto e : b->ev) cudaEventDestroy(e);
  for (auto s : b->streams) cudaStreamDestroy(s);
  if (b->origin) cudaStreamDestroy(b->origin);
}

void batch_enqueue(prc_d2z_batch* b, const float* const* delta, float* const* zreion, uint8_t* const* argmax) {
  cudaEventRecord(b->ev[0], b->origin);
  for (auto s : b->streams) cudaStreamWaitEvent(s, b->ev[0], 0);
  for (int i = 0; i < b->n; ++i) {
    prc_d2z_ctx* c = b->ctx[i];
    c->launches = 0;
    forward_r2c(c, delta[i], c->dinit);
    enqueue_sweeps(c, zreion[i], argmax ? argmax[i] : nullptr, nullptr);
  }
  for (size_t k = 0; k < b->streams.size(); ++k) {
    cudaEventRecord(b->ev[1 + k], b->streams[k]);
    cudaStreamWaitEvent(b->origin, b->ev[1 + k], 0);
  }
}

size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }

// A box joins a grouped launch when its size has grouped kernels and it asks
// for nothing they leave out (the faithful window runs per box).
bool groupable(const prc_d2z_ctx* c) { return c->ksl.grouped && !(c->flags & PRC_FLAG_FAITHFUL_WINDOW); }

// Groups of equal grid size, their sweeps and the layout of their tables.
// Sizes without grouped kernels keep per-box launches (no group).
int batch_group_setup(prc_d2z_batch* b) {
  for (auto e : b->gev) cudaEventDestroy(e);
  b->groups.clear();
  b->gev.clear();
  cudaFree(b->d_tab);
  b->d_tab = nullptr;
  if (b->h_tab) cudaFreeHost(b->h_tab);
  b->h_tab = nullptr;
  b->tab_bytes = 0;
  std::vector<int> sizes;
  for (auto* c : b->ctx)
    if (groupable(c) && std::find(sizes.begin(), sizes.end(), c->N) == sizes.end()) sizes.push_back(c->N);
  std::sort(sizes.begin(), sizes.end(), [](int x, int y) { return x > y; });
  size_t off = 0;
  for (int N : sizes) {
    BatchGroup g;
    g.N = N;
    for (int i = 0; i < b->n; ++i)
      if (b->ctx[i]->N == N && groupable(b->ctx[i])) {
        g.boxes.push_back(i);
        const prc_d2z_ctx* c = b->ctx[i];
        g.nsweeps = std::max(g.nsweeps, (c->nr + c->B - 1) / c->B);
      }
    for (int sw = 0; sw < g.nsweeps; ++sw) {
      std::vector<int> bx;
      for (int i : g.boxes)
        if (b->ctx[i]->nr > sw * b->ctx[i]->B) bx.push_back(i);
      auto nb_of = [&](int i) { return std::min(b->ctx[i]->B, b->ctx[i]->nr - sw * b->ctx[i]->B); };
      // most radii first: the boxes with more than y radii in the sweep are a
      // prefix, which the inverse y pass's slot y takes
      std::stable_sort(bx.begin(), bx.end(), [&](int x, int y) { return nb_of(x) > nb_of(y); });
      std::vector<int> nbs;
      for (int i : bx) nbs.push_back(nb_of(i));
      g.sw_box.push_back(bx);
      g.sw_nb.push_back(nbs);
    }
    const size_t nb = g.boxes.size();
    g.o_r2c = off;
    off = align256(off + nb * sizeof(BoxR2c));
    g.o_fy = off;
    off = align256(off + nb * sizeof(BoxCol));
    g.o_fx = off;
    off = align256(off + nb * sizeof(BoxCol));
    for (int sw = 0; sw < g.nsweeps; ++sw) {
      const size_t k = g.sw_box[sw].size();
      g.o_win.push_back(off);
      off = align256(off + k * sizeof(BoxCol));
      g.o_inv.push_back(off);
      off = align256(off + k * sizeof(BoxCol));
      g.o_line.push_back(off);
      off = align256(off + k * sizeof(BoxLine));
    }
    b->groups.push_back(g);
  }
  if (off) {
    int st;
    if ((st = dalloc(&b->d_tab, off, "batch tables")) != PRC_OK) return st;
    PRC_CU(cudaMallocHost((void**)&b->h_tab, off), "batch tables (host)");
    memset(b->h_tab, 0, off);
    b->tab_bytes = off;
  }
  for (size_t gi = 0; gi < b->groups.size(); ++gi) {
    b->groups[gi].st = b->streams[gi % b->streams.size()];
    cudaEvent_t e;
    PRC_CU(cudaEventCreateWithFlags(&e, cudaEventDisableTiming), "group event");
    b->gev.push_back(e);
  }
  return PRC_OK;
}

// Host image of every group's tables for these inputs and outputs.
void batch_group_fill(prc_d2z_batch* b, const float* const* delta, float* const* zreion, uint8_t* const* argmax) {
  char* h = b->h_tab;
  for (const auto& g : b->groups) {
    for (size_t k = 0; k < g.boxes.size(); ++k) {
      const int i = g.boxes[k];
      const prc_d2z_ctx* c = b->ctx[i];
      const long long NN = c->NN, H = c->H;
      float2* S = c->spec;
      BoxR2c r;
      r.delta = delta[i];
      r.S = S;
      r.Qt = S + NN * (H + 1);
      r.dinit = (float)c->dinit;
      memcpy(h + g.o_r2c + k * sizeof(BoxR2c), &r, sizeof r);
      BoxCol fy, fx;
      memset(&fy, 0, sizeof fy);
      memset(&fx, 0, sizeof fx);
      // y pass: main in place, Nyquist Qt -> Q (transposed); x pass: both in place
      fy.in0 = S, fy.out0 = S, fy.in1 = S + NN * (H + 1), fy.out1 = S + NN * H;
      fx.in0 = S, fx.out0 = S, fx.in1 = S + NN * H, fx.out1 = S + NN * H;
      memcpy(h + g.o_fy + k * sizeof(BoxCol), &fy, sizeof fy);
      memcpy(h + g.o_fx + k * sizeof(BoxCol), &fx, sizeof fx);
    }
    for (int sw = 0; sw < g.nsweeps; ++sw) {
      for (size_t k = 0; k < g.sw_box[sw].size(); ++k) {
        const int i = g.sw_box[sw][k];
        const prc_d2z_ctx* c = b->ctx[i];
        const long long NN = c->NN, H = c->H;
        const int r0 = sw * c->B, nb = g.sw_nb[sw][k];
        float2* U = c->slots;
        BoxCol w, v;
        memset(&w, 0, sizeof w);
        memset(&v, 0, sizeof v);
        w.in0 = c->spec, w.out0 = U, w.in1 = c->spec + NN * H, w.out1 = U + NN * H, w.nb = nb;
        for (int q = 0; q < nb; ++q) w.kr[q] = c->kr[r0 + q];
        v.in0 = U, v.out0 = U, v.in1 = U + NN * H, v.out1 = U + NN * H, v.nb = nb;
        memcpy(h + g.o_win[sw] + k * sizeof(BoxCol), &w, sizeof w);
        memcpy(h + g.o_inv[sw] + k * sizeof(BoxCol), &v, sizeof v);
        BoxLine L;
        memset(&L, 0, sizeof L);
        L.slots = U;
        L.zreion = L.zreion_out = zreion[i];
        L.argmax = L.argmax_out = argmax ? argmax[i] : nullptr;
        L.nb = nb, L.r0 = r0, L.first = (sw == 0), L.as = c->as;
        for (int q = 0; q < nb; ++q) L.cb[q] = c->cb[r0 + q];
        memcpy(h + g.o_line[sw] + k * sizeof(BoxLine), &L, sizeof L);
      }
    }
  }
}

// Every pass of every group as one launch over the group's boxes, groups on
// their own streams; boxes of sizes without grouped kernels as per-box
// launches on the batch's streams.  Kernels only (capturable).
void batch_enqueue_grouped(prc_d2z_batch* b, const float* const* delta, float* const* zreion,
                           uint8_t* const* argmax) {
  cudaEventRecord(b->ev[0], b->origin);
  for (auto s : b->streams) cudaStreamWaitEvent(s, b->ev[0], 0);
  int launches = 0;
  for (size_t gi = 0; gi < b->groups.size(); ++gi) {
    const BatchGroup& g = b->groups[gi];
    const prc_d2z_ctx* c0 = b->ctx[g.boxes[0]];
    const KernelSet& ks = c0->ksl;
    const int N = g.N, H = N / 2, sms = c0->sms, nbox = (int)g.boxes.size();
    const long long NN = c0->NN;
    float2* S0 = c0->spec;
    float2* U0 = c0->slots;
    ks.r2c_z_mb(ks, grid_for(N * N * nbox, ks.line_groups, ks.occ_mb_r2c, sms), g.st,
                reinterpret_cast<const BoxR2c*>(b->d_tab + g.o_r2c), nbox, c0->tw);
    auto cols = [&](int mode, TileSeg s0, TileSeg s1, size_t o, int nboxes, int gy, const int* nvb) {
      TileArgs a;
      memset(&a, 0, sizeof(a));
      if (mode == TM_WIN) {
        s0.tpo = H / ks.tile_w_mb_win;
        s1.tpo = N / ks.tile_w_mb_win;
      }
      a.seg[0] = s0;
      a.seg[1] = s1;
      a.slot_stride = c0->slot_f2;
      a.tw = c0->tw;
      a.box = reinterpret_cast<const BoxCol*>(b->d_tab + o);
      a.nbox = nboxes;
      if (nvb)
        for (int y = 0; y < gy; ++y) a.nvb[y] = nvb[y];
      const int tpb = s0.n_outer * s0.tpo + s1.n_outer * s1.tpo;
      const int occ = mode == TM_WIN ? ks.occ_mb_win : ks.occ_mb_tile;
      ks.tile_mb(ks, mode, dim3(grid_for(tpb * (nvb ? nvb[0] : nboxes), 1, occ, sms), gy, 1), g.st, a);
      ++launches;
    };
    cols(TM_FWD, mseg(c0, S0, S0, false), qseg(c0, S0 + NN * (H + 1), S0 + NN * H, true), g.o_fy, nbox, 1, nullptr);
    cols(TM_FWD, mseg(c0, S0, S0, true), qseg(c0, S0 + NN * H, S0 + NN * H, false), g.o_fx, nbox, 1, nullptr);
    for (int sw = 0; sw < g.nsweeps; ++sw) {
      const int ns = (int)g.sw_box[sw].size();
      const std::vector<int>& nbs = g.sw_nb[sw];
      cols(TM_WIN, mseg(c0, S0, U0, true), qseg(c0, S0 + NN * H, U0 + NN * H, true), g.o_win[sw], ns, 1, nullptr);
      int nvb[kMaxBatch];
      for (int y = 0; y < nbs[0]; ++y) {
        int k = 0;
        while (k < ns && nbs[k] > y) ++k;
        nvb[y] = k;
      }
      cols(TM_INV, mseg(c0, U0, U0, false), qseg(c0, U0 + NN * H, U0 + NN * H, false), g.o_inv[sw], ns, nbs[0],
           nvb);
      SweepArgs sa;
      memset(&sa, 0, sizeof(sa));
      sa.slot_stride = c0->slot_f2;
      sa.tw = c0->tw;
      sa.err = c0->err;
      sa.argmax = argmax ? argmax[g.sw_box[sw][0]] : nullptr;
      sa.box = reinterpret_cast<const BoxLine*>(b->d_tab + g.o_line[sw]);
      sa.nbox = ns;
      ks.c2r_z_mb(ks, grid_for(N * N * ns, ks.c2r_lines, ks.occ_mb_c2r, sms), g.st, sa);
      launches += 2;
    }
    launches += 1;
    cudaEventRecord(b->gev[gi], g.st);
    cudaStreamWaitEvent(b->origin, b->gev[gi], 0);
  }
  // sizes without grouped kernels: per-box launches
  for (int i = 0; i < b->n; ++i) {
    prc_d2z_ctx* c = b->ctx[i];
    if (groupable(c)) continue;
    c->launches = 0;
    forward_r2c(c, delta[i], c->dinit);
    enqueue_sweeps(c, zreion[i], argmax ? argmax[i] : nullptr, nullptr);
    launches += c->launches;
  }
  for (size_t k = 0; k < b->streams.size(); ++k) {
    cudaEventRecord(b->ev[1 + k], b->streams[k]);
    cudaStreamWaitEvent(b->origin, b->ev[1 + k], 0);
  }
  b->launches = launches;
}

}  // namespace

extern "C" {

int prc_d2z_supported(int N) { return kernel_set(N) != nullptr ? 1 : 0; }

int prc_d2z_test_withhold_copy(int calls) {
  if (calls < 0) return prc_fail(PRC_ERR_INVALID, "prc_d2z_test_withhold_copy: calls must be >= 0");
  g_withhold.store(calls);
  return PRC_OK;
}

int prc_d2z_create(const prc_d2z_desc* d, prc_d2z_ctx** out) {
  if (!d || !out) return prc_fail(PRC_ERR_INVALID, "prc_d2z_create: null argument");
  *out = nullptr;
  const KernelSet* ks = kernel_set(d->N);
  if (!ks) return prc_fail(PRC_ERR_UNSUPPORTED, "prc_d2z_create: no FFT plan for N=%d", d->N);
  if (d->n_radii < 1 || d->n_radii > PRC_MAX_RADII)
    return prc_fail(PRC_ERR_INVALID, "prc_d2z_create: n_radii=%d outside 1..%d", d->n_radii, PRC_MAX_RADII);
  if (!d->radii_mpc || !d->barrier_b) return prc_fail(PRC_ERR_INVALID, "prc_d2z_create: null radius table");
  if (!(d->box_mpc > 0)) return prc_fail(PRC_ERR_INVALID, "prc_d2z_create: box_mpc must be > 0");
  if (!(d->growth_init > 0)) return prc_fail(PRC_ERR_INVALID, "prc_d2z_create: growth factor must be > 0");
  if (!(d->barrier_a > 0)) return prc_fail(PRC_ERR_INVALID, "prc_d2z_create: barrier_a must be > 0");
  for (int r = 0; r < d->n_radii; ++r)
    if (!(d->radii_mpc[r] > 0)) return prc_fail(PRC_ERR_INVALID, "prc_d2z_create: radius %d not > 0", r);
  if (d->radius_batch < 0 || d->radius_batch > kMaxBatch)
    return prc_fail(PRC_ERR_INVALID, "prc_d2z_create: radius_batch must be 0..%d", kMaxBatch);

  prc_d2z_ctx* c = new prc_d2z_ctx();
  c->N = d->N;
  c->H = d->N / 2;
  c->nr = d->n_radii;
  c->flags = d->flags;
  c->NN = (long long)d->N * d->N;
  c->slot_f2 = c->NN * (c->H + 2);
  c->box = d->box_mpc;
  c->A = d->barrier_a;
  c->dinit = d->growth_init;
  c->st = (cudaStream_t)d->stream;
  c->ks = ks;
  c->ksl = *ks;
  // default radii per sweep: 16 (measured fastest up to 512^3: fewer re-reads
  // of the spectrum and of zreion), 8 at 1024^3 where one slot is 4.3 GB
  int B = d->radius_batch ? d->radius_batch : (d->N >= 1024 ? 8 : 16);
  if (B > c->nr) B = c->nr;
  c->B = B;
  c->slots_b = B;
  const double dk = 2.0 * M_PI / d->box_mpc;
  const double n3 = (double)d->N * d->N * d->N;
  c->as = (float)(d->barrier_a / n3);
  for (int r = 0; r < c->nr; ++r) {
    c->R.push_back(d->radii_mpc[r]);
    c->Bb.push_back(d->barrier_b[r]);
    c->kr.push_back((float)(dk * d->radii_mpc[r]));
    c->cb.push_back((float)(d->barrier_a * d->barrier_b[r] - 1.0));
  }
  int st;
  cudaError_t e = cudaGetDevice(&c->dev);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&c->sms, cudaDevAttrMultiProcessorCount, c->dev);
  if (e == cudaSuccess) e = ks->init(&c->ksl);
  if (e != cudaSuccess) {
    delete c;
    return cuda_fail(e, "prc_d2z_create: device set-up");
  }
  const long long n3l = (long long)c->NN * c->N;
  if ((st = dalloc(&c->spec, (size_t)c->slot_f2, "spectrum")) != PRC_OK ||
      (st = dalloc(&c->slots, (size_t)c->slot_f2 * c->B, "radius slots")) != PRC_OK ||
      (st = dalloc(&c->tw, (size_t)c->N, "twiddles")) != PRC_OK ||
      (st = dalloc(&c->sig, (size_t)c->nr, "sigma accumulators")) != PRC_OK ||
      (st = dalloc(&c->dB, (size_t)c->nr, "barrier gradient")) != PRC_OK ||
      (st = dalloc(&c->counts, (size_t)kNHistory, "history counts")) != PRC_OK) {
    free_all(c);
    delete c;
    return st;
  }
  if ((e = cudaHostAlloc((void**)&c->err_h, sizeof(int), cudaHostAllocMapped)) != cudaSuccess ||
      (e = cudaHostGetDevicePointer((void**)&c->err, c->err_h, 0)) != cudaSuccess) {
    free_all(c);
    delete c;
    return cuda_fail(e, "prc_d2z_create: error flag");
  }
  *c->err_h = 0;
  (void)n3l;
  // twiddles e^{+2 pi i k/N}, FP64 on the host
  std::vector<float2> tw(c->N);
  for (int k = 0; k < c->N; ++k) {
    const double ang = 2.0 * M_PI * (double)k / (double)c->N;
    tw[k] = make_float2((float)cos(ang), (float)sin(ang));
  }
  e = cudaMemcpy(c->tw, tw.data(), sizeof(float2) * c->N, cudaMemcpyHostToDevice);
  for (int i = 0; i < 4 && e == cudaSuccess; ++i) e = cudaEventCreate(&c->ev[i]);
  if (e != cudaSuccess) {
    free_all(c);
    delete c;
    return cuda_fail(e, "prc_d2z_create: upload");
  }
  *out = c;
  return PRC_OK;
}

namespace {
// Reads and clears the context's kernel error flag (after a synchronisation).
// After the stream synchronisation: the kernels' writes to the mapped word are
// complete and visible to the host.
int check_kernel_flag(prc_d2z_ctx* c, const char* who) {
  volatile int* h = c->err_h;
  if (*h) {
    *h = 0;
    return prc_fail(PRC_ERR_CUDA, "%s: a staging copy did not complete within the wait limit", who);
  }
  return PRC_OK;
}

// One cudaMemcpyAsync per piece of at most 256 MiB (a single 4 GiB host to
// device copy from pinned memory was measured at 28 GB/s, its 512 MiB pieces
// at the link's 207 GB/s).
cudaError_t copy_chunked(void* dst, const void* src, size_t bytes, cudaMemcpyKind kind, cudaStream_t s) {
  constexpr size_t kPiece = size_t(256) << 20;
  for (size_t off = 0; off < bytes; off += kPiece) {
    const size_t nb = (bytes - off < kPiece) ? bytes - off : kPiece;
    const cudaError_t e = cudaMemcpyAsync(static_cast<char*>(dst) + off, static_cast<const char*>(src) + off, nb,
                                          kind, s);
    if (e != cudaSuccess) return e;
  }
  return cudaSuccess;
}

// Device address of a host buffer the GPU reads and writes in place (pinned
// and mapped into the device's address space), or null (then it is staged).
void* mapped_view(const void* host) {
  cudaPointerAttributes at;
  if (cudaPointerGetAttributes(&at, host) != cudaSuccess) {
    cudaGetLastError();
    return nullptr;
  }
  return (at.type == cudaMemoryTypeHost) ? at.devicePointer : nullptr;
}
}  // namespace

int prc_d2z_forward(prc_d2z_ctx* c, const float* delta_lin, int delta_on_device, float* zreion,
                    uint8_t* argmax, int out_on_device, double* sigma_grid) {
  int st;
  if ((st = check_ctx(c)) != PRC_OK) return st;
  if (!delta_lin || !zreion) return prc_fail(PRC_ERR_INVALID, "prc_d2z_forward: null delta or zreion");
  if ((st = set_device(c)) != PRC_OK) return st;
  const int N = c->N, H = c->H;
  const long long NN = c->NN, n3 = NN * N;
  c->launches = 0;
  c->have_timing = 0;
  // device buffers
  // host buffers: a pinned, mapped one is read (delta) or written (the last
  // sweep's zreion / argmax) in place over the host link; others are staged
  const float* d_delta = delta_lin;
  if (!delta_on_device) {
    if (const void* v = mapped_view(delta_lin)) {
      d_delta = static_cast<const float*>(v);
    } else {
      float* stage = reinterpret_cast<float*>(c->slots);  // slot 0 main region holds N^3 floats
      PRC_CU(cudaMemcpyAsync(stage, delta_lin, sizeof(float) * n3, cudaMemcpyHostToDevice, c->st), "H2D delta");
      d_delta = stage;
    }
  }
  float* z_final = nullptr;     // mapped host output of the last sweep
  uint8_t* am_final = nullptr;
  if (!out_on_device) {
    void* zv = mapped_view(zreion);
    void* av = argmax ? mapped_view(argmax) : nullptr;
    if (zv && (!argmax || av)) {
      z_final = static_cast<float*>(zv);
      am_final = static_cast<uint8_t*>(av);
    }
  }
  float* d_z = zreion;
  uint8_t* d_am = argmax;
  const bool want_am = argmax != nullptr || (c->flags & PRC_FLAG_ARGMAX);
  if (!out_on_device || (want_am && !argmax)) {
    if (!out_on_device && !c->zre && (st = dalloc(&c->zre, (size_t)n3, "zreion")) != PRC_OK) return st;
    if (want_am && !c->am && (st = dalloc(&c->am, (size_t)n3, "argmax")) != PRC_OK) return st;
    if (!out_on_device) d_z = c->zre;
    if (want_am && (!out_on_device || !argmax)) d_am = c->am;
  }
  if (!want_am) d_am = nullptr;
  const bool want_sig = sigma_grid != nullptr || (c->flags & PRC_FLAG_SIGMA_GRID);
  if (want_sig) PRC_CU(cudaMemsetAsync(c->sig, 0, sizeof(double) * c->nr, c->st), "memset sigma");

  PRC_CU(cudaEventRecord(c->ev[0], c->st), "event");
  forward_r2c(c, d_delta, c->dinit);
  PRC_CU(cudaEventRecord(c->ev[1], c->st), "event");
  enqueue_sweeps(c, d_z, d_am, want_sig ? c->sig : nullptr, z_final, am_final, take_withhold());
  PRC_CU(cudaGetLastError(), "kernel launch");
  PRC_CU(cudaEventRecord(c->ev[2], c->st), "event");
  if (!out_on_device) {
    if (!z_final) {
      PRC_CU(cudaMemcpyAsync(zreion, d_z, sizeof(float) * n3, cudaMemcpyDeviceToHost, c->st), "D2H zreion");
      if (argmax) PRC_CU(cudaMemcpyAsync(argmax, d_am, n3, cudaMemcpyDeviceToHost, c->st), "D2H argmax");
    }
  } else if (argmax && d_am != argmax) {
    PRC_CU(cudaMemcpyAsync(argmax, d_am, n3, cudaMemcpyDeviceToDevice, c->st), "D2D argmax");
  }
  std::vector<double> sig;
  if (sigma_grid) {
    sig.resize(c->nr);
    PRC_CU(cudaMemcpyAsync(sig.data(), c->sig, sizeof(double) * c->nr, cudaMemcpyDeviceToHost, c->st), "D2H sigma");
  }
  PRC_CU(cudaStreamSynchronize(c->st), "prc_d2z_forward");
  if ((st = check_kernel_flag(c, "prc_d2z_forward")) != PRC_OK) return st;
  prof_collect(c);
  float t0, t1;
  PRC_CU(cudaEventElapsedTime(&t0, c->ev[0], c->ev[1]), "event time");
  PRC_CU(cudaEventElapsedTime(&t1, c->ev[1], c->ev[2]), "event time");
  c->last_ms[0] = t0;
  c->last_ms[1] = t1;
  c->last_ms[2] = t0 + t1;
  c->have_timing = 1;
  if (sigma_grid) {
    // GetMeanSigma (arrayoperations.C:4-35): sqrt(<delta_R^2>), delta_R = x / N^3
    const double n3d = (double)n3;
    for (int r = 0; r < c->nr; ++r) sigma_grid[r] = sqrt(sig[r] / (n3d * n3d * n3d));
  }
  return PRC_OK;
}

// Many boxes of this context's shape from host buffers, pipelined over two
// device copies of the input and outputs: box i's kernels run on the
// context's stream while box i+1's delta_lin is copied in on one copy stream
// and box i-1's zreion (argmax) copied out on the other.  Events order each
// buffer's reuse: box i+1's input copy waits for box i's R2C (hence for box
// i-1's, which used the same buffer), and box i+2's kernels wait for box i's
// output copy.  Pinned host buffers overlap;
// pageable ones are correct but serialise (their copies block the host).
int prc_d2z_forward_many(prc_d2z_ctx* c, int n, const float* const* delta, float* const* zreion,
                         uint8_t* const* argmax) {
  int st;
  if ((st = check_ctx(c)) != PRC_OK) return st;
  if (n < 0 || (n > 0 && (!delta || !zreion)))
    return prc_fail(PRC_ERR_INVALID, "prc_d2z_forward_many: bad box count or null pointer array");
  for (int i = 0; i < n; ++i)
    if (!delta[i] || !zreion[i] || (argmax && !argmax[i]))
      return prc_fail(PRC_ERR_INVALID, "prc_d2z_forward_many: null pointer for box %d", i);
  if (n == 0) return PRC_OK;
  if ((st = set_device(c)) != PRC_OK) return st;
  const long long n3 = c->NN * c->N;
  const bool want_am = argmax != nullptr;
  for (int k = 0; k < 2; ++k) {
    if (!c->m_delta[k] && (st = dalloc(&c->m_delta[k], (size_t)n3, "pipelined input")) != PRC_OK) return st;
    if (!c->m_z[k] && (st = dalloc(&c->m_z[k], (size_t)n3, "pipelined zreion")) != PRC_OK) return st;
    if (want_am && !c->m_am[k] && (st = dalloc(&c->m_am[k], (size_t)n3, "pipelined argmax")) != PRC_OK)
      return st;
    if (!c->m_copy[k]) PRC_CU(cudaStreamCreateWithFlags(&c->m_copy[k], cudaStreamNonBlocking), "copy stream");
    for (cudaEvent_t* e : {&c->m_in[k], &c->m_read[k], &c->m_done[k], &c->m_out[k]})
      if (!*e) PRC_CU(cudaEventCreateWithFlags(e, cudaEventDisableTiming), "pipeline event");
  }
  cudaStream_t cin = c->m_copy[0], cout = c->m_copy[1];
  c->launches = 0;
  c->have_timing = 0;
  // everything is queued by enqueue(); whatever it returns, the three streams
  // are drained before the call returns, so no copy touches a caller's buffer
  // afterwards
  auto enqueue = [&]() -> int {
    // the first input copies may not overtake work already queued on the stream
    PRC_CU(cudaEventRecord(c->m_read[0], c->st), "event");
    PRC_CU(cudaEventRecord(c->m_read[1], c->st), "event");
    PRC_CU(cudaEventRecord(c->m_out[0], c->st), "event");
    PRC_CU(cudaEventRecord(c->m_out[1], c->st), "event");
    for (int i = 0; i < n; ++i) {
      const int k = i & 1;
      // the first box has nothing to overlap its input copy with: a mapped
      // input is read in place by its R2C instead; likewise the last box's
      // final sweep writes mapped outputs in place
      const float* d_in = (i == 0) ? static_cast<const float*>(mapped_view(delta[0])) : nullptr;
      float* z_fin = nullptr;
      uint8_t* am_fin = nullptr;
      // (not when the previous box copies into the same buffer: that copy is
      // ordered on the output stream only)
      const bool reused = i > 0 && (zreion[i] == zreion[i - 1] || (want_am && argmax[i] == argmax[i - 1]));
      if (i == n - 1 && !reused) {
        z_fin = static_cast<float*>(mapped_view(zreion[i]));
        am_fin = want_am ? static_cast<uint8_t*>(mapped_view(argmax[i])) : nullptr;
        if (want_am && !am_fin) z_fin = nullptr;
      }
      if (!d_in) {
        // after the previous box's R2C: it may be reading its input over the
        // host link, and the box before it (same buffer) is past its R2C too
        PRC_CU(cudaStreamWaitEvent(cin, c->m_read[i == 0 ? k : (i - 1) & 1], 0), "wait");
        PRC_CU(copy_chunked(c->m_delta[k], delta[i], sizeof(float) * n3, cudaMemcpyHostToDevice, cin), "H2D delta");
        PRC_CU(cudaEventRecord(c->m_in[k], cin), "event");
        PRC_CU(cudaStreamWaitEvent(c->st, c->m_in[k], 0), "wait");
        d_in = c->m_delta[k];
      }
      PRC_CU(cudaStreamWaitEvent(c->st, c->m_out[k], 0), "wait");
      forward_r2c(c, d_in, c->dinit);
      PRC_CU(cudaEventRecord(c->m_read[k], c->st), "event");
      enqueue_sweeps(c, c->m_z[k], want_am ? c->m_am[k] : nullptr, nullptr, z_fin, am_fin);
      PRC_CU(cudaGetLastError(), "kernel launch");
      PRC_CU(cudaEventRecord(c->m_done[k], c->st), "event");
      if (!z_fin) {
        PRC_CU(cudaStreamWaitEvent(cout, c->m_done[k], 0), "wait");
        PRC_CU(copy_chunked(zreion[i], c->m_z[k], sizeof(float) * n3, cudaMemcpyDeviceToHost, cout), "D2H zreion");
        if (want_am)
          PRC_CU(copy_chunked(argmax[i], c->m_am[k], (size_t)n3, cudaMemcpyDeviceToHost, cout), "D2H argmax");
        PRC_CU(cudaEventRecord(c->m_out[k], cout), "event");
      }
    }
    return PRC_OK;
  };
  st = enqueue();
  const cudaError_t e0 = cudaStreamSynchronize(cin), e1 = cudaStreamSynchronize(cout),
                    e2 = cudaStreamSynchronize(c->st);
  if (st != PRC_OK) return st;
  PRC_CU(e0 != cudaSuccess ? e0 : (e1 != cudaSuccess ? e1 : e2), "prc_d2z_forward_many");
  if ((st = check_kernel_flag(c, "prc_d2z_forward_many")) != PRC_OK) return st;
  prof_collect(c);
  return PRC_OK;
}

int prc_d2z_smooth(prc_d2z_ctx* c, const float* delta_lin, int delta_on_device, int radius, float* delta_r,
                   int out_on_device) {
  int st;
  if ((st = check_ctx(c)) != PRC_OK) return st;
  if (!delta_lin || !delta_r) return prc_fail(PRC_ERR_INVALID, "prc_d2z_smooth: null argument");
  if (radius < 0 || radius >= c->nr) return prc_fail(PRC_ERR_INVALID, "prc_d2z_smooth: radius %d out of range", radius);
  if ((st = set_device(c)) != PRC_OK) return st;
  const int N = c->N, H = c->H;
  const long long NN = c->NN, n3 = NN * N;
  c->launches = 0;
  const float* d_delta = delta_lin;
  if (!delta_on_device) {
    float* stage = reinterpret_cast<float*>(c->slots);
    PRC_CU(cudaMemcpyAsync(stage, delta_lin, sizeof(float) * n3, cudaMemcpyHostToDevice, c->st), "H2D delta");
    d_delta = stage;
  }
  float* d_out = delta_r;
  if (!out_on_device) {
    if (!c->zre && (st = dalloc(&c->zre, (size_t)n3, "output stage")) != PRC_OK) return st;
    d_out = c->zre;
  }
  forward_r2c(c, d_delta, c->dinit);
  float2* U = c->slots;
  run_tile(c, TM_WIN, mseg(c, c->spec, U, true), qseg(c, c->spec + NN * H, U + NN * H, true), 1, 1, radius);
  run_tile(c, TM_INV, mseg(c, U, U, false), qseg(c, U + NN * H, U + NN * H, false), 1);
  AdjArgs fa;
  memset(&fa, 0, sizeof(fa));
  fa.slots = U;
  fa.tw = c->tw;
  fa.out = d_out;
  fa.scale = (float)(1.0 / (double)n3);
  c->ks->c2r_plain(c->ksl, grid_for(N * N, c->ksl.line_groups, c->ksl.occ_c2r_plain, c->sms), c->st, fa);
  c->launches++;
  PRC_CU(cudaGetLastError(), "kernel launch");
  if (!out_on_device)
    PRC_CU(cudaMemcpyAsync(delta_r, d_out, sizeof(float) * n3, cudaMemcpyDeviceToHost, c->st), "D2H delta_R");
  PRC_CU(cudaStreamSynchronize(c->st), "prc_d2z_smooth");
  prof_collect(c);
  return PRC_OK;
}

int prc_white_noise(float* d_out, long long n, unsigned int seed, void* stream) {
  if (!d_out || n < 0) return prc_fail(PRC_ERR_INVALID, "prc_white_noise: null output or negative count");
  if (n == 0) return PRC_OK;
  int dev = 0, sms = 0;
  PRC_CU(cudaGetDevice(&dev), "cudaGetDevice");
  PRC_CU(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev), "device query");
  const long long need = (n + 255) / 256;
  const int blocks = (int)(need < (long long)sms * 16 ? need : (long long)sms * 16);
  k_white_noise<<<blocks, 256, 0, (cudaStream_t)stream>>>(d_out, n, (uint32_t)seed);
  PRC_CU(cudaGetLastError(), "k_white_noise launch");
  return PRC_OK;
}

int prc_d2z_gaussian_field(prc_d2z_ctx* c, unsigned int seed, const float* amp, int n_amp, float* delta,
                           int out_on_device) {
  int st;
  if ((st = check_ctx(c)) != PRC_OK) return st;
  if (!amp || !delta) return prc_fail(PRC_ERR_INVALID, "prc_d2z_gaussian_field: null argument");
  const int N = c->N, H = c->H;
  const int need = 3 * H * H + 1;
  if (n_amp < need)
    return prc_fail(PRC_ERR_INVALID, "prc_d2z_gaussian_field: amplitude table has %d entries, needs %d", n_amp, need);
  if ((st = set_device(c)) != PRC_OK) return st;
  const long long NN = c->NN, n3 = NN * N;
  c->launches = 0;
  if (!c->grf_amp && (st = dalloc(&c->grf_amp, (size_t)need, "amplitude table")) != PRC_OK) return st;
  PRC_CU(cudaMemcpyAsync(c->grf_amp, amp, sizeof(float) * need, cudaMemcpyHostToDevice, c->st), "H2D amplitudes");
  float* d_out = delta;
  if (!out_on_device) {
    if (!c->zre && (st = dalloc(&c->zre, (size_t)n3, "output stage")) != PRC_OK) return st;
    d_out = c->zre;
  }
  if ((st = prc_white_noise(d_out, n3, seed, c->st)) != PRC_OK) return st;
  c->launches++;
  forward_r2c(c, d_out, 1.0);
  const long long total = NN * (H + 1);
  const long long blk = (total + 255) / 256;
  k_grf_amp<<<(int)(blk < (long long)c->sms * 16 ? blk : (long long)c->sms * 16), 256, 0, c->st>>>(c->spec, N,
                                                                                                    c->grf_amp);
  c->launches++;
  float2* U = c->slots;
  run_tile(c, TM_INV, mseg(c, c->spec, U, true), qseg(c, c->spec + NN * H, U + NN * H, true), 1);
  run_tile(c, TM_INV, mseg(c, U, U, false), qseg(c, U + NN * H, U + NN * H, false), 1);
  AdjArgs fa;
  memset(&fa, 0, sizeof(fa));
  fa.slots = U;
  fa.tw = c->tw;
  fa.out = d_out;
  fa.scale = 1.0f;
  c->ks->c2r_plain(c->ksl, grid_for(N * N, c->ksl.line_groups, c->ksl.occ_c2r_plain, c->sms), c->st, fa);
  c->launches++;
  PRC_CU(cudaGetLastError(), "kernel launch");
  if (!out_on_device)
    PRC_CU(cudaMemcpyAsync(delta, d_out, sizeof(float) * n3, cudaMemcpyDeviceToHost, c->st), "D2H field");
  PRC_CU(cudaStreamSynchronize(c->st), "prc_d2z_gaussian_field");
  return PRC_OK;
}

int prc_d2z_history(prc_d2z_ctx* c, const float* zreion, int zreion_on_device, uint32_t* counts,
                    float* history, float* history_z) {
  int st;
  if ((st = check_ctx(c)) != PRC_OK) return st;
  if (!zreion || !history) return prc_fail(PRC_ERR_INVALID, "prc_d2z_history: null zreion or history");
  if ((st = set_device(c)) != PRC_OK) return st;
  const long long n3 = c->NN * c->N;
  const float* d_z = zreion;
  if (!zreion_on_device) {
    if (!c->zre && (st = dalloc(&c->zre, (size_t)n3, "zreion")) != PRC_OK) return st;
    PRC_CU(cudaMemcpyAsync(c->zre, zreion, sizeof(float) * n3, cudaMemcpyHostToDevice, c->st), "H2D zreion");
    d_z = c->zre;
  }
  PRC_CU(cudaMemsetAsync(c->counts, 0, sizeof(uint32_t) * kNHistory, c->st), "memset counts");
  const float dzf = (float)((0.01 - 49.9) / (100000 - 1));  // allvars_d2z.h:1-3, bubblehistory_d2z.C:11
  int blocks = c->sms * 8;
  k_hist<<<blocks, 256, 0, c->st>>>(d_z, n3, c->counts, (double)dzf);
  PRC_CU(cudaGetLastError(), "k_hist launch");
  std::vector<uint32_t> h(kNHistory);
  PRC_CU(cudaMemcpyAsync(h.data(), c->counts, sizeof(uint32_t) * kNHistory, cudaMemcpyDeviceToHost, c->st),
         "D2H counts");
  PRC_CU(cudaStreamSynchronize(c->st), "prc_d2z_history");
  if (counts) memcpy(counts, h.data(), sizeof(uint32_t) * kNHistory);
  // bubblehistory_d2z.C:30-34: float counts / N^3 (double), then a float running sum
  const double n3d = pow((double)c->N, 3.0);
  for (int i = 0; i < kNHistory; ++i) history[i] = (float)((double)(float)h[i] / n3d);
  for (int i = 1; i < kNHistory; ++i) history[i] += history[i - 1];
  if (history_z) {
    history_z[0] = (float)49.9;
    // i*dz is an int x float product (float), then the double sum (bubblehistory_d2z.C:34)
    for (int i = 1; i < kNHistory; ++i) history_z[i] = (float)(49.9 + (double)(i * dzf));
  }
  return PRC_OK;
}

int prc_d2z_backward(prc_d2z_ctx* c, const float* dL_dz, const uint8_t* argmax, int in_on_device,
                     float* dL_ddelta, int out_on_device, double* dL_dB) {
  int st;
  if ((st = check_ctx(c)) != PRC_OK) return st;
  if (!dL_dz || !argmax || !dL_ddelta) return prc_fail(PRC_ERR_INVALID, "prc_d2z_backward: null argument");
  if ((st = set_device(c)) != PRC_OK) return st;
  const int N = c->N, H = c->H;
  const long long NN = c->NN, n3 = NN * N;
  c->launches = 0;
  c->have_timing = 0;
  const float* d_g = dL_dz;
  const uint8_t* d_am = argmax;
  if (!in_on_device) {
    if (!c->gstage && (st = dalloc(&c->gstage, (size_t)n3, "gradient stage")) != PRC_OK) return st;
    if (!c->amstage && (st = dalloc(&c->amstage, (size_t)n3, "argmax stage")) != PRC_OK) return st;
    PRC_CU(cudaMemcpyAsync(c->gstage, dL_dz, sizeof(float) * n3, cudaMemcpyHostToDevice, c->st), "H2D dL/dz");
    PRC_CU(cudaMemcpyAsync(c->amstage, argmax, n3, cudaMemcpyHostToDevice, c->st), "H2D argmax");
    d_g = c->gstage;
    d_am = c->amstage;
  }
  float* d_out = dL_ddelta;
  if (!out_on_device) {
    if (!c->zre && (st = dalloc(&c->zre, (size_t)n3, "output stage")) != PRC_OK) return st;
    d_out = c->zre;
  }
  if (dL_dB) PRC_CU(cudaMemsetAsync(c->dB, 0, sizeof(double) * c->nr, c->st), "memset dB");
  PRC_CU(cudaEventRecord(c->ev[0], c->st), "event");
  float2* U = c->slots;
  float2* acc = c->spec;
  for (int r0 = 0; r0 < c->nr; r0 += c->B) {
    const int nb = (c->nr - r0 < c->B) ? c->nr - r0 : c->B;
    AdjArgs aa;
    memset(&aa, 0, sizeof(aa));
    aa.g = d_g;
    aa.am = d_am;
    aa.A = (float)c->A;
    aa.slots = U;
    aa.slot_stride = c->slot_f2;
    aa.tw = c->tw;
    aa.dB = dL_dB ? c->dB : nullptr;
    aa.nb = nb;
    aa.r0 = r0;
    {
      Prof pf(c, PRC_KIND_ADJ_Z);
      c->ks->adj_z(c->ksl, grid_for(N * N, c->ksl.line_groups, c->ksl.occ_adj_z, c->sms), c->st, aa);
    }
    c->launches++;
    // forward y pass of each slot; Nyquist scratch Qt_b -> Q_b[ix][ky]
    run_tile(c, TM_FWD, mseg(c, U, U, false), qseg(c, U + NN * (H + 1), U + NN * H, true), nb);
    // forward x pass of each slot, acc += W_b * (.)
    run_tile(c, TM_ACC, mseg(c, U, acc, true), qseg(c, U + NN * H, acc + NN * H, false), 1, nb, r0, r0 == 0);
  }
  PRC_CU(cudaEventRecord(c->ev[1], c->st), "event");
  // inverse of the accumulated spectrum into slot 0, then the z C2R
  run_tile(c, TM_INV, mseg(c, acc, U, true), qseg(c, acc + NN * H, U + NN * H, true), 1);
  run_tile(c, TM_INV, mseg(c, U, U, false), qseg(c, U + NN * H, U + NN * H, false), 1);
  AdjArgs fa;
  memset(&fa, 0, sizeof(fa));
  fa.slots = U;
  fa.tw = c->tw;
  fa.out = d_out;
  fa.scale = (float)(1.0 / ((double)n3 * c->dinit));
  {
    Prof pf(c, PRC_KIND_C2R_PLAIN);
    c->ks->c2r_plain(c->ksl, grid_for(N * N, c->ksl.line_groups, c->ksl.occ_c2r_plain, c->sms), c->st, fa);
  }
  c->launches++;
  PRC_CU(cudaGetLastError(), "kernel launch");
  PRC_CU(cudaEventRecord(c->ev[2], c->st), "event");
  if (!out_on_device)
    PRC_CU(cudaMemcpyAsync(dL_ddelta, d_out, sizeof(float) * n3, cudaMemcpyDeviceToHost, c->st), "D2H gradient");
  if (dL_dB) PRC_CU(cudaMemcpyAsync(dL_dB, c->dB, sizeof(double) * c->nr, cudaMemcpyDeviceToHost, c->st), "D2H dB");
  PRC_CU(cudaStreamSynchronize(c->st), "prc_d2z_backward");
  prof_collect(c);
  float t0, t1;
  PRC_CU(cudaEventElapsedTime(&t0, c->ev[0], c->ev[1]), "event time");
  PRC_CU(cudaEventElapsedTime(&t1, c->ev[1], c->ev[2]), "event time");
  c->last_ms[0] = t1;
  c->last_ms[1] = t0;
  c->last_ms[2] = t0 + t1;
  c->have_timing = 1;
  return PRC_OK;
}

int prc_d2z_bubble_mfp(prc_d2z_ctx* c, const prc_mfp_setup* s, const float* zreion_host, const float* history,
                       float* mfp, float* mfp_x, float* dfdmfp) {
  int st;
  if ((st = check_ctx(c)) != PRC_OK) return st;
  if (!s || !zreion_host || !history || !mfp || !mfp_x || !dfdmfp)
    return prc_fail(PRC_ERR_INVALID, "prc_d2z_bubble_mfp: null argument");
  if (s->N != c->N) return prc_fail(PRC_ERR_INVALID, "prc_d2z_bubble_mfp: N=%d but the context has N=%d", s->N, c->N);
  if ((st = set_device(c)) != PRC_OK) return st;
  prc_hist::MfpPlan plan;
  if ((st = prc_hist::mfp_plan(s, zreion_host, history, &plan)) != PRC_OK) return st;
  const long long n3 = c->NN * c->N;
  const long long total = (long long)plan.nx * plan.ns;
  if (!c->zre && (st = dalloc(&c->zre, (size_t)n3, "zreion")) != PRC_OK) return st;
  int *d_start = nullptr, *d_steps = nullptr;
  float* d_zcur = nullptr;
  if ((st = dalloc(&d_start, (size_t)total * 3, "skewer starts")) != PRC_OK) return st;
  if ((st = dalloc(&d_steps, (size_t)total * 2, "skewer steps")) != PRC_OK) {
    cudaFree(d_start);
    return st;
  }
  if ((st = dalloc(&d_zcur, (size_t)plan.nx, "skewer redshifts")) != PRC_OK) {
    cudaFree(d_start);
    cudaFree(d_steps);
    return st;
  }
  std::vector<int> steps((size_t)total * 2);
  cudaError_t e = cudaMemcpyAsync(c->zre, zreion_host, sizeof(float) * n3, cudaMemcpyHostToDevice, c->st);
  if (e == cudaSuccess) e = cudaMemcpyAsync(d_start, plan.start.data(), sizeof(int) * 3 * total, cudaMemcpyHostToDevice, c->st);
  if (e == cudaSuccess) e = cudaMemcpyAsync(d_zcur, plan.zcur.data(), sizeof(float) * plan.nx, cudaMemcpyHostToDevice, c->st);
  if (e == cudaSuccess) {
    k_walks<<<c->sms * 16, 256, 0, c->st>>>(c->zre, c->N, d_start, d_zcur, plan.ns, total, d_steps);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaMemcpyAsync(steps.data(), d_steps, sizeof(int) * 2 * total, cudaMemcpyDeviceToHost, c->st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(c->st);
  cudaFree(d_start);
  cudaFree(d_steps);
  cudaFree(d_zcur);
  if (e != cudaSuccess) return cuda_fail(e, "prc_d2z_bubble_mfp");
  prc_hist::mfp_finish(plan, steps.data(), mfp, mfp_x, dfdmfp);
  return PRC_OK;
}

int prc_d2z_correct(prc_d2z_ctx* c, const float* zvz, float* zreion, int on_device) {
  int st;
  if ((st = check_ctx(c)) != PRC_OK) return st;
  if (!zvz || !zreion) return prc_fail(PRC_ERR_INVALID, "prc_d2z_correct: null argument");
  if ((st = set_device(c)) != PRC_OK) return st;
  const long long n3 = c->NN * c->N;
  float* d_z = zreion;
  if (!on_device) {
    if (!c->zre && (st = dalloc(&c->zre, (size_t)n3, "zreion")) != PRC_OK) return st;
    PRC_CU(cudaMemcpyAsync(c->zre, zreion, sizeof(float) * n3, cudaMemcpyHostToDevice, c->st), "H2D zreion");
    d_z = c->zre;
  }
  float* d_zvz = nullptr;
  if ((st = dalloc(&d_zvz, (size_t)kNHistory, "zvz")) != PRC_OK) return st;
  const float dzf = (float)((0.01 - 49.9) / (100000 - 1));
  cudaError_t e = cudaMemcpyAsync(d_zvz, zvz, sizeof(float) * kNHistory, cudaMemcpyHostToDevice, c->st);
  if (e == cudaSuccess) {
    k_remap<<<c->sms * 8, 256, 0, c->st>>>(d_z, n3, d_zvz, (double)dzf);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess && !on_device)
    e = cudaMemcpyAsync(zreion, d_z, sizeof(float) * n3, cudaMemcpyDeviceToHost, c->st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(c->st);
  cudaFree(d_zvz);
  if (e != cudaSuccess) return cuda_fail(e, "prc_d2z_correct");
  return PRC_OK;
}

int prc_d2z_set_barrier(prc_d2z_ctx* c, const double* barrier_b, double barrier_a) {
  int st;
  if ((st = check_ctx(c)) != PRC_OK) return st;
  if (!barrier_b || !(barrier_a > 0)) return prc_fail(PRC_ERR_INVALID, "prc_d2z_set_barrier: bad argument");
  const double n3 = (double)c->NN * c->N;
  c->A = barrier_a;
  c->as = (float)(barrier_a / n3);
  for (int r = 0; r < c->nr; ++r) {
    c->Bb[r] = barrier_b[r];
    c->cb[r] = (float)(barrier_a * barrier_b[r] - 1.0);
  }
  return PRC_OK;
}

int prc_d2z_win_variants(int N) {
  const KernelSet* ks = kernel_set(N);
  return ks ? ks->n_win_var : 0;
}

int prc_d2z_tune(prc_d2z_ctx* c, int radius_batch, int win_variant) {
  int st;
  if ((st = check_ctx(c)) != PRC_OK) return st;
  if (win_variant < 0 || win_variant >= c->ksl.n_win_var)
    return prc_fail(PRC_ERR_INVALID, "prc_d2z_tune: window variant %d outside 0..%d for N=%d", win_variant,
                    c->ksl.n_win_var - 1, c->N);
  if (radius_batch < 0 || radius_batch > kMaxBatch)
    return prc_fail(PRC_ERR_INVALID, "prc_d2z_tune: radius_batch must be 0..%d", kMaxBatch);
  int B = radius_batch ? radius_batch : c->B;
  if (B > c->nr) B = c->nr;
  if (B > c->slots_b) {  // more radius slots: a new, larger allocation
    if ((st = set_device(c)) != PRC_OK) return st;
    PRC_CU(cudaStreamSynchronize(c->st), "prc_d2z_tune");
    float2* ns = nullptr;
    if ((st = dalloc(&ns, (size_t)c->slot_f2 * B, "radius slots")) != PRC_OK) return st;
    cudaFree(c->slots);
    c->slots = ns;
    c->slots_b = B;
  }
  c->B = B;
  c->win_var = win_variant;
  return PRC_OK;
}

int prc_d2z_batch_tune(prc_d2z_batch* b, int box, int radius_batch, int win_variant) {
  if (!b) return prc_fail(PRC_ERR_INVALID, "prc_d2z_batch_tune: null batch");
  if (box < 0 || box >= b->n) return prc_fail(PRC_ERR_INVALID, "prc_d2z_batch_tune: box %d outside 0..%d", box, b->n - 1);
  int st;
  if ((st = prc_d2z_tune(b->ctx[box], radius_batch, win_variant)) != PRC_OK) return st;
  // the captured graph holds the old launches, the groups the old radius batch
  if (b->exec) cudaGraphExecDestroy(b->exec);
  if (b->graph) cudaGraphDestroy(b->graph);
  b->exec = nullptr;
  b->graph = nullptr;
  b->key.clear();
  b->exec_mode = -1;
  for (auto e : b->gev) cudaEventDestroy(e);
  b->groups.clear();
  b->gev.clear();
  return PRC_OK;
}

int prc_d2z_batch_create(int n_boxes, const prc_d2z_desc* descs, int n_streams, prc_d2z_batch** out) {
  if (!descs || !out || n_boxes < 1) return prc_fail(PRC_ERR_INVALID, "prc_d2z_batch_create: bad argument");
  if (n_streams < 1) n_streams = 1;
  if (n_streams > n_boxes) n_streams = n_boxes;
  *out = nullptr;
  prc_d2z_batch* b = new prc_d2z_batch();
  b->n = n_boxes;
  cudaError_t e = cudaGetDevice(&b->dev);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&b->origin, cudaStreamNonBlocking);
  for (int k = 0; k < n_streams && e == cudaSuccess; ++k) {
    cudaStream_t s;
    e = cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking);
    if (e == cudaSuccess) b->streams.push_back(s);
  }
  for (int k = 0; k <= n_streams && e == cudaSuccess; ++k) {
    cudaEvent_t ev;
    e = cudaEventCreateWithFlags(&ev, cudaEventDisableTiming);
    if (e == cudaSuccess) b->ev.push_back(ev);
  }
  if (e != cudaSuccess) {
    batch_free(b);
    delete b;
    return cuda_fail(e, "prc_d2z_batch_create");
  }
  // larger boxes first, so that the round-robin spreads the work evenly
  std::vector<int> order(n_boxes);
  for (int i = 0; i < n_boxes; ++i) order[i] = i;
  std::stable_sort(order.begin(), order.end(), [&](int x, int y) { return descs[x].N > descs[y].N; });
  b->ctx.assign(n_boxes, nullptr);
  for (int k = 0; k < n_boxes; ++k) {
    const int i = order[k];
    prc_d2z_desc d = descs[i];
    d.stream = b->streams[k % n_streams];
    int st = prc_d2z_create(&d, &b->ctx[i]);
    if (st != PRC_OK) {
      batch_free(b);
      delete b;
      return st;
    }
  }
  *out = b;
  return PRC_OK;
}

int prc_d2z_batch_forward(prc_d2z_batch* b, const float* const* delta, float* const* zreion,
                          uint8_t* const* argmax, int mode) {
  if (!b || !delta || !zreion) return prc_fail(PRC_ERR_INVALID, "prc_d2z_batch_forward: null argument");
  if (mode < PRC_BATCH_LOOP || mode > PRC_BATCH_GROUPED)
    return prc_fail(PRC_ERR_INVALID, "prc_d2z_batch_forward: mode %d is not one of PRC_BATCH_*", mode);
  for (int i = 0; i < b->n; ++i)
    if (!delta[i] || !zreion[i]) return prc_fail(PRC_ERR_INVALID, "prc_d2z_batch_forward: null pointer for box %d", i);
  if (mode == PRC_BATCH_GROUPED && argmax)
    for (int i = 0; i < b->n; ++i)
      if (!argmax[i])
        return prc_fail(PRC_ERR_INVALID, "prc_d2z_batch_forward: grouped launches record every box's argmax or none "
                                         "(box %d has none)", i);
  int cur = -1, st;
  PRC_CU(cudaGetDevice(&cur), "cudaGetDevice");
  if (cur != b->dev) PRC_CU(cudaSetDevice(b->dev), "cudaSetDevice");
  if (mode == PRC_BATCH_GROUPED) {
    // The grouped boxes' pointers live in the tables, so one capture serves
    // every call with the same argmax choice; boxes of sizes without grouped
    // kernels are captured with their pointers (recaptured when they change).
    const int gkey = argmax ? 3 : 2;
    if (b->groups.empty() && (st = batch_group_setup(b)) != PRC_OK) return st;
    // the previous call's table copy has finished reading the host image
    // (a call synchronises before it returns; this covers one that failed)
    PRC_CU(cudaStreamSynchronize(b->origin), "prc_d2z_batch_forward");
    batch_group_fill(b, delta, zreion, argmax);
    if (b->tab_bytes)
      PRC_CU(cudaMemcpyAsync(b->d_tab, b->h_tab, b->tab_bytes, cudaMemcpyHostToDevice, b->origin),
             "batch tables");
    std::vector<const void*> key;
    for (int i = 0; i < b->n; ++i)
      if (!groupable(b->ctx[i])) {
        key.push_back(delta[i]);
        key.push_back(zreion[i]);
        key.push_back(argmax ? argmax[i] : nullptr);
      }
    if (!b->exec || b->exec_mode != gkey || key != b->key) {
      if (b->exec) cudaGraphExecDestroy(b->exec);
      if (b->graph) cudaGraphDestroy(b->graph);
      b->exec = nullptr;
      b->graph = nullptr;
      PRC_CU(cudaStreamBeginCapture(b->origin, cudaStreamCaptureModeThreadLocal), "begin capture");
      batch_enqueue_grouped(b, delta, zreion, argmax);
      cudaGraph_t g = nullptr;
      cudaError_t e = cudaStreamEndCapture(b->origin, &g);
      if (e != cudaSuccess) return cuda_fail(e, "end capture");
      b->graph = g;
      PRC_CU(cudaGraphInstantiate(&b->exec, b->graph, 0), "graph instantiate");
      b->exec_mode = gkey;
      b->key = key;
    }
    PRC_CU(cudaGraphLaunch(b->exec, b->origin), "graph launch");
    PRC_CU(cudaStreamSynchronize(b->origin), "prc_d2z_batch_forward");
    for (auto* c : b->ctx)
      if ((st = check_kernel_flag(c, "prc_d2z_batch_forward")) != PRC_OK) return st;
    return PRC_OK;
  }
  if (b->exec_mode >= PRC_BATCH_GROUPED) {  // a grouped capture (2: without, 3: with argmax)
    if (b->exec) cudaGraphExecDestroy(b->exec);
    if (b->graph) cudaGraphDestroy(b->graph);
    b->exec = nullptr;
    b->graph = nullptr;
    b->key.clear();
  }
  b->exec_mode = mode;
  if (mode == PRC_BATCH_LOOP) {
    batch_enqueue(b, delta, zreion, argmax);
    PRC_CU(cudaGetLastError(), "prc_d2z_batch_forward");
    PRC_CU(cudaStreamSynchronize(b->origin), "prc_d2z_batch_forward");
    for (auto* c : b->ctx)
      if ((st = check_kernel_flag(c, "prc_d2z_batch_forward")) != PRC_OK) return st;
    return PRC_OK;
  }
  std::vector<const void*> key;
  for (int i = 0; i < b->n; ++i) {
    key.push_back(delta[i]);
    key.push_back(zreion[i]);
    key.push_back(argmax ? argmax[i] : nullptr);
  }
  if (!b->exec || key != b->key) {
    if (b->exec) cudaGraphExecDestroy(b->exec);
    if (b->graph) cudaGraphDestroy(b->graph);
    b->exec = nullptr;
    b->graph = nullptr;
    PRC_CU(cudaStreamBeginCapture(b->origin, cudaStreamCaptureModeThreadLocal), "begin capture");
    batch_enqueue(b, delta, zreion, argmax);
    cudaGraph_t g = nullptr;
    cudaError_t e = cudaStreamEndCapture(b->origin, &g);
    if (e != cudaSuccess) return cuda_fail(e, "end capture");
    b->graph = g;
    PRC_CU(cudaGraphInstantiate(&b->exec, b->graph, 0), "graph instantiate");
    b->key = key;
  }
  PRC_CU(cudaGraphLaunch(b->exec, b->origin), "graph launch");
  PRC_CU(cudaStreamSynchronize(b->origin), "prc_d2z_batch_forward");
  for (auto* c : b->ctx)
    if ((st = check_kernel_flag(c, "prc_d2z_batch_forward")) != PRC_OK) return st;
  return PRC_OK;
}

int prc_d2z_batch_launches(prc_d2z_batch* b, int* n) {
  if (!b || !n) return prc_fail(PRC_ERR_INVALID, "prc_d2z_batch_launches: null argument");
  int t = 0;
  if (b->exec_mode >= PRC_BATCH_GROUPED) {
    t = b->launches;
  } else {
    for (auto* c : b->ctx) t += c->launches;
  }
  *n = t;
  return PRC_OK;
}

int prc_d2z_batch_destroy(prc_d2z_batch* b) {
  if (!b) return PRC_OK;
  batch_free(b);
  delete b;
  return PRC_OK;
}

int prc_d2z_last_timing(prc_d2z_ctx* c, float* ms3) {
  int st;
  if ((st = check_ctx(c)) != PRC_OK) return st;
  if (!ms3 || !c->have_timing) return prc_fail(PRC_ERR_INVALID, "prc_d2z_last_timing: no timed call");
  for (int i = 0; i < 3; ++i) ms3[i] = c->last_ms[i];
  return PRC_OK;
}

int prc_d2z_last_launches(prc_d2z_ctx* c, int* n) {
  int st;
  if ((st = check_ctx(c)) != PRC_OK) return st;
  if (!n) return prc_fail(PRC_ERR_INVALID, "prc_d2z_last_launches: null output");
  *n = c->launches;
  return PRC_OK;
}

int prc_d2z_profile(prc_d2z_ctx* c, int enable) {
  int st;
  if ((st = check_ctx(c)) != PRC_OK) return st;
  c->prof = enable ? 1 : 0;
  for (int k = 0; k < PRC_NKINDS; ++k) {
    c->kind_ms[k] = 0;
    c->kind_n[k] = 0;
  }
  c->pused = 0;
  return PRC_OK;
}

int prc_d2z_profile_read(prc_d2z_ctx* c, double* ms, long long* launches) {
  int st;
  if ((st = check_ctx(c)) != PRC_OK) return st;
  if (!ms || !launches) return prc_fail(PRC_ERR_INVALID, "prc_d2z_profile_read: null output");
  for (int k = 0; k < PRC_NKINDS; ++k) {
    ms[k] = c->kind_ms[k];
    launches[k] = c->kind_n[k];
  }
  return PRC_OK;
}

int prc_d2z_destroy(prc_d2z_ctx* c) {
  if (!c) return PRC_OK;
  set_device(c);
  if (c->st) cudaStreamSynchronize(c->st);
  for (cudaStream_t s : c->m_copy)
    if (s) cudaStreamSynchronize(s);
  free_all(c);
  c->ks = nullptr;
  delete c;
  return PRC_OK;
}

}  // extern "C"
