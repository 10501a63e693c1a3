/*
 * prc_d2z.h — C ABI of the GB300 excursion-set reionization step (delta2zreion).
 *
 * The reference executable (pr-calc, c++/src) runs this step as the free function
 * `void delta2zreion()` (proto_d2z.h:27, delta2zreion_d2z.C:8-204) that talks to
 * main() only through globals (allvars_d2z.h:33-76) and FFTW-MPI plans
 * (main_d2z.C:45-48).  This header is the drop-in boundary that replaces that
 * code: main() keeps its CLI, parameter file, raw float32 grid I/O and the
 * post-processing, and calls the entry points below instead of
 * AllocateArrays, the fftwf_mpi_plan_dft_* calls, fftwf_execute and delta2zreion.
 *
 * Conventions
 *   - every entry point returns an int status: PRC_OK (0) or a negative code;
 *     prc_last_error() returns a message for the calling thread's last failure.
 *     No entry point calls exit().
 *   - grids are unpadded, x-major, z fastest (the order of the raw .delta and
 *     .zreion files, io_d2z.C:164-245): cell (i,j,k) is at i*N*N + j*N + k.
 *   - pointers flagged "on_device" are CUDA device pointers; otherwise host
 *     pointers (pinned or pageable) that the call copies through.
 *   - one context per host thread; calls on one context are serialised on the
 *     caller-supplied stream.  The library owns its device workspace, the caller
 *     owns every buffer it passes in.
 */
#ifndef PRC_D2Z_H
#define PRC_D2Z_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ------------------------------------------------------- */
#define PRC_OK               0
#define PRC_ERR_INVALID     -1   /* bad argument (size, pointer, radius list) */
#define PRC_ERR_UNSUPPORTED -2   /* grid size without a compiled FFT plan     */
#define PRC_ERR_CUDA        -3   /* CUDA runtime error                        */
#define PRC_ERR_ALLOC       -4   /* device allocation failed                  */
#define PRC_ERR_IO          -5   /* file could not be opened / short read     */
#define PRC_ERR_NUMERIC     -6   /* root finder / quadrature did not converge */

/* ---- flags for prc_d2z_desc.flags --------------------------------------- */
#define PRC_FLAG_ARGMAX      1   /* keep the per-cell winning radius index    */
#define PRC_FLAG_SIGMA_GRID  2   /* per-radius sqrt(<delta_R^2>) diagnostic   */
/* The window in the reference's own float arithmetic, operation by operation
 * (delta2zreion_d2z.C:41-43,59-82: k = i*dk - kmax, |k| = sqrt of the float
 * sum of squares, W = 3.*(sin(kR) - kR*cos(kR))/pow(kR,3) with its
 * cancellation at small kR), for runs that compare against the reference's
 * output.  Default off: the default window is accurate to the float rounding
 * of its argument at every kR.  Applies to the forward and smoothing passes;
 * the adjoint keeps the accurate window. */
#define PRC_FLAG_FAITHFUL_WINDOW 4

#define PRC_NHISTORY      100000 /* allvars_d2z.h:1 */
#define PRC_ARGMAX_NONE   255    /* argmax value of a cell never updated      */
#define PRC_MAX_RADII     254

/* ---- host tables (cosmology) -------------------------------------------
 * Replaces the scalar set-up of delta2zreion_d2z.C:14-38,55,97-100 and
 * main_d2z.C:57-64: normalize (cosmology.C:246-272), cdmehint
 * (cosmology.C:214-244), growth (cosmology.C:174-212), inverse_erfc
 * (math.C:23-61) and d2z's barrier constants (delta2zreion_d2z.C:206-216).
 * Inputs are the parameter-file and command-line values exactly as the
 * reference holds them (BoxSize in Mpc/h as read, Rmax in Mpc/h, M_min in
 * Msun).  Outputs are what the GPU path consumes. */
typedef struct {
  float Omegam, Omegab, Omegal, h, ns, sigma8, w;   /* Parameter, allvars_d2z.h:58-64 */
  float BoxSize;          /* Mpc/h, as in the parameter file                  */
  float zInit, Rmin;      /* Rmin in cells                                     */
  int   N, Nscales;
  float Rmax, zeta, M_min; /* clParameter, allvars_d2z.h:66-70                 */
} prc_params;

typedef struct {
  float  DInit, zHigh, DHigh;   /* growth(zInit), 20, growth(20)              */
  float  pnorm;                 /* sigma8 normalisation                        */
  float  erfizeta;              /* inverse_erfc(1/zeta)                        */
  float  sigma_min;             /* sqrt(sigma^2(M_min))                        */
  double barrier_a;             /* A = (1+zHigh)*DHigh/1.686 (float product)   */
  /* n = Nscales entries, caller-allocated: */
  double* radii_mpc;            /* R_r in Mpc (the float the reference uses)  */
  float*  sigma_r;              /* sigma(R_r)                                  */
  double* barrier_b;            /* B_r = sqrt(2(smin^2 - s_r^2)) * erfizeta     */
} prc_tables;

int prc_compute_tables(const prc_params* p, prc_tables* out);

/* Growth factor D(z) (cosmology.C:174-212). */
float prc_growth(float z, float omegam, float omegal, float w);
/* sigma^2(M) of a top-hat of mass M [Msun] (cosmology.C:214-244). */
int prc_sigma2(float omegam, float omegab, float h, float ns, float pnorm,
               float mass, float* sgm2);
/* erfc^-1(x) as the reference's bracketing root finder returns it (math.C:23-61). */
int prc_inverse_erfc(float x, float* out);
/* Thomson optical depth of an ionisation history (cosmology.C:52-83). */
float prc_tau(const float* za, const float* xa, int nz, float omegam,
              float omegab, float h);

/* ---- the GPU path --------------------------------------------------------- */
typedef struct prc_d2z_ctx prc_d2z_ctx;

typedef struct {
  int           N;                /* grid side (see prc_d2z_supported)          */
  int           n_radii;          /* Nscales, 1..PRC_MAX_RADII                  */
  double        box_mpc;          /* box side in Mpc (BoxSize/h)                */
  const double* radii_mpc;        /* n_radii top-hat radii [Mpc], processing order */
  const double* barrier_b;        /* n_radii barrier offsets B_r (NaN: radius never wins) */
  double        barrier_a;        /* A in z = A*(delta_R + B_r) - 1             */
  double        growth_init;      /* D(zInit); delta_lin is divided by it (main_d2z.C:59) */
  int           radius_batch;     /* radii per sweep, <= 64; 0 = 16 (8 for N >= 1024) */
  int           flags;            /* PRC_FLAG_*                                 */
  void*         stream;           /* cudaStream_t; NULL = default stream        */
} prc_d2z_desc;

/* Tuning knobs (no counterpart in the reference, whose FFTW plans are
 * chosen by FFTW).  prc_d2z_win_variants: how many window-pass variants (tile
 * width and radix plan) are compiled for grid side N (0: N unsupported).
 * prc_d2z_tune: the radius batch (radii per sweep, 0 = keep; a larger batch
 * reallocates the radius slots) and the window-pass variant of a context;
 * results do not depend on either beyond float rounding of the transform.
 * prc_d2z_batch_tune: the same for box `box` of a batch (the next forward
 * re-captures its graph).  prc_d2z.autotune picks both by timing. */
int prc_d2z_win_variants(int N);
int prc_d2z_tune(prc_d2z_ctx* ctx, int radius_batch, int win_variant);

/* Synthetic input fields (the producer of delta_lin; the role of the ics
 * generator, grf_ics.C:8-112, whose drand48 + Marsaglia-polar stream is
 * sequential by construction and is replaced by a counter-based one).
 *
 * prc_white_noise: n unit Gaussians into device memory, cell i from
 * Philox4x32-10 with counter (i mod 2^32, i div 2^32, 0, 0) and key (seed, 0),
 * Box-Muller in FP64 on words 0 and 1, rounded to float32; stream-ordered,
 * no synchronisation.  No counterpart in the reference. */
int prc_white_noise(float* d_out, long long n, unsigned int seed, void* stream);

/* Replaces the barrier table of a context (same radii): B_r and A as in the
 * descriptor.  For parameter scans (e.g. zeta) without a new workspace. */
int prc_d2z_set_barrier(prc_d2z_ctx* ctx, const double* barrier_b, double barrier_a);

/* 1 if N has a compiled FFT plan, else 0. */
int prc_d2z_supported(int N);

/* Allocates the device workspace for one box (replaces AllocateArrays,
 * allocate_d2z.C:5-44, and the FFTW plans, main_d2z.C:32-48). */
int prc_d2z_create(const prc_d2z_desc* desc, prc_d2z_ctx** out);

/* delta_lin (N^3, file order) -> zreion (N^3) and optional argmax (N^3 uint8,
 * PRC_ARGMAX_NONE where never updated) and sigma_grid (n_radii doubles).
 * Replaces main_d2z.C:57-71 (delta/=DInit, forward R2C, delta2zreion()),
 * i.e. the zreion field before GetHistory/CorrectHistory.  zreion starts at 0
 * (allocate_d2z.C:37); a radius updates a cell iff its z is strictly larger
 * (delta2zreion_d2z.C:138).  Returns PRC_ERR_CUDA (outputs incomplete) if a
 * kernel's bounded wait for a staging copy ran out; the context stays usable. */
int prc_d2z_forward(prc_d2z_ctx* ctx, const float* delta_lin, int delta_on_device,
                    float* zreion, uint8_t* argmax, int out_on_device,
                    double* sigma_grid);

/* prc_d2z_forward over n boxes of this context's shape, all from host
 * buffers (delta[i] -> zreion[i], argmax[i]; argmax may be null): a stream of
 * realisations, as a program that loops main_d2z.C:57-71 over input files
 * would run it.  Box i+1's input is copied in and box i-1's outputs copied
 * out by the copy engines while box i's kernels run (pinned buffers; pageable
 * ones are correct but serialise).  Results equal n calls of
 * prc_d2z_forward.  Output buffers of different boxes must not overlap unless
 * they are the same buffer (then the later box's result is what remains).
 * Returns when every output is on the host.  No
 * counterpart in the reference, which processes one box per run. */
int prc_d2z_forward_many(prc_d2z_ctx* ctx, int n, const float* const* delta,
                         float* const* zreion, uint8_t* const* argmax);

/* The smoothed field of one radius, delta_R = C2R(W_R * R2C(delta_lin/D_init))/N^3
 * (delta2zreion_d2z.C:57-93), written to delta_r (N^3).  A diagnostic beside
 * prc_d2z_forward, which never materialises delta_R. */
int prc_d2z_smooth(prc_d2z_ctx* ctx, const float* delta_lin, int delta_on_device, int radius,
                   float* delta_r, int out_on_device);

/* A Gaussian random field on the context's grid, written to delta (N^3 float32,
 * file order): w = prc_white_noise(seed), then delta = C2R(amp[|m|^2] * R2C(w)),
 * |m|^2 = fx^2 + fy^2 + fz^2 over the folded integer wavenumbers (|f| <= N/2).
 * amp (host, n_amp >= 3*(N/2)^2 + 1 floats) carries the whole spectral shape
 * and normalisation, including the 1/N^3 of the inverse transform and
 * amp[0] = 0; e.g. sqrt(N^3 P(k)/L^3)/N^3 gives the normalisation of
 * grf_ics.C:20-28,49-78.  Uses the context's spectrum and first radius slot. */
int prc_d2z_gaussian_field(prc_d2z_ctx* ctx, unsigned int seed, const float* amp, int n_amp,
                           float* delta, int out_on_device);

/* Ionisation-history histogram of a zreion grid (bubblehistory_d2z.C:17-34):
 * counts[PRC_NHISTORY] raw bin counts (optional) and history[PRC_NHISTORY], the
 * cumulative ionised fraction exactly as GetHistory forms it, and
 * history_z[PRC_NHISTORY] (optional). */
int prc_d2z_history(prc_d2z_ctx* ctx, const float* zreion, int zreion_on_device,
                    uint32_t* counts, float* history, float* history_z);

/* ---- history correction (main_d2z.C:76-101) -------------------------------
 * After the hot loop the reference turns the raw zreion field into its final
 * form: GetBubbleMFP (bubble mean free path from random skewers), GetCHistory
 * (the MFP-corrected ionisation history) and CorrectHistory (a per-cell map
 * of zreion through that history).  These entry points restate them. */
#define PRC_NCHISTORY 10000   /* allvars_d2z.h:5 */
#define PRC_NX_MFP    1000    /* allvars_d2z.h:9 */
#define PRC_NMFP      200     /* allvars_d2z.h:13 */
#define PRC_NSKEWERS  20000   /* allvars_d2z.h:17 */

/* Float2FloatTable (tables.C:9-38): f32 min, f32 max, i32 n, f32 table[n]. */
typedef struct {
  float minval, maxval, delta;
  int n;
  float* table;   /* malloc'd by prc_f2f_load, released by prc_f2f_free */
} prc_f2f_table;
int prc_f2f_load(const char* path, prc_f2f_table* t);
float prc_f2f_eval(const prc_f2f_table* t, float x);
void prc_f2f_free(prc_f2f_table* t);

/* deltac and the Press-Schechter collapsed fraction (cosmology.C:141-172,311-324). */
float prc_deltac(float z, float omegam, float omegal, float w, float* dcoll);
float prc_fcoll(float z, float zInit, float omegam, float omegal, float w, float sigma_min);

/* GetBubbleMFP (bubblehistory_d2z.C:82-252) at one rank: for n_x ionised
 * fractions x (0.01..0.999) and n_skewers random ionised start cells each
 * (glibc rand() from its unseeded state, as the reference draws them), walk
 * along y and z to the first neutral cell.  Outputs mfp[n_x], mfp_x[n_x] and
 * dfdmfp[PRC_NMFP * n_x].  zreion is a host grid (the rejection sampling of
 * the starts reads it); the walks run on the device. */
typedef struct {
  int N;
  float box_mpc;      /* BoxSize / h */
  int n_x;            /* PRC_NX_MFP in the reference */
  int n_skewers;      /* PRC_NSKEWERS in the reference */
} prc_mfp_setup;
int prc_d2z_bubble_mfp(prc_d2z_ctx* ctx, const prc_mfp_setup* s, const float* zreion_host,
                       const float* history, float* mfp, float* mfp_x, float* dfdmfp);

/* GetCHistory (bubblehistory_d2z.C:45-80): chistory[PRC_NCHISTORY] from the
 * fcoll table, the MFP curve (n_x points), rmfp (the -r value) and zeta. */
int prc_chistory(const prc_f2f_table* fcoll, const float* mfp, int n_x, float rmfp, float zeta,
                 float* chistory);
/* CorrectHistory's map (bubblehistory_d2z.C:314-326): zvz[PRC_NHISTORY]. */
int prc_zvz(const float* history, const float* chistory, float* zvz);
/* CorrectHistory's per-cell step (bubblehistory_d2z.C:328-341) on the device:
 * zreion = zvz[(int)((zreion - 49.9)/dz)].  Cells whose bin falls outside the
 * table (z > 50.4 or z < 0.01; the reference reads out of bounds there) are
 * left unchanged. */
int prc_d2z_correct(prc_d2z_ctx* ctx, const float* zvz, float* zreion, int zreion_on_device);

/* Adjoint of prc_d2z_forward (no reference counterpart: the reference has no
 * gradient).  dL_dz (N^3) and argmax (N^3) -> dL/d delta_lin (N^3) and
 * dL/dB_r (n_radii doubles, optional).  The host maps dL/dB_r to dL/dzeta and
 * dL/dM_min with prc_barrier_grad. */
int prc_d2z_backward(prc_d2z_ctx* ctx, const float* dL_dz, const uint8_t* argmax,
                     int in_on_device, float* dL_ddelta, int out_on_device,
                     double* dL_dB);

/* Time of the last forward/backward split by stage, in milliseconds, measured
 * with CUDA events on the context's stream: [0] forward R2C, [1] radius sweeps,
 * [2] total.  Returns PRC_ERR_INVALID if no timed call happened. */
int prc_d2z_last_timing(prc_d2z_ctx* ctx, float* ms3);

/* Kernel launches issued by the last forward/backward call. */
int prc_d2z_last_launches(prc_d2z_ctx* ctx, int* n);

/* ---- batches of boxes ------------------------------------------------------
 * Many independent boxes (realisations), possibly of different grid sizes,
 * one workspace per box.  delta, zreion (and argmax, nullable) are arrays of
 * n_boxes device pointers; every mode gives the same results bit for bit.
 * Modes of prc_d2z_batch_forward:
 *   PRC_BATCH_LOOP     each box's launches, boxes spread over n_streams streams;
 *   PRC_BATCH_GRAPH    the same launches captured once into a CUDA graph and
 *                      replayed with one launch per call (captured again when
 *                      the pointers change);
 *   PRC_BATCH_GROUPED  the boxes of each grid size form a group and every pass
 *                      of the step runs as ONE launch over all boxes of the
 *                      group: resident CTAs walk the (box, tile) or (box, line
 *                      group) items of that pass, with each box's pointers,
 *                      radius count and constants read from device tables;
 *                      the groups share out the n_streams streams (largest
 *                      grid size first), all captured once into a CUDA graph (about 3 + 3 x sweeps launches per grid size
 *                      instead of as many per box).  The tables are rewritten
 *                      at every call, so new pointers need no new capture.
 *                      Grid sizes up to 256 except 8..24 and 48 have grouped
 *                      kernels; boxes of other sizes run per box inside the same
 *                      graph.  argmax: every box or none; each box keeps its
 *                      own radius batch; the window pass uses variant 0 (boxes
 *                      with PRC_FLAG_FAITHFUL_WINDOW run per box).
 * No reference counterpart: the reference processes one box per run. */
#define PRC_BATCH_LOOP    0
#define PRC_BATCH_GRAPH   1
#define PRC_BATCH_GROUPED 2
typedef struct prc_d2z_batch prc_d2z_batch;
int prc_d2z_batch_create(int n_boxes, const prc_d2z_desc* descs, int n_streams, prc_d2z_batch** out);
int prc_d2z_batch_tune(prc_d2z_batch* batch, int box, int radius_batch, int win_variant);
int prc_d2z_batch_forward(prc_d2z_batch* batch, const float* const* delta, float* const* zreion,
                          uint8_t* const* argmax, int mode);
int prc_d2z_batch_launches(prc_d2z_batch* batch, int* n);
int prc_d2z_batch_destroy(prc_d2z_batch* batch);

/* Per-kernel timing: with profiling enabled every launch is bracketed by CUDA
 * events on the context's stream and the totals accumulate per kernel kind
 * (PRC_KIND_*) until the next prc_d2z_profile call resets them. */
#define PRC_KIND_R2C_Z     0   /* forward z pass (real -> half complex)         */
#define PRC_KIND_COL_FWD   1   /* forward column pass (y or x)                  */
#define PRC_KIND_WIN_X     2   /* window + inverse x pass, per sweep            */
#define PRC_KIND_COL_INV   3   /* inverse column pass (y), per sweep            */
#define PRC_KIND_C2R_Z     4   /* inverse z pass + barrier/max, per sweep       */
#define PRC_KIND_ADJ_Z     5   /* adjoint source z pass                         */
#define PRC_KIND_ADJ_X     6   /* adjoint x pass + window accumulate            */
#define PRC_KIND_C2R_PLAIN 7   /* plain inverse z pass                          */
#define PRC_NKINDS         8
int prc_d2z_profile(prc_d2z_ctx* ctx, int enable);
int prc_d2z_profile_read(prc_d2z_ctx* ctx, double* ms /*PRC_NKINDS*/, long long* launches /*PRC_NKINDS*/);

int prc_d2z_destroy(prc_d2z_ctx* ctx);

/* prc_d2z_forward for small boxes without any device allocation.  No
 * counterpart in the reference (pr-calc always allocates its FFTW buffers).
 * For callers that must not allocate device memory when they ask for a
 * result: a host framework that owns all device memory through its own pool,
 * or a latency-critical stage that cannot afford cudaMalloc/cudaFree, which may
 * synchronise the device.  The workspace is a fixed array inside the library
 * (about 2.2 MB, held by every GPU that loads it) that fits grids up to N = 64
 * (N in 8, 12, 16, 24, 32, 48, 64); larger N is rejected with PRC_ERR_INVALID.
 * delta_lin, zreion and argmax (nullable) are device pointers, N^3 each, laid
 * out as for prc_d2z_forward, whose zreion/argmax it reproduces; the call
 * returns after the work on `stream` has finished.  The first call on a device
 * performs a one-time set-up (it looks up the arrays' device addresses and
 * writes the twiddle tables of every supported N into the array), so make it
 * before any stream capture.  All calls share the one array: calls that
 * overlap on the GPU race, so serialise them.  Like prc_d2z_forward it returns
 * PRC_ERR_CUDA if a kernel's bounded wait for a staging copy ran out (the
 * error word it reads for that is a second static array of one int, cleared
 * by every call). */
int prc_d2z_forward_static(int N, int n_radii, double box_mpc, const double* radii_mpc,
                           const double* barrier_b, double barrier_a, double growth_init,
                           const float* delta_lin, float* zreion, uint8_t* argmax, void* stream);

/* Test hook for the failure path of the bounded waits (no counterpart in the
 * reference).  The next `calls` calls of prc_d2z_forward or
 * prc_d2z_forward_static run their first sweep with one staging copy of the
 * inverse z pass withheld (grids whose z pass stages lines by bulk copy:
 * every N >= 32 except 48): the waiting CTA gives up after a
 * short bounded wait with no copy in flight, the call returns PRC_ERR_CUDA
 * and the next call runs normally.  0 cancels; process-wide. */
int prc_d2z_test_withhold_copy(int calls);

const char* prc_last_error(void);

#ifdef __cplusplus
}
#endif
#endif /* PRC_D2Z_H */
