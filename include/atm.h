/*
 * atm.h -- C ABI of the GB300 split-step beam-propagation engine (libatm.so).
 *
 * The engine replaces pyAtmosphere's numpy/cupy Monte-Carlo path:
 *   sparse-spectrum phase screens  -> atm_screen / inside atm_run
 *   angular-spectrum vacuum steps  -> atm_vacuum / inside atm_run
 *   pupil + intensity moments      -> inside atm_run (measures_out)
 * Python binds it with ctypes (pyatmosphere_gb300/engine/_lib.py); any other
 * host language binds the same plain-C signatures.
 *
 * Conventions
 *   - Every array argument of atm_run / atm_screen / atm_vacuum is a DEVICE
 *     pointer on the device that was current at atm_plan_create.  Descriptor
 *     arrays (positions, radii, f_base) are HOST pointers, read during
 *     atm_plan_create only.
 *   - complex64 arrays are interleaved (re, im) float pairs, passed as void*.
 *   - Layouts are row-major; a field is [batch][N][N] with row index = y
 *     (top = -N/2 * delta), column = x, as RectGrid.get_y / get_x.
 *   - Spectra are [batch][n_screens][P]: rho, theta (float32), value
 *     (complex64), exactly PolarDiscreteFunction(rho, theta, value) of each
 *     SSPhaseScreen (phase_screens.py:98-103).
 *   - Calls are stream-ordered on `stream` (a cudaStream_t, NULL = legacy
 *     default stream) and return before the GPU work ends.  A plan serves one
 *     stream at a time; distinct plans are independent.
 *   - Every call returns ATM_OK (0) or a negative status; atm_last_error()
 *     gives the message (per host thread).  Nothing is printed, nothing exits.
 */
#ifndef ATM_H
#define ATM_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define ATM_ABI_VERSION 3  /* 2: AtmPlanInfo.tiled; atm_plan_check, atm_set_wait_budget;
                              3: atm_channel_draw_spectra */

#define ATM_OK 0
#define ATM_ERR_INVALID (-1)     /* bad argument */
#define ATM_ERR_UNSUPPORTED (-2) /* e.g. N not a power of two in [128, 4096] */
#define ATM_ERR_CUDA (-3)        /* CUDA runtime error (message has details) */
#define ATM_ERR_NOMEM (-4)       /* device allocation failed */
#define ATM_ERR_TIMEOUT (-5)     /* a kernel's bounded wait ran out (atm_plan_check) */
#define ATM_ERR_NONFINITE (-6)   /* NaN or infinite spectrum values were injected (atm_plan_check) */

#define ATM_SOURCE_GAUSSIAN 0    /* GaussianSource (sources.py:21-23) */
#define ATM_SOURCE_PLANE 1       /* PlaneSource (sources.py:16-18) */

#define ATM_MAX_PUPILS 8

/* AtmChannelDesc.flags */
#define ATM_FLAG_SIMT_GEMM 1     /* screen GEMM on FP32 SIMT cores (default below N = 256) */
#define ATM_FLAG_TC_GEMM 2       /* screen GEMM on tcgen05 tensor cores (the default for N >= 256) */
#define ATM_FLAG_TC_CPASYNC 4    /* tensor-core GEMM in its one-CTA-per-tile cp.async form instead of the
                                    persistent TMA form */
#define ATM_FLAG_STEP_MEASURES 8 /* also measure the field just after every screen (per-step measures) */
#define ATM_FLAG_TC_N256 16      /* persistent TMA GEMM with 128 x 256 tiles, two stages, one accumulator pair
                                    and TMA-stored result blocks (the default form; the flag is kept) */
#define ATM_FLAG_TC_N128 32      /* persistent TMA GEMM with 128 x 128 tiles, three stages and double-buffered
                                    accumulators instead of the default 128 x 256 form */
#define ATM_FLAG_TILED 64        /* keep the plan's field between passes in the tiled layout (4 x 4 blocks of
                                    128 bytes): the column pass then moves whole 128-byte lines; N in
                                    {512, 1024, 2048}.  Inputs and outputs of every call stay row-major. */
#define ATM_FLAG_ROWMAJOR 128    /* keep the plan's field row-major where the tiled layout would be the default */
#define ATM_FLAG_FFT_SCREENS 256 /* hold the workspace of atm_run_fft (one more complex64 field per realisation) */

/* per-realisation doubles in measures_out (slot index).  With
 * ATM_FLAG_STEP_MEASURES, ATM_STEP_SLOTS more doubles per screen i follow the
 * pupil and tracked slots, at ATM_OUT_PUPIL0 + n_pupils + n_tracked +
 * i * ATM_STEP_SLOTS: slots 0..7 below (eta_total .. I_center) of the field
 * just after screen i, the value PhaseScreensPath.generator yields
 * (pathes.py:61-75) and SIResult / BeamPropagationResult measure
 * (simulations/si.py:11-48, simulations/beam.py:83-114). */
#define ATM_STEP_SLOTS 8
/* per-realisation doubles in measures_out (slot index) */
#define ATM_OUT_ETA_TOTAL 0      /* measures.eta(pupil=False)      measures.py:7-8   */
#define ATM_OUT_MEAN_X 1         /* measures.mean_x                measures.py:11-13 */
#define ATM_OUT_MEAN_Y 2         /* measures.mean_y  (-y weighted) measures.py:16-18 */
#define ATM_OUT_MEAN_X2 3        /* measures.mean_x2               measures.py:26-28 */
#define ATM_OUT_MEAN_XY 4        /* measures.mean_xy (-x y)        measures.py:31-33 */
#define ATM_OUT_MEAN_Y2 5        /* measures.mean_y2               measures.py:36-38 */
#define ATM_OUT_MEAN_X2_R 6      /* BeamResult.mean_x2_r           simulations/beam.py:26-33 */
#define ATM_OUT_I_CENTER 7       /* |u|^2 at the origin pixel      simulations/si.py:11-12 */
#define ATM_OUT_PUPIL0 8         /* eta through pupil p (slot 8+p), then tracked pupils */

typedef struct AtmPlan AtmPlan;

typedef struct AtmChannelDesc {
  int32_t abi_version;        /* ATM_ABI_VERSION */
  int32_t resolution;         /* RectGrid.resolution N: power of two in [128, 4096] */
  double delta;               /* RectGrid.delta [m] */
  int32_t source_kind;        /* ATM_SOURCE_* */
  double wvl, w0, F0;         /* GaussianSource(wvl, w0, F0); F0 = +/-inf: collimated */
  int32_t n_screens;          /* screens on the path (0: VacuumPath) */
  const double* positions;    /* [n_screens] PhaseScreensPath.positions [m] */
  double length;              /* path length [m] */
  double losses_db;           /* AbstractPath.losses_db */
  int32_t path_output_loss;   /* 1: Channel.run (loss applied once more on exit,
                                 pathes.py:23-24); 0: Channel.generator */
  int32_t points;             /* RandLogPolarGrid.points P */
  const float* f_base;        /* [P] RandLogPolarGrid.base (annulus outer radii) */
  double shift_x, shift_y;    /* SSPhaseScreen.generate_phase_screen shift [m] */
  int32_t n_pupils;           /* fixed CirclePupils, <= ATM_MAX_PUPILS */
  const double* pupil_radius; /* [n_pupils] */
  const double* pupil_shift_x;/* [n_pupils] CirclePupil.get_pupil shift (may be NULL) */
  const double* pupil_shift_y;/* [n_pupils] (may be NULL) */
  int32_t n_tracked;          /* pupils centred on each realisation's centroid */
  const double* tracked_radius;/* [n_tracked] (TrackedPDTResult, simulations/pdt.py:51-66) */
  int32_t batch;              /* maximum realisations per atm_run */
  double cheb_cut;            /* low-frequency block: annuli below cheb_cut/(N delta); 0 = 4 */
  int32_t col_tile;           /* column-pass tile (columns per CTA); 0 = default */
  int32_t flags;              /* ATM_FLAG_*; 0 = defaults */
} AtmChannelDesc;

typedef struct AtmPlanInfo {
  int32_t n_out;              /* doubles per realisation in measures_out */
  int32_t low_annuli;         /* annuli folded into the Chebyshev block */
  int32_t cheb_terms;         /* Chebyshev terms per axis */
  int32_t gemm_k;             /* inner dimension of the screen GEMM */
  int64_t workspace_bytes;    /* device memory held by the plan */
  int32_t launches_per_run;   /* kernel launches of one atm_run (without tracked/field extras) */
  int32_t row_parts;          /* row-pass CTAs per realisation */
  int32_t col_tile;           /* columns per CTA of the column pass */
  int32_t row_variant;        /* 0: persistent pipelined row pass, 1: one CTA per row block,
                                 2: persistent pipelined with one row per CTA,
                                 3: as 2 with rows loaded by bulk copies (TMA),
                                 4: as 3 with twiddles formed from powers of two,
                                 5: tiled layout, four rows per CTA with a named barrier per row,
                                 6: as 5 with twiddles formed from powers of two,
                                 7: as 4 with each thread's twiddle bases held in registers,
                                 8: as 6 with each thread's twiddle bases held in registers,
                                 9: tiled layout, one row per CTA as 4 (tensor copies of the row's
                                    share of each 4 x 4 block),
                                 10: as 9 with each thread's twiddle bases held in registers,
                                 11: N = 1024 / 2048 only: one warp per row with warp FFTs (lane j holds
                                     elements j + 32 m; one exchange per transform, in the warp's own
                                     shared buffer); passes with measures run the form of 4 */
  int32_t col_variant;        /* 0: persistent pipelined column pass, 1: one CTA per column tile,
                                 2: persistent pipelined with twiddles formed from powers of two,
                                 3: persistent with tiles loaded by TMA (loads overlap the FFTs),
                                 4: as 3 with the FFT exchanges alternating between two buffers
                                    (one barrier per exchange instead of two),
                                 5: as 4 on the tiled layout (block columns of 4 columns),
                                 6: tiled layout, each column of a block column transformed by its own
                                    warps with their own named barrier; a producer warp loads and stores
                                    the block columns with TMA,
                                 7: as 4 with each thread's twiddle bases held in registers (the
                                    product-twiddle arithmetic of 2; tiles that the TMA form does
                                    not take run the form of 2),
                                 8: as 6 with each thread's twiddle bases held in registers,
                                 9: as 6 with twiddles formed from powers of two (the bits of 8),
                                 10: N = 1024 / 2048 / 4096, column tile 4: warp FFTs in two groups of
                                     four warps on a ring of three TMA-loaded, TMA-stored tiles of 4
                                     columns (2 columns of 64-lane transforms at 4096; one exchange per
                                     transform),
                                 13: as 10 on the tiled layout (tiles of whole 128-byte blocks),
                                 14: N = 4096, column tile 4: each 4096-point column transform as two
                                     2048-point warp FFTs (a radix-2 split in y), one per group of
                                     four warps, on tiles of 4 columns held as two 2048-row units in
                                     a ring of three; an inverse-only pass runs the form of 3,
                                 15: N = 2048, column tile 4: the split of 14 with 1024-point halves
                                     (32 elements per lane, 16 warps per SM), two pairs of groups
                                     per CTA sharing a ring of six 1024-row units; an inverse-only
                                     pass runs the form of 10 */
  int32_t tuned;              /* 1 after a successful atm_autotune */
  int32_t gemm_form;          /* screen GEMM: 0 FP32 SIMT, 1 tcgen05 cp.async form, 2 tcgen05 persistent TMA
                                 form with 128 x 128 tiles (ATM_FLAG_TC_N128), 3 the same with 128 x 256
                                 tiles and TMA-stored result blocks (the default) */
  int32_t tiled;              /* 1: the plan's field is kept in the tiled layout between passes */
} AtmPlanInfo;

/* ABI version of the loaded library (ATM_ABI_VERSION). */
int atm_abi_version(void);

/* Message of the last failed call on this host thread ("" if none). */
const char* atm_last_error(void);

/* Builds a plan for one channel geometry and batch size: validates the
 * descriptor, picks the low-frequency split and GEMM shape, uploads the
 * source / transfer-function tables and allocates the workspace.
 * Replaces the object graph built by Channel(...) (channels.py:17-29) with
 * IdenticalPhaseScreensPath / PhaseScreensPath (pathes.py:43-95),
 * GaussianSource (sources.py:21-23), RectGrid (grids.py:7-85),
 * RandLogPolarGrid (grids.py:88-119) and CirclePupil (pupils.py:4-13). */
int atm_plan_create(const AtmChannelDesc* desc, AtmPlan** plan);

/* Frees the plan and its workspace (waits for the device). */
int atm_plan_destroy(AtmPlan* plan);

/* Sizes chosen by atm_plan_create. */
int atm_plan_info(const AtmPlan* plan, AtmPlanInfo* info);

/* Runs `batch` realisations of the channel with the injected spectra.
 * Replaces Channel.run(pupil=False) (channels.py:31-35) driving
 * PhaseScreensPath.generator (pathes.py:61-75) with SSPhaseScreen screens,
 * followed by measures.* (measures.py:1-38), BeamResult.mean_x2_r
 * (simulations/beam.py:26-33) and PDTResult / TrackedPDTResult eta
 * (simulations/pdt.py:15-26, 51-66).
 *   measures_out   [batch][n_out] doubles (required)
 *   field_out      [batch][N][N] complex64 final field (nullable)
 *   mean_intensity [N][N] float32; the intensity of every realisation is
 *                  ADDED to it (nullable; the caller zeroes and divides). */
int atm_run(AtmPlan* plan, const float* rho, const float* theta, const void* value, int32_t batch,
            double* measures_out, void* field_out, float* mean_intensity, void* stream);

/* Synthesises screen `screen` of every realisation in the batch.
 * Replaces SSPhaseScreen.generate (phase_screens.py:25-28, 108-136).
 *   phi_out    [batch][N][N] float32 screen (nullable)
 *   phasor_out [batch][N][N] complex64 exp(-i phi) as applied on the path
 *              (pathes.py:72-73; nullable) */
int atm_screen(AtmPlan* plan, const float* rho, const float* theta, const void* value, int32_t batch,
               int32_t screen, float* phi_out, void* phasor_out, void* stream);

/* One angular-spectrum vacuum step of length dz, in place on a spatial
 * field [batch][N][N] complex64.  Replaces VacuumPath.output /
 * vacuum_propagation (pathes.py:27-40, theory/vacuum.py:5-7,
 * utils.py:42-50); dz <= 0 leaves the field unchanged. */
int atm_vacuum(AtmPlan* plan, void* field, int32_t batch, double dz, void* stream);

/* Measures of given spatial fields [batch][N][N] complex64 into
 * measures_out [batch][n_out] (same slots as atm_run).  Replaces calling
 * measures.eta / mean_x / mean_y / mean_x2 / mean_xy / mean_y2
 * (measures.py:1-38) on an output field, CirclePupil.output + eta
 * (pupils.py:12-13) and BeamResult.mean_x2_r (simulations/beam.py:26-33). */
int atm_measures(AtmPlan* plan, const void* field, int32_t batch, double* measures_out, void* stream);

/* FFT phase screens with subharmonics for every realisation in the batch.
 * Replaces FFTPhaseScreen.generate(complex=True) (phase_screens.py:37-67):
 * spectrum (a + i b) amp on the centred frequency grid (DC = 0), centred
 * inverse 2-D FFT times N^2, plus the 3x3 subharmonic levels, minus the
 * mean.  The engine's own FFT passes run it without shift copies; the
 * subharmonic sum sum_j X_j(x) Y_j(y) comes as FP64-built 1-D factors.
 *   normals    [batch][2][N][N] float32 (real, imaginary draws of the main grid)
 *   amp        [N][N] float32 sqrt(Phi_phi(|f|)) 2 pi df, centred order
 *   sub_x, sub_y [batch][n_sub][N] complex64; sub_mean [batch][2] float64
 *   screen_out [batch][N][N] complex64 (its real part is the phase) */
int atm_fft_screen(AtmPlan* plan, const float* normals, const float* amp, const void* sub_x, const void* sub_y,
                   const double* sub_mean, int32_t n_sub, int32_t batch, void* screen_out, void* stream);

/* atm_run with FFT phase screens in place of the sparse-spectrum ones: per
 * screen i the screen of atm_fft_screen is built for every realisation of the
 * batch (its own workspace; the plan needs ATM_FLAG_FFT_SCREENS) and the beam
 * is multiplied by exp(-i Re(screen)) between the vacuum steps, as
 * PhaseScreensPath.generator does with FFTPhaseScreen screens
 * (pathes.py:61-75, phase_screens.py:37-67).  Same outputs as atm_run.
 *   normals    [batch][n][2][N][N] float32 (main-grid draws of each screen)
 *   amp        [n][N][N] float32, each screen's sqrt(Phi_phi(|f|)) 2 pi df
 *   sub_x, sub_y [batch][n][n_sub][N] complex64; sub_mean [batch][n][2] float64
 * The plan's spectral grid (f_base) is not used. */
int atm_run_fft(AtmPlan* plan, const float* normals, const float* amp, const void* sub_x, const void* sub_y,
                const double* sub_mean, int32_t n_sub, int32_t batch, double* measures_out, void* field_out,
                void* stream);

/* Re-targets a plan to another channel of the same grid, spectral grid,
 * pupil counts and batch (source, positions, length, losses, shift and
 * pupil radii may change; the screen count may be any 1..n_screens of the
 * creating descriptor, and the spectra of later runs are then laid out
 * [batch][new count][P]) without reallocating; waits for the device first.
 * Replaces building a new Channel for each parameter point of a sweep
 * (channels.py:17-29). */
int atm_plan_update(AtmPlan* plan, const AtmChannelDesc* desc);

/* Channel table sets: the state atm_plan_update would set (source, path
 * geometry, losses, screen shift, pupil radii, and the device tables built
 * from them), built once per channel for a plan of the same grid, spectral
 * grid, pupil counts and batch.  atm_run_channel is atm_run with that state in
 * place of the plan's own; it computes on the host nothing and copies
 * nothing, so runs of many channels on one plan can be captured into one
 * CUDA graph (the mixed workload runs as one graph launch).  Results equal
 * those of a plan created (or re-targeted) for the channel.  A channel must
 * outlive the runs that use it; atm_channel_create and atm_channel_destroy
 * synchronise the device.  Replaces building a Channel per parameter point of
 * a mixed workload (channels.py:17-29). */
typedef struct AtmChannel AtmChannel;
int atm_channel_create(AtmPlan* plan, const AtmChannelDesc* desc, AtmChannel** channel);
int atm_channel_destroy(AtmChannel* channel);
int atm_run_channel(AtmPlan* plan, AtmChannel* channel, const float* rho, const float* theta, const void* value,
                    int32_t batch, double* measures_out, void* field_out, float* mean_intensity, void* stream);

/* Seeded spectra on the device: rho, theta [batch][n][P] float32 and value
 * [batch][n][P] complex64 for realisations first_realisation .. +batch-1,
 * drawn with a counter-based Philox4x32-10 generator keyed by `seed` (one
 * uniform per screen for the annulus radii, per annulus a uniform angle and
 * two normals) and formed with the reference's formulas (grids.py:98-107,
 * phase_screens.py:98-103); sqrt_psd [n][P] (device) holds sqrt of each
 * screen's annulus weights.  The stream of numbers differs from numpy's:
 * use host-drawn spectra where realisations must match the reference. */
int atm_draw_spectra(AtmPlan* plan, uint64_t seed, uint64_t first_realisation, const float* sqrt_psd,
                     int32_t batch, float* rho, float* theta, void* value, void* stream);

/* atm_draw_spectra for a channel table set: n is the channel's screen count
 * (not the plan's), so sqrt_psd is [n][P] and the outputs [batch][n][P] in the
 * layout atm_run_channel reads.  Replaces the draws of each screen's
 * _get_spectrum for one parameter point of a mixed workload
 * (phase_screens.py:93-106). */
int atm_channel_draw_spectra(AtmPlan* plan, AtmChannel* channel, uint64_t seed, uint64_t first_realisation,
                             const float* sqrt_psd, int32_t batch, float* rho, float* theta, void* value,
                             void* stream);

/* ---- PDT surrogate MLP (no reference counterpart: the learned part of the
 * engine; it answers PDTResult-style queries, simulations/pdt.py:11-66,
 * without running the channel).  widths[0..n_layers]; hidden layers use
 * GELU; BF16 weights in the GEMMs, FP32 accumulation, FP32 master weights
 * for Adam.  Arrays passed to forward / loss / backward / infer are device
 * arrays; parameters are packed W0 [w1][w0], b0 [w1], W1, b1, ... */
typedef struct AtmMlp AtmMlp;
int atm_mlp_create(int32_t n_layers, const int32_t* widths, int32_t max_batch, AtmMlp** mlp);
int atm_mlp_destroy(AtmMlp* mlp);
int64_t atm_mlp_num_params(const AtmMlp* mlp);
int atm_mlp_set_params(AtmMlp* mlp, const float* host_params);
int atm_mlp_get_params(AtmMlp* mlp, float* host_params, float* host_grads);
int atm_mlp_forward(AtmMlp* mlp, const float* x, int32_t batch, float* y, void* stream);
int atm_mlp_loss(AtmMlp* mlp, const float* target, int32_t batch, int32_t n_hist, float w_mse, double* loss_out,
                 float* dy, void* stream);
int atm_mlp_backward(AtmMlp* mlp, const float* dy, int32_t batch, float* grads, void* stream);
int atm_mlp_adam(AtmMlp* mlp, float lr, float beta1, float beta2, float eps, float weight_decay, int32_t step,
                 void* stream);
/* Inference: y [batch][out] with a softmax over the first n_hist outputs;
 * out_of_range[b] = 1 where an input leaves [lo, hi] (lo, hi NULL: no check).
 * Where the shape allows it (<= 32 inputs, equal hidden widths that are a
 * multiple of 64 and <= 256, <= 128 outputs) it runs as one fused kernel on
 * the tensor cores: tcgen05 BF16 MMAs with FP32 accumulation in TMEM, the
 * activations kept on chip as BF16, the inputs as two BF16 slices (about
 * 16 bits); any batch in one launch.  Otherwise (or after
 * atm_mlp_set_infer_form(mlp, 1)) the tile-GEMM form of atm_mlp_forward with
 * FP32 activations runs, max_batch queries per launch sequence. */
int atm_mlp_infer(AtmMlp* mlp, const float* x, int32_t batch, const float* lo, const float* hi, int32_t n_hist,
                  float* y, int32_t* out_of_range, void* stream);
/* 0: the tensor-core form where the shape allows it (default), 1: the tile-GEMM
 * form, 2: the tensor-core form (ATM_ERR_UNSUPPORTED if the shape does not allow it). */
int atm_mlp_set_infer_form(AtmMlp* mlp, int32_t form);
/* The form atm_mlp_infer runs: 1 tile GEMM, 2 tensor cores (or an error code). */
int atm_mlp_infer_form(const AtmMlp* mlp);
/* Synchronises the device and reports (then clears) a bounded wait of the
 * tensor-core inference that ran out: ATM_ERR_TIMEOUT, else ATM_OK. */
int atm_mlp_check(AtmMlp* mlp);

/* Unit-test entry point of the tensor-core screen GEMM: out[s][m][n] =
 * scale * sum_k A[s][m][k] B[s][n][k] for FP32 device arrays (row stride K),
 * computed with tcgen05 MMAs on FP16 hi/lo slices; M % 128 == 0,
 * N % 256 == 0.  variant 0: persistent TMA form (128 x 128 tiles), 1: cp.async
 * form, 2: persistent TMA form with 128 x 256 tiles.
 * Allocates its slice scratch; synchronises the stream.  No reference
 * counterpart (the reference's screen product is a cupy/numpy complex GEMM,
 * phase_screens.py:125-126). */
int atm_tc_gemm_test(const float* A, const float* B, int32_t S, int32_t M, int32_t N, int32_t K, float scale,
                     float* out, int32_t variant, void* stream);

/* Times the launch variants of the FFT passes on this plan's own workspace
 * (`batch` realisations, `repeats` timed launches each after one warm-up)
 * and keeps the fastest: row-pass variant (0..4 and 7; a tiled plan: 5, 6, 8, 9, 10),
 * column tile (2..16 columns, at most 512 threads per CTA; a tiled plan: 4)
 * and column-pass variant (0..4 and 7; a tiled plan: 5, 6, 8, 9).  The forms
 * that build twiddles as products of powers of two (row 4, 6..10; column
 * 2, 7, 8, 9) round differently from the table forms (FP32 round-off, well
 * inside the 1e-4 field bound); the results are otherwise the same.  Overwrites the
 * plan's field / screen workspace (zeroes) and blocks until the timing
 * launches finish, so it is called outside CUDA-graph capture, before the
 * runs it tunes.  The reference has no tuner: cupy picks cuFFT plans inside
 * the FFT calls of utils.py:42-50 (the boundary item atm_autotune). */
int atm_autotune(AtmPlan* plan, int32_t batch, int32_t repeats, void* stream);

/* Phase structure function of `batch` screens phi [batch][N][N] (float32,
 * device) along x, averaged over rows: sf_out[b][r - 1] = (1/N) sum_y
 * (1/(N - r)) sum_{x < N - r} (phi[b][y][x] - phi[b][y][x + r])^2 for
 * r = 1 .. N - 1 (FP64, device).  Replaces calculate_sf
 * (theory/phase_screens/sf.py:4-8) followed by the row mean of
 * calculate_structure_function (simulations/structure_function.py:11-12). */
int atm_structure_function(const float* phi, int32_t batch, int32_t N, double* sf_out, void* stream);

/* Sets the launch choices atm_autotune makes by hand: row-pass variant 0..4
 * or 7, column tile 2/4/8/16 with at most 512 threads per CTA, column-pass
 * variant 0..4 or 7; at N = 1024 and 2048 also row 11, and at N = 1024, 2048
 * and 4096 column 10, at N = 4096 column 14 and at N = 2048 column 15 (recorded with column tile 4),
 * the warp-FFT forms; a tiled plan (ATM_FLAG_TILED) takes row
 * 5, 6, 8, 9 or 10, column tile 4 and column 5, 6, 8 or 9 (and 13 at N = 1024
 * and 2048).  Results do not
 * change, except for FP32 round-off between the table-twiddle,
 * product-twiddle and warp-FFT forms.  No reference counterpart. */
int atm_plan_set_variants(AtmPlan* plan, int32_t row_variant, int32_t col_tile, int32_t col_variant);

/* Launch categories reported by atm_profile_end. */
#define ATM_KIND_SCREEN_PREP 0
#define ATM_KIND_SCREEN_TABLE 1
#define ATM_KIND_SCREEN_GEMM 2
#define ATM_KIND_ROW_PASS 3
#define ATM_KIND_COL_PASS 4
#define ATM_KIND_FINALIZE 5
#define ATM_KIND_TRACKED 6
#define ATM_KIND_SCREEN_EVAL 7
#define ATM_KIND_COUNT 8

/* Starts recording a CUDA event pair around each kernel launch of this plan
 * (at most max_launches launches), on the stream the kernel runs on.  No
 * reference counterpart: this is the engine's own per-kernel timer. */
int atm_profile_begin(AtmPlan* plan, int32_t max_launches);

/* Waits for the recorded launches and returns, per ATM_KIND_*, the summed
 * device milliseconds and the number of launches; stops recording. */
int atm_profile_end(AtmPlan* plan, double* ms_by_kind, int32_t* launches_by_kind, int32_t n_kinds);

/* FP32 FMA throughput probe: runs `blocks` x 256 threads of independent FMA
 * chains (`iters` iterations of 8 chains) on `stream` and returns the device
 * time in *ms; FLOPs = blocks * 256 * iters * 16.  No reference counterpart:
 * the roofline denominator for the FP32 screen GEMM. */
int atm_fma_probe(int32_t blocks, int32_t iters, double* ms, void* stream);

/* Waits for the plan's work on `stream` and reports what its kernels
 * recorded since the last check: ATM_ERR_TIMEOUT if a bounded device wait ran
 * out (a TMA-fed FFT pass or the tensor-core GEMM; the CTA drained its copies
 * and MMAs, freed its TMEM and returned), ATM_ERR_NONFINITE if a spectrum
 * value was NaN or infinite (the term was dropped).  Either way the runs since
 * the last check wrote NaN measures (the canary for callers that do not
 * check), and the call clears the record.  The reference has no counterpart:
 * its only failure handling is the KeyboardInterrupt flush of
 * Simulation.run (simulations/simulation.py:135-138). */
int atm_plan_check(AtmPlan* plan, void* stream);

/* Budget in ns (default 2e9) of the device waits for work in the FFT passes
 * and the screen GEMM on the current device: a tile or operand stage that has
 * not landed, a stage or accumulator not yet released.  The waits that drain
 * copies and MMAs before a CTA leaves keep their 2 s bound.  A budget far
 * below a kernel's latency makes the waits run out: the failure path that
 * atm_plan_check reports.  No reference counterpart. */
int atm_set_wait_budget(uint64_t ns);

/* Allocation-free variant of atm_vacuum, for callers that cannot allocate
 * device memory where they propagate (their framework's caching allocator
 * owns the memory budget, or they cannot afford cudaFree's implicit device
 * synchronisation).  No counterpart in the reference: it exists for such
 * callers of this library.  One vacuum step of length dz, in place on the
 * caller's spatial field [batch][N][N] complex64 (device), for a grid of
 * step `delta` and wavelength `wvl`; dz <= 0 leaves the field unchanged.
 * Needs no plan and calls no cudaMalloc / cudaFree: its tables live in one
 * static device array of 3 x 4096 complex64 (96 KiB) held by every GPU that
 * loads the library, so N must be a power of two in [128, 4096] (larger N:
 * ATM_ERR_UNSUPPORTED).  The first call on a device looks up that array's
 * address (cudaGetSymbolAddress, once per device); make it before capturing
 * any stream, and do not reset the device while the library is loaded (the
 * address is kept for the life of the process).  All calls share the array:
 * calls whose GPU work overlaps (unordered streams) race on it. */
int atm_vacuum_noalloc(void* field, int32_t N, int32_t batch, double delta, double wvl, double dz,
                       void* stream);

#ifdef __cplusplus
}
#endif

#endif /* ATM_H */
