// Structures shared by the kernels (atm_kernels.cu) and the plan / C-ABI
// layer (atm_abi.cu).  Not part of the public interface (include/atm.h).
#pragma once

#include <cstdint>
#include <cuda_fp16.h>
#include <cuda_runtime.h>

namespace atm {

// row-pass flags
enum : int {
  ROW_GEN = 1,      // generate the row from the separable tables ay[y] * ax[x]
  ROW_INV = 2,      // inverse row FFT first (input in the row-frequency domain)
  ROW_PHASOR = 4,   // multiply by the screen phasor Py[y] Px[x] exp(-i phi[y,x]) * loss
  ROW_FWD = 8,      // forward row FFT after the multiply
  ROW_STORE = 16,   // write the row back
  ROW_MEAS = 32,    // accumulate the measure partial sums (spatial domain)
  ROW_FOLDED = 64,  // phi already holds the 1-D phases in turns: the phasor is exp(-2 pi i phi) * loss
  ROW_STEP = 128,   // measure partial sums of the field just after the screen (per-step measures)
};

constexpr int kMaxPupils = 8;

// bits of a plan's device status word (atm_plan_check reads and clears it;
// while it is non-zero, finalize writes NaN measures)
enum : int {
  STATUS_PASS_WAIT = 1,   // an FFT pass gave up waiting for a staged tile or a free stage
  STATUS_GEMM_WAIT = 2,   // the tensor-core screen GEMM gave up waiting
  STATUS_NONFINITE = 4,   // a spectrum value (rho, theta or value) was NaN or infinite
};
// measure slots accumulated by the last row pass (before the delta^2 scale)
enum : int {
  MS_I = 0, MS_IX, MS_IMY, MS_IX2, MS_IMXY, MS_IY2, MS_PUPIL0,
};
// per-realisation output layout (doubles)
enum : int {
  MO_ETA_TOTAL = 0, MO_MEAN_X, MO_MEAN_Y, MO_MEAN_X2, MO_MEAN_XY, MO_MEAN_Y2,
  MO_MEAN_X2_R, MO_I_CENTER, MO_PUPIL0,
};

struct RowArgs {
  float2* field;            // [B][N][N]
  const float2* tw;         // exp(-2 pi i n / N), n < N
  const float2* ay;         // [N] (ROW_GEN)
  const float2* ax;         // [N] (ROW_GEN)
  const float2* Py;         // [B][N] screen phasor, rows
  const float2* Px;         // [B][N] screen phasor, columns
  const float* phi;         // [B][N][N] screen GEMM part
  float loss;               // amplitude factor of this step
  double* partials;         // [B][gridDim.x][n_meas]
  float* center;            // [B] intensity at the grid origin
  const int2* pupil_rows;   // [n_pupils][N] inclusive column interval per row
  float* mean_I;            // [N][N] intensity accumulator (nullable)
  float* intensity;         // [B][N][N] stored intensity (nullable)
  float2* out;              // [B][N][N] destination of ROW_STORE when store_out != 0
  int store_out;
  int n_pupils;
  int n_meas;
  int flags;
  float delta;
  double delta64;
  double* step_partials;    // [B][gridDim.x][6] partials of the post-screen field (ROW_STEP)
  float* step_center;       // [B] post-screen intensity at the grid origin (ROW_STEP)
  int variant;              // 0: persistent cp.async pipeline when aligned, 1: one CTA per row block,
                            // 2: persistent pipeline with one row per CTA (row blocks of several rows otherwise),
                            // 3: as 2 with the rows moved by bulk copies (TMA) from one thread,
                            // 4: as 3 with twiddles formed from powers of two (fewer shared loads),
                            // 5: four rows (one block row of the tiled layout) per CTA, each row's warps
                            //    synchronising on their own named barrier; 6: as 5 with product twiddles
  int tiled;                // variants 5 / 6: TILE_IN = field read in the tiled layout, TILE_OUT = field
                            // (not `out`) written in the tiled layout; row-major otherwise
  int* status;              // plan status word (nullable): STATUS_PASS_WAIT on a wait that runs out
};

// Tiled field layout: 4 x 4 blocks of complex64 (128 bytes), block rows of
// 4 N elements contiguous.  A column pass then moves whole 128-byte lines,
// and a block row is contiguous for the row pass.
enum : int { TILE_IN = 1, TILE_OUT = 2 };
__host__ __device__ inline size_t tiled_index(int N, int y, int x) {
  return (size_t)(y >> 2) * (size_t)(4 * N) + (size_t)(x >> 2) * 16 + (size_t)((y & 3) * 4 + (x & 3));
}
// N with a tiled form of the passes (4 rows of N/16 threads per CTA, three FFT stages)
inline bool tiled_supported(int N) { return N == 512 || N == 1024 || N == 2048; }

struct ColArgs {
  float2* field;            // [B][N][N]
  const float2* tw;
  const float2* hy;         // [N] transfer function along y incl. exp(i k dz) / N^2
  const float2* hx;         // [N] transfer function along x
  int inv_only;             // 1: inverse column FFT only (no forward FFT, no H)
  int variant;              // 0: persistent cp.async pipeline when aligned, 1: one CTA per column tile,
                            // 2: persistent pipeline with twiddles from powers of two (fewer shared loads),
                            // 3: persistent, tiles loaded by TMA (one thread) so loads overlap the FFTs,
                            // 4: as 3 with alternating exchange buffers,
                            // 5: as 4 on the tiled layout (one block column of 4 columns per item,
                            //    whole 128-byte lines in and out),
                            // 6: tiled layout with one independent thread group per column and a TMA
                            //    producer / store warp
  int* status;              // plan status word (nullable): STATUS_PASS_WAIT on a wait that runs out
};

// FFT screen (phase_screens.py:42-67) without shifts: screen[y][x] =
// (-1)^(x+y) IFFT2((-1)^(kx+ky) cn) + sum_j X_j[x] Y_j[y] - mean
struct FftScreenArgs {
  const float* normals;     // [B][2][N][N] real / imaginary standard normals (main grid)
  const float* amp;         // [N][N] sqrt(Phi_phi(|f|)) 2 pi df, centred order, DC = 0
  const float2* sub_x;      // [B][n_sub][N] subharmonic x factors (FP64-computed)
  const float2* sub_y;      // [B][n_sub][N] subharmonic y factors
  const double* sub_mean;   // [B][2] mean of the subharmonic part (re, im)
  int n_sub, N;
  float2* field;            // [B][N][N] workspace
  float2* out;              // [B][N][N] complex screen (when phi is null)
  float* phi;               // [B][N][N] the screen's real part in turns (Re / 2 pi), or null
  size_t nrm_stride;        // floats between realisations in normals (2 N^2 for one screen each)
  size_t sub_stride;        // float2 between realisations in sub_x / sub_y (n_sub N for one screen each)
  int mean_stride;          // doubles between realisations in sub_mean (2 for one screen each)
};

// one high-frequency spectral term, phases as 64-bit binary fractions of a turn
struct HighTerm {
  uint64_t sx, ox;          // x phase: turns = j * sx + ox  (mod 1)
  uint64_t sy, oy;          // y phase
  float2 v;                 // complex amplitude
  float2 pad_;
};

struct ScreenArgs {
  const float* rho;         // [B][n][P]
  const float* theta;       // [B][n][P]
  const float2* value;      // [B][n][P]
  int n_screens, screen, P;
  int N;
  double delta, sx, sy;     // grid step and screen shift
  int P_L;                  // annuli collapsed into the Chebyshev block
  int D;                    // Chebyshev terms 0..D-1
  int P_H;                  // high-frequency terms = P - P_L
  int KH;                   // GEMM rows of the high part (2 P_H padded)
  int KC;                   // GEMM rows of the Chebyshev part (D-1 padded)
  HighTerm* hterms;         // [B][KH/2]
  float2* Py;               // [B][N]
  float2* Px;               // [B][N]
  float* At;                // [B][KH][N]  A^T, high part (per screen)
  float* Bt;                // [B][KH+KC][N]
  double* Gy;               // [B][N] FP64 phase of the y-only part (nullable)
  double* Hx;               // [B][N] FP64 phase of the x-only part (nullable)
  // tensor-core layout (K-major FP16 hi/lo slices, [B][N][Kp]); null: FP32 SIMT layout
  __half* ta_hi;
  __half* ta_lo;
  __half* tb_hi;
  __half* tb_lo;
  int Kp;                   // padded K of the tensor-core layout
  int kc0;                  // first Chebyshev column (2 P_H)
  float* gy_t;              // [B][N] y-only phase in turns reduced to [-1/2, 1/2] (nullable)
  float* hx_t;              // [B][N] x-only phase in turns reduced to [-1/2, 1/2] (nullable)
  float2* s_int;            // [B][chunks][(D-1)^2] FP32 chunk sums of the Chebyshev interior
  double2* s_edge;          // [B][chunks][2D-1] FP64 chunk sums of its edge row / column
  int* status;              // plan status word (nullable): STATUS_NONFINITE on a NaN / infinite spectrum value
};

// GEMM: phi[s][y][x] = sum_k At[s][k][y] B[s][k][x], k < KH from At, then the
// shared Chebyshev rows Ach[k-KH][y]
struct GemmArgs {
  const float* At;          // [B][KH][N]
  const float* Ach;         // [KC][N]
  const float* Bt;          // [B][KH+KC][N]
  float* phi;               // [B][N][N]
  int N, KH, KC;
};

struct FinalArgs {
  const double* partials;   // [B][n_parts][n_meas]
  const float* center;      // [B]
  double* out;              // [B][n_out]
  int n_parts, n_meas, n_out, n_pupils;
  double delta;
  const int* status;        // plan status word (nullable): non-zero -> NaN measures
};

struct TrackedArgs {
  const float* intensity;   // [B][N][N]
  double* out;              // [B][n_out] (reads mean_x/mean_y, writes tracked etas)
  const double* radii;      // [n_tracked]
  int n_tracked, n_out, slot0, N;
  double delta;
  const int* status;        // plan status word (nullable): non-zero -> NaN
};

// kernel launchers (atm_kernels.cu); return cudaGetLastError()
cudaError_t launch_row_pass(int N, int B, const RowArgs& a, cudaStream_t st);
cudaError_t launch_col_pass(int N, int B, int col_tile, const ColArgs& a, cudaStream_t st);
cudaError_t launch_screen_terms(int B, const ScreenArgs& a, cudaStream_t st);
cudaError_t launch_screen_eval(int B, const ScreenArgs& a, cudaStream_t st);
cudaError_t launch_screen_table(int B, const ScreenArgs& a, cudaStream_t st);
cudaError_t launch_screen_gemm(int B, const GemmArgs& a, cudaStream_t st);
cudaError_t launch_compose_screen(int B, int N, const double* Gy, const double* Hx, const float* phiG,
                                  const float2* Py, const float2* Px, float* phi_out, float2* phasor_out,
                                  cudaStream_t st);
cudaError_t launch_fft_screen_spectrum(int B, const FftScreenArgs& a, cudaStream_t st);
cudaError_t launch_fft_screen_finish(int B, const FftScreenArgs& a, cudaStream_t st);
cudaError_t launch_finalize(int B, const FinalArgs& a, cudaStream_t st);
cudaError_t launch_tracked(int B, const TrackedArgs& a, cudaStream_t st);
cudaError_t launch_fma_probe(int blocks, int iters, cudaStream_t st);
cudaError_t launch_structure_function(const float* phi, int B, int N, double* out, cudaStream_t st);
cudaError_t launch_draw_spectra(uint64_t seed, uint64_t first, int n, int P, const float* fbase, const float* sqrt_psd,
                                int B, float* rho, float* theta, float2* value, cudaStream_t st);
int row_pass_rows(int N);          // rows per CTA of the row pass
int col_tile_default(int N);
bool supported_n(int N);
__host__ __device__ int prep_chunks(int P_L);
// FP16 slices of the tensor-core operands: a = hi + lo / kTcLoScale with
// hi = fp16(a), lo = fp16((a - hi) * kTcLoScale); the scale keeps the
// residual in FP16's normal range
constexpr float kTcLoScale = 2048.0f;
size_t tc_smem_bytes();
// TMA descriptors of one GEMM's operands ([S][M][Kp] and [S][Nn][Kp] FP16
// slices), encoded once on the host; null when the driver offers no encoder
struct TcPlan;
TcPlan* tc_plan_create(int S, int M, int Nn, int Kp, const __half* a_hi, const __half* a_lo, const __half* b_hi,
                       const __half* b_lo, int tn);  // tn: output tile width 256 or 128
void tc_plan_destroy(TcPlan* p);
// tensor map (128-byte storage of a CUtensorMap) of a complex64 field [B][N][N]
// in boxes of C columns x box_rows rows; false without an encoder or alignment
bool encode_field_tiles(void* map, const float2* field, int N, int B, int C, int box_rows);
bool encode_tiled_cols_plain(void* map, const float2* field, int N, int B, int box_blocks);
// tensor maps of a tiled field [B][N][N] (128-byte blocks, 128-byte swizzle):
// by_rows: 3-D {32, N^2/16, B}, consecutive blocks of a block row (boxes of box_blocks blocks);
// otherwise 3-D, one block column (boxes of box_blocks blocks down the column)
bool encode_tiled_field(void* map, const float2* field, int N, int B, bool by_rows, int box_blocks);
// tensor map of a tiled field [B][N][N] as {32 floats of a block, N^2/16 blocks, B} with boxes
// of 8 floats (one row's 4 complex64 of a block) x box_blocks blocks, no swizzle: one row of a
// block row per copy, landing as that row in row-major order
bool encode_tiled_rows(void* map, const float2* field, int N, int B, int box_blocks);
// fold_y [S][M] / fold_x [S][Nn] (nullable, turns): added to every output
cudaError_t launch_tc_gemm_tma(const TcPlan* p, int S, float* out, float scale, const float* fold_y,
                               const float* fold_x, int* status, cudaStream_t st);
// budget (ns) of the waits for work in the pass kernels / the tensor-core GEMM
// on the current device; the waits that drain copies keep their 2 s bound
cudaError_t set_pass_wait_budget(unsigned long long ns);
cudaError_t set_tc_wait_budget(unsigned long long ns);
// reads (and with reset, clears) the device-wide error word of the pass kernels
cudaError_t pass_error_flag(int* host_flag, bool reset);
cudaError_t launch_tc_gemm(int S, int M, int Nn, int Kp, const __half* a_hi, const __half* a_lo, const __half* b_hi,
                           const __half* b_lo, float* out, float scale, cudaStream_t st);
cudaError_t launch_screen_table_tc(int B, const ScreenArgs& a, cudaStream_t st);
cudaError_t launch_cheb_cols_tc(int B, int N, int Kp, int kc0, int D, const float* Ach, __half* hi, __half* lo,
                                cudaStream_t st);
cudaError_t tc_error_flag(int* host_flag, bool reset);
// fused tensor-core inference of the surrogate MLP: a packed BF16 weight
// image in pieces of <= 128 output rows, laid out as the MMAs read them
// (K blocks of 64, rows of 128 bytes, 16-byte chunk c of row r at c ^ (r % 8))
constexpr int kMlpMaxPieces = 16;
constexpr int kMlpMaxLayers = 8;
struct MlpPiece {
  uint32_t src;     // byte offset of the piece in the image
  uint32_t bytes;   // rows x K blocks x 128
  int32_t layer;    // the piece holds output rows [col0, col0 + rows) of this layer
  int32_t rows;     // a multiple of 16, <= 128
  int32_t col0;     // first output row = first TMEM column of the accumulator
  int32_t k_steps;  // MMAs of K = 16
};
struct MlpTcArgs {
  const float* x;    // [batch][in] FP32 inputs
  float* y;          // [batch][out]: softmax over the first n_hist outputs, the rest raw
  int* oor;          // [batch] 1 where an input leaves [lo, hi]; null: no check
  const float* lo;   // [in] or null
  const float* hi;
  const unsigned char* img;
  const float* bias[kMlpMaxLayers];
  int batch, in, k0, hidden, out, out_pad, layers, n_hist, n_pieces;
  int* status;       // STATUS_GEMM_WAIT on a wait that ran out
  MlpPiece pieces[kMlpMaxPieces];
};
cudaError_t launch_mlp_infer_tc(const MlpTcArgs& a, cudaStream_t st);
// records the message returned by atm_last_error() on this host thread; returns code
int set_error(int code, const char* fmt, ...);

}  // namespace atm
