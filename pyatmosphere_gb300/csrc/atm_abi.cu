// Plan construction and the extern "C" entry points of libatm.so
// (declared in include/atm.h).
#include <algorithm>
#include <cmath>
#include <complex>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/atm.h"
#include "atm_common.cuh"
#include "atm_internal.h"

using cd = std::complex<double>;

namespace {

thread_local std::string g_err;

int fail(int code, const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  g_err = buf;
  return code;
}

#define ATM_CUDA(call)                                                                       \
  do {                                                                                       \
    cudaError_t e_ = (call);                                                                 \
    if (e_ != cudaSuccess)                                                                   \
      return fail(ATM_ERR_CUDA, "%s failed: %s (%s:%d)", #call, cudaGetErrorString(e_), __FILE__, \
                  __LINE__);                                                                 \
  } while (0)

constexpr double kPi = 3.14159265358979323846;

// iterative radix-2 FFT, FP64, twiddles from std::polar (no recurrence)
void fft_host(std::vector<cd>& a, int sign) {
  const int n = (int)a.size();
  for (int i = 1, j = 0; i < n; ++i) {
    int bit = n >> 1;
    for (; j & bit; bit >>= 1) j ^= bit;
    j ^= bit;
    if (i < j) std::swap(a[i], a[j]);
  }
  for (int len = 2; len <= n; len <<= 1) {
    const double ang = sign * 2.0 * kPi / len;
    for (int k = 0; k < len / 2; ++k) {
      const cd w = std::polar(1.0, ang * k);
      for (int i = 0; i < n; i += len) {
        const cd u = a[i + k], v = a[i + k + len / 2] * w;
        a[i + k] = u + v;
        a[i + k + len / 2] = u - v;
      }
    }
  }
}

// exp(-i pi dz lambda f^2) on the unshifted frequency axis f_k = k df
// (k - N for k >= N/2), df = 1/(N delta), as theory/vacuum.py:7 evaluates it
// (argument ((pi dz) (2 pi / k)) f^2 in FP64)
std::vector<cd> transfer_1d(int N, double delta, double kw, double dz) {
  std::vector<cd> h(N);
  const double df = 1.0 / (N * delta);
  const double c1 = (kPi * dz) * (2.0 * kPi / kw);
  for (int k = 0; k < N; ++k) {
    const double f = (double)(k < N / 2 ? k : k - N) * df;
    const double arg = c1 * (f * f);
    h[k] = cd(std::cos(arg), -std::sin(arg));
  }
  return h;
}

cd global_phase(double kw, double dz) {
  const double ph = kw * dz;
  return cd(std::cos(ph), std::sin(ph));
}

struct DevBuf {
  void* p = nullptr;
  size_t bytes = 0;
};

int dev_alloc(DevBuf& b, size_t bytes, std::vector<DevBuf*>& all) {
  b.bytes = bytes;
  all.push_back(&b);
  if (bytes == 0) return ATM_OK;
  cudaError_t e = cudaMalloc(&b.p, bytes);
  if (e != cudaSuccess) {
    cudaGetLastError();
    return fail(ATM_ERR_NOMEM, "cudaMalloc of %zu bytes failed: %s", bytes, cudaGetErrorString(e));
  }
  return ATM_OK;
}

template <class T>
int upload(DevBuf& b, const std::vector<T>& v) {
  if (v.size() * sizeof(T) > b.bytes) return fail(ATM_ERR_INVALID, "table larger than its device buffer");
  ATM_CUDA(cudaMemcpy(b.p, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice));
  return ATM_OK;
}

std::vector<float2> to_c64(const std::vector<cd>& v) {
  std::vector<float2> o(v.size());
  for (size_t i = 0; i < v.size(); ++i) o[i] = make_float2((float)v[i].real(), (float)v[i].imag());
  return o;
}

}  // namespace

int atm::set_error(int code, const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  g_err = buf;
  return code;
}

namespace {
struct AtmPlanFwd;
}
struct AtmPlan;
namespace {
int check_device(const AtmPlan* pl);
}

struct AtmPlan {
  int device = 0;
  int N = 0, n = 0, P = 0, B = 0, n_pupils = 0, n_tracked = 0;
  int n_alloc = 0;  // screen count the workspace was sized for (atm_plan_update may lower n)
  double delta = 0, wvl = 0, w0 = 0, F0 = 0, length = 0, losses_db = 0, kw = 0, sx = 0, sy = 0;
  int path_output_loss = 0, source_kind = 0, col_tile = 0;
  int row_variant = 0, col_variant = 0, tuned = 0;  // launch choices (atm_autotune)
  bool tiled = false;  // field kept in the tiled layout between passes (ATM_FLAG_TILED)
  int P_L = 0, D = 2, P_H = 0, KH = 0, KC = 0;
  int rows = 1, n_parts = 0, n_meas = 0, n_out = 0;
  std::vector<double> positions, dz;      // dz[0..n]
  std::vector<float> loss;                // per screen amplitude factor
  float final_loss = 1.f;
  std::vector<double> tracked_radius;

  // profiling: event pairs around launches (atm_profile_begin / end)
  std::vector<cudaEvent_t> ev;
  std::vector<int> ev_kind;
  int ev_used = 0, ev_cap = 0;
  bool profiling = false;

  DevBuf field, phi, At, Bt, Ach, ht, Py, Px, Gy, Hx, tw, ay, ax, hy, hx, vac_h, partials, center, pupil_rows,
      intensity, tracked_r, fbase;
  std::vector<float> f_base;
  double cheb_cut = 0.0;
  bool use_tc = false;  // screen GEMM on tensor cores
  int Kp = 0, kc0 = 0;  // tensor-core layout
  DevBuf ta_hi, ta_lo, tb_hi, tb_lo;
  DevBuf s_int, s_edge;  // chunk sums of the low-frequency block
  DevBuf gy_t, hx_t;     // 1-D phases in turns, folded into the GEMM output (TMA form)
  DevBuf step_partials, step_center;  // per-step measures (ATM_FLAG_STEP_MEASURES)
  DevBuf status;                      // device status word (atm::STATUS_*), read by atm_plan_check
  DevBuf scr;                         // FFT-screen workspace (ATM_FLAG_FFT_SCREENS)
  bool step_meas = false;
  int step_slot0 = 0;
  atm::TcPlan* tcp = nullptr;  // TMA descriptors of the screen GEMM (null: cp.async form)
  bool tc_n256 = false;        // the TMA form with 128 x 256 tiles (the default; ATM_FLAG_TC_N128: 128 x 128)
  std::vector<DevBuf*> bufs;
  int64_t bytes() const {
    int64_t s = 0;
    for (auto* b : bufs) s += (int64_t)b->bytes;
    return s;
  }
  ~AtmPlan() {
    atm::tc_plan_destroy(tcp);
    for (auto* b : bufs)
      if (b->p) cudaFree(b->p);
    for (auto e : ev) cudaEventDestroy(e);
  }
};

// the per-channel state of a plan: what atm_plan_update changes (source, path
// geometry, losses, screen shift, pupil radii) and the device tables built
// from it.  An AtmChannel holds one such state, built once; atm_run_channel
// swaps it into the plan for one run.
struct ChannelState {
  int n = 0;
  double wvl = 0, w0 = 0, F0 = 0, length = 0, losses_db = 0, kw = 0, sx = 0, sy = 0;
  int path_output_loss = 0, source_kind = 0;
  std::vector<double> positions, dz, tracked_radius;
  std::vector<float> loss;
  float final_loss = 1.f;
  DevBuf ay, ax, hy, hx, pupil_rows, tracked_r;
};

struct AtmChannel {
  AtmPlan* plan = nullptr;
  ChannelState st;
  ~AtmChannel() {
    for (DevBuf* b : {&st.ay, &st.ax, &st.hy, &st.hx, &st.pupil_rows, &st.tracked_r})
      if (b->p) cudaFree(b->p);
  }
};

namespace {

int plan_tables(AtmPlan* pl, const AtmChannelDesc* d) {
  const int N = pl->N;
  // twiddles exp(-2 pi i n / N)
  std::vector<cd> tw(N);
  for (int i = 0; i < N; ++i) tw[i] = std::polar(1.0, -2.0 * kPi * i / N);
  if (int rc = upload(pl->tw, to_c64(tw))) return rc;

  // source rows g(x_j), x_j = (j - N/2) delta; u0(y, x) = g(y) g(x)
  std::vector<cd> g(N);
  for (int j = 0; j < N; ++j) {
    if (pl->source_kind == ATM_SOURCE_PLANE) {
      g[j] = 1.0;
    } else {
      const double x = (double)(j - N / 2) * pl->delta;
      const cd c(1.0 / (pl->w0 * pl->w0), std::isinf(pl->F0) ? 0.0 : 2.0 * kPi / pl->wvl / 2.0 / pl->F0);
      g[j] = std::pow(2.0 / kPi, 0.25) / std::sqrt(pl->w0) * std::exp(-c * (x * x));
    }
  }
  // first vacuum segment is separable: a = IFFT(h FFT(g))
  std::vector<cd> a = g, b;
  const double dz0 = pl->dz[0];
  cd gph = 1.0;
  if (dz0 > 0) {
    fft_host(a, -1);
    std::vector<cd> h = transfer_1d(N, pl->delta, pl->kw, dz0);
    for (int k = 0; k < N; ++k) a[k] *= h[k] / (double)N;
    fft_host(a, +1);
    gph = global_phase(pl->kw, dz0);
  }
  b = a;
  for (auto& v : a) v *= gph;
  if (int rc = upload(pl->ay, to_c64(a))) return rc;
  if (int rc = upload(pl->ax, to_c64(b))) return rc;

  // transfer functions of the steps after each screen: [n][N] (y incl. phase and 1/N^2)
  std::vector<float2> hyv((size_t)std::max(pl->n, 1) * N, make_float2(0.f, 0.f)), hxv = hyv;
  for (int i = 1; i <= pl->n; ++i) {
    const double dzi = pl->dz[i];
    if (!(dzi > 0)) continue;
    std::vector<cd> h = transfer_1d(N, pl->delta, pl->kw, dzi);
    const cd ph = global_phase(pl->kw, dzi) / ((double)N * (double)N);
    for (int k = 0; k < N; ++k) {
      const cd y = ph * h[k];
      hyv[(size_t)(i - 1) * N + k] = make_float2((float)y.real(), (float)y.imag());
      hxv[(size_t)(i - 1) * N + k] = make_float2((float)h[k].real(), (float)h[k].imag());
    }
  }
  if (int rc = upload(pl->hy, hyv)) return rc;
  if (int rc = upload(pl->hx, hxv)) return rc;

  // Chebyshev rows of A^T: T_e(t_y), e = 1..D-1, padded to KC rows
  if (pl->KC > 0) {
    std::vector<float> ach((size_t)pl->KC * N, 0.f);
    const double half = 0.5 * (N - 1);
    for (int e = 1; e < pl->D; ++e)
      for (int j = 0; j < N; ++j) {
        const double t = std::min(1.0, std::max(-1.0, ((double)j - half) / half));
        ach[(size_t)(e - 1) * N + j] = (float)std::cos(e * std::acos(t));
      }
    if (int rc = upload(pl->Ach, ach)) return rc;
  }

  // pupil masks as inclusive column intervals per row, FP64 predicate
  // (x - sx)^2 + (y + sy)^2 <= R^2 (pupils.py:8-10)
  if (pl->n_pupils > 0) {
    std::vector<int2> rows((size_t)pl->n_pupils * N);
    for (int p = 0; p < pl->n_pupils; ++p) {
      const double R = d->pupil_radius[p];
      const double psx = d->pupil_shift_x ? d->pupil_shift_x[p] : 0.0;
      const double psy = d->pupil_shift_y ? d->pupil_shift_y[p] : 0.0;
      for (int i = 0; i < N; ++i) {
        const double y = (double)(i - N / 2) * pl->delta;
        auto inside = [&](int j) {
          const double x = (double)(j - N / 2) * pl->delta;
          return (x - psx) * (x - psx) + (y + psy) * (y + psy) <= R * R;
        };
        int jc = (int)std::lround(psx / pl->delta) + N / 2;
        jc = std::min(N - 1, std::max(0, jc));
        int2 iv = make_int2(1, 0);
        if (inside(jc)) {
          int lo = 0, hi = jc;  // first inside in [0, jc]
          while (lo < hi) {
            const int m = (lo + hi) / 2;
            if (inside(m)) hi = m; else lo = m + 1;
          }
          iv.x = lo;
          lo = jc;
          hi = N - 1;  // last inside in [jc, N-1]
          while (lo < hi) {
            const int m = (lo + hi + 1) / 2;
            if (inside(m)) lo = m; else hi = m - 1;
          }
          iv.y = lo;
        }
        rows[(size_t)p * N + i] = iv;
      }
    }
    if (int rc = upload(pl->pupil_rows, rows)) return rc;
  }
  if (pl->n_tracked > 0) {
    if (int rc = upload(pl->tracked_r, pl->tracked_radius)) return rc;
  }
  return ATM_OK;
}

int choose_low_block(AtmPlan* pl, const AtmChannelDesc* d) {
  double cut = d->cheb_cut > 0 ? d->cheb_cut : 4.0;
  const double xh = 0.5 * (pl->N - 1) * pl->delta;
  for (int attempt = 0; attempt < 8; ++attempt) {
    const double fcut = cut / (pl->N * pl->delta);
    int PL = 0;
    while (PL < pl->P && (double)d->f_base[PL] <= fcut) ++PL;
    const double amax = 2.0 * kPi * fcut * xh;
    // smallest D with 2 |J_n(amax)| < 1e-10 for all n >= D (checked to D + 16)
    double J[96];
    atm::bessel_j(amax, 96, J);
    int D = 2;
    for (int n = 95; n >= 1; --n)
      if (2.0 * std::fabs(J[n]) >= 1e-10) {
        D = n + 1;
        break;
      }
    D = std::max(D, 2);
    if (D <= 64) {
      pl->P_L = PL;
      pl->D = PL > 0 ? D : 2;
      return ATM_OK;
    }
    cut *= 0.5;
  }
  return fail(ATM_ERR_UNSUPPORTED, "could not fit the low-frequency block into 64 Chebyshev terms");
}

// source / path / loss state that atm_plan_update may change
void set_geometry(AtmPlan* pl, const AtmChannelDesc* d) {
  pl->wvl = d->wvl;
  pl->w0 = d->w0;
  pl->F0 = d->F0;
  pl->length = d->length;
  pl->losses_db = d->losses_db;
  pl->kw = 2.0 * kPi / d->wvl;
  pl->sx = d->shift_x;
  pl->sy = d->shift_y;
  pl->path_output_loss = d->path_output_loss;
  pl->source_kind = d->source_kind;
  pl->tracked_radius.assign(d->tracked_radius, d->tracked_radius + d->n_tracked);
  // steps: dz[0] = z_0, dz[i] = z_i - z_{i-1}, dz[n] = L - z_{n-1} (pathes.py:68-75)
  pl->positions.clear();
  pl->dz.clear();
  if (pl->n > 0) {
    pl->positions.assign(d->positions, d->positions + pl->n);
    pl->dz.push_back(pl->positions[0]);
    for (int i = 1; i < pl->n; ++i) pl->dz.push_back(pl->positions[i] - pl->positions[i - 1]);
    pl->dz.push_back(pl->length - pl->positions[pl->n - 1]);
  } else {
    pl->dz.push_back(pl->length);
  }
  // losses: a step whose share is 0 falls back to the full path loss
  // (append_losses: `losses_db or self.losses_db`, pathes.py:19-21)
  pl->loss.clear();
  for (int i = 0; i < pl->n; ++i) {
    double ld = pl->losses_db * pl->dz[i] / pl->length;
    if (ld == 0.0) ld = pl->losses_db;
    pl->loss.push_back(ld != 0.0 ? (float)std::pow(10.0, -ld / 20.0) : 1.f);
  }
  pl->final_loss = (pl->path_output_loss && pl->losses_db != 0.0) ? (float)std::pow(10.0, -pl->losses_db / 20.0) : 1.f;
}

int validate(const AtmChannelDesc* d) {
  if (!d) return fail(ATM_ERR_INVALID, "descriptor is NULL");
  if (d->abi_version != ATM_ABI_VERSION)
    return fail(ATM_ERR_INVALID, "descriptor abi_version %d, library %d", d->abi_version, ATM_ABI_VERSION);
  if (!atm::supported_n(d->resolution))
    return fail(ATM_ERR_UNSUPPORTED, "resolution %d unsupported: need a power of two in [128, 4096]",
                d->resolution);
  if (!(d->delta > 0)) return fail(ATM_ERR_INVALID, "delta must be > 0");
  if (d->source_kind != ATM_SOURCE_GAUSSIAN && d->source_kind != ATM_SOURCE_PLANE)
    return fail(ATM_ERR_INVALID, "unknown source_kind %d", d->source_kind);
  if (d->source_kind == ATM_SOURCE_GAUSSIAN && !(d->w0 > 0)) return fail(ATM_ERR_INVALID, "w0 must be > 0");
  if (!(d->wvl > 0)) return fail(ATM_ERR_INVALID, "wvl must be > 0");
  if (d->n_screens < 0 || d->n_screens > 256) return fail(ATM_ERR_INVALID, "n_screens %d out of range", d->n_screens);
  if (d->n_screens > 0) {
    if (!d->positions) return fail(ATM_ERR_INVALID, "positions is NULL");
    if (d->points < 1 || !d->f_base) return fail(ATM_ERR_INVALID, "points / f_base missing");
  }
  if (d->n_pupils < 0 || d->n_pupils > ATM_MAX_PUPILS)
    return fail(ATM_ERR_INVALID, "n_pupils %d out of range [0, %d]", d->n_pupils, ATM_MAX_PUPILS);
  if (d->n_pupils > 0 && !d->pupil_radius) return fail(ATM_ERR_INVALID, "pupil_radius is NULL");
  if (d->n_tracked < 0 || d->n_pupils + d->n_tracked > 32) return fail(ATM_ERR_INVALID, "n_tracked out of range");
  if (d->n_tracked > 0 && !d->tracked_radius) return fail(ATM_ERR_INVALID, "tracked_radius is NULL");
  if (d->batch < 1 || d->batch > 65535) return fail(ATM_ERR_INVALID, "batch %d out of range", d->batch);
  return ATM_OK;
}

// exchanges the plan's per-channel state with `c` (device buffers by pointer)
void swap_state(AtmPlan* pl, ChannelState& c) {
  std::swap(pl->n, c.n);
  std::swap(pl->wvl, c.wvl);
  std::swap(pl->w0, c.w0);
  std::swap(pl->F0, c.F0);
  std::swap(pl->length, c.length);
  std::swap(pl->losses_db, c.losses_db);
  std::swap(pl->kw, c.kw);
  std::swap(pl->sx, c.sx);
  std::swap(pl->sy, c.sy);
  std::swap(pl->path_output_loss, c.path_output_loss);
  std::swap(pl->source_kind, c.source_kind);
  std::swap(pl->positions, c.positions);
  std::swap(pl->dz, c.dz);
  std::swap(pl->tracked_radius, c.tracked_radius);
  std::swap(pl->loss, c.loss);
  std::swap(pl->final_loss, c.final_loss);
  std::swap(pl->ay, c.ay);
  std::swap(pl->ax, c.ax);
  std::swap(pl->hy, c.hy);
  std::swap(pl->hx, c.hx);
  std::swap(pl->pupil_rows, c.pupil_rows);
  std::swap(pl->tracked_r, c.tracked_r);
}

// a descriptor the plan can be re-targeted to (atm_plan_update, atm_channel_create)
int check_retarget(const AtmPlan* pl, const AtmChannelDesc* d) {
  if (int rc = validate(d)) return rc;
  if (int rc = check_device(pl)) return rc;
  if (d->resolution != pl->N || d->delta != pl->delta || d->n_pupils != pl->n_pupils ||
      d->n_tracked != pl->n_tracked || d->batch > pl->B || d->cheb_cut != pl->cheb_cut)
    return fail(ATM_ERR_INVALID, "a re-targeted plan keeps grid, pupil counts, batch and cheb_cut");
  if (d->n_screens > pl->n_alloc || (pl->n_alloc > 0) != (d->n_screens > 0))
    return fail(ATM_ERR_INVALID, "a re-targeted plan takes 1..%d screens (the creating descriptor's count)",
                pl->n_alloc);
  if (pl->n_alloc > 0) {
    if (d->points != pl->P) return fail(ATM_ERR_INVALID, "a re-targeted plan keeps the spectral grid");
    for (int p = 0; p < pl->P; ++p)
      if (d->f_base[p] != pl->f_base[p]) return fail(ATM_ERR_INVALID, "a re-targeted plan keeps the spectral grid");
  }
  return ATM_OK;
}

}  // namespace

extern "C" {

int atm_abi_version(void) { return ATM_ABI_VERSION; }

const char* atm_last_error(void) { return g_err.c_str(); }

int atm_plan_create(const AtmChannelDesc* d, AtmPlan** out) {
  if (!out) return fail(ATM_ERR_INVALID, "plan output pointer is NULL");
  *out = nullptr;
  if (int rc = validate(d)) return rc;
  AtmPlan* pl = new AtmPlan();
  cudaGetDevice(&pl->device);
  pl->N = d->resolution;
  pl->n = d->n_screens;
  pl->n_alloc = d->n_screens;
  pl->P = d->n_screens > 0 ? d->points : 0;
  pl->B = d->batch;
  pl->delta = d->delta;
  pl->wvl = d->wvl;
  pl->w0 = d->w0;
  pl->F0 = d->F0;
  pl->length = d->length;
  pl->losses_db = d->losses_db;
  pl->kw = 2.0 * kPi / d->wvl;
  pl->sx = d->shift_x;
  pl->sy = d->shift_y;
  pl->path_output_loss = d->path_output_loss;
  pl->source_kind = d->source_kind;
  pl->n_pupils = d->n_pupils;
  pl->n_tracked = d->n_tracked;
  pl->col_tile = d->col_tile > 0 ? d->col_tile : atm::col_tile_default(pl->N);
  set_geometry(pl, d);

  int rc = ATM_OK;
  if (pl->n > 0) rc = choose_low_block(pl, d);
  if (rc) {
    delete pl;
    return rc;
  }
  pl->P_H = pl->P - pl->P_L;
  pl->KH = ((2 * pl->P_H + 7) / 8) * 8;
  pl->KC = pl->P_L > 0 ? ((pl->D - 1 + 7) / 8) * 8 : 0;
  if (pl->n > 0 && pl->KH + pl->KC == 0) pl->KH = 8;  // keep the GEMM well-formed
  // tensor cores by default for N >= 256 (the GEMM tile is 128 x 256); ATM_FLAG_SIMT_GEMM opts out
  pl->use_tc = pl->n > 0 && pl->N >= 256 && !(d->flags & ATM_FLAG_SIMT_GEMM);
  if (pl->use_tc) {
    pl->kc0 = 2 * pl->P_H;
    const int kraw = pl->kc0 + (pl->P_L > 0 ? pl->D - 1 : 0);
    pl->Kp = std::max(64, (kraw + 63) / 64 * 64);
  }
  // tiled layout: opt-in by flag; the tiled passes write one measure partial per row
  pl->tiled = atm::tiled_supported(pl->N) && (d->flags & ATM_FLAG_TILED) && !(d->flags & ATM_FLAG_ROWMAJOR);
  if (pl->tiled) {
    // one row per CTA (tensor copies of the row's share of each block) and the column
    // groups, both with product twiddles from the table's bases
    pl->row_variant = 9;
    pl->col_variant = 9;
    pl->col_tile = 4;
  }
  pl->rows = pl->tiled ? 1 : atm::row_pass_rows(pl->N);
  pl->n_parts = pl->N / pl->rows;
  pl->n_meas = 6 + pl->n_pupils;
  pl->n_out = ATM_OUT_PUPIL0 + pl->n_pupils + pl->n_tracked;
  pl->step_meas = pl->n > 0 && (d->flags & ATM_FLAG_STEP_MEASURES);
  pl->step_slot0 = pl->n_out;
  if (pl->step_meas) pl->n_out += ATM_STEP_SLOTS * pl->n;

  const size_t N = pl->N, B = pl->B, K = pl->KH + pl->KC;
  const size_t plane = N * N;
  auto& v = pl->bufs;
  if ((rc = dev_alloc(pl->field, B * plane * sizeof(float2), v)) ||
      (rc = dev_alloc(pl->tw, N * sizeof(float2), v)) || (rc = dev_alloc(pl->ay, N * sizeof(float2), v)) ||
      (rc = dev_alloc(pl->ax, N * sizeof(float2), v)) ||
      (rc = dev_alloc(pl->hy, (size_t)std::max(pl->n, 1) * N * sizeof(float2), v)) ||
      (rc = dev_alloc(pl->hx, (size_t)std::max(pl->n, 1) * N * sizeof(float2), v)) ||
      (rc = dev_alloc(pl->vac_h, 2 * N * sizeof(float2), v)) ||
      (rc = dev_alloc(pl->partials, B * pl->n_parts * pl->n_meas * sizeof(double), v)) ||
      (rc = dev_alloc(pl->center, B * sizeof(float), v)) ||
      (rc = dev_alloc(pl->pupil_rows, (size_t)pl->n_pupils * N * sizeof(int2), v)) ||
      (rc = dev_alloc(pl->tracked_r, (size_t)pl->n_tracked * sizeof(double), v)) ||
      (rc = dev_alloc(pl->intensity, pl->n_tracked > 0 ? B * plane * sizeof(float) : 0, v)) ||
      (rc = dev_alloc(pl->step_partials, pl->step_meas ? (size_t)pl->n * B * pl->n_parts * 6 * sizeof(double) : 0, v)) ||
      (rc = dev_alloc(pl->step_center, pl->step_meas ? (size_t)pl->n * B * sizeof(float) : 0, v)) ||
      (rc = dev_alloc(pl->status, sizeof(int), v))) {
    delete pl;
    return rc;
  }
  if (cudaMemset(pl->status.p, 0, sizeof(int)) != cudaSuccess) {
    delete pl;
    return fail(ATM_ERR_CUDA, "cudaMemset of the status word failed");
  }
  if (pl->use_tc) {
    const size_t th = B * N * (size_t)pl->Kp * sizeof(__half);
    if ((rc = dev_alloc(pl->ta_hi, th, v)) || (rc = dev_alloc(pl->ta_lo, th, v)) ||
        (rc = dev_alloc(pl->tb_hi, th, v)) || (rc = dev_alloc(pl->tb_lo, th, v))) {
      delete pl;
      return rc;
    }
    for (DevBuf* b : {&pl->ta_hi, &pl->ta_lo, &pl->tb_hi, &pl->tb_lo}) {
      if (cudaMemset(b->p, 0, b->bytes) != cudaSuccess) {
        delete pl;
        return fail(ATM_ERR_CUDA, "cudaMemset of the tensor-core tables failed");
      }
    }
    if (!(d->flags & ATM_FLAG_TC_CPASYNC))
      pl->tcp = atm::tc_plan_create(pl->B, pl->N, pl->N, pl->Kp, (const __half*)pl->ta_hi.p,
                                    (const __half*)pl->ta_lo.p, (const __half*)pl->tb_hi.p, (const __half*)pl->tb_lo.p,
                                    (d->flags & ATM_FLAG_TC_N128) ? 128 : 256);
    pl->tc_n256 = pl->tcp && !(d->flags & ATM_FLAG_TC_N128);
  }
  if (pl->n > 0) {
    const size_t simt_rows = pl->use_tc ? 0 : 1;  // FP32 SIMT tables only without tensor cores
    if ((rc = dev_alloc(pl->phi, B * plane * sizeof(float), v)) ||
        (rc = dev_alloc(pl->At, simt_rows * B * pl->KH * N * sizeof(float), v)) ||
        (rc = dev_alloc(pl->Bt, simt_rows * B * K * N * sizeof(float), v)) ||
        (rc = dev_alloc(pl->Ach, (size_t)pl->KC * N * sizeof(float), v)) ||
        (rc = dev_alloc(pl->ht, B * (pl->KH / 2) * sizeof(atm::HighTerm), v)) ||
        (rc = dev_alloc(pl->Py, B * N * sizeof(float2), v)) || (rc = dev_alloc(pl->Px, B * N * sizeof(float2), v)) ||
        (rc = dev_alloc(pl->Gy, B * N * sizeof(double), v)) || (rc = dev_alloc(pl->Hx, B * N * sizeof(double), v)) ||
        (rc = dev_alloc(pl->gy_t, B * N * sizeof(float), v)) || (rc = dev_alloc(pl->hx_t, B * N * sizeof(float), v)) ||
        (rc = dev_alloc(pl->s_int, B * atm::prep_chunks(pl->P_L) * (pl->D - 1) * (pl->D - 1) * sizeof(float2), v)) ||
        (rc = dev_alloc(pl->s_edge, B * atm::prep_chunks(pl->P_L) * (2 * pl->D - 1) * sizeof(double2), v))) {
      delete pl;
      return rc;
    }
  }
  if (pl->n > 0 && (d->flags & ATM_FLAG_FFT_SCREENS)) {
    if ((rc = dev_alloc(pl->scr, B * plane * sizeof(float2), v))) {
      delete pl;
      return rc;
    }
  }
  if (pl->n > 0) {
    if ((rc = dev_alloc(pl->fbase, (size_t)pl->P * sizeof(float), v))) {
      delete pl;
      return rc;
    }
    pl->f_base.assign(d->f_base, d->f_base + pl->P);
    if ((rc = upload(pl->fbase, pl->f_base))) {
      delete pl;
      return rc;
    }
  }
  pl->cheb_cut = d->cheb_cut;
  if ((rc = plan_tables(pl, d))) {
    delete pl;
    return rc;
  }
  if (pl->use_tc && pl->P_L > 0) {
    // Chebyshev columns of A are the same for every screen: written once
    cudaError_t e = atm::launch_cheb_cols_tc(pl->B, pl->N, pl->Kp, pl->kc0, pl->D, (const float*)pl->Ach.p,
                                             (__half*)pl->ta_hi.p, (__half*)pl->ta_lo.p, 0);
    if (e == cudaSuccess) e = cudaDeviceSynchronize();
    if (e != cudaSuccess) {
      delete pl;
      return fail(ATM_ERR_CUDA, "Chebyshev columns: %s", cudaGetErrorString(e));
    }
  }
  *out = pl;
  return ATM_OK;
}

int atm_plan_update(AtmPlan* pl, const AtmChannelDesc* d) {
  if (!pl) return fail(ATM_ERR_INVALID, "plan is NULL");
  if (int rc = check_retarget(pl, d)) return rc;
  ATM_CUDA(cudaDeviceSynchronize());  // tables may still be read by enqueued work
  pl->n = d->n_screens;
  set_geometry(pl, d);
  return plan_tables(pl, d);
}

int atm_channel_create(AtmPlan* pl, const AtmChannelDesc* d, AtmChannel** out) {
  if (!out) return fail(ATM_ERR_INVALID, "channel output pointer is NULL");
  *out = nullptr;
  if (!pl) return fail(ATM_ERR_INVALID, "plan is NULL");
  if (int rc = check_retarget(pl, d)) return rc;
  auto* ch = new AtmChannel();
  ch->plan = pl;
  std::vector<DevBuf*> owned;  // the channel frees its own buffers
  ChannelState& c = ch->st;
  int rc = dev_alloc(c.ay, pl->ay.bytes, owned);
  if (!rc) rc = dev_alloc(c.ax, pl->ax.bytes, owned);
  if (!rc) rc = dev_alloc(c.hy, pl->hy.bytes, owned);
  if (!rc) rc = dev_alloc(c.hx, pl->hx.bytes, owned);
  if (!rc) rc = dev_alloc(c.pupil_rows, pl->pupil_rows.bytes, owned);
  if (!rc) rc = dev_alloc(c.tracked_r, pl->tracked_r.bytes, owned);
  if (!rc && cudaDeviceSynchronize() != cudaSuccess) rc = fail(ATM_ERR_CUDA, "cudaDeviceSynchronize failed");
  if (!rc) {
    // build the channel's tables in the plan's place, then give the plan its own state back
    swap_state(pl, c);
    pl->n = d->n_screens;
    set_geometry(pl, d);
    rc = plan_tables(pl, d);
    swap_state(pl, c);
  }
  if (rc) {
    delete ch;
    return rc;
  }
  *out = ch;
  return ATM_OK;
}

int atm_channel_destroy(AtmChannel* ch) {
  if (!ch) return ATM_OK;
  cudaDeviceSynchronize();  // runs may still read its tables
  delete ch;
  return ATM_OK;
}

int atm_plan_destroy(AtmPlan* pl) {
  if (!pl) return ATM_OK;
  cudaDeviceSynchronize();
  delete pl;
  return ATM_OK;
}

int atm_plan_info(const AtmPlan* pl, AtmPlanInfo* info) {
  if (!pl || !info) return fail(ATM_ERR_INVALID, "NULL argument");
  info->n_out = pl->n_out;
  info->low_annuli = pl->P_L;
  info->cheb_terms = pl->D;
  info->gemm_k = pl->use_tc ? pl->Kp : pl->KH + pl->KC;
  info->workspace_bytes = pl->bytes();
  int launches = 0;
  // per screen: terms, eval, table, GEMM, row pass (+ column pass)
  for (int i = 0; i < pl->n; ++i) launches += 5 + (pl->dz[i + 1] > 0 ? 1 : 0);
  launches += (pl->n == 0 || pl->dz[pl->n] > 0) ? 1 : 0;
  launches += 1 + (pl->step_meas ? pl->n : 0);  // finalize (+ one per step)
  info->launches_per_run = launches;
  info->row_parts = pl->n_parts;
  info->col_tile = pl->col_tile;
  info->row_variant = pl->row_variant;
  info->col_variant = pl->col_variant;
  info->tuned = pl->tuned;
  info->gemm_form = pl->n == 0 ? 0 : (!pl->use_tc ? 0 : (pl->tcp ? (pl->tc_n256 ? 3 : 2) : 1));
  info->tiled = pl->tiled ? 1 : 0;
  return ATM_OK;
}

}  // extern "C"

namespace {

// brackets one launch with an event pair when the plan is profiling.  While
// the stream is being captured into a CUDA graph the pair is recorded as
// external event nodes, so that every replay of the graph records it.
struct Prof {
  AtmPlan* pl;
  int kind;
  cudaStream_t st;
  int slot = -1;
  static void record(cudaEvent_t e, cudaStream_t s) {
    cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
    if (cudaStreamIsCapturing(s, &cap) == cudaSuccess && cap == cudaStreamCaptureStatusActive)
      cudaEventRecordWithFlags(e, s, cudaEventRecordExternal);
    else
      cudaEventRecord(e, s);
  }
  Prof(AtmPlan* p, int k, cudaStream_t s) : pl(p), kind(k), st(s) {
    if (pl->profiling && pl->ev_used < pl->ev_cap) {
      slot = pl->ev_used++;
      pl->ev_kind[slot] = kind;
      record(pl->ev[2 * slot], st);
    }
  }
  ~Prof() {
    if (slot >= 0) record(pl->ev[2 * slot + 1], st);
  }
};

atm::ScreenArgs screen_args(AtmPlan* pl, const float* rho, const float* theta, const void* value, int screen) {
  atm::ScreenArgs s{};
  s.rho = rho;
  s.theta = theta;
  s.value = reinterpret_cast<const float2*>(value);
  s.n_screens = pl->n;
  s.screen = screen;
  s.P = pl->P;
  s.N = pl->N;
  s.delta = pl->delta;
  s.sx = pl->sx;
  s.sy = pl->sy;
  s.P_L = pl->P_L;
  s.D = pl->D;
  s.P_H = pl->P_H;
  s.KH = pl->KH;
  s.KC = pl->KC;
  s.hterms = (atm::HighTerm*)pl->ht.p;
  s.status = (int*)pl->status.p;
  s.s_int = (float2*)pl->s_int.p;
  s.s_edge = (double2*)pl->s_edge.p;
  s.Py = (float2*)pl->Py.p;
  s.Px = (float2*)pl->Px.p;
  s.At = (float*)pl->At.p;
  s.Bt = (float*)pl->Bt.p;
  s.Gy = nullptr;
  s.Hx = nullptr;
  if (pl->use_tc) {
    s.ta_hi = (__half*)pl->ta_hi.p;
    s.ta_lo = (__half*)pl->ta_lo.p;
    s.tb_hi = (__half*)pl->tb_hi.p;
    s.tb_lo = (__half*)pl->tb_lo.p;
    s.Kp = pl->Kp;
    s.kc0 = pl->kc0;
  }
  return s;
}

// fold: the GEMM output carries the 1-D phases too (persistent TMA form only);
// the row pass then multiplies by exp(-2 pi i phi) alone
bool folds(const AtmPlan* pl) { return pl->tcp != nullptr; }

int run_screen(AtmPlan* pl, atm::ScreenArgs s, int B, bool fold, cudaStream_t st) {
  fold = fold && folds(pl);
  s.gy_t = fold ? (float*)pl->gy_t.p : nullptr;
  s.hx_t = fold ? (float*)pl->hx_t.p : nullptr;
  {
    Prof p(pl, ATM_KIND_SCREEN_PREP, st);
    ATM_CUDA(atm::launch_screen_terms(B, s, st));
  }
  {
    Prof p(pl, ATM_KIND_SCREEN_EVAL, st);
    ATM_CUDA(atm::launch_screen_eval(B, s, st));
  }
  if (pl->use_tc) {
    {
      Prof p(pl, ATM_KIND_SCREEN_TABLE, st);
      ATM_CUDA(atm::launch_screen_table_tc(B, s, st));
    }
    Prof p(pl, ATM_KIND_SCREEN_GEMM, st);
    constexpr float kInv2Pi = 0.15915494309189533577f;  // phi_G in turns
    if (pl->tcp)
      ATM_CUDA(atm::launch_tc_gemm_tma(pl->tcp, B, (float*)pl->phi.p, kInv2Pi, s.gy_t, s.hx_t, (int*)pl->status.p,
                                       st));
    else
      ATM_CUDA(atm::launch_tc_gemm(B, pl->N, pl->N, pl->Kp, (const __half*)pl->ta_hi.p, (const __half*)pl->ta_lo.p,
                                   (const __half*)pl->tb_hi.p, (const __half*)pl->tb_lo.p, (float*)pl->phi.p, kInv2Pi,
                                   st));
    return ATM_OK;
  }
  if (pl->P_H > 0) {
    Prof p(pl, ATM_KIND_SCREEN_TABLE, st);
    ATM_CUDA(atm::launch_screen_table(B, s, st));
  }
  atm::GemmArgs g{};
  g.At = (const float*)pl->At.p;
  g.Ach = (const float*)pl->Ach.p;
  g.Bt = (const float*)pl->Bt.p;
  g.phi = (float*)pl->phi.p;
  g.N = pl->N;
  g.KH = pl->KH;
  g.KC = pl->KC;
  Prof p(pl, ATM_KIND_SCREEN_GEMM, st);
  ATM_CUDA(atm::launch_screen_gemm(B, g, st));
  return ATM_OK;
}

atm::RowArgs row_args(AtmPlan* pl, float* mean_intensity, void* field_out) {
  atm::RowArgs ra{};
  ra.field = (float2*)pl->field.p;
  ra.tw = (const float2*)pl->tw.p;
  ra.ay = (const float2*)pl->ay.p;
  ra.ax = (const float2*)pl->ax.p;
  ra.Py = (const float2*)pl->Py.p;
  ra.Px = (const float2*)pl->Px.p;
  ra.phi = (const float*)pl->phi.p;
  ra.partials = (double*)pl->partials.p;
  ra.center = (float*)pl->center.p;
  ra.pupil_rows = (const int2*)pl->pupil_rows.p;
  ra.mean_I = mean_intensity;
  ra.intensity = (float*)pl->intensity.p;
  ra.n_pupils = pl->n_pupils;
  ra.n_meas = pl->n_meas;
  ra.delta = (float)pl->delta;
  ra.delta64 = pl->delta;
  ra.out = (float2*)field_out;
  ra.variant = pl->row_variant;
  ra.tiled = pl->tiled ? (atm::TILE_IN | atm::TILE_OUT) : 0;
  ra.status = (int*)pl->status.p;
  return ra;
}

int finish_measures(AtmPlan* pl, int batch, double* measures, cudaStream_t st) {
  atm::FinalArgs fa{};
  fa.partials = (const double*)pl->partials.p;
  fa.center = (const float*)pl->center.p;
  fa.out = measures;
  fa.n_parts = pl->n_parts;
  fa.n_meas = pl->n_meas;
  fa.n_out = pl->n_out;
  fa.n_pupils = pl->n_pupils;
  fa.delta = pl->delta;
  fa.status = (const int*)pl->status.p;
  {
    Prof p(pl, ATM_KIND_FINALIZE, st);
    ATM_CUDA(atm::launch_finalize(batch, fa, st));
  }
  if (pl->n_tracked > 0) {
    Prof p(pl, ATM_KIND_TRACKED, st);
    atm::TrackedArgs ta{};
    ta.intensity = (const float*)pl->intensity.p;
    ta.out = measures;
    ta.radii = (const double*)pl->tracked_r.p;
    ta.n_tracked = pl->n_tracked;
    ta.n_out = pl->n_out;
    ta.slot0 = ATM_OUT_PUPIL0 + pl->n_pupils;
    ta.N = pl->N;
    ta.delta = pl->delta;
    ta.status = (const int*)pl->status.p;
    ATM_CUDA(atm::launch_tracked(batch, ta, st));
  }
  return ATM_OK;
}

// the split-step loop of a run: per screen, make_screen(i) leaves the screen in
// pl->phi (turns; `folded`: the whole phase, else the GEMM part beside Py / Px),
// then the row pass applies it between the vacuum steps' FFTs and the column
// pass the transfer function; the last row pass measures
template <class MakeScreen>
int propagate(AtmPlan* pl, int batch, MakeScreen&& make_screen, bool folded, double* measures, void* field_out,
              float* mean_intensity, cudaStream_t st) {
  const int N = pl->N, n = pl->n;
  atm::RowArgs ra = row_args(pl, mean_intensity, field_out);
  atm::ColArgs ca{};
  ca.field = (float2*)pl->field.p;
  ca.tw = (const float2*)pl->tw.p;
  ca.variant = pl->col_variant;
  ca.status = (int*)pl->status.p;

  bool measured = false;
  for (int i = 0; i < n; ++i) {
    if (int rc = make_screen(i)) return rc;
    int flags = (i == 0 ? atm::ROW_GEN : (pl->dz[i] > 0 ? atm::ROW_INV : 0)) | atm::ROW_PHASOR |
                (folded ? atm::ROW_FOLDED : 0);
    const bool next_vac = pl->dz[i + 1] > 0;
    if (next_vac) {
      flags |= atm::ROW_FWD | atm::ROW_STORE;
    } else if (i == n - 1) {
      flags |= atm::ROW_MEAS | (field_out ? atm::ROW_STORE : 0);
      measured = true;
    } else {
      flags |= atm::ROW_STORE;
    }
    if (pl->step_meas) {
      flags |= atm::ROW_STEP;
      ra.step_partials = (double*)pl->step_partials.p + (size_t)i * pl->B * pl->n_parts * 6;
      ra.step_center = (float*)pl->step_center.p + (size_t)i * pl->B;
    }
    ra.flags = flags;
    ra.loss = pl->loss[i] * ((i == n - 1 && !next_vac) ? pl->final_loss : 1.f);
    ra.store_out = (flags & atm::ROW_MEAS) ? 1 : 0;
    {
      Prof p(pl, ATM_KIND_ROW_PASS, st);
      ATM_CUDA(atm::launch_row_pass(N, batch, ra, st));
    }
    if (next_vac) {
      ca.hy = (const float2*)pl->hy.p + (size_t)i * N;
      ca.hx = (const float2*)pl->hx.p + (size_t)i * N;
      Prof p(pl, ATM_KIND_COL_PASS, st);
      ATM_CUDA(atm::launch_col_pass(N, batch, pl->col_tile, ca, st));
    }
  }
  if (!measured) {
    // last row pass: inverse row FFT (or the analytic field of a vacuum path)
    ra.flags = (n == 0 ? atm::ROW_GEN : atm::ROW_INV) | atm::ROW_MEAS | (field_out ? atm::ROW_STORE : 0);
    ra.loss = pl->final_loss;
    ra.store_out = 1;
    Prof p(pl, ATM_KIND_ROW_PASS, st);
    ATM_CUDA(atm::launch_row_pass(N, batch, ra, st));
  }
  if (int rc = finish_measures(pl, batch, measures, st)) return rc;
  for (int i = 0; pl->step_meas && i < n; ++i) {
    atm::FinalArgs fa{};
    fa.partials = (const double*)pl->step_partials.p + (size_t)i * pl->B * pl->n_parts * 6;
    fa.center = (const float*)pl->step_center.p + (size_t)i * pl->B;
    fa.out = measures + pl->step_slot0 + (size_t)i * ATM_STEP_SLOTS;
    fa.n_parts = pl->n_parts;
    fa.n_meas = 6;
    fa.n_out = pl->n_out;
    fa.n_pupils = 0;
    fa.delta = pl->delta;
    fa.status = (const int*)pl->status.p;
    Prof p(pl, ATM_KIND_FINALIZE, st);
    ATM_CUDA(atm::launch_finalize(batch, fa, st));
  }
  return ATM_OK;
}

int check_device(const AtmPlan* pl) {
  int dev = -1;
  cudaGetDevice(&dev);
  if (dev != pl->device) return fail(ATM_ERR_INVALID, "plan belongs to device %d, current device is %d", pl->device, dev);
  return ATM_OK;
}

}  // namespace

extern "C" {

int atm_run(AtmPlan* pl, const float* rho, const float* theta, const void* value, int32_t batch, double* measures,
            void* field_out, float* mean_intensity, void* stream) {
  if (!pl) return fail(ATM_ERR_INVALID, "plan is NULL");
  if (int rc = check_device(pl)) return rc;
  if (batch < 1 || batch > pl->B) return fail(ATM_ERR_INVALID, "batch %d out of range [1, %d]", batch, pl->B);
  if (!measures) return fail(ATM_ERR_INVALID, "measures_out is NULL");
  if (pl->n > 0 && (!rho || !theta || !value)) return fail(ATM_ERR_INVALID, "spectra pointers are NULL");
  cudaStream_t st = (cudaStream_t)stream;
  auto ss_screen = [&](int i) { return run_screen(pl, screen_args(pl, rho, theta, value, i), batch, true, st); };
  return propagate(pl, batch, ss_screen, folds(pl), measures, field_out, mean_intensity, st);
}

int atm_run_fft(AtmPlan* pl, const float* normals, const float* amp, const void* sub_x, const void* sub_y,
                const double* sub_mean, int32_t n_sub, int32_t batch, double* measures, void* field_out,
                void* stream) {
  if (!pl) return fail(ATM_ERR_INVALID, "plan is NULL");
  if (int rc = check_device(pl)) return rc;
  if (batch < 1 || batch > pl->B) return fail(ATM_ERR_INVALID, "batch %d out of range [1, %d]", batch, pl->B);
  if (!measures) return fail(ATM_ERR_INVALID, "measures_out is NULL");
  if (pl->n < 1 || !pl->scr.p) return fail(ATM_ERR_INVALID, "atm_run_fft needs a plan with screens and ATM_FLAG_FFT_SCREENS");
  if (!normals || !amp || !sub_mean) return fail(ATM_ERR_INVALID, "NULL screen input");
  if (n_sub < 0 || (n_sub > 0 && (!sub_x || !sub_y))) return fail(ATM_ERR_INVALID, "bad subharmonic tables");
  cudaStream_t st = (cudaStream_t)stream;
  const int N = pl->N, n = pl->n;
  const size_t plane = (size_t)N * N;
  auto fft_screen = [&](int i) -> int {
    atm::FftScreenArgs fa{};
    fa.normals = normals + (size_t)i * 2 * plane;
    fa.nrm_stride = (size_t)n * 2 * plane;
    fa.amp = amp + (size_t)i * plane;
    fa.sub_x = n_sub ? (const float2*)sub_x + (size_t)i * n_sub * N : nullptr;
    fa.sub_y = n_sub ? (const float2*)sub_y + (size_t)i * n_sub * N : nullptr;
    fa.sub_stride = (size_t)n * n_sub * N;
    fa.sub_mean = sub_mean + 2 * i;
    fa.mean_stride = 2 * n;
    fa.n_sub = n_sub;
    fa.N = N;
    fa.field = (float2*)pl->scr.p;
    fa.phi = (float*)pl->phi.p;
    {
      Prof p(pl, ATM_KIND_SCREEN_PREP, st);
      ATM_CUDA(atm::launch_fft_screen_spectrum(batch, fa, st));
    }
    // the screen's inverse 2-D transform on its own (row-major) workspace
    atm::RowArgs ra{};
    ra.field = (float2*)pl->scr.p;
    ra.tw = (const float2*)pl->tw.p;
    ra.loss = 1.f;
    ra.delta = (float)pl->delta;
    ra.delta64 = pl->delta;
    ra.flags = atm::ROW_INV | atm::ROW_STORE;
    ra.variant = pl->tiled ? 3 : pl->row_variant;
    ra.status = (int*)pl->status.p;
    {
      Prof p(pl, ATM_KIND_ROW_PASS, st);
      ATM_CUDA(atm::launch_row_pass(N, batch, ra, st));
    }
    atm::ColArgs ca{};
    ca.field = (float2*)pl->scr.p;
    ca.tw = (const float2*)pl->tw.p;
    ca.variant = pl->tiled ? 4 : pl->col_variant;
    ca.inv_only = 1;
    ca.status = (int*)pl->status.p;
    {
      Prof p(pl, ATM_KIND_COL_PASS, st);
      ATM_CUDA(atm::launch_col_pass(N, batch, pl->tiled ? 0 : pl->col_tile, ca, st));
    }
    Prof p(pl, ATM_KIND_SCREEN_EVAL, st);
    ATM_CUDA(atm::launch_fft_screen_finish(batch, fa, st));
    return ATM_OK;
  };
  return propagate(pl, batch, fft_screen, true, measures, field_out, nullptr, st);
}

int atm_run_channel(AtmPlan* pl, AtmChannel* ch, const float* rho, const float* theta, const void* value,
                    int32_t batch, double* measures, void* field_out, float* mean_intensity, void* stream) {
  if (!pl || !ch) return fail(ATM_ERR_INVALID, "plan / channel is NULL");
  if (ch->plan != pl) return fail(ATM_ERR_INVALID, "the channel was built for another plan");
  swap_state(pl, ch->st);
  const int rc = atm_run(pl, rho, theta, value, batch, measures, field_out, mean_intensity, stream);
  swap_state(pl, ch->st);
  return rc;
}

int atm_measures(AtmPlan* pl, const void* field, int32_t batch, double* measures, void* stream) {
  if (!pl) return fail(ATM_ERR_INVALID, "plan is NULL");
  if (int rc = check_device(pl)) return rc;
  if (batch < 1 || batch > pl->B) return fail(ATM_ERR_INVALID, "batch %d out of range [1, %d]", batch, pl->B);
  if (!field || !measures) return fail(ATM_ERR_INVALID, "field / measures_out is NULL");
  cudaStream_t st = (cudaStream_t)stream;
  atm::RowArgs ra = row_args(pl, nullptr, nullptr);
  ra.field = (float2*)field;
  ra.tiled = 0;  // the caller's field is row-major
  ra.flags = atm::ROW_MEAS;
  ra.loss = 1.f;
  {
    Prof p(pl, ATM_KIND_ROW_PASS, st);
    ATM_CUDA(atm::launch_row_pass(pl->N, batch, ra, st));
  }
  return finish_measures(pl, batch, measures, st);
}

int atm_screen(AtmPlan* pl, const float* rho, const float* theta, const void* value, int32_t batch, int32_t screen,
               float* phi_out, void* phasor_out, void* stream) {
  if (!pl) return fail(ATM_ERR_INVALID, "plan is NULL");
  if (int rc = check_device(pl)) return rc;
  if (pl->n < 1) return fail(ATM_ERR_INVALID, "plan has no screens");
  if (batch < 1 || batch > pl->B) return fail(ATM_ERR_INVALID, "batch %d out of range [1, %d]", batch, pl->B);
  if (screen < 0 || screen >= pl->n) return fail(ATM_ERR_INVALID, "screen %d out of range", screen);
  if (!rho || !theta || !value) return fail(ATM_ERR_INVALID, "spectra pointers are NULL");
  cudaStream_t st = (cudaStream_t)stream;
  atm::ScreenArgs s = screen_args(pl, rho, theta, value, screen);
  s.Gy = (double*)pl->Gy.p;
  s.Hx = (double*)pl->Hx.p;
  if (int rc = run_screen(pl, s, batch, false, st)) return rc;
  ATM_CUDA(atm::launch_compose_screen(batch, pl->N, (const double*)pl->Gy.p, (const double*)pl->Hx.p,
                                      (const float*)pl->phi.p, (const float2*)pl->Py.p, (const float2*)pl->Px.p,
                                      phi_out, (float2*)phasor_out, st));
  return ATM_OK;
}

int atm_autotune(AtmPlan* pl, int32_t batch, int32_t repeats, void* stream) {
  if (!pl) return fail(ATM_ERR_INVALID, "plan is NULL");
  if (int rc = check_device(pl)) return rc;
  if (batch < 1 || batch > pl->B) return fail(ATM_ERR_INVALID, "batch %d out of range [1, %d]", batch, pl->B);
  if (repeats < 1 || repeats > 100) return fail(ATM_ERR_INVALID, "repeats %d out of range [1, 100]", repeats);
  cudaStream_t st = (cudaStream_t)stream;
  const int N = pl->N;
  const size_t plane = (size_t)N * N;
  // the candidates read the field, the screen phase and the phasors: zeroes
  ATM_CUDA(cudaMemsetAsync(pl->field.p, 0, (size_t)batch * plane * sizeof(float2), st));
  if (pl->n > 0) {
    ATM_CUDA(cudaMemsetAsync(pl->phi.p, 0, (size_t)batch * plane * sizeof(float), st));
    ATM_CUDA(cudaMemsetAsync(pl->Py.p, 0, (size_t)batch * N * sizeof(float2), st));
    ATM_CUDA(cudaMemsetAsync(pl->Px.p, 0, (size_t)batch * N * sizeof(float2), st));
  }
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  if (cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess) {
    if (e0) cudaEventDestroy(e0);
    return fail(ATM_ERR_CUDA, "cudaEventCreate failed");
  }
  // mean device ms of `repeats` launches after one warm-up; < 0 if the candidate does not launch
  auto time_it = [&](auto&& launch) -> double {
    if (launch() != cudaSuccess) {
      cudaGetLastError();
      return -1.0;
    }
    cudaEventRecord(e0, st);
    for (int k = 0; k < repeats; ++k)
      if (launch() != cudaSuccess) {
        cudaGetLastError();
        cudaEventSynchronize(e0);
        return -1.0;
      }
    cudaEventRecord(e1, st);
    if (cudaEventSynchronize(e1) != cudaSuccess) return -1.0;
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    return (double)ms / repeats;
  };
  // row pass: a middle screen step (inverse FFT, phasor, forward FFT, store)
  atm::RowArgs ra = row_args(pl, nullptr, nullptr);
  ra.flags = atm::ROW_INV | atm::ROW_FWD | atm::ROW_STORE |
             (pl->n > 0 ? atm::ROW_PHASOR | (folds(pl) ? atm::ROW_FOLDED : 0) : 0);
  ra.loss = 1.f;
  double best_row = -1.0;
  int row_variant = 0;
  // a tiled plan chooses among the tiled forms only (the others do not know its layout)
  const bool warp_fft = N == 1024 || N == 2048;         // row 11: warp FFTs
  const bool col_warp = warp_fft || N == 4096;          // column 10: warp FFTs (64-lane transforms at 4096)
  std::vector<int> row_forms = pl->tiled ? std::vector<int>{5, 6, 8, 9, 10} : std::vector<int>{0, 1, 2, 3, 4, 7};
  if (!pl->tiled && warp_fft) row_forms.push_back(11);
  for (int v : row_forms) {
    ra.variant = v;
    const double ms = time_it([&] { return atm::launch_row_pass(N, batch, ra, st); });
    if (ms >= 0 && (best_row < 0 || ms < best_row)) {
      best_row = ms;
      row_variant = v;
    }
  }
  // column pass: every tile of at most 512 threads, every variant
  atm::ColArgs ca{};
  ca.field = (float2*)pl->field.p;
  ca.tw = (const float2*)pl->tw.p;
  ca.hy = (const float2*)pl->hy.p;
  ca.hx = (const float2*)pl->hx.p;
  double best_col = -1.0;
  int col_tile = pl->col_tile, col_variant = 0;
  for (int C : {2, 4, 8, 16}) {
    if (C * (N / 16) > 512 || C > N) continue;
    if (pl->tiled && C != 4) continue;
    std::vector<int> col_forms = pl->tiled ? std::vector<int>{5, 6, 8, 9} : std::vector<int>{0, 1, 2, 3, 4, 7};
    if (pl->tiled && warp_fft && C == 4) col_forms.push_back(13);
    for (int v : col_forms) {
      ca.variant = v;
      const double ms = time_it([&] { return atm::launch_col_pass(N, batch, C, ca, st); });
      if (ms >= 0 && (best_col < 0 || ms < best_col)) {
        best_col = ms;
        col_tile = C;
        col_variant = v;
      }
    }
  }
  // the warp-FFT column groups choose their own tile (4 columns, 2 at 4096; 14: 4096-row tiles of 4
  // columns as two 2048-point halves); recorded as column tile 4
  std::vector<int> warp_cols;
  if (!pl->tiled && col_warp) warp_cols.push_back(10);
  if (!pl->tiled && N == 4096) warp_cols.push_back(14);
  if (!pl->tiled && N == 2048) warp_cols.push_back(15);
  for (int v : warp_cols) {
    ca.variant = v;
    const double ms = time_it([&] { return atm::launch_col_pass(N, batch, 4, ca, st); });
    if (ms >= 0 && (best_col < 0 || ms < best_col)) {
      best_col = ms;
      col_tile = 4;
      col_variant = v;
    }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (best_row < 0 || best_col < 0) return fail(ATM_ERR_CUDA, "autotune: no candidate launched");
  pl->row_variant = row_variant;
  pl->col_tile = col_tile;
  pl->col_variant = col_variant;
  pl->tuned = 1;
  return ATM_OK;
}

int atm_structure_function(const float* phi, int32_t batch, int32_t N, double* sf_out, void* stream) {
  if (!phi || !sf_out) return fail(ATM_ERR_INVALID, "phi / sf_out is NULL");
  if (batch < 1 || batch > 65535) return fail(ATM_ERR_INVALID, "batch %d out of range", batch);
  if (N < 2 || N > 8192) return fail(ATM_ERR_INVALID, "N %d out of range [2, 8192]", N);
  ATM_CUDA(atm::launch_structure_function(phi, batch, N, sf_out, (cudaStream_t)stream));
  return ATM_OK;
}

int atm_plan_set_variants(AtmPlan* pl, int32_t row_variant, int32_t col_tile, int32_t col_variant) {
  if (!pl) return fail(ATM_ERR_INVALID, "plan is NULL");
  if (pl->tiled) {
    // a tiled plan's field is only understood by the tiled forms
    if (row_variant != 5 && row_variant != 6 && row_variant != 8 && row_variant != 9 && row_variant != 10)
      return fail(ATM_ERR_INVALID, "row_variant %d: a tiled plan takes 5, 6, 8, 9 or 10", row_variant);
    const bool warp13 = col_variant == 13 && (pl->N == 1024 || pl->N == 2048);
    if ((col_variant != 5 && col_variant != 6 && col_variant != 8 && col_variant != 9 && !warp13) || col_tile != 4)
      return fail(ATM_ERR_INVALID, "a tiled plan takes col_variant 5, 6, 8 or 9 (13 at N = 1024, 2048) with col_tile 4");
    pl->row_variant = row_variant;
    pl->col_variant = col_variant;
    return ATM_OK;
  }
  const bool warp_fft = pl->N == 1024 || pl->N == 2048;  // row 11: warp FFTs
  const bool col_warp = warp_fft || pl->N == 4096;         // column 10: warp FFTs
  if (row_variant < 0 || (row_variant > 4 && row_variant != 7 && !(row_variant == 11 && warp_fft)))
    return fail(ATM_ERR_INVALID, "row_variant %d not in 0..4, 7%s", row_variant, warp_fft ? " or 11" : "");
  const int split = pl->N == 4096 ? 14 : (pl->N == 2048 ? 15 : -1);  // two half-length warp FFTs per column
  if (col_variant < 0 ||
      (col_variant > 4 && col_variant != 7 && !(col_variant == 10 && col_warp) && col_variant != split))
    return fail(ATM_ERR_INVALID, "col_variant %d not in 0..4, 7%s%s", col_variant, col_warp ? ", 10" : "",
                split == 14 ? " or 14" : (split == 15 ? " or 15" : ""));
  if ((col_variant == 10 || col_variant == 14 || col_variant == 15) && col_tile != 4)
    return fail(ATM_ERR_INVALID, "col_variant %d takes col_tile 4", col_variant);
  if (col_tile != 2 && col_tile != 4 && col_tile != 8 && col_tile != 16)
    return fail(ATM_ERR_INVALID, "col_tile %d not in {2, 4, 8, 16}", col_tile);
  // (the warp-FFT column groups are 256 threads whatever the recorded tile)
  if (col_variant != 10 && col_variant != 14 && col_variant != 15 && (col_tile * (pl->N / 16) > 512 || col_tile > pl->N))
    return fail(ATM_ERR_UNSUPPORTED, "col_tile %d exceeds 512 threads per CTA at N = %d", col_tile, pl->N);
  pl->row_variant = row_variant;
  pl->col_tile = col_tile;
  pl->col_variant = col_variant;
  return ATM_OK;
}

int atm_vacuum(AtmPlan* pl, void* field, int32_t batch, double dz, void* stream) {
  if (!pl) return fail(ATM_ERR_INVALID, "plan is NULL");
  if (int rc = check_device(pl)) return rc;
  if (!field) return fail(ATM_ERR_INVALID, "field is NULL");
  if (batch < 1) return fail(ATM_ERR_INVALID, "batch must be >= 1");
  if (!(dz > 0)) return ATM_OK;
  cudaStream_t st = (cudaStream_t)stream;
  const int N = pl->N;
  std::vector<cd> h = transfer_1d(N, pl->delta, pl->kw, dz);
  const cd ph = global_phase(pl->kw, dz) / ((double)N * (double)N);
  std::vector<float2> tab(2 * (size_t)N);
  for (int k = 0; k < N; ++k) {
    const cd y = ph * h[k];
    tab[k] = make_float2((float)y.real(), (float)y.imag());
    tab[N + k] = make_float2((float)h[k].real(), (float)h[k].imag());
  }
  // the source is pageable: cudaMemcpyAsync returns once it has been staged
  ATM_CUDA(cudaMemcpyAsync(pl->vac_h.p, tab.data(), tab.size() * sizeof(float2), cudaMemcpyHostToDevice, st));
  // a tiled plan converts the caller's row-major field to the tiled layout in
  // the first row pass and back in the last (the tensor copies want the field
  // on a 128-byte boundary); otherwise the row-major forms run
  const bool tiled = pl->tiled && ((uintptr_t)field & 127) == 0;
  atm::RowArgs ra{};
  ra.field = (float2*)field;
  ra.tw = (const float2*)pl->tw.p;
  ra.loss = 1.f;
  ra.delta = (float)pl->delta;
  ra.delta64 = pl->delta;
  ra.variant = tiled ? pl->row_variant : 0;
  ra.tiled = tiled ? atm::TILE_OUT : 0;
  ra.status = (int*)pl->status.p;
  ra.flags = atm::ROW_FWD | atm::ROW_STORE;
  ATM_CUDA(atm::launch_row_pass(N, batch, ra, st));
  atm::ColArgs ca{};
  ca.field = (float2*)field;
  ca.tw = (const float2*)pl->tw.p;
  ca.variant = tiled ? pl->col_variant : (pl->tiled ? 4 : pl->col_variant);
  ca.status = (int*)pl->status.p;
  ca.hy = (const float2*)pl->vac_h.p;
  ca.hx = (const float2*)pl->vac_h.p + N;
  ATM_CUDA(atm::launch_col_pass(N, batch, pl->col_tile, ca, st));
  ra.tiled = tiled ? atm::TILE_IN : 0;
  ra.flags = atm::ROW_INV | atm::ROW_STORE;
  ATM_CUDA(atm::launch_row_pass(N, batch, ra, st));
  return ATM_OK;
}

int atm_fft_screen(AtmPlan* pl, const float* normals, const float* amp, const void* sub_x, const void* sub_y,
                   const double* sub_mean, int32_t n_sub, int32_t batch, void* screen_out, void* stream) {
  if (!pl) return fail(ATM_ERR_INVALID, "plan is NULL");
  if (int rc = check_device(pl)) return rc;
  if (batch < 1 || batch > pl->B) return fail(ATM_ERR_INVALID, "batch %d out of range [1, %d]", batch, pl->B);
  if (!normals || !amp || !screen_out) return fail(ATM_ERR_INVALID, "NULL input / output");
  if (n_sub < 0 || (n_sub > 0 && (!sub_x || !sub_y))) return fail(ATM_ERR_INVALID, "bad subharmonic tables");
  if (!sub_mean) return fail(ATM_ERR_INVALID, "sub_mean is NULL");
  cudaStream_t st = (cudaStream_t)stream;
  atm::FftScreenArgs fa{};
  fa.normals = normals;
  fa.amp = amp;
  fa.sub_x = (const float2*)sub_x;
  fa.sub_y = (const float2*)sub_y;
  fa.sub_mean = sub_mean;
  fa.n_sub = n_sub;
  fa.N = pl->N;
  fa.field = (float2*)pl->field.p;
  fa.out = (float2*)screen_out;
  fa.phi = nullptr;
  fa.nrm_stride = 2 * (size_t)pl->N * pl->N;
  fa.sub_stride = (size_t)n_sub * pl->N;
  fa.mean_stride = 2;
  ATM_CUDA(atm::launch_fft_screen_spectrum(batch, fa, st));
  atm::RowArgs ra{};
  ra.field = (float2*)pl->field.p;
  ra.tw = (const float2*)pl->tw.p;
  ra.loss = 1.f;
  ra.delta = (float)pl->delta;
  ra.delta64 = pl->delta;
  ra.flags = atm::ROW_INV | atm::ROW_STORE;
  {
    Prof p(pl, ATM_KIND_ROW_PASS, st);
    ATM_CUDA(atm::launch_row_pass(pl->N, batch, ra, st));
  }
  atm::ColArgs ca{};
  ca.field = (float2*)pl->field.p;
  ca.tw = (const float2*)pl->tw.p;
  ca.variant = pl->tiled ? 4 : pl->col_variant;  // this screen's workspace stays row-major
  ca.inv_only = 1;
  {
    Prof p(pl, ATM_KIND_COL_PASS, st);
    ATM_CUDA(atm::launch_col_pass(pl->N, batch, pl->col_tile, ca, st));
  }
  ATM_CUDA(atm::launch_fft_screen_finish(batch, fa, st));
  return ATM_OK;
}

int atm_draw_spectra(AtmPlan* pl, uint64_t seed, uint64_t first_realisation, const float* sqrt_psd, int32_t batch,
                     float* rho, float* theta, void* value, void* stream) {
  if (!pl) return fail(ATM_ERR_INVALID, "plan is NULL");
  if (int rc = check_device(pl)) return rc;
  if (pl->n < 1) return fail(ATM_ERR_INVALID, "plan has no screens");
  if (batch < 1 || batch > 65535) return fail(ATM_ERR_INVALID, "batch %d out of range", batch);
  if (!sqrt_psd || !rho || !theta || !value) return fail(ATM_ERR_INVALID, "NULL argument");
  ATM_CUDA(atm::launch_draw_spectra(seed, first_realisation, pl->n, pl->P, (const float*)pl->fbase.p, sqrt_psd,
                                    batch, rho, theta, (float2*)value, (cudaStream_t)stream));
  return ATM_OK;
}

int atm_channel_draw_spectra(AtmPlan* pl, AtmChannel* ch, uint64_t seed, uint64_t first_realisation,
                             const float* sqrt_psd, int32_t batch, float* rho, float* theta, void* value,
                             void* stream) {
  if (!pl || !ch) return fail(ATM_ERR_INVALID, "plan / channel is NULL");
  if (ch->plan != pl) return fail(ATM_ERR_INVALID, "the channel was built for another plan");
  swap_state(pl, ch->st);
  const int rc = atm_draw_spectra(pl, seed, first_realisation, sqrt_psd, batch, rho, theta, value, stream);
  swap_state(pl, ch->st);
  return rc;
}

int atm_profile_begin(AtmPlan* pl, int32_t max_launches) {
  if (!pl || max_launches < 1) return fail(ATM_ERR_INVALID, "bad profile arguments");
  if (int rc = check_device(pl)) return rc;
  if ((int)pl->ev.size() < 2 * max_launches) {
    for (auto e : pl->ev) cudaEventDestroy(e);
    pl->ev.assign(2 * (size_t)max_launches, nullptr);
    for (auto& e : pl->ev) ATM_CUDA(cudaEventCreate(&e));
  }
  pl->ev_kind.assign(max_launches, 0);
  pl->ev_cap = max_launches;
  pl->ev_used = 0;
  pl->profiling = true;
  return ATM_OK;
}

int atm_profile_end(AtmPlan* pl, double* ms, int32_t* count, int32_t n_kinds) {
  if (!pl || !ms || !count || n_kinds < 1) return fail(ATM_ERR_INVALID, "bad profile arguments");
  for (int k = 0; k < n_kinds; ++k) {
    ms[k] = 0.0;
    count[k] = 0;
  }
  pl->profiling = false;
  for (int i = 0; i < pl->ev_used; ++i) {
    ATM_CUDA(cudaEventSynchronize(pl->ev[2 * i + 1]));
    float t = 0.f;
    ATM_CUDA(cudaEventElapsedTime(&t, pl->ev[2 * i], pl->ev[2 * i + 1]));
    const int k = pl->ev_kind[i];
    if (k < n_kinds) {
      ms[k] += t;
      count[k] += 1;
    }
  }
  pl->ev_used = 0;
  return ATM_OK;
}

int atm_fma_probe(int32_t blocks, int32_t iters, double* ms, void* stream) {
  if (blocks < 1 || iters < 1 || !ms) return fail(ATM_ERR_INVALID, "bad probe arguments");
  cudaStream_t st = (cudaStream_t)stream;
  cudaEvent_t a, b;
  ATM_CUDA(cudaEventCreate(&a));
  ATM_CUDA(cudaEventCreate(&b));
  ATM_CUDA(cudaEventRecord(a, st));
  ATM_CUDA(atm::launch_fma_probe(blocks, iters, st));
  ATM_CUDA(cudaEventRecord(b, st));
  ATM_CUDA(cudaEventSynchronize(b));
  float t = 0.f;
  ATM_CUDA(cudaEventElapsedTime(&t, a, b));
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  *ms = t;
  return ATM_OK;
}

int atm_plan_check(AtmPlan* pl, void* stream) {
  if (!pl) return fail(ATM_ERR_INVALID, "plan is NULL");
  if (int rc = check_device(pl)) return rc;
  cudaStream_t st = (cudaStream_t)stream;
  ATM_CUDA(cudaStreamSynchronize(st));
  int word = 0, pass_flag = 0, tc_flag = 0;
  ATM_CUDA(cudaMemcpy(&word, pl->status.p, sizeof(int), cudaMemcpyDeviceToHost));
  ATM_CUDA(atm::pass_error_flag(&pass_flag, true));
  ATM_CUDA(atm::tc_error_flag(&tc_flag, true));
  if (word == 0 && !pass_flag && !tc_flag) return ATM_OK;
  ATM_CUDA(cudaMemset(pl->status.p, 0, sizeof(int)));
  if (word & atm::STATUS_NONFINITE)
    return fail(ATM_ERR_NONFINITE, "a spectrum value (rho, theta or value) was NaN or infinite; the measures of "
                                   "the runs since the last check are NaN");
  return fail(ATM_ERR_TIMEOUT, "a device wait ran out (%s%s%s); the kernels recorded it, drained their copies and "
                               "returned, and the measures of the runs since the last check are NaN",
              (word & atm::STATUS_PASS_WAIT) || pass_flag ? "FFT pass" : "",
              ((word & atm::STATUS_PASS_WAIT) || pass_flag) && ((word & atm::STATUS_GEMM_WAIT) || tc_flag) ? ", " : "",
              (word & atm::STATUS_GEMM_WAIT) || tc_flag ? "screen GEMM" : "");
}

int atm_set_wait_budget(uint64_t ns) {
  if (ns < 1 || ns > 60000000000ull) return fail(ATM_ERR_INVALID, "wait budget %llu ns not in [1, 6e10]",
                                                 (unsigned long long)ns);
  ATM_CUDA(atm::set_pass_wait_budget((unsigned long long)ns));
  ATM_CUDA(atm::set_tc_wait_budget((unsigned long long)ns));
  return ATM_OK;
}

}  // extern "C"
