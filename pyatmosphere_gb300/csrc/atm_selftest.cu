// Host-only emulation of the engine's FFT stages, Bessel coefficients and
// fixed-point phase reduction (libatm_selftest.so).  The functions called
// here are the same __host__ __device__ code the kernels run; the Stockham
// stages are executed thread by thread between the points where the kernels
// synchronise.  Used by the CPU test suite; needs no GPU.
#include <type_traits>
#include <vector>

#include "atm_common.cuh"

namespace {

struct Regs {
  float2 v[16];
};

template <int N, int DIR, int s, int TWREC>
void host_stages(std::vector<Regs>& R, float2* sm, const float2* tw) {
  constexpr int T = N / 16;
  if constexpr (s == atm::FftPlan<N>::S - 1) {
    for (int t = 0; t < T; ++t) atm::stage_last<N, DIR, 0, TWREC>(R[t].v, t, tw);
  } else {
    for (int t = 0; t < T; ++t) atm::stage_to_smem<N, s, DIR, 0, TWREC>(R[t].v, sm, t, tw);
    for (int t = 0; t < T; ++t) atm::stage_from_smem<N, s + 1>(R[t].v, sm, t);
    host_stages<N, DIR, s + 1, TWREC>(R, sm, tw);
  }
}

// the same stages with each emulated thread's twiddle bases held apart (the
// register-twiddle forms of the passes)
template <int N, int DIR, int s>
void host_stages_reg(std::vector<Regs>& R, float2* sm, const std::vector<atm::TwBases<N>>& tb) {
  constexpr int T = N / 16;
  if constexpr (s == atm::FftPlan<N>::S - 1) {
    for (int t = 0; t < T; ++t) atm::stage_last_reg<N, DIR>(R[t].v, t, tb[t]);
  } else {
    for (int t = 0; t < T; ++t) atm::stage_to_smem_reg<N, s, DIR>(R[t].v, sm, t, tb[t]);
    for (int t = 0; t < T; ++t) atm::stage_from_smem<N, s + 1>(R[t].v, sm, t);
    host_stages_reg<N, DIR, s + 1>(R, sm, tb);
  }
}

// TWREC = 2: bases per emulated thread, as the persistent passes hold them in registers
template <int N, int TWREC = 0>
int host_fft(int dir, const float* in, float* out) {
  constexpr int T = N / 16;
  std::vector<float2> tw(N), sm(atm::Padded<N>::value);
  for (int i = 0; i < N; ++i) {
    const double a = -2.0 * 3.14159265358979323846 * i / N;
    tw[i] = make_float2((float)cos(a), (float)sin(a));
  }
  std::vector<Regs> R(T);
  for (int t = 0; t < T; ++t)
    for (int m = 0; m < 16; ++m) R[t].v[m] = make_float2(in[2 * (t + m * T)], in[2 * (t + m * T) + 1]);
  if constexpr (TWREC == 2) {
    std::vector<atm::TwBases<N>> tb(T);
    for (int t = 0; t < T; ++t) atm::load_twiddle_bases<N>(tb[t], tw.data(), t);
    if (dir < 0)
      host_stages_reg<N, -1, 0>(R, sm.data(), tb);
    else
      host_stages_reg<N, 1, 0>(R, sm.data(), tb);
  } else if (dir < 0) {
    host_stages<N, -1, 0, TWREC>(R, sm.data(), tw.data());
  } else {
    host_stages<N, 1, 0, TWREC>(R, sm.data(), tw.data());
  }
  for (int t = 0; t < T; ++t)
    for (int m = 0; m < 16; ++m) {
      out[2 * (t + m * T)] = R[t].v[m].x;
      out[2 * (t + m * T) + 1] = R[t].v[m].y;
    }
  return 0;
}

// the warp FFT of length N = 32 R, its 32 lanes emulated one after another on
// each side of the exchange.  mode 0: the exchange swizzle of a warp that
// holds all 32 lanes (row pass); mode 1 + c: that of column c of a
// four-column group (column pass)
// NL = 64 lanes (N = 4096): mode 1 + c is the swizzle of column c of a
// two-column group, and the twiddles are formed as the column pass forms
// them, W^(j (kb & 7)) W^(8 j (kb >> 3))
template <int R, int NL = 32>
int host_wfft(int dir, int mode, const float* in, float* out) {
  constexpr int N = NL * R;
  std::vector<float2> tw(N), twt(R * NL), xbuf(N);
  for (int i = 0; i < N; ++i) {
    const double a = -2.0 * 3.14159265358979323846 * i / N;
    tw[i] = make_float2((float)cos(a), (float)sin(a));
  }
  for (int i = 0; i < R * NL; ++i) twt[i] = tw[(i / NL) * (i % NL)];
  auto sw = [&](int kb) {
    if (NL == 64) return (kb & 7) | ((mode - 1) << 3);
    return mode == 0 ? (kb & 15) : ((kb & 3) | ((mode - 1) << 2));
  };
  auto twiddle = [&](int kb, int j) {
    if (NL == 64) return atm::cmul(tw[j * (kb & 7)], tw[(8 * j * (kb >> 3)) % N]);
    return twt[kb * NL + j];
  };
  struct Lane {
    float2 v[R];
  };
  std::vector<Lane> L(NL);
  for (int j = 0; j < NL; ++j)
    for (int m = 0; m < R; ++m) L[j].v[m] = make_float2(in[2 * (j + NL * m)], in[2 * (j + NL * m) + 1]);
  auto run = [&](auto dirc) {
    constexpr int D = decltype(dirc)::value;
    for (int j = 0; j < NL; ++j)
      atm::wfft_stage1<R, D>(
          L[j].v, [&](int kb) { return twiddle(kb, j); },
          [&](int kb, float2 y) { xbuf[atm::wfft_slot_l<NL>(kb, j, sw(kb))] = y; });
    for (int j = 0; j < NL; ++j)
      atm::wfft_stage2<R, D, NL>(L[j].v, [&](int h, int jj) {
        const int kb = j + NL * h;
        return xbuf[atm::wfft_slot_l<NL>(kb, jj, sw(kb))];
      });
  };
  if (dir < 0)
    run(std::integral_constant<int, -1>{});
  else
    run(std::integral_constant<int, 1>{});
  for (int j = 0; j < NL; ++j)
    for (int q = 0; q < R; ++q) {
      out[2 * (j + NL * q)] = L[j].v[q].x;
      out[2 * (j + NL * q) + 1] = L[j].v[q].y;
    }
  return 0;
}

}  // namespace

extern "C" {

// length-N warp FFT (N = 1024 or 2048: 32 lanes; 4096: 64 lanes, modes 1 and
// 2 only; dir = -1 forward, +1 unnormalised inverse) of interleaved complex
// data, exchange swizzle `mode` (see host_wfft)
int atm_selftest_wfft(int N, int dir, int mode, const float* in, float* out) {
  if (mode < 0 || mode > 4) return -1;
  switch (N) {
    case 1024: return host_wfft<32>(dir, mode, in, out);
    case 2048: return host_wfft<64>(dir, mode, in, out);
    case 4096: return (mode == 1 || mode == 2) ? host_wfft<64, 64>(dir, mode, in, out) : -1;
  }
  return -1;
}

// length-N FFT (dir = -1 forward, +1 unnormalised inverse) of interleaved complex data
int atm_selftest_fft(int N, int dir, const float* in, float* out) {
  switch (N) {
    case 64: return host_fft<64>(dir, in, out);
    case 128: return host_fft<128>(dir, in, out);
    case 256: return host_fft<256>(dir, in, out);
    case 512: return host_fft<512>(dir, in, out);
    case 1024: return host_fft<1024>(dir, in, out);
    case 2048: return host_fft<2048>(dir, in, out);
    case 4096: return host_fft<4096>(dir, in, out);
  }
  return -1;
}

// the same with the twiddle bases held per thread (register-twiddle forms)
int atm_selftest_fft_twreg(int N, int dir, const float* in, float* out) {
  switch (N) {
    case 64: return host_fft<64, 2>(dir, in, out);
    case 128: return host_fft<128, 2>(dir, in, out);
    case 256: return host_fft<256, 2>(dir, in, out);
    case 512: return host_fft<512, 2>(dir, in, out);
    case 1024: return host_fft<1024, 2>(dir, in, out);
    case 2048: return host_fft<2048, 2>(dir, in, out);
    case 4096: return host_fft<4096, 2>(dir, in, out);
  }
  return -1;
}

// the same with twiddles formed from powers of two (column-pass variant 2)
int atm_selftest_fft_twrec(int N, int dir, const float* in, float* out) {
  switch (N) {
    case 64: return host_fft<64, 1>(dir, in, out);
    case 128: return host_fft<128, 1>(dir, in, out);
    case 256: return host_fft<256, 1>(dir, in, out);
    case 512: return host_fft<512, 1>(dir, in, out);
    case 1024: return host_fft<1024, 1>(dir, in, out);
    case 2048: return host_fft<2048, 1>(dir, in, out);
    case 4096: return host_fft<4096, 1>(dir, in, out);
  }
  return -1;
}

int atm_selftest_bessel(double a, int D, double* J) {
  if (D < 1 || D > 256) return -1;
  atm::bessel_j(a, D, J);
  return 0;
}

// half-turns of frac(j * S + O) for j < N through the 64-bit fixed-point path
int atm_selftest_turns(double S, double O, int N, float* half_turns) {
  const uint64_t s = atm::turns_to_fixed(S), o = atm::turns_to_fixed(O);
  for (int j = 0; j < N; ++j) half_turns[j] = atm::fixed_to_halfturns(s * (uint64_t)j + o);
  return 0;
}

int atm_selftest_philox(const uint32_t* ctr, const uint32_t* key, uint32_t* out) {
  atm::Philox4 c;
  for (int i = 0; i < 4; ++i) c.v[i] = ctr[i];
  const atm::Philox4 r = atm::philox4x32_10(c, key[0], key[1]);
  for (int i = 0; i < 4; ++i) out[i] = r.v[i];
  return 0;
}

}  // extern "C"
