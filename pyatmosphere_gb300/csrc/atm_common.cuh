// Shared device/host building blocks of the GB300 split-step engine.
//
// Everything in this header is __host__ __device__ so that the FFT stage
// arithmetic, the Bessel / Chebyshev coefficients of the low-frequency screen
// block and the fixed-point phase reduction can be exercised on the CPU
// (atm_selftest.cu) with exactly the code the kernels run.
#pragma once

#include <cstdint>
#include <cmath>
#include <cuda_runtime.h>

#if defined(__CUDACC__)
#define ATM_HD __host__ __device__ __forceinline__
#else
#define ATM_HD inline
#endif

namespace atm {

// ---------------------------------------------------------------------------
// complex helpers (complex64 = float2, complex128 = double2)
//
// On the device a complex add or subtract is one packed FP32x2 instruction
// (add / sub .rn.f32x2, sm_100 and later): each lane rounds like a scalar
// FADD, so the results are the scalar ones bit for bit, in half the issue
// slots.  The FFT butterflies are mostly such adds.
// ---------------------------------------------------------------------------
#if defined(__CUDA_ARCH__)
__device__ __forceinline__ uint64_t f2_bits(float2 a) {
  uint64_t r;
  asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(a.x), "f"(a.y));
  return r;
}
__device__ __forceinline__ float2 bits_f2(uint64_t r) {
  float2 a;
  asm("mov.b64 {%0, %1}, %2;" : "=f"(a.x), "=f"(a.y) : "l"(r));
  return a;
}
#endif
ATM_HD float2 cadd(float2 a, float2 b) {
#if defined(__CUDA_ARCH__)
  uint64_t d;
  asm("add.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(f2_bits(a)), "l"(f2_bits(b)));
  return bits_f2(d);
#else
  return make_float2(a.x + b.x, a.y + b.y);
#endif
}
ATM_HD float2 csub(float2 a, float2 b) {
#if defined(__CUDA_ARCH__)
  uint64_t d;
  asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(f2_bits(a)), "l"(f2_bits(b)));
  return bits_f2(d);
#else
  return make_float2(a.x - b.x, a.y - b.y);
#endif
}
// complex product with its two fused multiply-adds written out: every kernel
// (and the host emulation) rounds it the same way, whatever the compiler
// would otherwise contract, so launch forms that share the arithmetic share
// the bits
ATM_HD float2 cmul(float2 a, float2 b) {
  return make_float2(fmaf(a.x, b.x, -(a.y * b.y)), fmaf(a.x, b.y, a.y * b.x));
}
ATM_HD float2 cconj(float2 a) { return make_float2(a.x, -a.y); }
ATM_HD float2 cscale(float2 a, float s) { return make_float2(a.x * s, a.y * s); }
// multiply by -i (DIR=-1, forward) or +i (DIR=+1, inverse)
template <int DIR>
ATM_HD float2 cmul_i(float2 a) {
  return DIR < 0 ? make_float2(a.y, -a.x) : make_float2(-a.y, a.x);
}

// ---------------------------------------------------------------------------
// small DFTs, b_q = sum_m a_m exp(DIR * 2 pi i m q / R)
// ---------------------------------------------------------------------------
template <int DIR>
ATM_HD void dft2(float2& a0, float2& a1) {
  float2 t = a0;
  a0 = cadd(t, a1);
  a1 = csub(t, a1);
}

template <int DIR>
ATM_HD void dft4(float2& a0, float2& a1, float2& a2, float2& a3) {
  float2 s02 = cadd(a0, a2), d02 = csub(a0, a2);
  float2 s13 = cadd(a1, a3), d13 = cmul_i<DIR>(csub(a1, a3));
  a0 = cadd(s02, s13);
  a2 = csub(s02, s13);
  a1 = cadd(d02, d13);
  a3 = csub(d02, d13);
}

template <int DIR>
ATM_HD void dft8(float2 (&a)[8]) {
  // even / odd split: E = DFT4(a0,a2,a4,a6), O = DFT4(a1,a3,a5,a7)
  dft4<DIR>(a[0], a[2], a[4], a[6]);
  dft4<DIR>(a[1], a[3], a[5], a[7]);
  const float h = 0.70710678118654752440f;
  // twiddles w^q, w = exp(DIR 2 pi i / 8), applied to O_q (q = 1,2,3)
  float2 o1 = a[3], o2 = a[5], o3 = a[7];
  o1 = cmul(o1, make_float2(h, DIR * h));
  o2 = cmul_i<DIR>(o2);  // w^2 = exp(DIR i pi/2) = DIR * i
  o3 = cmul(o3, make_float2(-h, DIR * h));
  float2 e0 = a[0], e1 = a[2], e2 = a[4], e3 = a[6], o0 = a[1];
  a[0] = cadd(e0, o0);
  a[4] = csub(e0, o0);
  a[1] = cadd(e1, o1);
  a[5] = csub(e1, o1);
  a[2] = cadd(e2, o2);
  a[6] = csub(e2, o2);
  a[3] = cadd(e3, o3);
  a[7] = csub(e3, o3);
}

template <int DIR>
ATM_HD void dft16(float2 (&a)[16]) {
  // m = m1 + 4 m2, q = 4 q1 + q2:
  //   c[m1][q2] = sum_m2 a[m1 + 4 m2] W4^(m2 q2)   (DFT4 over stride-4 inputs)
  //   c[m1][q2] *= W16^(m1 q2)
  //   b[4 q1 + q2] = sum_m1 c[m1][q2] W4^(m1 q1)
  for (int m1 = 0; m1 < 4; ++m1) dft4<DIR>(a[m1], a[m1 + 4], a[m1 + 8], a[m1 + 12]);
  // after the first DFT4, a[m1 + 4 q2] holds c[m1][q2]
  const float c1 = 0.92387953251128675613f, s1 = 0.38268343236508977173f;
  const float h = 0.70710678118654752440f;
  // W16^1, W16^2, W16^3, W16^4(=W4^1), W16^6, W16^9 with W16 = exp(DIR 2 pi i/16)
  const float2 w1 = make_float2(c1, DIR * s1);
  const float2 w2 = make_float2(h, DIR * h);
  const float2 w3 = make_float2(s1, DIR * c1);
  const float2 w6 = make_float2(-h, DIR * h);
  const float2 w9 = make_float2(-c1, -DIR * s1);
  a[1 + 4 * 1] = cmul(a[1 + 4 * 1], w1);
  a[1 + 4 * 2] = cmul(a[1 + 4 * 2], w2);
  a[1 + 4 * 3] = cmul(a[1 + 4 * 3], w3);
  a[2 + 4 * 1] = cmul(a[2 + 4 * 1], w2);
  a[2 + 4 * 2] = cmul_i<DIR>(a[2 + 4 * 2]);  // W16^4 = DIR * i
  a[2 + 4 * 3] = cmul(a[2 + 4 * 3], w6);
  a[3 + 4 * 1] = cmul(a[3 + 4 * 1], w3);
  a[3 + 4 * 2] = cmul(a[3 + 4 * 2], w6);
  a[3 + 4 * 3] = cmul(a[3 + 4 * 3], w9);
  float2 b[16];
  for (int q2 = 0; q2 < 4; ++q2) {
    float2 x0 = a[0 + 4 * q2], x1 = a[1 + 4 * q2], x2 = a[2 + 4 * q2], x3 = a[3 + 4 * q2];
    dft4<DIR>(x0, x1, x2, x3);
    b[0 * 4 + q2] = x0;
    b[1 * 4 + q2] = x1;
    b[2 * 4 + q2] = x2;
    b[3 * 4 + q2] = x3;
  }
  for (int q = 0; q < 16; ++q) a[q] = b[q];
}

template <int R, int DIR>
ATM_HD void dft(float2 (&a)[R]);
template <>
ATM_HD void dft<2, -1>(float2 (&a)[2]) { dft2<-1>(a[0], a[1]); }
template <>
ATM_HD void dft<2, 1>(float2 (&a)[2]) { dft2<1>(a[0], a[1]); }
template <>
ATM_HD void dft<4, -1>(float2 (&a)[4]) { dft4<-1>(a[0], a[1], a[2], a[3]); }
template <>
ATM_HD void dft<4, 1>(float2 (&a)[4]) { dft4<1>(a[0], a[1], a[2], a[3]); }
template <>
ATM_HD void dft<8, -1>(float2 (&a)[8]) { dft8<-1>(a); }
template <>
ATM_HD void dft<8, 1>(float2 (&a)[8]) { dft8<1>(a); }
template <>
ATM_HD void dft<16, -1>(float2 (&a)[16]) { dft16<-1>(a); }
template <>
ATM_HD void dft<16, 1>(float2 (&a)[16]) { dft16<1>(a); }

// ---------------------------------------------------------------------------
// Stockham FFT of length N held by T = N/16 threads, 16 elements each.
//
// Radix plan: radix-16 stages first, the remainder (2, 4, 8 or 16) last.
// Register convention at the first stage's input and the last stage's
// output: v[m] holds element t + m*T.  So an inverse FFT followed by a
// forward FFT of the same row needs no exchange in between, and global loads
// and stores are coalesced across t.
//
// Stage (radix R, L = product of earlier radices), butterfly k in [0, N/R):
//   i = k mod L; inputs x[k + m N/R]; twiddle x_m *= W_{LR}^{i m};
//   DFT_R; outputs y[(k - i) R + i + q L].
// A thread runs butterflies k = t + b T, b in [0, 16/R).
// ---------------------------------------------------------------------------
template <int N>
struct FftPlan;
template <> struct FftPlan<64>   { static constexpr int S = 2; static constexpr int last = 4; };
template <> struct FftPlan<128>  { static constexpr int S = 2; static constexpr int last = 8; };
template <> struct FftPlan<256>  { static constexpr int S = 2; static constexpr int last = 16; };
template <> struct FftPlan<512>  { static constexpr int S = 3; static constexpr int last = 2; };
template <> struct FftPlan<1024> { static constexpr int S = 3; static constexpr int last = 4; };
template <> struct FftPlan<2048> { static constexpr int S = 3; static constexpr int last = 8; };
template <> struct FftPlan<4096> { static constexpr int S = 3; static constexpr int last = 16; };

template <int N, int s>
struct StageRadix {
  static constexpr int value = (s == FftPlan<N>::S - 1) ? FftPlan<N>::last : 16;
};
template <int N, int s>
struct StageL {
  static constexpr int value = (s == 0) ? 1 : StageL<N, s - 1>::value * StageRadix<N, s - 1>::value;
};
template <int N>
struct StageL<N, -1> {
  static constexpr int value = 1;
};

// shared-memory slot of element j: one pad slot per 16 elements
ATM_HD int pad16(int j) { return j + (j >> 4); }
template <int N>
struct Padded {
  static constexpr int value = N + N / 16;
};

// twiddle W_{LR}^{e} for e < L*R, from the length-N table tw[n] = exp(-2 pi i n / N);
// TWPAD = 1: the table is stored with one pad slot per 16 entries (shared memory)
template <int N, int LR, int DIR, int TWPAD = 0>
ATM_HD float2 twiddle(const float2* tw, int e) {
  const int n = e * (N / LR);
  float2 w = tw[TWPAD ? pad16(n) : n];
  return DIR < 0 ? w : cconj(w);
}

// twiddles w[m] = W_{LR}^{i m}, 1 <= m < R.  TWREC = 0: every one from the
// table; TWREC = 1: only W^i, W^2i, W^4i, W^8i from the table, the rest as
// products of at most three of them (a few ulp instead of half an ulp; fewer
// shared-memory loads)
template <int N, int LR, int R, int DIR, int TWPAD, int TWREC>
ATM_HD void stage_twiddles(const float2* tw, int i, float2 (&w)[R]) {
  if constexpr (TWREC == 0) {
#pragma unroll
    for (int m = 1; m < R; ++m) w[m] = twiddle<N, LR, DIR, TWPAD>(tw, i * m);
  } else {
#pragma unroll
    for (int m = 1; m < R; ++m) {
      const int hp = (m >= 8) ? 8 : (m >= 4) ? 4 : (m >= 2) ? 2 : 1;  // highest power of two <= m
      w[m] = (m == hp) ? twiddle<N, LR, DIR, TWPAD>(tw, i * m) : cmul(w[hp], w[m - hp]);
    }
  }
}

// butterflies of stage s on register inputs; results to shared memory
template <int N, int s, int DIR, int TWPAD = 0, int TWREC = 0>
ATM_HD void stage_to_smem(float2 (&v)[16], float2* sm, int t, const float2* tw) {
  constexpr int R = StageRadix<N, s>::value;
  constexpr int L = StageL<N, s>::value;
  constexpr int T = N / 16;
  constexpr int B = 16 / R;
#pragma unroll
  for (int b = 0; b < B; ++b) {
    const int k = t + b * T;
    const int i = k & (L - 1);
    float2 a[R];
#pragma unroll
    for (int m = 0; m < R; ++m) a[m] = v[b + B * m];
    if (L > 1) {
      float2 w[R];
      stage_twiddles<N, L * R, R, DIR, TWPAD, TWREC>(tw, i, w);
#pragma unroll
      for (int m = 1; m < R; ++m) a[m] = cmul(a[m], w[m]);
    }
    dft<R, DIR>(a);
    const int j = (k - i) * R + i;
#pragma unroll
    for (int q = 0; q < R; ++q) sm[pad16(j + q * L)] = a[q];
  }
}

// inputs of stage s from shared memory
template <int N, int s>
ATM_HD void stage_from_smem(float2 (&v)[16], const float2* sm, int t) {
  constexpr int R = StageRadix<N, s>::value;
  constexpr int T = N / 16;
  constexpr int B = 16 / R;
#pragma unroll
  for (int b = 0; b < B; ++b) {
#pragma unroll
    for (int m = 0; m < R; ++m) v[b + B * m] = sm[pad16(t + b * T + m * (N / R))];
  }
}

// last stage: outputs stay in registers, v[m] = element t + m T
template <int N, int DIR, int TWPAD = 0, int TWREC = 0>
ATM_HD void stage_last(float2 (&v)[16], int t, const float2* tw) {
  constexpr int s = FftPlan<N>::S - 1;
  constexpr int R = StageRadix<N, s>::value;
  constexpr int L = StageL<N, s>::value;
  constexpr int T = N / 16;
  constexpr int B = 16 / R;
  float2 o[16];
#pragma unroll
  for (int b = 0; b < B; ++b) {
    const int k = t + b * T;
    const int i = k & (L - 1);  // == k, since k < N/R == L
    float2 a[R];
#pragma unroll
    for (int m = 0; m < R; ++m) a[m] = v[b + B * m];
    float2 w[R];
    stage_twiddles<N, L * R, R, DIR, TWPAD, TWREC>(tw, i, w);
#pragma unroll
    for (int m = 1; m < R; ++m) a[m] = cmul(a[m], w[m]);
    dft<R, DIR>(a);
#pragma unroll
    for (int q = 0; q < R; ++q) o[b + B * q] = a[q];
  }
#pragma unroll
  for (int m = 0; m < 16; ++m) v[m] = o[m];
}

// ---------------------------------------------------------------------------
// Twiddles held in registers.  A persistent pass runs the same butterflies
// (the same i of every stage) for every row or column it transforms, so a
// thread's twiddles never change: it loads, once, the bases W_{LR}^{i p} for
// the powers p = 1, 2, 4, 8 below each stage's radix, and forms the other
// twiddles as products exactly as TWREC = 1 forms them from table loads.  The
// results are TWREC = 1's bit for bit, with no shared-memory twiddle traffic.
// ---------------------------------------------------------------------------
template <int N, int s>
struct StagePowers {
  static constexpr int R = StageRadix<N, s>::value;
  static constexpr int value = R == 16 ? 4 : R == 8 ? 3 : R == 4 ? 2 : 1;
};
template <int N, int s>
struct StageBases {
  static constexpr int value = (s == 0) ? 0 : (16 / StageRadix<N, s>::value) * StagePowers<N, s>::value;
};
template <int N, int s>
struct BasesBefore {
  static constexpr int value = BasesBefore<N, s - 1>::value + StageBases<N, s - 1>::value;
};
template <int N>
struct BasesBefore<N, 0> {
  static constexpr int value = 0;
};
template <int N>
struct TwBases {
  static constexpr int NB = BasesBefore<N, FftPlan<N>::S>::value;
  float2 w[NB > 0 ? NB : 1];  // forward-direction bases; the inverse transform conjugates them
};

template <int N, int s, int TWPAD>
ATM_HD void load_bases_stage(TwBases<N>& tb, const float2* tw, int t) {
  if constexpr (s < FftPlan<N>::S) {
    if constexpr (s > 0) {
      constexpr int R = StageRadix<N, s>::value;
      constexpr int L = StageL<N, s>::value;
      constexpr int T = N / 16;
      constexpr int B = 16 / R;
      constexpr int P = StagePowers<N, s>::value;
      constexpr int off = BasesBefore<N, s>::value;
#pragma unroll
      for (int b = 0; b < B; ++b) {
        const int i = (t + b * T) & (L - 1);
#pragma unroll
        for (int j = 0; j < P; ++j) tb.w[off + b * P + j] = twiddle<N, L * R, -1, TWPAD>(tw, i << j);
      }
    }
    load_bases_stage<N, s + 1, TWPAD>(tb, tw, t);
  }
}

// the bases of thread t (N / 16 threads per transform) from the table tw
template <int N, int TWPAD = 0>
ATM_HD void load_twiddle_bases(TwBases<N>& tb, const float2* tw, int t) {
  load_bases_stage<N, 0, TWPAD>(tb, tw, t);
}

// base w8 of a radix-16 butterfly (forward bases; the inverse conjugates)
template <int N>
ATM_HD float2 w8_of(const TwBases<N>& tb, int first, int DIR) {
  const float2 base = tb.w[first + 3];
  return DIR < 0 ? base : cconj(base);
}

// a[m] *= W_{LR}^{i m}, 1 <= m < R, for butterfly b of stage s, with the
// twiddles formed from the bases: w1, w2, w4, w8 are bases; w3 = w2 w1,
// w(4 + j) = w4 wj, w(8 + j) = w8 wj (j < 4, j < 8).  Each twiddle is applied
// as soon as it is formed, so only w1 .. w7 stay live for the w(8 + j).
template <int N, int s, int DIR, int R>
ATM_HD void apply_twiddles_reg(const TwBases<N>& tb, int b, float2 (&a)[R]) {
  constexpr int P = StagePowers<N, s>::value;
  constexpr int off = BasesBefore<N, s>::value;
  float2 w[R < 8 ? R : 8];
#pragma unroll
  for (int m = 1; m < R; ++m) {
    const int hp = (m >= 8) ? 8 : (m >= 4) ? 4 : (m >= 2) ? 2 : 1;
    float2 wm;
    if (m == hp) {
      const int lg = (m == 8) ? 3 : (m == 4) ? 2 : (m == 2) ? 1 : 0;
      const float2 base = tb.w[off + b * P + lg];
      wm = DIR < 0 ? base : cconj(base);
    } else {
      wm = cmul(m >= 8 ? w8_of(tb, off + b * P, DIR) : w[hp], w[m - hp]);
    }
    if (m < 8) w[m] = wm;
    a[m] = cmul(a[m], wm);
  }
}

// stage_to_smem / stage_last with the twiddles from the bases
template <int N, int s, int DIR>
ATM_HD void stage_to_smem_reg(float2 (&v)[16], float2* sm, int t, const TwBases<N>& tb) {
  constexpr int R = StageRadix<N, s>::value;
  constexpr int L = StageL<N, s>::value;
  constexpr int T = N / 16;
  constexpr int B = 16 / R;
#pragma unroll
  for (int b = 0; b < B; ++b) {
    const int k = t + b * T;
    const int i = k & (L - 1);
    float2 a[R];
#pragma unroll
    for (int m = 0; m < R; ++m) a[m] = v[b + B * m];
    if (L > 1) apply_twiddles_reg<N, s, DIR, R>(tb, b, a);
    dft<R, DIR>(a);
    const int j = (k - i) * R + i;
#pragma unroll
    for (int q = 0; q < R; ++q) sm[pad16(j + q * L)] = a[q];
  }
}

template <int N, int DIR>
ATM_HD void stage_last_reg(float2 (&v)[16], int t, const TwBases<N>& tb) {
  constexpr int s = FftPlan<N>::S - 1;
  constexpr int R = StageRadix<N, s>::value;
  constexpr int B = 16 / R;
  float2 o[16];
#pragma unroll
  for (int b = 0; b < B; ++b) {
    float2 a[R];
#pragma unroll
    for (int m = 0; m < R; ++m) a[m] = v[b + B * m];
    apply_twiddles_reg<N, s, DIR, R>(tb, b, a);
    dft<R, DIR>(a);
#pragma unroll
    for (int q = 0; q < R; ++q) o[b + B * q] = a[q];
  }
#pragma unroll
  for (int m = 0; m < 16; ++m) v[m] = o[m];
}

// ---------------------------------------------------------------------------
// Warp FFT: length N = 32 R (R = 32 or 64) held by 32 lanes, R elements each.
// Lane j holds element j + 32 m in v[m], before and after a transform, so a
// forward transform, a pointwise product and an inverse transform chain with
// no reordering.  With n = j + 32 m and k = kb + R ka:
//   X[kb + R ka] = sum_j W_32^(j ka) W_N^(j kb) sum_m x[j + 32 m] W_R^(m kb),
// W_L = exp(DIR 2 pi i / L).  A transform is
//   stage 1: DFT_R over m in registers, then the twiddle W_N^(j kb), then
//            Y[j][kb] into an exchange buffer (one 32 x R transpose);
//   stage 2: lane j takes kb = j + 32 h (h < R / 32), reads Y[0..31][kb] and
//            runs DFT_32 over them in registers.
// X[j + 32 h + R ka] is element j + 32 (h + (R / 32) ka), held in
// v[h + (R / 32) ka]: the input's layout.  Compared with the radix-16
// Stockham form (two exchanges per transform for N = 2048) the warp form
// exchanges once, and within one warp (or one lane group) only.
// ---------------------------------------------------------------------------
// cos(pi k / 32), k = 0..16 (FP64 values rounded to FP32)
ATM_HD constexpr float cos_pi32(int k) {
  return k == 0    ? 1.0f
         : k == 1  ? 0.99518472667219692873f
         : k == 2  ? 0.98078528040323043058f
         : k == 3  ? 0.95694033573220882438f
         : k == 4  ? 0.92387953251128673848f
         : k == 5  ? 0.88192126434835504956f
         : k == 6  ? 0.83146961230254523567f
         : k == 7  ? 0.77301045336273699338f
         : k == 8  ? 0.70710678118654757274f
         : k == 9  ? 0.63439328416364548779f
         : k == 10 ? 0.55557023301960228867f
         : k == 11 ? 0.47139673682599780857f
         : k == 12 ? 0.38268343236508983729f
         : k == 13 ? 0.29028467725446233105f
         : k == 14 ? 0.19509032201612833135f
         : k == 15 ? 0.09801714032956077016f
                   : 0.0f;
}

// W_64^e = exp(DIR 2 pi i e / 64)
template <int DIR>
ATM_HD constexpr float2 w64(int e) {
  e &= 63;
  const int q = e >> 4, r = e & 15;
  const float c = cos_pi32(r), s = cos_pi32(16 - r);  // cos, sin of pi r / 32
  const float cr = q == 0 ? c : q == 1 ? -s : q == 2 ? -c : s;
  const float sr = q == 0 ? s : q == 1 ? c : q == 2 ? -s : -c;
  return float2{cr, DIR < 0 ? -sr : sr};
}

// a W_R^e for R dividing 64 and e known when the caller is unrolled; the
// quarter turns are exact
template <int R, int DIR>
ATM_HD float2 twc(float2 a, int e) {
  const int e64 = (e * (64 / R)) & 63;
  if (e64 == 0) return a;
  if (e64 == 16) return cmul_i<DIR>(a);
  if (e64 == 32) return make_float2(-a.x, -a.y);
  if (e64 == 48) return cmul_i<-DIR>(a);
  return cmul(a, w64<DIR>(e64));
}

// natural-order DFT of length R1 R2 in registers, b_q = sum_m a_m W_(R1 R2)^(m q):
// with m = m1 + R1 m2 and q = q2 + R2 q1, DFT_R2 over m2, the twiddle
// W^(m1 q2), DFT_R1 over m1.  Streamed: input m passes through pre(m, x) as
// it is gathered and output q goes to emit(q, y) as soon as its group is
// formed, so that beside the R elements only one group of R1 or R2 values
// (and whatever pre / emit load for it) is live at a time.
template <int R1, int R2, int DIR, class PreF, class EmitF>
ATM_HD void dft_2l(float2 (&a)[R1 * R2], PreF&& pre, EmitF&& emit) {
  constexpr int R = R1 * R2;
#pragma unroll
  for (int m1 = 0; m1 < R1; ++m1) {
    float2 t[R2];
#pragma unroll
    for (int m2 = 0; m2 < R2; ++m2) t[m2] = pre(m1 + R1 * m2, a[m1 + R1 * m2]);
    dft<R2, DIR>(t);
#pragma unroll
    for (int q2 = 0; q2 < R2; ++q2) a[m1 + R1 * q2] = twc<R, DIR>(t[q2], m1 * q2);
  }
#pragma unroll
  for (int q2 = 0; q2 < R2; ++q2) {
    float2 t[R1];
#pragma unroll
    for (int m1 = 0; m1 < R1; ++m1) t[m1] = a[m1 + R1 * q2];
    dft<R1, DIR>(t);
#pragma unroll
    for (int q1 = 0; q1 < R1; ++q1) emit(q2 + R2 * q1, t[q1]);
  }
}

// the radix split of the warp FFT's in-register DFTs
template <int R>
struct WfftSplit;
template <> struct WfftSplit<32> { static constexpr int R1 = 4, R2 = 8; };
template <> struct WfftSplit<64> { static constexpr int R1 = 8, R2 = 8; };

struct WfftNoPre {
  ATM_HD float2 operator()(int, float2 x) const { return x; }
};

// stage 1 of lane j: pre(m, x) scales input m on the way in (a pointwise
// product between two transforms), tw(kb) returns exp(-2 pi i j kb / N) (the
// forward direction; the inverse conjugates it), put(kb, y) stores Y[j][kb]
template <int R, int DIR, class TwF, class PutF, class PreF = WfftNoPre>
ATM_HD void wfft_stage1(float2 (&v)[R], TwF&& tw, PutF&& put, PreF&& pre = PreF()) {
  dft_2l<WfftSplit<R>::R1, WfftSplit<R>::R2, DIR>(v, pre, [&](int kb, float2 y) {
    if (kb == 0) {
      put(0, y);
    } else {
      const float2 w = tw(kb);
      put(kb, cmul(y, DIR < 0 ? w : cconj(w)));
    }
  });
}

// stage 2 of lane j of an L-lane transform (L = 32 or 64): get(h, jj) returns
// Y[jj][j + L h]; output element q (the transform's element j + L q) passes
// through post(q, y) as it is formed.  With L lanes the derivation above
// reads n = j + L m, k = kb + R ka, N = L R: stage 1 is the same DFT_R over
// m with the twiddle W_N^(j kb), stage 2 a DFT_L over j per kb = j + L h.
template <int R, int DIR, int L = 32, class GetF, class PostF = WfftNoPre>
ATM_HD void wfft_stage2(float2 (&v)[R], GetF&& get, PostF&& post = PostF()) {
  static_assert(L == 32 || L == 64, "warp FFTs of 32 or 64 lanes");
  constexpr int H = R / L;
  static_assert(H >= 1 && H * L == R, "stage 2 needs R a multiple of L");
#pragma unroll
  for (int h = 0; h < H; ++h) {
    float2 u[L];
#pragma unroll
    for (int jj = 0; jj < L; ++jj) u[jj] = get(h, jj);
    dft_2l<WfftSplit<L>::R1, WfftSplit<L>::R2, DIR>(u, WfftNoPre(),
                                                       [&](int ka, float2 y) { v[h + H * ka] = post(h + H * ka, y); });
  }
}

// exchange-buffer slot of Y[jj][kb] for one transform of 32 x R elements:
// row kb of 32 slots, the lane index XOR-swizzled so that the stores of one
// kb (lanes jj) and the loads of one jj (lanes kb = j + 32 h) both spread
// over the 16 eight-byte bank pairs of each half warp.  `sw` is the
// swizzle of row kb: kb & 15 when the 32 lanes are one warp; (kb & 3) |
// (c << 2) when a warp holds lanes of four transforms c (8 lanes each).
ATM_HD int wfft_slot(int kb, int jj, int sw) { return kb * 32 + (jj ^ sw); }
// the same for an L-lane transform: row kb of L slots
template <int L>
ATM_HD int wfft_slot_l(int kb, int jj, int sw) { return kb * L + (jj ^ sw); }

// ---------------------------------------------------------------------------
// fixed-point phase: turns(j) = frac(j * S + O) held as a 64-bit binary
// fraction; the product wraps modulo one turn exactly.  Returned as
// half-turns in [-1, 1) for sincospif.
// ---------------------------------------------------------------------------
ATM_HD uint64_t turns_to_fixed(double turns) {
  double f = turns - floor(turns);  // [0, 1)
  // split to keep all 64 bits: hi 32 bits then the remainder
  double hi = floor(f * 4294967296.0);
  double lo = (f * 4294967296.0 - hi) * 4294967296.0;
  uint64_t h = (uint64_t)hi;
  uint64_t l = (uint64_t)lo;
  return (h << 32) + l;
}

ATM_HD float fixed_to_halfturns(uint64_t x) {
  int32_t top = (int32_t)(uint32_t)(x >> 32);
  return (float)top * 4.656612873077392578125e-10f;  // 2^-31
}

// ---------------------------------------------------------------------------
// Bessel J_0..J_{D-1}(a) by Miller's backward recurrence, normalised with
// J_0 + 2 sum_k J_2k = 1.  Used for the Jacobi-Anger (Chebyshev) expansion
//   exp(i a t) = J_0(a) + 2 sum_{n>=1} i^n J_n(a) T_n(t),  |t| <= 1.
// ---------------------------------------------------------------------------
ATM_HD void bessel_j(double a, int D, double* J /* [D] */) {
  const double sgn = a < 0 ? -1.0 : 1.0;
  a = fabs(a);
  if (a < 1e-30) {
    J[0] = 1.0;
    for (int n = 1; n < D; ++n) J[n] = 0.0;
    return;
  }
  // orders from n_top on are below 1e-18, since |J_n(a)| <= (a/2)^n / n!:
  // most low annuli have a << 1, and their recurrences get much shorter
  int n_top = D;
  double bound = 1.0;
  for (int n = 1; n < D; ++n) {
    bound *= 0.5 * a / n;
    if (bound < 1e-18) {
      n_top = n;
      break;
    }
  }
  // start well above both n_top and a: J_n0(a) is then below 1e-16 of the
  // kept orders (checked against scipy's jv for D <= 64 and every |a| up to
  // the largest the engine pairs with D, 2 |J_D(a)| < 1e-10: max error 9e-16)
  const int n0 = n_top + (int)a / 2 + 20;
  const double two_over_a = 2.0 / a;  // one FP64 divide, not one per step
  double jp1 = 0.0, j = 1e-200, norm = 0.0;
  for (int n = 0; n < D; ++n) J[n] = 0.0;
  for (int n = n0; n >= 1; --n) {
    // j = J_n (unnormalised), jp1 = J_{n+1}
    if (n < D) J[n] = j;
    if ((n & 1) == 0) norm += 2.0 * j;
    const double jm1 = ((double)n * two_over_a) * j - jp1;
    jp1 = j;
    j = jm1;
    if (fabs(j) > 1e200) {  // rescale to stay in range
      j *= 1e-200;
      jp1 *= 1e-200;
      norm *= 1e-200;
      for (int m = 0; m < D; ++m) J[m] *= 1e-200;
    }
  }
  // j = J_0
  norm += j;
  J[0] = j;
  const double inv = 1.0 / norm;
  for (int n = 0; n < D; ++n) J[n] *= inv;
  if (sgn < 0)
    for (int n = 1; n < D; n += 2) J[n] = -J[n];
}

// ---------------------------------------------------------------------------
// Philox4x32-10 counter-based generator (Salmon, Moraes, Dror and Shaw,
// "Parallel random numbers: as easy as 1, 2, 3", SC 2011): 10 rounds of
// multiply-xor with a Weyl key schedule.  Stateless: (key, counter) -> 4 words.
// ---------------------------------------------------------------------------
struct Philox4 {
  uint32_t v[4];
};

ATM_HD uint32_t mulhi32(uint32_t a, uint32_t b) { return (uint32_t)(((uint64_t)a * (uint64_t)b) >> 32); }

ATM_HD Philox4 philox4x32_10(Philox4 c, uint32_t k0, uint32_t k1) {
  const uint32_t M0 = 0xD2511F53u, M1 = 0xCD9E8D57u, W0 = 0x9E3779B9u, W1 = 0xBB67AE85u;
  for (int r = 0; r < 10; ++r) {
    const uint32_t hi0 = mulhi32(M0, c.v[0]), lo0 = M0 * c.v[0];
    const uint32_t hi1 = mulhi32(M1, c.v[2]), lo1 = M1 * c.v[2];
    Philox4 n;
    n.v[0] = hi1 ^ c.v[1] ^ k0;
    n.v[1] = lo1;
    n.v[2] = hi0 ^ c.v[3] ^ k1;
    n.v[3] = lo0;
    c = n;
    k0 += W0;
    k1 += W1;
  }
  return c;
}

// uniform in [0, 1) from the top 24 bits
ATM_HD float u01(uint32_t x) { return (float)(x >> 8) * 5.9604644775390625e-8f; }
// uniform in (0, 1]
ATM_HD float u01_open0(uint32_t x) { return ((float)(x >> 8) + 1.0f) * 5.9604644775390625e-8f; }

}  // namespace atm
