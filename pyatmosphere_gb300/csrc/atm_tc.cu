// 5th-generation tensor-core GEMM for the screen synthesis (sm_103a).
//
//   phi_G[s][y][x] = scale * sum_k A[s][y][k] B[s][x][k]
//
// Operands are FP32 values split into two scaled FP16 slices,
//   a = a_hi + a_lo / 2^11,  a_hi = fp16(a),  a_lo = fp16((a - a_hi) 2^11),
// so that a_hi b_hi + (a_hi b_lo + a_lo b_hi) / 2^11 carries ~22 bits: three
// tcgen05.mma (kind::f16, FP32 accumulation) per K step of 16 into two TMEM
// accumulators (D0 = sum hi.hi, D1 = sum of the cross terms, 2 x 256
// columns), combined in the epilogue.  Accumulating the cross terms apart
// matters: added into D0 they lose their low bits to the tensor core's
// alignment of small addends (2.8e-6 instead of < 2e-6 relative at K = 768).
//
// tc_gemm_tma_kernel (default): persistent, warp-specialised.  Warp 0 loads
// the four 128-byte-swizzled operand boxes of a K tile with TMA
// (cp.async.bulk.tensor) into a ring of stages, running ahead into the next
// tile; warp 1 issues the MMAs; warps 2-9 drain the accumulators (tcgen05.ld,
// combine, scale, optionally add 1-D phases fold_y[y] + fold_x[x], store).
// Default: 128 x 256 output tiles, two stages and one accumulator pair
// (2 x 256 TMEM columns).  Its MMAs run near the tensor peak (the operands of
// a 128-wide MMA need more shared-memory bandwidth per FLOP), but the pair
// must be drained before the next tile starts, so the drain is kept short:
// each epilogue warp reads its TMEM block, releases the pair after its last
// read, and stores the block through a 4 KB swizzled staging buffer with a
// TMA tensor store (one store per 32 x 32 block instead of 32 rows per store
// instruction).  The 128 x 128 form (three stages, two accumulator pairs:
// the drain overlaps the next tile's MMAs, global stores from registers)
// stays behind ATM_FLAG_TC_N128.  mbarriers: full / empty per stage,
// full / empty per accumulator pair.
// tc_gemm_kernel: the first form, one CTA per tile, operands through cp.async
// by all threads (kept for comparison and as the fallback when the driver
// offers no tensor-map encoder).
//
// Every mbarrier wait is bounded by %globaltimer: on timeout a CTA records an
// error, waits (bounded) for its copies and MMAs in flight, frees its TMEM
// and returns.
#include <cuda.h>  // CUtensorMap and the driver enums (the encoder is fetched at run time)
#include <cuda_bf16.h>
#include <cuda_fp16.h>

#include <algorithm>
#include <cstdint>
#include <mutex>

#include "../../include/atm.h"
#include "atm_internal.h"

namespace atm {
namespace {

constexpr int TM = 128, TN = 256, TK = 64;             // tile
constexpr int ROWB = TK * 2;                           // 128 bytes per tile row
constexpr int A_SLICE = TM * ROWB;                     // 16 KB
constexpr int B_SLICE = TN * ROWB;                     // 32 KB
constexpr int STAGE = 2 * A_SLICE + 2 * B_SLICE;       // 96 KB: A_hi, A_lo, B_hi, B_lo
constexpr int SMEM = 2 * STAGE + 1024;                 // + alignment slack
constexpr int THREADS = 128;
constexpr unsigned long long kTimeoutNs = 2000000000ull;  // 2 s

__device__ int g_tc_error;
// budget of the persistent form's waits for work (operands, an accumulator,
// a free stage); atm_set_wait_budget changes it.  Drains keep kTimeoutNs.
__device__ unsigned long long g_tc_wait_ns = kTimeoutNs;

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ uint64_t globaltimer() {
  uint64_t t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

__device__ __forceinline__ void cp_async16(uint32_t dst, const void* src) {
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(dst), "l"(src) : "memory");
}

__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;\n" ::"r"(bar), "r"(count) : "memory");
}

// bounded wait for the phase with the given parity; false on timeout
__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity) {
  const uint64_t t0 = globaltimer();
  while (true) {
    uint32_t ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(ok)
        : "r"(bar), "r"(parity)
        : "memory");
    if (ok) return true;
    if (globaltimer() - t0 > kTimeoutNs) return false;
  }
}

// SM100 shared-memory matrix descriptor: K-major, SWIZZLE_128B, 8-row groups
// 1024 bytes apart (stride byte offset), version 1.
__device__ __forceinline__ uint64_t smem_desc(uint32_t addr) {
  uint64_t d = 0;
  d |= (uint64_t)((addr & 0x3FFFF) >> 4);       // start address
  d |= (uint64_t)1 << 16;                       // leading byte offset (unused for swizzled K-major)
  d |= (uint64_t)(1024 >> 4) << 32;             // stride byte offset
  d |= (uint64_t)1 << 46;                       // version
  d |= (uint64_t)2 << 61;                       // SWIZZLE_128B
  return d;
}

// instruction descriptor: kind::f16, A = B = FP16, D = FP32, both K-major
__host__ __device__ constexpr uint32_t instr_desc() {
  return (1u << 4)                          // D format F32
         | (0u << 7) | (0u << 10)           // A, B format F16
         | ((uint32_t)(TN >> 3) << 17)      // N
         | ((uint32_t)(TM >> 4) << 24);     // M
}

__device__ __forceinline__ void mma_f16(uint32_t d_tmem, uint64_t a, uint64_t b, uint32_t accumulate) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
      " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(d_tmem),
      "l"(a), "l"(b), "r"(instr_desc()), "r"(accumulate)
      : "memory");
}

__device__ __forceinline__ void mma_commit(uint32_t bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(bar)
               : "memory");
}

// one tile row chunk: 16 bytes = 8 FP16 of K, swizzled within its 128-byte row
__device__ __forceinline__ uint32_t swz(int row, int chunk) {
  return (uint32_t)(row * ROWB + ((chunk ^ (row & 7)) << 4));
}

struct TcArgs {
  const __half* a_hi;   // [S][M][Kp]
  const __half* a_lo;
  const __half* b_hi;   // [S][Nn][Kp]
  const __half* b_lo;
  float* out;           // [S][M][Nn]
  int M, Nn, Kp;
  float scale;          // applied to the result (1/2pi for the screen)
};

__device__ __forceinline__ void load_stage(const TcArgs& a, int s, int m0, int n0, int kt, uint32_t st) {
  const size_t plane_a = (size_t)a.M * a.Kp, plane_b = (size_t)a.Nn * a.Kp;
  const __half* ah = a.a_hi + (size_t)s * plane_a + (size_t)m0 * a.Kp + kt * TK;
  const __half* al = a.a_lo + (size_t)s * plane_a + (size_t)m0 * a.Kp + kt * TK;
  const __half* bh = a.b_hi + (size_t)s * plane_b + (size_t)n0 * a.Kp + kt * TK;
  const __half* bl = a.b_lo + (size_t)s * plane_b + (size_t)n0 * a.Kp + kt * TK;
  for (int q = threadIdx.x; q < TM * 8; q += THREADS) {
    const int row = q >> 3, c = q & 7;
    cp_async16(st + swz(row, c), ah + (size_t)row * a.Kp + c * 8);
    cp_async16(st + A_SLICE + swz(row, c), al + (size_t)row * a.Kp + c * 8);
  }
  for (int q = threadIdx.x; q < TN * 8; q += THREADS) {
    const int row = q >> 3, c = q & 7;
    cp_async16(st + 2 * A_SLICE + swz(row, c), bh + (size_t)row * a.Kp + c * 8);
    cp_async16(st + 2 * A_SLICE + B_SLICE + swz(row, c), bl + (size_t)row * a.Kp + c * 8);
  }
}

__global__ void __launch_bounds__(THREADS, 1) tc_gemm_kernel(TcArgs a) {
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  __shared__ __align__(8) uint64_t bars[3];
  __shared__ uint32_t tmem_holder;
  __shared__ int abort_flag;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int s = blockIdx.z, m0 = blockIdx.y * TM, n0 = blockIdx.x * TN;
  const uint32_t base = (smem_u32(smem_raw) + 1023) & ~1023u;
  const uint32_t stage[2] = {base, base + STAGE};
  const int KT = a.Kp / TK;

  if (tid == 0) {
    mbar_init(smem_u32(&bars[0]), 1);
    mbar_init(smem_u32(&bars[1]), 1);
    mbar_init(smem_u32(&bars[2]), 1);
    abort_flag = 0;
    asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], 512;\n" ::"r"(smem_u32(&tmem_holder))
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n" ::: "memory");
  }
  asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
  const uint32_t tmem = tmem_holder;
  const uint32_t d0 = tmem, d1 = tmem + TN;  // columns [0, 256) and [256, 512)

  load_stage(a, s, m0, n0, 0, stage[0]);
  asm volatile("cp.async.commit_group;\n" ::: "memory");
  if (KT > 1) load_stage(a, s, m0, n0, 1, stage[1]);
  asm volatile("cp.async.commit_group;\n" ::: "memory");

  bool ok = true;
  for (int kt = 0; kt < KT; ++kt) {
    const int st = kt & 1;
    asm volatile("cp.async.wait_group 1;\n" ::: "memory");
    asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
    __syncthreads();
    if (tid == 0) {
      asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
      const uint32_t sa = stage[st], sal = sa + A_SLICE, sb = sa + 2 * A_SLICE, sbl = sb + B_SLICE;
#pragma unroll
      for (int k4 = 0; k4 < TK / 16; ++k4) {
        const uint32_t off = k4 * 32;  // 16 FP16 of K = 32 bytes inside the swizzle atom
        const uint32_t acc = (kt > 0 || k4 > 0) ? 1u : 0u;
        mma_f16(d0, smem_desc(sa + off), smem_desc(sb + off), acc);
        mma_f16(d1, smem_desc(sa + off), smem_desc(sbl + off), acc);
        mma_f16(d1, smem_desc(sal + off), smem_desc(sb + off), 1u);
      }
      mma_commit(smem_u32(&bars[st]));
    }
    if (kt + 2 < KT) {
      // the MMAs of k tile kt read stage st; refill it once they are done
      if (!mbar_wait(smem_u32(&bars[st]), (uint32_t)((kt >> 1) & 1))) ok = false;
      if (!ok) abort_flag = 1;
      __syncthreads();
      if (abort_flag) break;
      load_stage(a, s, m0, n0, kt + 2, stage[st]);
    }
    asm volatile("cp.async.commit_group;\n" ::: "memory");
  }
  asm volatile("cp.async.wait_all;\n" ::: "memory");

  // all MMAs done: the last commit covers every earlier MMA of this thread
  if (tid == 0 && !abort_flag) mma_commit(smem_u32(&bars[2]));
  __syncthreads();
  if (!abort_flag && !mbar_wait(smem_u32(&bars[2]), 0)) abort_flag = 1;
  asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
  __syncthreads();

  if (!abort_flag) {
    const int row = warp * 32 + lane;
    float* out = a.out + ((size_t)s * a.M + m0 + row) * a.Nn + n0;
    const uint32_t lane_addr = (uint32_t)(warp * 32) << 16;
#pragma unroll 1
    for (int c0 = 0; c0 < TN; c0 += 32) {
      uint32_t h[32], l[32];
      asm volatile(
          "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
          "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];\n"
          : "=r"(h[0]), "=r"(h[1]), "=r"(h[2]), "=r"(h[3]), "=r"(h[4]), "=r"(h[5]), "=r"(h[6]), "=r"(h[7]),
            "=r"(h[8]), "=r"(h[9]), "=r"(h[10]), "=r"(h[11]), "=r"(h[12]), "=r"(h[13]), "=r"(h[14]), "=r"(h[15]),
            "=r"(h[16]), "=r"(h[17]), "=r"(h[18]), "=r"(h[19]), "=r"(h[20]), "=r"(h[21]), "=r"(h[22]), "=r"(h[23]),
            "=r"(h[24]), "=r"(h[25]), "=r"(h[26]), "=r"(h[27]), "=r"(h[28]), "=r"(h[29]), "=r"(h[30]), "=r"(h[31])
          : "r"(d0 + lane_addr + c0));
      asm volatile(
          "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
          "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];\n"
          : "=r"(l[0]), "=r"(l[1]), "=r"(l[2]), "=r"(l[3]), "=r"(l[4]), "=r"(l[5]), "=r"(l[6]), "=r"(l[7]),
            "=r"(l[8]), "=r"(l[9]), "=r"(l[10]), "=r"(l[11]), "=r"(l[12]), "=r"(l[13]), "=r"(l[14]), "=r"(l[15]),
            "=r"(l[16]), "=r"(l[17]), "=r"(l[18]), "=r"(l[19]), "=r"(l[20]), "=r"(l[21]), "=r"(l[22]), "=r"(l[23]),
            "=r"(l[24]), "=r"(l[25]), "=r"(l[26]), "=r"(l[27]), "=r"(l[28]), "=r"(l[29]), "=r"(l[30]), "=r"(l[31])
          : "r"(d1 + lane_addr + c0));
      asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory");
      constexpr float lo_scale = 1.f / kTcLoScale;
#pragma unroll
      for (int j = 0; j < 32; j += 4) {
        float4 o;
        o.x = (__uint_as_float(h[j + 0]) + __uint_as_float(l[j + 0]) * lo_scale) * a.scale;
        o.y = (__uint_as_float(h[j + 1]) + __uint_as_float(l[j + 1]) * lo_scale) * a.scale;
        o.z = (__uint_as_float(h[j + 2]) + __uint_as_float(l[j + 2]) * lo_scale) * a.scale;
        o.w = (__uint_as_float(h[j + 3]) + __uint_as_float(l[j + 3]) * lo_scale) * a.scale;
        *reinterpret_cast<float4*>(out + c0 + j) = o;
      }
    }
  } else if (tid == 0) {
    atomicExch(&g_tc_error, 1);
  }
  asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
  __syncthreads();
  if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, 512;\n" ::"r"(tmem) : "memory");
}

// ---------------------------------------------------------------------------
// persistent, warp-specialised form: TMA producer, MMA issuer, epilogue warps.
// Template: output tile 128 x TNT, STG operand stages, NACC accumulator pairs
// in TMEM (NACC = 2: the epilogue of one tile overlaps the next tile's MMAs).
//   <256, 2, 1>: 2 x 256 TMEM columns, 96 KB stages
//   <128, 3, 2>: 4 x 128 TMEM columns, 64 KB stages
// ---------------------------------------------------------------------------
constexpr int P_THREADS = 320;    // warp 0: TMA, warp 1: MMA, warps 2-9: epilogue
constexpr int EPI_THREADS = 256;  // two warps per TMEM lane quarter, each draining half of the columns

// EPI = 1: each epilogue warp writes its 32 x 32 result blocks into its own
// 4 KB staging buffer (128-byte swizzle) and one lane stores the block with a
// TMA tensor store, instead of 32 rows per store instruction from registers.
constexpr int EPI_STAGE = 32 * 32 * 4;  // bytes per epilogue warp
template <int TNT, int STG, int NACC, int EPI = 0>
struct TmaCfg {
  static constexpr int B_SL = TNT * ROWB;                 // one FP16 slice of the B tile
  static constexpr int STAGE_B = 2 * A_SLICE + 2 * B_SL;  // A_hi, A_lo, B_hi, B_lo
  static constexpr int SMEM = STG * STAGE_B + (EPI ? 8 * EPI_STAGE : 0) + 1024;
  static_assert(NACC * 2 * TNT <= 512, "accumulators exceed the 512 TMEM columns");
  static_assert(SMEM <= 227 * 1024 - 256, "stages exceed shared memory");
  static_assert(STAGE_B % 1024 == 0, "staging buffers need 1024-byte alignment for the 128-byte swizzle");
};

template <int NT>
__host__ __device__ constexpr uint32_t instr_desc_n() {
  return (1u << 4)                          // D format F32
         | (0u << 7) | (0u << 10)           // A, B format F16
         | ((uint32_t)(NT >> 3) << 17)      // N
         | ((uint32_t)(TM >> 4) << 24);     // M
}

template <int NT>
__device__ __forceinline__ void mma_f16_n(uint32_t d_tmem, uint64_t a, uint64_t b, uint32_t accumulate) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
      " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(d_tmem),
      "l"(a), "l"(b), "r"(instr_desc_n<NT>()), "r"(accumulate)
      : "memory");
}

struct TmaOperands {
  CUtensorMap ah, al, bh, bl;  // [S][rows][Kp] FP16, boxes of 64 (K) x 128 or TNT rows
};

__device__ __forceinline__ void tma_load_3d(uint32_t dst, const CUtensorMap* map, int x, int y, int z, uint32_t bar) {
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], "
      "[%5];\n" ::"r"(dst),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(z), "r"(bar)
      : "memory");
}

__device__ __forceinline__ void tma_store_3d(const CUtensorMap* map, uint32_t src, int x, int y, int z) {
  asm volatile("cp.async.bulk.tensor.3d.global.shared::cta.tile.bulk_group [%0, {%1, %2, %3}], [%4];\n" ::"l"(
                   reinterpret_cast<uint64_t>(map)),
               "r"(x), "r"(y), "r"(z), "r"(src)
               : "memory");
}
__device__ __forceinline__ void bulk_commit() { asm volatile("cp.async.bulk.commit_group;\n" ::: "memory"); }
// the staging buffer may be rewritten: every committed store has read it
__device__ __forceinline__ void bulk_wait_read_all() { asm volatile("cp.async.bulk.wait_group.read 0;\n" ::: "memory"); }
// every committed store has completed
__device__ __forceinline__ void bulk_wait_all() { asm volatile("cp.async.bulk.wait_group 0;\n" ::: "memory"); }
__device__ __forceinline__ void mbar_arrive_expect_tx(uint32_t bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(bar), "r"(bytes) : "memory");
}

__device__ __forceinline__ void mbar_arrive(uint32_t bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];\n" ::"r"(bar) : "memory");
}

// bounded wait that also gives up once another role has set the abort flag;
// a timeout sets the flag itself
__device__ __forceinline__ bool mbar_wait_or_abort(uint32_t bar, uint32_t parity, volatile int* abort_flag) {
  const uint64_t t0 = globaltimer();
  const unsigned long long limit = g_tc_wait_ns;
  for (uint32_t spin = 1;; ++spin) {
    uint32_t ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(ok)
        : "r"(bar), "r"(parity)
        : "memory");
    if (ok) return true;
    if ((spin & 15) == 0) {
      if (*abort_flag) return false;
      if (globaltimer() - t0 > limit) {
        *abort_flag = 1;
        return false;
      }
    }
  }
}

__device__ __forceinline__ void tile_coords(int t, int tiles_m, int tiles_n, int tn, int* s, int* m0, int* n0) {
  const int per = tiles_m * tiles_n;
  *s = t / per;
  const int r = t - *s * per;
  *m0 = (r / tiles_n) * TM;
  *n0 = (r - (r / tiles_n) * tiles_n) * tn;
}

template <int TNT, int STG, int NACC, int EPI = 0>
__global__ void __launch_bounds__(P_THREADS, 1)
    tc_gemm_tma_kernel(const __grid_constant__ TmaOperands ops, const __grid_constant__ CUtensorMap outmap,
                       float* __restrict__ out, int S, int M, int Nn, int Kp, float scale,
                       const float* __restrict__ fold_y, const float* __restrict__ fold_x, int* status) {
  using Cfg = TmaCfg<TNT, STG, NACC, EPI>;
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  __shared__ __align__(8) uint64_t full_bar[STG], empty_bar[STG], accf_bar[NACC], acce_bar[NACC], drain_bar;
  __shared__ uint32_t tmem_holder;
  __shared__ int abort_word;
  volatile int* abort_flag = &abort_word;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const uint32_t base = (smem_u32(smem_raw) + 1023) & ~1023u;
  const int KT = Kp / TK;
  const int tiles_m = M / TM, tiles_n = Nn / TNT;
  const int n_tiles = S * tiles_m * tiles_n;

  if (threadIdx.x == 0) {
    for (int i = 0; i < STG; ++i) {
      mbar_init(smem_u32(&full_bar[i]), 1);
      mbar_init(smem_u32(&empty_bar[i]), 1);
    }
    for (int i = 0; i < NACC; ++i) {
      mbar_init(smem_u32(&accf_bar[i]), 1);
      mbar_init(smem_u32(&acce_bar[i]), EPI_THREADS);
    }
    mbar_init(smem_u32(&drain_bar), 1);
    *abort_flag = 0;
    asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
  }
  if (warp == 1) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], 512;\n" ::"r"(smem_u32(&tmem_holder))
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n" ::: "memory");
  }
  asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
  const uint32_t tmem = tmem_holder;

  if (warp == 0) {
    if (lane == 0) {
      // ---- TMA producer ----
      int stage = 0;
      uint32_t phase = 0;
      bool issued[STG] = {};
      uint32_t issued_phase[STG] = {};
      bool stop = false;
      for (int t = blockIdx.x; t < n_tiles && !stop; t += gridDim.x) {
        int s, m0, n0;
        tile_coords(t, tiles_m, tiles_n, TNT, &s, &m0, &n0);
        for (int kt = 0; kt < KT; ++kt) {
          if (!mbar_wait_or_abort(smem_u32(&empty_bar[stage]), phase ^ 1u, abort_flag)) {
            stop = true;
            break;
          }
          const uint32_t fb = smem_u32(&full_bar[stage]);
          mbar_arrive_expect_tx(fb, (uint32_t)Cfg::STAGE_B);
          const uint32_t st = base + stage * Cfg::STAGE_B;
          const int x = kt * TK;
          tma_load_3d(st, &ops.ah, x, m0, s, fb);
          tma_load_3d(st + A_SLICE, &ops.al, x, m0, s, fb);
          tma_load_3d(st + 2 * A_SLICE, &ops.bh, x, n0, s, fb);
          tma_load_3d(st + 2 * A_SLICE + Cfg::B_SL, &ops.bl, x, n0, s, fb);
          issued[stage] = true;
          issued_phase[stage] = phase;
          if (++stage == STG) {
            stage = 0;
            phase ^= 1u;
          }
        }
      }
      // before teardown: every issued copy has landed, and (normal path) the
      // MMAs have released every stage
      const bool aborted = *abort_flag != 0;
      for (int i = 0; i < STG; ++i)
        if (issued[i]) mbar_wait(smem_u32(aborted ? &full_bar[i] : &empty_bar[i]), issued_phase[i]);
    }
  } else if (warp == 1) {
    if (lane == 0) {
      // ---- MMA issuer ----
      int stage = 0, n_done = 0;
      uint32_t phase = 0;
      bool stop = false;
      for (int t = blockIdx.x; t < n_tiles && !stop; t += gridDim.x, ++n_done) {
        const int acc = n_done % NACC;
        const uint32_t aphase = (uint32_t)(n_done / NACC) & 1u;
        // the epilogue has drained this accumulator pair's previous tile
        if (!mbar_wait_or_abort(smem_u32(&acce_bar[acc]), aphase ^ 1u, abort_flag)) break;
        asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
        const uint32_t d0 = tmem + (uint32_t)(acc * 2 * TNT), d1 = d0 + TNT;
        for (int kt = 0; kt < KT; ++kt) {
          if (!mbar_wait_or_abort(smem_u32(&full_bar[stage]), phase, abort_flag)) {
            stop = true;
            break;
          }
          asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
          const uint32_t sa = base + stage * Cfg::STAGE_B, sal = sa + A_SLICE, sb = sa + 2 * A_SLICE,
                         sbl = sb + Cfg::B_SL;
#pragma unroll
          for (int k4 = 0; k4 < TK / 16; ++k4) {
            const uint32_t off = k4 * 32;  // 16 FP16 of K = 32 bytes inside the swizzle atom
            const uint32_t first = (kt > 0 || k4 > 0) ? 1u : 0u;
            mma_f16_n<TNT>(d0, smem_desc(sa + off), smem_desc(sb + off), first);
            mma_f16_n<TNT>(d1, smem_desc(sa + off), smem_desc(sbl + off), first);
            mma_f16_n<TNT>(d1, smem_desc(sal + off), smem_desc(sb + off), 1u);
          }
          mma_commit(smem_u32(&empty_bar[stage]));
          if (++stage == STG) {
            stage = 0;
            phase ^= 1u;
          }
        }
        if (stop) break;
        mma_commit(smem_u32(&accf_bar[acc]));
      }
      // every MMA of this thread has finished before TMEM is freed
      mma_commit(smem_u32(&drain_bar));
      mbar_wait(smem_u32(&drain_bar), 0);
    }
  } else {
    // ---- epilogue: warps 2-9; TMEM lane quarter warp % 4, column half (warp - 2) / 4 ----
    const int q = warp & 3;
    const int row = q * 32 + lane;
    const int cbeg = ((warp - 2) >> 2) * (TNT / 2);
    const uint32_t stg = base + (uint32_t)(STG * Cfg::STAGE_B) + (uint32_t)((warp - 2) * EPI_STAGE);
    int n_done = 0;
    for (int t = blockIdx.x; t < n_tiles; t += gridDim.x, ++n_done) {
      const int acc = n_done % NACC;
      const uint32_t aphase = (uint32_t)(n_done / NACC) & 1u;
      int s, m0, n0;
      tile_coords(t, tiles_m, tiles_n, TNT, &s, &m0, &n0);
      int ok = 0;
      if (lane == 0) ok = mbar_wait_or_abort(smem_u32(&accf_bar[acc]), aphase, abort_flag) ? 1 : 0;
      ok = __shfl_sync(0xffffffffu, ok, 0);
      if (!ok) break;
      asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
      const uint32_t lane_addr = (uint32_t)(q * 32) << 16;
      const uint32_t d0 = tmem + (uint32_t)(acc * 2 * TNT) + lane_addr, d1 = d0 + TNT;
      float* o = out + ((size_t)s * M + m0 + row) * Nn + n0;
      const float fy = fold_y ? fold_y[(size_t)s * M + m0 + row] : 0.f;
      const float* fx = fold_x ? fold_x + (size_t)s * Nn + n0 : nullptr;
#pragma unroll 1
      for (int c0 = cbeg; c0 < cbeg + TNT / 2; c0 += 32) {
        uint32_t h[32], l[32];
        asm volatile(
            "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
            "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];\n"
            : "=r"(h[0]), "=r"(h[1]), "=r"(h[2]), "=r"(h[3]), "=r"(h[4]), "=r"(h[5]), "=r"(h[6]), "=r"(h[7]),
              "=r"(h[8]), "=r"(h[9]), "=r"(h[10]), "=r"(h[11]), "=r"(h[12]), "=r"(h[13]), "=r"(h[14]), "=r"(h[15]),
              "=r"(h[16]), "=r"(h[17]), "=r"(h[18]), "=r"(h[19]), "=r"(h[20]), "=r"(h[21]), "=r"(h[22]), "=r"(h[23]),
              "=r"(h[24]), "=r"(h[25]), "=r"(h[26]), "=r"(h[27]), "=r"(h[28]), "=r"(h[29]), "=r"(h[30]), "=r"(h[31])
            : "r"(d0 + c0));
        asm volatile(
            "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
            "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];\n"
            : "=r"(l[0]), "=r"(l[1]), "=r"(l[2]), "=r"(l[3]), "=r"(l[4]), "=r"(l[5]), "=r"(l[6]), "=r"(l[7]),
              "=r"(l[8]), "=r"(l[9]), "=r"(l[10]), "=r"(l[11]), "=r"(l[12]), "=r"(l[13]), "=r"(l[14]), "=r"(l[15]),
              "=r"(l[16]), "=r"(l[17]), "=r"(l[18]), "=r"(l[19]), "=r"(l[20]), "=r"(l[21]), "=r"(l[22]), "=r"(l[23]),
              "=r"(l[24]), "=r"(l[25]), "=r"(l[26]), "=r"(l[27]), "=r"(l[28]), "=r"(l[29]), "=r"(l[30]), "=r"(l[31])
            : "r"(d1 + c0));
        asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory");
        if constexpr (EPI) {
          // this thread's last TMEM read of the tile: the MMAs of the next
          // tile may start while the block is combined and stored
          if (c0 + 32 == cbeg + TNT / 2) {
            asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
            mbar_arrive(smem_u32(&acce_bar[acc]));
          }
        }
        const float lo_scale = scale / kTcLoScale;
        if constexpr (EPI) {
          // the previous block's store has read the staging buffer
          if (lane == 0) bulk_wait_read_all();
          __syncwarp();
        }
#pragma unroll
        for (int j = 0; j < 32; j += 4) {
          // the 1-D phases (turns, each in [-1/2, 1/2]) join the product
          float4 f = make_float4(0.f, 0.f, 0.f, 0.f);
          if (fx) {
            f = *reinterpret_cast<const float4*>(fx + c0 + j);
            f.x += fy;
            f.y += fy;
            f.z += fy;
            f.w += fy;
          }
          float4 v;
          v.x = fmaf(__uint_as_float(l[j + 0]), lo_scale, fmaf(__uint_as_float(h[j + 0]), scale, f.x));
          v.y = fmaf(__uint_as_float(l[j + 1]), lo_scale, fmaf(__uint_as_float(h[j + 1]), scale, f.y));
          v.z = fmaf(__uint_as_float(l[j + 2]), lo_scale, fmaf(__uint_as_float(h[j + 2]), scale, f.z));
          v.w = fmaf(__uint_as_float(l[j + 3]), lo_scale, fmaf(__uint_as_float(h[j + 3]), scale, f.w));
          if constexpr (EPI) {
            // row `lane`, 16-byte chunk j / 4, 128-byte swizzle (chunk ^ row % 8)
            const uint32_t a16 = stg + (uint32_t)lane * 128u + ((uint32_t)((j >> 2) ^ (lane & 7)) << 4);
            asm volatile("st.shared.v4.f32 [%0], {%1, %2, %3, %4};\n" ::"r"(a16), "f"(v.x), "f"(v.y), "f"(v.z),
                         "f"(v.w)
                         : "memory");
          } else {
            *reinterpret_cast<float4*>(o + c0 + j) = v;
          }
        }
        if constexpr (EPI) {
          asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
          __syncwarp();
          if (lane == 0) {
            tma_store_3d(&outmap, stg, n0 + c0, m0 + q * 32, s);
            bulk_commit();
          }
        }
      }
      if constexpr (!EPI) {
        asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
        mbar_arrive(smem_u32(&acce_bar[acc]));
      }
    }
    // no store may read the staging buffer after the CTA leaves
    if constexpr (EPI)
      if (lane == 0) bulk_wait_all();
  }

  asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
  __syncthreads();
  if (threadIdx.x == 0 && *abort_flag) {
    atomicExch(&g_tc_error, 1);
    if (status) atomicOr(status, STATUS_GEMM_WAIT);
  }
  if (warp == 1) {
    asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, 512;\n" ::"r"(tmem) : "memory");
  }
}

// split FP32 [rows][K] (row stride lds) into FP16 hi / lo slices [rows][Kp] (zero padded)
__global__ void split_fp16_kernel(const float* __restrict__ src, int rows, int K, int lds, int Kp,
                                  __half* __restrict__ hi, __half* __restrict__ lo) {
  const size_t total = (size_t)rows * Kp;
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < total; i += (size_t)gridDim.x * blockDim.x) {
    const int r = (int)(i / Kp), k = (int)(i - (size_t)r * Kp);
    const float v = k < K ? src[(size_t)r * lds + k] : 0.f;
    const __half h = __float2half_rn(v);
    hi[i] = h;
    lo[i] = __float2half_rn((v - __half2float(h)) * kTcLoScale);
  }
}


// ---------------------------------------------------------------------------
// fused MLP inference on the tensor cores (the PDT surrogate's query path)
//
// One CTA per SM walks 128-query tiles.  Per tile the whole network runs
// without leaving the SM: the activations stay in shared memory as BF16
// (K-major, 128-byte swizzle: the A operand of the next layer's MMAs), the
// accumulators in TMEM (128 lanes = the tile's queries, one column per
// output unit).  Warp 0 streams the weights -- a packed image laid out as the
// MMAs read it, pieces of <= 128 output rows -- through two 64 KB slots with
// bulk copies; warp 1 issues tcgen05.mma kind::f16 (BF16 x BF16, FP32
// accumulation); warps 2-5 (one TMEM lane per thread = one query) add the
// bias, apply GELU, and write the next layer's operand, and after the last
// layer form the softmax histogram and store the outputs.  The inputs enter
// as two BF16 slices, x = hi + lo (the first layer's weights are repeated
// for the lo slice), so the features keep about 16 bits.
// mbarriers: full / empty per weight slot, accumulator full (MMA ->
// epilogue), operand ready (epilogue -> MMA).  Every wait is bounded.
// ---------------------------------------------------------------------------
constexpr int MLP_TM = 128;                        // queries per tile = TMEM lanes = MMA M
constexpr int MLP_EPI = 512;                       // epilogue threads: 4 column slices x 128 rows
constexpr int MLP_THREADS = 64 + MLP_EPI;          // warp 0 weights, warp 1 MMAs, warps 2-17 epilogue
constexpr int MLP_SLOT = 64 * 1024;                // one weight piece: <= 128 rows x 4 K blocks x 128 B
constexpr int MLP_KB_BYTES = MLP_TM * 128;         // one K block (64 BF16) of the activations
constexpr int MLP_ACT = 4 * MLP_KB_BYTES;          // activations: 128 x 256 BF16
constexpr int MLP_SMEM = MLP_ACT + 2 * MLP_SLOT + 1024;

// instruction descriptor: kind::f16 with A = B = BF16, D = FP32, both K-major, M = 128
__device__ __forceinline__ uint32_t mlp_idesc(int n) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(n >> 3) << 17) | ((uint32_t)(MLP_TM >> 4) << 24);
}

__device__ __forceinline__ void mma_bf16(uint32_t d_tmem, uint64_t a, uint64_t b, uint32_t idesc,
                                         uint32_t accumulate) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
      " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(d_tmem),
      "l"(a), "l"(b), "r"(idesc), "r"(accumulate)
      : "memory");
}

__device__ __forceinline__ void bulk_load(uint32_t dst, const void* src, uint32_t bytes, uint32_t bar) {
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];\n" ::"r"(dst),
               "l"(src), "r"(bytes), "r"(bar)
               : "memory");
}

// the epilogue warps (named barrier 1, MLP_EPI threads): true when every thread's flag is
__device__ __forceinline__ bool epi_all(bool ok) {
  uint32_t r;
  asm volatile(
      "{\n .reg .pred p, q;\n setp.ne.u32 p, %1, 0;\n bar.red.and.pred q, 1, 512, p;\n selp.u32 %0, 1, 0, q;\n}\n"
      : "=r"(r)
      : "r"((uint32_t)ok)
      : "memory");
  return r != 0;
}
__device__ __forceinline__ void epi_sync() { asm volatile("bar.sync 1, 512;\n" ::: "memory"); }

__device__ __forceinline__ float mlp_gelu(float z) { return 0.5f * z * (1.f + erff(z * 0.70710678118654752440f)); }

__device__ __forceinline__ uint32_t pack_bf16x2(float lo_elem, float hi_elem) {
  const __nv_bfloat162 h = __floats2bfloat162_rn(lo_elem, hi_elem);  // .x (first element) at the lower address
  return *reinterpret_cast<const uint32_t*>(&h);
}

// 16 consecutive FP32 accumulator columns of this thread's TMEM lane (no wait)
__device__ __forceinline__ void tmem_ld16(uint32_t addr, uint32_t (&r)[16]) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];\n"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
        "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(addr));
}
__device__ __forceinline__ void tmem_wait_ld() { asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory"); }

template <int K0>
__global__ void __launch_bounds__(MLP_THREADS, 1) mlp_infer_tc_kernel(const __grid_constant__ MlpTcArgs a) {
  static_assert(K0 == 16 || K0 == 32, "the input slices fill one K block");
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  __shared__ __align__(8) uint64_t wfull[2], wempty[2], accf, actr, drain;
  __shared__ uint32_t tmem_holder;
  __shared__ int abort_word;
  volatile int* abort_flag = &abort_word;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const uint32_t raw = smem_u32(smem_raw);
  const uint32_t act = (raw + 1023) & ~1023u, slot0 = act + MLP_ACT;
  unsigned char* act_p = smem_raw + (act - raw);  // generic pointer to the activations
  const int n_tiles = (a.batch + MLP_TM - 1) / MLP_TM;

  if (threadIdx.x == 0) {
    for (int s = 0; s < 2; ++s) {
      mbar_init(smem_u32(&wfull[s]), 1);
      mbar_init(smem_u32(&wempty[s]), 1);
    }
    mbar_init(smem_u32(&accf), 1);
    mbar_init(smem_u32(&actr), MLP_EPI);
    mbar_init(smem_u32(&drain), 1);
    *abort_flag = 0;
    asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
  }
  if (warp == 1) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], 256;\n" ::"r"(smem_u32(&tmem_holder))
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n" ::: "memory");
  }
  asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
  const uint32_t tmem = tmem_holder;

  if (warp == 0) {
    if (lane == 0) {
      // ---- weight producer: the pieces of every tile, in order, through two slots ----
      int gp = 0, fills[2] = {0, 0};
      bool stop = false;
      for (int t = blockIdx.x; t < n_tiles && !stop; t += gridDim.x) {
        for (int p = 0; p < a.n_pieces; ++p, ++gp) {
          const int s = gp & 1;
          // the MMAs of this slot's previous piece have completed
          if (gp >= 2 && !mbar_wait_or_abort(smem_u32(&wempty[s]), (uint32_t)(((gp >> 1) - 1) & 1), abort_flag)) {
            stop = true;
            break;
          }
          const uint32_t fb = smem_u32(&wfull[s]);
          mbar_arrive_expect_tx(fb, a.pieces[p].bytes);
          bulk_load(slot0 + (uint32_t)(s * MLP_SLOT), a.img + a.pieces[p].src, a.pieces[p].bytes, fb);
          ++fills[s];
        }
      }
      // no copy may land after the CTA leaves
      for (int s = 0; s < 2; ++s)
        if (fills[s]) mbar_wait(smem_u32(&wfull[s]), (uint32_t)((fills[s] - 1) & 1));
    }
  } else if (warp == 1) {
    if (lane == 0) {
      // ---- MMA issuer ----
      int gp = 0, n_act = 0;
      bool stop = false;
      for (int t = blockIdx.x; t < n_tiles && !stop; t += gridDim.x) {
        int p = 0;
        for (int l = 0; l < a.layers; ++l) {
          // the layer's operand is in shared memory, and TMEM has been read out
          if (!mbar_wait_or_abort(smem_u32(&actr), (uint32_t)(n_act & 1), abort_flag)) {
            stop = true;
            break;
          }
          ++n_act;
          asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
          for (; p < a.n_pieces && a.pieces[p].layer == l; ++p, ++gp) {
            const int s = gp & 1;
            if (!mbar_wait_or_abort(smem_u32(&wfull[s]), (uint32_t)((gp >> 1) & 1), abort_flag)) {
              stop = true;
              break;
            }
            asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
            const MlpPiece pc = a.pieces[p];
            const uint32_t idesc = mlp_idesc(pc.rows);
            const uint32_t wb = slot0 + (uint32_t)(s * MLP_SLOT), kb_bytes = (uint32_t)pc.rows * 128u;
            for (int k = 0; k < pc.k_steps; ++k) {
              const uint32_t kb = (uint32_t)(k >> 2), off = (uint32_t)(k & 3) * 32u;  // 16 BF16 of K = 32 bytes
              mma_bf16(tmem + (uint32_t)pc.col0, smem_desc(act + kb * MLP_KB_BYTES + off),
                       smem_desc(wb + kb * kb_bytes + off), idesc, k > 0 ? 1u : 0u);
            }
            mma_commit(smem_u32(&wempty[s]));
          }
          if (stop) break;
          mma_commit(smem_u32(&accf));
        }
      }
      // every MMA of this thread has finished before TMEM is freed
      mma_commit(smem_u32(&drain));
      mbar_wait(smem_u32(&drain), 0);
    }
  } else {
    // ---- epilogue: warps 2-17.  TMEM lane quarter q = warp % 4 (the tile's rows 32 q ..
    // 32 q + 31, one per lane), column slice cs = (warp - 2) / 4 of each hidden layer ----
    const int q = warp & 3;
    const int cs = (warp - 2) >> 2;
    const int row = q * 32 + lane;
    const int et = threadIdx.x - 64;  // 0 .. MLP_EPI - 1
    const uint32_t lane_addr = (uint32_t)(q * 32) << 16;
    unsigned char* arow = act_p + row * 128;
    const int sw = row & 7;
    const int slice = a.hidden / 4;  // columns of a hidden layer per slice: a multiple of 16
    int n_acc = 0;
    for (int t = blockIdx.x; t < n_tiles; t += gridDim.x) {
      const int m0 = t * MLP_TM;
      const int valid = min(MLP_TM, a.batch - m0);
      const bool live = row < valid;
      if (cs == 0) {
        // inputs -> K block 0 of the operand: x_hi at K [0, K0), x_lo at [K0, 2 K0); the box check
        float xs[K0];
        int out = 0;
#pragma unroll
        for (int j = 0; j < K0; ++j) {
          xs[j] = (live && j < a.in) ? a.x[(size_t)(m0 + row) * a.in + j] : 0.f;
          if (a.lo && live && j < a.in) out |= !(xs[j] >= a.lo[j] && xs[j] <= a.hi[j]);
        }
        if (a.oor && live) a.oor[m0 + row] = out;
        uint32_t hw[K0 / 2], lw[K0 / 2];
#pragma unroll
        for (int j = 0; j < K0; j += 2) {
          const __nv_bfloat16 h0 = __float2bfloat16_rn(xs[j]), h1 = __float2bfloat16_rn(xs[j + 1]);
          hw[j / 2] = pack_bf16x2(__bfloat162float(h0), __bfloat162float(h1));
          lw[j / 2] = pack_bf16x2(xs[j] - __bfloat162float(h0), xs[j + 1] - __bfloat162float(h1));
        }
#pragma unroll
        for (int c = 0; c < K0 / 8; ++c) {
          *reinterpret_cast<uint4*>(arow + ((c ^ sw) << 4)) =
              make_uint4(hw[4 * c], hw[4 * c + 1], hw[4 * c + 2], hw[4 * c + 3]);
          *reinterpret_cast<uint4*>(arow + (((c + K0 / 8) ^ sw) << 4)) =
              make_uint4(lw[4 * c], lw[4 * c + 1], lw[4 * c + 2], lw[4 * c + 3]);
        }
      }
      asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
      asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
      mbar_arrive(smem_u32(&actr));
      bool ok = true;
      for (int l = 0; l < a.layers; ++l) {
        int got = 0;
        if (lane == 0) got = mbar_wait_or_abort(smem_u32(&accf), (uint32_t)(n_acc & 1), abort_flag) ? 1 : 0;
        got = __shfl_sync(0xffffffffu, got, 0);
        ++n_acc;
        if (!epi_all(got != 0)) {
          ok = false;
          break;
        }
        asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
        const float* bias = a.bias[l];
        if (l < a.layers - 1) {
          // hidden layer, this warp's column slice: bias + GELU -> BF16 operand of the next layer
#pragma unroll 1
          for (int c0 = cs * slice; c0 < (cs + 1) * slice; c0 += 16) {
            uint32_t r[16];
            tmem_ld16(tmem + lane_addr + (uint32_t)c0, r);
            tmem_wait_ld();
            uint32_t pk[8];
#pragma unroll
            for (int j = 0; j < 16; j += 2)
              pk[j / 2] = pack_bf16x2(mlp_gelu(__uint_as_float(r[j]) + bias[c0 + j]),
                                      mlp_gelu(__uint_as_float(r[j + 1]) + bias[c0 + j + 1]));
            unsigned char* kb = arow + (c0 >> 6) * MLP_KB_BYTES;
            const int cc = (c0 & 63) >> 3;
            *reinterpret_cast<uint4*>(kb + ((cc ^ sw) << 4)) = make_uint4(pk[0], pk[1], pk[2], pk[3]);
            *reinterpret_cast<uint4*>(kb + (((cc + 1) ^ sw) << 4)) = make_uint4(pk[4], pk[5], pk[6], pk[7]);
          }
          asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
          asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
          mbar_arrive(smem_u32(&actr));
        } else {
          // output layer (slice 0's warps hold whole rows): softmax over the first n_hist
          // columns (online max / sum), the outputs staged as FP32 [valid][out] over the
          // operand (its MMAs have completed), then stored by all epilogue threads
          float* stg = reinterpret_cast<float*>(act_p);
          if (cs == 0) {
            float mx = -INFINITY, se = 0.f;
#pragma unroll 1
            for (int c0 = 0; c0 < a.n_hist; c0 += 16) {
              uint32_t r[16];
              tmem_ld16(tmem + lane_addr + (uint32_t)c0, r);
              tmem_wait_ld();
#pragma unroll
              for (int j = 0; j < 16; ++j) {
                if (c0 + j < a.n_hist) {
                  const float z = __uint_as_float(r[j]) + bias[c0 + j];
                  if (z > mx) {
                    se = se * expf(mx - z) + 1.f;
                    mx = z;
                  } else {
                    se += expf(z - mx);
                  }
                }
              }
            }
            const float inv = 1.f / se;
#pragma unroll 1
            for (int c0 = 0; c0 < a.out_pad; c0 += 16) {
              uint32_t r[16];
              tmem_ld16(tmem + lane_addr + (uint32_t)c0, r);
              tmem_wait_ld();
#pragma unroll
              for (int j = 0; j < 16; ++j) {
                const int c = c0 + j;
                if (live && c < a.out) {
                  const float z = __uint_as_float(r[j]) + bias[c];
                  stg[row * a.out + c] = c < a.n_hist ? expf(z - mx) * inv : z;
                }
              }
            }
          }
          asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
          epi_sync();
          float* y = a.y + (size_t)m0 * a.out;
          for (int i = et; i < valid * a.out; i += MLP_EPI) y[i] = stg[i];
          epi_sync();  // the next tile's inputs overwrite the staging
        }
      }
      if (!ok) break;
    }
  }

  asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
  __syncthreads();
  // the MLP's own status word (atm_mlp_check), not the plans' device-wide flag
  if (threadIdx.x == 0 && *abort_flag && a.status) atomicOr(a.status, STATUS_GEMM_WAIT);
  if (warp == 1) {
    asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, 256;\n" ::"r"(tmem) : "memory");
  }
}

}  // namespace

size_t tc_smem_bytes() { return SMEM; }

// ---------------------------------------------------------------------------
// host side of the TMA form
// ---------------------------------------------------------------------------
using EncodeTiledFn = CUresult (*)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                   const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                   CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

static EncodeTiledFn encode_tiled() {
  static std::once_flag once;
  static EncodeTiledFn fn = nullptr;
  std::call_once(once, [] {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q{};
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<EncodeTiledFn>(p);
    else
      cudaGetLastError();
  });
  return fn;
}

// [S][rows][Kp] FP16 operand, boxes of TK x box_rows, 128-byte swizzle
static bool encode_operand(EncodeTiledFn fn, CUtensorMap* map, const __half* base, int S, int rows, int Kp,
                           int box_rows) {
  if (((uintptr_t)base & 15) != 0) return false;
  const cuuint64_t dims[3] = {(cuuint64_t)Kp, (cuuint64_t)rows, (cuuint64_t)S};
  const cuuint64_t strides[2] = {(cuuint64_t)Kp * sizeof(__half), (cuuint64_t)rows * Kp * sizeof(__half)};
  const cuuint32_t box[3] = {(cuuint32_t)TK, (cuuint32_t)box_rows, 1};
  const cuuint32_t estr[3] = {1, 1, 1};
  return fn(map, CU_TENSOR_MAP_DATA_TYPE_FLOAT16, 3, const_cast<__half*>(base), dims, strides, box, estr,
            CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
            CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

// tensor map of a complex64 field [B][N][N] seen as FP32 [B][N][2N], boxes of
// C columns (2C floats) x box_rows rows: the column pass's tiles
bool encode_field_tiles(void* map, const float2* field, int N, int B, int C, int box_rows) {
  EncodeTiledFn fn = encode_tiled();
  if (!fn || !map || ((uintptr_t)field & 15) != 0 || (2 * C * 4) % 16 != 0) return false;
  const cuuint64_t dims[3] = {(cuuint64_t)2 * N, (cuuint64_t)N, (cuuint64_t)B};
  const cuuint64_t strides[2] = {(cuuint64_t)N * sizeof(float2), (cuuint64_t)N * N * sizeof(float2)};
  const cuuint32_t box[3] = {(cuuint32_t)(2 * C), (cuuint32_t)box_rows, 1};
  const cuuint32_t estr[3] = {1, 1, 1};
  return fn(static_cast<CUtensorMap*>(map), CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, const_cast<float2*>(field), dims,
            strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
            CU_TENSOR_MAP_L2_PROMOTION_NONE, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

bool encode_tiled_rows(void* map, const float2* field, int N, int B, int box_blocks) {
  EncodeTiledFn fn = encode_tiled();
  if (!fn || !map || ((uintptr_t)field & 127) != 0 || N < 16 || box_blocks < 1 || box_blocks > 256) return false;
  const cuuint32_t estr[3] = {1, 1, 1};
  const cuuint64_t dims[3] = {32, (cuuint64_t)N * N / 16, (cuuint64_t)B};
  const cuuint64_t strides[2] = {128, (cuuint64_t)N * N * sizeof(float2)};
  const cuuint32_t box[3] = {8, (cuuint32_t)box_blocks, 1};
  return fn(static_cast<CUtensorMap*>(map), CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, const_cast<float2*>(field), dims,
            strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
            CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

// tiled field [B][N][N] (4 x 4 blocks of complex64 = 32 FP32 = 128 bytes):
//   by_rows: 3-D {32, N^2 / 16, B}, boxes of box_blocks consecutive blocks (a block row is contiguous);
//   else:    3-D {32, N / 4, B N / 4}, boxes of box_blocks blocks of one block column.
// 128-byte swizzle: the 16-byte chunk c of box row j lands at chunk c ^ (j & 7), so the passes read
// a row or a column of the staged blocks without shared-memory bank conflicts.
bool encode_tiled_field(void* map, const float2* field, int N, int B, bool by_rows, int box_blocks) {
  EncodeTiledFn fn = encode_tiled();
  if (!fn || !map || ((uintptr_t)field & 127) != 0 || N < 16 || box_blocks < 1 || box_blocks > 256) return false;
  const cuuint32_t estr[3] = {1, 1, 1};
  if (by_rows) {
    // {block float, block index within a realisation, realisation}: coordinates stay below 2^31 for any batch
    const cuuint64_t dims[3] = {32, (cuuint64_t)N * N / 16, (cuuint64_t)B};
    const cuuint64_t strides[2] = {128, (cuuint64_t)N * N * sizeof(float2)};
    const cuuint32_t box[3] = {32, (cuuint32_t)box_blocks, 1};
    return fn(static_cast<CUtensorMap*>(map), CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, const_cast<float2*>(field), dims,
              strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
              CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
  }
  const cuuint64_t dims[3] = {32, (cuuint64_t)N / 4, (cuuint64_t)B * N / 4};
  const cuuint64_t strides[2] = {128, (cuuint64_t)N * 32};
  const cuuint32_t box[3] = {32, 1, (cuuint32_t)box_blocks};
  return fn(static_cast<CUtensorMap*>(map), CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, const_cast<float2*>(field), dims,
            strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
            CU_TENSOR_MAP_L2_PROMOTION_NONE, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

// the block columns of a tiled field without swizzle: a box of box_blocks
// blocks of one block column lands as [4 box_blocks rows][4 columns], the
// layout of a row-major column tile (the warp-FFT column pass reads either)
bool encode_tiled_cols_plain(void* map, const float2* field, int N, int B, int box_blocks) {
  EncodeTiledFn fn = encode_tiled();
  if (!fn || !map || ((uintptr_t)field & 127) != 0 || N < 16 || box_blocks < 1 || box_blocks > 256) return false;
  const cuuint32_t estr[3] = {1, 1, 1};
  const cuuint64_t dims[3] = {32, (cuuint64_t)N / 4, (cuuint64_t)B * N / 4};
  const cuuint64_t strides[2] = {128, (cuuint64_t)N * 32};
  const cuuint32_t box[3] = {32, 1, (cuuint32_t)box_blocks};
  return fn(static_cast<CUtensorMap*>(map), CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, const_cast<float2*>(field), dims,
            strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
            CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

struct TcPlan {
  TmaOperands ops;
  int S, M, Nn, Kp;
  int tn;  // output tile width: 256 (two stages, one accumulator pair) or 128 (three stages, two pairs)
};

TcPlan* tc_plan_create(int S, int M, int Nn, int Kp, const __half* a_hi, const __half* a_lo, const __half* b_hi,
                       const __half* b_lo, int tn) {
  if (tn != 128 && tn != 256) return nullptr;
  if (S < 1 || M % TM || Nn % tn || Kp % TK || Kp < TK) return nullptr;
  EncodeTiledFn fn = encode_tiled();
  if (!fn) return nullptr;
  TcPlan* p = new TcPlan{};
  p->S = S;
  p->M = M;
  p->Nn = Nn;
  p->Kp = Kp;
  p->tn = tn;
  if (!encode_operand(fn, &p->ops.ah, a_hi, S, M, Kp, TM) || !encode_operand(fn, &p->ops.al, a_lo, S, M, Kp, TM) ||
      !encode_operand(fn, &p->ops.bh, b_hi, S, Nn, Kp, tn) || !encode_operand(fn, &p->ops.bl, b_lo, S, Nn, Kp, tn)) {
    delete p;
    return nullptr;
  }
  return p;
}

void tc_plan_destroy(TcPlan* p) { delete p; }

// [S][M][Nn] FP32 output, boxes of 32 x 32, 128-byte swizzle: the staged
// epilogue's TMA stores
static bool encode_output(EncodeTiledFn fn, CUtensorMap* map, float* out, int S, int M, int Nn) {
  if (((uintptr_t)out & 15) != 0 || (Nn * 4) % 16 != 0) return false;
  const cuuint64_t dims[3] = {(cuuint64_t)Nn, (cuuint64_t)M, (cuuint64_t)S};
  const cuuint64_t strides[2] = {(cuuint64_t)Nn * sizeof(float), (cuuint64_t)M * Nn * sizeof(float)};
  const cuuint32_t box[3] = {32, 32, 1};
  const cuuint32_t estr[3] = {1, 1, 1};
  return fn(map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, out, dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
            CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_NONE,
            CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

template <int TNT, int STG, int NACC, int EPI>
static cudaError_t launch_tma_form(const TcPlan* p, int S, float* out, float scale, const float* fold_y,
                                   const float* fold_x, int* status, cudaStream_t st) {
  using Cfg = TmaCfg<TNT, STG, NACC, EPI>;
  alignas(64) CUtensorMap outmap{};
  if (EPI) {
    EncodeTiledFn fn = encode_tiled();
    if (!fn || !encode_output(fn, &outmap, out, S, p->M, p->Nn)) return cudaErrorNotSupported;
  }
  static int sms[64] = {};
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (dev < 0 || dev >= 64) return cudaErrorInvalidDevice;
  if (sms[dev] == 0) {
    e = cudaFuncSetAttribute(tc_gemm_tma_kernel<TNT, STG, NACC, EPI>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             Cfg::SMEM);
    if (e != cudaSuccess) return e;
    int n = 0;
    e = cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
    if (e != cudaSuccess) return e;
    sms[dev] = std::max(n, 1);
  }
  const int n_tiles = S * (p->M / TM) * (p->Nn / TNT);
  const int grid = std::min(n_tiles, sms[dev]);
  tc_gemm_tma_kernel<TNT, STG, NACC, EPI><<<grid, P_THREADS, Cfg::SMEM, st>>>(p->ops, outmap, out, S, p->M, p->Nn,
                                                                               p->Kp, scale, fold_y, fold_x, status);
  return cudaGetLastError();
}

cudaError_t launch_tc_gemm_tma(const TcPlan* p, int S, float* out, float scale, const float* fold_y,
                               const float* fold_x, int* status, cudaStream_t st) {
  if (!p || S < 1 || S > p->S || !out || (!fold_y) != (!fold_x)) return cudaErrorInvalidValue;
  if (((uintptr_t)fold_x & 15) != 0) return cudaErrorMisalignedAddress;
  if (p->tn == 128) return launch_tma_form<128, 3, 2, 0>(p, S, out, scale, fold_y, fold_x, status, st);
  return launch_tma_form<256, 2, 1, 1>(p, S, out, scale, fold_y, fold_x, status, st);
}

cudaError_t set_tc_wait_budget(unsigned long long ns) { return cudaMemcpyToSymbol(g_tc_wait_ns, &ns, sizeof(ns)); }

cudaError_t launch_tc_gemm(int S, int M, int Nn, int Kp, const __half* a_hi, const __half* a_lo, const __half* b_hi,
                           const __half* b_lo, float* out, float scale, cudaStream_t st) {
  if (M % TM || Nn % TN || Kp % TK || Kp < TK) return cudaErrorInvalidValue;
  static bool attr_done[64] = {};
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess || dev < 0 || dev >= 64) return e != cudaSuccess ? e : cudaErrorInvalidDevice;
  if (!attr_done[dev]) {
    e = cudaFuncSetAttribute(tc_gemm_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, SMEM);
    if (e != cudaSuccess) return e;
    attr_done[dev] = true;
  }
  TcArgs a{a_hi, a_lo, b_hi, b_lo, out, M, Nn, Kp, scale};
  dim3 grid(Nn / TN, M / TM, S);
  tc_gemm_kernel<<<grid, THREADS, SMEM, st>>>(a);
  return cudaGetLastError();
}

cudaError_t launch_split_fp16(const float* src, int rows, int K, int lds, int Kp, __half* hi, __half* lo,
                              cudaStream_t st) {
  const size_t total = (size_t)rows * Kp;
  const int grid = (int)std::min<size_t>((total + 255) / 256, 65535 * 8);
  split_fp16_kernel<<<grid, 256, 0, st>>>(src, rows, K, lds, Kp, hi, lo);
  return cudaGetLastError();
}

cudaError_t launch_mlp_infer_tc(const MlpTcArgs& a, cudaStream_t st) {
  if (a.batch <= 0) return cudaSuccess;
  if ((a.k0 != 16 && a.k0 != 32) || a.in > a.k0 || a.hidden < 64 || a.hidden > 256 || a.hidden % 64 ||
      a.out > 128 || a.out_pad < a.out || a.out_pad % 16 || a.n_hist > a.out || a.n_pieces > kMlpMaxPieces)
    return cudaErrorInvalidValue;
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (dev < 0 || dev >= 64) return cudaErrorInvalidDevice;
  static int sms[64] = {};
  static bool attr_done[64][2] = {};
  const int form = a.k0 == 16 ? 0 : 1;
  void (*kernel)(MlpTcArgs) = form == 0 ? mlp_infer_tc_kernel<16> : mlp_infer_tc_kernel<32>;
  if (!attr_done[dev][form]) {
    e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, MLP_SMEM);
    if (e != cudaSuccess) return e;
    attr_done[dev][form] = true;
  }
  if (!sms[dev]) {
    e = cudaDeviceGetAttribute(&sms[dev], cudaDevAttrMultiProcessorCount, dev);
    if (e != cudaSuccess) return e;
  }
  const int n_tiles = (a.batch + MLP_TM - 1) / MLP_TM;
  kernel<<<std::min(n_tiles, sms[dev]), MLP_THREADS, MLP_SMEM, st>>>(a);
  return cudaGetLastError();
}

cudaError_t tc_error_flag(int* host_flag, bool reset) {
  cudaError_t e = cudaMemcpyFromSymbol(host_flag, g_tc_error, sizeof(int));
  if (e != cudaSuccess) return e;
  if (reset) {
    const int z = 0;
    e = cudaMemcpyToSymbol(g_tc_error, &z, sizeof(int));
  }
  return e;
}

}  // namespace atm

// ---------------------------------------------------------------------------
// unit-test entry point of the tensor-core GEMM (device pointers):
//   out[s][m][n] = scale * sum_k A[s][m][k] B[s][n][k]  for FP32 A, B with K
//   columns (row strides K), via the FP16 hi/lo split; M % 128 == 0,
//   N % 256 == 0; variant 0 = TMA form with 128 x 128 tiles and double-buffered
//   accumulators, 1 = cp.async form, 2 = TMA form with 128 x 256 tiles.  Scratch for the
//   slices is allocated here (test path).
// ---------------------------------------------------------------------------
extern "C" int atm_tc_gemm_test(const float* A, const float* B, int32_t S, int32_t M, int32_t N, int32_t K,
                                float scale, float* out, int32_t variant, void* stream) {
  if (!A || !B || !out || S < 1 || M < 1 || N < 1 || K < 1)
    return atm::set_error(ATM_ERR_INVALID, "bad tc gemm arguments");
  if (M % 128 || N % 256) return atm::set_error(ATM_ERR_UNSUPPORTED, "M %% 128 and N %% 256 must be 0");
  if (variant < 0 || variant > 2) return atm::set_error(ATM_ERR_INVALID, "variant %d is not 0, 1 or 2", variant);
  cudaStream_t st = (cudaStream_t)stream;
  const int Kp = (K + 63) / 64 * 64;
  __half *ah = nullptr, *al = nullptr, *bh = nullptr, *bl = nullptr;
  const size_t na = (size_t)S * M * Kp, nb = (size_t)S * N * Kp;
  if (cudaMalloc(&ah, na * 2) != cudaSuccess || cudaMalloc(&al, na * 2) != cudaSuccess ||
      cudaMalloc(&bh, nb * 2) != cudaSuccess || cudaMalloc(&bl, nb * 2) != cudaSuccess) {
    cudaFree(ah);
    cudaFree(al);
    cudaFree(bh);
    cudaFree(bl);
    cudaGetLastError();
    return atm::set_error(ATM_ERR_NOMEM, "tc gemm test scratch");
  }
  cudaError_t e = atm::launch_split_fp16(A, S * M, K, K, Kp, ah, al, st);
  if (e == cudaSuccess) e = atm::launch_split_fp16(B, S * N, K, K, Kp, bh, bl, st);
  atm::TcPlan* tp = nullptr;
  if (e == cudaSuccess && variant != 1) {
    tp = atm::tc_plan_create(S, M, N, Kp, ah, al, bh, bl, variant == 2 ? 256 : 128);
    if (!tp) e = cudaErrorNotSupported;
  }
  if (e == cudaSuccess)
    e = variant != 1 ? atm::launch_tc_gemm_tma(tp, S, out, scale, nullptr, nullptr, nullptr, st)
                     : atm::launch_tc_gemm(S, M, N, Kp, ah, al, bh, bl, out, scale, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  int flag = 0;
  if (e == cudaSuccess) e = atm::tc_error_flag(&flag, true);
  atm::tc_plan_destroy(tp);
  cudaFree(ah);
  cudaFree(al);
  cudaFree(bh);
  cudaFree(bl);
  if (e != cudaSuccess) return atm::set_error(ATM_ERR_CUDA, "tc gemm: %s", cudaGetErrorString(e));
  if (flag) return atm::set_error(ATM_ERR_CUDA, "tc gemm: an mbarrier wait timed out");
  return ATM_OK;
}
