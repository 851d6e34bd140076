// 5th-generation tensor-core GEMM for the screen synthesis (sm_103a).
//
//   phi_G[s][y][x] = (1/2pi) sum_k A[s][y][k] B[s][x][k]
//
// Operands are FP32 values split into two scaled FP16 slices,
//   a = a_hi + a_lo / 2^11,  a_hi = fp16(a),  a_lo = fp16((a - a_hi) 2^11),
// so that a_hi b_hi + (a_hi b_lo + a_lo b_hi) / 2^11 carries ~22 bits: three
// tcgen05.mma (kind::f16, FP32 accumulation) per K step into two TMEM
// accumulators (D0 = sum hi.hi, D1 = sum of the cross terms), combined in the
// epilogue.  Tiles: M = 128 rows (y) x N = 256 columns (x) per CTA, K tile 64
// (one 128-byte swizzle atom of FP16), two shared-memory stages filled with
// cp.async into the K-major SWIZZLE_128B layout the MMA descriptors describe.
// One elected thread issues the MMAs; tcgen05.commit arrives on an mbarrier
// per stage.  Every mbarrier wait is bounded by %globaltimer: on timeout the
// CTA records an error, drains its copies, frees its TMEM and returns.
#include <cuda_fp16.h>

#include <algorithm>
#include <cstdint>

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
      const float lo_scale = 1.f / 2048.f;
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

// split FP32 [rows][K] (row stride lds) into scaled FP16 slices [rows][Kp] (zero padded)
__global__ void split_fp16_kernel(const float* __restrict__ src, int rows, int K, int lds, int Kp,
                                  __half* __restrict__ hi, __half* __restrict__ lo) {
  const size_t total = (size_t)rows * Kp;
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < total; i += (size_t)gridDim.x * blockDim.x) {
    const int r = (int)(i / Kp), k = (int)(i - (size_t)r * Kp);
    const float v = k < K ? src[(size_t)r * lds + k] : 0.f;
    const __half h = __float2half_rn(v);
    hi[i] = h;
    lo[i] = __float2half_rn((v - __half2float(h)) * 2048.f);
  }
}

}  // namespace

size_t tc_smem_bytes() { return SMEM; }

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
//   N % 256 == 0.  Scratch for the slices is allocated here (test path).
// ---------------------------------------------------------------------------
extern "C" int atm_tc_gemm_test(const float* A, const float* B, int32_t S, int32_t M, int32_t N, int32_t K,
                                float scale, float* out, void* stream) {
  if (!A || !B || !out || S < 1 || M < 1 || N < 1 || K < 1)
    return atm::set_error(ATM_ERR_INVALID, "bad tc gemm arguments");
  if (M % 128 || N % 256) return atm::set_error(ATM_ERR_UNSUPPORTED, "M %% 128 and N %% 256 must be 0");
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
  if (e == cudaSuccess) e = atm::launch_tc_gemm(S, M, N, Kp, ah, al, bh, bl, out, scale, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  int flag = 0;
  if (e == cudaSuccess) e = atm::tc_error_flag(&flag, true);
  cudaFree(ah);
  cudaFree(al);
  cudaFree(bh);
  cudaFree(bl);
  if (e != cudaSuccess) return atm::set_error(ATM_ERR_CUDA, "tc gemm: %s", cudaGetErrorString(e));
  if (flag) return atm::set_error(ATM_ERR_CUDA, "tc gemm: an mbarrier wait timed out");
  return ATM_OK;
}
