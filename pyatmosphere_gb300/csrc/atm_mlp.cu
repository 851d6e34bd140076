// Kernels and C ABI of the PDT surrogate: a small MLP (8 -> 256 -> 256 ->
// 256 -> 67, GELU) with BF16 weights, FP32 accumulation and FP32 master
// weights for Adam.  Forward, backward, loss (KL on a softmax histogram + MSE
// on moments), Adam and a fused inference pass with an out-of-range check.
#include <cuda_bf16.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "../../include/atm.h"
#include "atm_internal.h"

namespace {

constexpr int kMaxLayers = 8;
constexpr float kInvSqrt2 = 0.70710678118654752440f;
constexpr float kInvSqrt2Pi = 0.39894228040143267794f;

__device__ __forceinline__ float gelu(float z) { return 0.5f * z * (1.f + erff(z * kInvSqrt2)); }
__device__ __forceinline__ float gelu_grad(float z) {
  return 0.5f * (1.f + erff(z * kInvSqrt2)) + z * kInvSqrt2Pi * expf(-0.5f * z * z);
}

template <typename T>
__device__ __forceinline__ float ld(const T* p);
template <>
__device__ __forceinline__ float ld<float>(const float* p) { return *p; }
template <>
__device__ __forceinline__ float ld<__nv_bfloat16>(const __nv_bfloat16* p) { return __bfloat162float(*p); }

enum Epi { EPI_NONE = 0, EPI_BIAS = 1, EPI_BIAS_GELU = 2, EPI_GELU_GRAD = 3 };

// C[m][n] = sum_k A(m, k) B(k, n) (+ bias[n], GELU, or * gelu'(Z[m][n])),
// A(m, k) = A[m sam + k sak], B(k, n) = B[k sbk + n sbn].  64 x 64 tiles,
// 256 threads, 4 x 4 outputs per thread, K step 16.
template <typename TA, typename TB, int EPI>
__global__ void __launch_bounds__(256) mlp_gemm_kernel(int M, int N, int K, const TA* __restrict__ A, int sam,
                                                       int sak, const TB* __restrict__ B, int sbk, int sbn,
                                                       float* __restrict__ C, int ldc, const float* __restrict__ bias,
                                                       float* __restrict__ Z) {
  __shared__ float As[16][64 + 1];
  __shared__ float Bs[16][64 + 1];
  const int m0 = blockIdx.y * 64, n0 = blockIdx.x * 64;
  const int tid = threadIdx.x, tm = tid / 16, tn = tid % 16;
  float acc[4][4] = {};
  for (int k0 = 0; k0 < K; k0 += 16) {
    for (int e = tid; e < 16 * 64; e += 256) {
      const int kk = e / 64, mm = e % 64;
      const int m = m0 + mm, k = k0 + kk;
      As[kk][mm] = (m < M && k < K) ? ld(A + (size_t)m * sam + (size_t)k * sak) : 0.f;
      const int n = n0 + mm;
      Bs[kk][mm] = (n < N && k < K) ? ld(B + (size_t)k * sbk + (size_t)n * sbn) : 0.f;
    }
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < 16; ++kk) {
      float a[4], b[4];
#pragma unroll
      for (int i = 0; i < 4; ++i) a[i] = As[kk][tm + 16 * i];
#pragma unroll
      for (int j = 0; j < 4; ++j) b[j] = Bs[kk][tn + 16 * j];
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) acc[i][j] = fmaf(a[i], b[j], acc[i][j]);
    }
    __syncthreads();
  }
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    const int m = m0 + tm + 16 * i;
    if (m >= M) continue;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const int n = n0 + tn + 16 * j;
      if (n >= N) continue;
      float v = acc[i][j];
      const size_t o = (size_t)m * ldc + n;
      if (EPI == EPI_BIAS || EPI == EPI_BIAS_GELU) v += bias[n];
      if (EPI == EPI_BIAS_GELU) {
        Z[o] = v;
        v = gelu(v);
      }
      if (EPI == EPI_GELU_GRAD) v *= gelu_grad(Z[o]);
      C[o] = v;
    }
  }
}

template <typename TA, typename TB, int EPI>
cudaError_t gemm(int M, int N, int K, const TA* A, int sam, int sak, const TB* B, int sbk, int sbn, float* C, int ldc,
                 const float* bias, float* Z, cudaStream_t st) {
  dim3 grid((N + 63) / 64, (M + 63) / 64);
  mlp_gemm_kernel<TA, TB, EPI><<<grid, 256, 0, st>>>(M, N, K, A, sam, sak, B, sbk, sbn, C, ldc, bias, Z);
  return cudaGetLastError();
}

// db[n] = sum_m dZ[m][n]
__global__ void col_sum_kernel(const float* __restrict__ dZ, int M, int N, float* __restrict__ db) {
  const int n = blockIdx.x * blockDim.x + threadIdx.x;
  if (n >= N) return;
  float s = 0.f;
  for (int m = 0; m < M; ++m) s += dZ[(size_t)m * N + n];
  db[n] = s;
}

// one warp per sample: softmax over the first H outputs against a target
// histogram (KL), MSE on the remaining outputs; writes dY and adds the loss
__global__ void loss_kernel(const float* __restrict__ Y, const float* __restrict__ T, int B, int O, int H, float w_mse,
                            float* __restrict__ dY, double* __restrict__ loss) {
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) / 32, lane = threadIdx.x & 31;
  if (warp >= B) return;
  const float* y = Y + (size_t)warp * O;
  const float* t = T + (size_t)warp * O;
  float* dy = dY + (size_t)warp * O;
  float mx = -INFINITY;
  for (int j = lane; j < H; j += 32) mx = fmaxf(mx, y[j]);
  for (int off = 16; off; off >>= 1) mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, off));
  float se = 0.f;
  for (int j = lane; j < H; j += 32) se += expf(y[j] - mx);
  for (int off = 16; off; off >>= 1) se += __shfl_xor_sync(0xffffffffu, se, off);
  const float lse = mx + logf(se);
  float l = 0.f;
  const float invB = 1.f / (float)B;
  for (int j = lane; j < H; j += 32) {
    const float logp = y[j] - lse, tj = t[j];
    if (tj > 0.f) l += tj * (logf(tj) - logp);
    dy[j] = (expf(logp) - tj) * invB;
  }
  const int nm = O - H;
  for (int j = H + lane; j < O; j += 32) {
    const float d = y[j] - t[j];
    l += w_mse * d * d / (float)nm;
    dy[j] = 2.f * w_mse * d / (float)nm * invB;
  }
  for (int off = 16; off; off >>= 1) l += __shfl_xor_sync(0xffffffffu, l, off);
  if (lane == 0) atomicAdd(loss, (double)l * (double)invB);
}

__global__ void adam_kernel(float* __restrict__ w, __nv_bfloat16* __restrict__ wb, const float* __restrict__ g,
                            float* __restrict__ m, float* __restrict__ v, int n, float lr, float b1, float b2,
                            float eps, float c1, float c2, float wd) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float gi = g[i];
  const float mi = b1 * m[i] + (1.f - b1) * gi;
  const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
  m[i] = mi;
  v[i] = vi;
  const float wi = w[i] * (1.f - lr * wd) - lr * (mi / c1) / (sqrtf(vi / c2) + eps);  // AdamW decay
  w[i] = wi;
  wb[i] = __float2bfloat16_rn(wi);
}

__global__ void to_bf16_kernel(const float* __restrict__ w, __nv_bfloat16* __restrict__ wb, int n) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) wb[i] = __float2bfloat16_rn(w[i]);
}

// inference epilogue: softmax over the first H outputs (in place), flag
// queries whose inputs leave the training box [lo, hi]
__global__ void infer_finish_kernel(float* __restrict__ Y, const float* __restrict__ X, int B, int O, int H, int I,
                                    const float* __restrict__ lo, const float* __restrict__ hi, int* __restrict__ oor) {
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) / 32, lane = threadIdx.x & 31;
  if (warp >= B) return;
  float* y = Y + (size_t)warp * O;
  float mx = -INFINITY;
  for (int j = lane; j < H; j += 32) mx = fmaxf(mx, y[j]);
  for (int off = 16; off; off >>= 1) mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, off));
  float se = 0.f;
  for (int j = lane; j < H; j += 32) se += expf(y[j] - mx);
  for (int off = 16; off; off >>= 1) se += __shfl_xor_sync(0xffffffffu, se, off);
  const float inv = 1.f / se;
  for (int j = lane; j < H; j += 32) y[j] = expf(y[j] - mx) * inv;
  if (oor) {
    int out = 0;
    for (int j = lane; j < I; j += 32) {
      const float x = X[(size_t)warp * I + j];
      out |= !(x >= lo[j] && x <= hi[j]);
    }
    out = __any_sync(0xffffffffu, out);
    if (lane == 0) oor[warp] = out;
  }
}

// the packed weight image of the tensor-core inference: one thread per
// 16-byte chunk; layer 0 holds its weights twice along K ([0, k0) for the
// inputs' hi slice, [k0, 2 k0) for the lo slice)
struct MlpPackArgs {
  const uint16_t* w[atm::kMlpMaxLayers];  // BF16 bits [out][in] per layer
  int in[atm::kMlpMaxLayers], out[atm::kMlpMaxLayers];
  int k0, n_pieces;
  atm::MlpPiece pieces[atm::kMlpMaxPieces];
};

__global__ void mlp_pack_kernel(const __grid_constant__ MlpPackArgs a, uint4* __restrict__ img, int n_chunks) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n_chunks) return;
  const uint32_t byte = (uint32_t)i * 16u;
  int p = 0;
  while (p + 1 < a.n_pieces && a.pieces[p + 1].src <= byte) ++p;
  const atm::MlpPiece pc = a.pieces[p];
  const uint32_t local = byte - pc.src, kb_bytes = (uint32_t)pc.rows * 128u;
  const int kb = (int)(local / kb_bytes), rem = (int)(local % kb_bytes);
  const int r = rem >> 7, c = ((rem >> 4) & 7) ^ (r & 7);  // stored chunk -> logical chunk
  const int l = pc.layer, row = pc.col0 + r, I = a.in[l];
  uint32_t wv[4];
#pragma unroll
  for (int e = 0; e < 8; e += 2) {
    uint32_t bits[2];
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      int k = kb * 64 + c * 8 + e + h;
      if (l == 0) k = k < a.k0 ? k : (k < 2 * a.k0 ? k - a.k0 : I);
      bits[h] = (row < a.out[l] && k < I) ? a.w[l][(size_t)row * I + k] : 0u;
    }
    wv[e / 2] = bits[0] | (bits[1] << 16);  // the lower K index at the lower address
  }
  img[i] = make_uint4(wv[0], wv[1], wv[2], wv[3]);
}

}  // namespace

struct AtmMlp {
  int device = 0;
  int L = 0;                       // layers
  std::vector<int> width;          // L + 1
  int max_batch = 0;
  size_t n_params = 0;
  std::vector<size_t> w_off, b_off;
  float* w = nullptr;              // FP32 master parameters (W0, b0, W1, b1, ...)
  __nv_bfloat16* wb = nullptr;     // BF16 copies used by the GEMMs
  float* g = nullptr;              // gradients
  float* m = nullptr;
  float* v = nullptr;
  std::vector<float*> act;         // act[0] = input copy ... act[L] = output
  std::vector<float*> pre;         // pre-activations of hidden layers
  float* d0 = nullptr;             // gradient work buffers
  float* d1 = nullptr;
  // tensor-core inference (atm_mlp_infer's default where the shape allows it)
  bool tc_ok = false;
  int form = 0;                    // 0 auto, 1 tile GEMM, 2 tensor cores
  int k0 = 16, out_pad = 0;
  int n_pieces = 0;
  atm::MlpPiece pieces[atm::kMlpMaxPieces];
  unsigned char* img = nullptr;    // packed BF16 weights
  size_t img_bytes = 0;
  bool img_dirty = true;           // the weights changed since the last packing
  int* status = nullptr;           // device word: STATUS_GEMM_WAIT
  ~AtmMlp() {
    cudaFree(img);
    cudaFree(status);
    cudaFree(w);
    cudaFree(wb);
    cudaFree(g);
    cudaFree(m);
    cudaFree(v);
    for (auto p : act) cudaFree(p);
    for (auto p : pre) cudaFree(p);
    cudaFree(d0);
    cudaFree(d1);
  }
};

#define MLP_CUDA(call)                                                                              \
  do {                                                                                              \
    cudaError_t e_ = (call);                                                                        \
    if (e_ != cudaSuccess) return atm::set_error(ATM_ERR_CUDA, "%s: %s", #call, cudaGetErrorString(e_)); \
  } while (0)

extern "C" {

int atm_mlp_create(int32_t n_layers, const int32_t* widths, int32_t max_batch, AtmMlp** out) {
  if (!out || !widths) return atm::set_error(ATM_ERR_INVALID, "NULL argument");
  *out = nullptr;
  if (n_layers < 1 || n_layers > kMaxLayers) return atm::set_error(ATM_ERR_INVALID, "n_layers %d", n_layers);
  if (max_batch < 1) return atm::set_error(ATM_ERR_INVALID, "max_batch %d", max_batch);
  int maxw = 0;
  for (int i = 0; i <= n_layers; ++i) {
    if (widths[i] < 1 || widths[i] > 4096) return atm::set_error(ATM_ERR_INVALID, "width %d", widths[i]);
    maxw = std::max(maxw, (int)widths[i]);
  }
  AtmMlp* p = new AtmMlp();
  cudaGetDevice(&p->device);
  p->L = n_layers;
  p->width.assign(widths, widths + n_layers + 1);
  p->max_batch = max_batch;
  size_t off = 0;
  for (int l = 0; l < n_layers; ++l) {
    p->w_off.push_back(off);
    off += (size_t)widths[l + 1] * widths[l];
    p->b_off.push_back(off);
    off += widths[l + 1];
  }
  p->n_params = off;
  bool ok = cudaMalloc(&p->w, off * 4) == cudaSuccess && cudaMalloc(&p->wb, off * 2) == cudaSuccess &&
            cudaMalloc(&p->g, off * 4) == cudaSuccess && cudaMalloc(&p->m, off * 4) == cudaSuccess &&
            cudaMalloc(&p->v, off * 4) == cudaSuccess &&
            cudaMalloc(&p->d0, (size_t)max_batch * maxw * 4) == cudaSuccess &&
            cudaMalloc(&p->d1, (size_t)max_batch * maxw * 4) == cudaSuccess;
  for (int l = 0; ok && l <= n_layers; ++l) {
    float* a = nullptr;
    ok = cudaMalloc(&a, (size_t)max_batch * widths[l] * 4) == cudaSuccess;
    p->act.push_back(a);
    float* z = nullptr;
    if (ok && l > 0 && l < n_layers) ok = cudaMalloc(&z, (size_t)max_batch * widths[l] * 4) == cudaSuccess;
    p->pre.push_back(z);
  }
  if (!ok) {
    cudaGetLastError();
    delete p;
    return atm::set_error(ATM_ERR_NOMEM, "MLP allocation failed");
  }
  cudaMemset(p->m, 0, off * 4);
  cudaMemset(p->v, 0, off * 4);
  cudaMemset(p->g, 0, off * 4);
  // tensor-core inference: <= 32 inputs, equal hidden widths (a multiple of 64, <= 256), <= 128 outputs
  const int hid = widths[1];
  bool tc = n_layers >= 2 && widths[0] <= 32 && hid % 64 == 0 && hid <= 256 && widths[n_layers] <= 128;
  for (int l = 1; tc && l < n_layers; ++l) tc = widths[l] == hid;
  if (tc) {
    p->k0 = widths[0] <= 16 ? 16 : 32;
    p->out_pad = (widths[n_layers] + 15) / 16 * 16;
    uint32_t src = 0;
    for (int l = 0; tc && l < n_layers; ++l) {
      const int rows_l = l == n_layers - 1 ? p->out_pad : hid;
      const int kblocks = l == 0 ? 1 : hid / 64;
      for (int r0 = 0; r0 < rows_l; r0 += 128) {
        if (p->n_pieces == atm::kMlpMaxPieces) {
          tc = false;
          break;
        }
        atm::MlpPiece& pc = p->pieces[p->n_pieces++];
        pc.layer = l;
        pc.rows = std::min(128, rows_l - r0);
        pc.col0 = r0;
        pc.k_steps = l == 0 ? 2 * p->k0 / 16 : 4 * kblocks;
        pc.src = src;
        pc.bytes = (uint32_t)pc.rows * kblocks * 128u;
        src += pc.bytes;
      }
    }
    p->img_bytes = src;
    tc = tc && cudaMalloc(&p->img, p->img_bytes) == cudaSuccess && cudaMalloc(&p->status, sizeof(int)) == cudaSuccess;
    if (tc) cudaMemset(p->status, 0, sizeof(int));
    cudaGetLastError();
  }
  p->tc_ok = tc;
  *out = p;
  return ATM_OK;
}

int atm_mlp_destroy(AtmMlp* p) {
  if (!p) return ATM_OK;
  cudaDeviceSynchronize();
  delete p;
  return ATM_OK;
}

int64_t atm_mlp_num_params(const AtmMlp* p) { return p ? (int64_t)p->n_params : -1; }

int atm_mlp_set_params(AtmMlp* p, const float* host) {
  if (!p || !host) return atm::set_error(ATM_ERR_INVALID, "NULL argument");
  MLP_CUDA(cudaMemcpy(p->w, host, p->n_params * 4, cudaMemcpyHostToDevice));
  to_bf16_kernel<<<(unsigned)((p->n_params + 255) / 256), 256>>>(p->w, p->wb, (int)p->n_params);
  MLP_CUDA(cudaGetLastError());
  MLP_CUDA(cudaMemset(p->m, 0, p->n_params * 4));
  MLP_CUDA(cudaMemset(p->v, 0, p->n_params * 4));
  MLP_CUDA(cudaDeviceSynchronize());
  p->img_dirty = true;
  return ATM_OK;
}

int atm_mlp_get_params(AtmMlp* p, float* host, float* host_grad) {
  if (!p || !host) return atm::set_error(ATM_ERR_INVALID, "NULL argument");
  MLP_CUDA(cudaDeviceSynchronize());
  MLP_CUDA(cudaMemcpy(host, p->w, p->n_params * 4, cudaMemcpyDeviceToHost));
  if (host_grad) MLP_CUDA(cudaMemcpy(host_grad, p->g, p->n_params * 4, cudaMemcpyDeviceToHost));
  return ATM_OK;
}

// y [batch][out] = MLP(x [batch][in]) (raw outputs, no softmax); keeps the
// activations for atm_mlp_backward
int atm_mlp_forward(AtmMlp* p, const float* x, int32_t batch, float* y, void* stream) {
  if (!p || !x) return atm::set_error(ATM_ERR_INVALID, "NULL argument");
  if (batch < 1 || batch > p->max_batch) return atm::set_error(ATM_ERR_INVALID, "batch %d", batch);
  cudaStream_t st = (cudaStream_t)stream;
  MLP_CUDA(cudaMemcpyAsync(p->act[0], x, (size_t)batch * p->width[0] * 4, cudaMemcpyDeviceToDevice, st));
  for (int l = 0; l < p->L; ++l) {
    const int I = p->width[l], O = p->width[l + 1];
    const __nv_bfloat16* W = p->wb + p->w_off[l];
    const float* b = p->w + p->b_off[l];
    if (l < p->L - 1)
      MLP_CUDA((gemm<float, __nv_bfloat16, EPI_BIAS_GELU>(batch, O, I, p->act[l], I, 1, W, 1, I, p->act[l + 1], O, b,
                                                           p->pre[l + 1], st)));
    else
      MLP_CUDA((gemm<float, __nv_bfloat16, EPI_BIAS>(batch, O, I, p->act[l], I, 1, W, 1, I, p->act[l + 1], O, b,
                                                      nullptr, st)));
  }
  if (y) MLP_CUDA(cudaMemcpyAsync(y, p->act[p->L], (size_t)batch * p->width[p->L] * 4, cudaMemcpyDeviceToDevice, st));
  return ATM_OK;
}

// loss of the last forward pass against targets t [batch][out]: KL over the
// first n_hist outputs (softmax) + w_mse * MSE over the rest; loss_out (device,
// one double) is overwritten; dy [batch][out] (device) receives dLoss/dy
int atm_mlp_loss(AtmMlp* p, const float* t, int32_t batch, int32_t n_hist, float w_mse, double* loss_out, float* dy,
                 void* stream) {
  if (!p || !t || !loss_out || !dy) return atm::set_error(ATM_ERR_INVALID, "NULL argument");
  const int O = p->width[p->L];
  if (n_hist < 1 || n_hist > O) return atm::set_error(ATM_ERR_INVALID, "n_hist %d", n_hist);
  cudaStream_t st = (cudaStream_t)stream;
  MLP_CUDA(cudaMemsetAsync(loss_out, 0, sizeof(double), st));
  loss_kernel<<<(batch * 32 + 255) / 256, 256, 0, st>>>(p->act[p->L], t, batch, O, n_hist, w_mse, dy, loss_out);
  MLP_CUDA(cudaGetLastError());
  return ATM_OK;
}

// gradients of the parameters (kept in the MLP; copied to `grads` if given)
// from dy [batch][out] and the activations of the last forward pass
int atm_mlp_backward(AtmMlp* p, const float* dy, int32_t batch, float* grads, void* stream) {
  if (!p || !dy) return atm::set_error(ATM_ERR_INVALID, "NULL argument");
  if (batch < 1 || batch > p->max_batch) return atm::set_error(ATM_ERR_INVALID, "batch %d", batch);
  cudaStream_t st = (cudaStream_t)stream;
  const float* dz = dy;
  float* bufs[2] = {p->d0, p->d1};
  int which = 0;
  for (int l = p->L - 1; l >= 0; --l) {
    const int I = p->width[l], O = p->width[l + 1];
    // dW[o][i] = sum_b dz[b][o] x[b][i]
    MLP_CUDA((gemm<float, float, EPI_NONE>(O, I, batch, dz, 1, O, p->act[l], I, 1, p->g + p->w_off[l], I, nullptr,
                                           nullptr, st)));
    col_sum_kernel<<<(O + 255) / 256, 256, 0, st>>>(dz, batch, O, p->g + p->b_off[l]);
    MLP_CUDA(cudaGetLastError());
    if (l > 0) {
      // dx[b][i] = sum_o dz[b][o] W[o][i], times gelu'(z) of layer l's input
      const __nv_bfloat16* W = p->wb + p->w_off[l];
      float* dx = bufs[which];
      MLP_CUDA((gemm<float, __nv_bfloat16, EPI_GELU_GRAD>(batch, I, O, dz, O, 1, W, I, 1, dx, I, nullptr, p->pre[l],
                                                          st)));
      dz = dx;
      which ^= 1;
    }
  }
  if (grads) MLP_CUDA(cudaMemcpyAsync(grads, p->g, p->n_params * 4, cudaMemcpyDeviceToDevice, st));
  return ATM_OK;
}

int atm_mlp_adam(AtmMlp* p, float lr, float b1, float b2, float eps, float weight_decay, int32_t step,
                 void* stream) {
  if (!p || step < 1) return atm::set_error(ATM_ERR_INVALID, "bad Adam arguments");
  const float c1 = 1.f - powf(b1, (float)step), c2 = 1.f - powf(b2, (float)step);
  adam_kernel<<<(unsigned)((p->n_params + 255) / 256), 256, 0, (cudaStream_t)stream>>>(
      p->w, p->wb, p->g, p->m, p->v, (int)p->n_params, lr, b1, b2, eps, c1, c2, weight_decay);
  MLP_CUDA(cudaGetLastError());
  p->img_dirty = true;
  return ATM_OK;
}

// inference: y [batch][out] with a softmax over the first n_hist outputs;
// out_of_range[b] = 1 where an input leaves [lo, hi] (device arrays; lo/hi
// may be NULL to skip the check)
int atm_mlp_infer(AtmMlp* p, const float* x, int32_t batch, const float* lo, const float* hi, int32_t n_hist,
                  float* y, int32_t* out_of_range, void* stream) {
  if (!p || !x || !y) return atm::set_error(ATM_ERR_INVALID, "NULL argument");
  if (batch < 0) return atm::set_error(ATM_ERR_INVALID, "batch %d", batch);
  if (n_hist < 1 || n_hist > p->width[p->L]) return atm::set_error(ATM_ERR_INVALID, "n_hist %d", n_hist);
  cudaStream_t st = (cudaStream_t)stream;
  const int O = p->width[p->L], I0 = p->width[0];
  if (p->tc_ok && p->form != 1) {
    if (p->img_dirty) {
      MlpPackArgs pa{};
      for (int l = 0; l < p->L; ++l) {
        pa.w[l] = reinterpret_cast<const uint16_t*>(p->wb + p->w_off[l]);
        pa.in[l] = p->width[l];
        pa.out[l] = p->width[l + 1];
      }
      pa.k0 = p->k0;
      pa.n_pieces = p->n_pieces;
      std::copy(p->pieces, p->pieces + p->n_pieces, pa.pieces);
      const int n_chunks = (int)(p->img_bytes / 16);
      mlp_pack_kernel<<<(n_chunks + 255) / 256, 256, 0, st>>>(pa, reinterpret_cast<uint4*>(p->img), n_chunks);
      MLP_CUDA(cudaGetLastError());
      p->img_dirty = false;
    }
    atm::MlpTcArgs a{};
    a.x = x;
    a.y = y;
    a.oor = (lo && hi) ? out_of_range : nullptr;
    a.lo = (lo && hi && out_of_range) ? lo : nullptr;
    a.hi = (lo && hi && out_of_range) ? hi : nullptr;
    a.img = p->img;
    for (int l = 0; l < p->L; ++l) a.bias[l] = p->w + p->b_off[l];
    a.batch = batch;
    a.in = I0;
    a.k0 = p->k0;
    a.hidden = p->width[1];
    a.out = O;
    a.out_pad = p->out_pad;
    a.layers = p->L;
    a.n_hist = n_hist;
    a.n_pieces = p->n_pieces;
    a.status = p->status;
    std::copy(p->pieces, p->pieces + p->n_pieces, a.pieces);
    MLP_CUDA(atm::launch_mlp_infer_tc(a, st));
    return ATM_OK;
  }
  for (int b0 = 0; b0 < batch; b0 += p->max_batch) {
    const int nb = std::min(p->max_batch, batch - b0);
    if (int rc = atm_mlp_forward(p, x + (size_t)b0 * I0, nb, y + (size_t)b0 * O, stream)) return rc;
    infer_finish_kernel<<<(nb * 32 + 255) / 256, 256, 0, st>>>(y + (size_t)b0 * O, x + (size_t)b0 * I0, nb, O, n_hist,
                                                               I0, lo, hi,
                                                               (lo && hi && out_of_range) ? out_of_range + b0 : nullptr);
    MLP_CUDA(cudaGetLastError());
  }
  return ATM_OK;
}

int atm_mlp_set_infer_form(AtmMlp* p, int32_t form) {
  if (!p) return atm::set_error(ATM_ERR_INVALID, "NULL argument");
  if (form < 0 || form > 2) return atm::set_error(ATM_ERR_INVALID, "form %d", form);
  if (form == 2 && !p->tc_ok)
    return atm::set_error(ATM_ERR_UNSUPPORTED, "this MLP's shape has no tensor-core inference form");
  p->form = form;
  return ATM_OK;
}

int atm_mlp_infer_form(const AtmMlp* p) {
  if (!p) return atm::set_error(ATM_ERR_INVALID, "NULL argument");
  return p->tc_ok && p->form != 1 ? 2 : 1;
}

int atm_mlp_check(AtmMlp* p) {
  if (!p) return atm::set_error(ATM_ERR_INVALID, "NULL argument");
  MLP_CUDA(cudaDeviceSynchronize());
  if (!p->status) return ATM_OK;
  int word = 0;
  MLP_CUDA(cudaMemcpy(&word, p->status, sizeof(int), cudaMemcpyDeviceToHost));
  if (!word) return ATM_OK;
  MLP_CUDA(cudaMemset(p->status, 0, sizeof(int)));
  return atm::set_error(ATM_ERR_TIMEOUT, "a bounded wait of the tensor-core inference ran out");
}

}  // extern "C"
