// atm_vacuum_noalloc: the vacuum step of atm_vacuum without a plan and
// without any device allocation.
//
// Who needs it: callers that cannot call cudaMalloc / cudaFree on the path
// where they propagate a field -- e.g. a host framework whose caching
// allocator already holds the device memory budget (a raw cudaMalloc would
// fail or fragment it), or a latency-sensitive loop that must not pay the
// implicit device-wide synchronisation of cudaFree.  They pass the field
// (input and output) and the geometry; the engine keeps its per-call tables
// (FFT twiddles and the two 1-D transfer functions) in the fixed-size
// device array below.
//
// Rules of use:
//   * N is a power of two in [128, 4096]; larger N is rejected with
//     ATM_ERR_UNSUPPORTED, because the static table holds 3 x 4096 complex64
//     (96 KiB).  Every GPU that loads libatm.so holds that array until the
//     process exits.
//   * The first call on a device looks up the array's device address with
//     cudaGetSymbolAddress (once per device, with that device current); make
//     that first call before capturing any stream on the device.  The address
//     is kept for the life of the process: do not reset the device
//     (cudaDeviceReset) while the library is loaded, since the array may be
//     placed elsewhere in the new context.
//   * All calls share the one array.  Each call rewrites every table entry it
//     reads before reading it, so nothing carries over between calls, but
//     calls whose GPU work overlaps (different streams, no ordering) race on
//     the tables and give wrong results: order them on one stream.
#include <mutex>

#include "../../include/atm.h"
#include "atm_common.cuh"
#include "atm_internal.h"

namespace {

constexpr int kNoAllocMaxN = 4096;
constexpr int kMaxDevices = 64;

// [0, N): twiddles exp(-2 pi i n / N); [N, 2N): y transfer function incl.
// exp(i k dz) / N^2; [2N, 3N): x transfer function
__device__ __align__(256) float2 g_vacuum_tables[3 * kNoAllocMaxN];

std::mutex g_mu;
void* g_table_addr[kMaxDevices] = {};

// device address of g_vacuum_tables on the current device (set up once per device)
int table_address(float2** out) {
  int dev = -1;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return atm::set_error(ATM_ERR_CUDA, "cudaGetDevice failed: %s", cudaGetErrorString(e));
  if (dev < 0 || dev >= kMaxDevices) return atm::set_error(ATM_ERR_UNSUPPORTED, "device index %d too large", dev);
  std::lock_guard<std::mutex> lock(g_mu);
  if (!g_table_addr[dev]) {
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_vacuum_tables);
    if (e != cudaSuccess || !p)
      return atm::set_error(ATM_ERR_CUDA, "cudaGetSymbolAddress of the vacuum tables failed: %s",
                            cudaGetErrorString(e));
    g_table_addr[dev] = p;
  }
  *out = static_cast<float2*>(g_table_addr[dev]);
  return ATM_OK;
}

__global__ void vacuum_tables_kernel(float2* tab, int N, double delta, double kw, double dz) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= N) return;
  const double pi = 3.14159265358979323846;
  double s, c;
  sincospi(-2.0 * (double)k / (double)N, &s, &c);
  tab[k] = make_float2((float)c, (float)s);
  // same FP64 expressions as the plan's tables
  const double df = 1.0 / (N * delta);
  const double c1 = (pi * dz) * (2.0 * pi / kw);
  const double f = (double)(k < N / 2 ? k : k - N) * df;
  double sa, ca, gs, gc;
  sincos(c1 * (f * f), &sa, &ca);
  sincos(kw * dz, &gs, &gc);
  const double inv = 1.0 / ((double)N * (double)N);
  // (gc + i gs)(ca - i sa) / N^2
  tab[N + k] = make_float2((float)((gc * ca + gs * sa) * inv), (float)((gs * ca - gc * sa) * inv));
  tab[2 * N + k] = make_float2((float)ca, (float)-sa);
}

}  // namespace

extern "C" int atm_vacuum_noalloc(void* field, int32_t N, int32_t batch, double delta, double wvl, double dz,
                                  void* stream) {
  if (!field) return atm::set_error(ATM_ERR_INVALID, "field is NULL");
  if (batch < 1 || batch > 65535) return atm::set_error(ATM_ERR_INVALID, "batch %d out of range", batch);
  if (N > kNoAllocMaxN)
    return atm::set_error(ATM_ERR_UNSUPPORTED,
                          "N = %d exceeds the allocation-free maximum of %d (its static table holds 3 x %d complex64)",
                          N, kNoAllocMaxN, kNoAllocMaxN);
  if (!atm::supported_n(N))
    return atm::set_error(ATM_ERR_UNSUPPORTED, "N = %d unsupported: need a power of two in [128, %d]", N,
                          kNoAllocMaxN);
  if (!(delta > 0) || !(wvl > 0)) return atm::set_error(ATM_ERR_INVALID, "delta and wvl must be > 0");
  if (!(dz > 0)) return ATM_OK;  // VacuumPath: a step of length <= 0 is the identity
  float2* tab = nullptr;
  if (int rc = table_address(&tab)) return rc;
  cudaStream_t st = (cudaStream_t)stream;
  const double kw = 2.0 * 3.14159265358979323846 / wvl;
  vacuum_tables_kernel<<<(N + 255) / 256, 256, 0, st>>>(tab, N, delta, kw, dz);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return atm::set_error(ATM_ERR_CUDA, "vacuum table kernel: %s", cudaGetErrorString(e));
  atm::RowArgs ra{};
  ra.field = (float2*)field;
  ra.tw = tab;
  ra.loss = 1.f;
  ra.delta = (float)delta;
  ra.delta64 = delta;
  ra.flags = atm::ROW_FWD | atm::ROW_STORE;
  if ((e = atm::launch_row_pass(N, batch, ra, st)) != cudaSuccess)
    return atm::set_error(ATM_ERR_CUDA, "row pass: %s", cudaGetErrorString(e));
  atm::ColArgs ca{};
  ca.field = (float2*)field;
  ca.tw = tab;
  ca.hy = tab + N;
  ca.hx = tab + 2 * N;
  if ((e = atm::launch_col_pass(N, batch, 0, ca, st)) != cudaSuccess)
    return atm::set_error(ATM_ERR_CUDA, "column pass: %s", cudaGetErrorString(e));
  ra.flags = atm::ROW_INV | atm::ROW_STORE;
  if ((e = atm::launch_row_pass(N, batch, ra, st)) != cudaSuccess)
    return atm::set_error(ATM_ERR_CUDA, "row pass: %s", cudaGetErrorString(e));
  return ATM_OK;
}
