// pf_noalloc.cu -- max|div u| on caller-provided device arrays without any
// device allocation (pf_max_div_noalloc in include/pixelflow_gpu.h).
//
// Some host programs cannot call cudaMalloc at the point where they want this
// diagnostic: cudaMalloc and cudaFree synchronise the whole device, which a
// loop that keeps other requests running on other streams cannot afford, and
// some programs run under a memory budget owned by another allocator (a
// framework that has reserved the HBM up front) and may not take device memory
// of their own.  For them this entry point reduces into a fixed scratch array
// that lives in the library image itself, so a call launches kernels and does
// nothing else to the device.
//
// The scratch holds one partial maximum per grid row (j, k); it is
// PF_NOALLOC_MAX_ROWS entries (2 MiB), so a case with n*l rows above that is
// rejected.  Every GPU that loads the library keeps the array until the
// process exits.  Each call overwrites the first n*l entries and the final
// kernel reads exactly those, so nothing has to be cleared between calls.
// All calls share the one array: calls that overlap on the GPU (different
// streams, different host threads) race on it and must be serialised by the
// caller.  The first call on a device looks up the array's device address
// with cudaGetSymbolAddress (with that device current) and caches it; make
// that first call before any stream capture begins.  The cached address is
// the array's address in the device's primary context: it stays valid for
// the life of the process as long as the caller uses the primary context and
// does not reset the device (cudaDeviceReset unloads the library's module).
#include <cuda_runtime.h>

#include <mutex>

#include "pf_internal.cuh"

namespace pf {
namespace {

static __device__ __align__(256) unsigned long long g_noalloc_rows[PF_NOALLOC_MAX_ROWS];

constexpr int kMaxDevices = 64;
std::mutex g_noalloc_mu;
unsigned long long* g_noalloc_ptr[kMaxDevices] = {nullptr};

__device__ __forceinline__ unsigned long long abs_bits_d(double x) {
  return (unsigned long long)__double_as_longlong(x) & 0x7fffffffffffffffULL;
}

// One warp per row (j, k): max over i of |porosity-weighted divergence|, the
// same algebra as the case kernel k_div_diag:
//   gx*u_c + eps_c*(u_e - u_w)/(2dx) + ...,  gx = (eps_e - eps_w)/(2dx).
__global__ void k_rowmax_div(int dim, int m, int n, int l, long long ld1, long long ld2, double hx, double hy,
                             double hz, const double* __restrict__ u, const double* __restrict__ v,
                             const double* __restrict__ w, const double* __restrict__ po,
                             unsigned long long* __restrict__ rows) {
  const long long row = (long long)blockIdx.x * (blockDim.x / 32) + threadIdx.x / 32;
  const int lane = threadIdx.x & 31;
  const long long nrows = (long long)n * l;
  if (row >= nrows) return;  // whole warp leaves together
  const int j = (int)(row % n) + 1;
  const int k = dim == 3 ? (int)(row / n) + 1 : 0;
  const long long X = ld1, XY = ld1 * ld2;
  unsigned long long e = 0;
  for (int i = 1 + lane; i <= m; i += 32) {
    const long long q = (long long)i + X * ((long long)j + ld2 * k);
    const double gx = (po[q + 1] - po[q - 1]) * hx;
    const double gy = (po[q + X] - po[q - X]) * hy;
    double sd = (u[q + 1] - u[q - 1]) * hx;
    sd = fma(v[q + X] - v[q - X], hy, sd);
    double sg = gx * u[q];
    sg = fma(gy, v[q], sg);
    if (dim == 3) {
      const double gz = (po[q + XY] - po[q - XY]) * hz;
      sd = fma(w[q + XY] - w[q - XY], hz, sd);
      sg = fma(gz, w[q], sg);
    }
    const unsigned long long b = abs_bits_d(fma(po[q], sd, sg));
    e = b > e ? b : e;
  }
  for (int o = 16; o > 0; o >>= 1) {
    const unsigned long long t = __shfl_xor_sync(0xffffffffu, e, o);
    e = t > e ? t : e;
  }
  if (lane == 0) rows[row] = e;
}

// Single block: max over the row partials, written as a double.
__global__ void k_rows_to_max(const unsigned long long* __restrict__ rows, long long nrows, double* out) {
  __shared__ unsigned long long red[32];
  unsigned long long e = 0;
  for (long long r = threadIdx.x; r < nrows; r += blockDim.x) {
    const unsigned long long b = rows[r];
    e = b > e ? b : e;
  }
  for (int o = 16; o > 0; o >>= 1) {
    const unsigned long long t = __shfl_xor_sync(0xffffffffu, e, o);
    e = t > e ? t : e;
  }
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = e;
  __syncthreads();
  if (threadIdx.x < 32) {
    e = threadIdx.x < blockDim.x / 32 ? red[threadIdx.x] : 0ULL;
    for (int o = 16; o > 0; o >>= 1) {
      const unsigned long long t = __shfl_xor_sync(0xffffffffu, e, o);
      e = t > e ? t : e;
    }
    if (threadIdx.x == 0) *out = __longlong_as_double((long long)e);
  }
}

// Device address of the scratch array on the current device (looked up once).
int noalloc_scratch(unsigned long long** out) {
  int dev = 0;
  PF_CUDA(cudaGetDevice(&dev));
  if (dev < 0 || dev >= kMaxDevices) return fail(PF_E_INVALID, "device ordinal out of range");
  std::lock_guard<std::mutex> lock(g_noalloc_mu);
  if (!g_noalloc_ptr[dev]) {
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_rows);
    if (e != cudaSuccess) return cuda_fail(e, "cudaGetSymbolAddress(noalloc scratch)");
    g_noalloc_ptr[dev] = static_cast<unsigned long long*>(p);
  }
  *out = g_noalloc_ptr[dev];
  return PF_OK;
}

}  // namespace
}  // namespace pf

using namespace pf;

extern "C" int pf_max_div_noalloc(const pf_params* prm, const double* u, const double* v, const double* w,
                                  const double* porosity, int ld1, int ld2, double* max_div, void* stream) {
  if (!prm || !u || !v || !porosity || !max_div || (prm->dim == 3 && !w))
    return fail(PF_E_INVALID, "pf_max_div_noalloc: null argument");
  if (prm->dim != 2 && prm->dim != 3) return fail(PF_E_INVALID, "pf_max_div_noalloc: dim must be 2 or 3");
  if (prm->m < 3 || prm->n < 3 || (prm->dim == 3 && prm->l < 3))
    return fail(PF_E_INVALID, "pf_max_div_noalloc: grid sizes must be >= 3");
  if (ld1 < prm->m + 2 || ld2 < prm->n + 2)
    return fail(PF_E_INVALID, "pf_max_div_noalloc: leading dimensions smaller than m+2, n+2");
  if (!(prm->width > 0 && prm->height > 0 && (prm->dim == 2 || prm->depth > 0)))
    return fail(PF_E_INVALID, "pf_max_div_noalloc: width/height/depth must be > 0");
  const int l = prm->dim == 3 ? prm->l : 1;
  const long long nrows = (long long)prm->n * l;
  if (nrows > PF_NOALLOC_MAX_ROWS)
    return fail(PF_E_INVALID, "pf_max_div_noalloc: n*l = " + std::to_string(nrows) +
                                  " rows exceeds the scratch limit PF_NOALLOC_MAX_ROWS = " +
                                  std::to_string((long long)PF_NOALLOC_MAX_ROWS));
  unsigned long long* rows = nullptr;
  int rc = noalloc_scratch(&rows);
  if (rc) return rc;
  const double hx = 0.5 / (prm->width / double(prm->m - 1));
  const double hy = 0.5 / (prm->height / double(prm->n - 1));
  const double hz = prm->dim == 3 ? 0.5 / (prm->depth / double(prm->l - 1)) : 0.0;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  const int warps = 8;
  const unsigned blocks = (unsigned)((nrows + warps - 1) / warps);
  k_rowmax_div<<<blocks, warps * 32, 0, st>>>(prm->dim, prm->m, prm->n, l, ld1, ld2, hx, hy, hz, u, v, w,
                                              porosity, rows);
  k_rows_to_max<<<1, 1024, 0, st>>>(rows, nrows, max_div);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_fail(e, "pf_max_div_noalloc launch");
  return PF_OK;
}
