// pf_sor_list.cu -- the plain FP64 red-black half-sweep of 3D cases, driven
// by per-colour cell lists with the pure-fluid cells first.
//
// The reference's SOR update (ibm_3d_uniform_omp_cpu.f90:433-614) in the
// normalised form of k_sor_half,
//   p = (1-omega) p + bbn - sum_nb a_nb p_nb,
// costs 7 FP64 FMAs and 80 bytes of operator and pressure traffic per cell
// on GB300, whose FP64 pipe runs at 1/64 of the FP32 rate: k_sor_half sits
// on the FP64 roof and the HBM roof at the same time.  Most cells of a case
// are pure fluid: the cell and its six neighbours have porosity exactly 1,
// so the six normalised coefficients are the same constant a for every such
// cell (bit for bit, dx = dy = dz), and the update is
//   p = (1-omega) p + bbn - a * (p_e + p_w + p_n + p_s + p_t + p_b).
// Those cells skip the six coefficient loads (48 of the 80 bytes) and form
// the neighbour sum exactly, with integer arithmetic on the aligned
// significands, rounded once to FP64: two FP64 FMAs per update instead of
// seven.  Every other cell keeps k_sor_half's arithmetic.
//
// A warp must not mix the two paths (a masked-off lane still occupies the
// FP64 pipe, and a run of 32 cells along x that touches any obstacle would
// drop the whole warp to the slow path).  So at set-up each colour's cells
// are listed once, the fluid cells first and then the others, each part in
// memory order, and one launch per half-sweep walks the list: thread t
// updates cell list[t], and only the warp at the boundary of the two parts
// diverges.  Entries pack (h, j, k) into 32 bits (11 + 11 + 10 bits).
//
// Arithmetic against k_sor_half: the fluid cells' neighbour sum is rounded
// once instead of six times, so the iterates differ in the last bits; the
// red-black order, the neighbour values each update reads and the iteration
// count are the same.
#include <cuda_runtime.h>

#include <string.h>

#include <vector>

#include "pf_case.cuh"
#include "pf_cells.cuh"

namespace pf {

namespace {

constexpr int LIST_THREADS = 256;

// Exact sum of six doubles, rounded once to nearest (ties to even when no
// bits fell below the guard bits).  Each significand, with its implicit
// bit, is shifted to the scale 2^(Emax - 1075 - G) of the largest exponent
// with G = 7 guard bits; six terms below 2^60 add up without overflow in a
// signed 64-bit integer.  A term more than G binades below the largest
// loses the bits shifted out (truncated), an error below 2^-7 of the
// largest term's last place.  Returns false (result unset) when an input
// is Inf or NaN or the sum is not a normal number; the caller then adds in
// FP64.
__device__ __forceinline__ bool sum6_exact(const double (&x)[6], double& out) {
  constexpr int G = 7;
  unsigned long long mant[6];
  int ex[6];
  bool neg[6];
  int emax = 1;
  bool finite = true;
#pragma unroll
  for (int q = 0; q < 6; q++) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(x[q]);
    const int e = (int)((b >> 52) & 0x7ff);
    finite = finite && e != 0x7ff;
    mant[q] = (b & 0x000fffffffffffffULL) | (e ? (1ULL << 52) : 0ULL);
    ex[q] = e ? e : 1;
    neg[q] = (b >> 63) != 0;
    emax = max(emax, ex[q]);
  }
  long long s = 0;
#pragma unroll
  for (int q = 0; q < 6; q++) {
    const int d = emax - ex[q];
    const unsigned long long a = d <= G ? (mant[q] << (G - d)) : (d - G < 64 ? mant[q] >> (d - G) : 0ULL);
    s += neg[q] ? -(long long)a : (long long)a;
  }
  if (!finite) return false;
  if (s == 0) {
    out = 0.0;
    return true;
  }
  const bool sn = s < 0;
  unsigned long long u = sn ? (unsigned long long)(-s) : (unsigned long long)s;
  const int lead = 63 - __clzll((long long)u);
  int sh = lead - 52;
  unsigned long long m;
  if (sh > 0) {
    m = u >> sh;
    const unsigned long long rem = u & ((1ULL << sh) - 1), half = 1ULL << (sh - 1);
    if (rem > half || (rem == half && (m & 1))) m++;
    if (m == (1ULL << 53)) {
      m >>= 1;
      sh++;
    }
  } else {
    m = u << (-sh);
  }
  const int eb = emax - G + sh;  // biased exponent of the result
  if (eb <= 0 || eb >= 0x7ff) return false;
  const unsigned long long bits =
      (sn ? (1ULL << 63) : 0ULL) | ((unsigned long long)eb << 52) | (m & 0x000fffffffffffffULL);
  out = __longlong_as_double((long long)bits);
  return true;
}

// Per packed work item of one colour (the mapping of k_sor_half): 0 not a
// cell (i = 0 or m+1), 1 pure fluid (all six normalised coefficients equal
// the fluid constants, no outlet addend), 2 any other cell.  Block 0 also
// writes the fluid constants (a_e .. a_b of a cell and neighbours of
// porosity 1, normalised by omega/ap, by the same device arithmetic as
// k_setup_coef).
__global__ void k_fluid_flags(Geo g, Scal s, Coef<double> C, int colour, unsigned char* flags, double* consts) {
  double a[6], ap;
  coef_set(g, s, 1.0, 1.0, 1.0, 1.0, 1.0, 1.0, 1.0, a, ap);
  const double wap = s.omega / ap;
  double f[6];
#pragma unroll
  for (int d = 0; d < 6; d++) f[d] = a[d] * wap;
  if (blockIdx.x == 0 && threadIdx.x < 6) consts[threadIdx.x] = f[threadIdx.x];
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= packed_items(g)) return;
  int h, j, k;
  packed_item<3>(g, (int)t, h, j, k);
  const int sd = (colour + j + k) & 1;
  const int i = 2 * h + sd;
  unsigned char out = 0;
  if (i >= 1 && i <= g.m) {
    const idx_t q = pk_idx(g, h, j, k);
    bool fl = C.oadd[q] == 0.0;
#pragma unroll
    for (int d = 0; d < 6; d++)
      fl = fl && __double_as_longlong(C.a[d][q]) == __double_as_longlong(f[d]);
    out = fl ? 1 : 2;
  }
  flags[t] = out;
}

// One half-sweep over the list: entries [0, nfluid) are fluid cells,
// [nfluid, ntotal) the others.  ISO: the six fluid constants are equal
// (dx = dy = dz); otherwise the fluid cells use the three constants with
// FP64 FMAs (still without coefficient loads).  EARLY: the list entry and
// the operator load before griddepcontrol.wait (see k_sor_half).
template <bool TRACK, bool EARLY, bool ISO>
__global__ void __launch_bounds__(LIST_THREADS)
    k_sor_list3(Geo g, Coef<double> C, double* __restrict__ pc, const double* __restrict__ po, double omw,
                int colour, const unsigned* __restrict__ list, int nfluid, int ntotal, double ax, double ay,
                double az, unsigned long long* __restrict__ err, const int* __restrict__ skip) {
  const int t = blockIdx.x * LIST_THREADS + threadIdx.x;
  const bool act = t < ntotal;
  const bool fl = t < nfluid;
  int h = 0, j = 1, k = 1;
  idx_t q = 0;
  double cb = 0.0, c0 = 0.0, c1 = 0.0, c2 = 0.0, c3 = 0.0, c4 = 0.0, c5 = 0.0;
  auto locate = [&]() {
    const unsigned e = list[t];
    h = (int)(e & 0x7ffu);
    j = (int)((e >> 11) & 0x7ffu);
    k = (int)(e >> 22);
    q = pk_idx(g, h, j, k);
  };
  auto load_operator = [&]() {
    cb = C.bbn[q];
    if (!fl) {
      c0 = C.a[0][q];
      c1 = C.a[1][q];
      c2 = C.a[2][q];
      c3 = C.a[3][q];
      c4 = C.a[4][q];
      c5 = C.a[5][q];
    }
  };
  if (act) locate();
  if (EARLY && act) load_operator();
  pdl_begin();
  if (skip && *skip) return;
  if (!EARLY && act) load_operator();
  unsigned long long e = 0;
  if (act) {
    const int s = (colour + j + k) & 1;
    const idx_t H = g.H, HY = (idx_t)g.H * g.Y;
    const idx_t qn = (j == g.n) ? pk_idx(g, h, g.jn_n, k) : q + H;
    const idx_t qs = (j == 1) ? pk_idx(g, h, g.js_1, k) : q - H;
    const idx_t qt = (k == g.l) ? pk_idx(g, h, j, g.kt_l) : q + HY;
    const idx_t qb = (k == 1) ? pk_idx(g, h, j, g.kb_1) : q - HY;
    const double pold = pc[q];
    const double x[6] = {po[q + s], po[q - 1 + s], po[qn], po[qs], po[qt], po[qb]};
    double tt;
    if (fl) {
      if (ISO) {
        double sum;
        if (!sum6_exact(x, sum)) sum = ((((x[0] + x[1]) + x[2]) + x[3]) + x[4]) + x[5];
        tt = fma(-ax, sum, cb);
      } else {
        tt = cb;
        tt = fma(-ax, x[0], tt);
        tt = fma(-ax, x[1], tt);
        tt = fma(-ay, x[2], tt);
        tt = fma(-ay, x[3], tt);
        tt = fma(-az, x[4], tt);
        tt = fma(-az, x[5], tt);
      }
    } else {
      tt = cb;
      tt = fma(-c0, x[0], tt);
      tt = fma(-c1, x[1], tt);
      tt = fma(-c2, x[2], tt);
      tt = fma(-c3, x[3], tt);
      tt = fma(-c4, x[4], tt);
      tt = fma(-c5, x[5], tt);
    }
    const double pnew = fma(omw, pold, tt);
    pc[q] = pnew;
    if (TRACK) e = abs_diff_bits(pnew, pold);
  }
  if (TRACK) warp_max_atomic(e, err);
}

// Exact six-term sums of n groups (testing entry point).
__global__ void k_sum6(const double* __restrict__ x, int n, double* __restrict__ out, int* __restrict__ ok) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  double v[6];
#pragma unroll
  for (int q = 0; q < 6; q++) v[q] = x[6 * i + q];
  double r = 0.0;
  const bool good = sum6_exact(v, r);
  out[i] = good ? r : 0.0;
  ok[i] = good ? 1 : 0;
}

}  // namespace

bool sor_list_eligible(const Geo& g) {
  return g.dim == 3 && !g.wall && ((g.m >> 1) + 1) < 2048 && g.n < 2048 && g.l < 1024;
}

// Builds both colours' lists on the device: flags per work item, copied to
// the host, partitioned (fluid cells, then the rest, each in memory order),
// packed and copied back into one allocation.
int sor_list_setup(pf_case* c) {
  const Geo& g = c->g;
  const long long items = packed_items(g);
  unsigned char* dflags = nullptr;
  double* dconst = nullptr;
  PF_CUDA(cudaMalloc(&dflags, (size_t)items));
  cudaError_t e = cudaMalloc(&dconst, 6 * sizeof(double));
  if (e != cudaSuccess) {
    cudaFree(dflags);
    return cuda_fail(e, "cudaMalloc(fluid constants)");
  }
  std::vector<unsigned char> flags((size_t)items);
  std::vector<unsigned> lists[2];
  double consts[6] = {0, 0, 0, 0, 0, 0};
  const unsigned grid = (unsigned)((items + LIST_THREADS - 1) / LIST_THREADS);
  int rc = PF_OK;
  for (int col = 0; col < 2 && rc == PF_OK; col++) {
    k_fluid_flags<<<grid, LIST_THREADS, 0, c->st>>>(g, c->s, c->C[col], col, dflags, dconst);
    e = cudaMemcpyAsync(flags.data(), dflags, (size_t)items, cudaMemcpyDeviceToHost, c->st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(consts, dconst, sizeof(consts), cudaMemcpyDeviceToHost, c->st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->st);
    if (e != cudaSuccess) {
      rc = cuda_fail(e, "fluid flags");
      break;
    }
    std::vector<unsigned>& L = lists[col];
    const int W = packed_width(g);
    int nfl = 0;
    for (int pass = 1; pass <= 2; pass++) {
      for (long long t = 0; t < items; t++) {
        if (flags[(size_t)t] != pass) continue;
        const int row = (int)(t / W);
        const int h = (int)(t - (long long)row * W);
        const int k = row / g.n + 1, j = row - (k - 1) * g.n + 1;
        L.push_back((unsigned)h | ((unsigned)j << 11) | ((unsigned)k << 22));
      }
      if (pass == 1) nfl = (int)L.size();
    }
    c->list_nfluid[col] = nfl;
    c->list_ntotal[col] = (int)L.size();
  }
  cudaFree(dflags);
  cudaFree(dconst);
  if (rc) return rc;
  const size_t n0 = lists[0].size(), n1 = lists[1].size();
  unsigned* d = nullptr;
  PF_CUDA(cudaMalloc(&d, (n0 + n1) * sizeof(unsigned)));
  c->list_base = d;
  c->list[0] = d;
  c->list[1] = d + n0;
  c->list_bytes = (n0 + n1) * sizeof(unsigned);
  PF_CUDA(cudaMemcpyAsync(c->list[0], lists[0].data(), n0 * sizeof(unsigned), cudaMemcpyHostToDevice, c->st));
  PF_CUDA(cudaMemcpyAsync(c->list[1], lists[1].data(), n1 * sizeof(unsigned), cudaMemcpyHostToDevice, c->st));
  PF_CUDA(cudaStreamSynchronize(c->st));
  for (int d6 = 0; d6 < 6; d6++) c->list_const[d6] = consts[d6];
  const auto bits = [](double v) {
    unsigned long long b;
    memcpy(&b, &v, sizeof b);
    return b;
  };
  c->list_iso = bits(consts[0]) == bits(consts[1]) && bits(consts[0]) == bits(consts[2]) &&
                bits(consts[0]) == bits(consts[3]) && bits(consts[0]) == bits(consts[4]) &&
                bits(consts[0]) == bits(consts[5]);
  return PF_OK;
}

void launch_sor_list(const pf_case* c, int col, double omw, unsigned long long* err, bool early,
                     cudaStream_t st) {
  const Geo& g = c->g;
  const int nt = c->list_ntotal[col];
  const unsigned grid = (unsigned)((nt + LIST_THREADS - 1) / LIST_THREADS);
  const double ax = c->list_const[0], ay = c->list_const[2], az = c->list_const[4];
#define PF_SL(TR, EA, ISO)                                                                                      \
  launch_pdl(k_sor_list3<TR, EA, ISO>, dim3(grid), dim3(LIST_THREADS), st, g, c->C[col], c->p[col],          \
             (const double*)c->p[1 - col], omw, col, (const unsigned*)c->list[col], c->list_nfluid[col], nt, ax, \
             ay, az, err, (const int*)nullptr)
  if (c->list_iso) {
    if (err)
      early ? PF_SL(true, true, true) : PF_SL(true, false, true);
    else
      early ? PF_SL(false, true, true) : PF_SL(false, false, true);
  } else {
    if (err)
      early ? PF_SL(true, true, false) : PF_SL(true, false, false);
    else
      early ? PF_SL(false, true, false) : PF_SL(false, false, false);
  }
#undef PF_SL
}

}  // namespace pf

using namespace pf;

extern "C" int pf_debug_sum6(const double* x, int n, double* out, int* ok) {
  if (!x || !out || !ok || n < 0) return fail(PF_E_INVALID, "pf_debug_sum6: bad argument");
  if (n == 0) return PF_OK;
  double *dx = nullptr, *dout = nullptr;
  int* dok = nullptr;
  int rc = PF_OK;
  cudaError_t e = cudaMalloc(&dx, (size_t)n * 6 * sizeof(double));
  if (e == cudaSuccess) e = cudaMalloc(&dout, (size_t)n * sizeof(double));
  if (e == cudaSuccess) e = cudaMalloc(&dok, (size_t)n * sizeof(int));
  if (e == cudaSuccess) e = cudaMemcpy(dx, x, (size_t)n * 6 * sizeof(double), cudaMemcpyHostToDevice);
  if (e == cudaSuccess) {
    k_sum6<<<(n + 255) / 256, 256>>>(dx, n, dout, dok);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaMemcpy(out, dout, (size_t)n * sizeof(double), cudaMemcpyDeviceToHost);
  if (e == cudaSuccess) e = cudaMemcpy(ok, dok, (size_t)n * sizeof(int), cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) rc = cuda_fail(e, "pf_debug_sum6");
  cudaFree(dx);
  cudaFree(dout);
  cudaFree(dok);
  return rc;
}
