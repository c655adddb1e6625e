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
// are split into a fluid list and a list of the others, each in memory
// order and cut into chunks of 32 (one warp); the chunks of both lists are
// then merged by position, so a warp's chunk is all fluid or all other, and
// warps working side by side touch the same region of the arrays (a first
// version ran all fluid cells before all others: the others' sectors were
// fetched twice, +35 % DRAM reads).  An entry is the cell's packed index q
// (26 bits), its x parity and whether it sits on the first or last row or
// plane (the periodic neighbours), and the fluid bit, so every neighbour
// address is q plus a constant.
//
// The list entry is one more dependent load ahead of the cell's operands: a
// launch of one cell per thread (36 waves of short CTAs at 256^3) paid two
// DRAM round trips per wave and ran latency-bound (60 us at 192^3 against
// 49 us for the per-cell sweep, DRAM 58 %, issue 43 %).  The sweep is
// therefore one wave of persistent CTAs, each warp looping over chunks and
// loading the next chunk's entry while the current cell's operands are in
// flight.
//
// Arithmetic against k_sor_half: the fluid cells' neighbour sum is rounded
// once instead of six times, so the iterates differ in the last bits; the
// red-black order, the neighbour values each update reads and the iteration
// count are the same.
#include <cuda_runtime.h>

#include <string.h>

#include <algorithm>
#include <vector>

#include "pf_case.cuh"
#include "pf_cells.cuh"

namespace pf {

namespace {

// 128 threads per CTA: finer occupancy steps at 44 / 52 registers a thread
// than 256 (256^3: 93.1 -> 92.1 us per launch; 64 threads: 93.7)
constexpr int LIST_THREADS = 128;

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

constexpr unsigned LIST_Q = 0x03ffffffu;   // packed index field (26 bits)
constexpr unsigned LIST_NONE = LIST_Q;     // padding entry: no cell
constexpr int LIST_S = 26, LIST_JLO = 27, LIST_JHI = 28, LIST_KLO = 29, LIST_KHI = 30, LIST_FLUID = 31;

// Neighbour offsets of the periodic edges: a cell on row n reads row jn_n
// (the opposite interior row or the ghost row), and so on.
struct ListOffsets {
  idx_t H, HY, dN, dS, dT, dB;
};
__host__ __device__ inline ListOffsets list_offsets(const Geo& g) {
  ListOffsets o;
  o.H = g.H;
  o.HY = (idx_t)g.H * g.Y;
  o.dN = (idx_t)(g.jn_n - g.n) * g.H;
  o.dS = (idx_t)(g.js_1 - 1) * g.H;
  o.dT = (idx_t)(g.kt_l - g.l) * o.HY;
  o.dB = (idx_t)(g.kb_1 - 1) * o.HY;
  return o;
}

// The cell of entry e: its index and its six neighbours' (e, w, n, s, t, b).
__device__ __forceinline__ idx_t list_cell(unsigned e, const ListOffsets& o, idx_t nb[6]) {
  const idx_t q = (idx_t)(e & LIST_Q);
  const idx_t s = (e >> LIST_S) & 1u;
  nb[0] = q + s;
  nb[1] = q - 1 + s;
  nb[2] = q + (((e >> LIST_JHI) & 1u) ? o.dN : o.H);
  nb[3] = q + (((e >> LIST_JLO) & 1u) ? o.dS : -o.H);
  nb[4] = q + (((e >> LIST_KHI) & 1u) ? o.dT : o.HY);
  nb[5] = q + (((e >> LIST_KLO) & 1u) ? o.dB : -o.HY);
  return q;
}

// sum_nb a_nb p_nb of one cell: the exact sum times the fluid constant for a
// fluid cell (ISO), the three constants, or the cell's own coefficients.
template <bool ISO>
__device__ __forceinline__ double list_stencil(bool fl, const double (&x)[6], const Coef<double>& C, idx_t q,
                                               double tt, double ax, double ay, double az) {
  if (fl) {
    if (ISO) {
      double sum;
      if (!sum6_exact(x, sum)) sum = ((((x[0] + x[1]) + x[2]) + x[3]) + x[4]) + x[5];
      return fma(-ax, sum, tt);
    }
    tt = fma(-ax, x[0], tt);
    tt = fma(-ax, x[1], tt);
    tt = fma(-ay, x[2], tt);
    tt = fma(-ay, x[3], tt);
    tt = fma(-az, x[4], tt);
    return fma(-az, x[5], tt);
  }
  double c[6];
#pragma unroll
  for (int d = 0; d < 6; d++) c[d] = C.a[d][q];
#pragma unroll
  for (int d = 0; d < 6; d++) tt = fma(-c[d], x[d], tt);
  return tt;
}

// One half-sweep over the chunked list of one colour: warp w takes chunks
// w, w + W, ... (W warps in the grid), one entry per lane, and loads the
// next chunk's entry before working on the current one.  ISO: the six fluid
// constants are equal (dx = dy = dz); otherwise the fluid cells use the
// three constants with FP64 FMAs (still without coefficient loads).
template <bool TRACK, bool ISO>
__global__ void __launch_bounds__(LIST_THREADS)
    k_sor_list3(Geo g, Coef<double> C, double* __restrict__ pc, const double* __restrict__ po, double omw,
                const unsigned* __restrict__ list, int nchunks, double ax, double ay, double az,
                unsigned long long* __restrict__ err, const int* __restrict__ skip) {
  const int lane = threadIdx.x & 31;
  const int W = gridDim.x * (LIST_THREADS / 32);
  int w = blockIdx.x * (LIST_THREADS / 32) + (threadIdx.x >> 5);
  unsigned e = w < nchunks ? list[(size_t)w * 32 + lane] : LIST_NONE;
  pdl_begin();
  if (skip && *skip) return;
  const ListOffsets o = list_offsets(g);
  unsigned long long emax = 0;
  for (; w < nchunks; w += W) {
    const unsigned en = w + W < nchunks ? list[(size_t)(w + W) * 32 + lane] : LIST_NONE;
    if (e != LIST_NONE) {
      idx_t nb[6];
      const idx_t q = list_cell(e, o, nb);
      const bool fl = (e >> LIST_FLUID) & 1u;
      const double cb = C.bbn[q];
      const double pold = pc[q];
      double x[6];
#pragma unroll
      for (int d = 0; d < 6; d++) x[d] = po[nb[d]];
      const double pnew = fma(omw, pold, list_stencil<ISO>(fl, x, C, q, cb, ax, ay, az));
      pc[q] = pnew;
      if (TRACK) {
        const unsigned long long b = abs_diff_bits(pnew, pold);
        emax = b > emax ? b : emax;
      }
    }
    e = en;
  }
  if (TRACK) warp_max_atomic(emax, err);
}

// The precision form's FP64 residual over the same lists, r = bbn - omega p -
// sum_nb a_nb p_nb (normalised by omega/ap), stored as the FP32 right-hand
// side of the correction sweeps; zeroes the cell's correction and reduces
// max |r|.
template <bool ISO>
__global__ void __launch_bounds__(LIST_THREADS)
    k_residual_list3(Geo g, Coef<double> C, const double* __restrict__ pc, const double* __restrict__ po,
                     double omega, const unsigned* __restrict__ list, int nchunks, double ax, double ay, double az,
                     float* __restrict__ rf, float* __restrict__ ec, unsigned long long* __restrict__ rmax,
                     const int* __restrict__ skip) {
  const int lane = threadIdx.x & 31;
  const int W = gridDim.x * (LIST_THREADS / 32);
  int w = blockIdx.x * (LIST_THREADS / 32) + (threadIdx.x >> 5);
  unsigned e = w < nchunks ? list[(size_t)w * 32 + lane] : LIST_NONE;
  pdl_begin();
  if (skip && *skip) return;
  const ListOffsets o = list_offsets(g);
  unsigned long long rm = 0;
  for (; w < nchunks; w += W) {
    const unsigned en = w + W < nchunks ? list[(size_t)(w + W) * 32 + lane] : LIST_NONE;
    if (e != LIST_NONE) {
      idx_t nb[6];
      const idx_t q = list_cell(e, o, nb);
      const bool fl = (e >> LIST_FLUID) & 1u;
      double x[6];
#pragma unroll
      for (int d = 0; d < 6; d++) x[d] = po[nb[d]];
      double tt = list_stencil<ISO>(fl, x, C, q, C.bbn[q], ax, ay, az);
      tt = fma(-omega, pc[q], tt);
      rf[q] = (float)tt;
      ec[q] = 0.0f;
      const unsigned long long b = abs_bits(tt);
      rm = b > rm ? b : rm;
    }
    e = en;
  }
  warp_max_atomic(rm, rmax);
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

bool sor_list_eligible(const Geo& g) { return g.dim == 3 && !g.wall && g.pk < (long long)LIST_Q; }

// Device bytes of a case's lists, fixed by the grid alone (admission
// control needs it before the porosity is known): every cell once plus the
// padding of at most four partial chunks (two lists per colour).
size_t sor_list_bytes(const Geo& g) { return ((size_t)g.m * g.n * g.l + 4 * 32) * sizeof(unsigned); }

// Builds both colours' lists: flags per work item on the device, copied to
// the host; per colour the fluid cells and the others in memory order, cut
// into chunks of 32 entries (the last chunk of each padded with LIST_NONE),
// the two chunk sequences merged by the position of their first cell; one
// device allocation for both colours.  Also sizes the persistent launch.
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
  const int W = packed_width(g);
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
    std::vector<unsigned> part[2];  // [0] fluid, [1] the others
    for (long long t = 0; t < items; t++) {
      const unsigned char f = flags[(size_t)t];
      if (!f) continue;
      const int row = (int)(t / W);
      const int h = (int)(t - (long long)row * W);
      const int k = row / g.n + 1, j = row - (k - 1) * g.n + 1;
      const int sd = (col + j + k) & 1;
      const unsigned q = (unsigned)pk_idx(g, h, j, k);
      part[f == 1 ? 0 : 1].push_back(q | ((unsigned)sd << LIST_S) | ((unsigned)(j == 1) << LIST_JLO) |
                                      ((unsigned)(j == g.n) << LIST_JHI) | ((unsigned)(k == 1) << LIST_KLO) |
                                      ((unsigned)(k == g.l) << LIST_KHI) | ((unsigned)(f == 1) << LIST_FLUID));
    }
    c->list_nfluid[col] = (int)part[0].size();
    c->list_ntotal[col] = (int)(part[0].size() + part[1].size());
    std::vector<unsigned>& L = lists[col];
    size_t at[2] = {0, 0};
    while (at[0] < part[0].size() || at[1] < part[1].size()) {
      int pick;
      if (at[0] >= part[0].size())
        pick = 1;
      else if (at[1] >= part[1].size())
        pick = 0;
      else
        pick = (part[0][at[0]] & LIST_Q) < (part[1][at[1]] & LIST_Q) ? 0 : 1;
      for (int r = 0; r < 32; r++) L.push_back(at[pick] + r < part[pick].size() ? part[pick][at[pick] + r] : LIST_NONE);
      at[pick] += 32;
    }
    c->list_nchunks[col] = (int)(L.size() / 32);
  }
  cudaFree(dflags);
  cudaFree(dconst);
  if (rc) return rc;
  const size_t n0 = lists[0].size(), n1 = lists[1].size();
  if ((n0 + n1) * sizeof(unsigned) > sor_list_bytes(g)) return fail(PF_E_INVALID, "cell lists exceed their bound");
  unsigned* d = nullptr;
  PF_CUDA(cudaMalloc(&d, sor_list_bytes(g)));
  c->list_base = d;
  c->list[0] = d;
  c->list[1] = d + n0;
  c->list_bytes = sor_list_bytes(g);
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
  // one wave of persistent CTAs per kernel (the untracked sweep holds fewer
  // registers than the tracked one, so more of its CTAs fit an SM), no more
  // than the chunks need
  int dev = 0, sms = 0;
  PF_CUDA(cudaGetDevice(&dev));
  PF_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  const long long need = ((long long)std::max(c->list_nchunks[0], c->list_nchunks[1]) + LIST_THREADS / 32 - 1) /
                         (LIST_THREADS / 32);
  const bool iso = c->list_iso;
  const void* kern[3] = {iso ? (const void*)k_sor_list3<false, true> : (const void*)k_sor_list3<false, false>,
                         iso ? (const void*)k_sor_list3<true, true> : (const void*)k_sor_list3<true, false>,
                         iso ? (const void*)k_residual_list3<true> : (const void*)k_residual_list3<false>};
  for (int v = 0; v < 3; v++) {
    int per_sm = 0;
    PF_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern[v], LIST_THREADS, 0));
    c->list_grid[v] = (int)std::max(1LL, std::min<long long>((long long)sms * std::max(1, per_sm), need));
  }
  return PF_OK;
}

void launch_sor_list(const pf_case* c, int col, double omw, unsigned long long* err, bool /*early*/,
                     cudaStream_t st) {
  const double ax = c->list_const[0], ay = c->list_const[2], az = c->list_const[4];
#define PF_SL(TR, ISO)                                                                                          \
  launch_pdl(k_sor_list3<TR, ISO>, dim3(c->list_grid[TR ? 1 : 0]), dim3(LIST_THREADS), st, c->g, c->C[col],     \
             c->p[col],                                                                                         \
             (const double*)c->p[1 - col], omw, (const unsigned*)c->list[col], c->list_nchunks[col], ax, ay, az, \
             err, (const int*)nullptr)
  if (c->list_iso)
    err ? PF_SL(true, true) : PF_SL(false, true);
  else
    err ? PF_SL(true, false) : PF_SL(false, false);
#undef PF_SL
}

void launch_residual_list(const pf_case* c, int col, float* rf, float* ec, unsigned long long* rmax, const int* skip,
                          cudaStream_t st) {
  const double ax = c->list_const[0], ay = c->list_const[2], az = c->list_const[4];
  if (c->list_iso)
    launch_pdl(k_residual_list3<true>, dim3(c->list_grid[2]), dim3(LIST_THREADS), st, c->g, c->C[col],
               (const double*)c->p[col], (const double*)c->p[1 - col], c->s.omega, (const unsigned*)c->list[col],
               c->list_nchunks[col], ax, ay, az, rf, ec, rmax, skip);
  else
    launch_pdl(k_residual_list3<false>, dim3(c->list_grid[2]), dim3(LIST_THREADS), st, c->g, c->C[col],
               (const double*)c->p[col], (const double*)c->p[1 - col], c->s.omega, (const unsigned*)c->list[col],
               c->list_nchunks[col], ax, ay, az, rf, ec, rmax, skip);
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
