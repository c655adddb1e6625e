// pf_dc_list.cu -- the precision form's FP32 correction sweep of 3D cases,
// driven by per-colour lists of chunks with the all-fluid chunks apart.
//
// k_sor_dc4 gives each thread one chunk of four packed cells and rebuilds
// the chunk's operator from FP32 porosity: 15 vector loads per chunk, 6 of
// them porosity.  Away from the obstacles every porosity operand of a chunk
// is exactly 1.0f, so its faces are the constants of a fluid cell.  Testing
// that per thread does not pay: nearly every x row passes within the FP32
// porosity transition of some obstacle, so the warps mix both kinds of chunk
// and run both paths; a per-chunk flag read ahead of the porosity loads adds
// a dependent load to a latency-bound kernel.  So, as the plain sweep's cell
// lists do for the FP64 cells (pf_sor_list.cu), the chunks of a colour are
// classified once at set-up, split into an all-fluid list and a list of the
// others, each cut into groups of 32 (one warp) in memory order, and the
// groups of both lists merged by position.  A warp's group is then all of
// one kind; the fluid groups load only the corrections and the residual.
// The sweep is one wave of persistent CTAs whose warps walk the groups and
// load the next group's entry while the current chunk's operands are in
// flight.
//
// An entry is the chunk's packed index / 4 (24 bits), its colour side s,
// whether its row is the first or last (periodic neighbours), whether its
// plane is the first or last, whether it is the first or last chunk of its
// row (the only chunks with lanes outside 1 <= i <= m or on the inlet or
// outlet column), and the fluid bit.  Every chunk runs dc_chunk, the per-cell
// arithmetic of k_sor_dc4 and of the fused sweep, on the same values (a
// fluid chunk passes 1.0f for its porosity), so the three forms agree bit
// for bit.
#include <cuda_runtime.h>

#include <algorithm>
#include <vector>

#include "pf_case.cuh"
#include "pf_cells.cuh"

namespace pf {

namespace {

// 128 threads per CTA: the tracked sweep holds 96 registers a thread, so
// 5 CTAs of 4 warps fit an SM where 2 of 8 warps did (256^3: 41.7 -> 40.3 us
// per launch; a register cap of 80 spills and gains nothing)
constexpr int DCL_THREADS = 128;
constexpr int DCL_V = 4;
constexpr unsigned DCL_Q = 0x00ffffffu;  // chunk index: packed index / 4
constexpr unsigned DCL_NONE = DCL_Q;     // padding entry: no chunk
constexpr int DCL_S = 24, DCL_JLO = 25, DCL_JHI = 26, DCL_KLO = 27, DCL_KHI = 28, DCL_FIRST = 29, DCL_LAST = 30,
              DCL_FLUID = 31;

__host__ __device__ inline int dcl_chunks_per_row(const Geo& g) { return (g.m >> 1) / DCL_V + 1; }

// The porosity operands of a chunk, loaded as k_sor_dc4 loads them.
__device__ __forceinline__ void dcl_poro(const Geo& g, const float* __restrict__ epsc,
                                         const float* __restrict__ epso, idx_t q, int s, VecF<DCL_V>& PC,
                                         VecF<DCL_V>& PO, float& px, VecF<DCL_V>& PN, VecF<DCL_V>& PS,
                                         VecF<DCL_V>& PT, VecF<DCL_V>& PB) {
  const idx_t H = g.H, HY = (idx_t)g.H * g.Y;
  PC = ldv<DCL_V>(epsc + q);
  PO = ldv<DCL_V>(epso + q);
  px = s ? epso[q + DCL_V] : epso[q - 1];
  PN = ldv<DCL_V>(epso + q + H);
  PS = ldv<DCL_V>(epso + q - H);
  PT = ldv<DCL_V>(epso + q + HY);
  PB = ldv<DCL_V>(epso + q - HY);
}

// Per chunk t of one colour (k_sor_dc4's mapping: row-major over (row,
// chunk)): 0 no lane inside 1 <= i <= m, 1 every porosity operand 1.0f,
// 2 any other chunk.
__global__ void k_dc_chunk_class(Geo g, const float* __restrict__ epsc, const float* __restrict__ epso, int colour,
                                 unsigned char* __restrict__ out) {
  const int chunks = dcl_chunks_per_row(g);
  const long long t = (long long)blockIdx.x * DCL_THREADS + threadIdx.x;
  if (t >= (long long)chunks * g.n * g.l) return;
  const int row = (int)(t / chunks);
  const int h0 = (int)(t - (long long)row * chunks) * DCL_V;
  const int k = row / g.n + 1, j = row - (k - 1) * g.n + 1;
  const int s = (colour + j + k) & 1;
  const int ilo = 2 * h0 + s, ihi = 2 * (h0 + DCL_V - 1) + s;
  if (ihi < 1 || ilo > g.m) {
    out[t] = 0;
    return;
  }
  VecF<DCL_V> PC, PO, PN, PS, PT, PB;
  float px;
  dcl_poro(g, epsc, epso, pk_idx(g, h0, j, k), s, PC, PO, px, PN, PS, PT, PB);
  bool fl = px == 1.f;
#pragma unroll
  for (int u = 0; u < DCL_V; u++)
    fl = fl && PC.a[u] == 1.f && PO.a[u] == 1.f && PN.a[u] == 1.f && PS.a[u] == 1.f && PT.a[u] == 1.f &&
         PB.a[u] == 1.f;
  out[t] = fl ? 1 : 2;
}

// Neighbour offsets of the periodic edges (as the plain sweep's lists).
struct DclOffsets {
  idx_t H, HY, dN, dS, dT, dB;
};
__host__ __device__ inline DclOffsets dcl_offsets(const Geo& g) {
  DclOffsets o;
  o.H = g.H;
  o.HY = (idx_t)g.H * g.Y;
  o.dN = (idx_t)(g.jn_n - g.n) * g.H;
  o.dS = (idx_t)(g.js_1 - 1) * g.H;
  o.dT = (idx_t)(g.kt_l - g.l) * o.HY;
  o.dB = (idx_t)(g.kb_1 - 1) * o.HY;
  return o;
}

// One colour's sweep over its merged groups: warp w takes groups w, w + W,
// ... (W warps in the grid), one chunk per lane.  A middle chunk of a row
// has every lane inside the row and none on the inlet or outlet column, the
// same as a chunk at h0 = 4 (such chunks exist only when m >= 16), so h0
// is known from the first/last bits alone.
template <bool TRACK>
__global__ void __launch_bounds__(DCL_THREADS)
    k_sor_dc_list3(Geo g, DCConst K, const float* __restrict__ epsc, const float* __restrict__ epso,
                   const float* __restrict__ r, float* __restrict__ ec, const float* __restrict__ eo,
                   const unsigned* __restrict__ list, int ngroups, unsigned long long* __restrict__ err,
                   const int* __restrict__ skip) {
  const int lane = threadIdx.x & 31;
  const int W = gridDim.x * (DCL_THREADS / 32);
  int w = blockIdx.x * (DCL_THREADS / 32) + (threadIdx.x >> 5);
  unsigned en = w < ngroups ? list[(size_t)w * 32 + lane] : DCL_NONE;
  pdl_begin();
  if (skip && *skip) return;
  const DclOffsets o = dcl_offsets(g);
  const int last_h0 = (dcl_chunks_per_row(g) - 1) * DCL_V;
  unsigned em = 0;
  for (; w < ngroups; w += W) {
    const unsigned e = en;
    en = w + W < ngroups ? list[(size_t)(w + W) * 32 + lane] : DCL_NONE;
    if (e == DCL_NONE) continue;
    const idx_t q = (idx_t)(e & DCL_Q) * DCL_V;
    const int s = (e >> DCL_S) & 1u;
    const idx_t qn = q + (((e >> DCL_JHI) & 1u) ? o.dN : o.H);
    const idx_t qs = q + (((e >> DCL_JLO) & 1u) ? o.dS : -o.H);
    const idx_t qt = q + (((e >> DCL_KHI) & 1u) ? o.dT : o.HY);
    const idx_t qb = q + (((e >> DCL_KLO) & 1u) ? o.dB : -o.HY);
    const VecF<DCL_V> EC = ldv<DCL_V>(ec + q), R = ldv<DCL_V>(r + q), XO = ldv<DCL_V>(eo + q);
    const float xx = s ? eo[q + DCL_V] : eo[q - 1];
    const VecF<DCL_V> XN = ldv<DCL_V>(eo + qn), XS = ldv<DCL_V>(eo + qs);
    const VecF<DCL_V> XT = ldv<DCL_V>(eo + qt), XB = ldv<DCL_V>(eo + qb);
    const int h0 = ((e >> DCL_FIRST) & 1u) ? 0 : (((e >> DCL_LAST) & 1u) ? last_h0 : DCL_V);
    VecF<DCL_V> out;
    if ((e >> DCL_FLUID) & 1u) {  // uniform across the warp
      VecF<DCL_V> one;
#pragma unroll
      for (int u = 0; u < DCL_V; u++) one.a[u] = 1.f;
      out = dc_chunk<3, TRACK, DCL_V>(g, K, h0, s, EC, R, one, XO, one, xx, 1.f, XN, XS, one, one, XT, XB, one, one,
                                      em);
    } else {
      VecF<DCL_V> PC, PO, PN, PS, PT, PB;
      float px;
      dcl_poro(g, epsc, epso, q, s, PC, PO, px, PN, PS, PT, PB);
      out = dc_chunk<3, TRACK, DCL_V>(g, K, h0, s, EC, R, PC, XO, PO, xx, px, XN, XS, PN, PS, XT, XB, PT, PB, em);
    }
    *reinterpret_cast<VecF<DCL_V>*>(ec + q) = out;
  }
  if (TRACK) warp_max_atomic(em, err);
}

}  // namespace

bool dc_list_eligible(const Geo& g) {
  // chunk index in 24 bits, below the padding entry's DCL_Q: packed index
  // below 2^26 - 4
  return g.dim == 3 && !g.wall && g.pk < (1LL << 26) - 4;
}

// Device bytes of a case's chunk lists, fixed by the grid: every chunk of
// both colours once plus the padding of at most four partial groups.
size_t dc_list_bytes(const Geo& g) {
  return ((size_t)2 * dcl_chunks_per_row(g) * g.n * g.l + 4 * 32) * sizeof(unsigned);
}

// Classifies both colours' chunks on the device (the packed FP32 porosity
// must be in place), builds the merged lists on the host, uploads them in
// one allocation and sizes the persistent launches.
int dc_list_setup(pf_case* c) {
  const Geo& g = c->g;
  const int chunks = dcl_chunks_per_row(g);
  const long long items = (long long)chunks * g.n * g.l;
  unsigned char* dcls = nullptr;
  PF_CUDA(cudaMalloc(&dcls, (size_t)items));
  std::vector<unsigned char> cls((size_t)items);
  std::vector<unsigned> lists[2];
  const unsigned grid = (unsigned)((items + DCL_THREADS - 1) / DCL_THREADS);
  int rc = PF_OK;
  for (int col = 0; col < 2 && rc == PF_OK; col++) {
    k_dc_chunk_class<<<grid, DCL_THREADS, 0, c->st>>>(g, c->epsf[col], c->epsf[1 - col], col, dcls);
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaMemcpyAsync(cls.data(), dcls, (size_t)items, cudaMemcpyDeviceToHost, c->st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->st);
    if (e != cudaSuccess) {
      rc = cuda_fail(e, "chunk classes");
      break;
    }
    std::vector<unsigned> part[2];  // [0] all-fluid chunks, [1] the others
    for (long long t = 0; t < items; t++) {
      const unsigned char f = cls[(size_t)t];
      if (!f) continue;
      const int row = (int)(t / chunks);
      const int ch = (int)(t - (long long)row * chunks);
      const int k = row / g.n + 1, j = row - (k - 1) * g.n + 1;
      const int s = (col + j + k) & 1;
      const unsigned q4 = (unsigned)(pk_idx(g, ch * DCL_V, j, k) / DCL_V);
      part[f == 1 ? 0 : 1].push_back(q4 | ((unsigned)s << DCL_S) | ((unsigned)(j == 1) << DCL_JLO) |
                                      ((unsigned)(j == g.n) << DCL_JHI) | ((unsigned)(k == 1) << DCL_KLO) |
                                      ((unsigned)(k == g.l) << DCL_KHI) | ((unsigned)(ch == 0) << DCL_FIRST) |
                                      ((unsigned)(ch == chunks - 1) << DCL_LAST) | ((unsigned)(f == 1) << DCL_FLUID));
    }
    c->dcl_fluid[col] = (int)part[0].size();
    c->dcl_total[col] = (int)(part[0].size() + part[1].size());
    std::vector<unsigned>& L = lists[col];
    size_t at[2] = {0, 0};
    while (at[0] < part[0].size() || at[1] < part[1].size()) {
      int pick;
      if (at[0] >= part[0].size())
        pick = 1;
      else if (at[1] >= part[1].size())
        pick = 0;
      else
        pick = (part[0][at[0]] & DCL_Q) < (part[1][at[1]] & DCL_Q) ? 0 : 1;
      for (int x = 0; x < 32; x++) L.push_back(at[pick] + x < part[pick].size() ? part[pick][at[pick] + x] : DCL_NONE);
      at[pick] += 32;
    }
    c->dcl_ngroups[col] = (int)(L.size() / 32);
  }
  cudaFree(dcls);
  if (rc) return rc;
  const size_t n0 = lists[0].size(), n1 = lists[1].size();
  if ((n0 + n1) * sizeof(unsigned) > dc_list_bytes(g)) return fail(PF_E_INVALID, "chunk lists exceed their bound");
  unsigned* d = nullptr;
  PF_CUDA(cudaMalloc(&d, dc_list_bytes(g)));
  c->dcl_base = d;
  c->dcl[0] = d;
  c->dcl[1] = d + n0;
  c->list_bytes += dc_list_bytes(g);
  PF_CUDA(cudaMemcpyAsync(c->dcl[0], lists[0].data(), n0 * sizeof(unsigned), cudaMemcpyHostToDevice, c->st));
  PF_CUDA(cudaMemcpyAsync(c->dcl[1], lists[1].data(), n1 * sizeof(unsigned), cudaMemcpyHostToDevice, c->st));
  PF_CUDA(cudaStreamSynchronize(c->st));
  // one wave of persistent CTAs per variant, no more than the groups need
  int dev = 0, sms = 0;
  PF_CUDA(cudaGetDevice(&dev));
  PF_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  const long long need =
      ((long long)std::max(c->dcl_ngroups[0], c->dcl_ngroups[1]) + DCL_THREADS / 32 - 1) / (DCL_THREADS / 32);
  const void* kern[2] = {(const void*)k_sor_dc_list3<false>, (const void*)k_sor_dc_list3<true>};
  for (int v = 0; v < 2; v++) {
    int per_sm = 0;
    PF_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern[v], DCL_THREADS, 0));
    c->dcl_grid[v] = (int)std::max(1LL, std::min<long long>((long long)sms * std::max(1, per_sm), need));
  }
  return PF_OK;
}

void launch_sor_dc_list(const pf_case* c, int col, unsigned long long* err, const int* skip, cudaStream_t st) {
  const DCConst K = make_dc_const(c->s.dt, c->s.dx, c->s.dy, c->s.dz, 3, c->s.omega);
  if (err)
    launch_pdl(k_sor_dc_list3<true>, dim3(c->dcl_grid[1]), dim3(DCL_THREADS), st, c->g, K,
               (const float*)c->epsf[col], (const float*)c->epsf[1 - col], (const float*)c->rf[col], c->e[col],
               (const float*)c->e[1 - col], (const unsigned*)c->dcl[col], c->dcl_ngroups[col], err, skip);
  else
    launch_pdl(k_sor_dc_list3<false>, dim3(c->dcl_grid[0]), dim3(DCL_THREADS), st, c->g, K,
               (const float*)c->epsf[col], (const float*)c->epsf[1 - col], (const float*)c->rf[col], c->e[col],
               (const float*)c->e[1 - col], (const unsigned*)c->dcl[col], c->dcl_ngroups[col],
               (unsigned long long*)nullptr, skip);
}

}  // namespace pf
