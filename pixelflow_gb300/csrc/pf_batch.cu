// pf_batch.cu -- the batched form: many independent cases of uneven size
// advanced by one persistent kernel.
//
// Each case is an ordinary mixed-precision case (pf_case: FP64 state, FP32
// stencils, FP64 defect correction around FP32 red-black sweeps) whose arrays
// stay resident in HBM.  The persistent kernel is launched with thread-block
// clusters of `cluster` CTAs.  A cluster claims one case at a time from a
// device queue (largest cases first), advances it by its requested number of
// steps running every stage of the step itself -- the stages are separated by
// hardware cluster barriers -- and then claims the next case.  Cases never
// wait on each other, so the kernel has no inter-cluster synchronisation and
// no spin-wait of any kind, and any number of clusters (even one) finishes.
// While a cluster works on a case, the case's working set (a few MB for the
// largest 2D case) stays in the 129 MB L2, so the 100 sweeps of a step read
// L2 rather than HBM.
//
// The per-cell arithmetic is exactly the single-case kernels' (pf_cells.cuh),
// so a case gives the same result alone, in a batch, or in any mix.
#include <cooperative_groups.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <string>
#include <vector>

#include "pf_case.cuh"
#include "pf_cells.cuh"
#include "pf_internal.cuh"

namespace cg = cooperative_groups;

namespace pf {

// Everything the persistent kernel needs about one case.
struct CaseDesc {
  Geo g;
  Scal s;
  DCConst K;
  const double *poro, *gx, *gy, *gz;
  double *U[2], *V[2], *W[2];
  float *Uf, *Vf, *Wf, *divf;
  const float *gxf, *gyf, *gzf, *rinvf, *dampf;
  double* p[2];
  Coef<double> C[2];
  float *e[2], *rf[2];
  const float* epsf[2];
  unsigned long long* red;  // the case's reduction slots (RED_* layout)
  int cur;                  // current velocity buffer when the launch starts
  int nsteps;               // steps to advance in this launch
  int outer, inner, track;
  int smem_rows;            // 2D: rows per CTA held in shared memory (0: global-memory passes)
  int smem_pitch;           // shared-memory row pitch (floats)
};

namespace {

// Walks the items x = tid, tid + nth, ... of an (a, b, c) box (a fastest)
// with 32-bit counters and no division inside the loop.
struct Walk3 {
  int a, b, c;       // current coordinates (0-based)
  int na, nb;        // extents of the two fast dimensions
  int da, db, dc;    // step of nth items in (a, b, c) with carries
  __device__ __forceinline__ Walk3(int tid, int nth, int na_, int nb_) : na(na_), nb(nb_) {
    a = tid % na;
    int r = tid / na;
    b = r % nb;
    c = r / nb;
    da = nth % na;
    r = nth / na;
    db = r % nb;
    dc = r / nb;
  }
  __device__ __forceinline__ void next() {
    a += da;
    int cb = 0;
    if (a >= na) {
      a -= na;
      cb = 1;
    }
    b += db + cb;
    int cc = 0;
    if (b >= nb) {
      b -= nb;
      cc = 1;
    }
    c += dc + cc;
  }
};

// The defect-correction passes of a 2D case with the FP32 correction e, the
// FP32 porosity and the FP32 residual of each CTA's block of rows held in
// shared memory for all inner iterations.  CTA r of the cluster owns rows
// j0..j1 (R rows per CTA) plus a halo row on each side; after each
// half-sweep it writes its updated first and last rows straight into the
// halo rows of the CTAs that own the neighbouring rows (distributed shared
// memory, periodic in y), then one cluster barrier.  The halo rows therefore
// hold exactly what the reference's refreshed ghost rows hold (for an odd n
// the two rows that cross the periodic edge go to the other colour's array,
// as the ghost-row copy crosses colours there).  Arithmetic per
// cell is dc_update's, so results equal the global-memory passes bit for bit.
__device__ __forceinline__ void passes_smem_2d(const CaseDesc& d, cg::cluster_group& cl, int step, unsigned& emax,
                                               float* sm) {
  const Geo& g = d.g;
  const Scal& s = d.s;
  const int m = g.m, n = g.n, hc = (m + 1) / 2 + 1, P = d.smem_pitch, R = d.smem_rows;
  const int r = (int)cl.block_rank();
  const int j0 = 1 + r * R, j1 = min(n, j0 + R - 1), nr = j1 >= j0 ? j1 - j0 + 1 : 0;
  float* E[2] = {sm, sm + (R + 2) * P};
  float* EPS[2] = {sm + 2 * (R + 2) * P, sm + 3 * (R + 2) * P};
  float* RR[2] = {sm + 4 * (R + 2) * P, sm + 4 * (R + 2) * P + R * P};
  auto owner = [&](int row) { return (row - 1) / R; };
  auto rows_of = [&](int t) {
    const int a = 1 + t * R, b = min(n, a + R - 1);
    return b >= a ? b - a + 1 : 0;
  };
  const int tS = owner(j0 == 1 ? n : j0 - 1);  // receives my first row in its north halo
  const int tN = owner(j1 == n ? 1 : j1 + 1);  // receives my last row in its south halo
  const int nrS = rows_of(tS);
  const bool halo_p = n & 1;
  if (step == 0) {  // porosity rows j0-1 .. j1+1 (ghost rows included), once per claimed case
    for (int x = threadIdx.x; x < 2 * (nr + 2) * hc; x += blockDim.x) {
      const int col = x / ((nr + 2) * hc), y = x - col * (nr + 2) * hc, lr = y / hc, h = y - lr * hc;
      EPS[col][lr * P + h] = d.epsf[col][pk_idx(g, h, j0 - 1 + lr, 0)];
    }
  }
  for (int pass = 0; pass < d.outer; pass++) {
    // FP64 residual of my rows -> shared FP32 right-hand side; e = 0 incl. halos
    for (int x = threadIdx.x; x < 2 * (nr + 2) * hc; x += blockDim.x) {
      const int col = x / ((nr + 2) * hc), y = x - col * (nr + 2) * hc, lr = y / hc, h = y - lr * hc;
      E[col][lr * P + h] = 0.f;
      if (lr >= 1 && lr <= nr) {
        double t = 0.0;
        const bool ok = residual_value<2>(g, d.C[col], d.p[col], d.p[1 - col], s.omega, col, h, j0 + lr - 1, 0, t);
        RR[col][(lr - 1) * P + h] = ok ? (float)t : 0.f;
      }
    }
    cl.sync();  // no CTA pushes into a halo before its owner has zeroed it
    for (int it = 0; it < d.inner; it++) {
      for (int col = 0; col < 2; col++) {
        // (slot, row) walk without a division per cell
        for (Walk3 w(threadIdx.x, blockDim.x, hc, nr > 0 ? nr : 1); w.c == 0 && nr > 0; w.next()) {
          const int h = w.a, lr = 1 + w.b, j = j0 + w.b;
          const int sb = (col + j + 1) & 1, i = 2 * h + sb;
          if (i < 1 || i > m) continue;
          const float eold = E[col][lr * P + h];
          const float enew = dc_update_rows_2d(d.K, EPS[col] + lr * P, EPS[1 - col] + lr * P, E[1 - col] + lr * P, P,
                                               h, sb, i == 1, i == m, RR[col][(lr - 1) * P + h], eold);
          E[col][lr * P + h] = enew;
          emax = max(emax, abs_bits(enew - eold));
        }
        __syncthreads();
        if (nr > 0) {
          // Across the periodic edge of an odd n the neighbour is a ghost row,
          // which holds the opposite edge row of the other colour: row n
          // colour c is ghost row 0 colour 1-c (the reference's refresh before
          // every half-sweep), so those two pushes land in the other array.
          const int cS = (halo_p && j0 == 1) ? 1 - col : col;
          const int cN = (halo_p && j1 == n) ? 1 - col : col;
          float* dS = cl.map_shared_rank(E[cS], tS) + (nrS + 1) * P;
          float* dN = cl.map_shared_rank(E[cN], tN);
          for (int h = threadIdx.x; h < hc; h += blockDim.x) {
            dS[h] = E[col][P + h];
            dN[h] = E[col][nr * P + h];
          }
        }
        cl.sync();
      }
    }
    // p += e (FP64) for my rows
    for (int x = threadIdx.x; x < 2 * nr * hc; x += blockDim.x) {
      const int col = x / (nr * hc), y = x - col * nr * hc, lr = 1 + y / hc, h = y - (lr - 1) * hc;
      const int j = j0 + lr - 1, i = 2 * h + ((col + j + 1) & 1);
      if (i >= 1 && i <= m) d.p[col][pk_idx(g, h, j, 0)] += (double)E[col][lr * P + h];
    }
    cl.sync();
    if (halo_p) {
      for (int i = (int)cl.block_rank() * blockDim.x + threadIdx.x + 1; i <= m; i += cl.num_blocks() * blockDim.x)
        c_p_halo_y(g, d.p[0], d.p[1], i, 0);
      cl.sync();
    }
  }
}

template <int DIM, int BT>
__device__ __forceinline__ void run_case(const CaseDesc& d, cg::cluster_group& cl, int tid, int nth) {
  const Geo& g = d.g;
  const Scal& s = d.s;
  const int m = g.m, n = g.n, l = DIM == 3 ? g.l : 1;
  const int hc = (m + 1) / 2 + 1;
  const bool halo = (n & 1) || (DIM == 3 && (l & 1));
  int cur = d.cur;
  for (int step = 0; step < d.nsteps; step++) {
    const int o = cur, nw = 1 - cur;
    unsigned emax = 0;
    if (d.track && tid < RED_SLOTS) d.red[RED_ERRF + tid] = 0ULL;
    // divergence of the FP32 copy of u_old
    for (Walk3 w(tid, nth, m, n); w.c < l; w.next()) {
      const int i = 1 + w.a, j = 1 + w.b, k = DIM == 3 ? 1 + w.c : 0;
      c_divergence<float>(g, s, d.Uf, d.Vf, d.Wf, d.divf, i, j, k);
    }
    cl.sync();
    // predictor: FP32 increment on the FP64 state
    for (Walk3 w(tid, nth, m, n); w.c < l; w.next()) {
      const int i = 1 + w.a, j = 1 + w.b, k = DIM == 3 ? 1 + w.c : 0;
      c_predictor<float, double, DIM>(g, s, d.Uf, d.Vf, d.Wf, d.divf, d.gxf, d.gyf, d.gzf, d.rinvf, d.dampf,
                                      d.U[o], d.V[o], d.W[o], d.U[nw], d.V[nw], d.W[nw], i, j, k);
    }
    cl.sync();
    // FP64 right-hand side
    for (Walk3 w(tid, nth, m, n); w.c < l; w.next()) {
      const int i = 1 + w.a, j = 1 + w.b, k = DIM == 3 ? 1 + w.c : 0;
      c_rhs<double, DIM>(g, s, d.U[nw], d.V[nw], d.W[nw], d.poro, d.gx, d.gy, d.gz, d.C[0], d.C[1], i, j, k);
    }
    cl.sync();
    if (DIM == 2 && d.smem_rows > 0) {
      extern __shared__ float dyn_smem[];
      passes_smem_2d(d, cl, step, emax, dyn_smem);
    } else
    for (int pass = 0; pass < d.outer; pass++) {
      // FP64 residual of both colours -> FP32 right-hand side, e = 0
      for (Walk3 w(tid, nth, hc, n); w.c < 2 * l; w.next()) {
        const int col = w.c >= l;
        const int h = w.a, j = 1 + w.b, k = DIM == 3 ? 1 + w.c - col * l : 0;
        c_residual<DIM>(g, d.C[col], d.p[col], d.p[1 - col], s.omega, col, d.rf[col], d.e[col], h, j, k);
      }
      cl.sync();
      for (int it = 0; it < d.inner; it++) {
        for (int col = 0; col < 2; col++) {
          if (halo) {
            for (int x = tid; x < m * (n + l); x += nth) {
              const int i = 1 + x % m, a = 1 + x / m;
              if (a <= (DIM == 3 ? l : 1)) c_p_halo_y(g, d.e[0], d.e[1], i, DIM == 3 ? a : 0);
              else if (DIM == 3 && a - l <= n) c_p_halo_z(g, d.e[0], d.e[1], i, a - l);
            }
            cl.sync();
          }
          // four independent updates per thread per round, all loads first
          // (the sweep is L2-latency bound)
          Walk3 wk[4] = {Walk3(tid, 4 * nth, hc, n), Walk3(tid + nth, 4 * nth, hc, n),
                         Walk3(tid + 2 * nth, 4 * nth, hc, n), Walk3(tid + 3 * nth, 4 * nth, hc, n)};
          for (; wk[0].c < l;) {
            float eold[4], enew[4];
            bool ok[4];
            int qq[4];
#pragma unroll
            for (int u = 0; u < 4; u++) {
              const int h = wk[u].a, j = 1 + wk[u].b, k = DIM == 3 ? 1 + wk[u].c : 0;
              const int sb = (col + j + (DIM == 3 ? k : 1)) & 1;
              const int i = 2 * h + sb;
              ok[u] = wk[u].c < l && i >= 1 && i <= m;
              qq[u] = pk_idx(g, h, j, k);
              if (ok[u]) dc_update<DIM>(g, d.K, d.epsf[col], d.epsf[1 - col], d.rf[col], d.e[col], d.e[1 - col], h, j, k,
                                        sb, i, eold[u], enew[u]);
            }
#pragma unroll
            for (int u = 0; u < 4; u++) {
              if (ok[u]) {
                d.e[col][qq[u]] = enew[u];
                if (DIM == 2 || col == 1) emax = max(emax, abs_bits(enew[u] - eold[u]));
              }
              wk[u].next();
            }
          }
          cl.sync();
        }
      }
      // p += e (FP64)
      for (Walk3 w(tid, nth, hc, n); w.c < 2 * l; w.next()) {
        const int col = w.c >= l;
        const int h = w.a, j = 1 + w.b, k = DIM == 3 ? 1 + w.c - col * l : 0;
        c_accumulate<DIM>(g, d.p[col], d.e[col], col, h, j, k);
      }
      cl.sync();
      if (halo) {
        for (int x = tid; x < m * (n + l); x += nth) {
          const int i = 1 + x % m, a = 1 + x / m;
          if (a <= (DIM == 3 ? l : 1)) c_p_halo_y(g, d.p[0], d.p[1], i, DIM == 3 ? a : 0);
          else if (DIM == 3 && a - l <= n) c_p_halo_z(g, d.p[0], d.p[1], i, a - l);
        }
        cl.sync();
      }
    }
    // ghost rows of p for the projection (interior i)
    for (int x = tid; x < m * (n + l); x += nth) {
      const int i = 1 + x % m, a = 1 + x / m;
      if (a <= (DIM == 3 ? l : 1)) c_p_halo_y(g, d.p[0], d.p[1], i, DIM == 3 ? a : 0);
      else if (DIM == 3 && a - l <= n) c_p_halo_z(g, d.p[0], d.p[1], i, a - l);
    }
    cl.sync();
    for (Walk3 w(tid, nth, m, n); w.c < l; w.next()) {
      const int i = 1 + w.a, j = 1 + w.b, k = DIM == 3 ? 1 + w.c : 0;
      c_projection<double, DIM>(g, s, d.p[0], d.p[1], d.U[nw], d.V[nw], d.W[nw], i, j, k);
    }
    cl.sync();
    // boundary: x faces, then y faces, then z faces (the reference's order)
    for (int x = tid; x < n * l; x += nth) {
      const int j = 1 + x % n, k = DIM == 3 ? 1 + x / n : 0;
      c_bnd_x<double>(g, s, d.U[nw], d.V[nw], d.W[nw], d.p[0], d.p[1], j, k);
    }
    cl.sync();
    for (int x = tid; x < (m + 2) * (DIM == 3 ? l + 2 : 1); x += nth) {
      const int i = x % (m + 2), k = x / (m + 2);
      c_bnd_y<double>(g, d.U[nw], d.V[nw], d.W[nw], d.p[0], d.p[1], i, k);
    }
    cl.sync();
    if (DIM == 3) {
      for (int x = tid; x < (m + 2) * (n + 2); x += nth) {
        const int i = x % (m + 2), j = x / (m + 2);
        c_bnd_z<double>(g, d.U[nw], d.V[nw], d.W[nw], d.p[0], d.p[1], i, j);
      }
      cl.sync();
    }
    // FP32 copy of the new state for the next step's stencils
    for (int x = tid; x < (int)g.nat; x += nth) {
      d.Uf[x] = (float)d.U[nw][x];
      d.Vf[x] = (float)d.V[nw][x];
      if (DIM == 3) d.Wf[x] = (float)d.W[nw][x];
    }
    if (d.track) {
      emax = __reduce_max_sync(0xffffffffu, emax);
      if ((threadIdx.x & 31) == 0 && emax)
        atomicMax(reinterpret_cast<unsigned*>(&d.red[RED_ERRF + ((tid >> 5) & (RED_SLOTS - 1))]), emax);
    }
    cl.sync();
    cur = nw;
  }
}

template <int DIM, int BT>
__global__ void __launch_bounds__(BT) k_batch(const CaseDesc* __restrict__ descs, const int* __restrict__ order,
                                              const int* __restrict__ ncases, int* __restrict__ head) {
  cg::cluster_group cl = cg::this_cluster();
  __shared__ int claim;
  __shared__ CaseDesc d;
  const int tid = (int)cl.block_rank() * BT + threadIdx.x;
  const int nth = (int)cl.num_blocks() * BT;
  const int total = *ncases;
  while (true) {
    if (cl.block_rank() == 0 && threadIdx.x == 0) claim = atomicAdd(head, 1);
    cl.sync();
    const int c = *cl.map_shared_rank(&claim, 0);  // every CTA sees rank 0's claim
    if (threadIdx.x == 0 && c < total) d = descs[order[c]];
    // all reads of rank 0's `claim` are done before anyone leaves or rank 0
    // overwrites it, and d is loaded in every CTA
    cl.sync();
    if (c >= total) break;
    if (d.g.dim == DIM && d.nsteps > 0) run_case<DIM, BT>(d, cl, tid, nth);
    cl.sync();
  }
}

}  // namespace
}  // namespace pf

using namespace pf;

// ---------------------------------------------------------------------------
struct pf_batch {
  pf_batch_options opt{};
  cudaStream_t st = nullptr;
  std::vector<pf_case*> slots;     // nullptr = free
  std::vector<int> pending;        // steps requested per slot for the next launch
  CaseDesc* d_desc = nullptr;
  int* d_order = nullptr;
  int* d_misc = nullptr;           // [0] ncases 2D, [1] head 2D, [2] ncases 3D, [3] head 3D
  int capacity = 0;
  size_t bytes_in_use = 0;
  int64_t launches = 0;
  cudaEvent_t ev[2] = {nullptr, nullptr};
  double last_ms = 0.0;  // device time of the last pf_batch_step_slots
  std::vector<cudaEvent_t> case_ev;  // per slot: completion of a large case's steps
  // The persistent part of a call (descriptor upload + one launch per
  // dimension) as a CUDA graph: the descriptors are staged in pinned host
  // memory, which the graph's copy nodes read when it runs, so a graph fits
  // every call with the same composition (key).  The graphs of the last
  // kGraphCache compositions are kept (least recently used replaced), so
  // calls that alternate between a few compositions replay them.
  CaseDesc* h_desc = nullptr;
  int* h_order = nullptr;
  int* h_misc = nullptr;
  struct Graph {
    long long key[6];  // n2, n3, smem2, cluster, threads, grid clusters
    cudaGraphExec_t exec;
    int64_t used;
  };
  std::vector<Graph> graphs;
  int64_t graphs_captured = 0, graph_replays = 0;
};
static const size_t kGraphCache = 16;

// Launch shape of one dimension's persistent kernel: the function attributes
// (shared memory, non-portable cluster size) and the number of co-resident
// clusters.  Not a stream operation, so it runs before any capture.
template <int DIM, int BT>
static int prepare_batch_kernel(int cluster, size_t smem, int ncl, int* nclusters) {
  cudaError_t e = cudaFuncSetAttribute(k_batch<DIM, BT>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return cuda_fail(e, "cudaFuncSetAttribute(smem)");
  if (cluster > 8) {
    e = cudaFuncSetAttribute(k_batch<DIM, BT>, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
    if (e != cudaSuccess) return cuda_fail(e, "cudaFuncSetAttribute(cluster size)");
  }
  cudaLaunchConfig_t cfg = {};
  cfg.blockDim = dim3(BT);
  cfg.dynamicSmemBytes = smem;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = cluster;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  cfg.gridDim = dim3(cluster);
  int maxc = 0;
  e = cudaOccupancyMaxActiveClusters(&maxc, (void*)k_batch<DIM, BT>, &cfg);
  if (e != cudaSuccess) return cuda_fail(e, "cudaOccupancyMaxActiveClusters");
  if (maxc < 1) return fail(PF_E_INVALID, "batch: cluster configuration cannot be scheduled");
  *nclusters = std::max(1, std::min(maxc, ncl));
  return PF_OK;
}

template <int DIM, int BT>
static int launch_batch_kernel(pf_batch* b, int nclusters, int cluster, size_t smem, const int* order,
                               const int* ncases, int* head) {
  cudaLaunchConfig_t cfg = {};
  cfg.blockDim = dim3(BT);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = b->st;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = cluster;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  cfg.gridDim = dim3(nclusters * cluster);
  cudaError_t e = cudaLaunchKernelEx(&cfg, k_batch<DIM, BT>, (const CaseDesc*)b->d_desc, order, ncases, head);
  if (e != cudaSuccess) return cuda_fail(e, "cudaLaunchKernelEx(k_batch)");
  return PF_OK;
}

template <int DIM>
static int prepare_dim(pf_batch* b, size_t smem, int ncl, int* nclusters) {
  const int c = b->opt.cluster;
  if (b->opt.threads == 256) return prepare_batch_kernel<DIM, 256>(c, smem, ncl, nclusters);
  if (b->opt.threads == 512) return prepare_batch_kernel<DIM, 512>(c, smem, ncl, nclusters);
  return prepare_batch_kernel<DIM, 1024>(c, smem, ncl, nclusters);
}

template <int DIM>
static int launch_dim(pf_batch* b, int nclusters, size_t smem, const int* order, const int* ncases, int* head) {
  const int c = b->opt.cluster;
  if (b->opt.threads == 256) return launch_batch_kernel<DIM, 256>(b, nclusters, c, smem, order, ncases, head);
  if (b->opt.threads == 512) return launch_batch_kernel<DIM, 512>(b, nclusters, c, smem, order, ncases, head);
  return launch_batch_kernel<DIM, 1024>(b, nclusters, c, smem, order, ncases, head);
}

// The persistent part of a call, enqueued on the batch stream: the
// descriptor upload from the pinned staging and one launch per dimension.
static int enqueue_persistent(pf_batch* b, int n2, int n3, size_t smem2, int ncl2, int ncl3) {
  const int n = n2 + n3;
  PF_CUDA(cudaMemcpyAsync(b->d_desc, b->h_desc, sizeof(CaseDesc) * n, cudaMemcpyHostToDevice, b->st));
  PF_CUDA(cudaMemcpyAsync(b->d_order, b->h_order, sizeof(int) * n, cudaMemcpyHostToDevice, b->st));
  PF_CUDA(cudaMemcpyAsync(b->d_misc, b->h_misc, sizeof(int) * 8, cudaMemcpyHostToDevice, b->st));
  int rc = PF_OK;
  if (n2) rc = launch_dim<2>(b, ncl2, smem2, b->d_order, b->d_misc + 0, b->d_misc + 1);
  if (rc == PF_OK && n3) rc = launch_dim<3>(b, ncl3, 0, b->d_order + n2, b->d_misc + 2, b->d_misc + 3);
  return rc;
}

// Dynamic shared memory a CTA may take for the on-chip passes (the 227 KB
// per-CTA limit minus the kernel's static shared memory).
static const size_t kSmemCap = 227 * 1024 - 1024;

extern "C" {

void pf_batch_default_options(pf_batch_options* o) {
  if (!o) return;
  std::memset(o, 0, sizeof(*o));
  o->cluster = 4;
  o->threads = 512;
  o->max_cases = 1024;
  o->hbm_budget_bytes = (uint64_t)150 << 30;
  o->use_graph = 1;
}

int pf_batch_create(const pf_batch_options* opt, pf_batch** out) {
  if (!out) return fail(PF_E_INVALID, "pf_batch_create: null argument");
  *out = nullptr;
  pf_batch* b = new pf_batch();
  if (opt)
    b->opt = *opt;
  else
    pf_batch_default_options(&b->opt);
  if (!(b->opt.cluster == 1 || b->opt.cluster == 2 || b->opt.cluster == 4 || b->opt.cluster == 8 ||
        b->opt.cluster == 16) ||
      !(b->opt.threads == 256 || b->opt.threads == 512 || b->opt.threads == 1024) || b->opt.max_cases < 1) {
    delete b;
    return fail(PF_E_INVALID, "pf_batch_create: cluster must be 1,2,4,8,16; threads 256,512,1024; max_cases >= 1");
  }
  b->capacity = b->opt.max_cases;
  cudaError_t e = cudaStreamCreateWithFlags(&b->st, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaMalloc(&b->d_desc, sizeof(CaseDesc) * b->capacity);
  if (e == cudaSuccess) e = cudaMalloc(&b->d_order, sizeof(int) * 2 * b->capacity);
  if (e == cudaSuccess) e = cudaMalloc(&b->d_misc, sizeof(int) * 8);
  if (e == cudaSuccess) e = cudaEventCreate(&b->ev[0]);
  if (e == cudaSuccess) e = cudaEventCreate(&b->ev[1]);
  if (e == cudaSuccess) e = cudaHostAlloc(&b->h_desc, sizeof(CaseDesc) * b->capacity, cudaHostAllocDefault);
  if (e == cudaSuccess) e = cudaHostAlloc(&b->h_order, sizeof(int) * 2 * b->capacity, cudaHostAllocDefault);
  if (e == cudaSuccess) e = cudaHostAlloc(&b->h_misc, sizeof(int) * 8, cudaHostAllocDefault);
  if (e != cudaSuccess) {
    if (b->d_desc) cudaFree(b->d_desc);
    if (b->d_order) cudaFree(b->d_order);
    if (b->d_misc) cudaFree(b->d_misc);
    if (b->h_desc) cudaFreeHost(b->h_desc);
    if (b->h_order) cudaFreeHost(b->h_order);
    if (b->st) cudaStreamDestroy(b->st);
    delete b;
    return cuda_fail(e, "pf_batch_create");
  }
  b->slots.assign(b->capacity, nullptr);
  b->pending.assign(b->capacity, 0);
  b->case_ev.assign(b->capacity, nullptr);
  // 2D cases beyond ~100k cells no longer keep their rows in the shared
  // memory of a cluster and sweep from global memory (~50 M cell-steps/s on
  // a few SMs); as full-GPU step graphs beside the persistent kernel they run
  // faster and the batch with them (512 2D cases of 64..512 per side, 20
  // steps on GB300: 1326 Mcell-steps/s with 300k, 1792 with 130k, 1906 with
  // 100k, 1900 with 65k)
  if (b->opt.large_cells <= 0) b->opt.large_cells = 100000;
  *out = b;
  return PF_OK;
}

int pf_batch_destroy(pf_batch* b) {
  if (!b) return fail(PF_E_INVALID, "null batch");
  cudaStreamSynchronize(b->st);
  for (auto* c : b->slots)
    if (c) pf_destroy(c);
  for (auto e : b->case_ev)
    if (e) cudaEventDestroy(e);
  for (auto& gr : b->graphs) cudaGraphExecDestroy(gr.exec);
  cudaFree(b->d_desc);
  cudaFree(b->d_order);
  cudaFree(b->d_misc);
  cudaFreeHost(b->h_desc);
  cudaFreeHost(b->h_order);
  cudaFreeHost(b->h_misc);
  cudaEventDestroy(b->ev[0]);
  cudaEventDestroy(b->ev[1]);
  cudaStreamDestroy(b->st);
  delete b;
  return PF_OK;
}

static int device_sms() {
  int dev = 0, sms = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
    return 0;
  return sms;
}

// Bytes a case of these sizes takes on the device (admission control); the
// same array list as case_alloc / mixed_alloc.
int pf_case_bytes(const pf_params* prm, const pf_options* opt, size_t* bytes) {
  if (!prm || !bytes) return fail(PF_E_INVALID, "null argument");
  Geo g;
  int rc = make_geo(*prm, g);
  if (rc) return rc;
  const bool mixed = opt && opt->precision == PF_PREC_MIXED;
  auto r256 = [](size_t x) { return (x + 255) / 256 * 256; };
  const size_t nat8 = r256((size_t)g.nat * 8), pk8 = r256((size_t)g.pk * 8);
  const size_t nat4 = r256((size_t)g.nat * 4), pk4 = r256((size_t)g.pk * 4);
  const int d = g.dim;
  size_t b = nat8 * (6 + (d == 3) + 2 * d) + pk8 * (2 + 2 * (2 * d + 3));
  b += r256((size_t)(g.m + 2) * (g.n + 2) * g.Z * 8) + RED_TOTAL * sizeof(unsigned long long);
  if (mixed) b += nat4 * (d + 1 + 2 + (d == 3) + 2) + pk4 * (mixed_fused(g, *opt) ? 8 : 6) + 256;
  // the cell lists of the 3D sweep and residual: one 32-bit entry per cell
  if (sor_list_eligible(g) && (!opt || opt->sor_path == PF_SOR_AUTO)) b += sor_list_bytes(g);
  // the chunk lists of the split FP32 sweep (grids of more than one wave)
  if (mixed && opt->sor_path == PF_SOR_AUTO && dc_list_eligible(g) && !dc_one_wave(g, device_sms()))
    b += dc_list_bytes(g);
  *bytes = b;
  return PF_OK;
}

}  // extern "C"

template <typename Create>
static int batch_add_impl(pf_batch* b, const pf_params* prm, const pf_options* opt, int* slot, Create create) {
  if (!b || !prm || !slot) return fail(PF_E_INVALID, "pf_batch_add: null argument");
  int free_slot = -1;
  for (int i = 0; i < b->capacity; i++)
    if (!b->slots[i]) {
      free_slot = i;
      break;
    }
  if (free_slot < 0) return fail(PF_E_BUSY, "pf_batch_add: no free slot");
  pf_options o;
  if (opt)
    o = *opt;
  else
    pf_default_options(&o);
  o.precision = PF_PREC_MIXED;  // the batched form runs the precision form
  // cases too large for one cluster run full-GPU steps (graph replays) on
  // their own stream, concurrently with the persistent kernel
  const long long cells = (long long)prm->m * prm->n * (prm->dim == 3 ? prm->l : 1);
  o.use_graph = cells > b->opt.large_cells ? 1 : 0;
  // a case the persistent kernel steps never runs the single-case FP32 sweep:
  // no second correction array, no sweep-form timing at creation
  if (!o.use_graph) o.sweep_form = PF_SWEEP_SPLIT;
  size_t need = 0;
  int rc = pf_case_bytes(prm, &o, &need);
  if (rc) return rc;
  if (b->bytes_in_use + need > b->opt.hbm_budget_bytes)
    return fail(PF_E_NOMEM, "pf_batch_add: the case does not fit the HBM budget now");
  pf_case* c = nullptr;
  rc = create(&o, &c);
  if (rc) return rc;
  rc = pf_initial_conditions(c);
  if (rc == PF_OK) rc = pf_synchronize(c);
  if (rc) {
    pf_destroy(c);
    return rc;
  }
  b->slots[free_slot] = c;
  b->pending[free_slot] = 0;
  b->bytes_in_use += c->bytes + c->mixed_bytes + c->list_bytes;
  *slot = free_slot;
  return PF_OK;
}

extern "C" {

int pf_batch_add(pf_batch* b, const pf_params* prm, const pf_options* opt, const double* porosity_values,
                 int* slot) {
  if (!porosity_values) return fail(PF_E_INVALID, "pf_batch_add: null porosity");
  return batch_add_impl(b, prm, opt, slot,
                        [&](const pf_options* o, pf_case** c) { return pf_create(prm, o, porosity_values, c); });
}

int pf_batch_add_shapes(pf_batch* b, const pf_params* prm, const pf_options* opt, const pf_shape* shapes,
                        int nshapes, double edge, int* slot) {
  return batch_add_impl(b, prm, opt, slot, [&](const pf_options* o, pf_case** c) {
    return pf_create_shapes(prm, o, shapes, nshapes, edge, c);
  });
}

int pf_batch_remove(pf_batch* b, int slot) {
  if (!b || slot < 0 || slot >= b->capacity || !b->slots[slot]) return fail(PF_E_INVALID, "pf_batch_remove: bad slot");
  PF_CUDA(cudaStreamSynchronize(b->st));
  pf_case* c = b->slots[slot];
  b->bytes_in_use -= c->bytes + c->mixed_bytes + c->list_bytes;
  pf_destroy(c);
  b->slots[slot] = nullptr;
  b->pending[slot] = 0;
  return PF_OK;
}

pf_case* pf_batch_case(pf_batch* b, int slot) {
  if (!b || slot < 0 || slot >= b->capacity) return nullptr;
  return b->slots[slot];
}

// Advance the listed slots by their step counts in one persistent launch per
// dimension (2D and 3D cases run in separate launches on the batch stream).
// Cases with more than large_cells cells instead replay their single-case
// step graphs on their own streams, overlapping the persistent kernels: one
// cluster of a few SMs would take far longer over such a case than the whole
// GPU does, and the persistent kernels leave the SMs their clusters do not
// hold to those graphs.  Both paths run the same per-cell arithmetic.
int pf_batch_step_slots(pf_batch* b, const int* slots, const int* nsteps, int n) {
  if (!b || (n > 0 && (!slots || !nsteps))) return fail(PF_E_INVALID, "pf_batch_step_slots: null argument");
  std::vector<CaseDesc> desc;
  std::vector<std::pair<long long, int>> order2, order3;
  std::vector<std::pair<int, int>> large;  // (slot, steps) run on their own streams
  size_t smem2 = 0;  // dynamic shared memory of the 2D launch
  desc.reserve(n);
  for (int q = 0; q < n; q++) {
    const int sl = slots[q];
    if (sl < 0 || sl >= b->capacity || !b->slots[sl]) return fail(PF_E_INVALID, "pf_batch_step_slots: bad slot");
    if (nsteps[q] < 0) return fail(PF_E_INVALID, "pf_batch_step_slots: negative step count");
    if (nsteps[q] == 0) continue;
    pf_case* c = b->slots[sl];
    if ((long long)c->g.m * c->g.n * c->g.l > b->opt.large_cells) {
      large.push_back({sl, nsteps[q]});
      continue;
    }
    CaseDesc d;
    std::memset(&d, 0, sizeof(d));
    d.g = c->g;
    d.s = c->s;
    d.K = make_dc_const(c->s.dt, c->s.dx, c->s.dy, c->s.dz, c->g.dim, c->s.omega);
    d.poro = c->poro;
    d.gx = c->gx;
    d.gy = c->gy;
    d.gz = c->gz;
    for (int k = 0; k < 2; k++) {
      d.U[k] = c->U[k];
      d.V[k] = c->V[k];
      d.W[k] = c->W[k];
      d.p[k] = c->p[k];
      d.C[k] = c->C[k];
      d.e[k] = c->e[k];
      d.rf[k] = c->rf[k];
      d.epsf[k] = c->epsf[k];
    }
    d.Uf = c->Uf[0];
    d.Vf = c->Vf[0];
    d.Wf = c->Wf[0];
    d.divf = c->divf;
    d.gxf = c->gxf;
    d.gyf = c->gyf;
    d.gzf = c->gzf;
    d.rinvf = c->rinvf;
    d.dampf = c->dampf;
    d.red = c->red;
    d.cur = c->cur;
    d.nsteps = nsteps[q];
    d.outer = c->opt.outer_max;
    d.inner = c->opt.inner_sweeps;
    d.track = c->opt.track_sor_error;
    d.smem_rows = 0;
    d.smem_pitch = 0;
    if (c->g.dim == 2 && !b->opt.global_passes) {
      const int R = (c->g.n + b->opt.cluster - 1) / b->opt.cluster;
      const int P = (c->g.m + 1) / 2 + 1;
      const size_t need = (size_t)(6 * R + 8) * P * sizeof(float);
      if (need <= kSmemCap) {
        d.smem_rows = R;
        d.smem_pitch = P;
        smem2 = std::max(smem2, need);
      }
    }
    const long long work = (long long)c->g.m * c->g.n * c->g.l * nsteps[q];
    (c->g.dim == 3 ? order3 : order2).push_back({work, (int)desc.size()});
    desc.push_back(d);
    c->cur ^= (nsteps[q] & 1);
  }
  if (desc.empty() && large.empty()) return PF_OK;
  PF_CUDA(cudaEventRecord(b->ev[0], b->st));
  for (auto& lc : large) {
    pf_case* c = b->slots[lc.first];
    if (!b->case_ev[lc.first]) PF_CUDA(cudaEventCreateWithFlags(&b->case_ev[lc.first], cudaEventDisableTiming));
    PF_CUDA(cudaStreamWaitEvent(c->st, b->ev[0], 0));
    const int64_t l0 = c->launches;
    int rc = pf_step(c, lc.second);
    if (rc) return rc;
    b->launches += c->launches - l0;
    PF_CUDA(cudaEventRecord(b->case_ev[lc.first], c->st));
  }
  // longest work first, 2D list then 3D list
  auto by_work = [](const std::pair<long long, int>& a, const std::pair<long long, int>& c) { return a.first > c.first; };
  std::sort(order2.begin(), order2.end(), by_work);
  std::sort(order3.begin(), order3.end(), by_work);
  std::vector<int> order;
  for (auto& p : order2) order.push_back(p.second);
  for (auto& p : order3) order.push_back(p.second);
  if ((int)desc.size() > b->capacity) return fail(PF_E_INVALID, "too many cases");
  const int n2 = (int)order2.size(), n3 = (int)order3.size();
  int rc = PF_OK;
  if (!desc.empty()) {
    // the previous call ended with a stream synchronisation, so no copy of
    // an earlier call still reads the pinned staging
    std::memcpy(b->h_desc, desc.data(), sizeof(CaseDesc) * desc.size());
    std::memcpy(b->h_order, order.data(), sizeof(int) * order.size());
    const int misc[8] = {n2, 0, n3, 0, 0, 0, 0, 0};
    std::memcpy(b->h_misc, misc, sizeof(misc));
    int ncl2 = 0, ncl3 = 0;
    if (n2) rc = prepare_dim<2>(b, smem2, n2, &ncl2);
    if (rc == PF_OK && n3) rc = prepare_dim<3>(b, 0, n3, &ncl3);
    if (rc) return rc;
    if (!b->opt.use_graph) {
      rc = enqueue_persistent(b, n2, n3, smem2, ncl2, ncl3);
      if (rc) return rc;
    } else {
      const long long key[6] = {n2, n3, (long long)smem2, b->opt.cluster, b->opt.threads,
                                (long long)ncl2 * 65536 + ncl3};
      pf_batch::Graph* hit = nullptr;
      for (auto& gr : b->graphs)
        if (std::memcmp(key, gr.key, sizeof(key)) == 0) hit = &gr;
      if (!hit) {
        PF_CUDA(cudaStreamBeginCapture(b->st, cudaStreamCaptureModeThreadLocal));
        rc = enqueue_persistent(b, n2, n3, smem2, ncl2, ncl3);
        cudaGraph_t graph = nullptr;
        const cudaError_t ec = cudaStreamEndCapture(b->st, &graph);
        if (rc) {
          if (graph) cudaGraphDestroy(graph);
          return rc;
        }
        if (ec != cudaSuccess) return cuda_fail(ec, "cudaStreamEndCapture(batch)");
        cudaGraphExec_t exec = nullptr;
        const cudaError_t ei = cudaGraphInstantiate(&exec, graph, 0);
        cudaGraphDestroy(graph);
        if (ei != cudaSuccess) return cuda_fail(ei, "cudaGraphInstantiate(batch)");
        if (b->graphs.size() >= kGraphCache) {  // replace the least recently used
          auto lru = std::min_element(b->graphs.begin(), b->graphs.end(),
                                      [](const pf_batch::Graph& x, const pf_batch::Graph& y) { return x.used < y.used; });
          cudaGraphExecDestroy(lru->exec);
          b->graphs.erase(lru);
        }
        pf_batch::Graph gr;
        std::memcpy(gr.key, key, sizeof(key));
        gr.exec = exec;
        gr.used = 0;
        b->graphs.push_back(gr);
        hit = &b->graphs.back();
        b->graphs_captured++;
      } else {
        b->graph_replays++;
      }
      hit->used = b->graphs_captured + b->graph_replays;
      PF_CUDA(cudaGraphLaunch(hit->exec, b->st));
    }
    b->launches += (n2 ? 1 : 0) + (n3 ? 1 : 0);
  }
  for (auto& lc : large) PF_CUDA(cudaStreamWaitEvent(b->st, b->case_ev[lc.first], 0));
  PF_CUDA(cudaEventRecord(b->ev[1], b->st));
  // the host arrays above must outlive the async copies
  PF_CUDA(cudaStreamSynchronize(b->st));
  float ms = 0.f;
  PF_CUDA(cudaEventElapsedTime(&ms, b->ev[0], b->ev[1]));
  b->last_ms = ms;
  return PF_OK;
}

int pf_batch_step(pf_batch* b, int nsteps) {
  if (!b) return fail(PF_E_INVALID, "null batch");
  std::vector<int> sl, ns;
  for (int i = 0; i < b->capacity; i++)
    if (b->slots[i]) {
      sl.push_back(i);
      ns.push_back(nsteps);
    }
  return pf_batch_step_slots(b, sl.data(), ns.data(), (int)sl.size());
}

int pf_batch_synchronize(pf_batch* b) {
  if (!b) return fail(PF_E_INVALID, "null batch");
  PF_CUDA(cudaStreamSynchronize(b->st));
  return PF_OK;
}

int pf_batch_get_state(pf_batch* b, int slot, double* u, double* v, double* w, double* p, int ld1, int ld2) {
  if (!b || slot < 0 || slot >= b->capacity || !b->slots[slot]) return fail(PF_E_INVALID, "bad slot");
  PF_CUDA(cudaStreamSynchronize(b->st));
  PF_CUDA(cudaStreamSynchronize(b->slots[slot]->st));
  return pf_get_state(b->slots[slot], u, v, w, p, ld1, ld2);
}

int pf_batch_norms(pf_batch* b, int slot, double* max_div, double* sor_error) {
  if (!b || slot < 0 || slot >= b->capacity || !b->slots[slot]) return fail(PF_E_INVALID, "bad slot");
  PF_CUDA(cudaStreamSynchronize(b->st));
  PF_CUDA(cudaStreamSynchronize(b->slots[slot]->st));
  return pf_norms(b->slots[slot], max_div, sor_error);
}

int pf_batch_memory(pf_batch* b, size_t* in_use, size_t* budget) {
  if (!b) return fail(PF_E_INVALID, "null batch");
  if (in_use) *in_use = b->bytes_in_use;
  if (budget) *budget = b->opt.hbm_budget_bytes;
  return PF_OK;
}

int pf_batch_last_ms(pf_batch* b, double* ms) {
  if (!b || !ms) return fail(PF_E_INVALID, "null argument");
  *ms = b->last_ms;
  return PF_OK;
}

int pf_batch_configure(pf_batch* b, int cluster, int threads) {
  if (!b) return fail(PF_E_INVALID, "null batch");
  if (!(cluster == 1 || cluster == 2 || cluster == 4 || cluster == 8 || cluster == 16) ||
      !(threads == 256 || threads == 512 || threads == 1024))
    return fail(PF_E_INVALID, "pf_batch_configure: cluster must be 1,2,4,8,16 and threads 256,512,1024");
  b->opt.cluster = cluster;
  b->opt.threads = threads;
  return PF_OK;
}

int pf_batch_graph_stats(pf_batch* b, int64_t* captured, int64_t* replays) {
  if (!b) return fail(PF_E_INVALID, "null batch");
  if (captured) *captured = b->graphs_captured;
  if (replays) *replays = b->graph_replays;
  return PF_OK;
}

int pf_batch_kernel_launches(pf_batch* b, int64_t* n) {
  if (!b || !n) return fail(PF_E_INVALID, "null argument");
  *n = b->launches;
  return PF_OK;
}

}  // extern "C"
