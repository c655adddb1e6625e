// pf_kernels.cu -- sm_103a kernels of the plain immersed-boundary step.
//
// Stage map (reference routine -> kernel):
//   divergence of u_old  (ibm_2d:172-194, ibm_3d:185-222)  -> k_divergence
//   predictor u*,v*,w*   (ibm_2d:200-258, ibm_3d:228-381)  -> k_predictor
//   coefficients + bb    (ibm_2d:262-279, ibm_3d:386-414)
//     + boundrary_matrix (ibm_2d:410-454, ibm_3d:618-663)  -> k_setup_coef (once per case)
//                                                             + k_rhs (per step)
//   red-black SOR        (ibm_2d:293-406, ibm_3d:433-614)  -> k_sor_half (+ k_p_halo for odd n/l)
//   projection           (ibm_2d:103-115, ibm_3d:109-125)  -> k_projection
//   boundary             (ibm_2d:460-538, ibm_3d:669-752)  -> k_bnd_x, k_bnd_y, k_bnd_z
//   max|div u|           (output.f90:217-224, :929-941)   -> k_div_diag
//
// Arithmetic: the algebra of each reference expression is kept, but the
// operations are reordered for the GPU: divisions by dx, ap and porosity
// become multiplications by factors computed once per case, and products
// fuse into FMAs.  Results therefore differ from the reference in the last
// bits of each operation; the parity tests bound the drift over whole runs.
// The red-black colour order, the ghost semantics of every half-sweep and
// the SOR iteration count are the reference's exactly.
#include <cuda_runtime.h>

#include "pf_internal.cuh"
#include "pf_cells.cuh"

namespace pf {

namespace {

// Launch with programmatic stream serialization (the kernel starts with
// pdl_begin): the launch of the next kernel of the SOR loop overlaps the
// tail of the current one; CUDA graph capture keeps these as programmatic
// edges.
template <typename... KArgs, typename... Args>
void launch_pdl(void (*kernel)(KArgs...), dim3 grid, dim3 block, cudaStream_t st, Args... args) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = grid;
  cfg.blockDim = block;
  cfg.dynamicSmemBytes = 0;
  cfg.stream = st;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  cudaLaunchKernelEx(&cfg, kernel, args...);
}

inline dim3 grid_interior(const Geo& g) {
  return dim3((g.m + BX - 1) / BX, (g.n + BY - 1) / BY, g.dim == 3 ? g.l : 1);
}
inline dim3 grid_all(const Geo& g) {
  return dim3((g.m + 2 + BX - 1) / BX, (g.n + 2 + BY - 1) / BY, g.Z);
}

// ---------------------------------------------------------------------
// Time-invariant predictor factors from the porosity (once per case).
//   gx = (eps(i+1)-eps(i-1))/(2dx)  (same for y, z)
//   rinv = dt/eps                    (the "/porosity(i,j)" of the porosity terms)
//   damp = nu*dt*alpha*eps*(1-eps)^2/thickness^2  (nonslip; /dx^2 etc. applied per component)
__global__ void k_porosity_factors(Geo g, Scal s, const double* __restrict__ po, double* gx, double* gy,
                                   double* gz, double* rinv, double* damp) {
  const int i = blockIdx.x * BX + threadIdx.x + 1;
  const int j = blockIdx.y * BY + threadIdx.y + 1;
  const int k = (g.dim == 3) ? blockIdx.z + 1 : 0;
  if (i > g.m || j > g.n) return;
  const idx_t q = nat_idx(g, i, j, k);
  const idx_t X = g.X, XY = (idx_t)g.X * g.Y;
  const double e = po[q];
  gx[q] = (po[q + 1] - po[q - 1]) * s.hx;
  gy[q] = (po[q + X] - po[q - X]) * s.hy;
  if (g.dim == 3) gz[q] = (po[q + XY] - po[q - XY]) * s.hz;
  rinv[q] = s.dt / e;
  damp[q] = s.nonslip ? s.xnue * s.dt * 32.0 * e * (1.0 - e) * (1.0 - e) / (s.thickness * s.thickness) : 0.0;
}

// The reference's ae..ab (ibm_3d:386-400) of a cell from its own and its six
// neighbours' porosity (2D: the first four).
__device__ __forceinline__ void coef_set(const Geo& g, const Scal& s, double e, double pe, double pw, double pn,
                                         double ps, double pt, double pb, double a[6], double& ap) {
  const double small = 1.e-6, dt = s.dt;
  a[0] = dt * fmax(small, (pe + e) * 0.5) / s.dx / s.dx;
  a[1] = dt * fmax(small, (e + pw) * 0.5) / s.dx / s.dx;
  a[2] = dt * fmax(small, (pn + e) * 0.5) / s.dy / s.dy;
  a[3] = dt * fmax(small, (e + ps) * 0.5) / s.dy / s.dy;
  ap = -a[0] - a[1] - a[2] - a[3];
  if (g.dim == 3) {
    a[4] = dt * fmax(small, (pt + e) * 0.5) / s.dz / s.dz;
    a[5] = dt * fmax(small, (e + pb) * 0.5) / s.dz / s.dz;
    ap = ap - a[4] - a[5];
  } else {
    a[4] = a[5] = 0.0;
  }
}

// boundary_matrix of the air-condition program (ibm_3d_air_condition_omp_cpu.f90:
// 665-867) for one cell, faces in the reference's order (top, bottom, east,
// west, north, south; a = e, w, n, s, t, b): a wall or an inlet folds the
// outward coefficient into the inward one; an outlet cell (porosity >= 0.9)
// adds a_out * outlet_pressure (the ghost's value there) to bb and zeroes all
// six.  ap keeps the sum of the unedited coefficients.
__device__ __forceinline__ void wall_edits(const Geo& g, const Scal& s, int i, int j, int k, double e, double a[6],
                                           double& oadd) {
  const int face_on[6] = {k == g.l, k == 1, i == g.m, i == 1, j == g.n, j == 1};
  const int out_d[6] = {4, 5, 0, 1, 2, 3}, in_d[6] = {5, 4, 1, 0, 3, 2};
#pragma unroll
  for (int f = 0; f < 6; f++) {
    if (!face_on[f]) continue;
    const int t = s.walls[f];
    if (t == 2 && e >= 0.9) {
      oadd = oadd + a[out_d[f]] * s.outlet_pressure;
      for (int d = 0; d < 6; d++) a[d] = 0.0;
    } else {
      a[in_d[f]] = a[in_d[f]] + a[out_d[f]];
      a[out_d[f]] = 0.0;
    }
  }
}

// SOR operator of both colours, with boundrary_matrix applied, normalised
// by omega/ap.  Face coefficients follow the reference formula
// dt*max(small,(eps_a+eps_b)*0.5)/h/h with small = 1e-6.
__global__ void k_setup_coef(Geo g, Scal s, const double* __restrict__ po, Coef<double> c0, Coef<double> c1) {
  const int i = blockIdx.x * BX + threadIdx.x + 1;
  const int j = blockIdx.y * BY + threadIdx.y + 1;
  const int k = (g.dim == 3) ? blockIdx.z + 1 : 0;
  if (i > g.m || j > g.n) return;
  const idx_t q = nat_idx(g, i, j, k);
  const idx_t X = g.X, XY = (idx_t)g.X * g.Y;
  const double e = po[q];
  double a[6], ap;
  coef_set(g, s, e, po[q + 1], po[q - 1], po[q + X], po[q - X], g.dim == 3 ? po[q + XY] : 0.0,
           g.dim == 3 ? po[q - XY] : 0.0, a, ap);
  double oadd = 0.0;
  if (g.wall) {
    wall_edits(g, s, i, j, k, e, a, oadd);
  } else {
    // boundrary_matrix: inlet row i=1 (Neumann), outlet row i=m (Dirichlet p(m+1)).
    if (i == 1) {
      a[0] = a[0] + a[1];
      a[1] = 0.0;
    }
    if (i == g.m) {
      oadd = a[0] * s.outlet_pressure;
      for (int d = 0; d < 6; d++) a[d] = 0.0;
    }
  }
  const double wap = s.omega / ap;
  const int c = colour_of(g, i, j, k);
  const Coef<double> C = c ? c1 : c0;
  const idx_t r = pk_idx(g, i >> 1, j, k);
  for (int d = 0; d < 2 * g.dim; d++) C.a[d][r] = a[d] * wap;
  C.wap[r] = wap;
  C.oadd[r] = oadd;
  C.bbn[r] = 0.0;
}

// Divergence of u_old (interior).  The 2D v-term divides by dx, as the
// reference does (ibm_2d_uniform_omp_cpu.f90:176).  Ghost columns stay 0;
// the periodic ghost rows are read by wrapping in the predictor.
template <typename T>
__global__ void k_divergence(Geo g, Scal s, const T* __restrict__ uo, const T* __restrict__ vo,
                             const T* __restrict__ wo, T* __restrict__ div) {
  pdl_begin();
  const int i = blockIdx.x * BX + threadIdx.x + 1;
  const int j = blockIdx.y * BY + threadIdx.y + 1;
  const int k = (g.dim == 3) ? blockIdx.z + 1 : 0;
  if (i > g.m || j > g.n) return;
  c_divergence<T>(g, s, uo, vo, wo, div, i, j, k);
}

// Predictor: explicit Euler of the porosity-weighted momentum equation.
// Also copies the face ghosts of the old fields into the new ones, so the
// RHS sees the previous step's ghosts exactly as the reference does.
// T: type of the stencil arithmetic and of the arrays it reads; TS: type of
// the velocity state.  The predictor computes the increment u* - u_old in T
// and adds it to the TS state, so with T = float, TS = double the stencils run
// in FP32 while the state keeps FP64 precision.
template <typename T, typename TS, int DIM>
__global__ void __launch_bounds__(BX* BY) k_predictor(Geo g, Scal s, const T* __restrict__ uo,
                                                      const T* __restrict__ vo, const T* __restrict__ wo,
                                                      const T* __restrict__ div, const T* __restrict__ gxa,
                                                      const T* __restrict__ gya, const T* __restrict__ gza,
                                                      const T* __restrict__ rinva, const T* __restrict__ dampa,
                                                      const TS* __restrict__ su, const TS* __restrict__ sv,
                                                      const TS* __restrict__ sw, TS* __restrict__ u,
                                                      TS* __restrict__ v, TS* __restrict__ w) {
  pdl_begin();
  const int i = blockIdx.x * BX + threadIdx.x + 1;
  const int j = blockIdx.y * BY + threadIdx.y + 1;
  const int k = (DIM == 3) ? blockIdx.z + 1 : 0;
  if (i > g.m || j > g.n) return;
  c_predictor<T, TS, DIM>(g, s, uo, vo, wo, div, gxa, gya, gza, rinva, dampa, su, sv, sw, u, v, w, i, j, k);
}

// RHS: bb = density * porosity-weighted divergence of u*, written per colour
// and normalised, bbn = (bb + outlet addend) * omega/ap.
//   ((eps_e u_c + eps_c u_e)/2 - (eps_w u_c + eps_c u_w)/2)/dx
//     = gx*u_c + eps_c*(u_e - u_w)/(2dx)
template <typename T, int DIM>
__global__ void k_rhs(Geo g, Scal s, const T* __restrict__ u, const T* __restrict__ v, const T* __restrict__ w,
                      const double* __restrict__ po, const double* __restrict__ gxa,
                      const double* __restrict__ gya, const double* __restrict__ gza, Coef<double> c0,
                      Coef<double> c1) {
  pdl_begin();
  const int i = blockIdx.x * BX + threadIdx.x + 1;
  const int j = blockIdx.y * BY + threadIdx.y + 1;
  const int k = (DIM == 3) ? blockIdx.z + 1 : 0;
  if (i > g.m || j > g.n) return;
  c_rhs<T, DIM>(g, s, u, v, w, po, gxa, gya, gza, c0, c1, i, j, k);
}

// One red-black half-sweep of colour `colour`, in place:
//   p = (1-omega) p + bbn - sum_nb a_nb p_nb     (all neighbours: other colour)
// which is the reference's
//   p = (bb - sum a_nb p_old_nb)/ap*omega + p_old*(1-omega)
// because no neighbour of a cell changes during its own colour's sweep.
// With TRACK the block max of |p_new - p_old| goes to *err.
constexpr int SWEEP_THREADS = 256;

template <typename T, int DIM, bool TRACK>
__global__ void __launch_bounds__(SWEEP_THREADS) k_sor_half(Geo g, Coef<T> C, T* __restrict__ pc,
                                                            const T* __restrict__ po, T omw, int colour,
                                                            unsigned long long* __restrict__ err,
                                                            const int* __restrict__ skip) {
  pdl_begin();
  if (skip && *skip) return;  // uniform over the grid: defect correction converged
  const int t = blockIdx.x * SWEEP_THREADS + threadIdx.x;
  decltype(abs_bits(T(0))) e = 0;
  if (t < packed_items(g)) {
    int h, j, k;
    packed_item<DIM>(g, t, h, j, k);
    e = c_sor_half<T, DIM, TRACK>(g, C, pc, po, omw, colour, h, j, k);
  }
  if (TRACK) warp_max_atomic(e, err);
}

// Periodic ghost rows (and planes) of p for interior i, as the reference
// refreshes them before each half-sweep (ibm_2d:322-327; ibm_3d:463-480).
template <typename T>
__global__ void k_p_halo(Geo g, T* p0, T* p1, const int* __restrict__ skip) {
  pdl_begin();
  if (skip && *skip) return;
  const int i = blockIdx.x * blockDim.x + threadIdx.x + 1;
  const int a = blockIdx.y + 1;  // k for the y rows (3D), j for the z planes
  if (i > g.m) return;
  if (g.dim == 2) {
    if (a == 1) c_p_halo_y(g, p0, p1, i, 0);
  } else if (blockIdx.z == 0) {
    if (a <= g.l) c_p_halo_y(g, p0, p1, i, a);
  } else {
    if (a <= g.n) c_p_halo_z(g, p0, p1, i, a);
  }
}

// Projection u -= dt/rho * (p(i+1)-p(i-1))/(2dx), likewise v and w.
template <typename T, int DIM>
__global__ void k_projection(Geo g, Scal s, const double* __restrict__ p0, const double* __restrict__ p1, T* u,
                             T* v, T* w) {
  pdl_begin();
  const int i = blockIdx.x * BX + threadIdx.x + 1;
  const int j = blockIdx.y * BY + threadIdx.y + 1;
  const int k = (DIM == 3) ? blockIdx.z + 1 : 0;
  if (i > g.m || j > g.n) return;
  c_projection<T, DIM>(g, s, p0, p1, u, v, w, i, j, k);
}

// boundary, x faces: inflow at i=1 and its ghost, outflow copy at m+1.
template <typename T>
__global__ void k_bnd_x(Geo g, Scal s, T* u, T* v, T* w, double* p0, double* p1) {
  pdl_begin();
  const int j = blockIdx.x * blockDim.x + threadIdx.x + 1;
  const int k = (g.dim == 3) ? blockIdx.y + 1 : 0;
  if (j <= g.n) c_bnd_x(g, s, u, v, w, p0, p1, j, k);
}

// boundary, y faces: periodic ghost rows over i = 0..m+1 (and k = 0..l+1).
template <typename T>
__global__ void k_bnd_y(Geo g, T* u, T* v, T* w, double* p0, double* p1) {
  pdl_begin();
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i <= g.m + 1) c_bnd_y(g, u, v, w, p0, p1, i, blockIdx.y);  // k = 0 in 2D, 0..l+1 in 3D
}

// boundary, z faces (3D): periodic ghost planes over i = 0..m+1, j = 0..n+1.
template <typename T>
__global__ void k_bnd_z(Geo g, T* u, T* v, T* w, double* p0, double* p1) {
  pdl_begin();
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i <= g.m + 1) c_bnd_z(g, u, v, w, p0, p1, i, blockIdx.y);
}

// boundary of the air-condition program, one face per launch (the faces run
// in the reference's order: top, bottom, west, east, north, south).
template <int FACE, typename T>
__global__ void k_wall_face(Geo g, Scal s, T* u, T* v, T* w, double* p0, double* p1) {
  pdl_begin();
  const int a = blockIdx.x * blockDim.x + threadIdx.x;
  const int b = blockIdx.y;
  const int na = (FACE == 2 || FACE == 3) ? g.n + 2 : g.m + 2;
  if (a < na) c_wall_face<FACE, T>(g, s, u, v, w, p0, p1, a, b);
}

template <typename T>
__global__ void k_initial(Geo g, Scal s, T* u, T* v, T* w, double* p0, double* p1) {
  const int i = blockIdx.x * BX + threadIdx.x + 1;
  const int j = blockIdx.y * BY + threadIdx.y + 1;
  const int k = (g.dim == 3) ? blockIdx.z + 1 : 0;
  if (i > g.m || j > g.n) return;
  c_initial<T>(g, s, u, v, w, p0, p1, i, j, k);
}

// max |porosity-weighted divergence| of the current fields.
template <typename T>
__global__ void k_div_diag(Geo g, Scal s, const T* __restrict__ u, const T* __restrict__ v,
                           const T* __restrict__ w, const double* __restrict__ po,
                           const double* __restrict__ gxa, const double* __restrict__ gya,
                           const double* __restrict__ gza, unsigned long long* out) {
  const int i = blockIdx.x * BX + threadIdx.x + 1;
  const int j = blockIdx.y * BY + threadIdx.y + 1;
  const int k = (g.dim == 3) ? blockIdx.z + 1 : 0;
  unsigned long long e = 0;
  if (i <= g.m && j <= g.n) {
    const idx_t q = nat_idx(g, i, j, k);
    const idx_t X = g.X, XY = (idx_t)g.X * g.Y;
    double sd = ((double)u[q + 1] - (double)u[q - 1]) * s.hx;
    sd = fma((double)v[q + X] - (double)v[q - X], s.hy, sd);
    double sg = gxa[q] * (double)u[q];
    sg = fma(gya[q], (double)v[q], sg);
    if (g.dim == 3) {
      sd = fma((double)w[q + XY] - (double)w[q - XY], s.hz, sd);
      sg = fma(gza[q], (double)w[q], sg);
    }
    e = abs_bits(fma(po[q], sd, sg));
  }
  block_max_atomic(e, out);
}

// Force sums of the reference's force log (output.f90:244-305 2D,
// :1090-1165 3D): per cell the pressure part
//   -vol p 2 eps (1-eps) / (thickness h_d) n_d,  n = grad eps / max(|grad eps|, 1e-6)
// (central differences x 0.5) and the wall-friction part
//   vol alpha rho nu (eps (1-eps) / (thickness h_d))^2 u_d,  alpha = 32.
// Fluid cells (eps (1-eps) == 0) skip the normal (a square root and
// divisions in FP64) but still multiply their zero factors by p and u, so a
// non-finite field still makes the sums non-finite, as in the reference.
// Each block writes its six sums to part[6*block]; k_forces_sum adds the
// blocks in a fixed order, so the result does not depend on scheduling.
constexpr int FORCE_THREADS = 256;

__device__ __forceinline__ double block_sum_fixed(double v, double* sh) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  __syncthreads();
  if (lane == 0) sh[warp] = v;
  __syncthreads();
  double r = 0.0;
  if (threadIdx.x == 0)
    for (int w = 0; w < (int)(blockDim.x >> 5); w++) r += sh[w];
  return r;  // valid in thread 0
}

template <int DIM>
__global__ void __launch_bounds__(FORCE_THREADS) k_forces(Geo g, Scal s, const double* __restrict__ po,
                                                          const double* __restrict__ p0,
                                                          const double* __restrict__ p1,
                                                          const double* __restrict__ u,
                                                          const double* __restrict__ v,
                                                          const double* __restrict__ w, double* __restrict__ part) {
  __shared__ double sh[FORCE_THREADS / 32];
  const long long t = (long long)blockIdx.x * FORCE_THREADS + threadIdx.x;
  const long long cells = (long long)g.m * g.n * (DIM == 3 ? g.l : 1);
  double f[6] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
  if (t < cells) {
    const int i = (int)(t % g.m) + 1;
    const long long r = t / g.m;
    const int j = (int)(r % g.n) + 1;
    const int k = DIM == 3 ? (int)(r / g.n) + 1 : 0;
    const idx_t q = nat_idx(g, i, j, k);
    const idx_t X = g.X, XY = (idx_t)g.X * g.Y;
    const double e = po[q], ee = e * (1.0 - e);
    double fp[3] = {0.0, 0.0, 0.0}, fv[3] = {0.0, 0.0, 0.0};
    if (ee != 0.0) {
      const double small = 1.e-6, alpha = 32.0, th = s.thickness;
      const double gx = (po[q + 1] - po[q - 1]) * 0.5, gy = (po[q + X] - po[q - X]) * 0.5;
      const double gz = DIM == 3 ? (po[q + XY] - po[q - XY]) * 0.5 : 0.0;
      const double na = fmax(sqrt(gx * gx + gy * gy + gz * gz), small);
      const double vol = DIM == 3 ? s.dx * s.dy * s.dz : s.dx * s.dy;
      const double cp = -vol * 2.0 * e * (1.0 - e);
      const double cv = vol * alpha * s.density * s.xnue;
      const double h[3] = {s.dx, s.dy, s.dz}, gn[3] = {gx, gy, gz};
#pragma unroll
      for (int d = 0; d < DIM; d++) {
        const double td = ee / (th * h[d]);
        fp[d] = cp / (th * h[d]) * (gn[d] / na);
        fv[d] = cv * (td * td);
      }
    }
    const double pc = pref(g, p0, p1, i, j, k);
    f[0] = fp[0] * pc;
    f[1] = fp[1] * pc;
    f[3] = fv[0] * u[q];
    f[4] = fv[1] * v[q];
    if (DIM == 3) {
      f[2] = fp[2] * pc;
      f[5] = fv[2] * w[q];
    }
  }
  for (int c = 0; c < 6; c++) {
    const double r = block_sum_fixed(f[c], sh);
    if (threadIdx.x == 0) part[6 * (long long)blockIdx.x + c] = r;
  }
}

__global__ void k_forces_sum(const double* __restrict__ part, int nb, double* __restrict__ out) {
  __shared__ double sh[FORCE_THREADS / 32];
  for (int c = 0; c < 6; c++) {
    double v = 0.0;
    for (int b = threadIdx.x; b < nb; b += FORCE_THREADS) v += part[6 * (long long)b + c];
    const double r = block_sum_fixed(v, sh);
    if (threadIdx.x == 0) out[c] = r;
  }
}

// staging <-> layouts ---------------------------------------------------
__global__ void k_scatter_nat(Geo g, const double* __restrict__ st, double* __restrict__ dst) {
  const int i = blockIdx.x * BX + threadIdx.x;
  const int j = blockIdx.y * BY + threadIdx.y;
  const int k = blockIdx.z;
  if (i > g.m + 1 || j > g.n + 1) return;
  const idx_t d = (idx_t)i + (idx_t)(g.m + 2) * ((idx_t)j + (idx_t)(g.n + 2) * k);
  dst[nat_idx(g, i, j, k)] = st[d];
}
__global__ void k_gather_nat(Geo g, const double* __restrict__ src, double* __restrict__ st) {
  const int i = blockIdx.x * BX + threadIdx.x;
  const int j = blockIdx.y * BY + threadIdx.y;
  const int k = blockIdx.z;
  if (i > g.m + 1 || j > g.n + 1) return;
  const idx_t d = (idx_t)i + (idx_t)(g.m + 2) * ((idx_t)j + (idx_t)(g.n + 2) * k);
  st[d] = src[nat_idx(g, i, j, k)];
}
__global__ void k_scatter_pk(Geo g, const double* __restrict__ st, double* p0, double* p1) {
  const int i = blockIdx.x * BX + threadIdx.x;
  const int j = blockIdx.y * BY + threadIdx.y;
  const int k = blockIdx.z;
  if (i > g.m + 1 || j > g.n + 1) return;
  const idx_t d = (idx_t)i + (idx_t)(g.m + 2) * ((idx_t)j + (idx_t)(g.n + 2) * k);
  pref(g, p0, p1, i, j, k) = st[d];
}
__global__ void k_gather_pk(Geo g, const double* p0, const double* p1, double* __restrict__ st) {
  const int i = blockIdx.x * BX + threadIdx.x;
  const int j = blockIdx.y * BY + threadIdx.y;
  const int k = blockIdx.z;
  if (i > g.m + 1 || j > g.n + 1) return;
  const idx_t d = (idx_t)i + (idx_t)(g.m + 2) * ((idx_t)j + (idx_t)(g.n + 2) * k);
  int c;
  const idx_t r = pk_of(g, i, j, k, c);
  st[d] = c ? p1[r] : p0[r];
}


// ---------------------------------------------------------------------
// Mixed precision form: FP64 defect correction around FP32 sweeps.
//
// In normalised form the plain iteration is p <- (1-w) p + bbn - sum a p_nb.
// Writing p = p0 + e with p0 fixed during a pass gives exactly the same
// iteration on the correction e with the right-hand side
//   r = bbn - w p0 - sum a p0_nb     (the residual, normalised by w/ap),
// so k inner sweeps on e from e = 0 reproduce k plain sweeps from p0 in
// exact arithmetic.  r and p += e are FP64; the sweeps on e are FP32.

// FP64 residual of one colour, stored as FP32 right-hand side of the
// correction sweeps; also zeroes e of that colour and reduces max|r|.
template <int DIM>
__global__ void __launch_bounds__(SWEEP_THREADS) k_residual(Geo g, Coef<double> C, const double* __restrict__ pc,
                                                     const double* __restrict__ po, double omega, int colour,
                                                     float* __restrict__ rf, float* __restrict__ ec,
                                                     unsigned long long* __restrict__ rmax,
                                                     const int* __restrict__ skip) {
  pdl_begin();
  if (skip && *skip) return;
  const int t = blockIdx.x * SWEEP_THREADS + threadIdx.x;
  unsigned long long r = 0;
  if (t < packed_items(g)) {
    int h, j, k;
    packed_item<DIM>(g, t, h, j, k);
    r = c_residual<DIM>(g, C, pc, po, omega, colour, rf, ec, h, j, k);
  }
  block_max_atomic(r, rmax);
}

// FP32 correction sweep, four consecutive cells of one packed row per
// thread: every operand row is one aligned 16-byte load (the packed pitch H
// is a multiple of 32 and chunks start at multiples of 4), and the x
// neighbours of the four cells are the other colour's same four slots plus
// one slot before (s = 0) or after (s = 1) them.  15 loads per 4 updates in
// 3D instead of 15 per update; the per-cell arithmetic is dc_cell.
// Threads map to (row, chunk) with `chunks` chunks per interior row; lanes
// outside 1 <= i <= m store their old value back.
constexpr int DC4_THREADS = 256;

// V consecutive floats loaded as one aligned vector access.
template <int V>
struct alignas(4 * V) VecF {
  float a[V];
};
template <int V>
__device__ __forceinline__ VecF<V> ldv(const float* p) {
  return *reinterpret_cast<const VecF<V>*>(p);
}

template <int DIM, bool TRACK, int V>
__global__ void __launch_bounds__(DC4_THREADS) k_sor_dc4(Geo g, DCConst K, const float* __restrict__ epsc,
                                                         const float* __restrict__ epso,
                                                         const float* __restrict__ r, float* __restrict__ ec,
                                                         const float* __restrict__ eo, int colour, int chunks,
                                                         unsigned long long* __restrict__ err,
                                                         const int* __restrict__ skip) {
  pdl_begin();
  if (skip && *skip) return;
  const int t = blockIdx.x * DC4_THREADS + threadIdx.x;
  const int rows = DIM == 3 ? g.n * g.l : g.n;
  unsigned e = 0;
  if (t < chunks * rows) {
    const int row = t / chunks;
    const int h0 = (t - row * chunks) * V;
    const int k = DIM == 3 ? row / g.n + 1 : 0;
    const int j = DIM == 3 ? row - (k - 1) * g.n + 1 : row + 1;
    const int s = (colour + j + (DIM == 3 ? k : 1)) & 1;
    const idx_t H = g.H, HY = (idx_t)g.H * g.Y;
    const idx_t q = pk_idx(g, h0, j, k);
    const idx_t qn = (j == g.n) ? pk_idx(g, h0, g.jn_n, k) : q + H;
    const idx_t qs = (j == 1) ? pk_idx(g, h0, g.js_1, k) : q - H;
    const VecF<V> EC = ldv<V>(ec + q), R = ldv<V>(r + q), PC = ldv<V>(epsc + q);
    const VecF<V> XO = ldv<V>(eo + q), PO = ldv<V>(epso + q);
    const float xx = s ? eo[q + V] : eo[q - 1];
    const float px = s ? epso[q + V] : epso[q - 1];
    const VecF<V> XN = ldv<V>(eo + qn), XS = ldv<V>(eo + qs), PN = ldv<V>(epso + q + H), PS = ldv<V>(epso + q - H);
    VecF<V> XT{}, XB{}, PT{}, PB{};
    if (DIM == 3) {
      const idx_t qt = (k == g.l) ? pk_idx(g, h0, j, g.kt_l) : q + HY;
      const idx_t qb = (k == 1) ? pk_idx(g, h0, j, g.kb_1) : q - HY;
      XT = ldv<V>(eo + qt);
      XB = ldv<V>(eo + qb);
      PT = ldv<V>(epso + q + HY);
      PB = ldv<V>(epso + q - HY);
    }
    VecF<V> out;
#pragma unroll
    for (int u = 0; u < V; u++) {
      const int i = 2 * (h0 + u) + s;
      const float eold = EC.a[u];
      // east = other colour at h + s, west at h - 1 + s
      const float xe = s ? (u < V - 1 ? XO.a[u + 1] : xx) : XO.a[u];
      const float xw = s ? XO.a[u] : (u > 0 ? XO.a[u - 1] : xx);
      const float pe = s ? (u < V - 1 ? PO.a[u + 1] : px) : PO.a[u];
      const float pw = s ? PO.a[u] : (u > 0 ? PO.a[u - 1] : px);
      const float v = dc_cell<DIM>(K, PC.a[u], pe, pw, PN.a[u], PS.a[u], PT.a[u], PB.a[u], xe, xw, XN.a[u],
                                   XS.a[u], XT.a[u], XB.a[u], R.a[u], eold, i == 1, i == g.m);
      const bool in = i >= 1 && i <= g.m;
      out.a[u] = in ? v : eold;
      if (TRACK && in) e = max(e, abs_bits(v - eold));
    }
    *reinterpret_cast<VecF<V>*>(ec + q) = out;
  }
  if (TRACK) block_max_atomic(e, err);
}

// FP32 porosity packed by colour (all positions, ghosts included).
__global__ void k_pack_eps(Geo g, const double* __restrict__ po, float* e0, float* e1) {
  const int i = blockIdx.x * BX + threadIdx.x;
  const int j = blockIdx.y * BY + threadIdx.y;
  const int k = blockIdx.z;
  if (i > g.m + 1 || j > g.n + 1) return;
  int c;
  const idx_t r = pk_of(g, i, j, k, c);
  (c ? e1 : e0)[r] = (float)po[nat_idx(g, i, j, k)];
}

// p += e over the interior cells of both colours (FP64 accumulation).
template <int DIM>
__global__ void k_accumulate(Geo g, double* __restrict__ p0, double* __restrict__ p1, const float* __restrict__ e0,
                             const float* __restrict__ e1, const int* __restrict__ skip) {
  pdl_begin();
  if (skip && *skip) return;
  const int h = blockIdx.x * BX + threadIdx.x;
  const int j = blockIdx.y * BY + threadIdx.y + 1;
  const int colour = blockIdx.z & 1;
  const int k = (DIM == 3) ? (blockIdx.z >> 1) + 1 : 0;
  c_accumulate<DIM>(g, colour ? p1 : p0, colour ? e1 : e0, colour, h, j, k);
}

// Zero n reduction slots (or one int flag) inside a step: a kernel, not a
// memset, so the programmatic launch chain of the step is not interrupted.
__global__ void k_zero_u64(unsigned long long* p, int n) {
  pdl_begin();
  for (int i = threadIdx.x; i < n; i += blockDim.x) p[i] = 0ULL;
}
__global__ void k_zero_int(int* p) {
  pdl_begin();
  *p = 0;
}

// Stop the remaining passes of this step once max|r|/w <= tol.
__global__ void k_dc_check(const unsigned long long* rmax, double tol_w, int* skip) {
  pdl_begin();
  const double r = __longlong_as_double((long long)max_of_slots(rmax));
  if (r <= tol_w) *skip = 1;
}

__global__ void k_to_float(const double* __restrict__ a, float* __restrict__ b, long long n) {
  pdl_begin();
  const long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (q < n) b[q] = (float)a[q];
}
__global__ void k_to_double(const float* __restrict__ a, double* __restrict__ b, long long n) {
  const long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (q < n) b[q] = (double)a[q];
}

}  // namespace

// ---- launchers ----------------------------------------------------------
void launch_porosity_factors(const Geo& g, const Scal& s, const double* poro, double* gx, double* gy,
                             double* gz, double* rinv, double* damp, cudaStream_t st) {
  k_porosity_factors<<<grid_interior(g), dim3(BX, BY), 0, st>>>(g, s, poro, gx, gy, gz, rinv, damp);
}

void launch_setup_coef(const Geo& g, const Scal& s, const double* poro, Coef<double> c0, Coef<double> c1,
                       cudaStream_t st) {
  k_setup_coef<<<grid_interior(g), dim3(BX, BY), 0, st>>>(g, s, poro, c0, c1);
}

template <typename TV>
void launch_divergence(const Geo& g, const Scal& s, const TV* uo, const TV* vo, const TV* wo, TV* div,
                       cudaStream_t st) {
  launch_pdl(k_divergence<TV>, grid_interior(g), dim3(BX, BY), st, g, s, uo, vo, wo, div);
}

template <typename T, typename TS>
void launch_predictor(const Geo& g, const Scal& s, const T* uo, const T* vo, const T* wo, const T* div,
                      const T* gx, const T* gy, const T* gz, const T* rinv, const T* damp, const TS* us,
                      const TS* vs, const TS* ws, TS* u, TS* v, TS* w, cudaStream_t st) {
  if (g.dim == 3)
    launch_pdl(k_predictor<T, TS, 3>, grid_interior(g), dim3(BX, BY), st, g, s, uo, vo, wo, div, gx, gy, gz, rinv,
                                                                     damp, us, vs, ws, u, v, w);
  else
    launch_pdl(k_predictor<T, TS, 2>, grid_interior(g), dim3(BX, BY), st, g, s, uo, vo, wo, div, gx, gy, gz, rinv,
                                                                     damp, us, vs, ws, u, v, w);
}
template void launch_predictor<double, double>(const Geo&, const Scal&, const double*, const double*,
                                               const double*, const double*, const double*, const double*,
                                               const double*, const double*, const double*, const double*,
                                               const double*, const double*, double*, double*, double*,
                                               cudaStream_t);
template void launch_predictor<float, double>(const Geo&, const Scal&, const float*, const float*, const float*,
                                              const float*, const float*, const float*, const float*,
                                              const float*, const float*, const double*, const double*,
                                              const double*, double*, double*, double*, cudaStream_t);

template <typename TV>
void launch_rhs(const Geo& g, const Scal& s, const TV* u, const TV* v, const TV* w, const double* poro,
                const double* gx, const double* gy, const double* gz, Coef<double> c0, Coef<double> c1,
                cudaStream_t st) {
  if (g.dim == 3)
    launch_pdl(k_rhs<TV, 3>, grid_interior(g), dim3(BX, BY), st, g, s, u, v, w, poro, gx, gy, gz, c0, c1);
  else
    launch_pdl(k_rhs<TV, 2>, grid_interior(g), dim3(BX, BY), st, g, s, u, v, w, poro, gx, gy, gz, c0, c1);
}

static dim3 grid_packed(const Geo& g) {
  const int nh = (g.m + 1) / 2 + 1;
  return dim3((nh + BX - 1) / BX, (g.n + BY - 1) / BY, g.dim == 3 ? g.l : 1);
}

template <typename T>
void launch_sor_half(const Geo& g, const Coef<T>& cc, T* pc, const T* po, T one_minus_omega, int colour,
                     unsigned long long* err, const int* skip, cudaStream_t st) {
  const unsigned grid = (unsigned)((packed_items(g) + SWEEP_THREADS - 1) / SWEEP_THREADS);
  if (g.dim == 3) {
    if (err)
      launch_pdl(k_sor_half<T, 3, true>, grid, SWEEP_THREADS, st, g, cc, pc, po, one_minus_omega, colour, err, skip);
    else
      launch_pdl(k_sor_half<T, 3, false>, grid, SWEEP_THREADS, st, g, cc, pc, po, one_minus_omega, colour, err, skip);
  } else {
    if (err)
      launch_pdl(k_sor_half<T, 2, true>, grid, SWEEP_THREADS, st, g, cc, pc, po, one_minus_omega, colour, err, skip);
    else
      launch_pdl(k_sor_half<T, 2, false>, grid, SWEEP_THREADS, st, g, cc, pc, po, one_minus_omega, colour, err, skip);
  }
}

template <typename T>
void launch_p_halo(const Geo& g, T* p0, T* p1, const int* skip, cudaStream_t st) {
  const int a = g.dim == 3 ? (g.n > g.l ? g.n : g.l) : 1;
  launch_pdl(k_p_halo<T>, dim3((g.m + 127) / 128, a, g.dim == 3 ? 2 : 1), dim3(128), st, g, p0, p1, skip);
}

template <typename TV>
void launch_projection(const Geo& g, const Scal& s, const double* p0, const double* p1, TV* u, TV* v, TV* w,
                       cudaStream_t st) {
  if (g.dim == 3)
    launch_pdl(k_projection<TV, 3>, grid_interior(g), dim3(BX, BY), st, g, s, p0, p1, u, v, w);
  else
    launch_pdl(k_projection<TV, 2>, grid_interior(g), dim3(BX, BY), st, g, s, p0, p1, u, v, w);
}

template <typename TV>
void launch_boundary(const Geo& g, const Scal& s, TV* u, TV* v, TV* w, double* p0, double* p1,
                     cudaStream_t st) {
  if (g.wall) {
    const dim3 xy((g.m + 2 + 127) / 128, g.n + 2), yz((g.n + 2 + 127) / 128, g.l + 2),
        xz((g.m + 2 + 127) / 128, g.l + 2);
    launch_pdl(k_wall_face<0, TV>, xy, dim3(128), st, g, s, u, v, w, p0, p1);
    launch_pdl(k_wall_face<1, TV>, xy, dim3(128), st, g, s, u, v, w, p0, p1);
    launch_pdl(k_wall_face<3, TV>, yz, dim3(128), st, g, s, u, v, w, p0, p1);
    launch_pdl(k_wall_face<2, TV>, yz, dim3(128), st, g, s, u, v, w, p0, p1);
    launch_pdl(k_wall_face<4, TV>, xz, dim3(128), st, g, s, u, v, w, p0, p1);
    launch_pdl(k_wall_face<5, TV>, xz, dim3(128), st, g, s, u, v, w, p0, p1);
    return;
  }
  launch_pdl(k_bnd_x<TV>, dim3((g.n + 127) / 128, g.dim == 3 ? g.l : 1), dim3(128), st, g, s, u, v, w, p0, p1);
  launch_pdl(k_bnd_y<TV>, dim3((g.m + 2 + 127) / 128, g.dim == 3 ? g.l + 2 : 1), dim3(128), st, g, u, v, w, p0, p1);
  if (g.dim == 3) launch_pdl(k_bnd_z<TV>, dim3((g.m + 2 + 127) / 128, g.n + 2), dim3(128), st, g, u, v, w, p0, p1);
}

template <typename TV>
void launch_initial(const Geo& g, const Scal& s, TV* u, TV* v, TV* w, double* p0, double* p1,
                    cudaStream_t st) {
  k_initial<TV><<<grid_interior(g), dim3(BX, BY), 0, st>>>(g, s, u, v, w, p0, p1);
}

template <typename TV>
void launch_div_diag(const Geo& g, const Scal& s, const TV* u, const TV* v, const TV* w, const double* poro,
                     const double* gx, const double* gy, const double* gz, unsigned long long* out,
                     cudaStream_t st) {
  k_div_diag<TV><<<grid_interior(g), dim3(BX, BY), 0, st>>>(g, s, u, v, w, poro, gx, gy, gz, out);
}

void launch_residual(const Geo& g, const Coef<double>& C, const double* pc, const double* po, double omega,
                     int colour, float* rf, float* ec, unsigned long long* rmax, const int* skip,
                     cudaStream_t st) {
  const unsigned grid = (unsigned)((packed_items(g) + SWEEP_THREADS - 1) / SWEEP_THREADS);
  if (g.dim == 3)
    launch_pdl(k_residual<3>, grid, SWEEP_THREADS, st, g, C, pc, po, omega, colour, rf, ec, rmax, skip);
  else
    launch_pdl(k_residual<2>, grid, SWEEP_THREADS, st, g, C, pc, po, omega, colour, rf, ec, rmax, skip);
}

void launch_sor_dc(const Geo& g, const Scal& sc, const float* epsc, const float* epso, const float* r, float* ec,
                   const float* eo, int colour, unsigned long long* err, const int* skip, cudaStream_t st) {
  DCConst K;
  K.kx = (float)(sc.dt / sc.dx / sc.dx);
  K.ky = (float)(sc.dt / sc.dy / sc.dy);
  K.kz = g.dim == 3 ? (float)(sc.dt / sc.dz / sc.dz) : 0.f;
  K.small = 1.e-6f;
  K.omega = (float)sc.omega;
  K.omw = (float)(1.0 - sc.omega);
  // chunks of 4 slots covering h = 0 .. m/2 (the largest h of an interior cell);
  // 4 beat 2 per thread at 256^3 (1511 vs 1336 Mcell-steps/s for the step):
  // the extra occupancy of narrower chunks does not pay for their extra
  // instructions
  constexpr int V = 4;
  const int chunks = (g.m >> 1) / V + 1;
  const long long threads = (long long)chunks * g.n * (g.dim == 3 ? g.l : 1);
  const unsigned blocks = (unsigned)((threads + DC4_THREADS - 1) / DC4_THREADS);
#define PF_DC(DIMV, TR) \
  launch_pdl(k_sor_dc4<DIMV, TR, V>, dim3(blocks), dim3(DC4_THREADS), st, g, K, epsc, epso, r, ec, eo, colour, \
             chunks, err, skip)
  if (g.dim == 3) {
    if (err)
      PF_DC(3, true);
    else
      PF_DC(3, false);
  } else {
    if (err)
      PF_DC(2, true);
    else
      PF_DC(2, false);
  }
#undef PF_DC
}

int launch_forces(const Geo& g, const Scal& s, const double* poro, const double* p0, const double* p1,
                  const double* u, const double* v, const double* w, double* scratch, double* out,
                  cudaStream_t st) {
  const long long cells = (long long)g.m * g.n * (g.dim == 3 ? g.l : 1);
  const int nb = (int)((cells + FORCE_THREADS - 1) / FORCE_THREADS);
  if (g.dim == 3)
    k_forces<3><<<nb, FORCE_THREADS, 0, st>>>(g, s, poro, p0, p1, u, v, w, scratch);
  else
    k_forces<2><<<nb, FORCE_THREADS, 0, st>>>(g, s, poro, p0, p1, u, v, w, scratch);
  k_forces_sum<<<1, FORCE_THREADS, 0, st>>>(scratch, nb, out);
  return nb;
}

void launch_pack_eps(const Geo& g, const double* poro, float* e0, float* e1, cudaStream_t st) {
  k_pack_eps<<<grid_all(g), dim3(BX, BY), 0, st>>>(g, poro, e0, e1);
}

void launch_accumulate(const Geo& g, double* p0, double* p1, const float* e0, const float* e1, const int* skip,
                       cudaStream_t st) {
  dim3 grid = grid_packed(g);
  grid.z *= 2;
  if (g.dim == 3)
    launch_pdl(k_accumulate<3>, grid, dim3(BX, BY), st, g, p0, p1, e0, e1, skip);
  else
    launch_pdl(k_accumulate<2>, grid, dim3(BX, BY), st, g, p0, p1, e0, e1, skip);
}

void launch_zero_u64(unsigned long long* p, int n, cudaStream_t st) {
  launch_pdl(k_zero_u64, dim3(1), dim3(256), st, p, n);
}
void launch_zero_int(int* p, cudaStream_t st) { launch_pdl(k_zero_int, dim3(1), dim3(1), st, p); }

void launch_dc_check(const unsigned long long* rmax, double tol, int* skip, cudaStream_t st) {
  launch_pdl(k_dc_check, dim3(1), dim3(1), st, rmax, tol, skip);
}

void launch_to_float(const double* src, float* dst, long long n, cudaStream_t st) {
  launch_pdl(k_to_float, dim3((unsigned)((n + 255) / 256)), dim3(256), st, src, dst, n);
}
void launch_to_double(const float* src, double* dst, long long n, cudaStream_t st) {
  k_to_double<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(src, dst, n);
}

void launch_scatter_nat(const Geo& g, const double* stage, double* dst, cudaStream_t st) {
  k_scatter_nat<<<grid_all(g), dim3(BX, BY), 0, st>>>(g, stage, dst);
}
void launch_gather_nat(const Geo& g, const double* src, double* stage, cudaStream_t st) {
  k_gather_nat<<<grid_all(g), dim3(BX, BY), 0, st>>>(g, src, stage);
}
void launch_scatter_pk(const Geo& g, const double* stage, double* p0, double* p1, cudaStream_t st) {
  k_scatter_pk<<<grid_all(g), dim3(BX, BY), 0, st>>>(g, stage, p0, p1);
}
void launch_gather_pk(const Geo& g, const double* p0, const double* p1, double* stage, cudaStream_t st) {
  k_gather_pk<<<grid_all(g), dim3(BX, BY), 0, st>>>(g, p0, p1, stage);
}

// explicit instantiations ------------------------------------------------
#define PF_INST_V(TV)                                                                                        \
  template void launch_divergence<TV>(const Geo&, const Scal&, const TV*, const TV*, const TV*, TV*,         \
                                      cudaStream_t);                                                         \
  template void launch_rhs<TV>(const Geo&, const Scal&, const TV*, const TV*, const TV*, const double*,      \
                               const double*, const double*, const double*, Coef<double>, Coef<double>,     \
                               cudaStream_t);                                                                \
  template void launch_projection<TV>(const Geo&, const Scal&, const double*, const double*, TV*, TV*, TV*,  \
                                      cudaStream_t);                                                         \
  template void launch_boundary<TV>(const Geo&, const Scal&, TV*, TV*, TV*, double*, double*, cudaStream_t); \
  template void launch_initial<TV>(const Geo&, const Scal&, TV*, TV*, TV*, double*, double*, cudaStream_t);  \
  template void launch_div_diag<TV>(const Geo&, const Scal&, const TV*, const TV*, const TV*, const double*, \
                                    const double*, const double*, const double*, unsigned long long*,       \
                                    cudaStream_t);                                                           \
  template void launch_sor_half<TV>(const Geo&, const Coef<TV>&, TV*, const TV*, TV, int,                   \
                                    unsigned long long*, const int*, cudaStream_t);                          \
  template void launch_p_halo<TV>(const Geo&, TV*, TV*, const int*, cudaStream_t);
PF_INST_V(double)
PF_INST_V(float)
#undef PF_INST_V

}  // namespace pf
