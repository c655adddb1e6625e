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

#include <algorithm>

#include "pf_internal.cuh"
#include "pf_cells.cuh"

namespace pf {

namespace {

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
    // the symmetry rows the reference keeps commented out (2D :440-450),
    // applied after the inlet and outlet edits, as listed there
    if (g.slip && j == 1) {
      a[2] = a[2] + a[3];
      a[3] = 0.0;
    }
    if (g.slip && j == g.n) {
      a[3] = a[3] + a[2];
      a[2] = 0.0;
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
// the periodic ghost rows are read by wrapping in the predictor.  3D grids
// cover the planes k0+1 .. k0+gridDim.z.
template <typename T>
__global__ void k_divergence(Geo g, Scal s, const T* __restrict__ uo, const T* __restrict__ vo,
                             const T* __restrict__ wo, T* __restrict__ div, int k0) {
  pdl_begin();
  const int i = blockIdx.x * BX + threadIdx.x + 1;
  const int j = blockIdx.y * BY + threadIdx.y + 1;
  const int k = (g.dim == 3) ? blockIdx.z + 1 + k0 : 0;
  if (i > g.m || j > g.n) return;
  c_divergence<T>(g, s, uo, vo, wo, div, i, j, k);
}

// Predictor: explicit Euler of the porosity-weighted momentum equation.
// Also copies the face ghosts of the old fields into the new ones, so the
// RHS sees the previous step's ghosts exactly as the reference does.
// T: type of the stencil arithmetic and of the arrays it reads; TS: type of
// the velocity state.  The predictor computes the increment u* - u_old in T
// and adds it to the TS state, so with T = float, TS = double the stencils run
// in FP32 while the state keeps FP64 precision.  3D grids cover the planes
// k0+1 .. k0+gridDim.z.
template <typename T, typename TS, int DIM>
__device__ __forceinline__ void predictor_body(Geo g, Scal s, const T* __restrict__ uo,
                                                      const T* __restrict__ vo, const T* __restrict__ wo,
                                                      const T* __restrict__ div, const T* __restrict__ gxa,
                                                      const T* __restrict__ gya, const T* __restrict__ gza,
                                                      const T* __restrict__ rinva, const T* __restrict__ dampa,
                                                      const TS* __restrict__ su, const TS* __restrict__ sv,
                                                      const TS* __restrict__ sw, TS* __restrict__ u,
                                                      TS* __restrict__ v, TS* __restrict__ w, int k0) {
  pdl_begin();
  const int i = blockIdx.x * BX + threadIdx.x + 1;
  const int j = blockIdx.y * BY + threadIdx.y + 1;
  const int k = (DIM == 3) ? blockIdx.z + 1 + k0 : 0;
  const bool in = i <= g.m && j <= g.n;
  if (DIM == 3) {
    // A warp is one x-row of BX = 32 cells.  Where every cell of it has zero
    // porosity gradients and no non-slip damping (fluid away from the
    // obstacles), the porosity terms of all three components vanish and the
    // warp takes the shorter path: about a third fewer FP64 operations.  The
    // vote runs before any lane leaves; lanes past the grid count as fluid.
    bool fl = true;
    if (in) {
      const idx_t q = nat_idx(g, i, j, k);
      fl = gxa[q] == T(0) && gya[q] == T(0) && gza[q] == T(0) && dampa[q] == T(0);
    }
    const bool all = __all_sync(0xffffffffu, fl);
    if (!in) return;
    if (all)
      c_predictor<T, TS, DIM, true>(g, s, uo, vo, wo, div, gxa, gya, gza, rinva, dampa, su, sv, sw, u, v, w, i, j,
                                    k);
    else
      c_predictor<T, TS, DIM, false>(g, s, uo, vo, wo, div, gxa, gya, gza, rinva, dampa, su, sv, sw, u, v, w, i, j,
                                     k);
    return;
  }
  if (!in) return;
  c_predictor<T, TS, DIM>(g, s, uo, vo, wo, div, gxa, gya, gza, rinva, dampa, su, sv, sw, u, v, w, i, j, k);
}

#define PF_PRED_PARAMS                                                                                            \
  Geo g, Scal s, const T* __restrict__ uo, const T* __restrict__ vo, const T* __restrict__ wo,                    \
      const T* __restrict__ div, const T* __restrict__ gxa, const T* __restrict__ gya, const T* __restrict__ gza, \
      const T* __restrict__ rinva, const T* __restrict__ dampa, const TS* __restrict__ su,                        \
      const TS* __restrict__ sv, const TS* __restrict__ sw, TS* __restrict__ u, TS* __restrict__ v,             \
      TS* __restrict__ w, int k0
#define PF_PRED_ARGS g, s, uo, vo, wo, div, gxa, gya, gza, rinva, dampa, su, sv, sw, u, v, w, k0
template <typename T, typename TS, int DIM>
__global__ void __launch_bounds__(BX* BY) k_predictor(PF_PRED_PARAMS) {
  predictor_body<T, TS, DIM>(PF_PRED_ARGS);
}
// The FP64 3D form holds 94 registers a thread with the isotropic Laplacian;
// a bound of three CTAs per SM (80 registers, 8 bytes of spills) keeps more
// warps resident: 256^3 plain step 21.69 -> 21.42 ms (22.00 ms with the
// directional Laplacian at 64 registers).
template <typename TS, typename T = double>
__global__ void __launch_bounds__(BX* BY, 3) k_predictor_fp64_3d(PF_PRED_PARAMS) {
  predictor_body<double, TS, 3>(PF_PRED_ARGS);
}
#undef PF_PRED_PARAMS
#undef PF_PRED_ARGS

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

// One red-black half-sweep of colour `colour`, in place: for each cell
// (2h+s, j, k) of that colour,  p = (1-omega) p + bbn - sum_nb a_nb p_nb
// (all neighbours have the other colour), which is the reference's
//   p = (bb - sum a_nb p_old_nb)/ap*omega + p_old*(1-omega)
// because no neighbour of a cell changes during its own colour's sweep.
// With TRACK the max of |p_new - p_old| goes to err.
//
// EARLY: the cell's operator (bbn and the face coefficients) is loaded
// before griddepcontrol.wait.  Under programmatic dependent launch the
// grid's CTAs are resident before the previous half-sweep has finished; the
// operator was written by kernels that finished before that one could
// launch, so only the loads of p stay behind the wait, which shortens each
// half-sweep of the launch-bound small grids.  Not for the first half-sweep
// of a step, whose predecessor writes bbn.
template <typename T, int DIM, bool TRACK, bool EARLY>
__global__ void __launch_bounds__(SWEEP_THREADS) k_sor_half(Geo g, Coef<T> C, T* __restrict__ pc,
                                                            const T* __restrict__ po, T omw, int colour,
                                                            unsigned long long* __restrict__ err,
                                                            const int* __restrict__ skip) {
  const int t = blockIdx.x * SWEEP_THREADS + threadIdx.x;
  int h = 0, j = 1, k = 1;
  bool act = t < packed_items(g);
  if (act) packed_item<DIM>(g, t, h, j, k);
  const int s = (colour + j + (DIM == 3 ? k : 1)) & 1;
  const int i = 2 * h + s;
  act = act && j <= g.n && i >= 1 && i <= g.m;
  const idx_t q = pk_idx(g, h, j, k);
  T cb = T(0), c0 = T(0), c1 = T(0), c2 = T(0), c3 = T(0), c4 = T(0), c5 = T(0);
  auto load_operator = [&]() {
    cb = C.bbn[q];
    c0 = C.a[0][q];
    c1 = C.a[1][q];
    c2 = C.a[2][q];
    c3 = C.a[3][q];
    if (DIM == 3) {
      c4 = C.a[4][q];
      c5 = C.a[5][q];
    }
  };
  if (EARLY && act) load_operator();
  pdl_begin();
  if (skip && *skip) return;  // uniform over the grid: defect correction converged
  if (!EARLY && act) load_operator();
  decltype(abs_bits(T(0))) e = 0;
  if (act) {
    const idx_t H = g.H, HY = (idx_t)g.H * g.Y;
    const idx_t qn = (j == g.n) ? pk_idx(g, h, g.jn_n, k) : q + H;
    const idx_t qs = (j == 1) ? pk_idx(g, h, g.js_1, k) : q - H;
    const T pold = pc[q];
    T tt = cb;
    tt = fma(-c0, po[q + s], tt);
    tt = fma(-c1, po[q - 1 + s], tt);
    tt = fma(-c2, po[qn], tt);
    tt = fma(-c3, po[qs], tt);
    if (DIM == 3) {
      const idx_t qt = (k == g.l) ? pk_idx(g, h, j, g.kt_l) : q + HY;
      const idx_t qb = (k == 1) ? pk_idx(g, h, j, g.kb_1) : q - HY;
      tt = fma(-c4, po[qt], tt);
      tt = fma(-c5, po[qb], tt);
    }
    const T pnew = fma(omw, pold, tt);
    pc[q] = pnew;
    if (TRACK) e = abs_diff_bits(pnew, pold);
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

// boundary, symmetry rows (2D slip option) over i = 1..m, after the periodic
// ghost rows.
template <typename T>
__global__ void k_bnd_slip(Geo g, T* u, T* v, double* p0, double* p1) {
  pdl_begin();
  const int i = blockIdx.x * blockDim.x + threadIdx.x + 1;
  if (i <= g.m) c_bnd_slip(g, u, v, p0, p1, i);
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
  warp_max_atomic(r, rmax);
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
    *reinterpret_cast<VecF<V>*>(ec + q) =
        dc_chunk<DIM, TRACK, V>(g, K, h0, s, EC, R, PC, XO, PO, xx, px, XN, XS, PN, PS, XT, XB, PT, PB, e);
  }
  if (TRACK) warp_max_atomic(e, err);
}

// The same sweep for grids of one wave, where a launch's latency dominates:
// porosity (set-up time) and the residual r (written by the residual kernel
// of this colour, which finished before the kernel preceding this one could
// let it launch) are loaded before griddepcontrol.wait, the correction,
// which the preceding kernel may write, after it.  (On larger grids this
// order of the loads costs more than it saves: 256^3 step 1553 -> 1414
// Mcell-steps/s.)  The arithmetic is dc_chunk's, so the bits are k_sor_dc4's.
template <int DIM, bool TRACK, int V>
__global__ void __launch_bounds__(DC4_THREADS) k_sor_dc4_early(Geo g, DCConst K, const float* __restrict__ epsc,
                                                               const float* __restrict__ epso,
                                                               const float* __restrict__ r, float* __restrict__ ec,
                                                               const float* __restrict__ eo, int colour, int chunks,
                                                               unsigned long long* __restrict__ err,
                                                               const int* __restrict__ skip) {
  const int t = blockIdx.x * DC4_THREADS + threadIdx.x;
  const int rows = DIM == 3 ? g.n * g.l : g.n;
  const bool act = t < chunks * rows;
  const int row = act ? t / chunks : 0;
  const int h0 = (t - row * chunks) * V;
  const int k = DIM == 3 ? row / g.n + 1 : 0;
  const int j = DIM == 3 ? row - (k - 1) * g.n + 1 : row + 1;
  const int s = (colour + j + (DIM == 3 ? k : 1)) & 1;
  const idx_t H = g.H, HY = (idx_t)g.H * g.Y;
  const idx_t q = pk_idx(g, h0, j, k);
  VecF<V> R{}, PC{}, PO{}, PN{}, PS{}, PT{}, PB{};
  float px = 0.f;
  if (act) {
    R = ldv<V>(r + q);
    PC = ldv<V>(epsc + q);
    PO = ldv<V>(epso + q);
    px = s ? epso[q + V] : epso[q - 1];
    PN = ldv<V>(epso + q + H);
    PS = ldv<V>(epso + q - H);
    if (DIM == 3) {
      PT = ldv<V>(epso + q + HY);
      PB = ldv<V>(epso + q - HY);
    }
  }
  pdl_begin();
  if (skip && *skip) return;
  unsigned e = 0;
  if (act) {
    const idx_t qn = (j == g.n) ? pk_idx(g, h0, g.jn_n, k) : q + H;
    const idx_t qs = (j == 1) ? pk_idx(g, h0, g.js_1, k) : q - H;
    const VecF<V> EC = ldv<V>(ec + q), XO = ldv<V>(eo + q);
    const float xx = s ? eo[q + V] : eo[q - 1];
    const VecF<V> XN = ldv<V>(eo + qn), XS = ldv<V>(eo + qs);
    VecF<V> XT{}, XB{};
    if (DIM == 3) {
      const idx_t qt = (k == g.l) ? pk_idx(g, h0, j, g.kt_l) : q + HY;
      const idx_t qb = (k == 1) ? pk_idx(g, h0, j, g.kb_1) : q - HY;
      XT = ldv<V>(eo + qt);
      XB = ldv<V>(eo + qb);
    }
    *reinterpret_cast<VecF<V>*>(ec + q) =
        dc_chunk<DIM, TRACK, V>(g, K, h0, s, EC, R, PC, XO, PO, xx, px, XN, XS, PN, PS, XT, XB, PT, PB, e);
  }
  if (TRACK) warp_max_atomic(e, err);
}

// The fused kernel's chunk: dc_chunk (3D, colour side S) with the top faces
// either computed or given (ATIN: colour 1 takes them from the colour-0
// update of the plane above, whose bottom faces they are).  The bottom faces
// are returned in AB.
template <bool TRACK, bool ATIN>
__device__ __forceinline__ VecF<4> dc_chunk_f(const Geo& g, const DCConst& K, int h0, int S, const VecF<4>& EC,
                                              const VecF<4>& R, const VecF<4>& PC, const VecF<4>& XO,
                                              const VecF<4>& PO, float xx, float px, const VecF<4>& XN,
                                              const VecF<4>& XS, const VecF<4>& PN, const VecF<4>& PS,
                                              const VecF<4>& XT, const VecF<4>& XB, const VecF<4>& PT,
                                              const VecF<4>& PB, const VecF<4>& ATin, VecF<4>& AB, unsigned& e) {
  VecF<4> out;
#pragma unroll
  for (int u = 0; u < 4; u++) {
    const int i = 2 * (h0 + u) + S;
    const float eold = EC.a[u];
    const float xe = S ? (u < 3 ? XO.a[u + 1] : xx) : XO.a[u];
    const float xw = S ? XO.a[u] : (u > 0 ? XO.a[u - 1] : xx);
    const float pe = S ? (u < 3 ? PO.a[u + 1] : px) : PO.a[u];
    const float pw = S ? PO.a[u] : (u > 0 ? PO.a[u - 1] : px);
    const float pc = PC.a[u];
    const float at = ATIN ? ATin.a[u] : dc_face(K.hz, K, PT.a[u], pc);
    AB.a[u] = dc_face(K.hz, K, pc, PB.a[u]);
    const float v = dc_cell_faces<3>(K, dc_face(K.hx, K, pe, pc), dc_face(K.hx, K, pc, pw),
                                     dc_face(K.hy, K, PN.a[u], pc), dc_face(K.hy, K, pc, PS.a[u]), at, AB.a[u], xe,
                                     xw, XN.a[u], XS.a[u], XT.a[u], XB.a[u], R.a[u], eold, i == 1, i == g.m);
    const bool in = i >= 1 && i <= g.m;
    out.a[u] = in ? v : eold;
    if (TRACK && in) e = max(e, abs_bits(v - eold));
  }
  return out;
}

// Fused full correction sweep, 3D with even n and l (the periodic y/z edges
// then read the opposite interior rows, which have the other colour): both
// colours of one sweep in one launch, each operand row streamed from HBM
// once per sweep by the bulk-copy (TMA) engine.
//
// Work: tiles of ty rows over the whole x extent, walked in z.  The
// (tile, plane) pairs are dealt out to one persistent CTA per SM in
// contiguous runs; a run that crosses a tile boundary is two segments.
// Within a segment [k0, k1) of tile j0 .. j0+ny-1, step `it` (k = k0-1+it)
// updates colour 0 of plane k on rows j0-1 .. j0+ny, then colour 1 of plane
// k-1.  Each thread owns one chunk of V slots of one of those rows for the
// whole segment and walks it in z, so the z neighbours and its own colour-0
// results of the planes before stay in registers; only the other rows'
// values go through shared memory (a three-plane ring of colour-0 results).
// Halo rows and planes beyond a periodic edge are the opposite interior rows
// and planes.  Colour 0 of the halo rows and of planes k0-1 and k1 is
// recomputed here from the same operands, so every value equals the
// two-launch sweep's bit for bit.  The correction is read from ea (its state
// before the sweep) and written to eb, so a neighbouring CTA's halo
// computation sees old values.
//
// Staging: one thread issues, per step, the cp.async.bulk copies (one per
// run of rows contiguous in memory) of what the step FPRE steps ahead needs
// (for step it: colour-1 correction and porosity of plane k+1 with two rows
// of halo,
// colour-0 porosity, correction and residual of plane k, colour-1 residual of
// plane k-1) into shared-memory rings, and arms an mbarrier with their byte
// count; the consumers wait on it (bounded: after FUSED_WAIT_NS the CTA
// drains its copies in flight, raises PF_FLAG_FUSED_TIMEOUT and leaves).  A
// stage overwrites only ring slots whose last reader finished before the
// step's barrier.
constexpr int FUSED_MAX_THREADS = 512;
constexpr int FUSED_V = 4;
// stages in flight ahead of the one being read: 2 (whole precision-form step
// at 256^3 with the fused sweep: 1196, 1507, 1399 Mcell-steps/s for 1, 2, 3;
// one leaves the staging latency exposed, three makes the rings too deep for
// tall tiles)
constexpr int FPRE = 2;
constexpr int FZE = 2 + FPRE;    // ring depth of E1, P1: planes k, k+1 read, FPRE ahead
constexpr int FZP = 2 + FPRE;    // ring depth of P0: planes k-1, k read, FPRE ahead
constexpr int FZ1 = 1 + FPRE;    // ring depth of E0, R0, R1: one plane read, FPRE ahead
constexpr int FZR = 3;           // colour-0 result ring: plane k-1 read while plane k is written
constexpr int FSTAGES = 1 + FPRE;  // mbarriers: the stage being read and FPRE in flight
constexpr unsigned long long FUSED_WAIT_NS = 200000000ULL;  // 0.2 s; a stage lands in microseconds
constexpr int FUSED_WAIT_POLLS = 1 << 20;                    // backstop on the number of polls
constexpr size_t FUSED_SMEM_MAX = 232448;  // dynamic shared memory per CTA on sm_100-class parts

struct FusedArgs {
  const float* eps[2];  // packed FP32 porosity of colour 0, 1
  const float* r[2];    // packed FP32 residual
  const float* ea[2];   // correction before the sweep
  float* eb[2];         // correction after the sweep
  unsigned long long* err;
  unsigned long long* flags;
  const int* skip;
  int drop_stage;  // testing: a stage index never issued (its wait runs out), -1 otherwise
};

// Shared-memory layout in floats: mbarriers, then the rings, each region
// followed by one pad vector (reads one slot before a row's start or up to
// three past its end, by lanes whose results are discarded, stay inside).
struct FusedLayout {
  int e1, p1, p0, e0, r0, r1, red, total;
};
__host__ __device__ inline FusedLayout fused_layout(int ty, int H, int chunks) {
  FusedLayout L;
  const int rows1 = ty + 4, rows0 = ty + 2;
  int o = 16 + FUSED_V;
  L.e1 = o;
  o += FZE * rows1 * H + FUSED_V;
  L.p1 = o;
  o += FZE * rows1 * H + FUSED_V;
  L.p0 = o;
  o += FZP * rows0 * H + FUSED_V;
  L.e0 = o;
  o += FZ1 * rows0 * H + FUSED_V;
  L.r0 = o;
  o += FZ1 * rows0 * H + FUSED_V;
  L.r1 = o;
  o += FZ1 * ty * H + FUSED_V;
  L.red = o;
  o += FZR * rows0 * (chunks * FUSED_V + 2 * FUSED_V) + FUSED_V;
  L.total = o;
  return L;
}

__device__ __forceinline__ unsigned smem_addr(const void* p) { return (unsigned)__cvta_generic_to_shared(p); }
__device__ __forceinline__ void mbar_init(unsigned long long* bar, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(unsigned long long* bar, unsigned bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes)
               : "memory");
}
// One test of an mbarrier phase; a thread whose phase is not complete may be
// suspended for up to FUSED_SUSPEND_NS (woken early when the phase
// completes), so waiting warps do not spin on the issue slots.
constexpr unsigned FUSED_SUSPEND_NS = 20000;
__device__ __forceinline__ bool mbar_try_wait(unsigned long long* bar, unsigned parity) {
  unsigned ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, %3;\n\tselp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(smem_addr(bar)), "r"(parity), "r"(FUSED_SUSPEND_NS)
      : "memory");
  return ok != 0;
}
__device__ __forceinline__ unsigned long long global_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %globaltimer;" : "=l"(t));
  return t;
}
// Wait for a phase of an mbarrier, giving up after FUSED_WAIT_NS.
__device__ __forceinline__ bool mbar_wait_bounded(unsigned long long* bar, unsigned parity) {
  if (mbar_try_wait(bar, parity)) return true;
  const unsigned long long t0 = global_ns();
  for (int i = 1; i < FUSED_WAIT_POLLS; i++) {
    if (mbar_try_wait(bar, parity)) return true;
    if ((i & 63) == 0 && global_ns() - t0 > FUSED_WAIT_NS) return false;
  }
  return false;
}
__device__ __forceinline__ void bulk_copy(float* dst, const float* src, unsigned bytes, unsigned long long* bar) {
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                   smem_addr(dst)),
               "l"(src), "r"(bytes), "r"(smem_addr(bar))
               : "memory");
}

template <bool TRACK>
__global__ void __launch_bounds__(FUSED_MAX_THREADS)
    k_sor_fused3(Geo g, DCConst K, FusedArgs A, int chunks, int ty, int ntiles, int per_cta) {
  constexpr int V = FUSED_V;
  extern __shared__ __align__(128) float sm[];
  __shared__ int abort_flag;
  pdl_begin();
  if (A.skip && *A.skip) return;
  const int H = g.H;
  const FusedLayout L = fused_layout(ty, H, chunks);
  unsigned long long* bar = reinterpret_cast<unsigned long long*>(sm);
  const int P = chunks * V + 2 * V;  // result ring row pitch: slot h at V + h
  const int plane1 = (ty + 4) * H, plane0 = (ty + 2) * H, planeR1 = ty * H, planeRed = (ty + 2) * P;
  const unsigned rowb = (unsigned)H * sizeof(float);
  const long long total = (long long)ntiles * g.l;
  const long long lo = (long long)blockIdx.x * per_cta;
  const long long hi = lo + per_cta < total ? lo + per_cta : total;
  // the producer: lane 0 of the last warp, whose threads own the top halo row
  // (colour 0 only) or nothing
  const int producer = (blockDim.x - 1) & ~31;
  if (threadIdx.x == 0) {
    for (int b = 0; b < FSTAGES; b++) mbar_init(&bar[b], 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    abort_flag = 0;
  }
  for (int x = threadIdx.x; x < FZR * planeRed; x += blockDim.x) sm[L.red + x] = 0.f;
  __syncthreads();
  auto wrapy = [&](int j) { return j < 1 ? j + g.n : (j > g.n ? j - g.n : j); };
  auto wrapz = [&](int k) { return k < 1 ? k + g.l : (k > g.l ? k - g.l : k); };
  // stage counters: mbarrier count % FSTAGES, parity (count / FSTAGES) & 1;
  // `confirmed` stages are known (to the producer) to have landed
  unsigned issued = 0, waited = 0, confirmed = 0, dropped = ~0u;
  unsigned e = 0;
  bool ok = true;
  // this thread's chunk: row rl of the colour-0 rows j0-1 .. j0+ny, slots h0 ..
  const int rl = threadIdx.x / chunks;
  const int h0 = (threadIdx.x - rl * chunks) * V;
  for (long long pos = lo; pos < hi && ok;) {
    const int tile = (int)(pos / g.l);
    const int k0 = (int)(pos - (long long)tile * g.l) + 1;
    const int k1 = (int)(hi - pos < (long long)(g.l + 1 - k0) ? k0 + (hi - pos) : g.l + 1);
    pos += k1 - k0;
    const int j0 = 1 + tile * ty, ny = min(ty, g.n - j0 + 1);
    const int nit = k1 - k0 + 2;  // steps: colour 0 of planes k0-1 .. k1
    // stage `it`: the rows step `it` reads that no earlier stage brought
    auto issue = [&](int it) {
      if (it == A.drop_stage) {
        dropped = issued++;
        return;
      }
      const int k = k0 - 1 + it;
      const unsigned rows = (unsigned)(2 * (ny + 4) * (it == 0 ? 3 : 1) + 3 * (ny + 2) + (it >= 2 ? ny : 0));
      unsigned long long* b = &bar[issued % FSTAGES];
      mbar_expect_tx(b, rows * rowb);
      // rows jfirst .. jfirst+nrows-1 of plane kk (jfirst may lie up to two
      // rows beyond a periodic edge) of up to three arrays into consecutive
      // ring rows: one bulk copy per run of rows contiguous in memory
      auto rows_copy = [&](int jfirst, int nrows, int kk, float* d0, const float* s0, float* d1, const float* s1,
                           float* d2, const float* s2) {
        for (int r = 0; r < nrows;) {
          const int u = jfirst + r;
          const int len = min(nrows - r, u < 1 ? 1 - u : (u <= g.n ? g.n + 1 - u : 2 * g.n + 1 - u));
          const idx_t src = pk_idx(g, 0, wrapy(u), kk);
          const unsigned bytes = (unsigned)len * rowb;
          bulk_copy(d0 + r * H, s0 + src, bytes, b);
          if (d1) bulk_copy(d1 + r * H, s1 + src, bytes, b);
          if (d2) bulk_copy(d2 + r * H, s2 + src, bytes, b);
          r += len;
        }
      };
      for (int d = it == 0 ? -1 : 1; d <= 1; d++) {  // E1, P1 of plane k+d (plane index it+1+d)
        const int slot = (it + 1 + d) % FZE;
        rows_copy(j0 - 2, ny + 4, wrapz(k + d), sm + L.e1 + slot * plane1, A.ea[1], sm + L.p1 + slot * plane1,
                  A.eps[1], nullptr, nullptr);
      }
      rows_copy(j0 - 1, ny + 2, wrapz(k), sm + L.p0 + (it % FZP) * plane0, A.eps[0],
                sm + L.e0 + (it % FZ1) * plane0, A.ea[0], sm + L.r0 + (it % FZ1) * plane0, A.r[0]);
      if (it >= 2)  // R1 of plane k-1 (interior: k0 <= k-1 < k1)
        rows_copy(j0, ny, k - 1, sm + L.r1 + ((it - 1) % FZ1) * planeR1, A.r[1], nullptr, nullptr, nullptr,
                  nullptr);
      issued++;
    };
    if (threadIdx.x == producer)
      for (int i = 0; i < FPRE && i < nit; i++) issue(i);
    const bool red_item = rl < ny + 2;            // a colour-0 chunk of this tile
    const bool black_item = rl >= 1 && rl <= ny;  // ... whose row is the tile's own
    const int jw = wrapy(j0 - 1 + rl);
    // z queues of this chunk: colour-1 correction and porosity of its row at
    // planes k-1, k, k+1 (+ the side slot of planes k, k+1), colour-0
    // porosity and results at planes k-2, k-1, k
    VecF<V> qE0{}, qE1{}, qE2{}, qP0{}, qP1{}, qP2{}, c0{}, c1{}, c2{}, o0{}, o1{}, o2{};
    VecF<V> ab{};  // bottom faces of the colour-0 update of plane k (the top faces of colour 1, plane k-1)
    float sE1 = 0.f, sE2 = 0.f, sP1 = 0.f, sP2 = 0.f;
    for (int it = 0; it < nit; it++) {
      const int k = k0 - 1 + it, kw = wrapz(k);
      // a thread whose wait ran out neither reads the stage that never landed
      // nor stores a result from it; every thread leaves at the barrier below
      const bool landed = mbar_wait_bounded(&bar[waited % FSTAGES], (waited / FSTAGES) & 1);
      if (landed)
        confirmed = waited + 1;
      else
        abort_flag = 1;
      waited++;
      if (red_item && landed) {  // colour 0 of plane k
        const int s = (jw + kw) & 1;
        const float* E1c = sm + L.e1 + ((it + 1) % FZE) * plane1 + (rl + 1) * H + h0;  // row jw, plane k
        const float* E1p = sm + L.e1 + ((it + 2) % FZE) * plane1 + (rl + 1) * H + h0;  // plane k+1
        const float* P1c = sm + L.p1 + ((it + 1) % FZE) * plane1 + (rl + 1) * H + h0;
        const float* P1p = sm + L.p1 + ((it + 2) % FZE) * plane1 + (rl + 1) * H + h0;
        const int o = rl * H + h0;
        if (it == 0) {
          const float* E1m = sm + L.e1 + (it % FZE) * plane1 + (rl + 1) * H + h0;
          const float* P1m = sm + L.p1 + (it % FZE) * plane1 + (rl + 1) * H + h0;
          qE1 = ldv<V>(E1c);
          qP1 = ldv<V>(P1c);
          qE2 = ldv<V>(E1m);  // shifted into qE0 below
          qP2 = ldv<V>(P1m);
          sE2 = s ? E1c[V] : E1c[-1];
          sP2 = s ? P1c[V] : P1c[-1];
          qE0 = qE2;
          qP0 = qP2;
          sE1 = sE2;
          sP1 = sP2;
        } else {
          qE0 = qE1;
          qE1 = qE2;
          qP0 = qP1;
          qP1 = qP2;
          sE1 = sE2;
          sP1 = sP2;
        }
        qE2 = ldv<V>(E1p);
        qP2 = ldv<V>(P1p);
        sE2 = s ? E1p[-1] : E1p[V];  // plane k+1 has the other parity
        sP2 = s ? P1p[-1] : P1p[V];
        c0 = c1;
        c1 = c2;
        c2 = ldv<V>(sm + L.p0 + (it % FZP) * plane0 + o);
        const VecF<V> EC = ldv<V>(sm + L.e0 + (it % FZ1) * plane0 + o);
        const VecF<V> R = ldv<V>(sm + L.r0 + (it % FZ1) * plane0 + o);
        const VecF<V> XN = ldv<V>(E1c + H), XS = ldv<V>(E1c - H), PN = ldv<V>(P1c + H), PS = ldv<V>(P1c - H);
        unsigned unused = 0;
        o0 = o1;
        o1 = o2;
        o2 = dc_chunk_f<false, false>(g, K, h0, s, EC, R, c2, qE1, qP1, sE1, sP1, XN, XS, PN, PS, qE2, qE0, qP2,
                                      qP0, ab, ab, unused);
        *reinterpret_cast<VecF<V>*>(sm + L.red + (it % FZR) * planeRed + rl * P + V + h0) = o2;
        if (black_item && k >= k0 && k < k1)
          *reinterpret_cast<VecF<V>*>(A.eb[0] + pk_idx(g, h0, jw, kw)) = o2;
      }
      __syncthreads();
      if (abort_flag) {  // uniform after the barrier
        ok = false;
        break;
      }
      if (threadIdx.x == producer && it + FPRE < nit) {
        // the slots this stage overwrites were last read before the barrier
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        issue(it + FPRE);
      }
      if (it >= 2 && black_item) {  // colour 1 of plane kb = k-1, row jw
        const int kb = k - 1;
        const int s = (1 + jw + kb) & 1;
        const float* P0b = sm + L.p0 + ((it - 1) % FZP) * plane0 + rl * H + h0;
        const float* Rb = sm + L.red + ((it - 1) % FZR) * planeRed + rl * P + V + h0;
        const VecF<V> R = ldv<V>(sm + L.r1 + ((it - 1) % FZ1) * planeR1 + (rl - 1) * H + h0);
        const float px = s ? P0b[V] : P0b[-1];
        const float xx = s ? Rb[V] : Rb[-1];
        const VecF<V> PN = ldv<V>(P0b + H), PS = ldv<V>(P0b - H);
        const VecF<V> XN = ldv<V>(Rb + P), XS = ldv<V>(Rb - P);
        // top faces: the bottom faces of this chunk's colour-0 update of plane k
        VecF<V> abb;
        const VecF<V> out = dc_chunk_f<TRACK, true>(g, K, h0, s, qE0, R, qP0, o1, c1, xx, px, XN, XS, PN, PS, o2,
                                                    o0, c2, c0, ab, abb, e);
        *reinterpret_cast<VecF<V>*>(A.eb[1] + pk_idx(g, h0, jw, kb)) = out;
      }
    }
    __syncthreads();  // the next segment's first stages overwrite the rings
  }
  if (!ok) {
    // leave no copy in flight into this CTA's shared memory: wait (bounded)
    // for every stage issued and not seen to land, the one that ran out too
    if (threadIdx.x == producer) {
      for (unsigned sg = confirmed; sg < issued; sg++)
        if (sg != dropped) mbar_wait_bounded(&bar[sg % FSTAGES], (sg / FSTAGES) & 1);
      atomicOr(A.flags, (unsigned long long)PF_FLAG_FUSED_TIMEOUT);
    }
    return;
  }
  if (TRACK) block_max_atomic(e, A.err);
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
// FP32 copies of up to three FP64 arrays of n elements (n a multiple of 4,
// arrays 32-byte aligned) in one launch, four elements per thread and
// iteration: blockIdx.y selects the array.  The per-element conversion is
// k_to_float's.
struct Fields3 {
  const double* src[3];
  float* dst[3];
};
__global__ void k_to_float3(Fields3 f, long long n4) {
  pdl_begin();
  const double2* __restrict__ a = reinterpret_cast<const double2*>(f.src[blockIdx.y]);
  float4* __restrict__ b = reinterpret_cast<float4*>(f.dst[blockIdx.y]);
  for (long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x; q < n4; q += (long long)gridDim.x * blockDim.x) {
    const double2 x = a[2 * q], y = a[2 * q + 1];
    b[q] = make_float4((float)x.x, (float)x.y, (float)y.x, (float)y.y);
  }
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

// The interior planes k_lo .. k_hi of a 3D grid (k_hi < k_lo: all of them).
static dim3 grid_planes(const Geo& g, int k_lo, int k_hi) {
  dim3 grid = grid_interior(g);
  if (g.dim == 3 && k_hi >= k_lo) grid.z = k_hi - k_lo + 1;
  return grid;
}
static int plane_offset(const Geo& g, int k_lo, int k_hi) { return g.dim == 3 && k_hi >= k_lo ? k_lo - 1 : 0; }

template <typename TV>
void launch_divergence(const Geo& g, const Scal& s, const TV* uo, const TV* vo, const TV* wo, TV* div,
                       cudaStream_t st, int k_lo, int k_hi) {
  launch_pdl(k_divergence<TV>, grid_planes(g, k_lo, k_hi), dim3(BX, BY), st, g, s, uo, vo, wo, div,
             plane_offset(g, k_lo, k_hi));
}

template <typename T, typename TS>
void launch_predictor(const Geo& g, const Scal& s, const T* uo, const T* vo, const T* wo, const T* div,
                      const T* gx, const T* gy, const T* gz, const T* rinv, const T* damp, const TS* us,
                      const TS* vs, const TS* ws, TS* u, TS* v, TS* w, cudaStream_t st, int k_lo, int k_hi) {
  const dim3 grid = grid_planes(g, k_lo, k_hi);
  const int k0 = plane_offset(g, k_lo, k_hi);
  if constexpr (sizeof(T) == sizeof(double)) {
    if (g.dim == 3) {
      launch_pdl(k_predictor_fp64_3d<TS>, grid, dim3(BX, BY), st, g, s, uo, vo, wo, div, gx, gy, gz, rinv, damp, us,
                 vs, ws, u, v, w, k0);
      return;
    }
  }
  if (g.dim == 3)
    launch_pdl(k_predictor<T, TS, 3>, grid, dim3(BX, BY), st, g, s, uo, vo, wo, div, gx, gy, gz, rinv, damp, us,
               vs, ws, u, v, w, k0);
  else
    launch_pdl(k_predictor<T, TS, 2>, grid, dim3(BX, BY), st, g, s, uo, vo, wo, div, gx, gy, gz, rinv, damp, us,
               vs, ws, u, v, w, k0);
}
template void launch_predictor<double, double>(const Geo&, const Scal&, const double*, const double*,
                                               const double*, const double*, const double*, const double*,
                                               const double*, const double*, const double*, const double*,
                                               const double*, const double*, double*, double*, double*,
                                               cudaStream_t, int, int);
template void launch_predictor<float, double>(const Geo&, const Scal&, const float*, const float*, const float*,
                                              const float*, const float*, const float*, const float*,
                                              const float*, const float*, const double*, const double*,
                                              const double*, double*, double*, double*, cudaStream_t, int, int);

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
                     unsigned long long* err, const int* skip, bool early, cudaStream_t st) {
  const unsigned grid = (unsigned)((packed_items(g) + SWEEP_THREADS - 1) / SWEEP_THREADS);
#define PF_SH(D, TR, EA) \
  launch_pdl(k_sor_half<T, D, TR, EA>, grid, SWEEP_THREADS, st, g, cc, pc, po, one_minus_omega, colour, err, skip)
  if (g.dim == 3) {
    if (err)
      early ? PF_SH(3, true, true) : PF_SH(3, true, false);
    else
      early ? PF_SH(3, false, true) : PF_SH(3, false, false);
  } else {
    if (err)
      early ? PF_SH(2, true, true) : PF_SH(2, true, false);
    else
      early ? PF_SH(2, false, true) : PF_SH(2, false, false);
  }
#undef PF_SH
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
  if (g.slip) launch_pdl(k_bnd_slip<TV>, dim3((g.m + 127) / 128), dim3(128), st, g, u, v, p0, p1);
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

static DCConst dc_const(const Geo& g, const Scal& sc) {
  return make_dc_const(sc.dt, sc.dx, sc.dy, sc.dz, g.dim, sc.omega);
}

// Whether the FP32 split sweep's grid fits one wave of resident CTAs (its
// fixed operands then load before the dependency wait).
bool dc_one_wave(const Geo& g, int sms) {
  const int chunks = (g.m >> 1) / 4 + 1;
  const long long threads = (long long)chunks * g.n * (g.dim == 3 ? g.l : 1);
  const long long blocks = (threads + DC4_THREADS - 1) / DC4_THREADS;
  int per_sm = 0;
  if (g.dim == 3)
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_sor_dc4_early<3, true, 4>, DC4_THREADS, 0);
  else
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_sor_dc4_early<2, true, 4>, DC4_THREADS, 0);
  return blocks <= (long long)per_sm * sms;
}

void launch_sor_dc(const Geo& g, const Scal& sc, const float* epsc, const float* epso, const float* r, float* ec,
                   const float* eo, int colour, unsigned long long* err, const int* skip, bool early,
                   cudaStream_t st) {
  const DCConst K = dc_const(g, sc);
  // chunks of 4 slots covering h = 0 .. m/2 (the largest h of an interior cell);
  // 4 beat 2 and 8 per thread at 256^3 (1547 vs 1336 and 1508 Mcell-steps/s
  // for the step): the extra occupancy of narrower chunks does not pay for
  // their extra instructions, and 8 slots take 126 registers (two CTAs per SM)
  constexpr int V = 4;
  const int chunks = (g.m >> 1) / V + 1;
  const long long threads = (long long)chunks * g.n * (g.dim == 3 ? g.l : 1);
  const unsigned blocks = (unsigned)((threads + DC4_THREADS - 1) / DC4_THREADS);
#define PF_DC(DIMV, TR)                                                                                          \
  (early ? launch_pdl(k_sor_dc4_early<DIMV, TR, V>, dim3(blocks), dim3(DC4_THREADS), st, g, K, epsc, epso, r, ec, eo, \
                      colour, chunks, err, skip)                                                                     \
         : launch_pdl(k_sor_dc4<DIMV, TR, V>, dim3(blocks), dim3(DC4_THREADS), st, g, K, epsc, epso, r, ec, eo,       \
                      colour, chunks, err, skip))
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

static int fused_chunks(const Geo& g) { return (g.m >> 1) / FUSED_V + 1; }
static size_t fused_smem(const Geo& g, int ty) {
  return (size_t)fused_layout(ty, g.H, fused_chunks(g)).total * sizeof(float);
}

bool fused_eligible(const Geo& g) {
  return g.dim == 3 && !g.wall && g.n % 2 == 0 && g.l % 2 == 0 && fused_smem(g, 2) <= FUSED_SMEM_MAX &&
         4 * fused_chunks(g) <= FUSED_MAX_THREADS;
}

int fused_setup(const Geo& g, int ty_req, int tz_req, int sms, FusedShape& fs) {
  const int chunks = fused_chunks(g);
  // tile height: the largest whose rings fit and whose chunks fit one CTA.
  // A CTA's step is latency-bound, so more rows per step (more threads, fewer
  // steps per CTA) wins although the halo rows are updated twice: at 256^3
  // the sweep took 114, 105, 102 and 99 us with 8, 10, 11 and 12 rows.
  int ty = 0;
  for (int t = 1; t <= std::min(16, g.n); t++) {
    if (ty_req > 0 ? t != std::min(ty_req, g.n) : t < 2) continue;
    if (fused_smem(g, t) > FUSED_SMEM_MAX || (t + 2) * chunks > FUSED_MAX_THREADS) continue;
    ty = t;
  }
  if (ty == 0) return (int)cudaErrorInvalidValue;
  const size_t smem = fused_smem(g, ty);
  const int threads = ((ty + 2) * chunks + 31) / 32 * 32;  // one chunk per thread
  for (void* k : {(void*)k_sor_fused3<false>, (void*)k_sor_fused3<true>}) {
    cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return (int)e;
  }
  int per_sm = 0;
  cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_sor_fused3<true>, threads, smem);
  if (e != cudaSuccess) return (int)e;
  if (per_sm < 1) return (int)cudaErrorInvalidConfiguration;
  const int ntiles = (g.n + ty - 1) / ty;
  const long long pairs = (long long)ntiles * g.l;
  // one wave of persistent CTAs, each a contiguous run of (tile, plane) pairs
  long long per_cta = (pairs + (long long)sms * per_sm - 1) / ((long long)sms * per_sm);
  if (tz_req > 0) per_cta = std::min<long long>(per_cta, tz_req);
  fs.ty = ty;
  fs.per_cta = (int)per_cta;
  fs.threads = threads;
  fs.chunks = chunks;
  fs.ntiles = ntiles;
  fs.grid = (int)((pairs + per_cta - 1) / per_cta);
  fs.smem = smem;
  return 0;
}

void launch_sor_fused(const Geo& g, const Scal& sc, const FusedShape& fs, const float* const eps[2],
                      const float* const r[2], const float* const ea[2], float* const eb[2],
                      unsigned long long* err, unsigned long long* flags, const int* skip, cudaStream_t st) {
  FusedArgs A;
  for (int c = 0; c < 2; c++) {
    A.eps[c] = eps[c];
    A.r[c] = r[c];
    A.ea[c] = ea[c];
    A.eb[c] = eb[c];
  }
  A.err = err;
  A.flags = flags;
  A.skip = skip;
  A.drop_stage = fs.drop_stage;
  const DCConst K = dc_const(g, sc);
  if (err)
    launch_pdl_smem(k_sor_fused3<true>, dim3(fs.grid), dim3(fs.threads), fs.smem, st, g, K, A, fs.chunks, fs.ty,
                    fs.ntiles, fs.per_cta);
  else
    launch_pdl_smem(k_sor_fused3<false>, dim3(fs.grid), dim3(fs.threads), fs.smem, st, g, K, A, fs.chunks, fs.ty,
                    fs.ntiles, fs.per_cta);
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
void launch_to_float3(const double* const* src, float* const* dst, int nf, long long n, cudaStream_t st) {
  Fields3 f{};
  for (int i = 0; i < nf; i++) {
    f.src[i] = src[i];
    f.dst[i] = dst[i];
  }
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const long long n4 = n / 4;
  const long long want = (n4 + 255) / 256;
  const unsigned blocks = (unsigned)std::max(1LL, std::min<long long>(want, 8LL * std::max(1, sms)));
  launch_pdl(k_to_float3, dim3(blocks, nf), dim3(256), st, f, n4);
}
void launch_to_double(const float* src, double* dst, long long n, cudaStream_t st) {
  k_to_double<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(src, dst, n);
}

void launch_scatter_nat(const Geo& g, const double* stage, double* dst, cudaStream_t st) {
  k_scatter_nat<<<grid_all(g), dim3(BX, BY), 0, st>>>(g, stage, dst);
}
void launch_scatter_nat_planes(const Geo& g, const double* stage, double* dst, int k_lo, int k_hi,
                               cudaStream_t st) {
  Geo gp = g;  // the planes k_lo .. k_hi of both layouts, addressed from plane k_lo
  gp.Z = k_hi - k_lo + 1;
  const double* src = stage + (idx_t)k_lo * (g.m + 2) * (g.n + 2);
  k_scatter_nat<<<grid_all(gp), dim3(BX, BY), 0, st>>>(gp, src, dst + (idx_t)k_lo * g.X * g.Y);
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
                                      cudaStream_t, int, int);                                               \
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
                                    unsigned long long*, const int*, bool, cudaStream_t);                    \
  template void launch_p_halo<TV>(const Geo&, TV*, TV*, const int*, cudaStream_t);
PF_INST_V(double)
PF_INST_V(float)
#undef PF_INST_V

}  // namespace pf
