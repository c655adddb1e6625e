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

namespace pf {

namespace {

constexpr int BX = 32, BY = 8;

inline dim3 grid_interior(const Geo& g) {
  return dim3((g.m + BX - 1) / BX, (g.n + BY - 1) / BY, g.dim == 3 ? g.l : 1);
}
inline dim3 grid_all(const Geo& g) {
  return dim3((g.m + 2 + BX - 1) / BX, (g.n + 2 + BY - 1) / BY, g.Z);
}

__device__ __forceinline__ unsigned long long abs_bits(double x) {
  return (unsigned long long)__double_as_longlong(x) & 0x7fffffffffffffffULL;
}
__device__ __forceinline__ unsigned long long abs_bits(float x) {
  // widen so one accumulator type serves both precisions; |x| as double
  // keeps the ordering of the float magnitudes.
  return abs_bits((double)x);
}

// Block-wide max of non-negative IEEE bit patterns (integer order == value
// order for non-negative doubles; NaN patterns sort above +Inf), then one
// atomicMax per block.  Order independent, hence deterministic.
__device__ __forceinline__ void block_max_atomic(unsigned long long v, unsigned long long* out) {
  __shared__ unsigned long long red[32];
  for (int o = 16; o > 0; o >>= 1) {
    unsigned long long w = __shfl_xor_sync(0xffffffffu, v, o);
    v = w > v ? w : v;
  }
  const int tid = threadIdx.x + blockDim.x * (threadIdx.y + blockDim.y * threadIdx.z);
  const int nthr = blockDim.x * blockDim.y * blockDim.z;
  const int lane = tid & 31, warp = tid >> 5;
  if (lane == 0) red[warp] = v;
  __syncthreads();
  if (warp == 0) {
    v = (lane < (nthr + 31) / 32) ? red[lane] : 0ULL;
    for (int o = 16; o > 0; o >>= 1) {
      unsigned long long w = __shfl_xor_sync(0xffffffffu, v, o);
      v = w > v ? w : v;
    }
    if (lane == 0 && v) atomicMax(out, v);
  }
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
  const long long q = nat_idx(g, i, j, k);
  const long long X = g.X, XY = (long long)g.X * g.Y;
  const double e = po[q];
  gx[q] = (po[q + 1] - po[q - 1]) * (0.5 / s.dx);
  gy[q] = (po[q + X] - po[q - X]) * (0.5 / s.dy);
  if (g.dim == 3) gz[q] = (po[q + XY] - po[q - XY]) * (0.5 / s.dz);
  rinv[q] = s.dt / e;
  damp[q] = s.nonslip ? s.xnue * s.dt * 32.0 * e * (1.0 - e) * (1.0 - e) / (s.thickness * s.thickness) : 0.0;
}

// SOR operator of both colours, with boundrary_matrix applied, normalised
// by omega/ap.  Face coefficients follow the reference formula
// dt*max(small,(eps_a+eps_b)*0.5)/h/h with small = 1e-6.
__global__ void k_setup_coef(Geo g, Scal s, const double* __restrict__ po, Coef<double> c0, Coef<double> c1) {
  const int i = blockIdx.x * BX + threadIdx.x + 1;
  const int j = blockIdx.y * BY + threadIdx.y + 1;
  const int k = (g.dim == 3) ? blockIdx.z + 1 : 0;
  if (i > g.m || j > g.n) return;
  const long long q = nat_idx(g, i, j, k);
  const long long X = g.X, XY = (long long)g.X * g.Y;
  const double small = 1.e-6, dt = s.dt;
  const double e = po[q];
  double a[6];
  a[0] = dt * fmax(small, (po[q + 1] + e) * 0.5) / s.dx / s.dx;
  a[1] = dt * fmax(small, (e + po[q - 1]) * 0.5) / s.dx / s.dx;
  a[2] = dt * fmax(small, (po[q + X] + e) * 0.5) / s.dy / s.dy;
  a[3] = dt * fmax(small, (e + po[q - X]) * 0.5) / s.dy / s.dy;
  double ap = -a[0] - a[1] - a[2] - a[3];
  if (g.dim == 3) {
    a[4] = dt * fmax(small, (po[q + XY] + e) * 0.5) / s.dz / s.dz;
    a[5] = dt * fmax(small, (e + po[q - XY]) * 0.5) / s.dz / s.dz;
    ap = ap - a[4] - a[5];
  } else {
    a[4] = a[5] = 0.0;
  }
  // boundrary_matrix: inlet row i=1 (Neumann), outlet row i=m (Dirichlet p(m+1)).
  if (i == 1) {
    a[0] = a[0] + a[1];
    a[1] = 0.0;
  }
  double oadd = 0.0;
  if (i == g.m) {
    oadd = a[0] * s.outlet_pressure;
    for (int d = 0; d < 6; d++) a[d] = 0.0;
  }
  const double wap = s.omega / ap;
  const int c = colour_of(g, i, j, k);
  const Coef<double> C = c ? c1 : c0;
  const long long r = pk_idx(g, i >> 1, j, k);
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
  const int i = blockIdx.x * BX + threadIdx.x + 1;
  const int j = blockIdx.y * BY + threadIdx.y + 1;
  const int k = (g.dim == 3) ? blockIdx.z + 1 : 0;
  if (i > g.m || j > g.n) return;
  const long long q = nat_idx(g, i, j, k);
  const long long X = g.X, XY = (long long)g.X * g.Y;
  const T hx = (T)(0.5 / s.dx);
  if (g.dim == 3) {
    const T hy = (T)(0.5 / s.dy), hz = (T)(0.5 / s.dz);
    T d = (uo[q + 1] - uo[q - 1]) * hx;
    d = fma(vo[q + X] - vo[q - X], hy, d);
    d = fma(wo[q + XY] - wo[q - XY], hz, d);
    div[q] = d;
  } else {
    div[q] = fma(vo[q + X] - vo[q - X], hx, (uo[q + 1] - uo[q - 1]) * hx);
  }
}

// Predictor: explicit Euler of the porosity-weighted momentum equation.
// Also copies the face ghosts of the old fields into the new ones, so the
// RHS sees the previous step's ghosts exactly as the reference does.
template <typename T, int DIM>
__global__ void __launch_bounds__(BX* BY) k_predictor(Geo g, Scal s, const T* __restrict__ uo,
                                                      const T* __restrict__ vo, const T* __restrict__ wo,
                                                      const T* __restrict__ div, const T* __restrict__ gxa,
                                                      const T* __restrict__ gya, const T* __restrict__ gza,
                                                      const T* __restrict__ rinva, const T* __restrict__ dampa,
                                                      T* __restrict__ u, T* __restrict__ v, T* __restrict__ w) {
  const int i = blockIdx.x * BX + threadIdx.x + 1;
  const int j = blockIdx.y * BY + threadIdx.y + 1;
  const int k = (DIM == 3) ? blockIdx.z + 1 : 0;
  if (i > g.m || j > g.n) return;
  const long long q = nat_idx(g, i, j, k);
  const long long X = g.X, XY = (long long)g.X * g.Y;
  const T hx = (T)(0.5 / s.dx), hy = (T)(0.5 / s.dy);
  const T ix2 = (T)(1.0 / (s.dx * s.dx)), iy2 = (T)(1.0 / (s.dy * s.dy));
  const T dt = (T)s.dt, nu = (T)s.xnue, lam = (T)s.xlambda;
  const T dtnu = (T)(s.dt * s.xnue), dtnl = (T)(s.dt * (s.xnue + s.xlambda));
  const T two = (T)2;
  // div neighbours with the periodic wrap of the y (and z) ghost rows
  const long long jn = (j == g.n) ? q - (long long)(g.n - 1) * X : q + X;
  const long long js = (j == 1) ? q + (long long)(g.n - 1) * X : q - X;
  const T dc = div[q], dE = div[q + 1], dW = div[q - 1], dN = div[jn], dS = div[js];
  const T gx = gxa[q], gy = gya[q], rv = rinva[q], dp = dampa[q];

  const T uc = uo[q], ue = uo[q + 1], uw = uo[q - 1], un = uo[q + X], us = uo[q - X];
  const T vc = vo[q], ve = vo[q + 1], vw = vo[q - 1], vn = vo[q + X], vs = vo[q - X];
  const T dux = (ue - uw) * hx, duy = (un - us) * hy;
  const T dvx = (ve - vw) * hx, dvy = (vn - vs) * hy;
  const T lux = fma(-two, uc, ue + uw), luy = fma(-two, uc, un + us);
  const T lvx = fma(-two, vc, ve + vw), lvy = fma(-two, vc, vn + vs);
  if (DIM == 2) {
    // u
    T conv = fma(vc, duy, uc * dux);
    T lap = fma(luy, iy2, lux * ix2);
    T por = fma(duy + dvx, gy, (dux + dux) * gx) * nu;
    por = fma(lam * dc, gx, por);
    T t = fma(-dt, conv, uc);
    t = fma(dtnu, lap, t);
    t = fma(dtnl, (dE - dW) * hx, t);
    t = fma(rv, por, t);
    u[q] = fma(-uc, dp * ix2, t);
    // v (the reference damps v with (thickness*dx)^2 as well, ibm_2d:254)
    conv = fma(vc, dvy, uc * dvx);
    lap = fma(lvy, iy2, lvx * ix2);
    por = fma(dvy + dvy, gy, (dvx + duy) * gx) * nu;
    por = fma(lam * dc, gy, por);
    t = fma(-dt, conv, vc);
    t = fma(dtnu, lap, t);
    t = fma(dtnl, (dN - dS) * hy, t);
    t = fma(rv, por, t);
    v[q] = fma(-vc, dp * ix2, t);
  } else {
    const T hz = (T)(0.5 / s.dz), iz2 = (T)(1.0 / (s.dz * s.dz));
    const long long kt = (k == g.l) ? q - (long long)(g.l - 1) * XY : q + XY;
    const long long kb = (k == 1) ? q + (long long)(g.l - 1) * XY : q - XY;
    const T dT = div[kt], dB = div[kb];
    const T gz = gza[q];
    const T ut = uo[q + XY], ub = uo[q - XY], vt = vo[q + XY], vb = vo[q - XY];
    const T wc = wo[q], we = wo[q + 1], ww = wo[q - 1], wn = wo[q + X], ws = wo[q - X];
    const T wt = wo[q + XY], wb = wo[q - XY];
    const T duz = (ut - ub) * hz, dvz = (vt - vb) * hz;
    const T dwx = (we - ww) * hx, dwy = (wn - ws) * hy, dwz = (wt - wb) * hz;
    const T luz = fma(-two, uc, ut + ub), lvz = fma(-two, vc, vt + vb);
    const T lwx = fma(-two, wc, we + ww), lwy = fma(-two, wc, wn + ws), lwz = fma(-two, wc, wt + wb);
    // u
    T conv = fma(wc, duz, fma(vc, duy, uc * dux));
    T lap = fma(luz, iz2, fma(luy, iy2, lux * ix2));
    T por = fma(duz + dwx, gz, fma(duy + dvx, gy, (dux + dux) * gx)) * nu;
    por = fma(lam * dc, gx, por);
    T t = fma(-dt, conv, uc);
    t = fma(dtnu, lap, t);
    t = fma(dtnl, (dE - dW) * hx, t);
    t = fma(rv, por, t);
    u[q] = fma(-uc, dp * ix2, t);
    // v
    conv = fma(wc, dvz, fma(vc, dvy, uc * dvx));
    lap = fma(lvz, iz2, fma(lvy, iy2, lvx * ix2));
    por = fma(dvz + dwy, gz, fma(dvy + dvy, gy, (dvx + duy) * gx)) * nu;
    por = fma(lam * dc, gy, por);
    t = fma(-dt, conv, vc);
    t = fma(dtnu, lap, t);
    t = fma(dtnl, (dN - dS) * hy, t);
    t = fma(rv, por, t);
    v[q] = fma(-vc, dp * iy2, t);
    // w
    conv = fma(wc, dwz, fma(vc, dwy, uc * dwx));
    lap = fma(lwz, iz2, fma(lwy, iy2, lwx * ix2));
    por = fma(dwz + dwz, gz, fma(dwy + dvz, gy, (dwx + duz) * gx)) * nu;
    por = fma(lam * dc, gz, por);
    t = fma(-dt, conv, wc);
    t = fma(dtnu, lap, t);
    t = fma(dtnl, (dT - dB) * hz, t);
    t = fma(rv, por, t);
    w[q] = fma(-wc, dp * iz2, t);
  }
  // face ghosts of the old fields carry over (the reference's u keeps them)
  auto keep = [&](long long r) {
    u[r] = uo[r];
    v[r] = vo[r];
    if (DIM == 3) w[r] = wo[r];
  };
  if (i == 1) keep(q - 1);
  if (i == g.m) keep(q + 1);
  if (j == 1) keep(q - X);
  if (j == g.n) keep(q + X);
  if (DIM == 3) {
    if (k == 1) keep(q - XY);
    if (k == g.l) keep(q + XY);
  }
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
  const int i = blockIdx.x * BX + threadIdx.x + 1;
  const int j = blockIdx.y * BY + threadIdx.y + 1;
  const int k = (DIM == 3) ? blockIdx.z + 1 : 0;
  if (i > g.m || j > g.n) return;
  const long long q = nat_idx(g, i, j, k);
  const long long X = g.X, XY = (long long)g.X * g.Y;
  const double hx = 0.5 / s.dx, hy = 0.5 / s.dy;
  double sd = ((double)u[q + 1] - (double)u[q - 1]) * hx;
  sd = fma((double)v[q + X] - (double)v[q - X], hy, sd);
  double sg = gxa[q] * (double)u[q];
  sg = fma(gya[q], (double)v[q], sg);
  if (DIM == 3) {
    sd = fma((double)w[q + XY] - (double)w[q - XY], 0.5 / s.dz, sd);
    sg = fma(gza[q], (double)w[q], sg);
  }
  const double bb = s.density * fma(po[q], sd, sg);
  const int c = colour_of(g, i, j, k);
  const Coef<double> C = c ? c1 : c0;
  const long long r = pk_idx(g, i >> 1, j, k);
  C.bbn[r] = (bb + C.oadd[r]) * C.wap[r];
}

// One red-black half-sweep of colour `colour`, in place:
//   p = (1-omega) p + bbn - sum_nb a_nb p_nb     (all neighbours: other colour)
// which is the reference's
//   p = (bb - sum a_nb p_old_nb)/ap*omega + p_old*(1-omega)
// because no neighbour of a cell changes during its own colour's sweep.
// With TRACK the block max of |p_new - p_old| goes to *err.
template <typename T, int DIM, bool TRACK>
__global__ void __launch_bounds__(BX* BY) k_sor_half(Geo g, Coef<T> C, T* __restrict__ pc,
                                                     const T* __restrict__ po, T omw, int colour,
                                                     unsigned long long* __restrict__ err,
                                                     const int* __restrict__ skip) {
  if (skip && *skip) return;  // uniform over the grid: defect correction converged
  const int h = blockIdx.x * BX + threadIdx.x;
  const int j = blockIdx.y * BY + threadIdx.y + 1;
  const int k = (DIM == 3) ? blockIdx.z + 1 : 0;
  const int s = (colour + j + (DIM == 3 ? k : 1)) & 1;
  const int i = 2 * h + s;
  unsigned long long e = 0;
  if (j <= g.n && i >= 1 && i <= g.m) {
    const long long H = g.H, HY = (long long)g.H * g.Y;
    const long long q = pk_idx(g, h, j, k);
    const long long qn = (j == g.n) ? pk_idx(g, h, g.jn_n, k) : q + H;
    const long long qs = (j == 1) ? pk_idx(g, h, g.js_1, k) : q - H;
    const T pold = pc[q];
    T t = C.bbn[q];
    t = fma(-C.a[0][q], po[q + s], t);
    t = fma(-C.a[1][q], po[q - 1 + s], t);
    t = fma(-C.a[2][q], po[qn], t);
    t = fma(-C.a[3][q], po[qs], t);
    if (DIM == 3) {
      const long long qt = (k == g.l) ? pk_idx(g, h, j, g.kt_l) : q + HY;
      const long long qb = (k == 1) ? pk_idx(g, h, j, g.kb_1) : q - HY;
      t = fma(-C.a[4][q], po[qt], t);
      t = fma(-C.a[5][q], po[qb], t);
    }
    const T pnew = fma(omw, pold, t);
    pc[q] = pnew;
    if (TRACK) e = abs_bits(pnew - pold);
  }
  if (TRACK) block_max_atomic(e, err);
}

__device__ __forceinline__ long long pk_of(const Geo& g, int i, int j, int k, int& c) {
  c = colour_of(g, i, j, k);
  return pk_idx(g, i >> 1, j, k);
}

// Periodic ghost rows (and planes) of p for interior i, as the reference
// refreshes them before each half-sweep (ibm_2d:322-327; ibm_3d:463-480).
template <typename T>
__global__ void k_p_halo(Geo g, T* p0, T* p1, const int* __restrict__ skip) {
  if (skip && *skip) return;
  const int i = blockIdx.x * blockDim.x + threadIdx.x + 1;
  const int a = blockIdx.y + 1;  // k for the y rows (3D), j for the z planes
  if (i > g.m) return;
  T* P[2] = {p0, p1};
  int cs, cd;
  if (g.dim == 2) {
    if (a != 1) return;
    long long s0 = pk_of(g, i, g.n, 0, cs), d0 = pk_of(g, i, 0, 0, cd);
    P[cd][d0] = P[cs][s0];
    s0 = pk_of(g, i, 1, 0, cs);
    d0 = pk_of(g, i, g.n + 1, 0, cd);
    P[cd][d0] = P[cs][s0];
    return;
  }
  if (blockIdx.z == 0) {  // y rows, k = a in 1..l
    if (a > g.l) return;
    long long s0 = pk_of(g, i, g.n, a, cs), d0 = pk_of(g, i, 0, a, cd);
    P[cd][d0] = P[cs][s0];
    s0 = pk_of(g, i, 1, a, cs);
    d0 = pk_of(g, i, g.n + 1, a, cd);
    P[cd][d0] = P[cs][s0];
  } else {  // z planes, j = a in 1..n
    if (a > g.n) return;
    long long s0 = pk_of(g, i, a, g.l, cs), d0 = pk_of(g, i, a, 0, cd);
    P[cd][d0] = P[cs][s0];
    s0 = pk_of(g, i, a, 1, cs);
    d0 = pk_of(g, i, a, g.l + 1, cd);
    P[cd][d0] = P[cs][s0];
  }
}

// Projection u -= dt/rho * (p(i+1)-p(i-1))/(2dx), likewise v and w.
template <typename T, int DIM>
__global__ void k_projection(Geo g, Scal s, const double* __restrict__ p0, const double* __restrict__ p1, T* u,
                             T* v, T* w) {
  const int i = blockIdx.x * BX + threadIdx.x + 1;
  const int j = blockIdx.y * BY + threadIdx.y + 1;
  const int k = (DIM == 3) ? blockIdx.z + 1 : 0;
  if (i > g.m || j > g.n) return;
  const long long q = nat_idx(g, i, j, k);
  const int c = colour_of(g, i, j, k);
  const double* P = c ? p0 : p1;  // every neighbour has the other colour
  const long long H = g.H, HY = (long long)g.H * g.Y;
  const long long r = pk_idx(g, i >> 1, j, k);
  const int sx = i & 1;
  const double cdt = s.dt / s.density;
  u[q] = fma(-(T)(cdt * 0.5 / s.dx), (T)(P[r + sx] - P[r - 1 + sx]), u[q]);
  v[q] = fma(-(T)(cdt * 0.5 / s.dy), (T)(P[r + H] - P[r - H]), v[q]);
  if (DIM == 3) w[q] = fma(-(T)(cdt * 0.5 / s.dz), (T)(P[r + HY] - P[r - HY]), w[q]);
}

template <typename T>
__device__ __forceinline__ T& pref(const Geo& g, T* p0, T* p1, int i, int j, int k) {
  int c;
  long long r = pk_of(g, i, j, k, c);
  return c ? p1[r] : p0[r];
}

// boundary, x faces: inflow at i=1 and its ghost, outflow copy at m+1.
template <typename T>
__global__ void k_bnd_x(Geo g, Scal s, T* u, T* v, T* w, double* p0, double* p1) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x + 1;
  const int k = (g.dim == 3) ? blockIdx.y + 1 : 0;
  if (j > g.n) return;
  const long long q1 = nat_idx(g, 1, j, k), q0 = q1 - 1;
  u[q1] = (T)s.inlet_u;
  v[q1] = (T)s.inlet_v;
  u[q0] = u[q1];
  v[q0] = v[q1];
  if (g.dim == 3) {
    w[q1] = (T)0;
    w[q0] = w[q1];
  }
  pref(g, p0, p1, 0, j, k) = pref(g, p0, p1, 2, j, k);
  const long long qm = nat_idx(g, g.m + 1, j, k);
  u[qm] = u[qm - 2];
  v[qm] = v[qm - 2];
  if (g.dim == 3) w[qm] = w[qm - 2];
  pref(g, p0, p1, g.m + 1, j, k) = s.outlet_pressure;
}

// boundary, y faces: periodic ghost rows over i = 0..m+1 (and k = 0..l+1).
template <typename T>
__global__ void k_bnd_y(Geo g, T* u, T* v, T* w, double* p0, double* p1) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int k = blockIdx.y;  // 0 in 2D, 0..l+1 in 3D
  if (i > g.m + 1) return;
  const long long a = nat_idx(g, i, 0, k), b = nat_idx(g, i, g.n, k);
  const long long c = nat_idx(g, i, g.n + 1, k), d = nat_idx(g, i, 1, k);
  u[a] = u[b];
  v[a] = v[b];
  u[c] = u[d];
  v[c] = v[d];
  if (g.dim == 3) {
    w[a] = w[b];
    w[c] = w[d];
  }
  pref(g, p0, p1, i, 0, k) = pref(g, p0, p1, i, g.n, k);
  pref(g, p0, p1, i, g.n + 1, k) = pref(g, p0, p1, i, 1, k);
}

// boundary, z faces (3D): periodic ghost planes over i = 0..m+1, j = 0..n+1.
template <typename T>
__global__ void k_bnd_z(Geo g, T* u, T* v, T* w, double* p0, double* p1) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = blockIdx.y;
  if (i > g.m + 1) return;
  const long long a = nat_idx(g, i, j, 0), b = nat_idx(g, i, j, g.l);
  const long long c = nat_idx(g, i, j, g.l + 1), d = nat_idx(g, i, j, 1);
  u[a] = u[b];
  v[a] = v[b];
  w[a] = w[b];
  u[c] = u[d];
  v[c] = v[d];
  w[c] = w[d];
  pref(g, p0, p1, i, j, 0) = pref(g, p0, p1, i, j, g.l);
  pref(g, p0, p1, i, j, g.l + 1) = pref(g, p0, p1, i, j, 1);
}

template <typename T>
__global__ void k_initial(Geo g, Scal s, T* u, T* v, T* w, double* p0, double* p1) {
  const int i = blockIdx.x * BX + threadIdx.x + 1;
  const int j = blockIdx.y * BY + threadIdx.y + 1;
  const int k = (g.dim == 3) ? blockIdx.z + 1 : 0;
  if (i > g.m || j > g.n) return;
  const long long q = nat_idx(g, i, j, k);
  u[q] = (T)s.init_u;
  v[q] = (T)s.init_v;
  if (g.dim == 3) w[q] = (T)0;
  pref(g, p0, p1, i, j, k) = s.outlet_pressure;
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
    const long long q = nat_idx(g, i, j, k);
    const long long X = g.X, XY = (long long)g.X * g.Y;
    double sd = ((double)u[q + 1] - (double)u[q - 1]) * (0.5 / s.dx);
    sd = fma((double)v[q + X] - (double)v[q - X], 0.5 / s.dy, sd);
    double sg = gxa[q] * (double)u[q];
    sg = fma(gya[q], (double)v[q], sg);
    if (g.dim == 3) {
      sd = fma((double)w[q + XY] - (double)w[q - XY], 0.5 / s.dz, sd);
      sg = fma(gza[q], (double)w[q], sg);
    }
    e = abs_bits(fma(po[q], sd, sg));
  }
  block_max_atomic(e, out);
}

// staging <-> layouts ---------------------------------------------------
__global__ void k_scatter_nat(Geo g, const double* __restrict__ st, double* __restrict__ dst) {
  const int i = blockIdx.x * BX + threadIdx.x;
  const int j = blockIdx.y * BY + threadIdx.y;
  const int k = blockIdx.z;
  if (i > g.m + 1 || j > g.n + 1) return;
  const long long d = (long long)i + (long long)(g.m + 2) * ((long long)j + (long long)(g.n + 2) * k);
  dst[nat_idx(g, i, j, k)] = st[d];
}
__global__ void k_scatter_pk(Geo g, const double* __restrict__ st, double* p0, double* p1) {
  const int i = blockIdx.x * BX + threadIdx.x;
  const int j = blockIdx.y * BY + threadIdx.y;
  const int k = blockIdx.z;
  if (i > g.m + 1 || j > g.n + 1) return;
  const long long d = (long long)i + (long long)(g.m + 2) * ((long long)j + (long long)(g.n + 2) * k);
  pref(g, p0, p1, i, j, k) = st[d];
}
__global__ void k_gather_pk(Geo g, const double* p0, const double* p1, double* __restrict__ st) {
  const int i = blockIdx.x * BX + threadIdx.x;
  const int j = blockIdx.y * BY + threadIdx.y;
  const int k = blockIdx.z;
  if (i > g.m + 1 || j > g.n + 1) return;
  const long long d = (long long)i + (long long)(g.m + 2) * ((long long)j + (long long)(g.n + 2) * k);
  int c;
  const long long r = pk_of(g, i, j, k, c);
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
__global__ void __launch_bounds__(BX* BY) k_residual(Geo g, Coef<double> C, const double* __restrict__ pc,
                                                     const double* __restrict__ po, double omega, int colour,
                                                     float* __restrict__ rf, float* __restrict__ ec,
                                                     unsigned long long* __restrict__ rmax,
                                                     const int* __restrict__ skip) {
  if (skip && *skip) return;
  const int h = blockIdx.x * BX + threadIdx.x;
  const int j = blockIdx.y * BY + threadIdx.y + 1;
  const int k = (DIM == 3) ? blockIdx.z + 1 : 0;
  const int s = (colour + j + (DIM == 3 ? k : 1)) & 1;
  const int i = 2 * h + s;
  unsigned long long e = 0;
  if (j <= g.n && i >= 1 && i <= g.m) {
    const long long H = g.H, HY = (long long)g.H * g.Y;
    const long long q = pk_idx(g, h, j, k);
    const long long qn = (j == g.n) ? pk_idx(g, h, g.jn_n, k) : q + H;
    const long long qs = (j == 1) ? pk_idx(g, h, g.js_1, k) : q - H;
    double t = C.bbn[q];
    t = fma(-C.a[0][q], po[q + s], t);
    t = fma(-C.a[1][q], po[q - 1 + s], t);
    t = fma(-C.a[2][q], po[qn], t);
    t = fma(-C.a[3][q], po[qs], t);
    if (DIM == 3) {
      const long long qt = (k == g.l) ? pk_idx(g, h, j, g.kt_l) : q + HY;
      const long long qb = (k == 1) ? pk_idx(g, h, j, g.kb_1) : q - HY;
      t = fma(-C.a[4][q], po[qt], t);
      t = fma(-C.a[5][q], po[qb], t);
    }
    t = fma(-omega, pc[q], t);
    rf[q] = (float)t;
    ec[q] = 0.0f;
    e = abs_bits(t);
  }
  block_max_atomic(e, rmax);
}

// FP32 correction sweep with the operator rebuilt on the fly from the FP32
// porosity (packed by colour, ghosts included), so a half-sweep streams only
// porosity, r and e (24 bytes per update) instead of six stored
// coefficients.  Same operator as k_setup_coef up to FP32 rounding:
//   a_f = dt/h^2 * max(small, (eps_a+eps_b)/2), ap = -sum a_f (before the
//   inlet/outlet edits), inlet: a_e += a_w, a_w = 0; outlet: all a_f = 0,
//   e = (1-w) e + r - (w/ap) sum a_f e_f.
struct DCConst {
  float kx, ky, kz;  // dt/dx^2 etc.
  float small, omega, omw;
};

template <int DIM, bool TRACK>
__global__ void __launch_bounds__(BX* BY) k_sor_dc(Geo g, DCConst K, const float* __restrict__ epsc,
                                                   const float* __restrict__ epso, const float* __restrict__ r,
                                                   float* __restrict__ ec, const float* __restrict__ eo, int colour,
                                                   unsigned long long* __restrict__ err, const int* __restrict__ skip) {
  if (skip && *skip) return;
  const int h = blockIdx.x * BX + threadIdx.x;
  const int j = blockIdx.y * BY + threadIdx.y + 1;
  const int k = (DIM == 3) ? blockIdx.z + 1 : 0;
  const int s = (colour + j + (DIM == 3 ? k : 1)) & 1;
  const int i = 2 * h + s;
  unsigned long long e = 0;
  if (j <= g.n && i >= 1 && i <= g.m) {
    const long long H = g.H, HY = (long long)g.H * g.Y;
    const long long q = pk_idx(g, h, j, k);
    const long long qn = (j == g.n) ? pk_idx(g, h, g.jn_n, k) : q + H;
    const long long qs = (j == 1) ? pk_idx(g, h, g.js_1, k) : q - H;
    const float pc = epsc[q];
    float ae = K.kx * fmaxf(K.small, (epso[q + s] + pc) * 0.5f);
    float aw = K.kx * fmaxf(K.small, (pc + epso[q - 1 + s]) * 0.5f);
    const float an = K.ky * fmaxf(K.small, (epso[q + H] + pc) * 0.5f);
    const float as = K.ky * fmaxf(K.small, (pc + epso[q - H]) * 0.5f);
    float at = 0.f, ab = 0.f;
    if (DIM == 3) {
      at = K.kz * fmaxf(K.small, (epso[q + HY] + pc) * 0.5f);
      ab = K.kz * fmaxf(K.small, (pc + epso[q - HY]) * 0.5f);
    }
    const float ap = -ae - aw - an - as - at - ab;
    const float wap = K.omega / ap;
    const float eold = ec[q];
    float enew = fmaf(K.omw, eold, r[q]);
    if (i != g.m) {
      if (i == 1) {
        ae += aw;
        aw = 0.f;
      }
      float t = ae * eo[q + s];
      t = fmaf(aw, eo[q - 1 + s], t);
      t = fmaf(an, eo[qn], t);
      t = fmaf(as, eo[qs], t);
      if (DIM == 3) {
        const long long qt = (k == g.l) ? pk_idx(g, h, j, g.kt_l) : q + HY;
        const long long qb = (k == 1) ? pk_idx(g, h, j, g.kb_1) : q - HY;
        t = fmaf(at, eo[qt], t);
        t = fmaf(ab, eo[qb], t);
      }
      enew = fmaf(-wap, t, enew);
    }
    ec[q] = enew;
    if (TRACK) e = abs_bits(enew - eold);
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
  const long long r = pk_of(g, i, j, k, c);
  (c ? e1 : e0)[r] = (float)po[nat_idx(g, i, j, k)];
}

// p += e over the interior cells of both colours (FP64 accumulation).
template <int DIM>
__global__ void k_accumulate(Geo g, double* __restrict__ p0, double* __restrict__ p1, const float* __restrict__ e0,
                             const float* __restrict__ e1, const int* __restrict__ skip) {
  if (skip && *skip) return;
  const int h = blockIdx.x * BX + threadIdx.x;
  const int j = blockIdx.y * BY + threadIdx.y + 1;
  const int colour = blockIdx.z & 1;
  const int k = (DIM == 3) ? (blockIdx.z >> 1) + 1 : 0;
  const int s = (colour + j + (DIM == 3 ? k : 1)) & 1;
  const int i = 2 * h + s;
  if (j > g.n || i < 1 || i > g.m) return;
  const long long q = pk_idx(g, h, j, k);
  if (colour)
    p1[q] += (double)e1[q];
  else
    p0[q] += (double)e0[q];
}

// Stop the remaining passes of this step once max|r|/w <= tol.
__global__ void k_dc_check(const unsigned long long* rmax, double tol_w, int* skip) {
  const double r = __longlong_as_double((long long)*rmax);
  if (r <= tol_w) *skip = 1;
}

__global__ void k_coef_to_float(long long n, Coef<double> c, Coef<float> cf, int nd) {
  const long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= n) return;
  for (int d = 0; d < nd; d++) cf.a[d][q] = (float)c.a[d][q];
}

__global__ void k_to_float(const double* __restrict__ a, float* __restrict__ b, long long n) {
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
  k_divergence<TV><<<grid_interior(g), dim3(BX, BY), 0, st>>>(g, s, uo, vo, wo, div);
}

template <typename TV>
void launch_predictor(const Geo& g, const Scal& s, const TV* uo, const TV* vo, const TV* wo, const TV* div,
                      const TV* gx, const TV* gy, const TV* gz, const TV* rinv, const TV* damp, TV* u, TV* v,
                      TV* w, cudaStream_t st) {
  if (g.dim == 3)
    k_predictor<TV, 3><<<grid_interior(g), dim3(BX, BY), 0, st>>>(g, s, uo, vo, wo, div, gx, gy, gz, rinv,
                                                                  damp, u, v, w);
  else
    k_predictor<TV, 2><<<grid_interior(g), dim3(BX, BY), 0, st>>>(g, s, uo, vo, wo, div, gx, gy, gz, rinv,
                                                                  damp, u, v, w);
}

template <typename TV>
void launch_rhs(const Geo& g, const Scal& s, const TV* u, const TV* v, const TV* w, const double* poro,
                const double* gx, const double* gy, const double* gz, Coef<double> c0, Coef<double> c1,
                cudaStream_t st) {
  if (g.dim == 3)
    k_rhs<TV, 3><<<grid_interior(g), dim3(BX, BY), 0, st>>>(g, s, u, v, w, poro, gx, gy, gz, c0, c1);
  else
    k_rhs<TV, 2><<<grid_interior(g), dim3(BX, BY), 0, st>>>(g, s, u, v, w, poro, gx, gy, gz, c0, c1);
}

static dim3 grid_packed(const Geo& g) {
  const int nh = (g.m + 1) / 2 + 1;
  return dim3((nh + BX - 1) / BX, (g.n + BY - 1) / BY, g.dim == 3 ? g.l : 1);
}

template <typename T>
void launch_sor_half(const Geo& g, const Coef<T>& cc, T* pc, const T* po, T one_minus_omega, int colour,
                     unsigned long long* err, const int* skip, cudaStream_t st) {
  const dim3 grid = grid_packed(g);
  if (g.dim == 3) {
    if (err)
      k_sor_half<T, 3, true><<<grid, dim3(BX, BY), 0, st>>>(g, cc, pc, po, one_minus_omega, colour, err, skip);
    else
      k_sor_half<T, 3, false><<<grid, dim3(BX, BY), 0, st>>>(g, cc, pc, po, one_minus_omega, colour, err, skip);
  } else {
    if (err)
      k_sor_half<T, 2, true><<<grid, dim3(BX, BY), 0, st>>>(g, cc, pc, po, one_minus_omega, colour, err, skip);
    else
      k_sor_half<T, 2, false><<<grid, dim3(BX, BY), 0, st>>>(g, cc, pc, po, one_minus_omega, colour, err, skip);
  }
}

template <typename T>
void launch_p_halo(const Geo& g, T* p0, T* p1, const int* skip, cudaStream_t st) {
  const int a = g.dim == 3 ? (g.n > g.l ? g.n : g.l) : 1;
  k_p_halo<T><<<dim3((g.m + 127) / 128, a, g.dim == 3 ? 2 : 1), 128, 0, st>>>(g, p0, p1, skip);
}

template <typename TV>
void launch_projection(const Geo& g, const Scal& s, const double* p0, const double* p1, TV* u, TV* v, TV* w,
                       cudaStream_t st) {
  if (g.dim == 3)
    k_projection<TV, 3><<<grid_interior(g), dim3(BX, BY), 0, st>>>(g, s, p0, p1, u, v, w);
  else
    k_projection<TV, 2><<<grid_interior(g), dim3(BX, BY), 0, st>>>(g, s, p0, p1, u, v, w);
}

template <typename TV>
void launch_boundary(const Geo& g, const Scal& s, TV* u, TV* v, TV* w, double* p0, double* p1,
                     cudaStream_t st) {
  k_bnd_x<TV><<<dim3((g.n + 127) / 128, g.dim == 3 ? g.l : 1), 128, 0, st>>>(g, s, u, v, w, p0, p1);
  k_bnd_y<TV><<<dim3((g.m + 2 + 127) / 128, g.dim == 3 ? g.l + 2 : 1), 128, 0, st>>>(g, u, v, w, p0, p1);
  if (g.dim == 3) k_bnd_z<TV><<<dim3((g.m + 2 + 127) / 128, g.n + 2), 128, 0, st>>>(g, u, v, w, p0, p1);
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
  if (g.dim == 3)
    k_residual<3><<<grid_packed(g), dim3(BX, BY), 0, st>>>(g, C, pc, po, omega, colour, rf, ec, rmax, skip);
  else
    k_residual<2><<<grid_packed(g), dim3(BX, BY), 0, st>>>(g, C, pc, po, omega, colour, rf, ec, rmax, skip);
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
  const dim3 grid = grid_packed(g);
  if (g.dim == 3) {
    if (err)
      k_sor_dc<3, true><<<grid, dim3(BX, BY), 0, st>>>(g, K, epsc, epso, r, ec, eo, colour, err, skip);
    else
      k_sor_dc<3, false><<<grid, dim3(BX, BY), 0, st>>>(g, K, epsc, epso, r, ec, eo, colour, err, skip);
  } else {
    if (err)
      k_sor_dc<2, true><<<grid, dim3(BX, BY), 0, st>>>(g, K, epsc, epso, r, ec, eo, colour, err, skip);
    else
      k_sor_dc<2, false><<<grid, dim3(BX, BY), 0, st>>>(g, K, epsc, epso, r, ec, eo, colour, err, skip);
  }
}

void launch_pack_eps(const Geo& g, const double* poro, float* e0, float* e1, cudaStream_t st) {
  k_pack_eps<<<grid_all(g), dim3(BX, BY), 0, st>>>(g, poro, e0, e1);
}

void launch_accumulate(const Geo& g, double* p0, double* p1, const float* e0, const float* e1, const int* skip,
                       cudaStream_t st) {
  dim3 grid = grid_packed(g);
  grid.z *= 2;
  if (g.dim == 3)
    k_accumulate<3><<<grid, dim3(BX, BY), 0, st>>>(g, p0, p1, e0, e1, skip);
  else
    k_accumulate<2><<<grid, dim3(BX, BY), 0, st>>>(g, p0, p1, e0, e1, skip);
}

void launch_dc_check(const unsigned long long* rmax, double tol, int* skip, cudaStream_t st) {
  k_dc_check<<<1, 1, 0, st>>>(rmax, tol, skip);
}

void launch_coef_to_float(const Geo& g, const Coef<double>& c, Coef<float> cf, cudaStream_t st) {
  const long long n = g.pk;
  k_coef_to_float<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(n, c, cf, 2 * g.dim);
}

void launch_to_float(const double* src, float* dst, long long n, cudaStream_t st) {
  k_to_float<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(src, dst, n);
}
void launch_to_double(const float* src, double* dst, long long n, cudaStream_t st) {
  k_to_double<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(src, dst, n);
}

void launch_scatter_nat(const Geo& g, const double* stage, double* dst, cudaStream_t st) {
  k_scatter_nat<<<grid_all(g), dim3(BX, BY), 0, st>>>(g, stage, dst);
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
  template void launch_predictor<TV>(const Geo&, const Scal&, const TV*, const TV*, const TV*, const TV*,    \
                                     const TV*, const TV*, const TV*, const TV*, const TV*, TV*, TV*, TV*,  \
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
