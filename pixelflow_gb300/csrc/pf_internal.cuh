// pf_internal.cuh -- device layout, kernel declarations and host helpers
// shared by the translation units of libpixelflow_gb300.so.
//
// Device data layout (one case):
//  * "natural" arrays (u, v, w, div, porosity and time-invariant predictor
//    factors): i fastest with the ghost layer, element (i,j,k) at
//    i + X*(j + Y*k), X = m+2 rounded up to 32 elements (256 B rows for
//    FP64), Y = n+2, and Z = l+2 planes (one plane, k = 0, in 2D).
//  * "packed" red-black arrays (p, SOR coefficients, RHS): cell (i,j,k) has
//    colour c = (i + j + kk) & 1, kk = k in 3D and 1 in 2D, so colour 0 is
//    the reference's first half-sweep ((i+j) odd in 2D, (i+j+k) even in 3D).
//    It lives in the colour-c array at h = i >> 1, element h + H*(j + Y*k),
//    H = (m+2)/2 rounded up to 32.  A cell's x-neighbours are the
//    other-colour elements h-1+s and h+s (s = i & 1); its y/z neighbours are
//    element h of the neighbouring rows.  Each half-sweep therefore streams
//    one colour contiguously and reads the other colour contiguously.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <string>

#include "../../include/pixelflow_gpu.h"

namespace pf {

struct Geo {
  int dim, m, n, l;   // l == 1 in 2D
  int X, Y, Z;        // natural pitch, rows, planes
  int H;              // packed pitch
  long long nat;      // X*Y*Z elements per natural array
  long long pk;       // H*Y*Z elements per packed colour array
  // neighbour rows of the periodic edges used by the SOR: a wrap to the
  // opposite interior row when it has the other colour (even n / l), else
  // the ghost row, refreshed before every half-sweep like the reference.
  int jn_n, js_1, kt_l, kb_1;
  // 1: the air-condition program -- walls on every face, no periodic wrap
  // (the edge neighbours are the ghost rows, which hold boundary values)
  int wall;
  // 1 (2D): symmetry rows at j = 1 and j = n (the SOR's y coefficient across
  // the edge folded into the inward one; the periodic neighbours it still
  // addresses are multiplied by zero, as in the reference)
  int slip;
};

// Kernels of the boundary stage (for the launch counts).
__host__ __device__ inline int boundary_launches(const Geo& g) {
  return g.wall ? 6 : (g.dim == 3 ? 3 : (g.slip ? 3 : 2));
}

// Ghost rows of p refreshed before each half-sweep (odd periodic sizes).
__host__ __device__ inline bool periodic_halo(const Geo& g) {
  return !g.wall && ((g.n % 2) || (g.dim == 3 && (g.l % 2)));
}

// Element indices are 32-bit (make_geo rejects grids whose arrays exceed
// 2^31 elements): 64-bit index arithmetic was a large share of the
// instructions of the latency-bound sweeps.
using idx_t = int;
__host__ __device__ inline idx_t nat_idx(const Geo& g, int i, int j, int k) { return i + g.X * (j + g.Y * k); }
__host__ __device__ inline idx_t pk_idx(const Geo& g, int h, int j, int k) { return h + g.H * (j + g.Y * k); }
__host__ __device__ inline int colour_of(const Geo& g, int i, int j, int k) {
  return (i + j + (g.dim == 3 ? k : 1)) & 1;
}

// Reduction slots of a case: each max-reduction spreads its per-block
// atomics over RED_SLOTS addresses (one address would serialise tens of
// thousands of atomics per launch in L2); readers take the max of the slots.
constexpr int RED_SLOTS = 256;
enum { RED_ERR = 0, RED_ERRF = 256, RED_DIV = 512, RED_RMAX = 768, RED_FLAGS = 1024, RED_TOTAL = 1056 };
// Bits of the case's device error word (red[RED_FLAGS]), sticky until the
// case is destroyed; the host reports them as PF_E_TIMEOUT.
enum { PF_FLAG_FUSED_TIMEOUT = 1 };

// Scalars of one case, derived once on the host in double.
struct Scal {
  double dx, dy, dz, dt;
  double xnue, xlambda, density, thickness, threshold;
  double inlet_u, inlet_v, inlet_w;  // boundary() inflow values
  double inlet_velocity;             // the namelist value (wall-table inlets)
  double init_u, init_v;             // initial_conditions() values
  double outlet_pressure, omega;
  int nonslip;
  // Factors of the stencils, computed once on the host: an FP64 division per
  // cell costs tens of FP64-pipe instructions, and FP64 runs at 1/57 of the
  // FP32 rate on GB300.  Same correctly rounded values as computing them on
  // the device; the f-suffixed copies are those values rounded to float.
  double hx, hy, hz;     // 0.5/dx, 0.5/dy, 0.5/dz
  double ix2, iy2, iz2;  // 1/(dx*dx), ...
  int iso;               // 3D with dx = dy = dz: the three Laplacian factors are one
  double dtnu, dtnl;     // dt*nu, dt*(nu+lambda)
  // iso only (hx = hy = hz, ix2 = iy2 = iz2): -dt*hx, dtnu*ix2, dtnl*hx, the
  // factors of the fluid warps' predictor with the constants folded
  double mdt_h, dtnu_i2, dtnl_h;
  double pgx, pgy, pgz;  // dt/density*0.5/dx, ... (projection)
  float hxf, hyf, hzf, ix2f, iy2f, iz2f, dtf, nuf, lamf, dtnuf, dtnlf, pgxf, pgyf, pgzf;
  // non-null (the case's natural porosity array): inflow and initial
  // velocities are scaled by the porosity (the backstep program)
  const double* inflow_poro;
  // the air-condition program's wall table (top, bottom, east, west, north,
  // south: 0 wall, 1 inlet, 2 outlet) and the porosity its faces test, when
  // Geo::wall
  int walls[6];
  const double* wall_poro;
};

// The double or float copy of a factor, by the arithmetic type T.
template <typename T>
__host__ __device__ __forceinline__ T pick(double d, float f) {
  if constexpr (sizeof(T) == sizeof(float)) {
    (void)d;
    return f;
  } else {
    (void)f;
    return d;
  }
}

// Time-invariant SOR operator of one colour, normalised by omega/ap:
//   p_new = (1-omega) p + bbn - sum_nb a_nb p_nb
template <typename T>
struct Coef {
  T* a[6];   // e, w, n, s, t, b
  T* bbn;    // RHS * omega/ap (rewritten every step)
  T* wap;    // omega/ap
  T* oadd;   // ae*p(m+1) kept for the outlet row (boundrary_matrix), else 0
};

// ---- kernels (pf_kernels.cu) ----------------------------------------
// TV: velocity type, TP / TC: pressure and operator type.  The plain step
// uses double throughout; the mixed form uses float velocities with the
// FP64 pressure and operator, and float for the correction sweeps.
void launch_porosity_factors(const Geo& g, const Scal& s, const double* poro, double* gx, double* gy,
                             double* gz, double* rinv, double* damp, cudaStream_t st);
void launch_setup_coef(const Geo& g, const Scal& s, const double* poro, Coef<double> c0, Coef<double> c1,
                       cudaStream_t st);
// k_lo .. k_hi: the interior planes of a 3D grid to cover (default: all)
template <typename TV>
void launch_divergence(const Geo& g, const Scal& s, const TV* uo, const TV* vo, const TV* wo, TV* div,
                       cudaStream_t st, int k_lo = 1, int k_hi = 0);
template <typename T, typename TS>
void launch_predictor(const Geo& g, const Scal& s, const T* uo, const T* vo, const T* wo, const T* div,
                      const T* gx, const T* gy, const T* gz, const T* rinv, const T* damp, const TS* us,
                      const TS* vs, const TS* ws, TS* u, TS* v, TS* w, cudaStream_t st, int k_lo = 1,
                      int k_hi = 0);
template <typename TV>
void launch_rhs(const Geo& g, const Scal& s, const TV* u, const TV* v, const TV* w, const double* poro,
                const double* gx, const double* gy, const double* gz, Coef<double> c0, Coef<double> c1,
                cudaStream_t st);
template <typename T>
void launch_sor_half(const Geo& g, const Coef<T>& cc, T* pc, const T* po, T one_minus_omega, int colour,
                     unsigned long long* err, const int* skip, bool early, cudaStream_t st);
template <typename T>
void launch_p_halo(const Geo& g, T* p0, T* p1, const int* skip, cudaStream_t st);
template <typename TV>
void launch_projection(const Geo& g, const Scal& s, const double* p0, const double* p1, TV* u, TV* v, TV* w,
                       cudaStream_t st);
template <typename TV>
void launch_boundary(const Geo& g, const Scal& s, TV* u, TV* v, TV* w, double* p0, double* p1,
                     cudaStream_t st);
template <typename TV>
void launch_initial(const Geo& g, const Scal& s, TV* u, TV* v, TV* w, double* p0, double* p1,
                    cudaStream_t st);
template <typename TV>
void launch_div_diag(const Geo& g, const Scal& s, const TV* u, const TV* v, const TV* w, const double* poro,
                     const double* gx, const double* gy, const double* gz, unsigned long long* out,
                     cudaStream_t st);
// mixed precision form
void launch_residual(const Geo& g, const Coef<double>& C, const double* pc, const double* po, double omega,
                     int colour, float* rf, float* ec, unsigned long long* rmax, const int* skip,
                     cudaStream_t st);
void launch_accumulate(const Geo& g, double* p0, double* p1, const float* e0, const float* e1, const int* skip,
                       cudaStream_t st);
void launch_zero_u64(unsigned long long* p, int n, cudaStream_t st);
void launch_zero_int(int* p, cudaStream_t st);
void launch_dc_check(const unsigned long long* rmax, double tol, int* skip, cudaStream_t st);
// The FP32 split sweep (one colour); early: its grid fits one wave (see
// dc_one_wave), so its fixed operands load before the dependency wait.
bool dc_one_wave(const Geo& g, int sms);
void launch_sor_dc(const Geo& g, const Scal& sc, const float* epsc, const float* epso, const float* r, float* ec,
                   const float* eo, int colour, unsigned long long* err, const int* skip, bool early,
                   cudaStream_t st);
// Fused full correction sweep (both colours in one launch, 3D with even n
// and l): launch shape chosen once per case.
struct FusedShape {
  int ty = 0;              // rows per tile
  int per_cta = 0;         // (tile, plane) pairs per CTA
  int threads = 0, chunks = 0, ntiles = 0, grid = 0;
  size_t smem = 0;         // dynamic shared memory per CTA
  int drop_stage = -1;     // testing: a stage never issued, so its bounded wait runs out
};
// 3D, no walls, even n and l, and the staging rings of two-row tiles fit in
// shared memory.
bool fused_eligible(const Geo& g);
// ty_req <= 0 picks the tile height; tz_req > 0 caps the planes of a CTA's
// runs (more CTAs than SMs); sms = multiprocessors of the device.  Returns a
// cudaError_t value (0 on success).
int fused_setup(const Geo& g, int ty_req, int tz_req, int sms, FusedShape& fs);
void launch_sor_fused(const Geo& g, const Scal& sc, const FusedShape& fs, const float* const eps[2],
                      const float* const r[2], const float* const ea[2], float* const eb[2],
                      unsigned long long* err, unsigned long long* flags, const int* skip, cudaStream_t st);
void launch_pack_eps(const Geo& g, const double* poro, float* e0, float* e1, cudaStream_t st);
// Force-log sums: scratch holds 6 doubles per block of 256 cells; out[0..2]
// pressure part, out[3..5] friction part (device).  Returns the block count.
int launch_forces(const Geo& g, const Scal& s, const double* poro, const double* p0, const double* p1,
                  const double* u, const double* v, const double* w, double* scratch, double* out,
                  cudaStream_t st);
// FP32 copies of nf (<= 3) FP64 arrays of n elements (n a multiple of 4,
// 32-byte aligned arrays) in one launch.
void launch_to_float3(const double* const* src, float* const* dst, int nf, long long n, cudaStream_t st);
void launch_to_float(const double* src, float* dst, long long n, cudaStream_t st);
void launch_to_double(const float* src, double* dst, long long n, cudaStream_t st);
// staging (dense (m+2)(n+2)(l+2), i fastest) <-> device layouts
void launch_scatter_nat(const Geo& g, const double* stage, double* dst, cudaStream_t st);
// planes k_lo .. k_hi (ghost planes included) of the dense staging
void launch_scatter_nat_planes(const Geo& g, const double* stage, double* dst, int k_lo, int k_hi,
                               cudaStream_t st);
void launch_gather_nat(const Geo& g, const double* src, double* stage, cudaStream_t st);
void launch_scatter_pk(const Geo& g, const double* stage, double* p0, double* p1, cudaStream_t st);
void launch_gather_pk(const Geo& g, const double* p0, const double* p1, double* stage, cudaStream_t st);

// ---- host helpers (pf_api.cu) -------------------------------------------
int make_geo(const pf_params& p, Geo& g);
int make_scal(const pf_params& p, Scal& s);

// ---- host error plumbing (pf_api.cu) ----------------------------------
void set_error(const std::string& msg);
int fail(int code, const std::string& msg);
int cuda_fail(cudaError_t e, const char* what);

}  // namespace pf

#define PF_CUDA(call)                                   \
  do {                                                  \
    cudaError_t _e = (call);                            \
    if (_e != cudaSuccess) return pf::cuda_fail(_e, #call); \
  } while (0)
