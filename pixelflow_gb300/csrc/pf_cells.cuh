// pf_cells.cuh -- per-cell bodies of the step's stages, shared by the
// single-case kernels (pf_kernels.cu) and the persistent batch kernel
// (pf_batch.cu), so every form computes a cell with the same arithmetic.
//
// Arithmetic: the algebra of each reference expression is kept, but the
// operations are reordered for the GPU: divisions by dx, ap and porosity
// become multiplications by factors computed once per case, and products
// fuse into FMAs.  Results therefore differ from the reference in the last
// bits of each operation; the parity tests bound the drift over whole runs.
#pragma once
#include <cuda_runtime.h>

#include "pf_internal.cuh"

namespace pf {

constexpr int BX = 32, BY = 8;

__device__ __forceinline__ unsigned long long abs_bits(double x) {
  return (unsigned long long)__double_as_longlong(x) & 0x7fffffffffffffffULL;
}
__device__ __forceinline__ unsigned abs_bits(float x) { return __float_as_uint(x) & 0x7fffffffu; }

// Bits of |a - b|, the correctly rounded FP64 difference.  When a and b are
// normal with the same sign and exponent, a - b = (ma - mb) * 2^(E-1075) is
// exact in 52 bits, so the result is assembled with integer operations;
// otherwise (sign or exponent differ, zeros, subnormals, Inf, NaN, or a
// subnormal result) the FP64 subtraction.  Same bits either way.  Measured
// on the 256^3 plain step (Mcell-steps/s): tracking by FP64 subtraction 590,
// this form 641, no tracked value at all 663; a complete integer emulation
// of the subtraction (every operand class, no FP64 instruction) 584 -- its
// data-dependent branches split the warps.
__device__ __forceinline__ unsigned long long abs_diff_bits(double a, double b) {
  const unsigned long long A = (unsigned long long)__double_as_longlong(a);
  const unsigned long long B = (unsigned long long)__double_as_longlong(b);
  const unsigned top = (unsigned)(A >> 52) & 0x7ffu;
  if (((A ^ B) >> 52) == 0 && top != 0 && top != 0x7ffu) {
    constexpr unsigned long long M = 0x000fffffffffffffULL;
    const unsigned long long ma = A & M, mb = B & M;
    const unsigned long long d = ma > mb ? ma - mb : mb - ma;
    if (d == 0) return 0ULL;
    const int lead = 63 - __clzll((long long)d);  // 0 .. 51
    const int er = (int)top - 52 + lead;          // biased exponent of the difference
    if (er > 0) return ((unsigned long long)er << 52) | ((d << (52 - lead)) & M);
  }
  return abs_bits(a - b);
}
__device__ __forceinline__ unsigned abs_diff_bits(float a, float b) { return abs_bits(a - b); }

// Block-wide max of non-negative IEEE bit patterns (integer order == value
// order for non-negative numbers; NaN patterns sort above +Inf), then one
// atomicMax per block.  Order independent, hence deterministic.  The 64-bit
// patterns are compared as (hi, lo) 32-bit pairs so the reduction stays on
// the integer pipe (the FP64 pipe is the scarce one on GB300).
__device__ __forceinline__ void max_pair(unsigned& hi, unsigned& lo, unsigned h2, unsigned l2) {
  const bool gt = (h2 > hi) || (h2 == hi && l2 > lo);
  hi = gt ? h2 : hi;
  lo = gt ? l2 : lo;
}

// Programmatic dependent launch: the sweeps of the SOR loop are launched so
// that the next kernel may be scheduled while this one finishes.  Every CTA
// first waits for the previous grid to complete (its writes visible), then
// allows the next grid to launch; that grid can start only once every CTA of
// this one has reached this point, i.e. is already resident, so the waiting
// CTAs of the next grid never hold SM slots this grid still needs.
__device__ __forceinline__ void pdl_begin() {
  asm volatile("griddepcontrol.wait;" ::: "memory");
  asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
}

// Launch with programmatic stream serialization (the kernel starts with
// pdl_begin): the launch of the next kernel of the SOR loop overlaps the
// tail of the current one; CUDA graph capture keeps these as programmatic
// edges.
template <typename... KArgs, typename... Args>
void launch_pdl_smem(void (*kernel)(KArgs...), dim3 grid, dim3 block, size_t smem, cudaStream_t st,
                     Args... args) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = grid;
  cfg.blockDim = block;
  cfg.dynamicSmemBytes = smem;
  cfg.stream = st;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  cudaLaunchKernelEx(&cfg, kernel, args...);
}
template <typename... KArgs, typename... Args>
void launch_pdl(void (*kernel)(KArgs...), dim3 grid, dim3 block, cudaStream_t st, Args... args) {
  launch_pdl_smem(kernel, grid, block, 0, st, args...);
}

__device__ __forceinline__ int red_slot() {
  return (int)((blockIdx.x + 37u * blockIdx.y + 101u * blockIdx.z) & (RED_SLOTS - 1));
}

__device__ __forceinline__ unsigned long long max_of_slots(const unsigned long long* s) {
  unsigned long long r = 0;
  for (int i = 0; i < RED_SLOTS; i++) r = s[i] > r ? s[i] : r;
  return r;
}

// Exact warp max of 64-bit patterns: max of the high words, then the max low
// word among the lanes holding that high word (two hardware reductions).
__device__ __forceinline__ void warp_max64(unsigned& hi, unsigned& lo) {
  const unsigned h = __reduce_max_sync(0xffffffffu, hi);
  lo = __reduce_max_sync(0xffffffffu, hi == h ? lo : 0u);
  hi = h;
}

__device__ __forceinline__ void block_max_atomic(unsigned long long v, unsigned long long* out) {
  __shared__ unsigned long long red[32];
  unsigned hi = (unsigned)(v >> 32), lo = (unsigned)v;
  warp_max64(hi, lo);
  const int tid = threadIdx.x + blockDim.x * (threadIdx.y + blockDim.y * threadIdx.z);
  const int nthr = blockDim.x * blockDim.y * blockDim.z;
  const int lane = tid & 31, warp = tid >> 5;
  if (lane == 0) red[warp] = ((unsigned long long)hi << 32) | lo;
  __syncthreads();
  if (warp == 0) {
    const unsigned long long w = (lane < (nthr + 31) / 32) ? red[lane] : 0ULL;
    hi = (unsigned)(w >> 32);
    lo = (unsigned)w;
    warp_max64(hi, lo);
    const unsigned long long r = ((unsigned long long)hi << 32) | lo;
    if (lane == 0 && r) atomicMax(out + red_slot(), r);
  }
}

// Warp max straight into the spread slots, without a block barrier: for
// sweeps whose blocks should retire without waiting for each other.
__device__ __forceinline__ void warp_max_atomic(unsigned long long v, unsigned long long* out) {
  unsigned hi = (unsigned)(v >> 32), lo = (unsigned)v;
  warp_max64(hi, lo);
  const unsigned long long r = ((unsigned long long)hi << 32) | lo;
  if ((threadIdx.x & 31) == 0 && r) {
    const unsigned wid = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    atomicMax(out + (wid & (RED_SLOTS - 1)), r);
  }
}

// Warp max of FP32 magnitudes (32-bit patterns) into the low 32 bits of the
// spread slots, without a block barrier.
__device__ __forceinline__ void warp_max_atomic(unsigned v, unsigned long long* out) {
  const unsigned r = __reduce_max_sync(0xffffffffu, v);
  if ((threadIdx.x & 31) == 0 && r) {
    const unsigned wid = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    atomicMax(reinterpret_cast<unsigned*>(out + (wid & (RED_SLOTS - 1))), r);
  }
}

// FP32 magnitudes: 32-bit patterns, max into the low 32 bits of *slot.
__device__ __forceinline__ void block_max_atomic(unsigned v, unsigned long long* slot) {
  __shared__ unsigned red[32];
  v = __reduce_max_sync(0xffffffffu, v);
  const int tid = threadIdx.x + blockDim.x * (threadIdx.y + blockDim.y * threadIdx.z);
  const int nthr = blockDim.x * blockDim.y * blockDim.z;
  const int lane = tid & 31, warp = tid >> 5;
  if (lane == 0) red[warp] = v;
  __syncthreads();
  if (warp == 0) {
    v = (lane < (nthr + 31) / 32) ? red[lane] : 0u;
    v = __reduce_max_sync(0xffffffffu, v);
    if (lane == 0 && v) atomicMax(reinterpret_cast<unsigned*>(slot + red_slot()), v);
  }
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

// Packed sweeps over a flat thread index: slot h = 0 .. m/2 of every
// interior row, rows j fastest then planes k.  Warps are full across row
// ends (a 32-wide tile of the padded row pitch would leave one lane of 32
// working in the last warp of each row).
__host__ __device__ __forceinline__ int packed_width(const Geo& g) { return (g.m >> 1) + 1; }
__host__ __device__ __forceinline__ long long packed_items(const Geo& g) {
  return (long long)packed_width(g) * g.n * (g.dim == 3 ? g.l : 1);
}
template <int DIM>
__device__ __forceinline__ void packed_item(const Geo& g, int t, int& h, int& j, int& k) {
  const int W = packed_width(g);
  const int row = t / W;
  h = t - row * W;
  if (DIM == 3) {
    k = row / g.n + 1;
    j = row - (k - 1) * g.n + 1;
  } else {
    k = 0;
    j = row + 1;
  }
}

__device__ __forceinline__ idx_t pk_of(const Geo& g, int i, int j, int k, int& c) {
  c = colour_of(g, i, j, k);
  return pk_idx(g, i >> 1, j, k);
}


template <typename T>
__device__ __forceinline__ T& pref(const Geo& g, T* p0, T* p1, int i, int j, int k) {
  int c;
  idx_t r = pk_of(g, i, j, k, c);
  return c ? p1[r] : p0[r];
}


// The ghost cells of the old fields carry over into the new buffer (the
// reference's u keeps its ghosts through solve_p): every interior cell next to
// the ghost layer copies the ghost cells it touches -- faces, edges and
// corners, each ghost copied by exactly one interior cell.
template <typename T, int DIM>
__device__ __forceinline__ void keep_ghosts(const Geo& g, int i, int j, int k, idx_t q, const T* uo,
                                            const T* vo, const T* wo, T* u, T* v, T* w) {
  const int i0 = i == 1 ? -1 : 0, i1 = i == g.m ? 1 : 0;
  const int j0 = j == 1 ? -1 : 0, j1 = j == g.n ? 1 : 0;
  const int k0 = (DIM == 3 && k == 1) ? -1 : 0, k1 = (DIM == 3 && k == g.l) ? 1 : 0;
  if (!(i0 | i1 | j0 | j1 | k0 | k1)) return;
  const idx_t X = g.X, XY = (idx_t)g.X * g.Y;
  for (int dk = k0; dk <= k1; dk++)
    for (int dj = j0; dj <= j1; dj++)
      for (int di = i0; di <= i1; di++) {
        if (!(di | dj | dk)) continue;
        const idx_t r = q + di + X * dj + XY * dk;
        u[r] = uo[r];
        v[r] = vo[r];
        if (DIM == 3) w[r] = wo[r];
      }
}


template <typename T>
__device__ __forceinline__ void c_divergence(Geo g, Scal s, const T* __restrict__ uo, const T* __restrict__ vo,
                             const T* __restrict__ wo, T* __restrict__ div, int i, int j, int k) {
  const idx_t q = nat_idx(g, i, j, k);
  const idx_t X = g.X, XY = (idx_t)g.X * g.Y;
  const T hx = pick<T>(s.hx, s.hxf);
  if (g.dim == 3) {
    const T hy = pick<T>(s.hy, s.hyf), hz = pick<T>(s.hz, s.hzf);
    T d = (uo[q + 1] - uo[q - 1]) * hx;
    d = fma(vo[q + X] - vo[q - X], hy, d);
    d = fma(wo[q + XY] - wo[q - XY], hz, d);
    div[q] = d;
  } else {
    div[q] = fma(vo[q + X] - vo[q - X], hx, (uo[q + 1] - uo[q - 1]) * hx);
  }
}

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

// FLUID: the caller has found gx = gy = gz = damp = 0 for this cell (every
// cell of its warp): the porosity-gradient terms and the non-slip damping
// multiply zeros, so they are left out (the same values, up to the sign of a
// zero sum).
// The six-neighbour Laplacian numerator x_e + x_w + x_n + x_s + x_t + x_b
// - 6 x_c of a double field, the sum exact (sum6_exact, or added in order
// where it cannot be formed exactly: Inf, NaN, results out of the normal
// range).  A template only so that the float instantiation of the predictor
// compiles; doubles alone reach it.
template <typename T>
__device__ __forceinline__ T lap6_iso(T c, T e, T w, T n, T s, T t, T b) {
  const double x[6] = {(double)e, (double)w, (double)n, (double)s, (double)t, (double)b};
  double sum;
  if (!sum6_exact(x, sum)) sum = ((((x[0] + x[1]) + x[2]) + x[3]) + x[4]) + x[5];
  return (T)fma(-6.0, (double)c, sum);
}

template <typename T, typename TS, int DIM, bool FLUID = false>
__device__ __forceinline__ void c_predictor(Geo g, Scal s, const T* __restrict__ uo,
                                                      const T* __restrict__ vo, const T* __restrict__ wo,
                                                      const T* __restrict__ div, const T* __restrict__ gxa,
                                                      const T* __restrict__ gya, const T* __restrict__ gza,
                                                      const T* __restrict__ rinva, const T* __restrict__ dampa,
                                                      const TS* __restrict__ su, const TS* __restrict__ sv,
                                                      const TS* __restrict__ sw, TS* __restrict__ u,
                                                      TS* __restrict__ v, TS* __restrict__ w, int i, int j, int k) {
  const idx_t q = nat_idx(g, i, j, k);
  const idx_t X = g.X, XY = (idx_t)g.X * g.Y;
  const T hx = pick<T>(s.hx, s.hxf), hy = pick<T>(s.hy, s.hyf);
  const T ix2 = pick<T>(s.ix2, s.ix2f), iy2 = pick<T>(s.iy2, s.iy2f);
  const T dt = pick<T>(s.dt, s.dtf), nu = pick<T>(s.xnue, s.nuf), lam = pick<T>(s.xlambda, s.lamf);
  const T dtnu = pick<T>(s.dtnu, s.dtnuf), dtnl = pick<T>(s.dtnl, s.dtnlf);
  const T two = (T)2;
  // div neighbours with the periodic wrap of the y (and z) ghost rows
  // (walls: the ghost rows, which hold 0)
  const idx_t jn = (j == g.n && !g.wall) ? q - (idx_t)(g.n - 1) * X : q + X;
  const idx_t js = (j == 1 && !g.wall) ? q + (idx_t)(g.n - 1) * X : q - X;
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
    T t = -dt * conv;
    t = fma(dtnu, lap, t);
    t = fma(dtnl, (dE - dW) * hx, t);
    t = fma(rv, por, t);
    u[q] = su[q] + (TS)fma(-uc, dp * ix2, t);
    // v (the reference damps v with (thickness*dx)^2 as well, ibm_2d:254)
    conv = fma(vc, dvy, uc * dvx);
    lap = fma(lvy, iy2, lvx * ix2);
    por = fma(dvy + dvy, gy, (dvx + duy) * gx) * nu;
    por = fma(lam * dc, gy, por);
    t = -dt * conv;
    t = fma(dtnu, lap, t);
    t = fma(dtnl, (dN - dS) * hy, t);
    t = fma(rv, por, t);
    v[q] = sv[q] + (TS)fma(-vc, dp * ix2, t);
  } else {
    const T hz = pick<T>(s.hz, s.hzf), iz2 = pick<T>(s.iz2, s.iz2f);
    const idx_t kt = (k == g.l && !g.wall) ? q - (idx_t)(g.l - 1) * XY : q + XY;
    const idx_t kb = (k == 1 && !g.wall) ? q + (idx_t)(g.l - 1) * XY : q - XY;
    const T dT = div[kt], dB = div[kb];
    const T gz = gza[q];
    const T ut = uo[q + XY], ub = uo[q - XY], vt = vo[q + XY], vb = vo[q - XY];
    const T wc = wo[q], we = wo[q + 1], ww = wo[q - 1], wn = wo[q + X], ws = wo[q - X];
    const T wt = wo[q + XY], wb = wo[q - XY];
    if (FLUID && sizeof(T) == sizeof(double) && s.iso) {
      // Fluid warps of an isotropic FP64 grid: with hx = hy = hz the
      // convective differences share one factor, folded with -dt into one
      // constant, as are dt*nu with 1/dx^2 and dt*(nu+lambda) with 0.5/dx
      // (computed once on the host): 12 FP64 operations per component
      // instead of 17 on the FP64-bound predictor.  Different roundings
      // than the factored form only in the last bits.
      const T a = (T)s.mdt_h, b = (T)s.dtnu_i2, d = (T)s.dtnl_h;
      T conv = fma(wc, ut - ub, fma(vc, un - us, uc * (ue - uw)));
      T t = fma(b, lap6_iso<T>(uc, ue, uw, un, us, ut, ub), a * conv);
      u[q] = su[q] + (TS)fma(d, dE - dW, t);
      conv = fma(wc, vt - vb, fma(vc, vn - vs, uc * (ve - vw)));
      t = fma(b, lap6_iso<T>(vc, ve, vw, vn, vs, vt, vb), a * conv);
      v[q] = sv[q] + (TS)fma(d, dN - dS, t);
      conv = fma(wc, wt - wb, fma(vc, wn - ws, uc * (we - ww)));
      t = fma(b, lap6_iso<T>(wc, we, ww, wn, ws, wt, wb), a * conv);
      w[q] = sw[q] + (TS)fma(d, dT - dB, t);
      keep_ghosts<TS, DIM>(g, i, j, k, q, su, sv, sw, u, v, w);
      return;
    }
    const T duz = (ut - ub) * hz, dvz = (vt - vb) * hz;
    const T dwx = (we - ww) * hx, dwy = (wn - ws) * hy, dwz = (wt - wb) * hz;
    const T luz = fma(-two, uc, ut + ub), lvz = fma(-two, vc, vt + vb);
    const T lwx = fma(-two, wc, we + ww), lwy = fma(-two, wc, wn + ws), lwz = fma(-two, wc, wt + wb);
    // With dx = dy = dz (FP64) each component's Laplacian is one sum of
    // its six neighbours less six times the centre, times 1/dx^2: the sum is
    // formed exactly with integer arithmetic and rounded once (sum6_exact),
    // 2 FP64 operations per component instead of 9 on the FP64-bound
    // predictor.  The rounding differs from the directional form's only in
    // the last bits (the directional form stays for float and anisotropic
    // grids).
    const bool iso = sizeof(T) == sizeof(double) && s.iso;
    // u
    T conv = fma(wc, duz, fma(vc, duy, uc * dux));
    T lap = iso ? lap6_iso<T>(uc, ue, uw, un, us, ut, ub) * ix2 : fma(luz, iz2, fma(luy, iy2, lux * ix2));
    T t = -dt * conv;
    t = fma(dtnu, lap, t);
    t = fma(dtnl, (dE - dW) * hx, t);
    if (FLUID) {
      u[q] = su[q] + (TS)t;
    } else {
      T por = fma(duz + dwx, gz, fma(duy + dvx, gy, (dux + dux) * gx)) * nu;
      por = fma(lam * dc, gx, por);
      t = fma(rv, por, t);
      u[q] = su[q] + (TS)fma(-uc, dp * ix2, t);
    }
    // v
    conv = fma(wc, dvz, fma(vc, dvy, uc * dvx));
    lap = iso ? lap6_iso<T>(vc, ve, vw, vn, vs, vt, vb) * ix2 : fma(lvz, iz2, fma(lvy, iy2, lvx * ix2));
    t = -dt * conv;
    t = fma(dtnu, lap, t);
    t = fma(dtnl, (dN - dS) * hy, t);
    if (FLUID) {
      v[q] = sv[q] + (TS)t;
    } else {
      T por = fma(dvz + dwy, gz, fma(dvy + dvy, gy, (dvx + duy) * gx)) * nu;
      por = fma(lam * dc, gy, por);
      t = fma(rv, por, t);
      v[q] = sv[q] + (TS)fma(-vc, dp * iy2, t);
    }
    // w
    conv = fma(wc, dwz, fma(vc, dwy, uc * dwx));
    lap = iso ? lap6_iso<T>(wc, we, ww, wn, ws, wt, wb) * ix2 : fma(lwz, iz2, fma(lwy, iy2, lwx * ix2));
    t = -dt * conv;
    t = fma(dtnu, lap, t);
    t = fma(dtnl, (dT - dB) * hz, t);
    if (FLUID) {
      w[q] = sw[q] + (TS)t;
    } else {
      T por = fma(dwz + dwz, gz, fma(dwy + dvz, gy, (dwx + duz) * gx)) * nu;
      por = fma(lam * dc, gz, por);
      t = fma(rv, por, t);
      w[q] = sw[q] + (TS)fma(-wc, dp * iz2, t);
    }
  }
  keep_ghosts<TS, DIM>(g, i, j, k, q, su, sv, sw, u, v, w);
}

template <typename T, int DIM>
__device__ __forceinline__ void c_rhs(Geo g, Scal s, const T* __restrict__ u, const T* __restrict__ v, const T* __restrict__ w,
                      const double* __restrict__ po, const double* __restrict__ gxa,
                      const double* __restrict__ gya, const double* __restrict__ gza, Coef<double> c0,
                      Coef<double> c1, int i, int j, int k) {
  const idx_t X = g.X, XY = (idx_t)g.X * g.Y;
  const double hx = s.hx, hy = s.hy;
  auto raw = [&](idx_t q) {
    double sd = ((double)u[q + 1] - (double)u[q - 1]) * hx;
    sd = fma((double)v[q + X] - (double)v[q - X], hy, sd);
    double sg = gxa[q] * (double)u[q];
    sg = fma(gya[q], (double)v[q], sg);
    if (DIM == 3) {
      sd = fma((double)w[q + XY] - (double)w[q - XY], s.hz, sd);
      sg = fma(gza[q], (double)w[q], sg);
    }
    return s.density * fma(po[q], sd, sg);
  };
  const idx_t q = nat_idx(g, i, j, k);
  // the air-condition program's top outlet starts from bb of plane 1
  // (ibm_3d_air_condition_omp_cpu.f90:701)
  const bool top_copy = DIM == 3 && g.wall && s.walls[0] == 2 && k == g.l && po[q] >= 0.9;
  const double bb = raw(top_copy ? nat_idx(g, i, j, 1) : q);
  const int c = colour_of(g, i, j, k);
  const Coef<double> C = c ? c1 : c0;
  const idx_t r = pk_idx(g, i >> 1, j, k);
  C.bbn[r] = (bb + C.oadd[r]) * C.wap[r];
}

template <typename T, int DIM>
__device__ __forceinline__ void c_projection(Geo g, Scal s, const double* __restrict__ p0, const double* __restrict__ p1, T* u,
                             T* v, T* w, int i, int j, int k) {
  const idx_t q = nat_idx(g, i, j, k);
  const int c = colour_of(g, i, j, k);
  const double* P = c ? p0 : p1;  // every neighbour has the other colour
  const idx_t H = g.H, HY = (idx_t)g.H * g.Y;
  const idx_t r = pk_idx(g, i >> 1, j, k);
  const int sx = i & 1;
  u[q] = fma(-pick<T>(s.pgx, s.pgxf), (T)(P[r + sx] - P[r - 1 + sx]), u[q]);
  v[q] = fma(-pick<T>(s.pgy, s.pgyf), (T)(P[r + H] - P[r - H]), v[q]);
  if (DIM == 3) w[q] = fma(-pick<T>(s.pgz, s.pgzf), (T)(P[r + HY] - P[r - HY]), w[q]);
}

template <typename T>
__device__ __forceinline__ void c_initial(Geo g, Scal s, T* u, T* v, T* w, double* p0, double* p1, int i, int j, int k) {
  const idx_t q = nat_idx(g, i, j, k);
  if (g.wall) {  // the air-condition program starts at rest (:1194-1203)
    u[q] = (T)0;
    v[q] = (T)0;
    w[q] = (T)0;
  } else if (s.inflow_poro) {  // ibm_2d_backstep_omp_cpu.f90:615-618
    u[q] = (T)(s.init_u * s.inflow_poro[q]);
    v[q] = (T)(s.init_v * s.inflow_poro[q]);
  } else {
    u[q] = (T)s.init_u;
    v[q] = (T)s.init_v;
  }
  if (g.dim == 3) w[q] = (T)0;
  pref(g, p0, p1, i, j, k) = s.outlet_pressure;
}

// FP64 residual of one cell, r = bbn - w p - sum a p_nb (normalised by w/ap).
// Returns false for positions outside the grid.
template <int DIM>
__device__ __forceinline__ bool residual_value(const Geo& g, const Coef<double>& C, const double* __restrict__ pc,
                                               const double* __restrict__ po, double omega, int colour, int h, int j,
                                               int k, double& t) {
  const int s = (colour + j + (DIM == 3 ? k : 1)) & 1;
  const int i = 2 * h + s;
  if (!(j <= g.n && i >= 1 && i <= g.m)) return false;
  const idx_t H = g.H, HY = (idx_t)g.H * g.Y;
  const idx_t q = pk_idx(g, h, j, k);
  const idx_t qn = (j == g.n) ? pk_idx(g, h, g.jn_n, k) : q + H;
  const idx_t qs = (j == 1) ? pk_idx(g, h, g.js_1, k) : q - H;
  t = C.bbn[q];
  t = fma(-C.a[0][q], po[q + s], t);
  t = fma(-C.a[1][q], po[q - 1 + s], t);
  t = fma(-C.a[2][q], po[qn], t);
  t = fma(-C.a[3][q], po[qs], t);
  if (DIM == 3) {
    const idx_t qt = (k == g.l) ? pk_idx(g, h, j, g.kt_l) : q + HY;
    const idx_t qb = (k == 1) ? pk_idx(g, h, j, g.kb_1) : q - HY;
    t = fma(-C.a[4][q], po[qt], t);
    t = fma(-C.a[5][q], po[qb], t);
  }
  t = fma(-omega, pc[q], t);
  return true;
}

// The residual stored as the FP32 right-hand side of the correction sweeps;
// zeroes e of that cell; returns |r| as bits.
template <int DIM>
__device__ __forceinline__ unsigned long long c_residual(const Geo& g, const Coef<double>& C,
                                                         const double* __restrict__ pc, const double* __restrict__ po,
                                                         double omega, int colour, float* __restrict__ rf,
                                                         float* __restrict__ ec, int h, int j, int k) {
  double t;
  if (!residual_value<DIM>(g, C, pc, po, omega, colour, h, j, k, t)) return 0ULL;
  const idx_t q = pk_idx(g, h, j, k);
  rf[q] = (float)t;
  ec[q] = 0.0f;
  return abs_bits(t);
}

// p += e for one interior cell of the given colour.
template <int DIM>
__device__ __forceinline__ void c_accumulate(const Geo& g, double* __restrict__ pcol, const float* __restrict__ ecol,
                                             int colour, int h, int j, int k) {
  const int s = (colour + j + (DIM == 3 ? k : 1)) & 1;
  const int i = 2 * h + s;
  if (j > g.n || i < 1 || i > g.m) return;
  const idx_t q = pk_idx(g, h, j, k);
  pcol[q] += (double)ecol[q];
}

// Periodic ghost rows of a packed pair for interior i: y rows of plane k
// (ysel) or z planes of row j (3D), as the reference refreshes them before
// each half-sweep (ibm_2d:322-327; ibm_3d:463-480).
template <typename T>
__device__ __forceinline__ void c_p_halo_y(const Geo& g, T* p0, T* p1, int i, int k) {
  T* P[2] = {p0, p1};
  int cs, cd;
  idx_t s0 = pk_of(g, i, g.n, k, cs), d0 = pk_of(g, i, 0, k, cd);
  P[cd][d0] = P[cs][s0];
  s0 = pk_of(g, i, 1, k, cs);
  d0 = pk_of(g, i, g.n + 1, k, cd);
  P[cd][d0] = P[cs][s0];
}
template <typename T>
__device__ __forceinline__ void c_p_halo_z(const Geo& g, T* p0, T* p1, int i, int j) {
  T* P[2] = {p0, p1};
  int cs, cd;
  idx_t s0 = pk_of(g, i, j, g.l, cs), d0 = pk_of(g, i, j, 0, cd);
  P[cd][d0] = P[cs][s0];
  s0 = pk_of(g, i, j, 1, cs);
  d0 = pk_of(g, i, j, g.l + 1, cd);
  P[cd][d0] = P[cs][s0];
}

// boundary, x faces of row (j, k): inflow at i=1 and its ghost, outflow copy at m+1.
template <typename T>
__device__ __forceinline__ void c_bnd_x(const Geo& g, const Scal& s, T* u, T* v, T* w, double* p0, double* p1,
                                        int j, int k) {
  const idx_t q1 = nat_idx(g, 1, j, k), q0 = q1 - 1;
  if (s.inflow_poro) {  // ibm_2d_backstep_omp_cpu.f90:533-534
    u[q1] = (T)(s.inlet_u * s.inflow_poro[q1]);
    v[q1] = (T)(s.inlet_v * s.inflow_poro[q1]);
  } else {
    u[q1] = (T)s.inlet_u;
    v[q1] = (T)s.inlet_v;
  }
  u[q0] = u[q1];
  v[q0] = v[q1];
  if (g.dim == 3) {
    w[q1] = (T)0;
    w[q0] = w[q1];
  }
  pref(g, p0, p1, 0, j, k) = pref(g, p0, p1, 2, j, k);
  const idx_t qm = nat_idx(g, g.m + 1, j, k);
  u[qm] = u[qm - 2];
  v[qm] = v[qm - 2];
  if (g.dim == 3) w[qm] = w[qm - 2];
  pref(g, p0, p1, g.m + 1, j, k) = s.outlet_pressure;
}

// boundary() of the air-condition program (ibm_3d_air_condition_omp_cpu.f90:
// 873-1170) on one face, FACE = 0 top, 1 bottom, 2 east, 3 west, 4 north,
// 5 south (the wall table's order), at face coordinates (a, b) over the
// ghost-inclusive range.  An inlet (table 1) applies where the face cell's
// porosity is >= 0.9 -- for the bottom face the top plane's, as written --
// an outlet (2) likewise; everything else is a wall.  The inflow component
// and sign, the component a wall mirrors into the ghost and whether an
// outlet ghost copies the face or the inner cell follow each face's code.
template <int FACE, typename T>
__device__ __forceinline__ void c_wall_face(const Geo& g, const Scal& s, T* u, T* v, T* w, double* p0,
                                            double* p1, int a, int b) {
  const int m = g.m, n = g.n, l = g.l;
  int fi, fj, fk, gi, gj, gk, bi, bj, bk;
  int sign, comp, mirror;  // comp, mirror: 0 u, 1 v, 2 w
  bool out_inner;
  if (FACE == 0) {
    fi = gi = bi = a; fj = gj = bj = b; fk = l; gk = l + 1; bk = l - 1;
    sign = -1; comp = 2; mirror = 2; out_inner = true;
  } else if (FACE == 1) {
    fi = gi = bi = a; fj = gj = bj = b; fk = 1; gk = 0; bk = 2;
    sign = 1; comp = 2; mirror = 2; out_inner = false;
  } else if (FACE == 2) {
    fj = gj = bj = a; fk = gk = bk = b; fi = m; gi = m + 1; bi = m - 1;
    sign = -1; comp = 0; mirror = 0; out_inner = false;
  } else if (FACE == 3) {
    fj = gj = bj = a; fk = gk = bk = b; fi = 1; gi = 0; bi = 2;
    sign = 1; comp = 0; mirror = 0; out_inner = false;
  } else if (FACE == 4) {
    fi = gi = bi = a; fk = gk = bk = b; fj = n; gj = n + 1; bj = n - 1;
    sign = -1; comp = 0; mirror = 0; out_inner = false;
  } else {
    fi = gi = bi = a; fk = gk = bk = b; fj = 1; gj = 0; bj = 2;
    sign = 1; comp = 0; mirror = 1; out_inner = true;
  }
  const idx_t qf = nat_idx(g, fi, fj, fk), qg = nat_idx(g, gi, gj, gk), qb = nat_idx(g, bi, bj, bk);
  const int t = s.walls[FACE];
  const double pin = s.wall_poro[FACE == 1 ? nat_idx(g, fi, fj, l) : qf];
  const bool inlet = t == 1 && pin >= 0.9;
  const bool outlet = t == 2 && s.wall_poro[qf] >= 0.9;
  T* F[3] = {u, v, w};
  double& pg = pref(g, p0, p1, gi, gj, gk);
  if (inlet) {
    for (int d = 0; d < 3; d++) F[d][qf] = d == comp ? (T)(sign * s.inlet_velocity) : (T)0;
    for (int d = 0; d < 3; d++) F[d][qg] = F[d][qf];
    pg = pref(g, p0, p1, bi, bj, bk);
  } else if (outlet) {
    const idx_t qs = out_inner ? qb : qf;
    for (int d = 0; d < 3; d++) F[d][qg] = F[d][qs];
    pg = s.outlet_pressure;
  } else {
    for (int d = 0; d < 3; d++) F[d][qf] = (T)0;
    F[mirror][qg] = -F[mirror][qb];
    pg = pref(g, p0, p1, bi, bj, bk);
  }
}

// boundary, y faces: periodic ghost rows at column i of plane k.
template <typename T>
__device__ __forceinline__ void c_bnd_y(const Geo& g, T* u, T* v, T* w, double* p0, double* p1, int i, int k) {
  const idx_t a = nat_idx(g, i, 0, k), b = nat_idx(g, i, g.n, k);
  const idx_t c = nat_idx(g, i, g.n + 1, k), d = nat_idx(g, i, 1, k);
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

// boundary, the symmetry rows of the 2D slip option at column i (1..m), in
// the order of the reference's commented blocks (ibm_2d_uniform_omp_cpu.f90
// :512-526): j = 1 -- u mirrored into ghost row 0, v = 0 on the row and
// odd into the ghost, p even; then j = n likewise.
template <typename T>
__device__ __forceinline__ void c_bnd_slip(const Geo& g, T* u, T* v, double* p0, double* p1, int i) {
  const int n = g.n;
  u[nat_idx(g, i, 0, 0)] = u[nat_idx(g, i, 2, 0)];
  v[nat_idx(g, i, 1, 0)] = T(0);
  v[nat_idx(g, i, 0, 0)] = -v[nat_idx(g, i, 2, 0)];
  pref(g, p0, p1, i, 0, 0) = pref(g, p0, p1, i, 2, 0);
  u[nat_idx(g, i, n + 1, 0)] = u[nat_idx(g, i, n - 1, 0)];
  v[nat_idx(g, i, n, 0)] = T(0);
  v[nat_idx(g, i, n + 1, 0)] = -v[nat_idx(g, i, n - 1, 0)];
  pref(g, p0, p1, i, n + 1, 0) = pref(g, p0, p1, i, n - 1, 0);
}

// boundary, z faces (3D): periodic ghost planes at column i of row j.
template <typename T>
__device__ __forceinline__ void c_bnd_z(const Geo& g, T* u, T* v, T* w, double* p0, double* p1, int i, int j) {
  const idx_t a = nat_idx(g, i, j, 0), b = nat_idx(g, i, j, g.l);
  const idx_t c = nat_idx(g, i, j, g.l + 1), d = nat_idx(g, i, j, 1);
  u[a] = u[b];
  v[a] = v[b];
  w[a] = w[b];
  u[c] = u[d];
  v[c] = v[d];
  w[c] = w[d];
  pref(g, p0, p1, i, j, 0) = pref(g, p0, p1, i, j, g.l);
  pref(g, p0, p1, i, j, g.l + 1) = pref(g, p0, p1, i, j, 1);
}

// FP32 correction sweep with the operator rebuilt on the fly from the FP32
// porosity (packed by colour, ghosts included), so a half-sweep streams only
// porosity, r and e (24 bytes per update) instead of six stored
// coefficients.  Same operator as k_setup_coef up to FP32 rounding:
//   a_f = dt/h^2 * max(small, (eps_a+eps_b)/2), ap = -sum a_f (before the
//   inlet/outlet edits), inlet: a_e += a_w, a_w = 0; outlet: all a_f = 0,
//   e = (1-w) e + r - (w/ap) sum a_f e_f.
// Away from the outlet the update is evaluated as
//   e = e + r + (w/sigma) sum a_f (e_f - e),   sigma = sum a_f = -ap,
// the same value in exact arithmetic (the inlet edit keeps the sum).  In
// floats the two differ in what the rounding does to the operator's row sum:
// with (1-w) and w/ap rounded separately, a correction that is constant
// across a cell's neighbours is not reproduced, and that relative error of
// a few 1e-8 in the operator's diagonal acts on the smooth pressure modes
// that the 100 sweeps of a step never damp (the pressure error against the
// plain FP64 step is ~100x larger); here a constant correction gives
// e + r exactly.
struct DCConst {
  // half face factors 0.5*dt/dx^2 etc. (exact halves of the float dt/dx^2)
  // and twice the porosity floor: kx*max(small, (a+b)*0.5) is computed as
  // hx*max(small2, a+b), the same float because the scalings by 2 are exact
  float hx, hy, hz;
  float small2, omega, omw;
};
// From the case's double scalars: dt/dx^2 etc., omega and 1 - omega, each
// rounded to float once.
__host__ __device__ inline DCConst make_dc_const(double dt, double dx, double dy, double dz, int dim,
                                                 double omega) {
  DCConst K;
  K.hx = (float)(dt / dx / dx) * 0.5f;
  K.hy = (float)(dt / dy / dy) * 0.5f;
  K.hz = dim == 3 ? (float)(dt / dz / dz) * 0.5f : 0.f;
  K.small2 = 2.e-6f;  // 2 * 1e-6f, exactly
  K.omega = (float)omega;
  K.omw = (float)(1.0 - omega);
  return K;
}

// A face coefficient of the correction sweep's operator from the porosity of
// the two cells sharing the face: the same float for both cells (the sum is
// commutative), so a kernel may compute a face once for the two updates.
__device__ __forceinline__ float dc_face(float h, const DCConst& K, float pa, float pb) {
  return h * fmaxf(K.small2, pa + pb);
}

// One cell of the correction sweep from its face coefficients and the other
// colour's neighbour corrections.
template <int DIM>
__device__ __forceinline__ float dc_cell_faces(const DCConst& K, float ae, float aw, float an, float as, float at,
                                               float ab, float xe, float xw, float xn, float xs, float xt,
                                               float xb, float rr, float eold, bool inlet, bool outlet) {
  if (outlet) return fmaf(K.omw, eold, rr);
  const float sigma = ae + aw + an + as + at + ab;
  if (inlet) {
    ae += aw;
    aw = 0.f;
  }
  float t = ae * (xe - eold);
  t = fmaf(aw, xw - eold, t);
  t = fmaf(an, xn - eold, t);
  t = fmaf(as, xs - eold, t);
  if (DIM == 3) {
    t = fmaf(at, xt - eold, t);
    t = fmaf(ab, xb - eold, t);
  }
  return fmaf(__fdividef(K.omega, sigma), t, eold + rr);
}

// One cell of the correction sweep from its loaded operands.  Every form of
// the sweep (the vectorised single-case kernel, the fused kernel, the
// persistent batch kernel's global and shared-memory passes) reaches
// dc_cell_faces with faces from dc_face, so they agree bit for bit.
template <int DIM>
__device__ __forceinline__ float dc_cell(const DCConst& K, float pc, float pe, float pw, float pn, float ps,
                                         float pt, float pb, float xe, float xw, float xn, float xs, float xt,
                                         float xb, float rr, float eold, bool inlet, bool outlet) {
  const float at = DIM == 3 ? dc_face(K.hz, K, pt, pc) : 0.f;
  const float ab = DIM == 3 ? dc_face(K.hz, K, pc, pb) : 0.f;
  return dc_cell_faces<DIM>(K, dc_face(K.hx, K, pe, pc), dc_face(K.hx, K, pc, pw), dc_face(K.hy, K, pn, pc),
                            dc_face(K.hy, K, pc, ps), at, ab, xe, xw, xn, xs, xt, xb, rr, eold, inlet, outlet);
}

// V consecutive floats loaded as one aligned vector access.
template <int V>
struct alignas(4 * V) VecF {
  float a[V];
};
template <int V>
__device__ __forceinline__ VecF<V> ldv(const float* p) {
  return *reinterpret_cast<const VecF<V>*>(p);
}

// The V cells of one chunk from its loaded operand rows: own correction EC,
// residual R and porosity PC; the other colour's correction XO and porosity
// PO at the same slots plus the one slot before (s = 0) or after (s = 1)
// them (xx, px); the other colour's rows north/south/top/bottom.  Lanes
// outside 1 <= i <= m keep their old value.  Every chunked form of the sweep
// calls this, so they agree bit for bit.
template <int DIM, bool TRACK, int V>
__device__ __forceinline__ VecF<V> dc_chunk(const Geo& g, const DCConst& K, int h0, int s, const VecF<V>& EC,
                                            const VecF<V>& R, const VecF<V>& PC, const VecF<V>& XO,
                                            const VecF<V>& PO, float xx, float px, const VecF<V>& XN,
                                            const VecF<V>& XS, const VecF<V>& PN, const VecF<V>& PS,
                                            const VecF<V>& XT, const VecF<V>& XB, const VecF<V>& PT,
                                            const VecF<V>& PB, unsigned& e) {
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
    const float v = dc_cell<DIM>(K, PC.a[u], pe, pw, PN.a[u], PS.a[u], PT.a[u], PB.a[u], xe, xw, XN.a[u], XS.a[u],
                                 XT.a[u], XB.a[u], R.a[u], eold, i == 1, i == g.m);
    const bool in = i >= 1 && i <= g.m;
    out.a[u] = in ? v : eold;
    if (TRACK && in) e = max(e, abs_bits(v - eold));
  }
  return out;
}

template <int DIM>
__device__ __forceinline__ void dc_update(const Geo& g, const DCConst& K, const float* __restrict__ epsc,
                                          const float* __restrict__ epso, const float* __restrict__ r,
                                          float* __restrict__ ec, const float* __restrict__ eo, int h, int j,
                                          int k, int s, int i, float& eold, float& enew) {
  const idx_t H = g.H, HY = (idx_t)g.H * g.Y;
  const idx_t q = pk_idx(g, h, j, k);
  const idx_t qn = (j == g.n) ? pk_idx(g, h, g.jn_n, k) : q + H;
  const idx_t qs = (j == 1) ? pk_idx(g, h, g.js_1, k) : q - H;
  // all loads first: this kernel is latency bound, not ALU bound
  const float pc = epsc[q], pe = epso[q + s], pw = epso[q - 1 + s], pn = epso[q + H], ps = epso[q - H];
  const float xe = eo[q + s], xw = eo[q - 1 + s], xn = eo[qn], xs = eo[qs];
  const float rr = r[q];
  eold = ec[q];
  float pt = 0.f, pb = 0.f, xt = 0.f, xb = 0.f;
  if (DIM == 3) {
    const idx_t qt = (k == g.l) ? pk_idx(g, h, j, g.kt_l) : q + HY;
    const idx_t qb = (k == 1) ? pk_idx(g, h, j, g.kb_1) : q - HY;
    pt = epso[q + HY];
    pb = epso[q - HY];
    xt = eo[qt];
    xb = eo[qb];
  }
  enew = dc_cell<DIM>(K, pc, pe, pw, pn, ps, pt, pb, xe, xw, xn, xs, xt, xb, rr, eold, i == 1, i == g.m);
}


// The same update as dc_update for a 2D cell whose correction, porosity and
// residual rows are held in shared memory: E*/P* point at the cell's local
// row of the own (c) and other (o) colour arrays, `pitch` is the row pitch.
__device__ __forceinline__ float dc_update_rows_2d(const DCConst& K, const float* __restrict__ Pc,
                                                   const float* __restrict__ Po, const float* __restrict__ Eo,
                                                   int pitch, int h, int s, bool inlet, bool outlet, float rr,
                                                   float eold) {
  const float pc = Pc[h];
  const float pe = Po[h + s], pw = Po[h - 1 + s], pn = Po[h + pitch], ps = Po[h - pitch];
  const float xe = Eo[h + s], xw = Eo[h - 1 + s], xn = Eo[h + pitch], xs = Eo[h - pitch];
  return dc_cell<2>(K, pc, pe, pw, pn, ps, 0.f, 0.f, xe, xw, xn, xs, 0.f, 0.f, rr, eold, inlet, outlet);
}

}  // namespace pf
