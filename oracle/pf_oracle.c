/*
 * pf_oracle.c -- TEST INFRASTRUCTURE ONLY (the oracle).
 *
 * CPU restatement of PixelFlow's OpenMP immersed-boundary step, used only by
 * tests/, __graft_entry__.smoke() and the cpu_baseline / reference arm of
 * bench.py as the checker and as the timed CPU baseline.  The product
 * (pixelflow_gb300, the CUDA C-ABI library) never links or calls this file.
 *
 * Parity status: pinned on small grids.  The reference is Fortran 90 and
 * has no tests, golden vectors or expected outputs, and no Fortran compiler
 * exists here.  Its own programs are instead executed from their source
 * text by a translator for the Fortran subset they use
 * (tests/golden/fortran_subset.py, gfortran plain-FP64 semantics; fixtures
 * tests/golden/refpin_*.npz): this restatement reproduces their fields,
 * their divergence output and the drag program's force log bit for bit
 * (uniform 2D and 3D on even and odd grids, backstep, air-condition, drag,
 * and the uniform 2D program with its commented symmetry rows enabled;
 * tests/test_reference_pin.py).  It is also cross-checked
 * against an independent numpy restatement (oracle/np_oracle.py) and
 * physical invariants (tests/).
 *
 * Every routine below follows one reference subroutine statement for
 * statement, with the same loop nests, the same red-black linear-index
 * colour mapping and p_old snapshots, and the same left-to-right Fortran
 * evaluation order of each expression.  Build with -ffp-contract=off so no
 * multiply-add is fused: that is what gfortran emits on x86-64 without
 * -march flags, and it makes the result identical on x86 and aarch64.
 *
 * The file is compiled twice: REAL=double (the "plain FP64" build, i.e.
 * the reference with real promoted to 8 bytes) and REAL=float (the
 * reference's default `real`).  Arrays use the Fortran layout of the
 * reference with the leading dimensions exactly m+2, n+2 (0-based ghosts):
 * element (i,j[,k]) is at i + (m+2)*(j + (n+2)*k).
 *
 * Reference files (paths inside nobu-n2002/PixelFlow):
 *   2D: src/omp_parallel/ibm_2d_uniform_omp_cpu.f90
 *   3D: src/omp_parallel/ibm_3d_uniform_omp_cpu.f90
 *   3D with the wall table (wall_mode = 1):
 *       src/omp_parallel/ibm_3d_air_condition_omp_cpu.f90
 *   2D with symmetry rows at j = 1 and j = n (slip_y = 1): the options the
 *       2D file keeps commented out (:440-450, :512-526)
 *   grid: src/omp_parallel/lib/grid.f90, divergence: lib/output.f90
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#ifndef REAL
#define REAL double
#define SFX _d
#endif

#define CAT_(a, b) a##b
#define CAT(a, b) CAT_(a, b)
#define F(name) CAT(name, SFX)
#define R(x) ((REAL)(x))

/* Same field layout as pf_params in include/pixelflow_gpu.h (namelist values). */
typedef struct or_params {
  int32_t dim, m, n, l;
  double xnue, xlambda, density, width, height, depth, time;
  double inlet_velocity, outlet_pressure, aoa;
  int32_t istep_max, iter_max;
  double thickness, threshold, relux_factor;
  int32_t nonslip, inflow_porosity;
  int32_t wall_mode;  /* 1: the air-condition program (3D) */
  int32_t walls[6];   /* top, bottom, east, west, north, south: 0 wall, 1 inlet, 2 outlet */
  int32_t slip_y;     /* 1 (2D): the commented symmetry rows at j = 1 and j = n */
} or_params;

typedef struct F(or_ctx) {
  int dim, m, n, l;
  REAL xnue, xlambda, density, width, height, depth, time;
  REAL inlet_velocity, outlet_pressure, aoa, thickness, threshold, relux;
  REAL dx, dy, dz, dt;
  int nonslip, iter_max, istep_max;
  int inflow_porosity;   /* backstep program: inflow/initial velocity x porosity */
  int wall_mode, walls[6];
  int slip_y;            /* 2D symmetry rows (ibm_2d_uniform_omp_cpu.f90:440-450, 512-526) */
  const REAL *poro;      /* porosity of the case (set by or_grid_conditions) */
  size_t ncell; /* (m+2)(n+2)[(l+2)] */
  /* solve_p locals (static in the reference through -fno-automatic) */
  REAL *ap, *ae, *aw, *an, *as, *at, *ab, *bb, *div, *p_old;
  REAL last_error;
} F(or_ctx);

typedef F(or_ctx) CTX;

#define I2(i, j) ((size_t)(i) + (size_t)(c->m + 2) * (size_t)(j))
#define I3(i, j, k) \
  ((size_t)(i) + (size_t)(c->m + 2) * ((size_t)(j) + (size_t)(c->n + 2) * (size_t)(k)))

static REAL rmax(REAL a, REAL b) { return (a > b) ? a : b; } /* Fortran MAX(a,b) */

CTX *F(or_create)(const or_params *P) {
  CTX *c = (CTX *)calloc(1, sizeof(CTX));
  if (!c) return NULL;
  c->dim = P->dim;
  c->m = P->m;
  c->n = P->n;
  c->l = (P->dim == 3) ? P->l : 1;
  c->xnue = R(P->xnue);
  c->xlambda = R(P->xlambda);
  c->density = R(P->density);
  c->width = R(P->width);
  c->height = R(P->height);
  c->depth = R(P->depth);
  c->time = R(P->time);
  c->inlet_velocity = R(P->inlet_velocity);
  c->outlet_pressure = R(P->outlet_pressure);
  c->aoa = R(P->aoa);
  c->thickness = R(P->thickness);
  c->threshold = R(P->threshold);
  c->relux = R(P->relux_factor);
  c->nonslip = P->nonslip;
  c->inflow_porosity = P->inflow_porosity;
  c->wall_mode = (P->dim == 3) ? P->wall_mode : 0;
  for (int f = 0; f < 6; f++) c->walls[f] = P->walls[f];
  c->slip_y = (P->dim == 2) ? P->slip_y : 0;
  c->iter_max = P->iter_max;
  c->istep_max = P->istep_max;
  /* grid.f90:50-52 (2D), :297-300 (3D) */
  c->dx = c->width / R(c->m - 1);
  c->dy = c->height / R(c->n - 1);
  c->dz = (c->dim == 3) ? c->depth / R(c->l - 1) : R(0);
  c->dt = c->time / R(c->istep_max);
  c->ncell = (size_t)(c->m + 2) * (size_t)(c->n + 2) * (size_t)(c->dim == 3 ? c->l + 2 : 1);
  REAL **arrs[] = {&c->ap, &c->ae, &c->aw, &c->an, &c->as, &c->at, &c->ab, &c->bb, &c->div, &c->p_old};
  for (int q = 0; q < 10; q++) {
    *arrs[q] = (REAL *)calloc(c->ncell, sizeof(REAL));
    if (!*arrs[q]) return NULL;
  }
  return c;
}

void F(or_destroy)(CTX *c) {
  if (!c) return;
  free(c->ap); free(c->ae); free(c->aw); free(c->an); free(c->as);
  free(c->at); free(c->ab); free(c->bb); free(c->div); free(c->p_old);
  free(c);
}

/* Derived grid scalars, for the tests: dx, dy, dz, dt. */
void F(or_scalars)(const CTX *c, double *out4) {
  out4[0] = (double)c->dx; out4[1] = (double)c->dy; out4[2] = (double)c->dz; out4[3] = (double)c->dt;
}

/* Work array access for stage-wise tests: 0 ap,1 ae,2 aw,3 an,4 as,5 at,6 ab,7 bb,8 div. */
REAL *F(or_work)(CTX *c, int which) {
  REAL *w[] = {c->ap, c->ae, c->aw, c->an, c->as, c->at, c->ab, c->bb, c->div, c->p_old};
  return (which >= 0 && which < 10) ? w[which] : NULL;
}

double F(or_last_error)(const CTX *c) { return (double)c->last_error; }

/* ------------------------------------------------------------------ */
/* grid.f90:40-47, 92-106 (2D) and :285-292, 349-378 (3D).             */
/* vals: porosity values in CSV order (i fastest), already parsed.     */
void F(or_grid_conditions)(CTX *c, const double *vals, REAL *poro) {
  const int m = c->m, n = c->n, l = c->l;
  c->poro = poro;
  memset(poro, 0, c->ncell * sizeof(REAL)); /* static arrays start at zero */
  if (c->dim == 2) {
    size_t q = 0;
    for (int j = 1; j <= n; j++)
      for (int i = 1; i <= m; i++) poro[I2(i, j)] = rmax(R(vals[q++]), c->threshold);
    for (int j = 1; j <= n + 1; j++) {
      poro[I2(0, j)] = poro[I2(1, j)];
      poro[I2(m + 1, j)] = poro[I2(m, j)];
    }
    for (int i = 0; i <= m + 1; i++) {
      poro[I2(i, 0)] = poro[I2(i, n)];
      poro[I2(i, n + 1)] = poro[I2(i, 1)];
    }
  } else {
    size_t q = 0;
    for (int k = 1; k <= l; k++)
      for (int j = 1; j <= n; j++)
        for (int i = 1; i <= m; i++) poro[I3(i, j, k)] = rmax(R(vals[q++]), c->threshold);
    if (c->wall_mode) { /* grid_conditions_wall, grid.f90:208-244: copies, x then y then z */
      for (int j = 0; j <= n + 1; j++)
        for (int k = 0; k <= l + 1; k++) {
          poro[I3(0, j, k)] = poro[I3(1, j, k)];
          poro[I3(m + 1, j, k)] = poro[I3(m, j, k)];
        }
      for (int i = 0; i <= m + 1; i++)
        for (int k = 0; k <= l + 1; k++) {
          poro[I3(i, 0, k)] = poro[I3(i, 1, k)];
          poro[I3(i, n + 1, k)] = poro[I3(i, n, k)];
        }
      for (int i = 0; i <= m + 1; i++)
        for (int j = 0; j <= n + 1; j++) {
          poro[I3(i, j, 0)] = poro[I3(i, j, 1)];
          poro[I3(i, j, l + 1)] = poro[I3(i, j, l)];
        }
      return;
    }
    for (int j = 1; j <= n + 1; j++)
      for (int k = 1; k <= l + 1; k++) {
        poro[I3(0, j, k)] = poro[I3(1, j, k)];
        poro[I3(m + 1, j, k)] = poro[I3(m, j, k)];
      }
    for (int i = 0; i <= m + 1; i++)
      for (int k = 0; k <= l + 1; k++) {
        poro[I3(i, 0, k)] = poro[I3(i, n, k)];
        poro[I3(i, n + 1, k)] = poro[I3(i, 1, k)];
      }
    for (int i = 0; i <= m + 1; i++)
      for (int j = 0; j <= n + 1; j++) {
        poro[I3(i, j, 0)] = poro[I3(i, j, l)];
        poro[I3(i, j, l + 1)] = poro[I3(i, j, 1)];
      }
  }
}

/* ------------------------------------------------------------------ */
/* boundary: 2D ibm_2d_uniform_omp_cpu.f90:460-538, 3D ibm_3d:669-752 */
/* boundary() of the air-condition program (:873-1170): faces in the order
   top, bottom, west, east, north, south over the ghost-inclusive ranges, each
   a wall, an inlet or an outlet by the wall table, inlet and outlet applying
   where the face cell's porosity is >= 0.9 (the bottom inlet tests the top
   plane's porosity, as the reference does).  Walls zero the face velocity and
   mirror one component into the ghost, which component by face as written. */
static void F(wall_boundary)(CTX *c, REAL *p, REAL *u, REAL *v, REAL *w) {
  const int m = c->m, n = c->n, l = c->l;
  const REAL *po = c->poro, lim = R(0.9), U = c->inlet_velocity, pout = c->outlet_pressure;
  for (int i = 0; i <= m + 1; i++) /* top */
    for (int j = 0; j <= n + 1; j++) {
      const size_t f = I3(i, j, l), g = I3(i, j, l + 1), b = I3(i, j, l - 1);
      const int t = c->walls[0];
      if (t == 1 && po[f] >= lim) {
        u[f] = R(0.); v[f] = R(0.); w[f] = -U;
        u[g] = u[f]; v[g] = v[f]; w[g] = w[f]; p[g] = p[b];
      } else if (t == 2 && po[f] >= lim) {
        u[g] = u[b]; v[g] = v[b]; w[g] = w[b]; p[g] = pout;
      } else {
        u[f] = R(0.); v[f] = R(0.); w[f] = R(0.);
        w[g] = -w[b]; p[g] = p[b];
      }
    }
  for (int i = 0; i <= m + 1; i++) /* bottom */
    for (int j = 0; j <= n + 1; j++) {
      const size_t f = I3(i, j, 1), g = I3(i, j, 0), b = I3(i, j, 2);
      const int t = c->walls[1];
      if (t == 1 && po[I3(i, j, l)] >= lim) {
        u[f] = R(0.); v[f] = R(0.); w[f] = U;
        u[g] = u[f]; v[g] = v[f]; w[g] = w[f]; p[g] = p[b];
      } else if (t == 2 && po[f] >= lim) {
        u[g] = u[f]; v[g] = v[f]; w[g] = w[f]; p[g] = pout;
      } else {
        u[f] = R(0.); v[f] = R(0.); w[f] = R(0.);
        w[g] = -w[b]; p[g] = p[b];
      }
    }
  for (int j = 0; j <= n + 1; j++) /* west */
    for (int k = 0; k <= l + 1; k++) {
      const size_t f = I3(1, j, k), g = I3(0, j, k), b = I3(2, j, k);
      const int t = c->walls[3];
      if (t == 1 && po[f] >= lim) {
        u[f] = U; v[f] = R(0.); w[f] = R(0.);
        u[g] = u[f]; v[g] = v[f]; w[g] = w[f]; p[g] = p[b];
      } else if (t == 2 && po[f] >= lim) {
        u[g] = u[f]; v[g] = v[f]; w[g] = w[f]; p[g] = pout;
      } else {
        u[f] = R(0.); v[f] = R(0.); w[f] = R(0.);
        u[g] = -u[b]; p[g] = p[b];
      }
    }
  for (int j = 0; j <= n + 1; j++) /* east */
    for (int k = 0; k <= l + 1; k++) {
      const size_t f = I3(m, j, k), g = I3(m + 1, j, k), b = I3(m - 1, j, k);
      const int t = c->walls[2];
      if (t == 1 && po[f] >= lim) {
        u[f] = -U; v[f] = R(0.); w[f] = R(0.);
        u[g] = u[f]; v[g] = v[f]; w[g] = w[f]; p[g] = p[b];
      } else if (t == 2 && po[f] >= lim) {
        u[g] = u[f]; v[g] = v[f]; w[g] = w[f]; p[g] = pout;
      } else {
        u[f] = R(0.); v[f] = R(0.); w[f] = R(0.);
        u[g] = -u[b]; p[g] = p[b];
      }
    }
  for (int i = 0; i <= m + 1; i++) /* north */
    for (int k = 0; k <= l + 1; k++) {
      const size_t f = I3(i, n, k), g = I3(i, n + 1, k), b = I3(i, n - 1, k);
      const int t = c->walls[4];
      if (t == 1 && po[f] >= lim) {
        u[f] = -U; v[f] = R(0.); w[f] = R(0.);
        u[g] = u[f]; v[g] = v[f]; w[g] = w[f]; p[g] = p[b];
      } else if (t == 2 && po[f] >= lim) {
        u[g] = u[f]; v[g] = v[f]; w[g] = w[f]; p[g] = pout;
      } else {
        u[f] = R(0.); v[f] = R(0.); w[f] = R(0.);
        u[g] = -u[b]; p[g] = p[b];
      }
    }
  for (int i = 0; i <= m + 1; i++) /* south */
    for (int k = 0; k <= l + 1; k++) {
      const size_t f = I3(i, 1, k), g = I3(i, 0, k), b = I3(i, 2, k);
      const int t = c->walls[5];
      if (t == 1 && po[f] >= lim) {
        u[f] = U; v[f] = R(0.); w[f] = R(0.);
        u[g] = u[f]; v[g] = v[f]; w[g] = w[f]; p[g] = p[b];
      } else if (t == 2 && po[f] >= lim) {
        u[g] = u[b]; v[g] = v[b]; w[g] = w[b]; p[g] = pout;
      } else {
        u[f] = R(0.); v[f] = R(0.); w[f] = R(0.);
        v[g] = -v[b]; p[g] = p[b];
      }
    }
}

void F(or_boundary)(CTX *c, REAL *p, REAL *u, REAL *v, REAL *w) {
  const int m = c->m, n = c->n, l = c->l;
  if (c->wall_mode) {
    F(wall_boundary)(c, p, u, v, w);
    return;
  }
  if (c->dim == 2) {
    const REAL pai = (REAL)atan(R(1.)) * R(4.);
    for (int j = 1; j <= n; j++) {
      u[I2(1, j)] = c->inlet_velocity * (REAL)cos(c->aoa / R(180.) * pai);
      v[I2(1, j)] = c->inlet_velocity * (REAL)sin(c->aoa / R(180.) * pai);
      if (c->inflow_porosity) { /* ibm_2d_backstep_omp_cpu.f90:533-534 */
        u[I2(1, j)] = u[I2(1, j)] * c->poro[I2(1, j)];
        v[I2(1, j)] = v[I2(1, j)] * c->poro[I2(1, j)];
      }
      u[I2(0, j)] = u[I2(1, j)];
      v[I2(0, j)] = v[I2(1, j)];
      p[I2(0, j)] = p[I2(2, j)];
    }
    for (int j = 1; j <= n; j++) {
      u[I2(m + 1, j)] = u[I2(m - 1, j)];
      v[I2(m + 1, j)] = v[I2(m - 1, j)];
      p[I2(m + 1, j)] = c->outlet_pressure;
    }
    for (int i = 0; i <= m + 1; i++) {
      u[I2(i, 0)] = u[I2(i, n)];
      v[I2(i, 0)] = v[I2(i, n)];
      p[I2(i, 0)] = p[I2(i, n)];
      u[I2(i, n + 1)] = u[I2(i, 1)];
      v[I2(i, n + 1)] = v[I2(i, 1)];
      p[I2(i, n + 1)] = p[I2(i, 1)];
    }
    if (c->slip_y) { /* :512-526, the commented symmetry options at j = 1 and j = n */
      for (int i = 1; i <= m; i++) {
        u[I2(i, 0)] = u[I2(i, 2)];
        v[I2(i, 1)] = R(0.);
        v[I2(i, 0)] = -v[I2(i, 2)];
        p[I2(i, 0)] = p[I2(i, 2)];
      }
      for (int i = 1; i <= m; i++) {
        u[I2(i, n + 1)] = u[I2(i, n - 1)];
        v[I2(i, n)] = R(0.);
        v[I2(i, n + 1)] = -v[I2(i, n - 1)];
        p[I2(i, n + 1)] = p[I2(i, n - 1)];
      }
    }
  } else {
    const REAL pi = (REAL)atan(R(1.)) * R(4.);
#pragma omp parallel for
    for (int k = 1; k <= l; k++)
      for (int j = 1; j <= n; j++) {
        u[I3(1, j, k)] = c->inlet_velocity * (REAL)cos(c->aoa / R(1300.) * pi);
        v[I3(1, j, k)] = c->inlet_velocity * (REAL)sin(c->aoa / R(1300.) * pi);
        if (c->inflow_porosity) { /* the 2D backstep rule applied in 3D */
          u[I3(1, j, k)] = u[I3(1, j, k)] * c->poro[I3(1, j, k)];
          v[I3(1, j, k)] = v[I3(1, j, k)] * c->poro[I3(1, j, k)];
        }
        w[I3(1, j, k)] = R(0.);
        u[I3(0, j, k)] = u[I3(1, j, k)];
        v[I3(0, j, k)] = v[I3(1, j, k)];
        w[I3(0, j, k)] = w[I3(1, j, k)];
        p[I3(0, j, k)] = p[I3(2, j, k)];
      }
#pragma omp parallel for
    for (int k = 1; k <= l; k++)
      for (int j = 1; j <= n; j++) {
        u[I3(m + 1, j, k)] = u[I3(m - 1, j, k)];
        v[I3(m + 1, j, k)] = v[I3(m - 1, j, k)];
        w[I3(m + 1, j, k)] = w[I3(m - 1, j, k)];
        p[I3(m + 1, j, k)] = c->outlet_pressure;
      }
#pragma omp parallel for
    for (int k = 0; k <= l + 1; k++)
      for (int i = 0; i <= m + 1; i++) {
        u[I3(i, 0, k)] = u[I3(i, n, k)];
        v[I3(i, 0, k)] = v[I3(i, n, k)];
        w[I3(i, 0, k)] = w[I3(i, n, k)];
        p[I3(i, 0, k)] = p[I3(i, n, k)];
        u[I3(i, n + 1, k)] = u[I3(i, 1, k)];
        v[I3(i, n + 1, k)] = v[I3(i, 1, k)];
        w[I3(i, n + 1, k)] = w[I3(i, 1, k)];
        p[I3(i, n + 1, k)] = p[I3(i, 1, k)];
      }
#pragma omp parallel for
    for (int j = 0; j <= n + 1; j++)
      for (int i = 0; i <= m + 1; i++) {
        u[I3(i, j, 0)] = u[I3(i, j, l)];
        v[I3(i, j, 0)] = v[I3(i, j, l)];
        w[I3(i, j, 0)] = w[I3(i, j, l)];
        p[I3(i, j, 0)] = p[I3(i, j, l)];
        u[I3(i, j, l + 1)] = u[I3(i, j, 1)];
        v[I3(i, j, l + 1)] = v[I3(i, j, 1)];
        w[I3(i, j, l + 1)] = w[I3(i, j, 1)];
        p[I3(i, j, l + 1)] = p[I3(i, j, 1)];
      }
  }
}

/* ------------------------------------------------------------------ */
/* initial_conditions: 2D :542-568, 3D :756-793; followed by boundary as */
/* in the main programs (2D :67-70, 3D :68-71).  Arrays start at zero.  */
void F(or_initialize)(CTX *c, REAL *p, REAL *u, REAL *v, REAL *w) {
  const int m = c->m, n = c->n, l = c->l;
  memset(p, 0, c->ncell * sizeof(REAL));
  memset(u, 0, c->ncell * sizeof(REAL));
  memset(v, 0, c->ncell * sizeof(REAL));
  if (w) memset(w, 0, c->ncell * sizeof(REAL));
  if (c->dim == 2) {
    const REAL pai = (REAL)atan(R(1.)) * R(4.);
    for (int j = 1; j <= n; j++)
      for (int i = 1; i <= m; i++) {
        u[I2(i, j)] = c->inlet_velocity * (REAL)cos(c->aoa / R(180) * pai);
        v[I2(i, j)] = c->inlet_velocity * (REAL)sin(c->aoa / R(180) * pai);
        if (c->inflow_porosity) { /* ibm_2d_backstep_omp_cpu.f90:615-618 */
          u[I2(i, j)] = u[I2(i, j)] * c->poro[I2(i, j)];
          v[I2(i, j)] = v[I2(i, j)] * c->poro[I2(i, j)];
        }
        p[I2(i, j)] = c->outlet_pressure;
      }
  } else if (c->wall_mode) { /* air-condition initial_conditions (:1174-1209) */
    for (int k = 1; k <= l; k++)
      for (int j = 1; j <= n; j++)
        for (int i = 1; i <= m; i++) {
          u[I3(i, j, k)] = R(0.);
          v[I3(i, j, k)] = R(0.);
          w[I3(i, j, k)] = R(0.);
          p[I3(i, j, k)] = c->outlet_pressure;
        }
  } else {
    const REAL pi = (REAL)atan(R(1.)) * R(4.);
    for (int k = 1; k <= l; k++)
      for (int j = 1; j <= n; j++)
        for (int i = 1; i <= m; i++) {
          u[I3(i, j, k)] = c->inlet_velocity * (REAL)cos(c->aoa / R(360) * pi);
          v[I3(i, j, k)] = c->inlet_velocity * (REAL)sin(c->aoa / R(360) * pi);
          if (c->inflow_porosity) {
            u[I3(i, j, k)] = u[I3(i, j, k)] * c->poro[I3(i, j, k)];
            v[I3(i, j, k)] = v[I3(i, j, k)] * c->poro[I3(i, j, k)];
          }
          w[I3(i, j, k)] = R(0.);
          p[I3(i, j, k)] = c->outlet_pressure;
        }
  }
  F(or_boundary)(c, p, u, v, w);
}

/* ------------------------------------------------------------------ */
/* solve_p part 1: divergence of u_old (2D :172-194, 3D :185-222).       */
void F(or_divergence)(CTX *c, const REAL *uo, const REAL *vo, const REAL *wo) {
  const int m = c->m, n = c->n, l = c->l;
  const REAL dx = c->dx, dy = c->dy, dz = c->dz;
  REAL *div = c->div;
  if (c->dim == 2) {
#pragma omp parallel for
    for (int i = 1; i <= m; i++)
      for (int j = 1; j <= n; j++)
        /* the v-term divides by dx in the reference (:176) */
        div[I2(i, j)] = (uo[I2(i + 1, j)] - uo[I2(i - 1, j)]) / dx * R(.5) +
                        (vo[I2(i, j + 1)] - vo[I2(i, j - 1)]) / dx * R(.5);
    for (int j = 1; j <= n; j++) {
      div[I2(0, j)] = R(0.);
      div[I2(m + 1, j)] = R(0.);
    }
    for (int i = 1; i <= m; i++) {
      div[I2(i, 0)] = div[I2(i, n)];
      div[I2(i, n + 1)] = div[I2(i, 1)];
    }
  } else {
#pragma omp parallel for
    for (int k = 1; k <= l; k++)
      for (int j = 1; j <= n; j++)
        for (int i = 1; i <= m; i++)
          div[I3(i, j, k)] = (uo[I3(i + 1, j, k)] - uo[I3(i - 1, j, k)]) / dx * R(0.5) +
                             (vo[I3(i, j + 1, k)] - vo[I3(i, j - 1, k)]) / dy * R(0.5) +
                             (wo[I3(i, j, k + 1)] - wo[I3(i, j, k - 1)]) / dz * R(0.5);
#pragma omp parallel for
    for (int k = 1; k <= l; k++)
      for (int j = 1; j <= n; j++) {
        div[I3(0, j, k)] = R(0.);
        div[I3(m + 1, j, k)] = R(0.);
      }
    if (c->wall_mode) { /* air-condition :210-238: every face ghost 0 */
      for (int j = 1; j <= n; j++)
        for (int i = 1; i <= m; i++) {
          div[I3(i, j, 0)] = R(0.);
          div[I3(i, j, l + 1)] = R(0.);
        }
      for (int k = 1; k <= l; k++)
        for (int i = 1; i <= m; i++) {
          div[I3(i, 0, k)] = R(0.);
          div[I3(i, n + 1, k)] = R(0.);
        }
      return;
    }
#pragma omp parallel for
    for (int k = 1; k <= l; k++)
      for (int i = 1; i <= m; i++) {
        div[I3(i, 0, k)] = div[I3(i, n, k)];
        div[I3(i, n + 1, k)] = div[I3(i, 1, k)];
      }
#pragma omp parallel for
    for (int j = 1; j <= n; j++)
      for (int i = 1; i <= m; i++) {
        div[I3(i, j, 0)] = div[I3(i, j, l)];
        div[I3(i, j, l + 1)] = div[I3(i, j, 1)];
      }
  }
}

/* ------------------------------------------------------------------ */
/* solve_p part 2: predictor (2D :200-258, 3D :228-381).                 */
void F(or_predictor)(CTX *c, REAL *u, REAL *v, REAL *w, const REAL *uo, const REAL *vo,
                     const REAL *wo, const REAL *po) {
  const int m = c->m, n = c->n, l = c->l;
  const REAL dx = c->dx, dy = c->dy, dz = c->dz, dt = c->dt;
  const REAL xnue = c->xnue, xlambda = c->xlambda, thickness = c->thickness;
  const REAL alpha = R(32.0);
  const REAL *div = c->div;
  if (c->dim == 2) {
#pragma omp parallel for
    for (int i = 1; i <= m; i++)
      for (int j = 1; j <= n; j++) {
        REAL t;
        t = uo[I2(i, j)] - dt * (uo[I2(i, j)] * (uo[I2(i + 1, j)] - uo[I2(i - 1, j)]) / dx / R(2.));
        t = t - dt * (vo[I2(i, j)] * (uo[I2(i, j + 1)] - uo[I2(i, j - 1)]) / dy / R(2.));
        t = t + dt * xnue * (uo[I2(i + 1, j)] - R(2.) * uo[I2(i, j)] + uo[I2(i - 1, j)]) / dx / dx;
        t = t + dt * xnue * (uo[I2(i, j + 1)] - R(2.) * uo[I2(i, j)] + uo[I2(i, j - 1)]) / dy / dy;
        t = t + dt * (xnue + xlambda) * (div[I2(i + 1, j)] - div[I2(i - 1, j)]) / dx * R(.5);
        t = t + dt *
                    (((uo[I2(i + 1, j)] - uo[I2(i - 1, j)]) / dx * R(.5) +
                      (uo[I2(i + 1, j)] - uo[I2(i - 1, j)]) / dx * R(.5)) *
                         xnue * (po[I2(i + 1, j)] - po[I2(i - 1, j)]) / dx * R(.5) +
                     ((uo[I2(i, j + 1)] - uo[I2(i, j - 1)]) / dy * R(.5) +
                      (vo[I2(i + 1, j)] - vo[I2(i - 1, j)]) / dx * R(.5)) *
                         xnue * (po[I2(i, j + 1)] - po[I2(i, j - 1)]) / dy * R(.5) +
                     div[I2(i, j)] * (po[I2(i + 1, j)] - po[I2(i - 1, j)]) / dx * R(0.5) * xlambda) /
                    po[I2(i, j)];
        if (c->nonslip)
          t = t - dt * xnue * uo[I2(i, j)] / ((thickness * dx) * (thickness * dx)) * alpha *
                      po[I2(i, j)] * (R(1.) - po[I2(i, j)]) * (R(1.) - po[I2(i, j)]);
        u[I2(i, j)] = t;
      }
#pragma omp parallel for
    for (int i = 1; i <= m; i++)
      for (int j = 1; j <= n; j++) {
        REAL t;
        t = vo[I2(i, j)] - dt * (uo[I2(i, j)] * (vo[I2(i + 1, j)] - vo[I2(i - 1, j)]) / dx / R(2.));
        t = t - dt * (vo[I2(i, j)] * (vo[I2(i, j + 1)] - vo[I2(i, j - 1)]) / dy / R(2.));
        t = t + dt * xnue * (vo[I2(i + 1, j)] - R(2.) * vo[I2(i, j)] + vo[I2(i - 1, j)]) / dx / dx;
        t = t + dt * xnue * (vo[I2(i, j + 1)] - R(2.) * vo[I2(i, j)] + vo[I2(i, j - 1)]) / dy / dy;
        t = t + dt * (xnue + xlambda) * (div[I2(i, j + 1)] - div[I2(i, j - 1)]) / dy * R(.5);
        t = t + dt *
                    (((vo[I2(i + 1, j)] - vo[I2(i - 1, j)]) / dx * R(.5) +
                      (uo[I2(i, j + 1)] - uo[I2(i, j - 1)]) / dy * R(.5)) *
                         xnue * (po[I2(i + 1, j)] - po[I2(i - 1, j)]) / dx * R(.5) +
                     ((vo[I2(i, j + 1)] - vo[I2(i, j - 1)]) / dy * R(.5) +
                      (vo[I2(i, j + 1)] - vo[I2(i, j - 1)]) / dy * R(.5)) *
                         xnue * (po[I2(i, j + 1)] - po[I2(i, j - 1)]) / dy * R(.5) +
                     div[I2(i, j)] * (po[I2(i, j + 1)] - po[I2(i, j - 1)]) / dy * R(0.5) * xlambda) /
                    po[I2(i, j)];
        if (c->nonslip)
          t = t - dt * xnue * vo[I2(i, j)] / ((thickness * dx) * (thickness * dx)) * alpha *
                      po[I2(i, j)] * (R(1.) - po[I2(i, j)]) * (R(1.) - po[I2(i, j)]);
        v[I2(i, j)] = t;
      }
  } else {
#define UO(a, b, d) uo[I3(a, b, d)]
#define VO(a, b, d) vo[I3(a, b, d)]
#define WO(a, b, d) wo[I3(a, b, d)]
#define PO(a, b, d) po[I3(a, b, d)]
#define DV(a, b, d) div[I3(a, b, d)]
#pragma omp parallel for
    for (int k = 1; k <= l; k++)
      for (int j = 1; j <= n; j++)
        for (int i = 1; i <= m; i++) {
          REAL t;
          t = UO(i, j, k) - dt * UO(i, j, k) * (UO(i + 1, j, k) - UO(i - 1, j, k)) / dx * R(0.5);
          t = t - dt * VO(i, j, k) * (UO(i, j + 1, k) - UO(i, j - 1, k)) / dy * R(0.5);
          t = t - dt * WO(i, j, k) * (UO(i, j, k + 1) - UO(i, j, k - 1)) / dz * R(0.5);
          t = t + dt * xnue * (UO(i + 1, j, k) - R(2.) * UO(i, j, k) + UO(i - 1, j, k)) / dx / dx;
          t = t + dt * xnue * (UO(i, j + 1, k) - R(2.) * UO(i, j, k) + UO(i, j - 1, k)) / dy / dy;
          t = t + dt * xnue * (UO(i, j, k + 1) - R(2.) * UO(i, j, k) + UO(i, j, k - 1)) / dz / dz;
          t = t + dt * (xnue + xlambda) * (DV(i + 1, j, k) - DV(i - 1, j, k)) / dx * R(0.5);
          t = t + dt *
                      (((UO(i + 1, j, k) - UO(i - 1, j, k)) / dx * R(0.5) +
                        (UO(i + 1, j, k) - UO(i - 1, j, k)) / dx * R(0.5)) *
                           xnue * (PO(i + 1, j, k) - PO(i - 1, j, k)) / dx * R(0.5) +
                       ((UO(i, j + 1, k) - UO(i, j - 1, k)) / dy * R(0.5) +
                        (VO(i + 1, j, k) - VO(i - 1, j, k)) / dx * R(0.5)) *
                           xnue * (PO(i, j + 1, k) - PO(i, j - 1, k)) / dy * R(0.5) +
                       ((UO(i, j, k + 1) - UO(i, j, k - 1)) / dz * R(0.5) +
                        (WO(i + 1, j, k) - WO(i - 1, j, k)) / dx * R(0.5)) *
                           xnue * (PO(i, j, k + 1) - PO(i, j, k - 1)) / dz * R(0.5) +
                       DV(i, j, k) * (PO(i + 1, j, k) - PO(i - 1, j, k)) / dx * R(0.5) * xlambda) /
                      PO(i, j, k);
          if (c->nonslip)
            t = t - dt * xnue * UO(i, j, k) / ((thickness * dx) * (thickness * dx)) * alpha *
                        PO(i, j, k) * (R(1.) - PO(i, j, k)) * (R(1.) - PO(i, j, k));
          u[I3(i, j, k)] = t;
        }
#pragma omp parallel for
    for (int k = 1; k <= l; k++)
      for (int j = 1; j <= n; j++)
        for (int i = 1; i <= m; i++) {
          REAL t;
          t = VO(i, j, k) - dt * UO(i, j, k) * (VO(i + 1, j, k) - VO(i - 1, j, k)) / dx * R(0.5);
          t = t - dt * VO(i, j, k) * (VO(i, j + 1, k) - VO(i, j - 1, k)) / dy * R(0.5);
          t = t - dt * WO(i, j, k) * (VO(i, j, k + 1) - VO(i, j, k - 1)) / dz * R(0.5);
          t = t + dt * xnue * (VO(i + 1, j, k) - R(2.) * VO(i, j, k) + VO(i - 1, j, k)) / dx / dx;
          t = t + dt * xnue * (VO(i, j + 1, k) - R(2.) * VO(i, j, k) + VO(i, j - 1, k)) / dy / dy;
          t = t + dt * xnue * (VO(i, j, k + 1) - R(2.) * VO(i, j, k) + VO(i, j, k - 1)) / dz / dz;
          t = t + dt * (xnue + xlambda) * (DV(i, j + 1, k) - DV(i, j - 1, k)) / dy * R(0.5);
          t = t + dt *
                      (((VO(i + 1, j, k) - VO(i - 1, j, k)) / dx * R(0.5) +
                        (UO(i, j + 1, k) - UO(i, j - 1, k)) / dy * R(0.5)) *
                           xnue * (PO(i + 1, j, k) - PO(i - 1, j, k)) / dx * R(0.5) +
                       ((VO(i, j + 1, k) - VO(i, j - 1, k)) / dy * R(.5) +
                        (VO(i, j + 1, k) - VO(i, j - 1, k)) / dy * R(0.5)) *
                           xnue * (PO(i, j + 1, k) - PO(i, j - 1, k)) / dy * R(0.5) +
                       ((VO(i, j, k + 1) - VO(i, j, k - 1)) / dz * R(.5) +
                        (WO(i, j + 1, k) - WO(i, j - 1, k)) / dy * R(0.5)) *
                           xnue * (PO(i, j, k + 1) - PO(i, j, k - 1)) / dz * R(0.5) +
                       DV(i, j, k) * (PO(i, j + 1, k) - PO(i, j - 1, k)) / dy * R(0.5) * xlambda) /
                      PO(i, j, k);
          if (c->nonslip)
            t = t - dt * xnue * VO(i, j, k) / ((thickness * dy) * (thickness * dy)) * alpha *
                        PO(i, j, k) * (R(1.) - PO(i, j, k)) * (R(1.) - PO(i, j, k));
          v[I3(i, j, k)] = t;
        }
#pragma omp parallel for
    for (int k = 1; k <= l; k++)
      for (int j = 1; j <= n; j++)
        for (int i = 1; i <= m; i++) {
          REAL t;
          t = WO(i, j, k) - dt * UO(i, j, k) * (WO(i + 1, j, k) - WO(i - 1, j, k)) / dx * R(0.5);
          t = t - dt * VO(i, j, k) * (WO(i, j + 1, k) - WO(i, j - 1, k)) / dy * R(0.5);
          t = t - dt * WO(i, j, k) * (WO(i, j, k + 1) - WO(i, j, k - 1)) / dz * R(0.5);
          t = t + dt * xnue * (WO(i + 1, j, k) - R(2.) * WO(i, j, k) + WO(i - 1, j, k)) / dx / dx;
          t = t + dt * xnue * (WO(i, j + 1, k) - R(2.) * WO(i, j, k) + WO(i, j - 1, k)) / dy / dy;
          t = t + dt * xnue * (WO(i, j, k + 1) - R(2.) * WO(i, j, k) + WO(i, j, k - 1)) / dz / dz;
          t = t + dt * (xnue + xlambda) * (DV(i, j, k + 1) - DV(i, j, k - 1)) / dz * R(0.5);
          t = t + dt *
                      (((WO(i + 1, j, k) - WO(i - 1, j, k)) / dx * R(0.5) +
                        (UO(i, j, k + 1) - UO(i, j, k - 1)) / dz * R(0.5)) *
                           xnue * (PO(i + 1, j, k) - PO(i - 1, j, k)) / dx * R(0.5) +
                       ((WO(i, j + 1, k) - WO(i, j - 1, k)) / dy * R(0.5) +
                        (VO(i, j, k + 1) - VO(i, j, k - 1)) / dz * R(0.5)) *
                           xnue * (PO(i, j + 1, k) - PO(i, j - 1, k)) / dy * R(0.5) +
                       ((WO(i, j, k + 1) - WO(i, j, k - 1)) / dz * R(0.5) +
                        (WO(i, j, k + 1) - WO(i, j, k - 1)) / dz * R(0.5)) *
                           xnue * (PO(i, j, k + 1) - PO(i, j, k - 1)) / dz * R(0.5) +
                       DV(i, j, k) * (PO(i, j, k + 1) - PO(i, j, k - 1)) / dz * R(0.5) * xlambda) /
                      PO(i, j, k);
          if (c->nonslip)
            t = t - dt * xnue * WO(i, j, k) / ((thickness * dz) * (thickness * dz)) * alpha *
                        PO(i, j, k) * (R(1.) - PO(i, j, k)) * (R(1.) - PO(i, j, k));
          w[I3(i, j, k)] = t;
        }
#undef UO
#undef VO
#undef WO
#undef PO
#undef DV
  }
}

/* ------------------------------------------------------------------ */
/* solve_p part 3: matrix coefficients and RHS (2D :262-279, 3D :386-414) */
void F(or_coefficients)(CTX *c, const REAL *u, const REAL *v, const REAL *w, const REAL *po) {
  const int m = c->m, n = c->n, l = c->l;
  const REAL dx = c->dx, dy = c->dy, dz = c->dz, dt = c->dt, density = c->density;
  const REAL small = R(1.e-6);
  if (c->dim == 2) {
#pragma omp parallel for
    for (int i = 1; i <= m; i++)
      for (int j = 1; j <= n; j++) {
        const size_t q = I2(i, j);
        c->ae[q] = dt * rmax(small, (po[I2(i + 1, j)] + po[q]) * R(0.5)) / dx / dx;
        c->aw[q] = dt * rmax(small, (po[q] + po[I2(i - 1, j)]) * R(0.5)) / dx / dx;
        c->an[q] = dt * rmax(small, (po[I2(i, j + 1)] + po[q]) * R(0.5)) / dy / dy;
        c->as[q] = dt * rmax(small, (po[q] + po[I2(i, j - 1)]) * R(0.5)) / dy / dy;
        c->ap[q] = -c->ae[q] - c->aw[q] - c->an[q] - c->as[q];
        c->bb[q] = ((po[I2(i + 1, j)] * u[q] + po[q] * u[I2(i + 1, j)]) * R(0.5) -
                    (po[I2(i - 1, j)] * u[q] + po[q] * u[I2(i - 1, j)]) * R(0.5)) *
                       density / dx +
                   ((po[I2(i, j + 1)] * v[q] + po[q] * v[I2(i, j + 1)]) * R(0.5) -
                    (po[I2(i, j - 1)] * v[q] + po[q] * v[I2(i, j - 1)]) * R(0.5)) *
                       density / dy;
      }
  } else {
#pragma omp parallel for
    for (int k = 1; k <= l; k++)
      for (int j = 1; j <= n; j++)
        for (int i = 1; i <= m; i++) {
          const size_t q = I3(i, j, k);
          c->ae[q] = dt * rmax(small, (po[I3(i + 1, j, k)] + po[q]) * R(0.5)) / dx / dx;
          c->aw[q] = dt * rmax(small, (po[q] + po[I3(i - 1, j, k)]) * R(0.5)) / dx / dx;
          c->an[q] = dt * rmax(small, (po[I3(i, j + 1, k)] + po[q]) * R(0.5)) / dy / dy;
          c->as[q] = dt * rmax(small, (po[q] + po[I3(i, j - 1, k)]) * R(0.5)) / dy / dy;
          c->at[q] = dt * rmax(small, (po[I3(i, j, k + 1)] + po[q]) * R(0.5)) / dz / dz;
          c->ab[q] = dt * rmax(small, (po[q] + po[I3(i, j, k - 1)]) * R(0.5)) / dz / dz;
          c->ap[q] = -c->ae[q] - c->aw[q] - c->an[q] - c->as[q] - c->at[q] - c->ab[q];
          c->bb[q] = ((po[I3(i + 1, j, k)] * u[q] + po[q] * u[I3(i + 1, j, k)]) * R(0.5) -
                      (po[I3(i - 1, j, k)] * u[q] + po[q] * u[I3(i - 1, j, k)]) * R(0.5)) *
                         density / dx +
                     ((po[I3(i, j + 1, k)] * v[q] + po[q] * v[I3(i, j + 1, k)]) * R(0.5) -
                      (po[I3(i, j - 1, k)] * v[q] + po[q] * v[I3(i, j - 1, k)]) * R(0.5)) *
                         density / dy +
                     ((po[I3(i, j, k + 1)] * w[q] + po[q] * w[I3(i, j, k + 1)]) * R(0.5) -
                      (po[I3(i, j, k - 1)] * w[q] + po[q] * w[I3(i, j, k - 1)]) * R(0.5)) *
                         density / dz;
        }
  }
}

/* boundrary_matrix: 2D :410-454, 3D :618-663 (omp semantics). */
/* boundary_matrix of the air-condition program (:665-867), face by face in
   the reference's order over the ghost-inclusive ranges: a wall (or an inlet)
   folds the outward coefficient into the inward one (dp/dn = 0); an outlet
   cell with porosity >= 0.9 adds a_out * p_ghost to bb and zeroes all six
   coefficients (the top outlet starts from bb of plane 1, as the reference
   writes it). */
static void F(wall_matrix)(CTX *c, const REAL *p) {
  const int m = c->m, n = c->n, l = c->l;
  REAL *ae = c->ae, *aw = c->aw, *an = c->an, *as = c->as, *at = c->at, *ab = c->ab, *bb = c->bb;
  const REAL *po = c->poro, lim = R(0.9);
#define PF_ZERO6(q) (ae[q] = aw[q] = an[q] = as[q] = at[q] = ab[q] = R(0.))
  for (int i = 0; i <= m + 1; i++) /* top, k = l */
    for (int j = 0; j <= n + 1; j++) {
      const size_t q = I3(i, j, l);
      const int t = c->walls[0];
      if (t == 0 || t == 1 || (t == 2 && po[q] < lim)) {
        ab[q] = ab[q] + at[q];
        at[q] = R(0.);
      } else if (t == 2) {
        bb[q] = bb[I3(i, j, 1)] + at[q] * p[I3(i, j, l + 1)];
        PF_ZERO6(q);
      }
    }
  for (int i = 0; i <= m + 1; i++) /* bottom, k = 1 */
    for (int j = 0; j <= n + 1; j++) {
      const size_t q = I3(i, j, 1);
      const int t = c->walls[1];
      if (t == 0 || t == 1 || (t == 2 && po[q] < lim)) {
        at[q] = at[q] + ab[q];
        ab[q] = R(0.);
      } else if (t == 2) {
        bb[q] = bb[q] + ab[q] * p[I3(i, j, 0)];
        PF_ZERO6(q);
      }
    }
  for (int j = 0; j <= n + 1; j++) /* east, i = m */
    for (int k = 0; k <= l + 1; k++) {
      const size_t q = I3(m, j, k);
      const int t = c->walls[2];
      if (t == 0 || t == 1 || (t == 2 && po[q] < lim)) {
        aw[q] = aw[q] + ae[q];
        ae[q] = R(0.);
      } else if (t == 2) {
        bb[q] = bb[q] + ae[q] * p[I3(m + 1, j, k)];
        PF_ZERO6(q);
      }
    }
  for (int j = 0; j <= n + 1; j++) /* west, i = 1 */
    for (int k = 0; k <= l + 1; k++) {
      const size_t q = I3(1, j, k);
      const int t = c->walls[3];
      if (t == 0 || t == 1 || (t == 2 && po[q] < lim)) {
        ae[q] = ae[q] + aw[q];
        aw[q] = R(0.);
      } else if (t == 2) {
        bb[q] = bb[q] + aw[q] * p[I3(0, j, k)];
        PF_ZERO6(q);
      }
    }
  for (int i = 0; i <= m + 1; i++) /* north, j = n */
    for (int k = 0; k <= l + 1; k++) {
      const size_t q = I3(i, n, k);
      const int t = c->walls[4];
      if (t == 0 || t == 1 || (t == 2 && po[q] < lim)) {
        as[q] = as[q] + an[q];
        an[q] = R(0.);
      } else if (t == 2) {
        bb[q] = bb[q] + an[q] * p[I3(i, n + 1, k)];
        PF_ZERO6(q);
      }
    }
  for (int i = 0; i <= m + 1; i++) /* south, j = 1 */
    for (int k = 0; k <= l + 1; k++) {
      const size_t q = I3(i, 1, k);
      const int t = c->walls[5];
      if (t == 0 || t == 1 || (t == 2 && po[q] < lim)) {
        an[q] = an[q] + as[q];
        as[q] = R(0.);
      } else if (t == 2) {
        bb[q] = bb[q] + as[q] * p[I3(i, 0, k)];
        PF_ZERO6(q);
      }
    }
#undef PF_ZERO6
}

void F(or_boundary_matrix)(CTX *c, const REAL *p) {
  const int m = c->m, n = c->n, l = c->l;
  if (c->wall_mode) {
    F(wall_matrix)(c, p);
    return;
  }
  if (c->dim == 2) {
    for (int j = 1; j <= n; j++) {
      c->ae[I2(1, j)] = c->ae[I2(1, j)] + c->aw[I2(1, j)];
      c->aw[I2(1, j)] = R(0.);
    }
    for (int j = 1; j <= n; j++) {
      c->bb[I2(m, j)] = c->bb[I2(m, j)] + c->ae[I2(m, j)] * p[I2(m + 1, j)];
      c->ae[I2(m, j)] = R(0.);
      c->aw[I2(m, j)] = R(0.);
      c->an[I2(m, j)] = R(0.);
      c->as[I2(m, j)] = R(0.);
    }
    if (c->slip_y) { /* :440-450, the commented symmetry rows (dp/dy = 0) */
      for (int i = 1; i <= m; i++) {
        c->an[I2(i, 1)] = c->an[I2(i, 1)] + c->as[I2(i, 1)];
        c->as[I2(i, 1)] = R(0.);
      }
      for (int i = 1; i <= m; i++) {
        c->as[I2(i, n)] = c->as[I2(i, n)] + c->an[I2(i, n)];
        c->an[I2(i, n)] = R(0.);
      }
    }
  } else {
    for (int k = 1; k <= l; k++)
      for (int j = 1; j <= n; j++) {
        c->ae[I3(1, j, k)] = c->ae[I3(1, j, k)] + c->aw[I3(1, j, k)];
        c->aw[I3(1, j, k)] = R(0.);
      }
    for (int k = 1; k <= l; k++)
      for (int j = 1; j <= n; j++) {
        const size_t q = I3(m, j, k);
        c->bb[q] = c->bb[q] + c->ae[q] * p[I3(m + 1, j, k)];
        c->ae[q] = R(0.);
        c->aw[q] = R(0.);
        c->an[q] = R(0.);
        c->as[q] = R(0.);
        c->at[q] = R(0.);
        c->ab[q] = R(0.);
      }
  }
}

/* ------------------------------------------------------------------ */
/* solve_matrix_vec_omp: 2D :293-406, 3D :433-614.                        */
/* Red-black SOR with the reference's linear-index colour mapping and   */
/* p_old snapshots.  Returns the reference's `error` (printed there).   */
double F(or_sor)(CTX *c, REAL *p) {
  const int m = c->m, n = c->n, l = c->l;
  const REAL relux = c->relux;
  REAL *po = c->p_old;
  REAL error = R(0.0);
  if (c->dim == 2) {
    for (int iter = 1; iter <= c->iter_max; iter++) {
      for (int i = 1; i <= m; i++) {
        p[I2(i, 0)] = p[I2(i, n)];
        p[I2(i, n + 1)] = p[I2(i, 1)];
      }
#pragma omp parallel for
      for (int i = 0; i <= m + 1; i++)
        for (int j = 0; j <= n + 1; j++) po[I2(i, j)] = p[I2(i, j)];
#pragma omp parallel for reduction(max : error)
      for (int k = 2; k <= m * n; k += 2) {
        int j = (k - 1) / m + 1;
        int i = k - (j - 1) * m;
        if (m % 2 == 0 && j % 2 == 0) i = i - 1;
        const size_t q = I2(i, j);
        p[q] = (c->bb[q] - c->ae[q] * po[I2(i + 1, j)] - c->aw[q] * po[I2(i - 1, j)] -
                c->an[q] * po[I2(i, j + 1)] - c->as[q] * po[I2(i, j - 1)]) /
                   c->ap[q] * relux +
               po[q] * (R(1.) - relux);
        REAL d = (REAL)fabs((double)(p[q] - po[q]));
        error = rmax(error, d);
      }
      for (int i = 1; i <= m; i++) {
        p[I2(i, 0)] = p[I2(i, n)];
        p[I2(i, n + 1)] = p[I2(i, 1)];
      }
#pragma omp parallel for
      for (int i = 0; i <= m + 1; i++)
        for (int j = 0; j <= n + 1; j++) po[I2(i, j)] = p[I2(i, j)];
#pragma omp parallel for reduction(max : error)
      for (int k = 1; k <= m * n; k += 2) {
        int j = (k - 1) / m + 1;
        int i = k - (j - 1) * m;
        if (m % 2 == 0 && j % 2 == 0) i = i + 1;
        const size_t q = I2(i, j);
        p[q] = (c->bb[q] - c->ae[q] * po[I2(i + 1, j)] - c->aw[q] * po[I2(i - 1, j)] -
                c->an[q] * po[I2(i, j + 1)] - c->as[q] * po[I2(i, j - 1)]) /
                   c->ap[q] * relux +
               po[q] * (R(1.) - relux);
        REAL d = (REAL)fabs((double)(p[q] - po[q]));
        error = rmax(error, d);
      }
    }
    for (int i = 1; i <= m; i++) {
      p[I2(i, 0)] = p[I2(i, n)];
      p[I2(i, n + 1)] = p[I2(i, 1)];
    }
  } else {
    const long mn = (long)m * n, mnl = (long)m * n * l;
    for (int iter = 1; iter <= c->iter_max; iter++) {
      for (int pass = 0; pass < 2; pass++) {
        /* the air-condition program has no periodic refresh (:507-526) */
#pragma omp parallel for if (!c->wall_mode)
        for (int i = 1; i <= (c->wall_mode ? 0 : m); i++)
          for (int k = 1; k <= l; k++) {
            p[I3(i, 0, k)] = p[I3(i, n, k)];
            p[I3(i, n + 1, k)] = p[I3(i, 1, k)];
          }
#pragma omp parallel for if (!c->wall_mode)
        for (int i = 1; i <= (c->wall_mode ? 0 : m); i++)
          for (int j = 1; j <= n; j++) {
            p[I3(i, j, 0)] = p[I3(i, j, l)];
            p[I3(i, j, l + 1)] = p[I3(i, j, 1)];
          }
        /* The reference nests i,j,k with k innermost; the copy itself is
           order independent, so it is written in storage order here. */
#pragma omp parallel for
        for (int k = 0; k <= l + 1; k++)
          for (int j = 0; j <= n + 1; j++)
            for (int i = 0; i <= m + 1; i++) po[I3(i, j, k)] = p[I3(i, j, k)];
        /* pass 0: "evenspace" ii = 2,4,..  pass 1: "odd space" ii = 1,3,.. */
#pragma omp parallel for
        for (long ii = 2 - pass; ii <= mnl; ii += 2) {
          int k = (int)((ii - 1) / mn + 1);
          int j = (int)(((ii - 1) / m + 1) - (long)(k - 1) * n);
          int i = (int)((ii - (long)(j - 1) * m) - (long)(k - 1) * mn);
          if (m % 2 != 0 && n % 2 == 0 && k % 2 == 0) {
            if (i % 2 != 0)
              j = (pass == 0) ? j - 1 : j + 1;
            else
              j = (pass == 0) ? j + 1 : j - 1;
          } else if (m % 2 == 0 && (j % 2 + k % 2 == 1)) {
            i = (pass == 0) ? i - 1 : i + 1;
          }
          const size_t q = I3(i, j, k);
          p[q] = (c->bb[q] - c->ae[q] * po[I3(i + 1, j, k)] - c->aw[q] * po[I3(i - 1, j, k)] -
                  c->an[q] * po[I3(i, j + 1, k)] - c->as[q] * po[I3(i, j - 1, k)] -
                  c->at[q] * po[I3(i, j, k + 1)] - c->ab[q] * po[I3(i, j, k - 1)]) /
                     c->ap[q] * relux +
                 po[q] * (R(1.) - relux);
        }
      }
#pragma omp parallel for reduction(max : error)
      for (int k = 1; k <= l; k++)
        for (int j = 1; j <= n; j++)
          for (int i = 1; i <= m; i++) {
            REAL d = (REAL)fabs((double)(p[I3(i, j, k)] - po[I3(i, j, k)]));
            error = rmax(error, d);
          }
    }
    if (!c->wall_mode) {
#pragma omp parallel for
      for (int i = 1; i <= m; i++)
        for (int k = 1; k <= l; k++) {
          p[I3(i, 0, k)] = p[I3(i, n, k)];
          p[I3(i, n + 1, k)] = p[I3(i, 1, k)];
        }
#pragma omp parallel for
      for (int i = 1; i <= m; i++)
        for (int j = 1; j <= n; j++) {
          p[I3(i, j, 0)] = p[I3(i, j, l)];
          p[I3(i, j, l + 1)] = p[I3(i, j, 1)];
        }
    }
  }
  c->last_error = error;
  return (double)error;
}

/* solve_p: 2D :142-286, 3D :151-426.  Returns the SOR error. */
double F(or_solve_p)(CTX *c, REAL *p, REAL *u, REAL *v, REAL *w, const REAL *uo, const REAL *vo,
                     const REAL *wo, const REAL *po) {
  F(or_divergence)(c, uo, vo, wo);
  F(or_predictor)(c, u, v, w, uo, vo, wo, po);
  F(or_coefficients)(c, u, v, w, po);
  F(or_boundary_matrix)(c, p);
  return F(or_sor)(c, p);
}

/* projection: 2D :103-115, 3D :109-125. */
void F(or_projection)(CTX *c, const REAL *p, REAL *u, REAL *v, REAL *w) {
  const int m = c->m, n = c->n, l = c->l;
  const REAL dx = c->dx, dy = c->dy, dz = c->dz, dt = c->dt, density = c->density;
  if (c->dim == 2) {
#pragma omp parallel for
    for (int j = 1; j <= n; j++)
      for (int i = 1; i <= m; i++) {
        u[I2(i, j)] = u[I2(i, j)] - dt / density * (p[I2(i + 1, j)] - p[I2(i - 1, j)]) / dx * R(0.5);
        v[I2(i, j)] = v[I2(i, j)] - dt / density * (p[I2(i, j + 1)] - p[I2(i, j - 1)]) / dy * R(0.5);
      }
  } else {
#pragma omp parallel for
    for (int k = 1; k <= l; k++)
      for (int j = 1; j <= n; j++)
        for (int i = 1; i <= m; i++) {
          const size_t q = I3(i, j, k);
          u[q] = u[q] - dt / density * (p[I3(i + 1, j, k)] - p[I3(i - 1, j, k)]) / dx * R(0.5);
          v[q] = v[q] - dt / density * (p[I3(i, j + 1, k)] - p[I3(i, j - 1, k)]) / dy * R(0.5);
          w[q] = w[q] - dt / density * (p[I3(i, j, k + 1)] - p[I3(i, j, k - 1)]) / dz * R(0.5);
        }
  }
}

/* One pass of the main-program step loop (2D :80-125, 3D :81-132),     */
/* repeated nsteps times.  uo/vo/wo are the u_old work arrays.          */
double F(or_step)(CTX *c, int nsteps, REAL *p, REAL *u, REAL *v, REAL *w, REAL *uo, REAL *vo, REAL *wo,
                  const REAL *po) {
  double err = 0.0;
  for (int s = 0; s < nsteps; s++) {
    memcpy(uo, u, c->ncell * sizeof(REAL));
    memcpy(vo, v, c->ncell * sizeof(REAL));
    if (c->dim == 3) memcpy(wo, w, c->ncell * sizeof(REAL));
    err = F(or_solve_p)(c, p, u, v, w, uo, vo, wo, po);
    F(or_projection)(c, p, u, v, w);
    F(or_boundary)(c, p, u, v, w);
  }
  return err;
}

/* Porosity-weighted divergence (output.f90:217-224 2D, :929-941 3D).   */
/* Writes div (interior) when out != NULL; returns max |div|.           */
double F(or_divergence_diag)(CTX *c, const REAL *u, const REAL *v, const REAL *w, const REAL *po,
                             REAL *out) {
  const int m = c->m, n = c->n, l = c->l;
  const REAL dx = c->dx, dy = c->dy, dz = c->dz;
  REAL mx = R(0);
  if (c->dim == 2) {
    for (int i = 1; i <= m; i++)
      for (int j = 1; j <= n; j++) {
        const size_t q = I2(i, j);
        REAL d = ((po[I2(i + 1, j)] * u[q] + po[q] * u[I2(i + 1, j)]) / R(2) -
                  (po[I2(i - 1, j)] * u[q] + po[q] * u[I2(i - 1, j)]) / R(2)) /
                     dx +
                 ((po[I2(i, j + 1)] * v[q] + po[q] * v[I2(i, j + 1)]) / R(2) -
                  (po[I2(i, j - 1)] * v[q] + po[q] * v[I2(i, j - 1)]) / R(2)) /
                     dy;
        if (out) out[q] = d;
        mx = rmax(mx, (REAL)fabs((double)d));
      }
  } else {
#pragma omp parallel for reduction(max : mx)
    for (int k = 1; k <= l; k++)
      for (int j = 1; j <= n; j++)
        for (int i = 1; i <= m; i++) {
          const size_t q = I3(i, j, k);
          REAL d = ((po[I3(i + 1, j, k)] * u[q] + po[q] * u[I3(i + 1, j, k)]) / R(2) -
                    (po[I3(i - 1, j, k)] * u[q] + po[q] * u[I3(i - 1, j, k)]) / R(2)) /
                       dx +
                   ((po[I3(i, j + 1, k)] * v[q] + po[q] * v[I3(i, j + 1, k)]) / R(2) -
                    (po[I3(i, j - 1, k)] * v[q] + po[q] * v[I3(i, j - 1, k)]) / R(2)) /
                       dy +
                   ((po[I3(i, j, k + 1)] * w[q] + po[q] * w[I3(i, j, k + 1)]) / R(2) -
                    (po[I3(i, j, k - 1)] * w[q] + po[q] * w[I3(i, j, k - 1)]) / R(2)) /
                       dz;
          if (out) out[q] = d;
          mx = rmax(mx, (REAL)fabs((double)d));
        }
  }
  return (double)mx;
}

/* ------------------------------------------------------------------ */
/* Force sums of output_force_log_2d (output.f90:244-305) and           */
/* output_force_log_3d (output.f90:1090-1165): pressure part out[0..2]  */
/* and wall-friction part out[3..5], summed sequentially in the         */
/* reference's loop order (2D: i outer, j inner; 3D: k, j, i).          */
void F(or_forces)(CTX *c, const REAL *p, const REAL *u, const REAL *v, const REAL *w, const REAL *po,
                  double *out) {
  const int m = c->m, n = c->n, l = c->l;
  const REAL small = R(1.e-6), alpha = R(32.0);
  const REAL dx = c->dx, dy = c->dy, dz = c->dz, th = c->thickness;
  REAL fpx = R(0), fpy = R(0), fpz = R(0), fvx = R(0), fvy = R(0), fvz = R(0);
  if (c->dim == 2) {
    for (int i = 1; i <= m; i++)
      for (int j = 1; j <= n; j++) {
        const size_t q = I2(i, j);
        const REAL gx = (po[I2(i + 1, j)] - po[I2(i - 1, j)]) * R(0.5);
        const REAL gy = (po[I2(i, j + 1)] - po[I2(i, j - 1)]) * R(0.5);
        const REAL na = (REAL)sqrt((double)(gx * gx + gy * gy));
        const REAL nx = gx / rmax(na, small), ny = gy / rmax(na, small);
        const REAL e = po[q], ee = e * (R(1.0) - e);
        fpx = fpx + (-dx * dy * p[q] * R(2) * e * (R(1.0) - e) / (th * dx) * nx);
        fpy = fpy + (-dx * dy * p[q] * R(2) * e * (R(1.0) - e) / (th * dy) * ny);
        const REAL tx = ee / (th * dx), ty = ee / (th * dy);
        fvx = fvx + (dx * dy * alpha * c->density * c->xnue * (tx * tx) * u[q]);
        fvy = fvy + (dx * dy * alpha * c->density * c->xnue * (ty * ty) * v[q]);
      }
  } else {
    for (int k = 1; k <= l; k++)
      for (int j = 1; j <= n; j++)
        for (int i = 1; i <= m; i++) {
          const size_t q = I3(i, j, k);
          const REAL gx = (po[I3(i + 1, j, k)] - po[I3(i - 1, j, k)]) * R(0.5);
          const REAL gy = (po[I3(i, j + 1, k)] - po[I3(i, j - 1, k)]) * R(0.5);
          const REAL gz = (po[I3(i, j, k + 1)] - po[I3(i, j, k - 1)]) * R(0.5);
          const REAL na = (REAL)sqrt((double)(gx * gx + gy * gy + gz * gz));
          const REAL nx = gx / rmax(na, small), ny = gy / rmax(na, small), nz = gz / rmax(na, small);
          const REAL e = po[q], ee = e * (R(1.0) - e);
          const REAL vol = dx * dy * dz;
          fpx = fpx + (-vol * p[q] * R(2) * e * (R(1.0) - e) / (th * dx) * nx);
          fpy = fpy + (-vol * p[q] * R(2) * e * (R(1.0) - e) / (th * dy) * ny);
          fpz = fpz + (-vol * p[q] * R(2) * e * (R(1.0) - e) / (th * dz) * nz);
          const REAL tx = ee / (th * dx), ty = ee / (th * dy), tz = ee / (th * dz);
          fvx = fvx + (vol * alpha * c->density * c->xnue * (tx * tx) * u[q]);
          fvy = fvy + (vol * alpha * c->density * c->xnue * (ty * ty) * v[q]);
          fvz = fvz + (vol * alpha * c->density * c->xnue * (tz * tz) * w[q]);
        }
  }
  out[0] = (double)fpx;
  out[1] = (double)fpy;
  out[2] = (double)fpz;
  out[3] = (double)fvx;
  out[4] = (double)fvy;
  out[5] = (double)fvz;
}
