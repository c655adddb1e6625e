// pf_geometry.cu -- porosity generated on the device from analytic shapes.
//
// The reference's preprocessing tools write a porosity CSV from a signed
// distance: 0.5*tanh(sdf/thickness) + 0.5 with sdf in cells, positive in the
// fluid (tools/cylinder/make_porosity_2d_cylinder.py:119-122,
// tools/channel/channel.py:27).  For serving, where every request brings a new
// geometry, the same profile is evaluated here on the GPU -- sdf = min over the
// shapes, profile half-width `edge` cells -- straight into a case, skipping the
// host generation and the host->device copy of m*n*l values.  The grid.f90
// threshold clamp and ghost fill are applied as for a CSV input.
#include <cuda_runtime.h>

#include <string>
#include <vector>

#include "pf_case.cuh"
#include "pf_internal.cuh"

namespace pf {
namespace {

// Signed distance of node (x, y[, z]) to shape s (positive outside).
__device__ double shape_sdf(const pf_shape& s, double x, double y, double z) {
  const double dx = x - s.cx, dy = y - s.cy, dz = z - s.cz;
  if (s.kind == PF_SHAPE_SPHERE) return sqrt(dx * dx + dy * dy + dz * dz) - s.a;
  if (s.kind == PF_SHAPE_CIRCLE || s.a == s.b) return sqrt(dx * dx + dy * dy) - s.a;
  // rotated ellipse: first-order distance (q - 1)/|grad q|, q = |(xr/a, yr/b)|
  const double c = cos(s.angle), sn = sin(s.angle);
  const double xr = dx * c + dy * sn, yr = -dx * sn + dy * c;
  const double q = sqrt((xr / s.a) * (xr / s.a) + (yr / s.b) * (yr / s.b));
  const double g = sqrt((xr / (s.a * s.a)) * (xr / (s.a * s.a)) + (yr / (s.b * s.b)) * (yr / (s.b * s.b)));
  return g > 0 ? (q - 1.0) * q / g : -fmin(s.a, s.b);
}

struct ShapeList {
  pf_shape s[PF_MAX_SHAPES];
};

// Interior values in the dense staging layout (m+2)(n+2)(l+2), clamped.
__global__ void k_shapes_porosity(Geo g, Scal s, ShapeList shapes, int nshapes, double edge, double threshold,
                                  double* __restrict__ stage) {
  const int i = blockIdx.x * 32 + threadIdx.x + 1;
  const int j = blockIdx.y * 8 + threadIdx.y + 1;
  const int k = g.dim == 3 ? blockIdx.z + 1 : 0;
  if (i > g.m || j > g.n) return;
  const double x = (i - 1) * s.dx, y = (j - 1) * s.dy, z = g.dim == 3 ? (k - 1) * s.dz : 0.0;
  double d = 1e300;
  for (int q = 0; q < nshapes; q++) d = fmin(d, shape_sdf(shapes.s[q], x, y, z));
  double v = 0.5 * tanh(d / (edge * s.dx)) + 0.5;
  v = v > threshold ? v : threshold;
  stage[(long long)i + (long long)(g.m + 2) * ((long long)j + (long long)(g.n + 2) * k)] = v;
}

// grid_conditions ghosts in the staging layout: x copy, then y (then z) periodic.
__global__ void k_stage_ghost_x(Geo g, double* st) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x + 1;  // 1..n+1
  const int k = g.dim == 3 ? blockIdx.y + 1 : 0;             // 1..l+1
  if (j > g.n + 1) return;
  const long long M = g.m + 2, N = g.n + 2;
  const long long r = M * ((long long)j + N * k);
  st[r] = st[r + 1];
  st[r + g.m + 1] = st[r + g.m];
}
__global__ void k_stage_ghost_y(Geo g, double* st) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;  // 0..m+1
  const int k = blockIdx.y;                               // 0..l+1 (0 in 2D)
  if (i > g.m + 1) return;
  const long long M = g.m + 2, N = g.n + 2;
  st[i + M * (0 + N * k)] = st[i + M * (g.n + N * k)];
  st[i + M * (g.n + 1 + N * k)] = st[i + M * (1 + N * k)];
}
__global__ void k_stage_ghost_z(Geo g, double* st) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;  // 0..m+1
  const int j = blockIdx.y;                               // 0..n+1
  if (i > g.m + 1) return;
  const long long M = g.m + 2, N = g.n + 2;
  st[i + M * (j + N * 0LL)] = st[i + M * (j + N * (long long)g.l)];
  st[i + M * (j + N * (long long)(g.l + 1))] = st[i + M * (j + N * 1LL)];
}

// grid_conditions_wall (grid.f90:208-244): ghosts copy the adjacent interior
// plane, x then y then z, over the ghost-inclusive ranges.
__global__ void k_stage_wall_x(Geo g, double* st) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;  // 0..n+1
  const int k = blockIdx.y;                               // 0..l+1
  if (j > g.n + 1) return;
  const long long M = g.m + 2, N = g.n + 2, r = M * ((long long)j + N * k);
  st[r] = st[r + 1];
  st[r + g.m + 1] = st[r + g.m];
}
__global__ void k_stage_wall_y(Geo g, double* st) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;  // 0..m+1
  const int k = blockIdx.y;                               // 0..l+1
  if (i > g.m + 1) return;
  const long long M = g.m + 2, N = g.n + 2;
  st[i + M * (0 + N * k)] = st[i + M * (1 + N * k)];
  st[i + M * (g.n + 1 + N * k)] = st[i + M * (g.n + N * k)];
}
__global__ void k_stage_wall_z(Geo g, double* st) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;  // 0..m+1
  const int j = blockIdx.y;                               // 0..n+1
  if (i > g.m + 1) return;
  const long long M = g.m + 2, N = g.n + 2;
  st[i + M * (j + N * 0LL)] = st[i + M * (j + N * 1LL)];
  st[i + M * (j + N * (long long)(g.l + 1))] = st[i + M * (j + N * (long long)g.l)];
}

}  // namespace

// Fill c->stage with the clamped, ghost-filled porosity of the shapes.
int geometry_to_stage(pf_case* c, const pf_shape* shapes, int nshapes, double edge) {
  if (nshapes < 0 || nshapes > PF_MAX_SHAPES || (nshapes > 0 && !shapes))
    return fail(PF_E_INVALID, "geometry: between 0 and PF_MAX_SHAPES shapes required");
  if (!(edge > 0)) return fail(PF_E_INVALID, "geometry: edge must be > 0");
  for (int q = 0; q < nshapes; q++) {
    const pf_shape& sh = shapes[q];
    if (sh.kind < PF_SHAPE_CIRCLE || sh.kind > PF_SHAPE_SPHERE || !(sh.a > 0) ||
        (sh.kind == PF_SHAPE_ELLIPSE && !(sh.b > 0)) || (sh.kind == PF_SHAPE_SPHERE && c->g.dim != 3) ||
        (sh.kind != PF_SHAPE_SPHERE && c->g.dim != 2))
      return fail(PF_E_INVALID, "geometry: bad shape " + std::to_string(q));
  }
  const Geo& g = c->g;
  ShapeList d{};
  for (int q = 0; q < nshapes; q++) d.s[q] = shapes[q];
  PF_CUDA(cudaMemsetAsync(c->stage, 0, (size_t)(g.m + 2) * (g.n + 2) * g.Z * sizeof(double), c->st));
  k_shapes_porosity<<<dim3((g.m + 31) / 32, (g.n + 7) / 8, g.dim == 3 ? g.l : 1), dim3(32, 8), 0, c->st>>>(
      g, c->s, d, nshapes, edge, c->prm.threshold, c->stage);
  if (g.wall) {
    k_stage_wall_x<<<dim3((g.n + 2 + 127) / 128, g.l + 2), 128, 0, c->st>>>(g, c->stage);
    k_stage_wall_y<<<dim3((g.m + 2 + 127) / 128, g.l + 2), 128, 0, c->st>>>(g, c->stage);
    k_stage_wall_z<<<dim3((g.m + 2 + 127) / 128, g.n + 2), 128, 0, c->st>>>(g, c->stage);
  } else {
    k_stage_ghost_x<<<dim3((g.n + 1 + 127) / 128, g.dim == 3 ? g.l + 1 : 1), 128, 0, c->st>>>(g, c->stage);
    k_stage_ghost_y<<<dim3((g.m + 2 + 127) / 128, g.dim == 3 ? g.l + 2 : 1), 128, 0, c->st>>>(g, c->stage);
    if (g.dim == 3) k_stage_ghost_z<<<dim3((g.m + 2 + 127) / 128, g.n + 2), 128, 0, c->st>>>(g, c->stage);
  }
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_fail(e, "geometry kernels");
  c->launches += g.dim == 3 ? 4 : 3;
  return PF_OK;
}

}  // namespace pf
