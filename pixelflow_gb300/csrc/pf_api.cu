// pf_api.cu -- the extern "C" entry points of include/pixelflow_gpu.h for
// single cases: set-up, field exchange in the reference's Fortran layout,
// and the step orchestration (stream-ordered launches, CUDA-graph replay,
// profiling events).
#include <cuda_runtime.h>

#include <cmath>
#include <cstdio>
#include <algorithm>
#include <cstring>
#include <string>
#include <vector>

#include "pf_internal.cuh"
#include "pf_case.cuh"

namespace pf {

static thread_local std::string g_last_error;

void set_error(const std::string& msg) { g_last_error = msg; }
int fail(int code, const std::string& msg) {
  set_error(msg);
  return code;
}
int cuda_fail(cudaError_t e, const char* what) {
  return fail(e == cudaErrorMemoryAllocation ? PF_E_NOMEM : PF_E_CUDA,
              std::string(what) + ": " + cudaGetErrorString(e));
}

static int round_up(int a, int b) { return (a + b - 1) / b * b; }

// one field in the dense (m+2)(n+2)[(l+2)] host layout
static size_t dense_bytes(const Geo& g) { return (size_t)(g.m + 2) * (g.n + 2) * g.Z * sizeof(double); }

int make_geo(const pf_params& p, Geo& g) {
  if (p.dim != 2 && p.dim != 3) return fail(PF_E_INVALID, "dim must be 2 or 3");
  if (p.m < 3 || p.n < 3 || (p.dim == 3 && p.l < 3))
    return fail(PF_E_INVALID, "grid sizes must be >= 3 in every direction");
  if (p.m > (1 << 20) || p.n > (1 << 20) || (p.dim == 3 && p.l > (1 << 20)))
    return fail(PF_E_INVALID, "grid size too large");
  g.dim = p.dim;
  g.m = p.m;
  g.n = p.n;
  g.l = p.dim == 3 ? p.l : 1;
  g.X = round_up(g.m + 2, 32);
  g.Y = g.n + 2;
  g.Z = p.dim == 3 ? g.l + 2 : 1;
  g.H = round_up((g.m + 1) / 2 + 1, 32);
  g.nat = (long long)g.X * g.Y * g.Z;
  g.pk = (long long)g.H * g.Y * g.Z;
  const long long dense = (long long)(g.m + 2) * (g.n + 2) * g.Z;
  if (g.nat >= (1LL << 31) || g.pk >= (1LL << 31) || dense >= (1LL << 31))
    return fail(PF_E_INVALID, "grid too large: arrays are limited to 2^31 elements");
  g.wall = p.wall_mode ? 1 : 0;
  if (g.wall && p.dim != 3) return fail(PF_E_INVALID, "wall_mode: the air-condition program is 3D");
  for (int f = 0; g.wall && f < 6; f++)
    if (p.walls[f] < 0 || p.walls[f] > 2) return fail(PF_E_INVALID, "walls: each entry must be 0, 1 or 2");
  g.slip = p.slip_y ? 1 : 0;
  if (g.slip && (p.dim != 2 || g.wall)) return fail(PF_E_INVALID, "slip_y: the symmetry rows are a 2D option");
  if (g.wall) {  // non-periodic: the edge rows' neighbours are the ghost rows
    g.jn_n = g.n + 1;
    g.js_1 = 0;
    g.kt_l = g.l + 1;
    g.kb_1 = 0;
  } else {
    g.jn_n = (g.n % 2 == 0) ? 1 : g.n + 1;
    g.js_1 = (g.n % 2 == 0) ? g.n : 0;
    g.kt_l = (g.l % 2 == 0) ? 1 : g.l + 1;
    g.kb_1 = (g.l % 2 == 0) ? g.l : 0;
  }
  return PF_OK;
}

int make_scal(const pf_params& p, Scal& s) {
  if (!(p.istep_max > 0)) return fail(PF_E_INVALID, "istep_max must be > 0");
  if (p.iter_max < 0) return fail(PF_E_INVALID, "iter_max must be >= 0");
  if (!(p.density != 0.0)) return fail(PF_E_INVALID, "density must be nonzero");
  if (!(p.width > 0 && p.height > 0 && (p.dim == 2 || p.depth > 0)))
    return fail(PF_E_INVALID, "width/height/depth must be > 0");
  s.dx = p.width / double(p.m - 1);
  s.dy = p.height / double(p.n - 1);
  s.dz = p.dim == 3 ? p.depth / double(p.l - 1) : 0.0;
  s.dt = p.time / double(p.istep_max);
  s.xnue = p.xnue;
  s.xlambda = p.xlambda;
  s.density = p.density;
  s.thickness = p.thickness;
  s.threshold = p.threshold;
  s.outlet_pressure = p.outlet_pressure;
  s.omega = p.relux_factor;
  s.nonslip = p.nonslip ? 1 : 0;
  s.inflow_poro = nullptr;  // set to the case's porosity once it is allocated
  s.wall_poro = nullptr;
  for (int f = 0; f < 6; f++) s.walls[f] = p.wall_mode ? p.walls[f] : 0;
  const double pi = std::atan(1.0) * 4.0;
  // boundary(): 2D cos(AoA/180*pi) (ibm_2d:478), 3D cos(AoA/1300*pi) (ibm_3d:695)
  const double ab = p.dim == 3 ? p.aoa / 1300.0 * pi : p.aoa / 180.0 * pi;
  s.inlet_u = p.inlet_velocity * std::cos(ab);
  s.inlet_v = p.inlet_velocity * std::sin(ab);
  s.inlet_w = 0.0;
  s.inlet_velocity = p.inlet_velocity;
  // initial_conditions(): 2D AoA/180 (ibm_2d:560), 3D AoA/360 (ibm_3d:782)
  const double ai = p.dim == 3 ? p.aoa / 360.0 * pi : p.aoa / 180.0 * pi;
  s.init_u = p.inlet_velocity * std::cos(ai);
  s.init_v = p.inlet_velocity * std::sin(ai);
  s.hx = 0.5 / s.dx;
  s.hy = 0.5 / s.dy;
  s.hz = p.dim == 3 ? 0.5 / s.dz : 0.0;
  s.ix2 = 1.0 / (s.dx * s.dx);
  s.iy2 = 1.0 / (s.dy * s.dy);
  s.iz2 = p.dim == 3 ? 1.0 / (s.dz * s.dz) : 0.0;
  s.iso = p.dim == 3 && s.dx == s.dy && s.dx == s.dz;
  s.dtnu = s.dt * s.xnue;
  s.dtnl = s.dt * (s.xnue + s.xlambda);
  s.mdt_h = -s.dt * s.hx;
  s.dtnu_i2 = s.dtnu * s.ix2;
  s.dtnl_h = s.dtnl * s.hx;
  const double cdt = s.dt / s.density;
  s.pgx = cdt * 0.5 / s.dx;
  s.pgy = cdt * 0.5 / s.dy;
  s.pgz = p.dim == 3 ? cdt * 0.5 / s.dz : 0.0;
  s.hxf = (float)s.hx;
  s.hyf = (float)s.hy;
  s.hzf = (float)s.hz;
  s.ix2f = (float)s.ix2;
  s.iy2f = (float)s.iy2;
  s.iz2f = (float)s.iz2;
  s.dtf = (float)s.dt;
  s.nuf = (float)s.xnue;
  s.lamf = (float)s.xlambda;
  s.dtnuf = (float)s.dtnu;
  s.dtnlf = (float)s.dtnl;
  s.pgxf = (float)s.pgx;
  s.pgyf = (float)s.pgy;
  s.pgzf = (float)s.pgz;
  return PF_OK;
}

// Porosity with ghosts in the dense staging layout, as grid_conditions does:
// clamp max(value, threshold) (grid.f90:43), x-ghost copy, then periodic y
// (and z) ghosts (grid.f90:92-106 2D, :349-378 3D).
void build_porosity(const Geo& g, double threshold, const double* vals, std::vector<double>& out) {
  const int m = g.m, n = g.n, l = g.l;
  const long long M = m + 2, N = n + 2;
  out.assign((size_t)M * N * g.Z, 0.0);
  auto at = [&](int i, int j, int k) -> double& { return out[(size_t)i + M * ((size_t)j + N * k)]; };
  const int k0 = g.dim == 3 ? 1 : 0, k1 = g.dim == 3 ? l : 0;
  size_t q = 0;
  for (int k = k0; k <= k1; k++)
    for (int j = 1; j <= n; j++)
      for (int i = 1; i <= m; i++) {
        const double v = vals[q++];
        at(i, j, k) = v > threshold ? v : threshold;
      }
  if (g.wall) {  // grid_conditions_wall (grid.f90:208-244): copies x, y, z
    for (int j = 0; j <= n + 1; j++)
      for (int k = 0; k <= l + 1; k++) {
        at(0, j, k) = at(1, j, k);
        at(m + 1, j, k) = at(m, j, k);
      }
    for (int i = 0; i <= m + 1; i++)
      for (int k = 0; k <= l + 1; k++) {
        at(i, 0, k) = at(i, 1, k);
        at(i, n + 1, k) = at(i, n, k);
      }
    for (int i = 0; i <= m + 1; i++)
      for (int j = 0; j <= n + 1; j++) {
        at(i, j, 0) = at(i, j, 1);
        at(i, j, l + 1) = at(i, j, l);
      }
    return;
  }
  if (g.dim == 2) {
    for (int j = 1; j <= n + 1; j++) {
      at(0, j, 0) = at(1, j, 0);
      at(m + 1, j, 0) = at(m, j, 0);
    }
    for (int i = 0; i <= m + 1; i++) {
      at(i, 0, 0) = at(i, n, 0);
      at(i, n + 1, 0) = at(i, 1, 0);
    }
  } else {
    for (int j = 1; j <= n + 1; j++)
      for (int k = 1; k <= l + 1; k++) {
        at(0, j, k) = at(1, j, k);
        at(m + 1, j, k) = at(m, j, k);
      }
    for (int i = 0; i <= m + 1; i++)
      for (int k = 0; k <= l + 1; k++) {
        at(i, 0, k) = at(i, n, k);
        at(i, n + 1, k) = at(i, 1, k);
      }
    for (int i = 0; i <= m + 1; i++)
      for (int j = 0; j <= n + 1; j++) {
        at(i, j, 0) = at(i, j, l);
        at(i, j, l + 1) = at(i, j, 1);
      }
  }
}

}  // namespace pf

using namespace pf;

// ---------------------------------------------------------------------------
// Device memory of one case: one allocation carved into 256-byte aligned
// arrays (natural fields, packed p and SOR operator, staging, reductions).
static int case_alloc(pf_case* c) {
  const Geo& g = c->g;
  const size_t nat = (size_t)g.nat * sizeof(double), pk = (size_t)g.pk * sizeof(double);
  const size_t stage = (size_t)(g.m + 2) * (g.n + 2) * g.Z * sizeof(double);
  const bool three = g.dim == 3;
  struct Req {
    void** dst;
    size_t bytes;
    Req(double** d, size_t b) : dst(reinterpret_cast<void**>(d)), bytes(b) {}
  };
  std::vector<Req> req;
  req.push_back({&c->poro, nat});
  req.push_back({&c->gx, nat});
  req.push_back({&c->gy, nat});
  req.push_back({&c->gz, three ? nat : 0});
  req.push_back({&c->rinv, nat});
  req.push_back({&c->damp, nat});
  req.push_back({&c->div, nat});
  for (int b = 0; b < 2; b++) {
    req.push_back({&c->U[b], nat});
    req.push_back({&c->V[b], nat});
    req.push_back({&c->W[b], three ? nat : 0});
  }
  req.push_back({&c->p[0], pk});
  req.push_back({&c->p[1], pk});
  for (int col = 0; col < 2; col++) {
    for (int d = 0; d < 6; d++) req.push_back({&c->C[col].a[d], (d < 2 * g.dim) ? pk : 0});
    req.push_back({&c->C[col].bbn, pk});
    req.push_back({&c->C[col].wap, pk});
    req.push_back({&c->C[col].oadd, pk});
  }
  req.push_back({&c->stage, stage});
  size_t total = 0;
  for (auto& r : req) total += (r.bytes + 255) / 256 * 256;
  total += RED_TOTAL * sizeof(unsigned long long);  // reductions
  char* base = nullptr;
  cudaError_t e = cudaMalloc(&base, total);
  if (e != cudaSuccess) return cuda_fail(e, "cudaMalloc(case)");
  c->base = base;
  c->bytes = total;
  size_t off = 0;
  for (auto& r : req) {
    *r.dst = r.bytes ? static_cast<void*>(base + off) : nullptr;
    off += (r.bytes + 255) / 256 * 256;
  }
  c->red = reinterpret_cast<unsigned long long*>(base + off);
  PF_CUDA(cudaMemsetAsync(base, 0, total, c->st));
  return PF_OK;
}

static void case_free(pf_case* c) {
  if (!c) return;
  for (auto& part : c->gexec)
    for (auto& x : part)
      if (x) cudaGraphExecDestroy(x);
  for (auto& e : c->events) cudaEventDestroy(e);
  for (auto& e : c->ev_io) cudaEventDestroy(e);
  if (c->iostage) cudaFree(c->iostage);
  if (c->st_io) cudaStreamDestroy(c->st_io);
  if (c->base) cudaFree(c->base);
  if (c->list_base) cudaFree(c->list_base);
  if (c->dcl_base) cudaFree(c->dcl_base);
  mixed_free(c);
  if (c->hred) cudaFreeHost(c->hred);
  if (c->snap) cudaFree(c->snap);
  if (c->hsnap) cudaFreeHost(c->hsnap);
  for (auto& e : c->ev_snap)
    if (e) cudaEventDestroy(e);
  if (c->st_snap) cudaStreamDestroy(c->st_snap);
  if (c->st) cudaStreamDestroy(c->st);
  delete c;
}

// solve_p on the device: snapshot (buffer swap), divergence, predictor,
// RHS, SOR.  Only stream-ordered launches, so it can be graph-captured.
// head = false leaves out the divergence and the predictor (pf_step_host
// issues them plane range by plane range as the input planes arrive).
static void enqueue_solve_p(pf_case* c, bool prof, bool head) {
  const Geo& g = c->g;
  const Scal& s = c->s;
  cudaStream_t st = c->st;
  const int o = c->cur, nw = 1 - c->cur;
  const bool track = c->opt.track_sor_error != 0;
  if (track) launch_zero_u64(&c->red[RED_ERR], RED_SLOTS, st);
  if (head) {
    launch_divergence<double>(g, s, c->U[o], c->V[o], c->W[o], c->div, st);
    launch_predictor<double, double>(g, s, c->U[o], c->V[o], c->W[o], c->div, c->gx, c->gy, c->gz, c->rinv,
                                     c->damp, c->U[o], c->V[o], c->W[o], c->U[nw], c->V[nw], c->W[nw], st);
  }
  if (prof) cudaEventRecord(c->ev_cur[4], st);
  launch_rhs<double>(g, s, c->U[nw], c->V[nw], c->W[nw], c->poro, c->gx, c->gy, c->gz, c->C[0], c->C[1], st);
  if (prof) cudaEventRecord(c->ev_cur[1], st);
  const bool halo = periodic_halo(g);
  const double omw = 1.0 - s.omega;
  for (int it = 0; it < c->prm.iter_max; it++) {
    for (int col = 0; col < 2; col++) {
      if (halo) launch_p_halo<double>(g, c->p[0], c->p[1], nullptr, st);
      // 2D tracks both half-sweeps (ibm_2d:351,385); 3D only the second (ibm_3d:575-583)
      unsigned long long* err = (track && (g.dim == 2 || col == 1)) ? &c->red[RED_ERR] : nullptr;
      // the operator loads may precede the dependency wait unless the previous
      // kernel is the RHS, which writes bbn
      const bool early = it > 0 || col > 0 || halo;
      if (c->use_list)
        launch_sor_list(c, col, omw, err, early, st);
      else
        launch_sor_half<double>(g, c->C[col], c->p[col], c->p[1 - col], omw, col, err, nullptr, early, st);
    }
  }
  if (prof) cudaEventRecord(c->ev_cur[2], st);
  if (!g.wall) launch_p_halo<double>(g, c->p[0], c->p[1], nullptr, st);
  c->launches += (head ? 3 : 1) + (track ? 1 : 0) + (g.wall ? 0 : 1) + (int64_t)c->prm.iter_max * 2 * (halo ? 2 : 1);
  c->cur = nw;
}

static void enqueue_projection(pf_case* c) {
  const int b = c->cur;
  c->launches += 1;
  launch_projection<double>(c->g, c->s, c->p[0], c->p[1], c->U[b], c->V[b], c->W[b], c->st);
}

static void enqueue_boundary(pf_case* c) {
  const int b = c->cur;
  c->launches += boundary_launches(c->g);
  launch_boundary<double>(c->g, c->s, c->U[b], c->V[b], c->W[b], c->p[0], c->p[1], c->st);
}

// head = false: the step after the predictor (plain FP64 form only)
static void enqueue_step(pf_case* c, bool prof, bool head = true) {
  if (c->opt.precision == PF_PREC_MIXED) {
    enqueue_solve_p_mixed(c, prof);
    enqueue_projection_mixed(c);
    enqueue_boundary_mixed(c);
  } else {
    enqueue_solve_p(c, prof, head);
    enqueue_projection(c);
    enqueue_boundary(c);
  }
}

static int check_launch(const char* what) {
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_fail(e, what);
  return PF_OK;
}

// Replays the captured step (head = false: the part after the predictor),
// capturing it on first use for the current buffer.
static int step_graph(pf_case* c, bool head = true) {
  const int b = c->cur, part = head ? 0 : 1;
  cudaGraphExec_t& x = c->gexec[part][b];
  if (!x) {
    cudaGraph_t graph = nullptr;
    PF_CUDA(cudaStreamBeginCapture(c->st, cudaStreamCaptureModeThreadLocal));
    const int64_t before = c->launches;
    enqueue_step(c, false, head);
    c->graph_kernels[part][b] = c->launches - before;
    c->launches = before;
    cudaError_t e = cudaStreamEndCapture(c->st, &graph);
    c->cur = b;  // capture only recorded the swap
    if (e != cudaSuccess) return cuda_fail(e, "cudaStreamEndCapture");
    e = cudaGraphInstantiate(&x, graph, 0);
    cudaGraphDestroy(graph);
    if (e != cudaSuccess) return cuda_fail(e, "cudaGraphInstantiate");
  }
  PF_CUDA(cudaGraphLaunch(x, c->st));
  c->launches += c->graph_kernels[part][b];
  c->cur = 1 - b;
  return PF_OK;
}

static int ensure_events(pf_case* c, size_t need) {
  while (c->events.size() < need) {
    cudaEvent_t e;
    PF_CUDA(cudaEventCreate(&e));
    c->events.push_back(e);
  }
  return PF_OK;
}

extern "C" {

const char* pf_last_error(void) { return g_last_error.c_str(); }

const char* pf_strerror(int code) {
  switch (code) {
    case PF_OK: return "ok";
    case PF_E_INVALID: return "invalid argument";
    case PF_E_CUDA: return "CUDA error";
    case PF_E_NOMEM: return "out of device memory";
    case PF_E_NONFINITE: return "non-finite values in the fields";
    case PF_E_TIMEOUT: return "bounded device wait expired";
    case PF_E_STATE: return "invalid state";
    case PF_E_BUSY: return "no free slot";
    default: return "unknown error";
  }
}

int pf_abi_version(void) { return PF_ABI_VERSION; }

int pf_set_device(int device) {
  PF_CUDA(cudaSetDevice(device));
  return PF_OK;
}

int pf_device_count(int* count) {
  if (!count) return fail(PF_E_INVALID, "null argument");
  PF_CUDA(cudaGetDeviceCount(count));
  return PF_OK;
}

void pf_default_options(pf_options* opt) {
  if (!opt) return;
  std::memset(opt, 0, sizeof(*opt));
  opt->precision = PF_PREC_FP64;
  opt->outer_max = 4;
  opt->inner_sweeps = 25;
  opt->track_sor_error = 1;
  opt->dc_tol = 0.0;
  opt->use_graph = 1;
}

}  // extern "C"

// Allocation and scalars of a new case; the porosity comes next.
static int create_case(const pf_params* prm, const pf_options* opt, pf_case** out) {
  *out = nullptr;
  pf_case* c = new pf_case();
  c->prm = *prm;
  if (opt)
    c->opt = *opt;
  else
    pf_default_options(&c->opt);
  int rc = make_geo(c->prm, c->g);
  if (rc == PF_OK) rc = make_scal(c->prm, c->s);
  if (rc == PF_OK && c->opt.precision != PF_PREC_FP64 && c->opt.precision != PF_PREC_MIXED)
    rc = fail(PF_E_INVALID, "unknown precision");
  if (rc == PF_OK && c->opt.precision == PF_PREC_MIXED && (c->opt.outer_max < 0 || c->opt.inner_sweeps < 0))
    rc = fail(PF_E_INVALID, "outer_max and inner_sweeps must be >= 0");
  if (rc == PF_OK && c->g.wall && c->opt.precision != PF_PREC_FP64)
    rc = fail(PF_E_INVALID, "wall_mode: the air-condition program runs in the plain FP64 form only");
  if (rc == PF_OK && c->g.slip && c->opt.precision != PF_PREC_FP64)
    rc = fail(PF_E_INVALID, "slip_y: the symmetry rows run in the plain FP64 form only");
  if (rc == PF_OK && c->opt.sweep_form != PF_SWEEP_AUTO && c->opt.sweep_form != PF_SWEEP_SPLIT &&
      c->opt.sweep_form != PF_SWEEP_FUSED)
    rc = fail(PF_E_INVALID, "unknown sweep_form");
  if (rc == PF_OK && (c->opt.fused_rows < 0 || c->opt.fused_planes < 0))
    rc = fail(PF_E_INVALID, "fused_rows and fused_planes must be >= 0");
  if (rc == PF_OK && c->opt.sor_path != PF_SOR_AUTO && c->opt.sor_path != PF_SOR_CELLS)
    rc = fail(PF_E_INVALID, "unknown sor_path");
  if (rc != PF_OK) {
    delete c;
    return rc;
  }
  cudaError_t e = cudaStreamCreateWithFlags(&c->st, cudaStreamNonBlocking);
  if (e != cudaSuccess) {
    delete c;
    return cuda_fail(e, "cudaStreamCreate");
  }
  rc = case_alloc(c);
  if (rc == PF_OK) {
    e = cudaHostAlloc(&c->hred, RED_TOTAL * sizeof(unsigned long long), cudaHostAllocDefault);
    if (e != cudaSuccess) rc = cuda_fail(e, "cudaHostAlloc");
  }
  if (rc == PF_OK && c->opt.precision == PF_PREC_MIXED) rc = mixed_alloc(c);
  if (rc != PF_OK) {
    case_free(c);
    return rc;
  }
  c->s.inflow_poro = c->prm.inflow_porosity ? c->poro : nullptr;
  c->s.wall_poro = c->g.wall ? c->poro : nullptr;
  *out = c;
  return PF_OK;
}

// Porosity in c->stage (dense, ghosts filled) -> device layouts and the
// time-invariant factors and operator.
static int finish_setup(pf_case* c) {
  const Geo& g = c->g;
  launch_scatter_nat(g, c->stage, c->poro, c->st);
  launch_porosity_factors(g, c->s, c->poro, c->gx, c->gy, c->gz, c->rinv, c->damp, c->st);
  launch_setup_coef(g, c->s, c->poro, c->C[0], c->C[1], c->st);
  if (c->opt.precision == PF_PREC_MIXED) mixed_setup(c);
  int rc = check_launch("case set-up kernels");
  if (rc) return rc;
  PF_CUDA(cudaStreamSynchronize(c->st));
  if (c->opt.sor_path == PF_SOR_AUTO && sor_list_eligible(g)) {
    rc = sor_list_setup(c);
    if (rc) return rc;
    c->use_list = true;
  }
  // the split FP32 sweep walks chunk lists where its grid is more than one
  // wave (a one-wave grid loads its fixed operands ahead of the dependency
  // wait instead, k_sor_dc4_early)
  if (c->opt.precision == PF_PREC_MIXED && c->opt.sor_path == PF_SOR_AUTO && dc_list_eligible(g) && !c->dc_early) {
    rc = dc_list_setup(c);
    if (rc) return rc;
    c->use_dcl = true;
  }
  if (c->opt.precision == PF_PREC_MIXED) return mixed_choose_sweep(c);
  return PF_OK;
}

extern "C" {

int pf_create(const pf_params* prm, const pf_options* opt, const double* porosity_values, pf_case** out) {
  if (!prm || !porosity_values || !out) return fail(PF_E_INVALID, "pf_create: null argument");
  pf_case* c = nullptr;
  int rc = create_case(prm, opt, &c);
  if (rc) return rc;
  // porosity with ghosts (host, once), then the time-invariant factors
  std::vector<double> por;
  build_porosity(c->g, c->prm.threshold, porosity_values, por);
  cudaError_t e =
      cudaMemcpyAsync(c->stage, por.data(), por.size() * sizeof(double), cudaMemcpyHostToDevice, c->st);
  rc = e != cudaSuccess ? cuda_fail(e, "cudaMemcpyAsync(porosity)") : finish_setup(c);
  if (rc) {
    case_free(c);
    return rc;
  }
  *out = c;
  return PF_OK;
}

int pf_create_shapes(const pf_params* prm, const pf_options* opt, const pf_shape* shapes, int nshapes,
                     double edge, pf_case** out) {
  if (!prm || !out) return fail(PF_E_INVALID, "pf_create_shapes: null argument");
  pf_case* c = nullptr;
  int rc = create_case(prm, opt, &c);
  if (rc) return rc;
  rc = geometry_to_stage(c, shapes, nshapes, edge);
  if (rc == PF_OK) rc = finish_setup(c);
  if (rc) {
    case_free(c);
    return rc;
  }
  *out = c;
  return PF_OK;
}

int pf_destroy(pf_case* c) {
  if (!c) return fail(PF_E_INVALID, "pf_destroy: null handle");
  cudaStreamSynchronize(c->st);
  case_free(c);
  return PF_OK;
}

int pf_initial_conditions(pf_case* c) {
  if (!c) return fail(PF_E_INVALID, "null handle");
  const Geo& g = c->g;
  const size_t nat = (size_t)g.nat * sizeof(double), pk = (size_t)g.pk * sizeof(double);
  c->cur = 0;
  PF_CUDA(cudaMemsetAsync(c->U[0], 0, nat, c->st));
  PF_CUDA(cudaMemsetAsync(c->V[0], 0, nat, c->st));
  if (g.dim == 3) PF_CUDA(cudaMemsetAsync(c->W[0], 0, nat, c->st));
  PF_CUDA(cudaMemsetAsync(c->p[0], 0, pk, c->st));
  PF_CUDA(cudaMemsetAsync(c->p[1], 0, pk, c->st));
  launch_initial<double>(g, c->s, c->U[0], c->V[0], c->W[0], c->p[0], c->p[1], c->st);
  launch_boundary<double>(g, c->s, c->U[0], c->V[0], c->W[0], c->p[0], c->p[1], c->st);
  c->launches += 1 + boundary_launches(g);
  if (c->opt.precision == PF_PREC_MIXED) mixed_sync_from_fp64(c);
  return check_launch("pf_initial_conditions");
}

static int check_ld(const pf_case* c, int ld1, int ld2) {
  if (ld1 < c->g.m + 2 || ld2 < c->g.n + 2) return fail(PF_E_INVALID, "leading dimensions smaller than m+2, n+2");
  return PF_OK;
}

static cudaMemcpy3DParms copy_params(const pf_case* c, const void* src, size_t src_pitch, int src_rows,
                                     void* dst, size_t dst_pitch, int dst_rows, cudaMemcpyKind kind) {
  const Geo& g = c->g;
  cudaMemcpy3DParms P;
  std::memset(&P, 0, sizeof(P));
  P.srcPtr = make_cudaPitchedPtr(const_cast<void*>(src), src_pitch, (size_t)(g.m + 2) * sizeof(double), src_rows);
  P.dstPtr = make_cudaPitchedPtr(dst, dst_pitch, (size_t)(g.m + 2) * sizeof(double), dst_rows);
  P.extent = make_cudaExtent((size_t)(g.m + 2) * sizeof(double), g.n + 2, g.Z);
  P.kind = kind;
  return P;
}

// The device error word: a bounded wait inside a kernel that gave up.
static int flags_fail(unsigned long long f) {
  if (f & PF_FLAG_FUSED_TIMEOUT)
    return fail(PF_E_TIMEOUT, "fused correction sweep: a shared-memory staging wait expired");
  return fail(PF_E_CUDA, "unknown device error flag");
}
// Reads the device error word behind everything enqueued on the case's
// stream, so it also waits for that work.
static int check_flags(pf_case* c) {
  PF_CUDA(cudaMemcpyAsync(&c->hred[RED_FLAGS], &c->red[RED_FLAGS], sizeof(unsigned long long),
                          cudaMemcpyDeviceToHost, c->st));
  PF_CUDA(cudaStreamSynchronize(c->st));
  const unsigned long long f = c->hred[RED_FLAGS];
  return f ? flags_fail(f) : PF_OK;
}

int pf_set_state(pf_case* c, const double* u, const double* v, const double* w, const double* p, int ld1,
                 int ld2) {
  if (!c || !u || !v || !p || (c->g.dim == 3 && !w)) return fail(PF_E_INVALID, "pf_set_state: null argument");
  int rc = check_ld(c, ld1, ld2);
  if (rc) return rc;
  const Geo& g = c->g;
  const size_t hp = (size_t)ld1 * sizeof(double), dp = (size_t)g.X * sizeof(double);
  const int b = c->cur;
  const double* src[3] = {u, v, w};
  double* dst[3] = {c->U[b], c->V[b], c->W[b]};
  // Host blocks with exactly the ghosted extents are contiguous: one flat copy
  // into the staging array, then a device kernel into the pitched layout
  // (a pitched copy from the host moves one row per DMA descriptor).
  const bool flat = ld1 == g.m + 2 && ld2 == g.n + 2;
  const size_t dense = (size_t)(g.m + 2) * (g.n + 2) * g.Z * sizeof(double);
  for (int f = 0; f < g.dim; f++) {
    if (flat) {
      PF_CUDA(cudaMemcpyAsync(c->stage, src[f], dense, cudaMemcpyHostToDevice, c->st));
      launch_scatter_nat(g, c->stage, dst[f], c->st);
      c->launches += 1;
    } else {
      cudaMemcpy3DParms P = copy_params(c, src[f], hp, ld2, dst[f], dp, g.Y, cudaMemcpyHostToDevice);
      PF_CUDA(cudaMemcpy3DAsync(&P, c->st));
    }
  }
  if (flat) {
    PF_CUDA(cudaMemcpyAsync(c->stage, p, dense, cudaMemcpyHostToDevice, c->st));
  } else {
    cudaMemcpy3DParms P = copy_params(c, p, hp, ld2, c->stage, (size_t)(g.m + 2) * sizeof(double), g.n + 2,
                                      cudaMemcpyHostToDevice);
    PF_CUDA(cudaMemcpy3DAsync(&P, c->st));
  }
  launch_scatter_pk(g, c->stage, c->p[0], c->p[1], c->st);
  c->launches += 1;
  if (c->opt.precision == PF_PREC_MIXED) mixed_sync_from_fp64(c);
  return check_launch("pf_set_state");
}

int pf_get_state(pf_case* c, double* u, double* v, double* w, double* p, int ld1, int ld2) {
  if (!c) return fail(PF_E_INVALID, "null handle");
  int rc = check_ld(c, ld1, ld2);
  if (rc) return rc;
  const Geo& g = c->g;
  const size_t hp = (size_t)ld1 * sizeof(double), dp = (size_t)g.X * sizeof(double);
  const int b = c->cur;
  double* dst[3] = {u, v, w};
  const double* src[3] = {c->U[b], c->V[b], c->W[b]};
  const bool flat = ld1 == g.m + 2 && ld2 == g.n + 2;  // contiguous host blocks (see pf_set_state)
  const size_t dense = (size_t)(g.m + 2) * (g.n + 2) * g.Z * sizeof(double);
  for (int f = 0; f < g.dim; f++) {
    if (!dst[f]) continue;
    if (flat) {
      launch_gather_nat(g, src[f], c->stage, c->st);
      c->launches += 1;
      PF_CUDA(cudaMemcpyAsync(dst[f], c->stage, dense, cudaMemcpyDeviceToHost, c->st));
    } else {
      cudaMemcpy3DParms P = copy_params(c, src[f], dp, g.Y, dst[f], hp, ld2, cudaMemcpyDeviceToHost);
      PF_CUDA(cudaMemcpy3DAsync(&P, c->st));
    }
  }
  if (p) {
    launch_gather_pk(g, c->p[0], c->p[1], c->stage, c->st);
    c->launches += 1;
    if (flat) {
      PF_CUDA(cudaMemcpyAsync(p, c->stage, dense, cudaMemcpyDeviceToHost, c->st));
    } else {
      cudaMemcpy3DParms P = copy_params(c, c->stage, (size_t)(g.m + 2) * sizeof(double), g.n + 2, p, hp, ld2,
                                        cudaMemcpyDeviceToHost);
      PF_CUDA(cudaMemcpy3DAsync(&P, c->st));
    }
  }
  rc = check_launch("pf_get_state");
  if (rc) return rc;
  return check_flags(c);  // waits for the copies too
}

// ---- one step from host state to host state ------------------------------
// pf_step_host = pf_set_state + pf_step(1) + pf_get_state with the copies
// overlapped with the step's first stages.  A step's input and its result
// are dependent, but the divergence and the predictor at plane k read the old
// velocities of planes k-1 .. k+1 only (the periodic z-wrap of the
// divergence aside).  So the input arrives on a second stream in slabs of
// planes and the case's stream runs the divergence and the predictor over
// each range of planes whose inputs are in place while the next slabs are in
// flight; p (read first by the SOR) comes last.  Plane 1 of the predictor
// reads the divergence of plane l through the wrap and runs after the last
// slab.  Each cell's arithmetic is the step's own, so the results are those of
// the three calls (tested bit for bit).  The readback overlaps the gathers of
// the next fields with the copies of the previous ones.
static constexpr int IO_SLABS = 16;  // slabs of the input (the first one is exposed)

static bool step_host_overlaps(const pf_case* c, int ld1, int ld2) {
  const Geo& g = c->g;
  return g.dim == 3 && !g.wall && c->opt.precision == PF_PREC_FP64 && !c->profiling && ld1 == g.m + 2 &&
         ld2 == g.n + 2;
}

// The schedule over the l+2 planes (ghosts included) of a 3D case: slab b
// brings planes k0 .. k1; after it the divergence covers div_lo .. div_hi and
// the predictor pred_lo .. pred_hi (empty when hi < lo).  The divergence at k
// reads the old velocities at k-1 .. k+1; the predictor at k reads them and
// the divergence at k-1 .. k+1 (plane l: l-1, l and plane 1 through the
// wrap).  Plane 1 reads the divergence of plane l and runs after the last slab.
struct HostSlab {
  int k0, k1, div_lo, div_hi, pred_lo, pred_hi;
};
static std::vector<HostSlab> host_step_plan(int l) {
  const int Z = l + 2;
  const int slab = std::max(2, (Z + IO_SLABS - 1) / IO_SLABS);
  std::vector<HostSlab> plan;
  int div_to = 0, pred_to = 1;  // the last plane done (the predictor starts at plane 2)
  for (int k0 = 0; k0 < Z; k0 += slab) {
    HostSlab h{k0, std::min(k0 + slab, Z) - 1, 0, -1, 0, -1};
    const int d = std::min(h.k1 - 1, l);
    if (d > div_to) {
      h.div_lo = div_to + 1;
      h.div_hi = div_to = d;
    }
    const int pr = div_to == l ? l : div_to - 1;
    if (pr > pred_to) {
      h.pred_lo = pred_to + 1;
      h.pred_hi = pred_to = pr;
    }
    plan.push_back(h);
  }
  return plan;
}

static int io_setup(pf_case* c, size_t nevents) {
  if (!c->iostage) {
    cudaError_t e = cudaMalloc(&c->iostage, 3 * dense_bytes(c->g));
    if (e != cudaSuccess) {
      c->iostage = nullptr;
      return cuda_fail(e, "cudaMalloc(host-step staging)");
    }
  }
  if (!c->st_io) PF_CUDA(cudaStreamCreateWithFlags(&c->st_io, cudaStreamNonBlocking));
  while (c->ev_io.size() < nevents) {
    cudaEvent_t e;
    PF_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    c->ev_io.push_back(e);
  }
  return PF_OK;
}

static int step_host_overlapped(pf_case* c, const double* const* in, double* const* out) {
  const Geo& g = c->g;
  const Scal& s = c->s;
  const std::vector<HostSlab> plan = host_step_plan(g.l);
  const int nslabs = (int)plan.size();
  int rc = io_setup(c, (size_t)nslabs + 6);
  if (rc) return rc;
  cudaEvent_t* ev = c->ev_io.data();  // [0] start, [1..nslabs] slabs, then p in, 4 fields out
  cudaEvent_t ev_p = ev[nslabs + 1];
  const size_t plane = (size_t)(g.m + 2) * (g.n + 2), field = plane * g.Z;
  const int o = c->cur, nw = 1 - o;
  double* vel[3] = {c->U[o], c->V[o], c->W[o]};
  // the staging and the old fields may still be in use by earlier calls
  PF_CUDA(cudaEventRecord(ev[0], c->st));
  PF_CUDA(cudaStreamWaitEvent(c->st_io, ev[0], 0));
  for (int b = 0; b < nslabs; b++) {
    const size_t k0 = plan[b].k0, nk = plan[b].k1 - plan[b].k0 + 1;
    for (int f = 0; f < 3; f++)
      PF_CUDA(cudaMemcpyAsync(c->iostage + f * field + k0 * plane, in[f] + k0 * plane, nk * plane * sizeof(double),
                              cudaMemcpyHostToDevice, c->st_io));
    PF_CUDA(cudaEventRecord(ev[1 + b], c->st_io));
  }
  PF_CUDA(cudaMemcpyAsync(c->stage, in[3], field * sizeof(double), cudaMemcpyHostToDevice, c->st_io));
  PF_CUDA(cudaEventRecord(ev_p, c->st_io));
  for (int b = 0; b < nslabs; b++) {
    const HostSlab& h = plan[b];
    PF_CUDA(cudaStreamWaitEvent(c->st, ev[1 + b], 0));
    for (int f = 0; f < 3; f++) launch_scatter_nat_planes(g, c->iostage + f * field, vel[f], h.k0, h.k1, c->st);
    c->launches += 3;
    if (h.div_hi >= h.div_lo) {
      launch_divergence<double>(g, s, vel[0], vel[1], vel[2], c->div, c->st, h.div_lo, h.div_hi);
      c->launches += 1;
    }
    if (h.pred_hi >= h.pred_lo) {
      launch_predictor<double, double>(g, s, vel[0], vel[1], vel[2], c->div, c->gx, c->gy, c->gz, c->rinv,
                                       c->damp, vel[0], vel[1], vel[2], c->U[nw], c->V[nw], c->W[nw], c->st,
                                       h.pred_lo, h.pred_hi);
      c->launches += 1;
    }
  }
  launch_predictor<double, double>(g, s, vel[0], vel[1], vel[2], c->div, c->gx, c->gy, c->gz, c->rinv, c->damp,
                                   vel[0], vel[1], vel[2], c->U[nw], c->V[nw], c->W[nw], c->st, 1, 1);
  PF_CUDA(cudaStreamWaitEvent(c->st, ev_p, 0));
  launch_scatter_pk(g, c->stage, c->p[0], c->p[1], c->st);
  c->launches += 2;
  rc = check_launch("pf_step_host");
  if (rc) return rc;
  // the rest of the step: RHS, SOR, projection, boundary
  if (c->opt.use_graph) {
    rc = step_graph(c, false);
    if (rc) return rc;
  } else {
    enqueue_step(c, false, false);
  }
  // readback: the gather of a field overlaps the copy of the previous one
  const int b = c->cur;
  const double* src[3] = {c->U[b], c->V[b], c->W[b]};
  for (int f = 0; f < 4; f++) {
    if (!out[f]) continue;
    double* stg = f < 3 ? c->iostage + f * field : c->stage;
    if (f < 3)
      launch_gather_nat(g, src[f], stg, c->st);
    else
      launch_gather_pk(g, c->p[0], c->p[1], stg, c->st);
    c->launches += 1;
    PF_CUDA(cudaEventRecord(ev[nslabs + 2 + f], c->st));
    PF_CUDA(cudaStreamWaitEvent(c->st_io, ev[nslabs + 2 + f], 0));
    PF_CUDA(cudaMemcpyAsync(out[f], stg, field * sizeof(double), cudaMemcpyDeviceToHost, c->st_io));
  }
  rc = check_launch("pf_step_host");
  if (rc) return rc;
  PF_CUDA(cudaStreamSynchronize(c->st_io));
  return check_flags(c);  // waits for the case's stream
}

int pf_step_host(pf_case* c, const double* u, const double* v, const double* w, const double* p, double* u_out,
                 double* v_out, double* w_out, double* p_out, int ld1, int ld2) {
  if (!c || !u || !v || !p || (c->g.dim == 3 && !w)) return fail(PF_E_INVALID, "pf_step_host: null argument");
  int rc = check_ld(c, ld1, ld2);
  if (rc) return rc;
  if (step_host_overlaps(c, ld1, ld2)) {
    const double* in[4] = {u, v, w, p};
    double* out[4] = {u_out, v_out, w_out, p_out};
    return step_host_overlapped(c, in, out);
  }
  rc = pf_set_state(c, u, v, w, p, ld1, ld2);
  if (rc == PF_OK) rc = pf_step(c, 1);
  if (rc == PF_OK) rc = pf_get_state(c, u_out, v_out, w_out, p_out, ld1, ld2);
  return rc;
}

int pf_snapshot_begin(pf_case* c) {
  if (!c) return fail(PF_E_INVALID, "null handle");
  if (c->snap_pending) return fail(PF_E_BUSY, "pf_snapshot_begin: the previous snapshot was not collected");
  const Geo& g = c->g;
  const size_t dense = (size_t)(g.m + 2) * (g.n + 2) * g.Z;
  const int nf = g.dim + 1;
  if (!c->snap) {  // first use: all four resources or none
    double *dsnap = nullptr, *hsnap = nullptr;
    cudaStream_t ss = nullptr;
    cudaEvent_t ev[2] = {nullptr, nullptr};
    cudaError_t e = cudaMalloc(&dsnap, nf * dense * sizeof(double));
    if (e == cudaSuccess) e = cudaHostAlloc(&hsnap, nf * dense * sizeof(double), cudaHostAllocDefault);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&ss, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&ev[0], cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&ev[1], cudaEventDisableTiming);
    if (e != cudaSuccess) {
      if (dsnap) cudaFree(dsnap);
      if (hsnap) cudaFreeHost(hsnap);
      if (ss) cudaStreamDestroy(ss);
      for (auto x : ev)
        if (x) cudaEventDestroy(x);
      return cuda_fail(e, "pf_snapshot_begin: snapshot buffers");
    }
    c->snap = dsnap;
    c->hsnap = hsnap;
    c->st_snap = ss;
    c->ev_snap[0] = ev[0];
    c->ev_snap[1] = ev[1];
  }
  // device-side copies on the case's stream: the state as of the last enqueued step
  const int b = c->cur;
  const double* src[3] = {c->U[b], c->V[b], c->W[b]};
  const size_t dp = (size_t)(g.m + 2) * sizeof(double);
  for (int f = 0; f < g.dim; f++) {
    cudaMemcpy3DParms P = copy_params(c, src[f], (size_t)g.X * sizeof(double), g.Y, c->snap + f * dense, dp, g.n + 2,
                                      cudaMemcpyDeviceToDevice);
    PF_CUDA(cudaMemcpy3DAsync(&P, c->st));
  }
  launch_gather_pk(g, c->p[0], c->p[1], c->snap + g.dim * dense, c->st);
  c->launches += 1;
  int rc = check_launch("pf_snapshot_begin");
  if (rc) return rc;
  PF_CUDA(cudaEventRecord(c->ev_snap[0], c->st));
  // the copy to the host runs on the second stream, overlapping later steps
  PF_CUDA(cudaStreamWaitEvent(c->st_snap, c->ev_snap[0], 0));
  PF_CUDA(cudaMemcpyAsync(c->hsnap, c->snap, nf * dense * sizeof(double), cudaMemcpyDeviceToHost, c->st_snap));
  PF_CUDA(cudaEventRecord(c->ev_snap[1], c->st_snap));
  c->snap_pending = true;
  return PF_OK;
}

int pf_snapshot_wait(pf_case* c, double* u, double* v, double* w, double* p, int ld1, int ld2) {
  if (!c) return fail(PF_E_INVALID, "null handle");
  if (!c->snap_pending) return fail(PF_E_STATE, "pf_snapshot_wait: no snapshot in flight");
  int rc = check_ld(c, ld1, ld2);
  if (rc) return rc;
  PF_CUDA(cudaEventSynchronize(c->ev_snap[1]));
  c->snap_pending = false;
  const Geo& g = c->g;
  const size_t dense = (size_t)(g.m + 2) * (g.n + 2) * g.Z, row = (size_t)(g.m + 2) * sizeof(double);
  double* dst[4] = {u, v, g.dim == 3 ? w : p, p};
  for (int f = 0; f < g.dim + 1; f++) {
    double* d = dst[f];
    if (!d) continue;
    const double* s = c->hsnap + f * dense;
    for (int k = 0; k < g.Z; k++)
      for (int j = 0; j < g.n + 2; j++)
        std::memcpy(d + (size_t)ld1 * ((size_t)j + (size_t)ld2 * k), s + (size_t)(g.m + 2) * (j + (size_t)(g.n + 2) * k),
                    row);
  }
  return PF_OK;
}

int pf_get_porosity(pf_case* c, double* poro, int ld1, int ld2) {
  if (!c || !poro) return fail(PF_E_INVALID, "null argument");
  int rc = check_ld(c, ld1, ld2);
  if (rc) return rc;
  const Geo& g = c->g;
  cudaMemcpy3DParms P = copy_params(c, c->poro, (size_t)g.X * sizeof(double), g.Y, poro,
                                    (size_t)ld1 * sizeof(double), ld2, cudaMemcpyDeviceToHost);
  PF_CUDA(cudaMemcpy3DAsync(&P, c->st));
  PF_CUDA(cudaStreamSynchronize(c->st));
  return PF_OK;
}

int pf_solve_p(pf_case* c) {
  if (!c) return fail(PF_E_INVALID, "null handle");
  if (c->opt.precision == PF_PREC_MIXED)
    enqueue_solve_p_mixed(c, false);
  else
    enqueue_solve_p(c, false, true);
  return check_launch("pf_solve_p");
}

int pf_projection(pf_case* c) {
  if (!c) return fail(PF_E_INVALID, "null handle");
  if (c->opt.precision == PF_PREC_MIXED)
    enqueue_projection_mixed(c);
  else
    enqueue_projection(c);
  return check_launch("pf_projection");
}

int pf_boundary(pf_case* c) {
  if (!c) return fail(PF_E_INVALID, "null handle");
  if (c->opt.precision == PF_PREC_MIXED)
    enqueue_boundary_mixed(c);
  else
    enqueue_boundary(c);
  return check_launch("pf_boundary");
}

int pf_step(pf_case* c, int nsteps) {
  if (!c) return fail(PF_E_INVALID, "null handle");
  if (nsteps < 0) return fail(PF_E_INVALID, "nsteps < 0");
  for (int s = 0; s < nsteps; s++) {
    if (c->profiling) {
      // per step: [0] start, [4] after the predictor, [1] after the RHS,
      // [2] after the SOR, [3] end
      int rc = ensure_events(c, (size_t)(c->prof_steps + 1) * pf_case::PROF_EVENTS);
      if (rc) return rc;
      cudaEvent_t* ev = &c->events[(size_t)c->prof_steps * pf_case::PROF_EVENTS];
      c->ev_cur = ev;
      cudaEventRecord(ev[0], c->st);
      enqueue_step(c, true);
      cudaEventRecord(ev[3], c->st);
      c->prof_steps++;
    } else if (c->opt.use_graph) {
      int rc = step_graph(c);
      if (rc) return rc;
    } else {
      enqueue_step(c, false);
    }
  }
  return check_launch("pf_step");
}

int pf_synchronize(pf_case* c) {
  if (!c) return fail(PF_E_INVALID, "null handle");
  return check_flags(c);
}

int pf_norms(pf_case* c, double* max_div, double* sor_error) {
  if (!c) return fail(PF_E_INVALID, "null handle");
  const Geo& g = c->g;
  PF_CUDA(cudaMemsetAsync(&c->red[RED_DIV], 0, RED_SLOTS * sizeof(unsigned long long), c->st));
  const int b = c->cur;
  launch_div_diag<double>(g, c->s, c->U[b], c->V[b], c->W[b], c->poro, c->gx, c->gy, c->gz, &c->red[RED_DIV], c->st);
  c->launches += 1;
  int rc = check_launch("pf_norms");
  if (rc) return rc;
  PF_CUDA(cudaMemcpyAsync(c->hred, c->red, RED_TOTAL * sizeof(unsigned long long), cudaMemcpyDeviceToHost, c->st));
  PF_CUDA(cudaStreamSynchronize(c->st));
  unsigned long long be = 0, bd = 0;
  unsigned bf = 0;
  for (int q = 0; q < RED_SLOTS; q++) {
    be = std::max(be, c->hred[RED_ERR + q]);
    bd = std::max(bd, c->hred[RED_DIV + q]);
    // FP32 sweeps of the mixed form track their max change in the low halves
    bf = std::max(bf, (unsigned)(c->hred[RED_ERRF + q] & 0xffffffffULL));
  }
  double e, d;
  std::memcpy(&e, &be, sizeof(double));
  std::memcpy(&d, &bd, sizeof(double));
  float ef;
  std::memcpy(&ef, &bf, sizeof(float));
  if (std::isnan(ef) || (double)ef > e) e = (double)ef;  // NaN propagates
  if (sor_error) *sor_error = e;
  if (max_div) *max_div = d;
  if (c->hred[RED_FLAGS]) return flags_fail(c->hred[RED_FLAGS]);
  if (!std::isfinite(d)) return fail(PF_E_NONFINITE, "max|div u| is not finite");
  return PF_OK;
}

int pf_forces(pf_case* c, double force_p[3], double force_v[3]) {
  if (!c || !force_p || !force_v) return fail(PF_E_INVALID, "pf_forces: null argument");
  const Geo& g = c->g;
  const int b = c->cur;
  // scratch: the staging array, (m+2)(n+2)[(l+2)] doubles >= 6 per 256 cells + 6
  const long long cells = (long long)g.m * g.n * (g.dim == 3 ? g.l : 1);
  const long long nb = (cells + 255) / 256;
  if (6 * nb + 6 > (long long)(g.m + 2) * (g.n + 2) * g.Z) return fail(PF_E_INVALID, "pf_forces: grid too small");
  double* out = c->stage + 6 * nb;
  launch_forces(g, c->s, c->poro, c->p[0], c->p[1], c->U[b], c->V[b], c->W[b], c->stage, out, c->st);
  c->launches += 2;
  int rc = check_launch("pf_forces");
  if (rc) return rc;
  double h[6];
  PF_CUDA(cudaMemcpyAsync(h, out, sizeof(h), cudaMemcpyDeviceToHost, c->st));
  PF_CUDA(cudaStreamSynchronize(c->st));
  for (int d = 0; d < 3; d++) {
    force_p[d] = h[d];
    force_v[d] = h[3 + d];
  }
  return PF_OK;
}

int pf_host_register(void* ptr, size_t bytes) {
  if (!ptr || !bytes) return fail(PF_E_INVALID, "null argument");
  PF_CUDA(cudaHostRegister(ptr, bytes, cudaHostRegisterDefault));
  return PF_OK;
}

int pf_host_unregister(void* ptr) {
  if (!ptr) return fail(PF_E_INVALID, "null argument");
  PF_CUDA(cudaHostUnregister(ptr));
  return PF_OK;
}

int pf_profile_begin(pf_case* c) {
  if (!c) return fail(PF_E_INVALID, "null handle");
  c->profiling = true;
  c->prof_steps = 0;
  return PF_OK;
}

int pf_profile_end(pf_case* c, double* sor_ms, int64_t* sor_launches, double* step_ms, int64_t* steps) {
  if (!c) return fail(PF_E_INVALID, "null handle");
  if (!c->profiling) return fail(PF_E_STATE, "profiling not started");
  PF_CUDA(cudaStreamSynchronize(c->st));
  double sor = 0, step = 0;
  c->step_times.clear();
  for (double& x : c->stage_ms) x = 0.0;
  for (int64_t s = 0; s < c->prof_steps; s++) {
    float a = 0, b = 0, t0 = 0, t1 = 0, t3 = 0;
    cudaEvent_t* ev = &c->events[(size_t)s * pf_case::PROF_EVENTS];
    PF_CUDA(cudaEventElapsedTime(&a, ev[1], ev[2]));
    PF_CUDA(cudaEventElapsedTime(&b, ev[0], ev[3]));
    PF_CUDA(cudaEventElapsedTime(&t0, ev[0], ev[4]));
    PF_CUDA(cudaEventElapsedTime(&t1, ev[4], ev[1]));
    PF_CUDA(cudaEventElapsedTime(&t3, ev[2], ev[3]));
    sor += a;
    step += b;
    c->stage_ms[0] += t0;
    c->stage_ms[1] += t1;
    c->stage_ms[2] += a;
    c->stage_ms[3] += t3;
    c->step_times.push_back(b);
  }
  if (sor_ms) *sor_ms = sor;
  if (step_ms) *step_ms = step;
  if (steps) *steps = c->prof_steps;
  if (sor_launches) *sor_launches = c->prof_steps * c->sor_launches_per_step();
  c->profiling = false;
  return PF_OK;
}

int pf_profile_stages(pf_case* c, double* ms) {
  if (!c || !ms) return fail(PF_E_INVALID, "null argument");
  for (int k = 0; k < 4; k++) ms[k] = c->stage_ms[k];
  return PF_OK;
}

int pf_profile_step_times(pf_case* c, double* ms, int64_t max_steps, int64_t* n) {
  if (!c || !ms || !n) return fail(PF_E_INVALID, "null argument");
  int64_t k = 0;
  for (; k < max_steps && k < (int64_t)c->step_times.size(); k++) ms[k] = c->step_times[(size_t)k];
  *n = k;
  return PF_OK;
}

int pf_kernel_launches(pf_case* c, int64_t* count) {
  if (!c || !count) return fail(PF_E_INVALID, "null argument");
  *count = c->launches;
  return PF_OK;
}

int pf_sweep_info(pf_case* c, int* fused, float* split_ms, float* fused_ms) {
  if (!c || !fused) return fail(PF_E_INVALID, "null argument");
  *fused = c->use_fused ? 1 : 0;
  if (split_ms) *split_ms = c->sweep_ms[0];
  if (fused_ms) *fused_ms = c->sweep_ms[1];
  return PF_OK;
}

int pf_debug_step_host_plan(int l, int* slabs, int capacity) {
  if (l < 3 || l > (1 << 20) || capacity < 0 || (capacity > 0 && !slabs))
    return fail(PF_E_INVALID, "pf_debug_step_host_plan: bad argument");
  const std::vector<HostSlab> plan = host_step_plan(l);
  for (int b = 0; b < (int)plan.size() && b < capacity; b++) {
    const HostSlab& h = plan[b];
    const int v[6] = {h.k0, h.k1, h.div_lo, h.div_hi, h.pred_lo, h.pred_hi};
    std::memcpy(slabs + 6 * b, v, sizeof v);
  }
  return (int)plan.size();
}

int pf_debug_fused_drop_stage(pf_case* c, int stage) {
  if (!c) return fail(PF_E_INVALID, "null handle");
  if (!c->use_fused) return fail(PF_E_STATE, "the case does not run the fused correction sweep");
  c->fused.drop_stage = stage < 0 ? -1 : stage;
  for (auto& part : c->gexec)  // captured launches hold the old value
    for (auto& x : part)
      if (x) {
        cudaGraphExecDestroy(x);
        x = nullptr;
      }
  return PF_OK;
}

int pf_memory_bytes(pf_case* c, size_t* bytes) {
  if (!c || !bytes) return fail(PF_E_INVALID, "null argument");
  *bytes = c->bytes + c->mixed_bytes + c->list_bytes + (c->iostage ? 3 * dense_bytes(c->g) : 0);
  return PF_OK;
}

int pf_dc_list_info(pf_case* c, int* listed, int fluid[2], int total[2]) {
  if (!c || !listed) return fail(PF_E_INVALID, "null argument");
  *listed = c->use_dcl ? 1 : 0;
  for (int col = 0; col < 2; col++) {
    if (fluid) fluid[col] = c->dcl_fluid[col];
    if (total) total[col] = c->dcl_total[col];
  }
  return PF_OK;
}

int pf_sor_info(pf_case* c, int* listed, int fluid[2], int total[2]) {
  if (!c || !listed) return fail(PF_E_INVALID, "null argument");
  *listed = c->use_list ? 1 : 0;
  for (int col = 0; col < 2; col++) {
    if (fluid) fluid[col] = c->list_nfluid[col];
    if (total) total[col] = c->list_ntotal[col];
  }
  return PF_OK;
}

}  // extern "C"
