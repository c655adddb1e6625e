// pf_case.cuh -- the case handle behind the opaque pf_case of the C ABI.
#pragma once
#include <cuda_runtime.h>

#include <vector>

#include "pf_internal.cuh"

struct pf_case {
  pf_params prm{};
  pf_options opt{};
  pf::Geo g{};
  pf::Scal s{};
  cudaStream_t st = nullptr;
  char* base = nullptr;  // one device allocation for the FP64 arrays
  size_t bytes = 0;
  // natural layout, FP64
  double *poro = nullptr, *gx = nullptr, *gy = nullptr, *gz = nullptr, *rinv = nullptr, *damp = nullptr;
  double* div = nullptr;
  double *U[2] = {nullptr, nullptr}, *V[2] = {nullptr, nullptr}, *W[2] = {nullptr, nullptr};
  int cur = 0;  // buffer holding the current velocities
  // packed red-black, FP64
  double* p[2] = {nullptr, nullptr};
  pf::Coef<double> C[2]{};
  double* stage = nullptr;          // dense (m+2)(n+2)[(l+2)] staging
  unsigned long long* red = nullptr;   // [0] SOR error bits, [1] max|div| bits, [2] max|r| bits, [3] flag
  unsigned long long* hred = nullptr;  // pinned host mirror
  // step graphs [part][buffer]: part 0 the whole step, part 1 the step after
  // the predictor (pf_step_host issues the divergence and predictor itself)
  cudaGraphExec_t gexec[2][2] = {{nullptr, nullptr}, {nullptr, nullptr}};
  // profiling: PROF_EVENTS events per profiled step
  static constexpr int PROF_EVENTS = 5;
  bool profiling = false;
  int64_t prof_steps = 0;
  std::vector<cudaEvent_t> events;
  cudaEvent_t* ev_cur = nullptr;
  std::vector<double> step_times;  // ms, last profiling session
  double stage_ms[4] = {0, 0, 0, 0};  // predictor, RHS, SOR, projection + boundary (pf_profile_stages)
  int64_t launches = 0;            // kernels launched so far
  // asynchronous snapshots (pf_snapshot_begin / _wait), allocated on first use:
  // dense (m+2)(n+2)[(l+2)] copies of u, v, [w,] p on the device and pinned
  // on the host, drained on a second stream while the case keeps stepping
  double* snap = nullptr;
  double* hsnap = nullptr;
  cudaStream_t st_snap = nullptr;
  cudaEvent_t ev_snap[2] = {nullptr, nullptr};
  bool snap_pending = false;
  int64_t graph_kernels[2][2] = {{0, 0}, {0, 0}};
  // pf_step_host, allocated on first use: dense staging of u, v, w, the
  // stream that copies between host and staging, and its events
  double* iostage = nullptr;
  cudaStream_t st_io = nullptr;
  std::vector<cudaEvent_t> ev_io;

  // ---- the plain 3D sweep driven by cell lists (pf_sor_list.cu) ----
  // per colour: every cell's packed index and flags, in chunks of 32 that
  // are all fluid or all other cells, merged by position
  bool use_list = false;
  unsigned* list_base = nullptr;
  unsigned* list[2] = {nullptr, nullptr};
  size_t list_bytes = 0;
  int list_nfluid[2] = {0, 0}, list_ntotal[2] = {0, 0};  // cells per colour: fluid, all
  int list_nchunks[2] = {0, 0};                            // chunks of 32 entries per colour
  int list_grid[3] = {0, 0, 0};  // CTAs of the persistent launches: sweep, tracked sweep, residual
  double list_const[6] = {0, 0, 0, 0, 0, 0};  // the fluid cells' normalised coefficients
  bool list_iso = false;                        // all six equal (dx = dy = dz)

  // ---- mixed precision form (pf_mixed.cu) ----
  char* mbase = nullptr;
  size_t mixed_bytes = 0;
  float *Uf[2] = {nullptr, nullptr}, *Vf[2] = {nullptr, nullptr}, *Wf[2] = {nullptr, nullptr};
  float* divf = nullptr;
  float *gxf = nullptr, *gyf = nullptr, *gzf = nullptr, *rinvf = nullptr, *dampf = nullptr;
  float* e[2] = {nullptr, nullptr};     // packed FP32 correction
  // fused sweep (both colours per launch): the correction ping-pongs between
  // e and e2 within a pass; e2 is allocated when the case may run it
  float* e2[2] = {nullptr, nullptr};
  pf::FusedShape fused;
  bool use_fused = false;
  bool dc_early = false;  // the split FP32 sweep's grid fits one wave: early operand loads
  float sweep_ms[2] = {0.f, 0.f};  // PF_SWEEP_AUTO: ms per sweep measured at creation (split, fused)
  float* rf[2] = {nullptr, nullptr};    // packed FP32 normalised residual (RHS of the sweeps)
  float* epsf[2] = {nullptr, nullptr};  // packed FP32 porosity (operator rebuilt on the fly)
  int* skip = nullptr;                  // device flag: defect correction converged
  // the split FP32 sweep over chunk lists (3D, pf_dc_list.cu); their bytes
  // are counted in list_bytes
  bool use_dcl = false;
  unsigned* dcl_base = nullptr;
  unsigned* dcl[2] = {nullptr, nullptr};
  int dcl_ngroups[2] = {0, 0};                           // groups of 32 entries per colour
  int dcl_fluid[2] = {0, 0}, dcl_total[2] = {0, 0};      // all-fluid chunks, all chunks
  int dcl_grid[2] = {0, 0};                              // persistent CTAs: untracked, tracked

  int64_t sor_launches_per_step() const {
    if (opt.precision == PF_PREC_MIXED) return (use_fused ? 1LL : 2LL) * opt.outer_max * opt.inner_sweeps;
    return 2LL * prm.iter_max;
  }
};

namespace pf {
// The precision form with the fused sweep (both colours per launch).
bool mixed_fused(const Geo& g, const pf_options& opt);
int mixed_alloc(pf_case* c);
// After set-up: the sweep form (PF_SWEEP_AUTO times both forms on the case).
int mixed_choose_sweep(pf_case* c);
void mixed_free(pf_case* c);
void mixed_setup(pf_case* c);
void mixed_sync_from_fp64(pf_case* c);
void mixed_sync_to_fp64(pf_case* c);
void enqueue_solve_p_mixed(pf_case* c, bool prof);
void enqueue_projection_mixed(pf_case* c);
void enqueue_boundary_mixed(pf_case* c);
int geometry_to_stage(pf_case* c, const pf_shape* shapes, int nshapes, double edge);
// The list-driven plain sweep (3D, no walls, sizes that pack into 32 bits).
bool sor_list_eligible(const Geo& g);
size_t sor_list_bytes(const Geo& g);
int sor_list_setup(pf_case* c);
void launch_sor_list(const pf_case* c, int col, double omw, unsigned long long* err, bool early,
                     cudaStream_t st);
// The precision form's split FP32 sweep over chunk lists (3D, no walls).
bool dc_list_eligible(const Geo& g);
size_t dc_list_bytes(const Geo& g);
int dc_list_setup(pf_case* c);
void launch_sor_dc_list(const pf_case* c, int col, unsigned long long* err, const int* skip, cudaStream_t st);
// The precision form's FP64 residual over the same lists.
void launch_residual_list(const pf_case* c, int col, float* rf, float* ec, unsigned long long* rmax, const int* skip,
                          cudaStream_t st);
}  // namespace pf
