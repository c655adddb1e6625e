// pf_mixed.cu -- the precision form of the step: FP32 stencils and FP32
// red-black sweeps inside an FP64 defect-correction loop.
//
// FP64: the velocity and pressure state, the accumulations into it (u_old +
// predictor increment, p += e, the projection), the RHS bb, the Poisson
// residual r (normalised by omega/ap) and every norm.
// FP32: the velocity stencils (divergence, the predictor's increment, read
// from an FP32 copy of the state), and the correction sweeps on e, whose
// operator is rebuilt on the fly from FP32 porosity (k_sor_dc, 24 bytes per
// update).
// Per step: outer_max passes of { r = bbn - w p - sum a p_nb (FP64);
// inner_sweeps FP32 SOR iterations on e from e = 0; p += e (FP64) }.
// With outer_max * inner_sweeps == iter_max the passes reproduce the plain
// SOR's iterates up to the FP32 rounding of e (stationary iteration on the
// residual equation); dc_tol > 0 ends the passes of a step early once
// max|r|/omega <= dc_tol (a device flag, so the step stays one graph).
#include <cuda_runtime.h>

#include <algorithm>

#include "pf_case.cuh"
#include "pf_internal.cuh"

namespace pf {

bool mixed_fused(const Geo& g, const pf_options& opt) {
  return opt.precision == PF_PREC_MIXED && opt.sweep_form != PF_SWEEP_SPLIT && fused_eligible(g);
}

// The sweep form of the case.  PF_SWEEP_AUTO runs a few sweeps of each form
// on the case's own arrays while the residual and the correction are still
// zero (so they stay zero: the state is untouched) and keeps the faster; the
// forms' speeds depend on the grid's shape in ways no simple rule captures
// (measured: the fused sweep is 5 % faster at 384^3, 6 % at 320^3, 1 % slower
// at 256^3, 11 % slower at 512 x 256 x 256, 39 % slower at 128^3).
int mixed_choose_sweep(pf_case* c) {
  c->use_fused = c->e2[0] != nullptr;
  if (!c->use_fused || c->opt.sweep_form != PF_SWEEP_AUTO) return PF_OK;
  const Geo& g = c->g;
  const Scal& s = c->s;
  cudaStream_t st = c->st;
  cudaEvent_t ev[3];
  for (auto& e : ev) PF_CUDA(cudaEventCreate(&e));
  constexpr int SWEEPS = 4, REPEATS = 3;
  // the launches of a step: with error tracking, colour 1 of each split sweep
  // and every fused sweep track (a change of 0 here; the slots are zeroed at
  // the start of each step)
  unsigned long long* err = c->opt.track_sor_error ? &c->red[RED_ERRF] : nullptr;
  float best[2] = {1e30f, 1e30f};
  for (int rep = 0; rep < REPEATS; rep++) {
    cudaEventRecord(ev[0], st);
    for (int it = 0; it < SWEEPS; it++)
      for (int col = 0; col < 2; col++) {
        if (c->use_dcl)
          launch_sor_dc_list(c, col, col == 1 ? err : nullptr, nullptr, st);
        else
          launch_sor_dc(g, s, c->epsf[col], c->epsf[1 - col], c->rf[col], c->e[col], c->e[1 - col], col,
                        col == 1 ? err : nullptr, nullptr, c->dc_early, st);
      }
    cudaEventRecord(ev[1], st);
    for (int it = 0; it < SWEEPS; it++) {
      const float* ea[2] = {it & 1 ? c->e2[0] : c->e[0], it & 1 ? c->e2[1] : c->e[1]};
      float* eb[2] = {it & 1 ? c->e[0] : c->e2[0], it & 1 ? c->e[1] : c->e2[1]};
      launch_sor_fused(g, s, c->fused, c->epsf, c->rf, ea, eb, err, &c->red[RED_FLAGS], nullptr, st);
    }
    cudaEventRecord(ev[2], st);
    cudaError_t e = cudaEventSynchronize(ev[2]);
    float ms[2] = {0.f, 0.f};
    if (e == cudaSuccess) e = cudaEventElapsedTime(&ms[0], ev[0], ev[1]);
    if (e == cudaSuccess) e = cudaEventElapsedTime(&ms[1], ev[1], ev[2]);
    if (e != cudaSuccess) {
      for (auto& x : ev) cudaEventDestroy(x);
      return cuda_fail(e, "sweep form timing");
    }
    for (int f = 0; f < 2; f++) best[f] = std::min(best[f], ms[f] / SWEEPS);
  }
  for (auto& x : ev) cudaEventDestroy(x);
  c->launches += (int64_t)REPEATS * SWEEPS * 3;
  c->sweep_ms[0] = best[0];
  c->sweep_ms[1] = best[1];
  c->use_fused = best[1] < best[0];
  return PF_OK;
}

int mixed_alloc(pf_case* c) {
  const Geo& g = c->g;
  const size_t nat = (size_t)g.nat * sizeof(float), pk = (size_t)g.pk * sizeof(float);
  const bool three = g.dim == 3;
  struct Req {
    float** dst;
    size_t bytes;
  };
  Req req[32];
  int nr = 0;
  req[nr++] = {&c->Uf[0], nat};
  req[nr++] = {&c->Vf[0], nat};
  req[nr++] = {&c->Wf[0], three ? nat : 0};
  req[nr++] = {&c->divf, nat};
  req[nr++] = {&c->gxf, nat};
  req[nr++] = {&c->gyf, nat};
  req[nr++] = {&c->gzf, three ? nat : 0};
  req[nr++] = {&c->rinvf, nat};
  req[nr++] = {&c->dampf, nat};
  const bool fused = mixed_fused(c->g, c->opt);
  for (int col = 0; col < 2; col++) {
    req[nr++] = {&c->e[col], pk};
    req[nr++] = {&c->rf[col], pk};
    req[nr++] = {&c->epsf[col], pk};
    req[nr++] = {&c->e2[col], fused ? pk : 0};
  }
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  c->dc_early = dc_one_wave(c->g, sms);
  if (fused) {
    const int fe = fused_setup(c->g, c->opt.fused_rows, c->opt.fused_planes, sms, c->fused);
    if (fe) return cuda_fail((cudaError_t)fe, "fused sweep set-up");
  }
  size_t total = 256;  // flag
  for (int r = 0; r < nr; r++) total += (req[r].bytes + 255) / 256 * 256;
  char* base = nullptr;
  cudaError_t e = cudaMalloc(&base, total);
  if (e != cudaSuccess) return cuda_fail(e, "cudaMalloc(mixed)");
  c->mbase = base;
  c->mixed_bytes = total;
  size_t off = 0;
  for (int r = 0; r < nr; r++) {
    *req[r].dst = req[r].bytes ? reinterpret_cast<float*>(base + off) : nullptr;
    off += (req[r].bytes + 255) / 256 * 256;
  }
  c->skip = reinterpret_cast<int*>(base + off);
  PF_CUDA(cudaMemsetAsync(base, 0, total, c->st));
  return PF_OK;
}

void mixed_free(pf_case* c) {
  if (c->mbase) cudaFree(c->mbase);
  c->mbase = nullptr;
}

void mixed_setup(pf_case* c) {
  const long long n = c->g.nat;
  launch_to_float(c->gx, c->gxf, n, c->st);
  launch_to_float(c->gy, c->gyf, n, c->st);
  if (c->g.dim == 3) launch_to_float(c->gz, c->gzf, n, c->st);
  launch_to_float(c->rinv, c->rinvf, n, c->st);
  launch_to_float(c->damp, c->dampf, n, c->st);
  launch_pack_eps(c->g, c->poro, c->epsf[0], c->epsf[1], c->st);
}

// FP32 copy of the current FP64 velocity state, read by the stencils.
void mixed_sync_from_fp64(pf_case* c) {
  const int b = c->cur;
  const double* src[3] = {c->U[b], c->V[b], c->W[b]};
  float* dst[3] = {c->Uf[0], c->Vf[0], c->Wf[0]};
  launch_to_float3(src, dst, c->g.dim, c->g.nat, c->st);
  c->launches += 1;
}

void mixed_sync_to_fp64(pf_case*) {}  // the state is FP64 already

void enqueue_solve_p_mixed(pf_case* c, bool prof) {
  const Geo& g = c->g;
  const Scal& s = c->s;
  cudaStream_t st = c->st;
  const int o = c->cur, nw = 1 - c->cur;
  const bool track = c->opt.track_sor_error != 0;
  const bool early = c->opt.dc_tol > 0.0;
  const int* skip = early ? c->skip : nullptr;
  if (track) launch_zero_u64(&c->red[RED_ERRF], RED_SLOTS, st);
  if (early) launch_zero_int(c->skip, st);
  launch_divergence<float>(g, s, c->Uf[0], c->Vf[0], c->Wf[0], c->divf, st);
  launch_predictor<float, double>(g, s, c->Uf[0], c->Vf[0], c->Wf[0], c->divf, c->gxf, c->gyf, c->gzf, c->rinvf,
                                  c->dampf, c->U[o], c->V[o], c->W[o], c->U[nw], c->V[nw], c->W[nw], st);
  if (prof) cudaEventRecord(c->ev_cur[4], st);
  launch_rhs<double>(g, s, c->U[nw], c->V[nw], c->W[nw], c->poro, c->gx, c->gy, c->gz, c->C[0], c->C[1], st);
  if (prof) cudaEventRecord(c->ev_cur[1], st);
  const bool halo = periodic_halo(g);
  const bool fused = c->use_fused;
  for (int pass = 0; pass < c->opt.outer_max; pass++) {
    launch_zero_u64(&c->red[RED_RMAX], RED_SLOTS, st);
    for (int col = 0; col < 2; col++) {
      if (c->use_list)
        launch_residual_list(c, col, c->rf[col], c->e[col], &c->red[RED_RMAX], skip, st);
      else
        launch_residual(g, c->C[col], c->p[col], c->p[1 - col], s.omega, col, c->rf[col], c->e[col],
                        &c->red[RED_RMAX], skip, st);
    }
    if (early) launch_dc_check(&c->red[RED_RMAX], c->opt.dc_tol * s.omega, c->skip, st);
    const float* efin[2] = {c->e[0], c->e[1]};
    if (fused) {
      // e (zeroed by the residual) -> e2 -> e -> ...: the result of an odd
      // number of sweeps is in e2
      for (int it = 0; it < c->opt.inner_sweeps; it++) {
        const float* ea[2] = {it & 1 ? c->e2[0] : c->e[0], it & 1 ? c->e2[1] : c->e[1]};
        float* eb[2] = {it & 1 ? c->e[0] : c->e2[0], it & 1 ? c->e[1] : c->e2[1]};
        launch_sor_fused(g, s, c->fused, c->epsf, c->rf, ea, eb, track ? &c->red[RED_ERRF] : nullptr,
                         &c->red[RED_FLAGS], skip, st);
      }
      if (c->opt.inner_sweeps & 1) {
        efin[0] = c->e2[0];
        efin[1] = c->e2[1];
      }
    } else {
      for (int it = 0; it < c->opt.inner_sweeps; it++) {
        for (int col = 0; col < 2; col++) {
          if (halo) launch_p_halo<float>(g, c->e[0], c->e[1], skip, st);
          unsigned long long* err = (track && (g.dim == 2 || col == 1)) ? &c->red[RED_ERRF] : nullptr;
          if (c->use_dcl)
            launch_sor_dc_list(c, col, err, skip, st);
          else
            launch_sor_dc(g, s, c->epsf[col], c->epsf[1 - col], c->rf[col], c->e[col], c->e[1 - col], col, err,
                          skip, c->dc_early, st);
        }
      }
    }
    launch_accumulate(g, c->p[0], c->p[1], efin[0], efin[1], skip, st);
    if (halo) launch_p_halo<double>(g, c->p[0], c->p[1], skip, st);
  }
  if (prof) cudaEventRecord(c->ev_cur[2], st);
  launch_p_halo<double>(g, c->p[0], c->p[1], nullptr, st);
  const int64_t per_sweep = fused ? 1 : 2 * (halo ? 2 : 1);
  c->launches += 4 + (track ? 1 : 0) + (early ? 1 : 0) +
                 (int64_t)c->opt.outer_max *
                     (4 + (early ? 1 : 0) + (halo ? 1 : 0) + (int64_t)c->opt.inner_sweeps * per_sweep);
  c->cur = nw;
}

void enqueue_projection_mixed(pf_case* c) {
  const int b = c->cur;
  c->launches += 1;
  launch_projection<double>(c->g, c->s, c->p[0], c->p[1], c->U[b], c->V[b], c->W[b], c->st);
}

void enqueue_boundary_mixed(pf_case* c) {
  const int b = c->cur;
  c->launches += boundary_launches(c->g);
  launch_boundary<double>(c->g, c->s, c->U[b], c->V[b], c->W[b], c->p[0], c->p[1], c->st);
  mixed_sync_from_fp64(c);
}

}  // namespace pf
