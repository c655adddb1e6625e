/* A C caller of libpixelflow_gb300.so (test infrastructure): prints the
 * offset and size of every field of the ABI structs as the C compiler lays
 * them out from include/pixelflow_gpu.h, then calls the entry points that
 * need no GPU.  tests/test_abi_c.py compares the layout with the ctypes and
 * Fortran bindings. */
#include <stddef.h>
#include <stdio.h>
#include <string.h>

#include "pixelflow_gpu.h"

#define F(T, f) printf("\"%s.%s\": [%zu, %zu],\n", #T, #f, offsetof(T, f), sizeof(((T *)0)->f))

int main(int argc, char **argv) {
  printf("{\n");
  F(pf_params, dim); F(pf_params, m); F(pf_params, n); F(pf_params, l);
  F(pf_params, xnue); F(pf_params, xlambda); F(pf_params, density); F(pf_params, width);
  F(pf_params, height); F(pf_params, depth); F(pf_params, time); F(pf_params, inlet_velocity);
  F(pf_params, outlet_pressure); F(pf_params, aoa); F(pf_params, istep_max); F(pf_params, iter_max);
  F(pf_params, thickness); F(pf_params, threshold); F(pf_params, relux_factor); F(pf_params, nonslip);
  F(pf_params, inflow_porosity); F(pf_params, wall_mode); F(pf_params, walls); F(pf_params, slip_y);
  F(pf_options, precision); F(pf_options, outer_max); F(pf_options, inner_sweeps);
  F(pf_options, track_sor_error); F(pf_options, dc_tol); F(pf_options, use_graph); F(pf_options, sweep_form);
  F(pf_options, fused_rows); F(pf_options, fused_planes); F(pf_options, sor_path); F(pf_options, reserved);
  F(pf_shape, kind); F(pf_shape, reserved); F(pf_shape, cx); F(pf_shape, cy); F(pf_shape, cz);
  F(pf_shape, a); F(pf_shape, b); F(pf_shape, angle);
  F(pf_batch_options, cluster); F(pf_batch_options, threads); F(pf_batch_options, max_cases);
  F(pf_batch_options, global_passes); F(pf_batch_options, hbm_budget_bytes); F(pf_batch_options, large_cells);
  F(pf_batch_options, use_graph); F(pf_batch_options, reserved);
  printf("\"sizeof.pf_params\": [0, %zu],\n\"sizeof.pf_options\": [0, %zu],\n", sizeof(pf_params),
         sizeof(pf_options));
  printf("\"sizeof.pf_shape\": [0, %zu],\n\"sizeof.pf_batch_options\": [0, %zu],\n", sizeof(pf_shape),
         sizeof(pf_batch_options));
  /* GPU-free calls through the library */
  pf_options o;
  memset(&o, 0xff, sizeof o);
  pf_default_options(&o);
  pf_batch_options bo;
  memset(&bo, 0xff, sizeof bo);
  pf_batch_default_options(&bo);
  int slabs[6 * 64];
  const int ns = pf_debug_step_host_plan(256, slabs, 64);
  printf("\"abi_version\": [0, %d],\n\"default.precision\": [0, %d],\n\"default.use_graph\": [0, %d],\n",
         pf_abi_version(), o.precision, o.use_graph);
  printf("\"default.sor_path\": [0, %d],\n\"batch.use_graph\": [0, %d],\n\"batch.cluster\": [0, %d],\n", o.sor_path,
         bo.use_graph, bo.cluster);
  printf("\"step_host_slabs_256\": [0, %d],\n\"strerror_timeout_len\": [0, %zu]\n}\n", ns,
         strlen(pf_strerror(PF_E_TIMEOUT)));
  (void)argc;
  (void)argv;
  return 0;
}
