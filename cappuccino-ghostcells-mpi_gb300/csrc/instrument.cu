// instrument.cu -- timing and counters for benchmarks: CUDA events on the
// library's stream, the kernel launch count, pinned host buffers for
// end-to-end measurements, and single hot-kernel timing with the
// algorithmic bytes each one moves.
#include "common.cuh"
#include "kernels.cuh"
#include "wavefront.cuh"

namespace cap {
int profile_unit(int which, double* algo_bytes);
}

using namespace cap;

extern "C" {

int cappgpu_timer_start(void) {
  CAP_REQUIRE_INIT();
  CAP_CUDA(cudaEventRecord(ctx().ev[0], ctx().st));
  return CAPPGPU_OK;
}

int cappgpu_timer_stop(double* ms) {
  CAP_REQUIRE_INIT();
  Ctx& c = ctx();
  CAP_CUDA(cudaEventRecord(c.ev[1], c.st));
  CAP_CUDA(cudaEventSynchronize(c.ev[1]));
  float f = 0.f;
  CAP_CUDA(cudaEventElapsedTime(&f, c.ev[0], c.ev[1]));
  if (ms) *ms = f;
  return CAPPGPU_OK;
}

int cappgpu_get_stats(cappgpu_stats* s) {
  CAP_REQUIRE_INIT();
  if (!s) return CAPPGPU_E_ARG;
  Ctx& c = ctx();
  s->launches = (long long)c.launches;
  s->p_solve_ms = c.p_solve_ms;
  s->p_report = c.p_rep;
  return CAPPGPU_OK;
}

int cappgpu_host_alloc(void** p, int64_t bytes) {
  if (!p || bytes <= 0) return CAPPGPU_E_ARG;
  CAP_CUDA(cudaMallocHost(p, (size_t)bytes));
  return CAPPGPU_OK;
}

int cappgpu_host_free(void* p) {
  if (p) CAP_CUDA(cudaFreeHost(p));
  return CAPPGPU_OK;
}

// Time `reps` back-to-back runs of one hot-path unit on the current device
// state with CUDA events on the library stream.
//   which 0: SIP forward substitution over the interior (pcg-sip.f90:204-212)
//         1: SIP backward substitution (pcg-sip.f90:218-227)
//         2: 7-point product with fused dot (pcg-sip.f90:248-259)
//         3: grad_gauss of u (GRAD_GAUSS.f90)
//         4: fluxuvw, east faces (fluxuvw-overrelaxed-correction.f90)
//         5: piso_assemble_pressure_eq, east faces, ipc=1
//         6: SIP factorisation (pcg-sip.f90:174-193)
//         7, 8: FP32 forward / backward substitution of the precision-1 form
// Units 0,1,2,6,7,8 work on solver scratch vectors; 3-5 overwrite the module
// arrays they write (gradu, su.., ae/aw, f1, be), as the routines do.
int cappgpu_profile_kernel(int which, int reps, double* ms_per_unit, double* algo_bytes) {
  CAP_REQUIRE_INIT();
  if (reps < 1 || which < 0 || which > 10) { set_error("profile_kernel: bad arguments"); return CAPPGPU_E_ARG; }
  Ctx& c = ctx();
  double bytes = 0.0;
  int rc = profile_unit(which, &bytes);   // warm-up
  if (rc) return rc;
  CAP_CUDA(cudaEventRecord(c.ev[2], c.st));
  for (int r = 0; r < reps; ++r)
    if ((rc = profile_unit(which, &bytes))) return rc;
  CAP_CUDA(cudaEventRecord(c.ev[3], c.st));
  CAP_CUDA(cudaEventSynchronize(c.ev[3]));
  float f = 0.f;
  CAP_CUDA(cudaEventElapsedTime(&f, c.ev[2], c.ev[3]));
  if (ms_per_unit) *ms_per_unit = f / reps;
  if (algo_bytes) *algo_bytes = bytes;
  return CAPPGPU_OK;
}

}  // extern "C"
