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

namespace cap {
namespace {

// FP64 issue-rate probe: eight independent multiply-add chains per thread
// (compiled without fused multiply-add, so each line is one FP64 multiply
// and one FP64 add), every SM filled with 2048 threads.  The result is the
// rate at which this GPU retires FP64 lane-operations, the ceiling of the
// FP64 kernels here whose work per byte is above about 0.08 operations.
constexpr int kRateIters = 2048;
constexpr int kRateChains = 8;

__global__ void __launch_bounds__(256) k_fp64_rate(double* out, double a, double b) {
  double x[kRateChains];
#pragma unroll
  for (int q = 0; q < kRateChains; ++q) x[q] = 1e-3 * (threadIdx.x + q);
  for (int it = 0; it < kRateIters; ++it) {
#pragma unroll
    for (int q = 0; q < kRateChains; ++q) x[q] = x[q] * a + b;
  }
  double s = 0.0;
#pragma unroll
  for (int q = 0; q < kRateChains; ++q) s += x[q];
  if (s == -1.0) out[0] = s;   // never true; keeps the chains live
}

int fp64_rate_unit(double* lane_ops) {
  Ctx& c = ctx();
  int sms = 0;
  CAP_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, c.device));
  const int blocks = sms * 8;
  launch(k_fp64_rate, blocks, 256, c.st, c.dscal + 15, 0.999999, 1e-6);
  CAP_CHECK_LAUNCH();
  *lane_ops = (double)blocks * 256 * kRateIters * kRateChains * 2;
  return CAPPGPU_OK;
}

}  // namespace
}  // namespace cap

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

int cappgpu_sweep_stats(double* ms_total, long long* launches, int reset) {
  CAP_REQUIRE_INIT();
  Ctx& c = ctx();
  if (ms_total) *ms_total = c.sw_ms;
  if (launches) *launches = c.sw_n;
  if (reset) {
    c.sw_ms = 0.0;
    c.sw_n = 0;
  }
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
//   which 0: SIP forward substitution over the interior (pcg-sip.f90:98-106)
//         1: SIP backward substitution (pcg-sip.f90:112-121)
//         2: 7-point product with fused dot (pcg-sip.f90:142-153)
//         3: grad_gauss of u (GRAD_GAUSS.f90)
//         4: fluxuvw, east faces (fluxuvw-overrelaxed-correction.f90)
//         5: piso_assemble_pressure_eq, east faces, ipc=1
//         6: SIP factorisation (pcg-sip.f90:68-87)
//         7, 8: FP32 forward / backward substitution of the precision-1 form
//         9, 10: the learned guess's net (inference; training pass)
//         11: the FP64 issue-rate probe (algo_bytes = FP64 lane-operations)
// Units 0,1,2,6,7,8 work on solver scratch vectors; 3-5 overwrite the module
// arrays they write (gradu, su.., ae/aw, f1, be), as the routines do.
int cappgpu_profile_kernel(int which, int reps, double* ms_per_unit, double* algo_bytes) {
  CAP_REQUIRE_INIT();
  if (reps < 1 || which < 0 || which > 11) { set_error("profile_kernel: bad arguments"); return CAPPGPU_E_ARG; }
  Ctx& c = ctx();
  double bytes = 0.0;
  auto unit = [&](double* b) { return which == 11 ? fp64_rate_unit(b) : profile_unit(which, b); };
  int rc = unit(&bytes);   // warm-up
  if (rc) return rc;
  CAP_CUDA(cudaEventRecord(c.ev[2], c.st));
  for (int r = 0; r < reps; ++r)
    if ((rc = unit(&bytes))) return rc;
  CAP_CUDA(cudaEventRecord(c.ev[3], c.st));
  CAP_CUDA(cudaEventSynchronize(c.ev[3]));
  float f = 0.f;
  CAP_CUDA(cudaEventElapsedTime(&f, c.ev[2], c.ev[3]));
  if (ms_per_unit) *ms_per_unit = f / reps;
  if (algo_bytes) *algo_bytes = bytes;
  return CAPPGPU_OK;
}

}  // extern "C"
