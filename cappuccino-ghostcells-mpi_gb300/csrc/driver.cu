// driver.cu -- device-resident step drivers: the body of the reference's
// iteration loop (main.f90:134-207) for PISO and SIMPLE, with every field
// kept on the device between routines.
#include <string.h>

#include "common.cuh"
#include "kernels.cuh"

namespace cap {

// calcuvw.f90:254 and calc_vis_les.f90:174 address the top wall with
// lk(nimm); that is inside the array only when nimm+1 <= nk (params.top_plane
// = 1 takes lk(nkmm) instead).
static int check_top_wall_index() {
  const Dims& d = ctx().d;
  if (!ctx().prm.top_plane && d.nimm + 1 > d.nk) {
    set_error("top wall index lk(nimm) of calcuvw.f90:254 leaves the array (ni=%d > nk=%d)", d.ni, d.nk);
    return CAPPGPU_E_ARG;
  }
  return CAPPGPU_OK;
}

// main.f90:140-157: time-level shift at the start of a time step; te and
// ed shift on every step, with or without the turbulence equations, as
// the reference's unconditional assignments do (the LES path writes te's
// ghost cells)
static int shift_time_levels() {
  Ctx& c = ctx();
  size_t nb = sizeof(double) * c.d.nijk;
  double** F = c.f;
  if (c.prm.bdf) {
    CAP_CUDA(cudaMemcpyAsync(F[CAP_UOO], F[CAP_UO], nb, cudaMemcpyDeviceToDevice, c.st));
    CAP_CUDA(cudaMemcpyAsync(F[CAP_VOO], F[CAP_VO], nb, cudaMemcpyDeviceToDevice, c.st));
    CAP_CUDA(cudaMemcpyAsync(F[CAP_WOO], F[CAP_WO], nb, cudaMemcpyDeviceToDevice, c.st));
    CAP_CUDA(cudaMemcpyAsync(F[CAP_TEOO], F[CAP_TEO], nb, cudaMemcpyDeviceToDevice, c.st));
    CAP_CUDA(cudaMemcpyAsync(F[CAP_EDOO], F[CAP_EDO], nb, cudaMemcpyDeviceToDevice, c.st));
  }
  CAP_CUDA(cudaMemcpyAsync(F[CAP_UO], F[CAP_U], nb, cudaMemcpyDeviceToDevice, c.st));
  CAP_CUDA(cudaMemcpyAsync(F[CAP_VO], F[CAP_V], nb, cudaMemcpyDeviceToDevice, c.st));
  CAP_CUDA(cudaMemcpyAsync(F[CAP_WO], F[CAP_W], nb, cudaMemcpyDeviceToDevice, c.st));
  CAP_CUDA(cudaMemcpyAsync(F[CAP_TEO], F[CAP_TE], nb, cudaMemcpyDeviceToDevice, c.st));
  CAP_CUDA(cudaMemcpyAsync(F[CAP_EDO], F[CAP_ED], nb, cudaMemcpyDeviceToDevice, c.st));
  return CAPPGPU_OK;
}

// main.f90:196-205 after the pressure-velocity coupling: the k and omega
// equations (calcscm) when lcal(ite) / lcal(ied) with the SST model, then
// the eddy viscosity (modvis) or, with lles, the sub-grid viscosity (its
// strain is formed here: the reference forms it in calcscm, which does not
// run on the LES path)
static int turbulence() {
  const cappgpu_params& P = ctx().prm;
  int rc;
  cappgpu_solve_report rep;
  if (P.sst && P.lcal[CAP_ITE - 1] && (rc = calcscm(CAP_ITE, &rep)) < 0) return rc;
  if (P.sst && P.lcal[CAP_IED - 1] && (rc = calcscm(CAP_IED, &rep)) < 0) return rc;
  if (P.lcal[CAP_IVIS - 1] && !P.lles && P.sst && (rc = modvis())) return rc;
  if (!P.lcal[CAP_IVIS - 1] || !P.lles) return CAPPGPU_OK;
  if ((rc = find_strain_rate())) return rc;
  return calc_vis_les();
}

int piso_steps(int nsteps, cappgpu_solve_report* last) {
  Ctx& c = ctx();
  int rc = check_top_wall_index();
  if (rc) return rc;
  int agg = 0;
  for (int st = 0; st < nsteps; ++st) {
    if ((rc = shift_time_levels())) return rc;
    if ((rc = courant())) return rc;          // CourantNo.h included at main.f90:169
    if ((rc = ghost_update())) return rc;     // main.f90:185
    cappgpu_solve_report r3[3];
    rc = calcuvw(r3);                         // main.f90:188
    if (rc < 0) return rc;
    if (!c.prm.const_mflux && (rc = outbc())) return rc;   // main.f90:190
    cappgpu_solve_report reps[64];
    int nrep = c.prm.ncorr * c.prm.npcor;
    if (nrep > 64) { set_error("ncorr*npcor > 64"); return CAPPGPU_E_ARG; }
    rc = piso_multiple_correction(reps);      // main.f90:193
    if (rc < 0) return rc;
    agg |= rc;
    if (last) *last = reps[nrep - 1];
    if ((rc = turbulence())) return rc;       // main.f90:196-205
    if (c.prm.ltransient && c.prm.const_mflux && (rc = const_massflux_correction())) return rc;   // main.f90:252
  }
  return agg;
}

int simple_iters(int niters, cappgpu_solve_report* last) {
  Ctx& c = ctx();
  int rc = check_top_wall_index();
  if (rc) return rc;
  int agg = 0;
  for (int it = 0; it < niters; ++it) {
    if ((rc = ghost_update())) return rc;
    cappgpu_solve_report r3[3];
    rc = calcuvw(r3);
    if (rc < 0) return rc;
    if (!c.prm.const_mflux && (rc = outbc())) return rc;
    cappgpu_solve_report reps[64];
    int nrep = c.prm.ncorr * c.prm.npcor;
    if (nrep > 64) { set_error("ncorr*npcor > 64"); return CAPPGPU_E_ARG; }
    rc = calcp(reps);
    if (rc < 0) return rc;
    agg |= rc;
    if (last) *last = reps[nrep - 1];
    if ((rc = turbulence())) return rc;       // main.f90:196-205
  }
  return agg;
}

}  // namespace cap

using namespace cap;

extern "C" {

int cappgpu_piso_steps(int nsteps, cappgpu_solve_report* last_p_report) {
  CAP_REQUIRE_INIT();
  if (nsteps < 0) { set_error("nsteps < 0"); return CAPPGPU_E_ARG; }
  int rc = piso_steps(nsteps, last_p_report);
  CAP_CUDA(cudaStreamSynchronize(ctx().st));
  return rc;
}

int cappgpu_simple_iters(int niters, cappgpu_solve_report* last_p_report) {
  CAP_REQUIRE_INIT();
  if (niters < 0) { set_error("niters < 0"); return CAPPGPU_E_ARG; }
  int rc = simple_iters(niters, last_p_report);
  CAP_CUDA(cudaStreamSynchronize(ctx().st));
  return rc;
}

}  // extern "C"
