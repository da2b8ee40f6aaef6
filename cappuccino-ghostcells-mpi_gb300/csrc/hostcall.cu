// hostcall.cu -- the host-pointer ("_h") entry points: the reference's
// routines for a host program that keeps its module arrays in host memory,
// as the Fortran code does (modules_allocatable.f90:111-398), and calls the
// routines one at a time with its own arrays as arguments.
//
// A host array is known to the library by its address: cappgpu_register
// ties a plain array to a field, cappgpu_register_vec3 an interleaved
// (3, nijk) array -- the reference's gradu(3,nxyza) layout -- to three
// component fields.  Every drop-in here runs in a frame:
//   1. the registered module arrays the routine reads are copied to the
//      device, and each argument array is resolved: a registered array is
//      its field (copied in), any other array is copied into a staging
//      array (the gfortran temporaries of array sections land here);
//   2. the device routine runs on those fields, exactly as the field-id
//      entry point does;
//   3. the registered module arrays the routine writes, and the written
//      argument arrays, are copied back, and the call synchronises.
// Grid geometry (nodes, centres, vol, fx..fz, face areas, walldist) is
// device-resident: it is uploaded once with cappgpu_set_field (or built
// with cappgpu_build_geometry) and never copied by a frame; registering a
// geometry array only lets the frame recognise it as an argument.
// The scalars of the reference's modules go through cappgpu_set_params /
// cappgpu_get_params around the calls (the Fortran shim does this).
#include <math.h>
#include <stdio.h>
#include <string.h>

#include <vector>

#include "common.cuh"
#include "kernels.cuh"

namespace cap {
namespace {

__global__ void k_split3(long long n, const double* __restrict__ aos, double* x, double* y, double* z) {
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < n; t += (long long)gridDim.x * blockDim.x) {
    x[t] = aos[3 * t];
    y[t] = aos[3 * t + 1];
    z[t] = aos[3 * t + 2];
  }
}

__global__ void k_join3(long long n, const double* __restrict__ x, const double* __restrict__ y,
                        const double* __restrict__ z, double* aos) {
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < n; t += (long long)gridDim.x * blockDim.x) {
    aos[3 * t] = x[t];
    aos[3 * t + 1] = y[t];
    aos[3 * t + 2] = z[t];
  }
}

bool is_geometry(int q) { return q >= CAP_X && q <= CAP_WALLDIST; }

// the x-component field of the interleaved gradient array q belongs to, or -1
int vec3_base(int q) {
  for (int b : {CAP_GRADU_X, CAP_GRADV_X, CAP_GRADW_X, CAP_GRADP_X, CAP_GRADTE_X, CAP_GRADED_X})
    if (q >= b && q < b + 3) return b;
  return -1;
}

int ensure_vec3buf() {
  Ctx& c = ctx();
  if (c.vec3buf) return CAPPGPU_OK;
  if (cudaMalloc(&c.vec3buf, sizeof(double) * 3 * (size_t)c.d.nijk) != cudaSuccess) {
    cudaGetLastError();
    c.vec3buf = nullptr;
    set_error("host call: out of device memory for an interleaved array");
    return CAPPGPU_E_NOMEM;
  }
  return CAPPGPU_OK;
}

int vec3_in(int base) {
  Ctx& c = ctx();
  int rc = ensure_vec3buf();
  if (rc) return rc;
  const long long n = c.d.nijk;
  CAP_CUDA(cudaMemcpyAsync(c.vec3buf, c.host_vec3[base], sizeof(double) * 3 * n, cudaMemcpyHostToDevice, c.st));
  launch(k_split3, grid_for(n), kThreads, c.st, n, (const double*)c.vec3buf, c.f[base], c.f[base + 1], c.f[base + 2]);
  CAP_CHECK_LAUNCH();
  return CAPPGPU_OK;
}

int vec3_out(int base) {
  Ctx& c = ctx();
  int rc = ensure_vec3buf();
  if (rc) return rc;
  const long long n = c.d.nijk;
  launch(k_join3, grid_for(n), kThreads, c.st, n, (const double*)c.f[base], (const double*)c.f[base + 1],
         (const double*)c.f[base + 2], c.vec3buf);
  CAP_CHECK_LAUNCH();
  CAP_CUDA(cudaMemcpyAsync(c.host_vec3[base], c.vec3buf, sizeof(double) * 3 * n, cudaMemcpyDeviceToHost, c.st));
  return CAPPGPU_OK;
}

// every field that is not grid geometry: the read and write set of the
// composite routines (calcuvw, PISO_getHbyA, PISO_multiple_correction)
std::vector<int> all_state() {
  std::vector<int> v;
  for (int q = CAP_WALLDIST + 1; q < CAP_NFIELDS; ++q) v.push_back(q);
  return v;
}

class Frame {
 public:
  Frame(std::vector<int> in, std::vector<int> out) : in_(std::move(in)), out_(std::move(out)) {}

  // The field a host argument array stands for: a registered array's own
  // field, otherwise a staging array holding a copy.  Written arguments are
  // copied back at the end.
  int arg(const double* host, bool written, int* id) {
    Ctx& c = ctx();
    if (!host) { set_error("host call: null array argument"); return CAPPGPU_E_ARG; }
    for (int q = 0; q < CAP_NFIELDS; ++q)
      if (c.host_reg[q] == host) {
        *id = q;
        if (!is_geometry(q)) args_.push_back({const_cast<double*>(host), q, written});
        return CAPPGPU_OK;
      }
    const int k = nstage_++;
    if (k >= kStageSlots) { set_error("host call: more than %d unregistered array arguments", kStageSlots); return CAPPGPU_E_ARG; }
    const int q = CAP_NFIELDS + k;
    if (!c.f[q] && cudaMalloc(&c.f[q], sizeof(double) * (size_t)c.d.nijk) != cudaSuccess) {
      cudaGetLastError();
      c.f[q] = nullptr;
      set_error("host call: out of device memory for a staging array");
      return CAPPGPU_E_NOMEM;
    }
    *id = q;
    args_.push_back({const_cast<double*>(host), q, written});
    return CAPPGPU_OK;
  }

  // module arrays and argument arrays to the device
  int begin() {
    Ctx& c = ctx();
    const size_t nb = sizeof(double) * (size_t)c.d.nijk;
    bool done3[CAP_NFIELDS] = {};
    for (int q : in_) {
      if (is_geometry(q)) continue;
      const int b = vec3_base(q);
      if (b >= 0 && c.host_vec3[b]) {
        if (!done3[b]) {
          int rc = vec3_in(b);
          if (rc) return rc;
          done3[b] = true;
        }
      } else if (c.host_reg[q]) {
        CAP_CUDA(cudaMemcpyAsync(c.f[q], c.host_reg[q], nb, cudaMemcpyHostToDevice, c.st));
        note_write(q);
      }
    }
    // every argument array goes in whole: the routines write only part of
    // their output arrays, the rest must keep the host's values
    for (const A& a : args_) {
      CAP_CUDA(cudaMemcpyAsync(c.f[a.id], a.host, nb, cudaMemcpyHostToDevice, c.st));
      note_write(a.id);
    }
    return CAPPGPU_OK;
  }

  // written arrays back to the host; synchronises
  int end(int rc) {
    Ctx& c = ctx();
    if (rc < 0) {
      cudaStreamSynchronize(c.st);
      return rc;
    }
    const size_t nb = sizeof(double) * (size_t)c.d.nijk;
    bool done3[CAP_NFIELDS] = {};
    for (int q : out_) {
      if (is_geometry(q)) continue;
      const int b = vec3_base(q);
      if (b >= 0 && c.host_vec3[b]) {
        if (!done3[b]) {
          int r = vec3_out(b);
          if (r) return r;
          done3[b] = true;
        }
      } else if (c.host_reg[q]) {
        CAP_CUDA(cudaMemcpyAsync(c.host_reg[q], c.f[q], nb, cudaMemcpyDeviceToHost, c.st));
      }
    }
    for (const A& a : args_)
      if (a.written) CAP_CUDA(cudaMemcpyAsync(a.host, c.f[a.id], nb, cudaMemcpyDeviceToHost, c.st));
    CAP_CUDA(cudaStreamSynchronize(c.st));
    return rc;
  }

 private:
  struct A {
    double* host;
    int id;
    bool written;
  };
  std::vector<int> in_, out_;
  std::vector<A> args_;
  int nstage_ = 0;
};

const std::vector<int> kGrad9 = {CAP_GRADU_X, CAP_GRADU_Y, CAP_GRADU_Z, CAP_GRADV_X, CAP_GRADV_Y,
                                 CAP_GRADV_Z, CAP_GRADW_X, CAP_GRADW_Y, CAP_GRADW_Z};

std::vector<int> cat(std::vector<int> a, const std::vector<int>& b) {
  a.insert(a.end(), b.begin(), b.end());
  return a;
}

// Fortran 1PE10.3: one digit before the point, three after, exponent
// E+dd (or +ddd without the E when it needs three digits), right-justified
// in ten columns.
void fortran_e10_3(double v, char out[16]) {
  if (isnan(v)) { snprintf(out, 16, "%10s", "NaN"); return; }
  if (isinf(v)) { snprintf(out, 16, "%10s", v < 0 ? "-Infinity" : "Infinity"); return; }
  char m[32];
  snprintf(m, sizeof m, "%.3E", v);   // d.dddE+xx or d.dddE+xxx
  char* e = strchr(m, 'E');
  char body[48];
  if (e && strlen(e + 1) == 4) {   // three exponent digits: the E is dropped
    *e = '\0';
    snprintf(body, sizeof body, "%s%s", m, e + 1);
  } else {
    snprintf(body, sizeof body, "%s", m);
  }
  snprintf(out, 16, "%10.15s", body);
}

}  // namespace
}  // namespace cap

using namespace cap;

extern "C" {

int cappgpu_register_vec3(int field_x, double* host) {
  CAP_REQUIRE_INIT();
  if (vec3_base(field_x) != field_x) {
    set_error("register_vec3: %d is not the x component of a gradient (gradu, gradv, gradw, gradp, gradte, graded)", field_x);
    return CAPPGPU_E_ARG;
  }
  ctx().host_vec3[field_x] = host;
  return CAPPGPU_OK;
}

// update_values_at_ghostcells (update_values_at_ghostcells_nonperiodic.f90:
// 47-640, update_values_at_ghostcells.f90:40-145): ghost values of u, v, w,
// te, ed, t, vis.
int cappgpu_update_values_at_ghostcells_h(void) {
  CAP_REQUIRE_INIT();
  const std::vector<int> f = {CAP_U, CAP_V, CAP_W, CAP_TE, CAP_ED, CAP_T, CAP_VIS};
  Frame fr(f, f);
  int rc = fr.begin();
  if (rc) return fr.end(rc);
  return fr.end(ghost_update());
}

// bpres(p), bpres.f90:3-81
int cappgpu_bpres_h(double* p) {
  CAP_REQUIRE_INIT();
  Frame fr({}, {});
  int id, rc;
  if ((rc = fr.arg(p, true, &id)) || (rc = fr.begin())) return fr.end(rc);
  return fr.end(bpres(id));
}

// exchange(phi), exchange_mpi.f90:4-89: one rank exchanges with itself,
// so phi is unchanged.
int cappgpu_exchange_h(double* phi) {
  CAP_REQUIRE_INIT();
  if (!phi) { set_error("exchange_h: null array"); return CAPPGPU_E_ARG; }
  return CAPPGPU_OK;
}

// fluxuvw(idew,idns,idtb,arvx,arvy,arvz,fif,acfe,acfw,fcf),
// fluxuvw-overrelaxed-correction.f90:3-659: reads u, v, w, vis and the
// velocity gradients, adds to su, sv, sw and uses bp, bt, bb as scratch
// (zero on return, :652-656).
int cappgpu_fluxuvw_h(int idew, int idns, int idtb, const double* arvx, const double* arvy, const double* arvz,
                      const double* fif, double* acfe, double* acfw, const double* fcf) {
  CAP_REQUIRE_INIT();
  const std::vector<int> rw = {CAP_SU, CAP_SV, CAP_SW, CAP_BP, CAP_BT, CAP_BB};
  Frame fr(cat(cat({CAP_U, CAP_V, CAP_W, CAP_VIS, CAP_DEN}, kGrad9), rw), rw);
  int ix, iy, iz, ifx, ie, iw, ic, rc;
  if ((rc = fr.arg(arvx, false, &ix)) || (rc = fr.arg(arvy, false, &iy)) || (rc = fr.arg(arvz, false, &iz)) ||
      (rc = fr.arg(fif, false, &ifx)) || (rc = fr.arg(acfe, true, &ie)) || (rc = fr.arg(acfw, true, &iw)) ||
      (rc = fr.arg(fcf, false, &ic)) || (rc = fr.begin()))
    return fr.end(rc);
  return fr.end(fluxuvw(idew, idns, idtb, ix, iy, iz, ifx, ie, iw, ic));
}

// piso_assemble_pressure_eq(...,ipc,bp), PISO_assemble_pressure_eq.f90:
// 3-257: acfe, acfw and bp always, fcf and su when ipc > 0.
int cappgpu_piso_assemble_pressure_eq_h(int idew, int idns, int idtb, const double* arvx, const double* arvy,
                                        const double* arvz, const double* fif, double* acfe, double* acfw,
                                        double* fcf, int ipc, double* bp) {
  CAP_REQUIRE_INIT();
  const std::vector<int> grads = cat(kGrad9, {CAP_GRADP_X, CAP_GRADP_Y, CAP_GRADP_Z});
  Frame fr(cat({CAP_DEN, CAP_APU, CAP_P, CAP_U, CAP_V, CAP_W, CAP_SU}, grads), {CAP_SU});
  int ix, iy, iz, ifx, ie, iw, ic, ib, rc;
  if ((rc = fr.arg(arvx, false, &ix)) || (rc = fr.arg(arvy, false, &iy)) || (rc = fr.arg(arvz, false, &iz)) ||
      (rc = fr.arg(fif, false, &ifx)) || (rc = fr.arg(acfe, true, &ie)) || (rc = fr.arg(acfw, true, &iw)) ||
      (rc = fr.arg(fcf, true, &ic)) || (rc = fr.arg(bp, true, &ib)) || (rc = fr.begin()))
    return fr.end(rc);
  return fr.end(piso_assemble(idew, idns, idtb, ix, iy, iz, ifx, ie, iw, ic, ipc, ib));
}

// assemble_pressure_eq(...), assemble_pressure_eq.f90:3-124
int cappgpu_assemble_pressure_eq_h(int idew, int idns, int idtb, const double* arvx, const double* arvy,
                                   const double* arvz, const double* fif, double* acfe, double* acfw, double* fcf) {
  CAP_REQUIRE_INIT();
  Frame fr({CAP_SU, CAP_SV, CAP_SW}, {});
  int ix, iy, iz, ifx, ie, iw, ic, rc;
  if ((rc = fr.arg(arvx, false, &ix)) || (rc = fr.arg(arvy, false, &iy)) || (rc = fr.arg(arvz, false, &iz)) ||
      (rc = fr.arg(fif, false, &ifx)) || (rc = fr.arg(acfe, true, &ie)) || (rc = fr.arg(acfw, true, &iw)) ||
      (rc = fr.arg(fcf, true, &ic)) || (rc = fr.begin()))
    return fr.end(rc);
  return fr.end(assemble_pressure_eq(idew, idns, idtb, ix, iy, iz, ifx, ie, iw, ic));
}

// calcuvw (calcuvw.f90:3-464); rep may be NULL or point to 3 reports.
int cappgpu_calcuvw_h(cappgpu_solve_report* rep) {
  CAP_REQUIRE_INIT();
  Frame fr(all_state(), all_state());
  int rc = fr.begin();
  if (rc) return fr.end(rc);
  return fr.end(calcuvw(rep));
}

// PISO_getHbyA (PISO_getHbyA.f90:3-233)
int cappgpu_piso_gethbya_h(void) {
  CAP_REQUIRE_INIT();
  Frame fr(all_state(), all_state());
  int rc = fr.begin();
  if (rc) return fr.end(rc);
  return fr.end(piso_gethbya());
}

// PISO_multiple_correction (PISO_multiple_correction.f90:3-296); rep may
// be NULL or point to ncorr*npcor reports.
int cappgpu_piso_multiple_correction_h(cappgpu_solve_report* rep) {
  CAP_REQUIRE_INIT();
  Frame fr(all_state(), all_state());
  int rc = fr.begin();
  if (rc) return fr.end(rc);
  return fr.end(piso_multiple_correction(rep));
}

// calcscm(fi,gradfi,ifi) (calcscm.f90:3-602): fi is the registered te or
// ed, gradfi the interleaved array registered for gradte or graded
int cappgpu_calcscm_h(double* fi, double* gradfi, int ifi) {
  CAP_REQUIRE_INIT();
  Ctx& c = ctx();
  const int f = ifi == CAP_ITE ? CAP_TE : ifi == CAP_IED ? CAP_ED : -1;
  const int g = ifi == CAP_ITE ? CAP_GRADTE_X : CAP_GRADED_X;
  if (f < 0 || !fi || c.host_reg[f] != fi || !gradfi || c.host_vec3[g] != gradfi) {
    set_error("calcscm_h: fi and gradfi must be the registered te/gradte (ifi = 5) or ed/graded (ifi = 6)");
    return CAPPGPU_E_ARG;
  }
  Frame fr(all_state(), all_state());
  int rc = fr.begin();
  if (rc) return fr.end(rc);
  cappgpu_solve_report rep;
  return fr.end(calcscm(ifi, &rep));
}

// modvis (modvis.f90:195-236, SST)
int cappgpu_modvis_h(void) {
  CAP_REQUIRE_INIT();
  const std::vector<int> in = {CAP_TE, CAP_ED, CAP_DEN, CAP_STRAIN, CAP_VIS};
  Frame fr(in, {CAP_VIS});
  int rc = fr.begin();
  if (rc) return fr.end(rc);
  return fr.end(modvis());
}

int cappgpu_last_report(int* solver, int* ifi, cappgpu_solve_report* rep) {
  CAP_REQUIRE_INIT();
  const Ctx& c = ctx();
  if (solver) *solver = c.last_solver;
  if (ifi) *ifi = c.last_ifi;
  if (rep) *rep = c.last_rep;
  return CAPPGPU_OK;
}

// The reference's unit-66 report line of a linear solve, e.g.
// pcg-sip.f90:195-197, sipsol.f90:101-103, iccg.f90:192-194,
// cgstab.f90:278-280, cgstab_sip.f90:273-275, pcg-jacobi.f90:150-152.  The
// iteration number is the Fortran loop index after the loop: the
// iteration that passed the exit test, or nsw + 1 when none did.
int cappgpu_solver_report_line(int solver, int ifi, const cappgpu_solve_report* rep, int icorr, int ipcorr,
                               char* buf, int n) {
  if (!rep || !buf || n < 1 || ifi < 1 || ifi > CAP_NPHI) return CAPPGPU_E_ARG;
  static const char* const names[CAP_NPHI] = {"U", "V", "W", "p", "k", "epsilon", "Energy", "Visc", "VarTemp", "Conc"};
  const char* name = names[ifi - 1];
  char r0[16], rl[16];
  fortran_e10_3(rep->res0, r0);
  fortran_e10_3(rep->resl, rl);
  const int l = rep->status == CAPPGPU_NOT_CONVERGED ? rep->iters + 1 : rep->iters;
  int w;
  switch (solver) {
    case CAPPGPU_SOLVER_PCGSIP:
      w = snprintf(buf, n, "PCG(SIP):  Solving for %s, Initial residual = %s, fFinal residual = %s, No Iterations %d",
                   name, r0, rl, l);
      break;
    case CAPPGPU_SOLVER_SIPSOL:
      w = snprintf(buf, n, "SIP:  Solving for %s, Initial residual = %s, Final residual = %s, No Iterations %d", name,
                   r0, rl, l);
      break;
    case CAPPGPU_SOLVER_ICCG:
      w = snprintf(buf, n, "PCG(IC0):  Solving for %s, Initial residual = %s, Final residual = %s, No Iterations %d",
                   name, r0, rl, l);
      break;
    case CAPPGPU_SOLVER_CGSTAB:
      w = snprintf(buf, n,
                   "BiCGStab(ILU(0)):  Solving for %s, Initial residual = %s, Final residual = %s, No Iterations %d",
                   name, r0, rl, l);
      break;
    case CAPPGPU_SOLVER_CGSTAB_SIP: {
      // i1 edit descriptors: one column, '*' when the value does not fit
      const char c1[2] = {(icorr >= 0 && icorr <= 9) ? (char)('0' + icorr) : '*', 0};
      const char c2[2] = {(ipcorr >= 0 && ipcorr <= 9) ? (char)('0' + ipcorr) : '*', 0};
      w = snprintf(buf, n,
                   "BiCGStab(SIP):  Solving for %s(icorr=%s,npcor=%s), Initial residual = %s, Final residual = %s, "
                   "No Iterations %d",
                   name, c1, c2, r0, rl, l);
      break;
    }
    case CAPPGPU_SOLVER_DPCG:
      w = snprintf(buf, n, "PCG(Jacobi):  Solving for %s, Initial residual = %s, Final residual = %s, No Iterations %d",
                   name, r0, rl, l);
      break;
    default:
      return CAPPGPU_E_ARG;
  }
  return w < n ? CAPPGPU_OK : CAPPGPU_E_ARG;
}

}  // extern "C"
