// kernels.cuh -- internal (stream-ordered, non-synchronising) entry points
// shared between the library's translation units.
#pragma once
#include "common.cuh"

namespace cap {

int ghost_update();
int grad_gauss(int uf, int dxf, int dyf, int dzf);
int bpres(int pf);
int correct_bc();

// linear solvers on field fi with parameter slot ifi (1-based)
int solve(int solver, int fi, int ifi, cappgpu_solve_report* rep);
int sipsol(int fi, int ifi, cappgpu_solve_report* rep);
int pcgsip(int fi, int ifi, cappgpu_solve_report* rep);
int iccg(int fi, int ifi, cappgpu_solve_report* rep);
int bicgstab(int fi, int ifi, bool sip, cappgpu_solve_report* rep);
int dpcg(int fi, int ifi, cappgpu_solve_report* rep);
int pcgsip_fast(int fi, int ifi, cappgpu_solve_report* rep);
int pcgsip_mixed(int fi, int ifi, cappgpu_solve_report* rep);
int sipsol_fast(int fi, int ifi, cappgpu_solve_report* rep);
int cgstab_sip_fast(int fi, int ifi, cappgpu_solve_report* rep);
int iccg_fast(int fi, int ifi, cappgpu_solve_report* rep);
int resid_natural_k(int fif, int k0, int k1, double* res0);
int sipsol_mixed(int fi, int ifi, cappgpu_solve_report* rep);
int fast_profile_unit(int which, double* bytes);
void fast_free();
// per-face geometry cache of the FP64 face kernels (assembly.cu) and the
// 1/vol cache of the FP64 gradient (stencil.cu)
void facegeo_free();
void volr_free();
// outlet face lists of outbc (assembly.cu)
void outbc_free();
// learned initial guess (learned.cu)
void learned_free();
int learned_solve_start(int fif, double res0);
int learned_solve_end(int fif);
int learned_profile_unit(int which, double* flops);
int learned_set_conv(int impl);
int learned_set_loss(int kind);
// natural-layout residual r = su - A fi over the interior of an arbitrary
// field array, written to res, with its L1 norm (solvers.cu)
int resid_into(const double* fi, double* res, double* l1);
// z = A p over the interior (p's ghost values included) and (r.z, z.z)
int spmv_dot2_natural(const double* p, double* z, const double* r, double* out2);
// (a1.b1, a2.b2) over the interior (natural layout)
int dot2_natural(const double* a1, const double* b1, const double* a2, const double* b2, double* out2);

// assembly
int fluxuvw(int idew, int idns, int idtb, int arvx, int arvy, int arvz, int fif, int acfe, int acfw, int fcf);
int calcuvw(cappgpu_solve_report* rep3);
int piso_assemble(int idew, int idns, int idtb, int arvx, int arvy, int arvz, int fif, int acfe, int acfw,
                  int fcf, int ipc, int bp);
int assemble_pressure_eq(int idew, int idns, int idtb, int arvx, int arvy, int arvz, int fif, int acfe,
                         int acfw, int fcf);
int piso_gethbya();
int piso_multiple_correction(cappgpu_solve_report* reps);
int fluxmass(int idew, int idns, int idtb, int arvx, int arvy, int arvz, int fif, int acfe, int acfw, int fcf);
int calcp(cappgpu_solve_report* reps);
int outbc();
int courant();
int continuity_errors();
// LES sub-grid viscosity (les.cu)
int find_strain_rate();
int calc_vis_les();
// constant mass-flux forcing (mflux.cu)
int const_massflux_correction();
// k-omega SST (turb.cu): calcscm for ifi = ite / ied, modvis
int calcscm(int ifi, cappgpu_solve_report* rep);
int modvis();

}  // namespace cap
