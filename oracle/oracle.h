/*
 * oracle.h -- CPU restatement of the reference's hot path (TEST
 * INFRASTRUCTURE ONLY: the checker for the CUDA library, never shipped or
 * timed as the product).
 *
 * Parity status: pinned against the reference's own source.  The
 * reference is Fortran and no Fortran compiler exists in the build
 * container, so it is not compiled; instead tests/golden/make_golden.py
 * runs the reference's subroutines, read from their source files, through
 * a Fortran-subset executor (tests/golden/f90exec.py: gfortran -O2
 * arithmetic, default-real literals in single precision) on 96 seeded
 * cases -- setind, the grid geometry of init.f90 with intfac.f90, all six
 * solvers, ghost cells, grad_gauss, bpres,
 * correctBoundaryConditions, fluxuvw (10 schemes x 3 directions), both
 * pressure assemblies, fluxmass, PISO_getHbyA, calcuvw,
 * PISO_multiple_correction, calcp, outbc, the LES viscosity, calcscm,
 * modvis, main.f90's Courant-number, continuity-error and constant
 * mass-flux fragments, and its time-loop body (PISO and SIMPLE steps) --
 * and tests/test_golden_reference.py holds this restatement to
 * those outputs bit for bit (every module array, the module scalars and
 * the unit-66 solver lines).  The reference's own known-answer vectors
 * (test_intersection_point.f90:8-38) pin find_intersection_point.
 *
 * Layout: the state mirrors the reference's Fortran modules.  Each module
 * array is a 0-based double array of length nijk whose element ijk-1 is
 * the reference's element ijk.  Loops run over 1-based i,j,k with the
 * reference's bounds; ixk(i,j,k) = lk(k)+li(i)+j-1.
 *
 * Floating point: compiled with -ffp-contract=off so that a*b+c is two
 * rounded operations, as gfortran -O2 evaluates it on x86-64; expressions
 * are evaluated left to right with the reference's parentheses.  Fortran
 * default-real literals (1e-30, 0.1, 1.e20, ...) are single precision in
 * the reference and are reproduced as (double)<float literal>.
 */
#ifndef CAP_ORACLE_H
#define CAP_ORACLE_H

#include "../include/cappgpu.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct cap_state {
  int ni, nj, nk, nim, njm, nkm, nimm, njmm, nkmm, nij, nik, njk, nijk;
  int *li, *lk;                 /* li[1..ni], lk[1..nk] (index 0 unused) */
  double *f[CAP_NFIELDS];
  int *bc[CAP_NBC];
  cappgpu_params prm;
} cap_state;

cap_state* cap_new(int ni, int nj, int nk);
void cap_free(cap_state* s);
double* cap_field(cap_state* s, int fid);
int* cap_bc(cap_state* s, int face);
cappgpu_params* cap_params(cap_state* s);
int* cap_li(cap_state* s);
int* cap_lk(cap_state* s);
int cap_nijk(cap_state* s);

/* geometry from nodes x,y,z: face areas (init.f90:54-136) and
   interpolation factors (init.f90:142-144 -> intfac.f90:25-48). */
void cap_face_areas(cap_state* s);
void cap_intfac_all(cap_state* s);
void cap_find_intersection_point(const double* p15, double* out3);

void cap_update_values_at_ghostcells(cap_state* s);
void cap_grad_gauss(cap_state* s, int u, int dx, int dy, int dz);
void cap_bpres(cap_state* s, int p);

int cap_sipsol(cap_state* s, int fi, int ifi, cappgpu_solve_report* rep);
int cap_pcgsip(cap_state* s, int fi, int ifi, cappgpu_solve_report* rep);
int cap_iccg(cap_state* s, int fi, int ifi, cappgpu_solve_report* rep);
int cap_cgstab(cap_state* s, int fi, int ifi, cappgpu_solve_report* rep);
int cap_cgstab_sip(cap_state* s, int fi, int ifi, cappgpu_solve_report* rep);
int cap_dpcg(cap_state* s, int fi, int ifi, cappgpu_solve_report* rep);
double cap_spmv(cap_state* s, int pk, int zk);

void cap_fluxuvw(cap_state* s, int idew, int idns, int idtb, int arvx, int arvy, int arvz,
                 int fif, int acfe, int acfw, int fcf);
int cap_calcuvw(cap_state* s, cappgpu_solve_report* rep3);
void cap_piso_assemble_pressure_eq(cap_state* s, int idew, int idns, int idtb, int arvx,
                                   int arvy, int arvz, int fif, int acfe, int acfw, int fcf,
                                   int ipc, int bp);
void cap_assemble_pressure_eq(cap_state* s, int idew, int idns, int idtb, int arvx, int arvy,
                              int arvz, int fif, int acfe, int acfw, int fcf);
void cap_piso_gethbya(cap_state* s);
int cap_piso_multiple_correction(cap_state* s, cappgpu_solve_report* reps);
void cap_fluxmass(cap_state* s, int idew, int idns, int idtb, int arvx, int arvy, int arvz,
                  int fif, int acfe, int acfw, int fcf);
double cap_fluxmc(cap_state* s, int inp1, int idew, int idns, int idtb, int fif);
int cap_calcp(cap_state* s, cappgpu_solve_report* reps);
void cap_outbc(cap_state* s);
void cap_correct_boundary_conditions(cap_state* s);
void cap_courant(cap_state* s);
void cap_continuity_errors(cap_state* s);
/* find_strain_rate.f90:20-79 (gauss branch), calc_vis_les.f90:38-249 */
void cap_find_strain_rate(cap_state* s);
void cap_calc_vis_les(cap_state* s);
/* const_massflux_correction.f90:1-22 */
void cap_const_massflux_correction(cap_state* s);
/* k-omega SST (oracle_turb.c): calculate_stuff_for_sst.f90, fluxscm-
   overrelaxed-correction.f90, calcscm.f90 for ifi = ite / ied, modvis.f90 */
void cap_calculate_stuff_for_sst(cap_state* s);
void cap_fluxscm(cap_state* s, int idew, int idns, int idtb, int fi, int gx, int ifi, int arvx, int arvy, int arvz,
                 int fif, int acfe, int acfw, int fcf);
int cap_calcscm(cap_state* s, int ifi, cappgpu_solve_report* rep);
void cap_modvis(cap_state* s);
int cap_piso_steps(cap_state* s, int nsteps, cappgpu_solve_report* last);
int cap_simple_iters(cap_state* s, int niters, cappgpu_solve_report* last);

#ifdef __cplusplus
}
#endif
#endif
