/*
 * cappgpu.h -- C ABI of the GB300 (sm_103a) implementation of Cappuccino's
 * SIMPLE/PISO step on a structured single-block ghost-cell grid.
 *
 * Reference: kiranhegde/cappuccino-ghostcells-mpi (Fortran 90).  The
 * reference routines communicate through Fortran module globals
 * (modules_allocatable.f90:111-398) rather than arguments.  This ABI keeps
 * that model: one process owns one grid on one GPU ("the context"), module
 * arrays live on the device as named fields, and every routine of the hot
 * path is an entry point with the reference's name and argument meaning.
 *
 * Conventions (identical to the reference):
 *  - a field is a double array of length nijk = ni*nj*nk; element
 *    ijk-1 (0-based) holds the reference's element ijk (1-based), with
 *    ijk = lk(k)+li(i)+j, li(i)=(i-1)*nj, lk(k)=(k-1)*ni*nj (setind.f90:34-40);
 *  - interior cells are i=3..ni-2, j=3..nj-2, k=3..nk-2; layers 2 and n-1
 *    are ghost cells, layers 1 and n are storage padding;
 *  - integer indices are 1-based i,j,k exactly as in the reference loops.
 *
 * Return codes: 0 = OK, >0 = informational (linear solver hit nsw without
 * reaching sor, as the reference does silently), <0 = error (see
 * CAPPGPU_E_*).  cappgpu_last_error() gives a one-line message.
 *
 * Threading: the library is single-threaded, not re-entrant, and uses one
 * CUDA stream.  Every entry point is synchronous at return.
 */
#ifndef CAPPGPU_H
#define CAPPGPU_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---------------------------------------------------------------- errors */
#define CAPPGPU_OK               0
#define CAPPGPU_NOT_CONVERGED    1   /* solver used nsw(ifi) sweeps          */
#define CAPPGPU_E_NOINIT        -1   /* cappgpu_init not called              */
#define CAPPGPU_E_ARG           -2   /* bad argument (field id, size, dims)  */
#define CAPPGPU_E_CUDA          -3   /* CUDA runtime error                   */
#define CAPPGPU_E_NONFINITE     -4   /* NaN/Inf in a solver residual         */
#define CAPPGPU_E_SPIN          -5   /* wavefront spin limit exceeded        */
#define CAPPGPU_E_DIVERGED      -6   /* main.f90:227 divergence guard        */
#define CAPPGPU_E_NOMEM         -7   /* device allocation failed             */

/* ------------------------------------------------- variable identifiers  */
/* modules_allocatable.f90:37 (iu=1 .. icon=10); 1-based like the reference */
#define CAP_IU   1
#define CAP_IV   2
#define CAP_IW   3
#define CAP_IP   4
#define CAP_ITE  5
#define CAP_IED  6
#define CAP_IEN  7
#define CAP_IVIS 8
#define CAP_IVART 9
#define CAP_ICON 10
#define CAP_NPHI 10

/* ------------------------------------------------------------ field ids  */
/* One id per reference module array that the hot path reads or writes.   */
enum cappgpu_field {
  /* module geometry (modules_allocatable.f90:147-159) */
  CAP_X = 0, CAP_Y, CAP_Z, CAP_XC, CAP_YC, CAP_ZC, CAP_VOL,
  CAP_FX, CAP_FY, CAP_FZ,
  CAP_AR1X, CAP_AR1Y, CAP_AR1Z, CAP_AR2X, CAP_AR2Y, CAP_AR2Z,
  CAP_AR3X, CAP_AR3Y, CAP_AR3Z, CAP_WALLDIST,
  /* module variables (:274-296) */
  CAP_U, CAP_V, CAP_W, CAP_P, CAP_PP, CAP_F1, CAP_F2, CAP_F3,
  CAP_VIS, CAP_DEN, CAP_TE, CAP_ED, CAP_T, CAP_STRAIN,
  /* module time_mod (:337-343) */
  CAP_UO, CAP_VO, CAP_WO, CAP_UOO, CAP_VOO, CAP_WOO,
  /* module coef (:161-170) */
  CAP_AE, CAP_AW, CAP_AN, CAP_AS, CAP_AT, CAP_AB, CAP_AP,
  CAP_SP, CAP_SPV, CAP_SU, CAP_SV, CAP_SW, CAP_RES,
  CAP_APU, CAP_APV, CAP_APW,
  /* module coefb (:172-180) -- SIP factors, full extent (ghost layers are
     read by the factorisation, sipsol.f90:34-46) */
  CAP_BB, CAP_BS, CAP_BW, CAP_BP, CAP_BN, CAP_BE, CAP_BT,
  /* module hcoef (:182-190) */
  CAP_HE, CAP_HW, CAP_HN, CAP_HS, CAP_HT, CAP_HB,
  /* module gradients (:389-398), stored as three component arrays each
     (the reference stores (3,nxyza); component c of cell ijk is
     gradX(c,ijk)) */
  CAP_GRADU_X, CAP_GRADU_Y, CAP_GRADU_Z,
  CAP_GRADV_X, CAP_GRADV_Y, CAP_GRADV_Z,
  CAP_GRADW_X, CAP_GRADW_Y, CAP_GRADW_Z,
  CAP_GRADP_X, CAP_GRADP_Y, CAP_GRADP_Z,
  /* two-equation turbulence models (calcscm.f90, calculate_stuff_for_sst.f90,
     modules variables, time_mod, gradients and omega_turb_models): gradte
     and graded as component arrays, the production gen, the SST blending
     results alphasst, bettasst, domega, prtinv_te, prtinv_ed, and the old
     time levels of te and ed */
  CAP_GRADTE_X, CAP_GRADTE_Y, CAP_GRADTE_Z,
  CAP_GRADED_X, CAP_GRADED_Y, CAP_GRADED_Z,
  CAP_GEN, CAP_ALPHASST, CAP_BETTASST, CAP_DOMEGA, CAP_PRTINV_TE, CAP_PRTINV_ED,
  CAP_TEO, CAP_EDO, CAP_TEOO, CAP_EDOO,
  CAP_NFIELDS
};

/* BC code arrays (module bc, modules_allocatable.f90:215-219):
   lbw/lbe indexed (j-1)*nk+k (length nj*nk), lbs/lbn (i-1)*nk+k (ni*nk),
   lbb/lbt (i-1)*nj+j (ni*nj).  Codes: 1 inlet, 2 outlet, 3 symmetry,
   4 wall (update_values_at_ghostcells_nonperiodic.f90:73,88,103,119). */
enum cappgpu_bcface { CAP_LBW = 0, CAP_LBE, CAP_LBS, CAP_LBN, CAP_LBB, CAP_LBT, CAP_NBC };

/* ------------------------------------------------------------ parameters */
/* Scalars of modules parameters/time_mod/inlet/boundc that the hot path
   reads or writes (modules_allocatable.f90:15-109, 324-344, 380-387).
   Arrays indexed [ifi-1].  Logical flags are 0/1 ints. */
typedef struct cappgpu_params {
  double alfa;          /* SIP factor, init.f90:164 (0.92)                 */
  double densit, viscos;
  double timestep, btime, time;
  double uin, vin, win, tein, edin, tin;
  double flowin, zero;  /* zero == 0.0d0, init.f90:342                   */
  double cappa, elog;   /* init.f90:167-168                                */
  double gradpcmf;
  double gravx, gravy, gravz, beta, tref;
  double conumfixvalue, conum, meanconum;
  double localconterr, sumlocalconterr, globalconterr, cumulativeconterr;
  double sor[CAP_NPHI], resor[CAP_NPHI], snorin[CAP_NPHI];
  double urf[CAP_NPHI], gds[CAP_NPHI];
  int    nsw[CAP_NPHI];
  int    lcal[CAP_NPHI];
  int    ipr, jpr, kpr;             /* pressure reference cell             */
  int    ncorr, npcor, icorr, ipcorr;
  int    bdf, cn;
  int    lcds, lluds, lquds, lsmart, lavl, lmuscl, lumist, lgamma, lcds4;
  int    flux_limiter;
  int    const_mflux, lbuoy, boussinesq, lout, ltransient, lles;
  int    periodic;                  /* 1: update_values_at_ghostcells.f90,
                                       0: ..._nonperiodic.f90              */
  int    conumfix;
  int    isol_p;                    /* calcp p' solver, calcp...f90:22 (5)  */
  int    piso_solver;               /* PISO p solver, PISO_multiple_correction.f90:138-142 (4 = pcgsip) */
  int    low, loe, los, lon, lob, lot;   /* outlet faces present, read with the
                                       grid (read_grid.f90:140); outbc    */
  int    sst;                       /* Menter k-omega SST for te (k) and ed
                                       (omega) when lcal(ite), lcal(ied)  */
  double cmu;                       /* module cmu: init.f90:177 sets 0.09 for
                                       standard k-epsilon only; modvis reads
                                       it in the SST branch as well       */
  int    top_plane;                 /* top-wall plane of calcuvw.f90:254 and
                                       calc_vis_les.f90:174: 0 = lk(nimm) as
                                       the reference writes it (the top wall
                                       only when ni = nk), 1 = lk(nkmm)    */
  int    pad_;
} cappgpu_params;

/* Report of one linear solve (the reference writes these three numbers to
   unit 66, e.g. pcg-sip.f90:195-197). */
typedef struct cappgpu_solve_report {
  double res0;      /* initial L1 residual                                 */
  double resl;      /* final L1 residual                                   */
  int    iters;     /* sweeps / iterations done (the reference's l or n)   */
  int    status;    /* CAPPGPU_OK / CAPPGPU_NOT_CONVERGED / <0             */
} cappgpu_solve_report;

/* Solver selector values (match the reference's isol switches,
   calcp-multiple_correction_SIMPLE.f90:98-102). */
#define CAPPGPU_SOLVER_SIPSOL     1
#define CAPPGPU_SOLVER_CGSTAB     2
#define CAPPGPU_SOLVER_ICCG       3
#define CAPPGPU_SOLVER_PCGSIP     4
#define CAPPGPU_SOLVER_CGSTAB_SIP 5
#define CAPPGPU_SOLVER_DPCG       6

/* ======================================================= lifecycle / data */

/* Create the context for an ni x nj x nk grid (storage extents, i.e.
   interior cells + 4 per axis).  Replaces set_parameters (set_parameters.f90:22-41,
   with nxyza := nxyz) + allocate_arrays + setind (setind.f90:21-58).
   Every field is zero-initialised on the device. */
int cappgpu_init(int ni, int nj, int nk);
int cappgpu_finalize(void);
const char* cappgpu_last_error(void);
const char* cappgpu_field_name(int field);
int cappgpu_field_id(const char* name);     /* -1 if unknown */

/* Copy a whole field host->device / device->host (n must equal nijk). */
int cappgpu_set_field(int field, const double* host, int64_t n);
int cappgpu_get_field(int field, double* host, int64_t n);
/* BC codes (read_grid.f90:136-140). */
int cappgpu_set_bc(int face, const int* codes, int64_t n);
/* Module scalars (read_input.f90:28-59 / init.f90:164-344). */
int cappgpu_set_params(const cappgpu_params* p);
int cappgpu_get_params(cappgpu_params* p);

/* Address registry for the drop-in (host-pointer) entry points: associates
   a host module array (e.g. the Fortran shim's c_loc(u)) with a field.
   Entry points ending in _h accept host pointers; a registered pointer is
   copied to its field before the call and back after it. */
int cappgpu_register(int field, double* host);
int cappgpu_unregister_all(void);

/* ============================================================== geometry */
/* Face area vectors ar1*,ar2*,ar3* and interpolation factors fx,fy,fz from
   the nodes x,y,z and cell centres xc,yc,zc already set in the context:
   init.f90:54-136 (face areas) and init.f90:142-144 -> intfac.f90:25-48.
   orient = 0 keeps init.f90's cross products verbatim (on a right-handed
   grid they point east faces to +i but north/top faces to -j/-k);
   orient = 1 negates ar2*,ar3* so that all three point to increasing index,
   the orientation GRAD_GAUSS.f90:57-81 and the flux routines assume. */
int cappgpu_build_geometry(int orient);
/* find_intersection_point.f90:1-76 evaluated on the device; p holds
   x1,y1,z1,...,x5,y5,z5 (15 doubles), out receives xj,yj,zj. */
int cappgpu_find_intersection_point(const double* p, double* out);

/* Run-time options.  "wave": 1 = SIP factorisation/substitutions of pcgsip
   as persistent hyperplane wavefronts (default), 0 = one kernel launch per
   hyperplane (the simple form, kept for cross-checks).
   "tight_correctors": 0 = the reference's tolerances (default: every PISO
   corrector but the last solves p to sor(ip) = 0.1 only,
   PISO_multiple_correction.f90:131-135), 1 = every corrector solves to the
   last one's tolerance.  Where the first corrector stops decides the step's
   result to well above the arithmetic's precision, so two precision modes
   are compared with 1; it is not the reference's algorithm.
   "fp32_parts": bitmask of the parts that run in FP32 in precision modes
   1-2 (default 11 = 1|2|8): 1 the pressure solve (pcgsip), 2 the momentum
   solves (sipsol), 4 the momentum assembly (fluxuvw, LES strain rate and
   viscosity), 8 the velocity gradients (grad_gauss of u, v, w), 16 the
   PISO pressure-equation assembly.  Parts 1, 2 and 8 keep every field
   within 1e-5 (velocity components) of the FP64 form over 20 steps of the
   128^3 channel; parts 4 and 16 change the FP64 system the refinement
   solves and are off by default.
   "sweep_timing": 1 = CUDA events around every FP64 pcgsip forward
   substitution (read by cappgpu_sweep_stats; default 0).
   "fused_dot": 1 = the FP32 CG of precision modes 1-2 forms sk = r.z in the
   backward substitution (wavefront engine 0, default); 0 = in a vector
   pass after it, as the other engines do (the same sum in another order).
   "lane_wave": engine of the FP32 SIP substitutions of precision modes 1-2:
   0 = the persistent hyperplane wavefront, one thread per line (default);
   1 = one warp per tile of 32 x 8 lines, neighbours by shuffles and
   registers, no barrier per hyperplane.  Both give the same bits; on GB300
   1 is slower at 128^3 (192 vs 152 us per forward sweep) and level at 256^3.
   "face_geo": 1 = the FP64 face kernels of fluxuvw and the PISO pressure
   assembly read the geometric part of each face (centre distance, face
   area, cosine of the non-orthogonality, area/volume ratios, face-centre
   offsets), and the FP64 Gauss gradient 1/vol, from arrays built once per
   grid, rebuilt after any write into a geometry field or vol (default; 37
   arrays of nijk doubles); 0 = evaluate them on every call.  Both give the
   same bits.
   "sip_slabs": in precision modes 1-2 with lane_wave 0 the FP32 SIP
   factorisation and substitutions restart at every slab of the interior
   (1..4096, default 4096; 1 = over the whole box): block-local SIP per
   slab, as the reference's SIP runs per MPI rank, so the slabs'
   recurrences run side by side.  The FP32 blocks are 8 lines along i and
   32 along k; the count used is the largest n <= sip_slabs, n >= 2, that
   divides the number of block columns along i (ceil(Ni/8)), or along k for
   which the interior extent is a multiple of n x 32; with none, the whole
   box.  The default makes every 8-line block column along i a slab of its
   own.  It changes the preconditioner of the refinement, not its FP64 exit
   test.
   "sip_slab_axis": the axis of those slabs, 0 = i (default), 1 = k.
   "cg_batch": conjugate-gradient iterations of pcgsip launched between two
   host reads of the device-side exit test (1..64, default 4; surplus
   iterations after the exit return at once).
   "inner_drop": in precision modes 1-2 the FP32 conjugate-gradient loop of
   pcgsip stops once its residual has dropped by 10^-inner_drop (1..9,
   default 4) and restarts from the FP64 residual.
   "learn_conv": convolutions of the learned guess's net, 1 = tcgen05
   (default), 0 = mma.sync (kept for cross-checks).
   "learn_loss": the training loss of cappgpu_learn_train, 0 = residual
   norm |A^ d - r^|^2/|r^|^2 on the window (default; the learned-guess
   configuration's), 1 = supervised |d - t^|^2/|t^|^2 against the recorded
   converged correction, 2 = its energy norm (d - t^)'A^(d - t^)/t^'A^t^.
   "spin_limit": polls a wavefront block makes on a predecessor's edge
   states (and 64x as many on its own input copies) before it gives up,
   raises the device-wide abort flag and the solve returns CAPPGPU_E_SPIN
   (>= 1, default 2^21, about a second).  After CAPPGPU_E_SPIN the library
   resets the block tickets and edge mailboxes, so the next solve runs
   normally. */
int cappgpu_set_option(const char* key, int value);

/* Arithmetic of the step.  0 = FP64 plain, the reference's arithmetic
   (default).  1 = FP32 inside FP64 iterative refinement:
   - pcgsip: the SIP factors and both substitutions in FP32 inside conjugate
     gradients in FP32, wrapped in an FP64 refinement loop whose exit test
     is the reference's (L1 norm of the FP64 residual su - A fi over res0
     below sor(ifi), pcg-sip.f90:185-188);
   - sipsol: FP64 residual and exit test per sweep (sipsol.f90:60-69, 96),
     FP32 factors and substitutions, FP64 update of fi;
   - the velocity gradients in FP32 arithmetic with FP64 storage (and, when
     option fp32_parts asks for them, the coefficient assembly);
   residuals, norms, dot products, the flux and velocity corrections, the
   pressure gradient and the continuity error stay FP64.  The iterates are
   not the reference's.  2 = mode 1 with the learned initial guess of the
   pressure solve (below).  Returns CAPPGPU_E_ARG for other modes. */
int cappgpu_precision(int mode);

/* ================================================ learned initial guess */
/* No counterpart in the reference.  A 3-level 3-D convolutional U-Net
   (3x3x3 kernels, 16/32/64 channels, average pooling, nearest up-sampling,
   skip concatenation, ReLU, then 1x1x1 to one channel; BF16 on the tensor
   cores, FP32 accumulation and master weights, Adam) predicts the
   correction d of a pressure solve, A d = r0, from its initial residual
   normalised by its RMS, trained on the residual-norm loss
   |A^ d - r^|^2/|r^|^2 with the solve's own operator (normalised by the
   mean diagonal) on random block^3 windows.  In precision mode 2 the
   refinement form of cappgpu_pcgsip starts from fi + alpha*guess (alpha by
   least squares) when that lowers the FP64 residual and from fi otherwise;
   its exit test stays relative to the residual of fi, so the plain solve is
   judge and fallback.
   cappgpu_learn_reset     (re)creates the net with seeded weights and room
                           for max_samples recorded pairs of this grid
   cappgpu_learn_windows   records random block^3 windows of the solves
                           instead of the whole interior, per_solve windows
                           per solve, into the room of max_samples windows
                           (block a multiple of 4 within the interior);
                           clears the recorded pairs
   cappgpu_learn_collect   records (initial residual, operator) of the
                           pressure solves that follow (precision 1 or 2)
   cappgpu_learn_train     Adam on random block^3 windows of the pairs
                           (block rounded down to a multiple of 4);
                           *loss = mean loss of the last epoch
   cappgpu_learn_params    FP32 parameters out (direction 0) or in (1, Adam's
                           moments reset); with host == NULL returns the
                           parameter count
   cappgpu_learn_stats     pairs recorded, guesses kept, guesses discarded,
                           residual ratio of the last guess
   cappgpu_learn_check     one forward and backward pass on a D x H x W
                           normalised residual and its window operator
                           (7 planes xp, xm, yp, ym, zp, zm, diag; extents
                           multiples of 4) from the host, for tests: output,
                           parameter gradients and loss
   cappgpu_learn_check_loss the same with the loss kind of option
                           "learn_loss" (0 residual norm |A d - r|^2/|r|^2,
                           1 supervised |d - t|^2/|t|^2, 2 energy norm
                           (d - t)'A(d - t)/t'At) and, for kinds 1-2, the
                           target t
   cappgpu_learn_sample    copies recorded pair `index` out: 9 planes of
                           the sample's extent (r^ = r0/rms(r0); A^ = A /
                           mean(ap) as xp, xm, yp, ym, zp, zm, diag; the
                           solve's converged correction t^ = (fi_end -
                           fi_start) mean(ap)/rms(r0), so A^ t^ = r^ to the
                           solve's tolerance); n must be that count */
int cappgpu_learn_reset(int max_samples, unsigned long long seed);
int cappgpu_learn_windows(int block, int per_solve);
int cappgpu_learn_collect(int on);
int cappgpu_learn_train(int epochs, int block, double lr, double* loss);
int cappgpu_learn_params(float* host, int n, int direction);
int cappgpu_learn_stats(int* samples, int* guesses, int* fallbacks, double* last_ratio);
/* Amplitude alpha and level beta of the last guess (fi + alpha d + beta on
   the interior, Galerkin projection onto span{d, 1}). */
int cappgpu_learn_fit(double* alpha, double* beta);
int cappgpu_learn_check(const float* rhs, const float* coef, int D, int H, int W, float* output, float* grad,
                        double* loss);
int cappgpu_learn_check_loss(int kind, const float* rhs, const float* coef, const float* target, int D, int H, int W,
                             float* output, float* grad, double* loss);
int cappgpu_learn_sample(int index, float* host, long long n);

/* ================================================= LES sub-grid viscosity */
/* find_strain_rate.f90:20-79 (gauss branch): Green-Gauss gradients of u, v,
   w into the module gradients, then strain = sqrt(2 s_ij s_ij) on
   k=2..nkm, i=3..nimm, j=3..njmm (the vorticity invariant is not kept). */
int cappgpu_find_strain_rate(void);
/* calc_vis_les.f90:38-249: Smagorinsky viscosity with Van Driest damping
   into vis (same box, under-relaxed by urf(ivis)), then the wall-function
   viscosity of the bottom and top ghost layers.  The step drivers call both
   after the pressure-velocity coupling when lcal(ivis) and lles are set
   (main.f90:205). */
int cappgpu_calc_vis_les(void);
/* const_massflux_correction.f90:1-22: the volume-weighted averages of u and
   apu (fieldManipulation.f90:10-44), the pressure-gradient increment that
   restores the bulk velocity uin, u += apu * increment (whole array),
   gradpcmf += increment.  cappgpu_piso_steps runs it at the end of every
   step when ltransient and const_mflux are set (main.f90:252). */
int cappgpu_const_massflux_correction(void);

/* ===================================================== k-omega SST (RANS) */
/* calcscm(fi,gradfi,ifi) (calcscm.f90:3-602) for ifi = ite (k in te) or
   ied (omega in ed) with the SST model (params.sst): the gradient of fi
   into gradte / graded, the volume sources (k: production |vis - viscos|
   S^2 limited to 0.9 rho k omega, destruction; omega:
   calculate_stuff_for_sst.f90:27-70 -- blending, cross diffusion --, then
   alphasst P / nu_t and bettasst rho omega), the implicit time term, the
   face fluxes of fluxscm-overrelaxed-correction.f90:40-230 in three
   directions, Crank-Nicolson terms, ap and under-relaxation, sipsol
   (rep), and fi >= small on the whole array.  The step drivers run both
   after the pressure-velocity coupling when lcal(ite) / lcal(ied) and sst
   are set (main.f90:196-197). */
int cappgpu_calcscm(int ifi, cappgpu_solve_report* rep);
/* modvis (modvis.f90:195-236, SST branch): eddy viscosity
   viscos + rho a1 k / max(a1, omega, S F2) (the reference's three-argument
   MAX), under-relaxed by urf(ivis); run by the step drivers when
   lcal(ivis), sst and not lles (main.f90:203). */
int cappgpu_modvis(void);
/* Host-pointer drop-ins: fi must be the registered te or ed and gradfi
   the interleaved array registered for gradte or graded. */
int cappgpu_calcscm_h(double* fi, double* gradfi, int ifi);
int cappgpu_modvis_h(void);

/* ======================================================= index maps (a1) */
/* setind.f90:34-40: li(i)=(i-1)*nj for i=1..ni, lk(k)=(k-1)*nij.  Writes
   the device copies back (tests compare them element-wise). */
int cappgpu_get_index_maps(int* li, int* lk);
/* ijk of the pressure reference cell, setind.f90:56 */
int cappgpu_ijkpr(void);

/* ====================================================== ghost cells (a2) */
/* update_values_at_ghostcells: nonperiodic variant
   (update_values_at_ghostcells_nonperiodic.f90:47-640) when
   params.periodic == 0, periodic variant (update_values_at_ghostcells.f90:40-145)
   otherwise.  Writes ghost values of u,v,w,te,ed,t,vis. */
int cappgpu_update_values_at_ghostcells(void);
/* exchange(phi), exchange_mpi.f90:4-89: on one GPU there is no neighbour
   rank, so the halo exchange is the identity on phi (the reference's
   single-rank self-SENDRECV_REPLACE). Kept for drop-in completeness. */
int cappgpu_exchange(int field);
/* global_sum / global_max (global_sum_mpi.f90:4-36, global_max_mpi.f90:4-35):
   identity on one rank; the device reductions inside the kernels replace
   the MPI_ALLREDUCE. */
int cappgpu_global_sum(double* phi);
int cappgpu_global_max(double* phi);

/* ========================================================= gradient (a3) */
/* grad_gauss(u,dudx,dudy,dudz), GRAD_GAUSS.f90:1-105. */
int cappgpu_grad_gauss(int u, int dudx, int dudy, int dudz);
int cappgpu_grad_gauss_h(const double* u, double* dudx, double* dudy, double* dudz);

/* ======================================================= linear solvers  */
/* Each solves the 7-diagonal system ae..ab,ap,su of module coef for field
   fi with parameters sor(ifi), nsw(ifi); writes resor(ifi), res and (SIP
   based) the factors bb..bt, exactly as the reference routine.
   sipsol.f90:3-106, pcg-sip.f90:3-200, iccg.f90:3-197, cgstab.f90:3-283,
   cgstab_sip.f90:3-279, pcg-jacobi.f90:3-155. */
int cappgpu_sipsol(int fi, int ifi, cappgpu_solve_report* rep);
int cappgpu_pcgsip(int fi, int ifi, cappgpu_solve_report* rep);
int cappgpu_iccg(int fi, int ifi, cappgpu_solve_report* rep);
int cappgpu_cgstab(int fi, int ifi, cappgpu_solve_report* rep);
int cappgpu_cgstab_sip(int fi, int ifi, cappgpu_solve_report* rep);
int cappgpu_dpcg(int fi, int ifi, cappgpu_solve_report* rep);
/* Host-pointer drop-ins: fi is a registered host module array. */
int cappgpu_sipsol_h(double* fi, int ifi);
int cappgpu_pcgsip_h(double* fi, int ifi);
int cappgpu_iccg_h(double* fi, int ifi);
int cappgpu_cgstab_h(double* fi, int ifi);
int cappgpu_cgstab_sip_h(double* fi, int ifi);
int cappgpu_dpcg_h(double* fi, int ifi);

/* 7-point product z = A p (the pcgsip SpMV pass, pcg-sip.f90:142-153) with
   the fused dot pk.z over the interior; exposed for tests and benches.
   zk may not be pk, a matrix coefficient (ae..ap) or a geometry field
   (CAPPGPU_E_ARG). */
int cappgpu_spmv(int pk, int zk, double* dot);

/* cappgpu_spmv without any device allocation; no counterpart in the
   reference.  For callers that cannot allocate device memory where they need
   the product (the device pool is held by another allocator, or cudaMalloc's
   implicit synchronisation is not acceptable inside the step loop).  zk is
   the same as cappgpu_spmv's (and obeys the same restrictions); the dot is
   summed in a different fixed order.  The device current at the call must
   be the one cappgpu_init ran on (CAPPGPU_E_ARG otherwise).
   The reduction scratch is a fixed 32 KB device array: grids with more than
   8,388,608 interior cells are rejected with CAPPGPU_E_ARG.  The first call
   on a device performs a one-time set-up (it looks up the array's device
   address) and should come before any stream capture.  Calls that overlap
   share the scratch and race. */
int cappgpu_spmv_noalloc(int pk, int zk, double* dot);

/* ================================================ assembly / PISO / SIMPLE */
/* fluxuvw(idew,idns,idtb, arvx,arvy,arvz, fif,acfe,acfw,fcf),
   fluxuvw-overrelaxed-correction.f90:3-659.  Field ids for the arrays. */
int cappgpu_fluxuvw(int idew, int idns, int idtb, int arvx, int arvy, int arvz,
                    int fif, int acfe, int acfw, int fcf);
/* calcuvw (calcuvw.f90:3-464): gradients, sources, face fluxes, wall terms,
   assembly and three sipsol solves.  rep may be NULL or point to 3 reports. */
int cappgpu_calcuvw(cappgpu_solve_report* rep);
/* piso_assemble_pressure_eq(..., ipc, bp), PISO_assemble_pressure_eq.f90:3-257 */
int cappgpu_piso_assemble_pressure_eq(int idew, int idns, int idtb, int arvx, int arvy,
                                      int arvz, int fif, int acfe, int acfw, int fcf,
                                      int ipc, int bp);
/* assemble_pressure_eq(...), assemble_pressure_eq.f90:3-124 (not in the
   reference build; drop-in interface only). */
int cappgpu_assemble_pressure_eq(int idew, int idns, int idtb, int arvx, int arvy,
                                 int arvz, int fif, int acfe, int acfw, int fcf);
/* PISO_getHbyA, PISO_getHbyA.f90:3-233 */
int cappgpu_piso_gethbya(void);
/* bpres(p), bpres.f90:3-81 */
int cappgpu_bpres(int p);
/* PISO_multiple_correction, PISO_multiple_correction.f90:3-296.  rep may be
   NULL or point to ncorr*npcor reports (one per pressure solve). */
int cappgpu_piso_multiple_correction(cappgpu_solve_report* rep);
/* fluxmass(...), fluxmass2.f90:3-195 (Rhie-Chow face flux) */
int cappgpu_fluxmass(int idew, int idns, int idtb, int arvx, int arvy, int arvz,
                     int fif, int acfe, int acfw, int fcf);
/* calcp (SIMPLE), calcp-multiple_correction_SIMPLE.f90:3-238 */
int cappgpu_calcp(cappgpu_solve_report* rep);
/* outbc, outbc.f90:3-318: with lout, rescales the outlet faces (code 2)
   of the face sets flagged low..lot so that their mass flow equals
   flowin.  The flow is summed in the routine's loop order (on the host,
   from the device-formed face fluxes), so the result is bit-exact. */
int cappgpu_outbc(void);
/* correctBoundaryConditions, correctBoundaryConditions.f90:1-86 */
int cappgpu_correct_boundary_conditions(void);
/* CourantNo.h:10-66 (timestep may change when conumfix) */
int cappgpu_courant(void);
/* continuityErrors.h:55-83 */
int cappgpu_continuity_errors(void);

/* ============================================================ step drivers */
/* One iteration of main.f90:178-207 for PISO (ghost update, calcuvw, outbc,
   PISO_multiple_correction) preceded, when transient, by the time-level
   shift of main.f90:140-157 and CourantNo.h.  nsteps time steps. */
int cappgpu_piso_steps(int nsteps, cappgpu_solve_report* last_p_report);
/* nsteps SIMPLE outer iterations (ghost update, calcuvw, calcp). */
int cappgpu_simple_iters(int niters, cappgpu_solve_report* last_p_report);

/* ====================================== host-pointer drop-ins (assembly) */
/* For a host program that keeps the reference's module arrays in host
   memory and calls the routines one at a time with its own arrays (the
   Fortran shim).  Each call copies the registered module arrays the
   routine reads to the device, resolves every array argument by address
   (a registered array is its field; any other array is copied into a
   staging array, at most 8 per call), runs the routine, copies back the
   registered arrays it writes and the written arguments, and synchronises.
   Grid geometry is device-resident: uploaded once with cappgpu_set_field
   (or cappgpu_build_geometry) and never copied by these calls; register
   geometry arrays only so that they are recognised as arguments. */
/* Interleaved (3, nijk) host array -- the reference's gradu(3,nxyza)
   layout -- for the three component fields starting at field_x (one of
   CAP_GRADU_X, CAP_GRADV_X, CAP_GRADW_X, CAP_GRADP_X, CAP_GRADTE_X,
   CAP_GRADED_X); NULL unregisters. */
int cappgpu_register_vec3(int field_x, double* host);
/* update_values_at_ghostcells (update_values_at_ghostcells_nonperiodic.f90:3-642) */
int cappgpu_update_values_at_ghostcells_h(void);
/* bpres(p) (bpres.f90:3-81) */
int cappgpu_bpres_h(double* p);
/* exchange(phi) (exchange_mpi.f90:4-89): the identity on one rank */
int cappgpu_exchange_h(double* phi);
/* fluxuvw(idew,idns,idtb,arvx,arvy,arvz,fif,acfe,acfw,fcf)
   (fluxuvw-overrelaxed-correction.f90:3) */
int cappgpu_fluxuvw_h(int idew, int idns, int idtb, const double* arvx, const double* arvy, const double* arvz,
                      const double* fif, double* acfe, double* acfw, const double* fcf);
/* piso_assemble_pressure_eq(idew,idns,idtb,arvx,arvy,arvz,fif,acfe,acfw,fcf,ipc,bp)
   (PISO_assemble_pressure_eq.f90:3) */
int cappgpu_piso_assemble_pressure_eq_h(int idew, int idns, int idtb, const double* arvx, const double* arvy,
                                        const double* arvz, const double* fif, double* acfe, double* acfw,
                                        double* fcf, int ipc, double* bp);
/* assemble_pressure_eq(idew,idns,idtb,arvx,arvy,arvz,fif,acfe,acfw,fcf)
   (assemble_pressure_eq.f90:3) */
int cappgpu_assemble_pressure_eq_h(int idew, int idns, int idtb, const double* arvx, const double* arvy,
                                   const double* arvz, const double* fif, double* acfe, double* acfw, double* fcf);
/* calcuvw (calcuvw.f90:3), PISO_getHbyA (PISO_getHbyA.f90:3) and
   PISO_multiple_correction (PISO_multiple_correction.f90:3): every
   registered non-geometry module array is copied in before and back
   after.  rep as for the field-id entry points. */
int cappgpu_calcuvw_h(cappgpu_solve_report* rep);
int cappgpu_piso_gethbya_h(void);
int cappgpu_piso_multiple_correction_h(cappgpu_solve_report* rep);
/* The last linear solve run through the solver selector (the *_h and
   field-id solver entry points, PISO and SIMPLE pressure solves): solver
   code, ifi and report. */
int cappgpu_last_report(int* solver, int* ifi, cappgpu_solve_report* rep);
/* The reference's unit-66 line for a solve report (pcg-sip.f90:195-197,
   sipsol.f90:101-103, iccg.f90:192-194, cgstab.f90:278-280,
   cgstab_sip.f90:273-275 with icorr and ipcorr, pcg-jacobi.f90:150-152)
   into buf (n bytes, NUL-terminated); the iteration number is the Fortran
   loop index (iters + 1 when the solve did not converge). */
int cappgpu_solver_report_line(int solver, int ifi, const cappgpu_solve_report* rep, int icorr, int ipcorr,
                               char* buf, int n);

/* ======================================================= instrumentation */
typedef struct cappgpu_stats {
  long long launches;               /* kernels launched since cappgpu_init  */
  double    p_solve_ms;             /* device time of the last pressure solve */
  cappgpu_solve_report p_report;    /* its report                           */
} cappgpu_stats;

/* CUDA events on the library's stream around a region of calls. */
int cappgpu_timer_start(void);
/* With option "sweep_timing" 1: the summed duration (CUDA events on the
   library's stream) and count of the FP64 pcgsip forward SIP substitutions
   that ran since the last reset (those of iterations after the exit test,
   which return at once, are not counted); reset != 0 zeroes both after
   reading. */
int cappgpu_sweep_stats(double* ms_total, long long* launches, int reset);
int cappgpu_timer_stop(double* ms);
int cappgpu_get_stats(cappgpu_stats* s);
/* Page-locked host buffers (for host<->device copies at full speed). */
int cappgpu_host_alloc(void** p, int64_t bytes);
int cappgpu_host_free(void* p);
/* Time reps runs of one hot-path unit (0 SIP forward sweep, 1 SIP backward
   sweep, 2 7-point product + dot, 3 grad_gauss, 4 fluxuvw east, 5 PISO
   pressure assembly east, 6 SIP factorisation, 7 / 8 FP32 forward / backward
   sweep of the precision-1 form, 9 forward pass of the learned guess's net
   on this grid, 10 its forward and backward pass on a 64^3 window of the
   first recorded pair, 11 the FP64 issue-rate probe: independent FP64
   multiplies and adds filling every SM) on the current state; returns
   device ms per unit and its algorithmic bytes (units 9 and 10:
   algorithmic FLOPs; unit 11: FP64 lane-operations). */
int cappgpu_profile_kernel(int which, int reps, double* ms_per_unit, double* algo_bytes);

#ifdef __cplusplus
}
#endif
#endif /* CAPPGPU_H */
