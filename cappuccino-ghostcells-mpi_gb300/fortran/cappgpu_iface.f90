!***********************************************************************
!
! cappgpu_iface.f90 -- iso_c_binding interface to libcappgpu.so and the
! drop-in replacements of the reference's hot-path subroutines.
!
! A reference build leaves out its own pcg-sip.f90, sipsol.f90, iccg.f90,
! cgstab.f90, cgstab_sip.f90, pcg-jacobi.f90, GRAD_GAUSS.f90,
! fluxuvw-overrelaxed-correction.f90, calcuvw.f90,
! PISO_assemble_pressure_eq.f90, assemble_pressure_eq.f90, PISO_getHbyA.f90,
! PISO_multiple_correction.f90, bpres.f90, update_values_at_ghostcells*.f90,
! calcscm.f90, modvis.f90, exchange_mpi.f90, global_sum_mpi.f90 and
! global_max_mpi.f90, and links
! this file instead.  Each replacement below keeps the reference's name and
! dummy arguments.
!
! Module arrays are registered once by address with cappgpu_attach (after
! allocate_arrays and init).  Every drop-in then
!   1. hands the module scalars to the library (cappgpu_push_params),
!   2. calls the host-pointer entry point, which copies the registered
!      arrays the routine reads to the device, runs it there and copies
!      back what it writes (array arguments that are not module arrays --
!      gfortran temporaries of array sections -- are staged the same way),
!   3. takes back the scalars the routine sets (resor, time step, Courant
!      numbers, continuity errors, gradpcmf; cappgpu_pull_params),
!   4. writes the solver report lines to unit 66 in the reference's
!      formats, so that a log diffs against the reference's.
! Host code between the calls keeps working on the host arrays unchanged.
! A negative return code is fatal: it is written to unit 66 and the run
! ends through abort_mission, the reference's fatal path.
!
! Field ids and solver codes match include/cappgpu.h.
!
!***********************************************************************
module cappgpu
  use iso_c_binding
  implicit none

  integer(c_int), parameter :: CAP_X=0, CAP_Y=1, CAP_Z=2, CAP_XC=3, CAP_YC=4, CAP_ZC=5, CAP_VOL=6, &
       CAP_FX=7, CAP_FY=8, CAP_FZ=9, CAP_AR1X=10, CAP_AR1Y=11, CAP_AR1Z=12, CAP_AR2X=13, CAP_AR2Y=14, &
       CAP_AR2Z=15, CAP_AR3X=16, CAP_AR3Y=17, CAP_AR3Z=18, CAP_WALLDIST=19, CAP_U=20, CAP_V=21, CAP_W=22, &
       CAP_P=23, CAP_PP=24, CAP_F1=25, CAP_F2=26, CAP_F3=27, CAP_VIS=28, CAP_DEN=29, CAP_TE=30, CAP_ED=31, &
       CAP_T=32, CAP_STRAIN=33, CAP_UO=34, CAP_VO=35, CAP_WO=36, CAP_UOO=37, CAP_VOO=38, CAP_WOO=39, &
       CAP_AE=40, CAP_AW=41, CAP_AN=42, CAP_AS=43, CAP_AT=44, CAP_AB=45, CAP_AP=46, CAP_SP=47, CAP_SPV=48, &
       CAP_SU=49, CAP_SV=50, CAP_SW=51, CAP_RES=52, CAP_APU=53, CAP_APV=54, CAP_APW=55, &
       CAP_BB=56, CAP_BS=57, CAP_BW=58, CAP_BP=59, CAP_BN=60, CAP_BE=61, CAP_BT=62, &
       CAP_HE=63, CAP_HW=64, CAP_HN=65, CAP_HS=66, CAP_HT=67, CAP_HB=68, &
       CAP_GRADU_X=69, CAP_GRADV_X=72, CAP_GRADW_X=75, CAP_GRADP_X=78, &
       CAP_GRADTE_X=81, CAP_GRADED_X=84, CAP_GEN=87, CAP_ALPHASST=88, CAP_BETTASST=89, CAP_DOMEGA=90, &
       CAP_PRTINV_TE=91, CAP_PRTINV_ED=92, CAP_TEO=93, CAP_EDO=94, CAP_TEOO=95, CAP_EDOO=96, CAP_NFIELDS=97

  integer(c_int), parameter :: CAPPGPU_NOT_CONVERGED=1
  integer(c_int), parameter :: SOLVER_SIPSOL=1, SOLVER_CGSTAB=2, SOLVER_ICCG=3, SOLVER_PCGSIP=4, &
       SOLVER_CGSTAB_SIP=5, SOLVER_DPCG=6

  ! solvers of the composite routines: the pressure solve of PISO
  ! (PISO_multiple_correction.f90:138-142) and of SIMPLE (calcp, isol = 5)
  integer(c_int) :: cap_piso_solver = SOLVER_PCGSIP
  integer(c_int) :: cap_isol_p = SOLVER_CGSTAB_SIP

  ! C mirror of cappgpu_solve_report
  type, bind(c) :: cappgpu_solve_report
    real(c_double) :: res0, resl
    integer(c_int) :: iters, status
  end type

  ! C mirror of cappgpu_params (same members, same order)
  type, bind(c) :: cappgpu_params
    real(c_double) :: alfa, densit, viscos, timestep, btime, time
    real(c_double) :: uin, vin, win, tein, edin, tin
    real(c_double) :: flowin, zero, cappa, elog, gradpcmf
    real(c_double) :: gravx, gravy, gravz, beta, tref
    real(c_double) :: conumfixvalue, conum, meanconum
    real(c_double) :: localconterr, sumlocalconterr, globalconterr, cumulativeconterr
    real(c_double) :: sor(10), resor(10), snorin(10), urf(10), gds(10)
    integer(c_int) :: nsw(10), lcal(10)
    integer(c_int) :: ipr, jpr, kpr, ncorr, npcor, icorr, ipcorr, bdf, cn
    integer(c_int) :: lcds, lluds, lquds, lsmart, lavl, lmuscl, lumist, lgamma, lcds4, flux_limiter
    integer(c_int) :: const_mflux, lbuoy, boussinesq, lout, ltransient, lles, periodic, conumfix
    integer(c_int) :: isol_p, piso_solver, low, loe, los, lon, lob, lot, sst
    real(c_double) :: cmu
    integer(c_int) :: top_plane, pad_
  end type

  interface
    integer(c_int) function cappgpu_init(ni, nj, nk) bind(c, name="cappgpu_init")
      import :: c_int
      integer(c_int), value :: ni, nj, nk
    end function
    integer(c_int) function cappgpu_finalize() bind(c, name="cappgpu_finalize")
      import :: c_int
    end function
    ! 0 = FP64 plain (the reference's arithmetic), 1 = FP32 + FP64 refinement,
    ! 2 = 1 + the learned initial guess of the pressure solve
    integer(c_int) function cappgpu_precision(mode) bind(c, name="cappgpu_precision")
      import :: c_int
      integer(c_int), value :: mode
    end function
    ! key: NUL-terminated, e.g. "fp32_parts"//c_null_char
    integer(c_int) function cappgpu_set_option(key, val) bind(c, name="cappgpu_set_option")
      import :: c_int, c_char
      character(kind=c_char), intent(in) :: key(*)
      integer(c_int), value :: val
    end function
    ! learned initial guess: record pairs, train, report
    integer(c_int) function cappgpu_learn_reset(max_samples, seed) bind(c, name="cappgpu_learn_reset")
      import :: c_int, c_long_long
      integer(c_int), value :: max_samples
      integer(c_long_long), value :: seed
    end function
    integer(c_int) function cappgpu_learn_collect(on) bind(c, name="cappgpu_learn_collect")
      import :: c_int
      integer(c_int), value :: on
    end function
    integer(c_int) function cappgpu_learn_train(epochs, block, lr, loss) bind(c, name="cappgpu_learn_train")
      import :: c_int, c_double
      integer(c_int), value :: epochs, block
      real(c_double), value :: lr
      real(c_double), intent(out) :: loss
    end function
    integer(c_int) function cappgpu_learn_stats(samples, guesses, fallbacks, last_ratio) &
        bind(c, name="cappgpu_learn_stats")
      import :: c_int, c_double
      integer(c_int), intent(out) :: samples, guesses, fallbacks
      real(c_double), intent(out) :: last_ratio
    end function
    integer(c_int) function cappgpu_set_field(field, host, n) bind(c, name="cappgpu_set_field")
      import :: c_int, c_double, c_int64_t
      integer(c_int), value :: field
      real(c_double), intent(in) :: host(*)
      integer(c_int64_t), value :: n
    end function
    integer(c_int) function cappgpu_get_field(field, host, n) bind(c, name="cappgpu_get_field")
      import :: c_int, c_double, c_int64_t
      integer(c_int), value :: field
      real(c_double), intent(inout) :: host(*)
      integer(c_int64_t), value :: n
    end function
    integer(c_int) function cappgpu_set_bc(face, codes, n) bind(c, name="cappgpu_set_bc")
      import :: c_int, c_int64_t
      integer(c_int), value :: face
      integer(c_int), intent(in) :: codes(*)
      integer(c_int64_t), value :: n
    end function
    integer(c_int) function cappgpu_set_params(p) bind(c, name="cappgpu_set_params")
      import :: c_int, cappgpu_params
      type(cappgpu_params), intent(in) :: p
    end function
    integer(c_int) function cappgpu_get_params(p) bind(c, name="cappgpu_get_params")
      import :: c_int, cappgpu_params
      type(cappgpu_params), intent(out) :: p
    end function
    integer(c_int) function cappgpu_register(field, host) bind(c, name="cappgpu_register")
      import :: c_int, c_ptr
      integer(c_int), value :: field
      type(c_ptr), value :: host
    end function
    integer(c_int) function cappgpu_register_vec3(field_x, host) bind(c, name="cappgpu_register_vec3")
      import :: c_int, c_ptr
      integer(c_int), value :: field_x
      type(c_ptr), value :: host
    end function
    ! linear solvers on a registered module array fi
    integer(c_int) function cappgpu_pcgsip_h(fi, ifi) bind(c, name="cappgpu_pcgsip_h")
      import :: c_int, c_double
      real(c_double), intent(inout) :: fi(*)
      integer(c_int), value :: ifi
    end function
    integer(c_int) function cappgpu_sipsol_h(fi, ifi) bind(c, name="cappgpu_sipsol_h")
      import :: c_int, c_double
      real(c_double), intent(inout) :: fi(*)
      integer(c_int), value :: ifi
    end function
    integer(c_int) function cappgpu_iccg_h(fi, ifi) bind(c, name="cappgpu_iccg_h")
      import :: c_int, c_double
      real(c_double), intent(inout) :: fi(*)
      integer(c_int), value :: ifi
    end function
    integer(c_int) function cappgpu_cgstab_h(fi, ifi) bind(c, name="cappgpu_cgstab_h")
      import :: c_int, c_double
      real(c_double), intent(inout) :: fi(*)
      integer(c_int), value :: ifi
    end function
    integer(c_int) function cappgpu_cgstab_sip_h(fi, ifi) bind(c, name="cappgpu_cgstab_sip_h")
      import :: c_int, c_double
      real(c_double), intent(inout) :: fi(*)
      integer(c_int), value :: ifi
    end function
    integer(c_int) function cappgpu_dpcg_h(fi, ifi) bind(c, name="cappgpu_dpcg_h")
      import :: c_int, c_double
      real(c_double), intent(inout) :: fi(*)
      integer(c_int), value :: ifi
    end function
    integer(c_int) function cappgpu_last_report(solver, ifi, rep) bind(c, name="cappgpu_last_report")
      import :: c_int, cappgpu_solve_report
      integer(c_int), intent(out) :: solver, ifi
      type(cappgpu_solve_report), intent(out) :: rep
    end function
    integer(c_int) function cappgpu_grad_gauss_h(u, dudx, dudy, dudz) bind(c, name="cappgpu_grad_gauss_h")
      import :: c_int, c_double
      real(c_double), intent(in) :: u(*)
      real(c_double), intent(inout) :: dudx(*), dudy(*), dudz(*)
    end function
    ! assembly, ghost cells, PISO (host arrays resolved by address)
    integer(c_int) function cappgpu_fluxuvw_h(idew, idns, idtb, arvx, arvy, arvz, fif, acfe, acfw, fcf) &
        bind(c, name="cappgpu_fluxuvw_h")
      import :: c_int, c_double
      integer(c_int), value :: idew, idns, idtb
      real(c_double), intent(in) :: arvx(*), arvy(*), arvz(*), fif(*), fcf(*)
      real(c_double), intent(inout) :: acfe(*), acfw(*)
    end function
    integer(c_int) function cappgpu_piso_assemble_pressure_eq_h(idew, idns, idtb, arvx, arvy, arvz, fif, acfe, &
        acfw, fcf, ipc, bp) bind(c, name="cappgpu_piso_assemble_pressure_eq_h")
      import :: c_int, c_double
      integer(c_int), value :: idew, idns, idtb, ipc
      real(c_double), intent(in) :: arvx(*), arvy(*), arvz(*), fif(*)
      real(c_double), intent(inout) :: acfe(*), acfw(*), fcf(*), bp(*)
    end function
    integer(c_int) function cappgpu_assemble_pressure_eq_h(idew, idns, idtb, arvx, arvy, arvz, fif, acfe, acfw, &
        fcf) bind(c, name="cappgpu_assemble_pressure_eq_h")
      import :: c_int, c_double
      integer(c_int), value :: idew, idns, idtb
      real(c_double), intent(in) :: arvx(*), arvy(*), arvz(*), fif(*)
      real(c_double), intent(inout) :: acfe(*), acfw(*), fcf(*)
    end function
    integer(c_int) function cappgpu_update_values_at_ghostcells_h() &
        bind(c, name="cappgpu_update_values_at_ghostcells_h")
      import :: c_int
    end function
    integer(c_int) function cappgpu_bpres_h(p) bind(c, name="cappgpu_bpres_h")
      import :: c_int, c_double
      real(c_double), intent(inout) :: p(*)
    end function
    integer(c_int) function cappgpu_exchange_h(phi) bind(c, name="cappgpu_exchange_h")
      import :: c_int, c_double
      real(c_double), intent(inout) :: phi(*)
    end function
    integer(c_int) function cappgpu_global_sum(phi) bind(c, name="cappgpu_global_sum")
      import :: c_int, c_double
      real(c_double), intent(inout) :: phi
    end function
    integer(c_int) function cappgpu_global_max(phi) bind(c, name="cappgpu_global_max")
      import :: c_int, c_double
      real(c_double), intent(inout) :: phi
    end function
    integer(c_int) function cappgpu_calcuvw_h(rep) bind(c, name="cappgpu_calcuvw_h")
      import :: c_int, cappgpu_solve_report
      type(cappgpu_solve_report), intent(out) :: rep(3)
    end function
    integer(c_int) function cappgpu_calcscm_h(fi, gradfi, ifi) bind(c, name="cappgpu_calcscm_h")
      import :: c_int, c_double
      real(c_double), intent(inout) :: fi(*), gradfi(*)
      integer(c_int), value :: ifi
    end function
    integer(c_int) function cappgpu_modvis_h() bind(c, name="cappgpu_modvis_h")
      import :: c_int
    end function
    integer(c_int) function cappgpu_piso_gethbya_h() bind(c, name="cappgpu_piso_gethbya_h")
      import :: c_int
    end function
    integer(c_int) function cappgpu_piso_multiple_correction_h(rep) &
        bind(c, name="cappgpu_piso_multiple_correction_h")
      import :: c_int, cappgpu_solve_report
      type(cappgpu_solve_report), intent(out) :: rep(*)
    end function
  end interface

contains

  ! Register the module arrays of modules_allocatable.f90 with the library
  ! (call once after init).  Geometry and BC codes are uploaded here; the
  ! other arrays are copied by the drop-ins as each routine needs them.
  subroutine cappgpu_attach()
    use types
    use parameters
    use indexes
    use geometry
    use coef
    use coefb
    use hcoef
    use variables
    use time_mod
    use gradients
    use omega_turb_models
    use bc
    integer(c_int) :: rc
    integer(c_int64_t) :: n
    n = int(nijk, c_int64_t)
    rc = cappgpu_init(ni, nj, nk)
    call chk(rc, 'cappgpu_init')
    ! geometry: device-resident from here on; registered so that the
    ! drop-ins recognise these arrays as arguments
    call put(CAP_X, x); call put(CAP_Y, y); call put(CAP_Z, z)
    call put(CAP_XC, xc); call put(CAP_YC, yc); call put(CAP_ZC, zc); call put(CAP_VOL, vol)
    call put(CAP_FX, fx); call put(CAP_FY, fy); call put(CAP_FZ, fz)
    call put(CAP_AR1X, ar1x); call put(CAP_AR1Y, ar1y); call put(CAP_AR1Z, ar1z)
    call put(CAP_AR2X, ar2x); call put(CAP_AR2Y, ar2y); call put(CAP_AR2Z, ar2z)
    call put(CAP_AR3X, ar3x); call put(CAP_AR3Y, ar3y); call put(CAP_AR3Z, ar3z)
    call put(CAP_WALLDIST, wallDistance)
    rc = cappgpu_set_bc(0, lbw, int(njk, c_int64_t)); call chk(rc, 'lbw')
    rc = cappgpu_set_bc(1, lbe, int(njk, c_int64_t)); call chk(rc, 'lbe')
    rc = cappgpu_set_bc(2, lbs, int(nik, c_int64_t)); call chk(rc, 'lbs')
    rc = cappgpu_set_bc(3, lbn, int(nik, c_int64_t)); call chk(rc, 'lbn')
    rc = cappgpu_set_bc(4, lbb, int(nij, c_int64_t)); call chk(rc, 'lbb')
    rc = cappgpu_set_bc(5, lbt, int(nij, c_int64_t)); call chk(rc, 'lbt')
    ! state: module variables, time levels, matrix, SIP factors, H-coefficients
    call reg(CAP_U, u); call reg(CAP_V, v); call reg(CAP_W, w); call reg(CAP_P, p); call reg(CAP_PP, pp)
    call reg(CAP_F1, f1); call reg(CAP_F2, f2); call reg(CAP_F3, f3)
    call reg(CAP_VIS, vis); call reg(CAP_DEN, den); call reg(CAP_TE, te); call reg(CAP_ED, ed)
    call reg(CAP_T, t); call reg(CAP_STRAIN, strain)
    call reg(CAP_UO, uo); call reg(CAP_VO, vo); call reg(CAP_WO, wo)
    call reg(CAP_UOO, uoo); call reg(CAP_VOO, voo); call reg(CAP_WOO, woo)
    call reg(CAP_AE, ae); call reg(CAP_AW, aw); call reg(CAP_AN, an); call reg(CAP_AS, as)
    call reg(CAP_AT, at); call reg(CAP_AB, ab); call reg(CAP_AP, ap)
    call reg(CAP_SP, sp); call reg(CAP_SU, su); call reg(CAP_SV, sv); call reg(CAP_SW, sw)
    call reg(CAP_RES, res); call reg(CAP_APU, apu); call reg(CAP_APV, apv); call reg(CAP_APW, apw)
    call reg(CAP_BB, bb); call reg(CAP_BS, bs); call reg(CAP_BW, bw); call reg(CAP_BP, bp)
    call reg(CAP_BN, bn); call reg(CAP_BE, be); call reg(CAP_BT, bt)
    call reg(CAP_SPV, spv)
    call reg(CAP_HE, he); call reg(CAP_HW, hw); call reg(CAP_HN, hn); call reg(CAP_HS, hs)
    call reg(CAP_HT, ht); call reg(CAP_HB, hb)
    ! gradients are stored (3,nxyza): one interleaved registration each
    rc = cappgpu_register_vec3(CAP_GRADU_X, c_loc(gradu(1,1))); call chk(rc, 'gradu')
    rc = cappgpu_register_vec3(CAP_GRADV_X, c_loc(gradv(1,1))); call chk(rc, 'gradv')
    rc = cappgpu_register_vec3(CAP_GRADW_X, c_loc(gradw(1,1))); call chk(rc, 'gradw')
    rc = cappgpu_register_vec3(CAP_GRADP_X, c_loc(gradp(1,1))); call chk(rc, 'gradp')
    ! two-equation turbulence models (arrays allocated only with lturb)
    call reg(CAP_GEN, gen)
    call reg(CAP_TEO, teo); call reg(CAP_EDO, edo)
    if (allocated(teoo)) then
      call reg(CAP_TEOO, teoo); call reg(CAP_EDOO, edoo)
    endif
    if (allocated(gradte)) then
      rc = cappgpu_register_vec3(CAP_GRADTE_X, c_loc(gradte(1,1))); call chk(rc, 'gradte')
      rc = cappgpu_register_vec3(CAP_GRADED_X, c_loc(graded(1,1))); call chk(rc, 'graded')
    endif
    if (allocated(alphasst)) then
      call reg(CAP_ALPHASST, alphasst); call reg(CAP_BETTASST, bettasst); call reg(CAP_DOMEGA, domega)
      call reg(CAP_PRTINV_TE, prtinv_te); call reg(CAP_PRTINV_ED, prtinv_ed)
    endif
  contains
    subroutine put(f, a)
      integer(c_int), intent(in) :: f
      real(c_double), target, intent(inout) :: a(:)
      integer(c_int) :: r
      r = cappgpu_set_field(f, a, n)
      call chk(r, 'set_field')
      r = cappgpu_register(f, c_loc(a(1)))
      call chk(r, 'register')
    end subroutine
    subroutine reg(f, a)
      integer(c_int), intent(in) :: f
      real(c_double), target, intent(inout) :: a(:)
      integer(c_int) :: r
      r = cappgpu_register(f, c_loc(a(1)))
      call chk(r, 'register')
    end subroutine
  end subroutine

  ! The module scalars the routines read (read_input.f90, init.f90 values)
  ! into the library.
  subroutine cappgpu_push_params()
    use types
    use parameters
    use indexes
    use time_mod
    use inlet
    use boundc
    use buoy
    use bc
    type(cappgpu_params) :: q
    integer(c_int) :: rc
    rc = cappgpu_get_params(q)
    call chk(rc, 'get_params')
    q%alfa = alfa; q%densit = densit; q%viscos = viscos
    q%timestep = timestep; q%btime = btime; q%time = time
    q%uin = uin; q%vin = vin; q%win = win; q%tein = tein; q%edin = edin; q%tin = tin
    q%flowin = flowin; q%zero = zero; q%cappa = cappa; q%elog = elog; q%gradpcmf = gradpcmf
    q%gravx = gravx; q%gravy = gravy; q%gravz = gravz; q%beta = beta; q%tref = tref
    q%conumfixvalue = conumfixvalue; q%conum = conum; q%meanconum = meanconum
    q%localconterr = localconterr; q%sumlocalconterr = sumlocalconterr
    q%globalconterr = globalconterr; q%cumulativeconterr = cumulativeconterr
    q%sor = sor; q%resor = resor; q%snorin = snorin; q%urf = urf; q%gds = gds
    q%nsw = nsw; q%lcal = merge(1, 0, lcal)
    q%ipr = ipr; q%jpr = jpr; q%kpr = kpr
    q%ncorr = ncorr; q%npcor = npcor; q%icorr = icorr; q%ipcorr = ipcorr
    q%bdf = merge(1, 0, bdf); q%cn = merge(1, 0, cn)
    q%lcds = merge(1, 0, lcds); q%lluds = merge(1, 0, lluds); q%lquds = merge(1, 0, lquds)
    q%lsmart = merge(1, 0, lsmart); q%lavl = merge(1, 0, lavl); q%lmuscl = merge(1, 0, lmuscl)
    q%lumist = merge(1, 0, lumist); q%lgamma = merge(1, 0, lgamma); q%lcds4 = merge(1, 0, lcds4)
    q%flux_limiter = merge(1, 0, flux_limiter)
    q%const_mflux = merge(1, 0, const_mflux); q%lbuoy = merge(1, 0, lbuoy)
    q%boussinesq = merge(1, 0, boussinesq); q%lout = merge(1, 0, lout)
    q%ltransient = merge(1, 0, ltransient); q%lles = merge(1, 0, lles)
    q%periodic = merge(1, 0, periodic_boundary); q%conumfix = merge(1, 0, conumfix)
    q%isol_p = cap_isol_p; q%piso_solver = cap_piso_solver
    q%low = merge(1, 0, low); q%loe = merge(1, 0, loe); q%los = merge(1, 0, los)
    q%lon = merge(1, 0, lon); q%lob = merge(1, 0, lob); q%lot = merge(1, 0, lot)
    q%sst = merge(1, 0, sst); q%cmu = cmu
    rc = cappgpu_set_params(q)
    call chk(rc, 'set_params')
  end subroutine

  ! The scalars a routine sets, back into the modules.
  subroutine cappgpu_pull_params()
    use types
    use parameters
    use time_mod
    type(cappgpu_params) :: q
    integer(c_int) :: rc
    rc = cappgpu_get_params(q)
    call chk(rc, 'get_params')
    resor = q%resor
    timestep = q%timestep; time = q%time; conum = q%conum; meanconum = q%meanconum
    localconterr = q%localconterr; sumlocalconterr = q%sumlocalconterr
    globalconterr = q%globalconterr; cumulativeconterr = q%cumulativeconterr
    gradpcmf = q%gradpcmf
  end subroutine

  ! The unit-66 report line of a linear solve, in the reference solver's
  ! own format (pcg-sip.f90:195-197, sipsol.f90:101-103, iccg.f90:192-194,
  ! cgstab.f90:278-280, cgstab_sip.f90:273-275, pcg-jacobi.f90:150-152).
  ! l is the Fortran loop index after the solver loop: the iteration that
  ! passed the exit test, or nsw+1 when none did.
  subroutine solver_line(solver, ifi, rep)
    use parameters
    use title_mod
    integer(c_int), intent(in) :: solver, ifi
    type(cappgpu_solve_report), intent(in) :: rep
    integer :: l
    l = rep%iters
    if (rep%status == CAPPGPU_NOT_CONVERGED) l = l + 1
    select case (solver)
    case (SOLVER_PCGSIP)
      write(66,'(3a,1pe10.3,a,1pe10.3,a,i0)') &
      'PCG(SIP):  Solving for ',trim(chvarsolver(ifi)), &
      ', Initial residual = ',rep%res0,', fFinal residual = ',rep%resl,', No Iterations ',l
    case (SOLVER_SIPSOL)
      write(66,'(3a,1PE10.3,a,1PE10.3,a,I0)') &
      'SIP:  Solving for ',trim(chvarSolver(ifi)), &
      ', Initial residual = ',rep%res0,', Final residual = ',rep%resl,', No Iterations ',l
    case (SOLVER_ICCG)
      write(66,'(3a,1PE10.3,a,1PE10.3,a,I0)') &
      'PCG(IC0):  Solving for ',trim(chvarSolver(ifi)), &
      ', Initial residual = ',rep%res0,', Final residual = ',rep%resl,', No Iterations ',l
    case (SOLVER_CGSTAB)
      write(66,'(3a,1PE10.3,a,1PE10.3,a,I0)') &
      'BiCGStab(ILU(0)):  Solving for ',trim(chvarSolver(ifi)), &
      ', Initial residual = ',rep%res0,', Final residual = ',rep%resl,', No Iterations ',l
    case (SOLVER_CGSTAB_SIP)
      write(66,'(3a,i1,a,i1,2a,1PE10.3,a,1PE10.3,a,I0)') &
      'BiCGStab(SIP):  Solving for ',trim(chvarSolver(ifi)),'(icorr=',icorr,',npcor=',ipcorr,')', &
      ', Initial residual = ',rep%res0,', Final residual = ',rep%resl,', No Iterations ',l
    case (SOLVER_DPCG)
      write(66,'(3a,1PE10.3,a,1PE10.3,a,I0)') &
      'PCG(Jacobi):  Solving for ',trim(chvarSolver(ifi)), &
      ', Initial residual = ',rep%res0,', Final residual = ',rep%resl,', No Iterations ',l
    end select
  end subroutine

  ! A solver drop-in: parameters in, the solve, parameters out, the line.
  subroutine run_solver(rc, what)
    integer(c_int), intent(in) :: rc
    character(*), intent(in) :: what
    integer(c_int) :: solver, ifi, r
    type(cappgpu_solve_report) :: rep
    call chk(rc, what)
    call cappgpu_pull_params()
    r = cappgpu_last_report(solver, ifi, rep)
    call chk(r, 'last_report')
    call solver_line(solver, ifi, rep)
  end subroutine

  ! <0 from the library is fatal (abort_mission_mpi.f90:18-20 semantics)
  subroutine chk(rc, what)
    integer(c_int), intent(in) :: rc
    character(*), intent(in) :: what
    if (rc < 0) then
      write(66,'(a,a,a,i0)') ' cappgpu: ', what, ' failed, code ', rc
      call abort_mission
    endif
  end subroutine

end module cappgpu

!-----------------------------------------------------------------------
! Drop-in replacements with the reference's names and dummy arguments.
!-----------------------------------------------------------------------

! pcg-sip.f90:3-200
subroutine pcgsip(fi, ifi)
  use types
  use parameters
  use cappgpu
  implicit none
  integer, intent(in) :: ifi
  real(prec), dimension(nxyza) :: fi
  call cappgpu_push_params()
  call run_solver(cappgpu_pcgsip_h(fi, int(ifi, c_int)), 'pcgsip')
end subroutine

! sipsol.f90:3-106
subroutine sipsol(fi, ifi)
  use types
  use parameters
  use cappgpu
  implicit none
  integer, intent(in) :: ifi
  real(prec), dimension(nxyza) :: fi
  call cappgpu_push_params()
  call run_solver(cappgpu_sipsol_h(fi, int(ifi, c_int)), 'sipsol')
end subroutine

! iccg.f90:3-197
subroutine iccg(fi, ifi)
  use types
  use parameters
  use cappgpu
  implicit none
  integer, intent(in) :: ifi
  real(prec), dimension(nxyza) :: fi
  call cappgpu_push_params()
  call run_solver(cappgpu_iccg_h(fi, int(ifi, c_int)), 'iccg')
end subroutine

! cgstab.f90:3-283
subroutine cgstab(fi, ifi)
  use types
  use parameters
  use cappgpu
  implicit none
  integer, intent(in) :: ifi
  real(prec), dimension(nxyza) :: fi
  call cappgpu_push_params()
  call run_solver(cappgpu_cgstab_h(fi, int(ifi, c_int)), 'cgstab')
end subroutine

! cgstab_sip.f90:3-279
subroutine cgstab_sip(fi, ifi)
  use types
  use parameters
  use cappgpu
  implicit none
  integer, intent(in) :: ifi
  real(prec), dimension(nxyza) :: fi
  call cappgpu_push_params()
  call run_solver(cappgpu_cgstab_sip_h(fi, int(ifi, c_int)), 'cgstab_sip')
end subroutine

! pcg-jacobi.f90:3-155
subroutine Diagonally_Preconditioned_CG(fi, ifi)
  use types
  use parameters
  use cappgpu
  implicit none
  integer, intent(in) :: ifi
  real(prec), dimension(nxyza) :: fi
  call cappgpu_push_params()
  call run_solver(cappgpu_dpcg_h(fi, int(ifi, c_int)), 'dpcg')
end subroutine

! GRAD_GAUSS.f90:1-105 (the gfortran temporaries of gradu(1,:) sections
! arrive here as contiguous host arrays)
subroutine grad_gauss(u, dudx, dudy, dudz)
  use types
  use parameters
  use cappgpu
  implicit none
  real(prec), dimension(nxyza), intent(in) :: u
  real(prec), dimension(nxyza), intent(inout) :: dudx, dudy, dudz
  call chk(cappgpu_grad_gauss_h(u, dudx, dudy, dudz), 'grad_gauss')
end subroutine

! fluxuvw-overrelaxed-correction.f90:3-659
subroutine fluxuvw(idew, idns, idtb, arvx, arvy, arvz, fif, acfe, acfw, fcf)
  use types
  use parameters
  use cappgpu
  implicit none
  integer, intent(in) :: idew, idns, idtb
  real(prec), dimension(nxyza) :: arvx, arvy, arvz
  real(prec), dimension(nxyza) :: fif, acfe, acfw, fcf
  call cappgpu_push_params()
  call chk(cappgpu_fluxuvw_h(int(idew, c_int), int(idns, c_int), int(idtb, c_int), arvx, arvy, arvz, fif, &
           acfe, acfw, fcf), 'fluxuvw')
end subroutine

! PISO_assemble_pressure_eq.f90:3-257
subroutine piso_assemble_pressure_eq(idew, idns, idtb, arvx, arvy, arvz, fif, acfe, acfw, fcf, ipc, bp)
  use types
  use parameters
  use cappgpu
  implicit none
  integer, intent(in) :: idew, idns, idtb, ipc
  real(prec), dimension(nxyza) :: arvx, arvy, arvz, fif, acfe, acfw, fcf, bp
  call cappgpu_push_params()
  call chk(cappgpu_piso_assemble_pressure_eq_h(int(idew, c_int), int(idns, c_int), int(idtb, c_int), arvx, &
           arvy, arvz, fif, acfe, acfw, fcf, int(ipc, c_int), bp), 'piso_assemble_pressure_eq')
end subroutine

! assemble_pressure_eq.f90:3-124
subroutine assemble_pressure_eq(idew, idns, idtb, arvx, arvy, arvz, fif, acfe, acfw, fcf)
  use types
  use parameters
  use cappgpu
  implicit none
  integer, intent(in) :: idew, idns, idtb
  real(prec), dimension(nxyza) :: arvx, arvy, arvz, fif, acfe, acfw, fcf
  call cappgpu_push_params()
  call chk(cappgpu_assemble_pressure_eq_h(int(idew, c_int), int(idns, c_int), int(idtb, c_int), arvx, arvy, &
           arvz, fif, acfe, acfw, fcf), 'assemble_pressure_eq')
end subroutine

! update_values_at_ghostcells_nonperiodic.f90:3-642 and
! update_values_at_ghostcells.f90 (the periodic variant follows
! periodic_boundary, handed over by cappgpu_push_params)
subroutine update_values_at_ghostcells
  use cappgpu
  implicit none
  call cappgpu_push_params()
  call chk(cappgpu_update_values_at_ghostcells_h(), 'update_values_at_ghostcells')
end subroutine

! bpres.f90:3-81
subroutine bpres(p)
  use types
  use parameters
  use cappgpu
  implicit none
  real(prec), dimension(nxyza) :: p
  call chk(cappgpu_bpres_h(p), 'bpres')
end subroutine

! calcuvw.f90:3-464: the three momentum solves report as sipsol does
! (calcuvw.f90:388,424,460)
subroutine calcuvw
  use types
  use parameters
  use cappgpu
  implicit none
  type(cappgpu_solve_report) :: rep(3)
  integer :: q
  call cappgpu_push_params()
  call chk(cappgpu_calcuvw_h(rep), 'calcuvw')
  call cappgpu_pull_params()
  do q = 1, 3
    call solver_line(SOLVER_SIPSOL, int(q, c_int), rep(q))
  end do
end subroutine

! calcscm.f90:3-602 (k-omega SST): fi is te or ed, gradfi gradte or graded
subroutine calcscm(fi, gradfi, ifi)
  use types
  use parameters
  use cappgpu
  implicit none
  integer, intent(in) :: ifi
  real(prec), dimension(nxyza) :: fi
  real(prec), dimension(3,nxyza) :: gradfi
  call cappgpu_push_params()
  call run_solver(cappgpu_calcscm_h(fi, gradfi, int(ifi, c_int)), 'calcscm')
end subroutine

! modvis.f90:3-345 (the SST branch, :195-236)
subroutine modvis
  use cappgpu
  implicit none
  call cappgpu_push_params()
  call chk(cappgpu_modvis_h(), 'modvis')
end subroutine

! PISO_getHbyA.f90:3-233
subroutine PISO_getHbyA
  use cappgpu
  implicit none
  call cappgpu_push_params()
  call chk(cappgpu_piso_gethbya_h(), 'PISO_getHbyA')
end subroutine

! PISO_multiple_correction.f90:3-296: one pressure solve per corrector and
! non-orthogonal correction, each reporting in its solver's format
subroutine PISO_multiple_correction
  use types
  use parameters
  use cappgpu
  implicit none
  type(cappgpu_solve_report), allocatable :: rep(:)
  integer :: q
  allocate(rep(max(1, ncorr * npcor)))
  call cappgpu_push_params()
  call chk(cappgpu_piso_multiple_correction_h(rep), 'PISO_multiple_correction')
  call cappgpu_pull_params()
  do q = 1, ncorr * npcor
    call solver_line(cap_piso_solver, int(ip, c_int), rep(q))
  end do
  deallocate(rep)
end subroutine

! exchange_mpi.f90:4-89: a single rank exchanges with itself (identity)
subroutine exchange(phi)
  use types
  use parameters
  use cappgpu
  implicit none
  real(dp), dimension(nxyza) :: phi
  call chk(cappgpu_exchange_h(phi), 'exchange')
end subroutine

! global_sum_mpi.f90:4-36: the sum over one rank
subroutine global_sum(phi)
  use types
  use cappgpu
  implicit none
  real(dp) :: phi
  call chk(cappgpu_global_sum(phi), 'global_sum')
end subroutine

! global_max_mpi.f90:4-35: the maximum over one rank
subroutine global_max(phi)
  use types
  use cappgpu
  implicit none
  real(dp) :: phi
  call chk(cappgpu_global_max(phi), 'global_max')
end subroutine
