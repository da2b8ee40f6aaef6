!***********************************************************************
!
! cappgpu_iface.f90 -- iso_c_binding interface to libcappgpu.so and the
! drop-in replacements of the reference's hot-path subroutines.
!
! A reference build swaps its own sipsol.f90, pcg-sip.f90, iccg.f90,
! cgstab.f90, cgstab_sip.f90, GRAD_GAUSS.f90, calcuvw.f90,
! PISO_multiple_correction.f90 and update_values_at_ghostcells*.f90 for
! this file (see INTEGRATION.md).  Each replacement keeps the reference's
! name and dummy arguments.  Module arrays are registered once with
! cappgpu_attach (after allocate_arrays/init); every drop-in then copies
! the registered arrays it reads to the device, runs the routine there and
! copies back what it writes, so host code in between keeps working on
! the host arrays unchanged.
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
       CAP_GRADU_X=69, CAP_GRADP_X=78, CAP_NFIELDS=81

  ! C mirror of cappgpu_solve_report
  type, bind(c) :: cappgpu_solve_report
    real(c_double) :: res0, resl
    integer(c_int) :: iters, status
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
    integer(c_int) function cappgpu_register(field, host) bind(c, name="cappgpu_register")
      import :: c_int, c_ptr
      integer(c_int), value :: field
      type(c_ptr), value :: host
    end function
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
    integer(c_int) function cappgpu_grad_gauss_h(u, dudx, dudy, dudz) bind(c, name="cappgpu_grad_gauss_h")
      import :: c_int, c_double
      real(c_double), intent(in) :: u(*)
      real(c_double), intent(inout) :: dudx(*), dudy(*), dudz(*)
    end function
    integer(c_int) function cappgpu_update_values_at_ghostcells() &
        bind(c, name="cappgpu_update_values_at_ghostcells")
      import :: c_int
    end function
    integer(c_int) function cappgpu_calcuvw(rep) bind(c, name="cappgpu_calcuvw")
      import :: c_int, cappgpu_solve_report
      type(cappgpu_solve_report), intent(out) :: rep(3)
    end function
    integer(c_int) function cappgpu_piso_multiple_correction(rep) &
        bind(c, name="cappgpu_piso_multiple_correction")
      import :: c_int, cappgpu_solve_report
      type(cappgpu_solve_report), intent(out) :: rep(*)
    end function
  end interface

contains

  ! Register the module arrays of modules_allocatable.f90 with the library
  ! (call once after init).  Geometry and BC codes are uploaded here; the
  ! fields are uploaded by the drop-ins as they need them.
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
    use bc
    integer(c_int) :: rc
    integer(c_int64_t) :: n
    n = int(nijk, c_int64_t)
    rc = cappgpu_init(ni, nj, nk)
    call chk(rc, 'cappgpu_init')
    call put(CAP_X, x); call put(CAP_Y, y); call put(CAP_Z, z)
    call put(CAP_XC, xc); call put(CAP_YC, yc); call put(CAP_ZC, zc); call put(CAP_VOL, vol)
    call put(CAP_FX, fx); call put(CAP_FY, fy); call put(CAP_FZ, fz)
    call put(CAP_AR1X, ar1x); call put(CAP_AR1Y, ar1y); call put(CAP_AR1Z, ar1z)
    call put(CAP_AR2X, ar2x); call put(CAP_AR2Y, ar2y); call put(CAP_AR2Z, ar2z)
    call put(CAP_AR3X, ar3x); call put(CAP_AR3Y, ar3y); call put(CAP_AR3Z, ar3z)
    rc = cappgpu_set_bc(0, lbw, int(njk, c_int64_t)); call chk(rc, 'lbw')
    rc = cappgpu_set_bc(1, lbe, int(njk, c_int64_t)); call chk(rc, 'lbe')
    rc = cappgpu_set_bc(2, lbs, int(nik, c_int64_t)); call chk(rc, 'lbs')
    rc = cappgpu_set_bc(3, lbn, int(nik, c_int64_t)); call chk(rc, 'lbn')
    rc = cappgpu_set_bc(4, lbb, int(nij, c_int64_t)); call chk(rc, 'lbb')
    rc = cappgpu_set_bc(5, lbt, int(nij, c_int64_t)); call chk(rc, 'lbt')
    ! matrix, SIP factors and solver vectors: registered for the _h drop-ins
    call reg(CAP_AE, ae); call reg(CAP_AW, aw); call reg(CAP_AN, an); call reg(CAP_AS, as)
    call reg(CAP_AT, at); call reg(CAP_AB, ab); call reg(CAP_AP, ap); call reg(CAP_SU, su)
    call reg(CAP_RES, res)
    call reg(CAP_BB, bb); call reg(CAP_BS, bs); call reg(CAP_BW, bw); call reg(CAP_BP, bp)
    call reg(CAP_BN, bn); call reg(CAP_BE, be); call reg(CAP_BT, bt)
    call reg(CAP_U, u); call reg(CAP_V, v); call reg(CAP_W, w); call reg(CAP_P, p); call reg(CAP_PP, pp)
  contains
    subroutine put(f, a)
      integer(c_int), intent(in) :: f
      real(c_double), intent(in) :: a(:)
      integer(c_int) :: r
      r = cappgpu_set_field(f, a, n)
      call chk(r, 'set_field')
    end subroutine
    subroutine reg(f, a)
      integer(c_int), intent(in) :: f
      real(c_double), target, intent(inout) :: a(:)
      integer(c_int) :: r
      r = cappgpu_register(f, c_loc(a(1)))
      call chk(r, 'register')
    end subroutine
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
  real(prec), dimension(*) :: fi
  integer(c_int) :: rc
  rc = cappgpu_pcgsip_h(fi, int(ifi, c_int))
  call chk(rc, 'pcgsip')
end subroutine

! sipsol.f90:3-106
subroutine sipsol(fi, ifi)
  use types
  use parameters
  use cappgpu
  implicit none
  integer, intent(in) :: ifi
  real(prec), dimension(*) :: fi
  integer(c_int) :: rc
  rc = cappgpu_sipsol_h(fi, int(ifi, c_int))
  call chk(rc, 'sipsol')
end subroutine

! iccg.f90:3-197
subroutine iccg(fi, ifi)
  use types
  use parameters
  use cappgpu
  implicit none
  integer, intent(in) :: ifi
  real(prec), dimension(*) :: fi
  integer(c_int) :: rc
  rc = cappgpu_iccg_h(fi, int(ifi, c_int))
  call chk(rc, 'iccg')
end subroutine

! cgstab.f90:3-283
subroutine cgstab(fi, ifi)
  use types
  use parameters
  use cappgpu
  implicit none
  integer, intent(in) :: ifi
  real(prec), dimension(*) :: fi
  integer(c_int) :: rc
  rc = cappgpu_cgstab_h(fi, int(ifi, c_int))
  call chk(rc, 'cgstab')
end subroutine

! cgstab_sip.f90:3-279
subroutine cgstab_sip(fi, ifi)
  use types
  use parameters
  use cappgpu
  implicit none
  integer, intent(in) :: ifi
  real(prec), dimension(*) :: fi
  integer(c_int) :: rc
  rc = cappgpu_cgstab_sip_h(fi, int(ifi, c_int))
  call chk(rc, 'cgstab_sip')
end subroutine

! GRAD_GAUSS.f90:1-105 (the gfortran temporaries of gradu(1,:) sections
! arrive here as contiguous host arrays)
subroutine grad_gauss(u, dudx, dudy, dudz)
  use types
  use cappgpu
  implicit none
  real(prec), dimension(*), intent(in) :: u
  real(prec), dimension(*), intent(inout) :: dudx, dudy, dudz
  integer(c_int) :: rc
  rc = cappgpu_grad_gauss_h(u, dudx, dudy, dudz)
  call chk(rc, 'grad_gauss')
end subroutine
