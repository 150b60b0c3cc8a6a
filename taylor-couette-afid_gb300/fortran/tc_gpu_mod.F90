!-----------------------------------------------------------------------
! tc_gpu_mod.F90 -- ISO_C_BINDING interface to libtcgb300.so and drop-in
! replacements for the reference routines of the time step.
!
! A Fortran host built from the reference sources links this module and
! libtcgb300.so in place of TimeMarcher.F90, CalcMaxCFL.F90,
! CheckDivergence.F90 and CalcTorque.F90 (Makefile:37-47 object list).  The
! module arrays qt, qr, qz, pr of `local_arrays` stay the host mirror of the
! device state: they are copied to the device once after the initial
! condition / ReadFlowField, and back before any routine that reads them on
! the host (statistics, dumps, WriteFlowField).
!
! Not compiled in this repository (no Fortran compiler in the build image);
! the C ABI it binds is exercised by the Python tests through ctypes.
!-----------------------------------------------------------------------
      module tc_gpu
      use iso_c_binding
      implicit none

      type, bind(C) :: tc_bou
        integer(c_int)  :: nthm, nzm, nrm, nsst, idtv, nread
        integer(c_int)  :: ntst
        real(c_double)  :: tout, tmax
        integer(c_int)  :: ireset
        real(c_double)  :: walltimemax
        real(c_double)  :: alx3, rint, rext
        integer(c_int)  :: istr
        real(c_double)  :: str, lamb
        real(c_double)  :: virotint, virotext, sizepert, omegapert
        real(c_double)  :: ren, romeg, resid, limitCFL
        real(c_double)  :: tsta
        integer(c_int)  :: starea
        real(c_double)  :: dtmin, dtmax, limitVel, cfllim
        integer(c_int)  :: nslabr, dpthcut, dpstave
        real(c_double)  :: tframe2d
        integer(c_int)  :: dpfullf
        real(c_double)  :: tframe3d
        integer(c_int)  :: minstrt, minstrz, multmin
      end type tc_bou

      type(c_ptr), save :: tch = c_null_ptr

      interface
        integer(c_int) function tc_create(cfg, h) bind(C, name='tc_create')
          import
          type(tc_bou), intent(in) :: cfg
          type(c_ptr), intent(out) :: h
        end function
        subroutine tc_destroy(h) bind(C, name='tc_destroy')
          import
          type(c_ptr), value :: h
        end subroutine
        integer(c_int) function tc_set_state(h, qt, qr, qz, pr) bind(C, name='tc_set_state')
          import
          type(c_ptr), value :: h
          real(c_double), intent(in) :: qt(*), qr(*), qz(*), pr(*)
        end function
        integer(c_int) function tc_get_state(h, qt, qr, qz, pr) bind(C, name='tc_get_state')
          import
          type(c_ptr), value :: h
          real(c_double), intent(out) :: qt(*), qr(*), qz(*), pr(*)
        end function
        integer(c_int) function tc_time_marcher(h, dt, time) bind(C, name='tc_time_marcher')
          import
          type(c_ptr), value :: h
          real(c_double), value :: dt, time
        end function
        integer(c_int) function tc_calc_max_cfl(h, cflm) bind(C, name='tc_calc_max_cfl')
          import
          type(c_ptr), value :: h
          real(c_double), intent(out) :: cflm
        end function
        integer(c_int) function tc_check_divergence(h, qmax) bind(C, name='tc_check_divergence')
          import
          type(c_ptr), value :: h
          real(c_double), intent(out) :: qmax
        end function
        integer(c_int) function tc_calc_torque(h, tin, tout) bind(C, name='tc_calc_torque')
          import
          type(c_ptr), value :: h
          real(c_double), intent(out) :: tin, tout
        end function
      end interface

      contains

!     Build the handle from the `param` module values (after ReadInputFile)
      subroutine TcGpuInit
      use param
      use local_arrays, only: qt, qr, qz, pr
      type(tc_bou) :: b
      integer(c_int) :: rc
      b%nthm = nthm; b%nzm = nzm; b%nrm = nrm; b%nsst = nsst
      b%idtv = idtv; b%nread = nread; b%ntst = ntst; b%tout = tout
      b%tmax = tmax; b%ireset = ireset; b%walltimemax = walltimemax
      b%alx3 = alx3; b%rint = rint; b%rext = rext; b%istr = istr
      b%str = str; b%lamb = lamb; b%virotint = virotint
      b%virotext = virotext; b%sizepert = sizepert
      b%omegapert = omegapert; b%ren = ren; b%romeg = romeg
      b%resid = resid; b%limitCFL = limitCFL; b%tsta = tsta
      b%starea = starea; b%dtmin = dtmin; b%dtmax = dtmax
      b%limitVel = limitVel; b%cfllim = cfllim; b%nslabr = nslabr
      b%dpthcut = dpthcut; b%dpstave = dpstave; b%tframe2d = tframe2d
      b%dpfullf = dpfullf; b%tframe3d = tframe3d
      b%minstrt = minstrt; b%minstrz = minstrz; b%multmin = multmin
      rc = tc_create(b, tch)
      if (rc .ne. 0) call QuitRoutine((/0.d0,0.d0,0.d0/), .false., rc)
      rc = tc_set_state(tch, qt, qr, qz, pr)
      if (rc .ne. 0) call QuitRoutine((/0.d0,0.d0,0.d0/), .false., rc)
      end subroutine TcGpuInit

!     Copy the device state into the host mirror (before host-side I/O)
      subroutine TcGpuSync
      use local_arrays, only: qt, qr, qz, pr
      integer(c_int) :: rc
      rc = tc_get_state(tch, qt, qr, qz, pr)
      if (rc .ne. 0) call QuitRoutine((/0.d0,0.d0,0.d0/), .false., rc)
      end subroutine TcGpuSync

      end module tc_gpu

!     Drop-in replacements (same names and interfaces as the reference)
      subroutine TimeMarcher
      use param, only: dt, time
      use tc_gpu
      integer(c_int) :: rc
      rc = tc_time_marcher(tch, dt, time)
      if (rc .ne. 0) call QuitRoutine((/0.d0,0.d0,0.d0/), .false., rc)
      end subroutine TimeMarcher

      subroutine CalcMaxCFL(cflm)
      use tc_gpu
      real, intent(inout) :: cflm
      integer(c_int) :: rc
      rc = tc_calc_max_cfl(tch, cflm)
      end subroutine CalcMaxCFL

      subroutine CheckDivergence(qmax)
      use tc_gpu
      real, intent(out) :: qmax
      integer(c_int) :: rc
      rc = tc_check_divergence(tch, qmax)
      end subroutine CheckDivergence

      subroutine CalcTorque
      use param, only: time, ismaster
      use tc_gpu
      real(c_double) :: anusslow, anussup
      integer(c_int) :: rc
      rc = tc_calc_torque(tch, anusslow, anussup)
      if(ismaster) write(97,546) time, anusslow, anussup
 546  format(3(1x,e14.6))
      end subroutine CalcTorque
