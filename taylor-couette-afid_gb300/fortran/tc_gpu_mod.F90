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
! For routine-by-routine work (parity bisection, or replacing the routines
! one at a time under the reference's own TimeMarcher.F90) link
! tc_gpu_routines.F90 instead of the TimeMarcher replacement at the end of
! this file: it supplies InnerCylVelocity, SlipBCs, ExplicitTermsQT/QR/QZ,
! ImplicitAndUpdateQT/QR/QZ, CalcLocalDivergence, SolvePressureCorrection,
! CorrectVelocity and CorrectPressure on the device.
!
! Every entry point returns a status; a non-zero status stops the run
! through QuitRoutine with that code (main.F90:229-259 does the same with
! the reference's own error codes).
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

!     enum tc_field of tc_capi.h (arrays readable with tc_get_field)
      integer(c_int), parameter :: TC_F_QT = 0, TC_F_QR = 1, TC_F_QZ = 2, &
        TC_F_PR = 3, TC_F_DPH = 4, TC_F_RHS_T = 5, TC_F_RHS_R = 6,       &
        TC_F_RHS_Z = 7, TC_F_RU1 = 8, TC_F_RU2 = 9, TC_F_RU3 = 10,       &
        TC_F_DQ = 11, TC_F_HR = 12, TC_F_QCAP = 13

      type(c_ptr), save :: tch = c_null_ptr
!     timer array handed to QuitRoutine (which writes tin(3))
      real, save :: tctin(3) = 0.0

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
        integer(c_int) function tc_get_field(h, which, out) bind(C, name='tc_get_field')
          import
          type(c_ptr), value :: h
          integer(c_int), value :: which
          real(c_double), intent(out) :: out(*)
        end function
        integer(c_int) function tc_set_field(h, which, in) bind(C, name='tc_set_field')
          import
          type(c_ptr), value :: h
          integer(c_int), value :: which
          real(c_double), intent(in) :: in(*)
        end function
        integer(c_int) function tc_time_marcher(h, dt, time) bind(C, name='tc_time_marcher')
          import
          type(c_ptr), value :: h
          real(c_double), value :: dt, time
        end function
        integer(c_int) function tc_begin_step(h, dt, time) bind(C, name='tc_begin_step')
          import
          type(c_ptr), value :: h
          real(c_double), value :: dt, time
        end function
        integer(c_int) function tc_set_substep(h, ns) bind(C, name='tc_set_substep')
          import
          type(c_ptr), value :: h
          integer(c_int), value :: ns
        end function
!       one routine each (h only)
        integer(c_int) function tc_explicit_terms_qt(h) bind(C, name='tc_explicit_terms_qt')
          import
          type(c_ptr), value :: h
        end function
        integer(c_int) function tc_explicit_terms_qr(h) bind(C, name='tc_explicit_terms_qr')
          import
          type(c_ptr), value :: h
        end function
        integer(c_int) function tc_explicit_terms_qz(h) bind(C, name='tc_explicit_terms_qz')
          import
          type(c_ptr), value :: h
        end function
        integer(c_int) function tc_implicit_and_update_qt(h) bind(C, name='tc_implicit_and_update_qt')
          import
          type(c_ptr), value :: h
        end function
        integer(c_int) function tc_implicit_and_update_qr(h) bind(C, name='tc_implicit_and_update_qr')
          import
          type(c_ptr), value :: h
        end function
        integer(c_int) function tc_implicit_and_update_qz(h) bind(C, name='tc_implicit_and_update_qz')
          import
          type(c_ptr), value :: h
        end function
        integer(c_int) function tc_calc_local_divergence(h) bind(C, name='tc_calc_local_divergence')
          import
          type(c_ptr), value :: h
        end function
        integer(c_int) function tc_solve_pressure_correction(h) bind(C, name='tc_solve_pressure_correction')
          import
          type(c_ptr), value :: h
        end function
        integer(c_int) function tc_correct_velocity(h) bind(C, name='tc_correct_velocity')
          import
          type(c_ptr), value :: h
        end function
        integer(c_int) function tc_correct_pressure(h) bind(C, name='tc_correct_pressure')
          import
          type(c_ptr), value :: h
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

!     Stop the run through the reference's QuitRoutine on a non-zero status
      subroutine TcCheck(rc)
      integer(c_int), intent(in) :: rc
      integer :: code
      if (rc .ne. 0) then
        code = rc
        call QuitRoutine(tctin, .false., code)
      end if
      end subroutine TcCheck

!     Build the handle from the `param` module values (after ReadInputFile)
      subroutine TcGpuInit
      use param
      use local_arrays, only: qt, qr, qz, pr
      type(tc_bou) :: b
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
      call TcCheck(tc_create(b, tch))
      call TcCheck(tc_set_state(tch, qt, qr, qz, pr))
      end subroutine TcGpuInit

!     Copy the device state into the host mirror (before host-side I/O)
      subroutine TcGpuSync
      use local_arrays, only: qt, qr, qz, pr
      call TcCheck(tc_get_state(tch, qt, qr, qz, pr))
      end subroutine TcGpuSync

!     Select the RK substep whose coefficients the host set in al, ga, ro
!     (TimeMarcher.F90:27-29) before a per-routine call
      subroutine TcSyncSubstep
      use param, only: al, ga, ro, alm, gam, rom, nsst
      integer :: ns
      do ns = 1, nsst
        if (al .eq. alm(ns) .and. ga .eq. gam(ns) .and. ro .eq. rom(ns)) then
          call TcCheck(tc_set_substep(tch, int(ns, c_int)))
          return
        end if
      end do
      call TcCheck(2006_c_int)
      end subroutine TcSyncSubstep

      end module tc_gpu

!     Drop-in replacements (same names and interfaces as the reference)
      subroutine TimeMarcher
      use param, only: dt, time
      use tc_gpu
      call TcCheck(tc_time_marcher(tch, dt, time))
      end subroutine TimeMarcher

      subroutine CalcMaxCFL(cflm)
      use tc_gpu
      real, intent(inout) :: cflm
      real(c_double) :: v
      call TcCheck(tc_calc_max_cfl(tch, v))
      cflm = v
      end subroutine CalcMaxCFL

      subroutine CheckDivergence(qmax)
      use tc_gpu
      real, intent(out) :: qmax
      real(c_double) :: v
!     a NaN in the fields returns 169, which stops the run here
      call TcCheck(tc_check_divergence(tch, v))
      qmax = v
      end subroutine CheckDivergence

      subroutine CalcTorque
      use param, only: time, ismaster
      use tc_gpu
      real(c_double) :: anusslow, anussup
      call TcCheck(tc_calc_torque(tch, anusslow, anussup))
      if(ismaster) write(97,546) time, anusslow, anussup
 546  format(3(1x,e14.6))
      end subroutine CalcTorque
