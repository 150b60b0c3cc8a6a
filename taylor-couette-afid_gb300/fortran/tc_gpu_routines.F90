!-----------------------------------------------------------------------
! tc_gpu_routines.F90 -- the routines of one time step on the device, one
! C entry point each, under the reference's own names, for use with the
! reference's TimeMarcher.F90 (TimeMarcher.F90:20-54 calls them in order).
!
! Link this file, tc_gpu_mod.F90 (without its TimeMarcher replacement) and
! libtcgb300.so in place of InnerCylVelocity.o, ExplicitTermsQ{T,R,Z}.o,
! ImplicitAndUpdateQ{T,R,Z}.o, SolveImpEqnUpdate_Q{T,R,Z}.o,
! CalcLocalDivergence.o, SolvePressureCorrection.o, CorrectVelocity.o and
! CorrectPressure.o.  SlipBCs.o stays the reference's (CreateGrid calls it
! at start-up for the host mask; the device forms its own mask in
! tc_begin_step).  The update_halo calls of TimeMarcher then act on the
! host mirror only and change nothing on the device, whose fields are
! periodic by index wrap.
!
! For bisection, keep any subset of the reference objects instead and move
! the arrays between host and device around them with tc_get_field /
! tc_set_field (TC_F_DQ, TC_F_HR, TC_F_QCAP, TC_F_RHS_*, TC_F_RU*, TC_F_DPH)
! and tc_get_state / tc_set_state.
!
! Each routine selects the RK substep from the al, ga, ro that
! TimeMarcher.F90:27-29 set (TcSyncSubstep) and stops the run through
! QuitRoutine on a non-zero status.  Not compiled in this repository (no
! Fortran compiler in the build image).
!-----------------------------------------------------------------------

!     InnerCylVelocity.F90:15-16 on the host (the values the host's own
!     routines read), and on the device the start of the step:
!     beta, InnerCylVelocity and SlipBCs (TimeMarcher.F90:20-23)
      subroutine InnerCylVelocity
      use param
      use tc_gpu
      implicit none
      vinner_t = sizepert*sin(2.*pi*omegapert*time)
      dvinner_t= 2.*pi*omegapert*sizepert*cos(2.*pi*omegapert*time)*dt
      call TcCheck(tc_begin_step(tch, dt, time))
      end subroutine InnerCylVelocity

      subroutine ExplicitTermsQT
      use tc_gpu
      call TcSyncSubstep
      call TcCheck(tc_explicit_terms_qt(tch))
      end subroutine ExplicitTermsQT

      subroutine ExplicitTermsQR
      use tc_gpu
      call TcSyncSubstep
      call TcCheck(tc_explicit_terms_qr(tch))
      end subroutine ExplicitTermsQR

      subroutine ExplicitTermsQZ
      use tc_gpu
      call TcSyncSubstep
      call TcCheck(tc_explicit_terms_qz(tch))
      end subroutine ExplicitTermsQZ

!     ImplicitAndUpdateQ* call their SolveImpEqnUpdate_Q* inside the one
!     entry point (ImplicitAndUpdateQT.F90:121, ImplicitAndUpdateQR.F90:68,
!     ImplicitAndUpdateQZ.F90:119)
      subroutine ImplicitAndUpdateQT
      use tc_gpu
      call TcSyncSubstep
      call TcCheck(tc_implicit_and_update_qt(tch))
      end subroutine ImplicitAndUpdateQT

      subroutine ImplicitAndUpdateQR
      use tc_gpu
      call TcSyncSubstep
      call TcCheck(tc_implicit_and_update_qr(tch))
      end subroutine ImplicitAndUpdateQR

      subroutine ImplicitAndUpdateQZ
      use tc_gpu
      call TcSyncSubstep
      call TcCheck(tc_implicit_and_update_qz(tch))
      end subroutine ImplicitAndUpdateQZ

      subroutine CalcLocalDivergence
      use tc_gpu
      call TcSyncSubstep
      call TcCheck(tc_calc_local_divergence(tch))
      end subroutine CalcLocalDivergence

      subroutine SolvePressureCorrection
      use tc_gpu
      call TcCheck(tc_solve_pressure_correction(tch))
      end subroutine SolvePressureCorrection

      subroutine CorrectVelocity
      use tc_gpu
      call TcSyncSubstep
      call TcCheck(tc_correct_velocity(tch))
      end subroutine CorrectVelocity

      subroutine CorrectPressure
      use tc_gpu
      call TcSyncSubstep
      call TcCheck(tc_correct_pressure(tch))
      end subroutine CorrectPressure
