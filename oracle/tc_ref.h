/*
 * tc_ref.h -- C interface of the CPU oracle for the Taylor-Couette time step.
 *
 * TEST INFRASTRUCTURE ONLY.  This is a serial-semantics restatement of the
 * reference Fortran routines (rodosti/Taylor-Couette-AFiD) in the reference's
 * own array layout: q(k=r, j=z, i=theta), r fastest, one periodic halo cell in
 * z and theta.  Only tests/, __graft_entry__.smoke() and bench.py's CPU
 * baseline leg use it, always as the checker or the timed CPU baseline, never
 * as part of the product path.
 *
 * Parity status: pinned to runs of the reference's own source.  The
 * reference ships no tests or golden vectors, and its Fortran/MPI/FFTW/HDF5
 * build cannot be compiled here (no Fortran compiler, MPI, FFTW or LAPACK
 * libraries).  Its main program and time-step routines were instead executed
 * on one rank by a translator of the Fortran subset they use
 * (tests/golden/fortran_subset.py; LAPACK through SciPy, FFTW through
 * numpy.fft), and the runs are committed as fixtures
 * (tests/golden/reference_runs.npz) that tests/test_reference_runs.py checks
 * this restatement against.  It is also cross-checked against an independent
 * NumPy/SciPy restatement (oracle/tc_np.py) and physics known-answer tests
 * (laminar Couette torque, divergence-free projection, FFT round trips).
 */
#ifndef TC_REF_H
#define TC_REF_H

#ifdef __cplusplus
extern "C" {
#endif

/* bou.in values in file order (ReadInputFile.F90:17-39).  Same memory
 * layout as tc_bou in include/tc_capi.h. */
typedef struct tcref_bou {
    int nthm, nzm, nrm, nsst, idtv, nread;
    int ntst; double tout, tmax; int ireset; double walltimemax;
    double alx3, rint, rext; int istr; double str, lamb;
    double virotint, virotext, sizepert, omegapert;
    double ren, romeg, resid, limitCFL;
    double tsta; int starea;
    double dtmin, dtmax, limitVel, cfllim;
    int nslabr, dpthcut, dpstave; double tframe2d;
    int dpfullf; double tframe3d;
    int minstrt, minstrz, multmin;
} tcref_bou;

/* Treatment of the singular k_theta = k_z = 0 pressure mode
 * (SolvePressureCorrection.F90:127-148 with the zero-flux rows of
 * InitPressureSolver.F90:22-32). */
enum {
    TCREF_MODE00_LAPACK = 0,  /* LAPACK ?gttrs arithmetic: divides by the roundoff pivot */
    TCREF_MODE00_PIN = 1      /* drop the last (dependent) row: phi(nrm) = 0 for that mode */
};

/* 3-D arrays that can be read or written (reference layout). */
enum {
    TCREF_QT = 0, TCREF_QR, TCREF_QZ, TCREF_PR, TCREF_DPH,   /* (nr, nzm+2, nthm+2) */
    TCREF_RHS, TCREF_RU1, TCREF_RU2, TCREF_RU3, TCREF_DQ, TCREF_QCAP  /* (nr, nzm, nthm) */
};

/* 1-D grid arrays (length nr, 1-based in the reference, 0-based here). */
enum {
    TCREF_G_RC = 0, TCREF_G_RM, TCREF_G_G2RC, TCREF_G_G2RM, TCREF_G_USRC, TCREF_G_USRM,
    TCREF_G_UDX1VIS1, TCREF_G_UDX1VIS2, TCREF_G_UDX1QM, TCREF_G_UDX2C, TCREF_G_UDX2M,
    TCREF_G_RUDX2C, TCREF_G_UDX2RM,
    TCREF_G_AP1J, TCREF_G_AM1J, TCREF_G_AC1J, TCREF_G_AP2J, TCREF_G_AM2J, TCREF_G_AC2J,
    TCREF_G_AP2JE, TCREF_G_AM2JE, TCREF_G_AC2JE, TCREF_G_AP3J, TCREF_G_AM3J, TCREF_G_AC3J,
    TCREF_G_APPH, TCREF_G_AMPH, TCREF_G_ACPH,
    TCREF_G_PVOL, TCREF_G_UDX2MM, TCREF_G_UDX2CC,
    TCREF_G_AK1, /* length nthm */
    TCREF_G_AK3, /* length nzm  */
    TCREF_G_COUNT
};

void*  tcref_create(const tcref_bou* b, int mode00);
void   tcref_destroy(void* h);
void   tcref_set_threads(int n);
int    tcref_get_threads(void);

void   tcref_set_array(void* h, int which, const double* src);
void   tcref_get_array(void* h, int which, double* dst);
int    tcref_get_grid(void* h, int which, double* dst);   /* returns length */
void   tcref_get_scalars(void* h, double* out8);           /* dxt dxz dxr beta al ga ro vinner_t */
void   tcref_get_dvinner(void* h, double* out1);
void   tcref_get_slip(void* h, int* icylsl, int* ocylsl);  /* (nzm, nthm) column-major */

/* TimeMarcher.F90:20-23: beta, InnerCylVelocity, SlipBCs for a step of
 * length dt starting at time. */
void   tcref_begin_step(void* h, double dt, double time);
/* TimeMarcher.F90:27-29: al, ga, ro for substep ns (1-based). */
void   tcref_set_substep(void* h, int ns);

void   tcref_explicit_terms_qt(void* h);
void   tcref_explicit_terms_qr(void* h);
void   tcref_explicit_terms_qz(void* h);
/* ImplicitAndUpdateQ* without the solve (rhs and ru update only). */
void   tcref_implicit_rhs_qt(void* h);
void   tcref_implicit_rhs_qr(void* h);
void   tcref_implicit_rhs_qz(void* h);
void   tcref_solve_imp_eqn_update_qt(void* h);
void   tcref_solve_imp_eqn_update_qr(void* h);   /* includes the qr wall reset */
void   tcref_solve_imp_eqn_update_qz(void* h);
void   tcref_update_halo(void* h, int which);
void   tcref_calc_local_divergence(void* h);
void   tcref_solve_pressure_correction(void* h);
void   tcref_correct_velocity(void* h);
void   tcref_correct_pressure(void* h);

/* One full TimeMarcher call (NSST substeps). */
void   tcref_time_marcher(void* h, double dt, double time);

double tcref_calc_max_cfl(void* h);
double tcref_check_divergence(void* h);
void   tcref_calc_torque(void* h, double* inner, double* outer);
/* CalcVelocityStats.F90:21-65: vmax(3) and rms(3). */
void   tcref_calc_velocity_stats(void* h, double* vmax3, double* rms3);

/* statistics (StatRoutines.F90, CalcVorticity.F90, CalcDissipation.F90) */
enum tcref_stat {
    TCREF_ST_VT_MEAN = 0, TCREF_ST_VR_MEAN, TCREF_ST_VZ_MEAN, TCREF_ST_WT_MEAN, TCREF_ST_WR_MEAN,
    TCREF_ST_WZ_MEAN, TCREF_ST_VT_RMS, TCREF_ST_VR_RMS, TCREF_ST_VZ_RMS, TCREF_ST_WT_RMS,
    TCREF_ST_WR_RMS, TCREF_ST_WZ_RMS, TCREF_ST_VTVR_MEAN, TCREF_ST_VTVZ_MEAN, TCREF_ST_VRVZ_MEAN,
    TCREF_ST_PR_MEAN, TCREF_ST_PR_RMS, TCREF_ST_DISSTE, TCREF_ST_COUNT
};
void   tcref_calc_stats(void* h);
double tcref_calc_dissipation(void* h);
void   tcref_get_stat(void* h, int which, double* out);     /* (nrm, nzm), k fastest */
int    tcref_stat_samples(void* h);
void   tcref_get_vorticity(void* h, int comp, double* out); /* (nrm, nzm, nthm), k fastest */

/* main.F90:152-226 time loop restricted to the step semantics: dt control,
 * TimeMarcher, time advance and the error codes it can raise (165, 166, 169,
 * 266, 333, 555).  Runs at most nsteps steps starting from time *time with
 * step counter starting at ntime0.  On return *time and *dt hold the final
 * values; returns the error code (0 when nsteps steps ran without one). */
int    tcref_run(void* h, int ntime0, int nsteps, double* time, double* dt);

#ifdef __cplusplus
}
#endif
#endif
