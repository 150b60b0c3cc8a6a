/*
 * tc_capi.h -- C ABI of the GB300 Taylor-Couette time step (libtcgb300.so).
 *
 * Drop-in for the time-step path of rodosti/Taylor-Couette-AFiD.  The
 * reference has no plugin API: its routines take no arguments and talk
 * through the Fortran modules `param` and `local_arrays` (param.F90:4-102).
 * Each entry point below replaces the reference routine(s) named in its
 * comment; a Fortran host binds them with ISO_C_BINDING through the module
 * taylor-couette-afid_gb300/fortran/tc_gpu_mod.F90.
 *
 * Conventions
 *  - Every function returns an int status: 0 = OK.  165, 166, 169, 266, 333
 *    and 555 are the reference's error codes (main.F90:148-259); 1000-1999 are
 *    CUDA or allocation failures; 2000-2999 are invalid arguments or
 *    configurations; 3000-3999 are failures the kernels report (3001: a
 *    bounded wait gave up).  tc_last_error() returns a message for the last
 *    failure.
 *  - Host arrays of 3-D fields use the reference layout: Fortran
 *    q(1:nr, 0:nzm+1, 0:nthm+1), r fastest, one periodic halo cell in z and
 *    theta (InitVariables.F90:26-35).  pr/qt/qz entries at k = nr are not
 *    part of the step (never read by any routine of the path).
 *  - All work is ordered on the handle's CUDA stream.  Calls that return
 *    host scalars synchronise that stream.  A handle is used by one host
 *    thread at a time; distinct handles are independent.
 *  - Handles made by tc_create compute in IEEE FP64; tc_create_ex can make a
 *    mixed FP32/FP64 handle (see enum tc_precision_mode).
 */
#ifndef TC_CAPI_H
#define TC_CAPI_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

/* bou.in values, in file order (ReadInputFile.F90:17-39, param.F90:9-27). */
typedef struct tc_bou {
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
} tc_bou;

typedef struct tc_handle tc_handle;
typedef struct tc_ensemble tc_ensemble;

/* Precision of a handle.  TC_PREC_FP64: the plain path, every operation in
 * IEEE FP64 (the drop-in).  TC_PREC_MIXED: velocity fields, explicit terms,
 * implicit momentum sweeps and FFTs in FP32 with FP32 accumulation; the
 * radial pressure tridiagonals (on the FP32 spectrum, widened), the pressure
 * accumulation of CorrectPressure and the CFL/divergence/torque reductions
 * in FP64.  TC_PREC_MIXED_FF: TC_PREC_MIXED with the pressure tridiagonals
 * in float-float arithmetic (about 48 significant bits, on the FP32 pipes)
 * instead of FP64.  Host arrays are FP64 in all three. */
enum tc_precision_mode { TC_PREC_FP64 = 0, TC_PREC_MIXED = 1, TC_PREC_MIXED_FF = 2 };

/* 1-D grid/coefficient arrays, 0-based (entry m = reference index m+1). */
enum tc_grid_array {
    TC_G_RC = 0, TC_G_RM, TC_G_G2RC, TC_G_G2RM, TC_G_USRC, TC_G_USRM,
    TC_G_UDX1VIS1, TC_G_UDX1VIS2, TC_G_UDX1QM, TC_G_UDX2C, TC_G_UDX2M,
    TC_G_RUDX2C, TC_G_UDX2RM,
    TC_G_AP1J, TC_G_AM1J, TC_G_AC1J, TC_G_AP2J, TC_G_AM2J, TC_G_AC2J,
    TC_G_AP2JE, TC_G_AM2JE, TC_G_AC2JE, TC_G_AP3J, TC_G_AM3J, TC_G_AC3J,
    TC_G_APPH, TC_G_AMPH, TC_G_ACPH,
    TC_G_PVOL, TC_G_UDX2MM, TC_G_UDX2CC,   /* statistics metrics (CreateGrid.F90:141-173) */
    TC_G_AK1,  /* length nthm */
    TC_G_AK3,  /* length nzm  */
    TC_G_COUNT
};

/* 3-D arrays readable through tc_get_field (reference layout). */
enum tc_field {
    TC_F_QT = 0, TC_F_QR, TC_F_QZ, TC_F_PR, TC_F_DPH,       /* (nr, nzm+2, nthm+2) */
    TC_F_RHS_T, TC_F_RHS_R, TC_F_RHS_Z,                    /* (nr, nzm, nthm): rhs of each component */
    TC_F_RU1, TC_F_RU2, TC_F_RU3,                          /* (nr, nzm, nthm) */
    TC_F_DQ, TC_F_HR, TC_F_QCAP,                           /* explicit terms of qt, qr, qz */
    TC_F_COUNT
};

/* ---- host-only entry points (no GPU needed) ---------------------------- */

/* ReadInputFile.F90:10-74: parse bou.in (list-directed, one header record
 * before each value record).  Returns 0, or 2001 (cannot open) / 2002
 * (malformed).  err (may be NULL) receives a message. */
int tc_read_bou(const char* path, tc_bou* out, char* err, int errlen);

/* CreateGrid.F90:24-324 and InitPressureSolver.F90:22-66 on the host:
 * writes grid array `which` (enum tc_grid_array) into out[0..len-1] and
 * returns its length, or a negative status on bad input. */
int tc_grid_array(const tc_bou* cfg, int which, double* out, int len);

/* Library version string. */
const char* tc_version(void);

/* ---- handle lifecycle --------------------------------------------------- */

/* InitTimeMarchScheme + InitVariables + CreateGrid + InitPressureSolver
 * (main.F90:70-94): validate cfg, build the grid and coefficients, allocate
 * all device state on the current CUDA device, zero it.  Fields start at zero
 * and time at 0; load a start with tc_set_state.  The transform lengths
 * NTM/2 (theta, real transform of NTM points) and NZM may have no prime
 * factor above 13 (status 2003 otherwise; the reference's FFTW plans take
 * any length). */
int tc_create(const tc_bou* cfg, tc_handle** out);
/* tc_create with a precision (enum tc_precision_mode); tc_create is
 * tc_create_ex(cfg, TC_PREC_FP64, out).  No counterpart in the reference,
 * which is FP64 only. */
int tc_create_ex(const tc_bou* cfg, int precision, tc_handle** out);
int tc_precision(const tc_handle* h);
/* Mixed handles: stage the momentum march's input planes in shared memory
 * with TMA loads (1; the grid needs nthm a multiple of 4 and at least 64) or
 * load them through the read-only cache (0, the default: on GB300 it runs
 * the march about 5 % faster).  Both compute the same bits.  2019 when the
 * handle has no TMA descriptors.  No counterpart in the reference. */
int tc_use_tma(tc_handle* h, int enable);
/* The configuration the handle was created with (TMAX as tc_set_tmax or a
 * restart left it). */
int tc_get_bou(const tc_handle* h, tc_bou* out);
/* TMAX of the stop test 333 (main.F90:206).  ReadFlowField.F90:149 adds the
 * restart time to it; tc_h5_read_continua does the same through this call,
 * and a host that reads the continuation files itself sets it here. */
int tc_set_tmax(tc_handle* h, double tmax);
void tc_destroy(tc_handle* h);
const char* tc_last_error(const tc_handle* h);   /* h may be NULL */

/* Order all later work of h on this CUDA stream (cudaStream_t, NULL = the
 * legacy default stream). */
int tc_set_stream(tc_handle* h, void* cuda_stream);

/* Host memory for tc_set_state / tc_get_state and the other host arrays:
 * `bytes` of zeroed, page-locked memory on transparent huge pages (aligned
 * to the huge-page size), registered with the CUDA driver.  Copies from and
 * into it keep the CPU-GPU link rate however long the GPU has been busy,
 * which copies through memory of 64 KiB pages did not on the GB300 host.
 * 1002 when the mapping fails, 1000 + cudaError_t when the registration
 * does.  No counterpart in the reference (its arrays are Fortran
 * allocatables). */
int tc_host_alloc(size_t bytes, void** ptr);
/* Unregister and unmap a tc_host_alloc buffer (2000 for any other pointer). */
int tc_host_free(void* ptr);

/* ---- state transfer (ReadFlowField.F90:135-140 / WriteFlowField) -------- */

/* Copy a start into the handle: host arrays in the reference layout; halo
 * entries are ignored (the device keeps the fields periodic by index wrap).
 * The wall faces qr(1,:,:) and qr(nr,:,:) are kept as given: the
 * reference reads them until ImplicitAndUpdateQR sets them to 0 in the
 * first substep (CreateInitialConditions leaves qr(1) non-zero).  pr may be
 * NULL (zero pressure, as ReadFlowField leaves it).  Also zeroes ru1..ru3. */
int tc_set_state(tc_handle* h, const double* qt, const double* qr,
                 const double* qz, const double* pr);
/* Copy the state back into host arrays in the reference layout with the
 * periodic halo filled (the values update_halo would leave). */
int tc_get_state(tc_handle* h, double* qt, double* qr, double* qz, double* pr);
/* Copy any 3-D array (enum tc_field) back; see the shapes in the enum. */
int tc_get_field(tc_handle* h, int which, double* out);
/* Overwrite a 3-D array (enum tc_field) from the host, same shapes. */
int tc_set_field(tc_handle* h, int which, const double* in);

/* ---- restart files (HDF5, without libhdf5) --------------------------------
 * The reference's continuation files in the layout its HDF5 routines use
 * (HdfRoutines.F90:388-477): continua_qt.h5, continua_qr.h5, continua_qz.h5
 * with one float64 dataset "var" of dataspace [nthm][nzm][nr] (Fortran
 * q(1:nr, 1:nzm, 1:nthm), r fastest), and continua_master.h5 with the
 * scalars nr, nth, nz, istr (int32) and time, rint, rext, str, alx3, lamb
 * (float64).  Files are written in the HDF5 1.8 format subset that library
 * writes by default (superblock 0, symbol-table groups, contiguous storage)
 * and read back from it; chunked, compressed and new-style-group files are
 * rejected with 2022.  dir may be NULL (current directory). */

/* WriteFlowField.F90:17-47: the state of h at simulated time `time`. */
int tc_h5_write_continua(tc_handle* h, const char* dir, double time);
/* ReadFlowField.F90:31-149: load the files into h (tc_set_state; pr = 0)
 * and return their time (0 when IRESET = 1, ReadFlowField.F90:144); h's
 * TMAX becomes TMAX + that time (ReadFlowField.F90:149).  Files of another grid (nth, nz, nr, istr or str
 * differ) are interpolated onto h's grid as interp.F90 does (its quirks
 * kept: the old field's halos are linear extrapolations, qr and qz are
 * placed at (tm, zc, rm) and (tm, zm, rc), the radial direction takes the
 * lower plane, istr = 0 grids are built as rext x + rint); a grid more than
 * twice as fine in any direction, or ISTR other than 0 and 6, fails with
 * 2024. */
int tc_h5_read_continua(tc_handle* h, const char* dir, double* time);
/* The same as host arrays, without a handle (no GPU): qt, qr, qz receive
 * the fields in the reference layout of cfg's grid (halos 0); the time is
 * 0 when IRESET = 1, and TMAX is the caller's to extend. */
int tc_h5_load_continua(const tc_bou* cfg, const char* dir, double* qt, double* qr, double* qz,
                        double* time);
/* Scalar datasets (int32 where is_int[i], else float64) in a new file, as
 * HdfSerialWrite{Int,Real}Scalar write them. */
int tc_h5_write_scalars(const char* path, int n, const char* const* names, const double* values,
                        const int* is_int);
/* WriteGridInfo.F90:22-33: cordin_info.h5 with rm(1:nrm), rc(1:nr),
 * tm(1:nthm), zm(1:nzm) (host only). */
int tc_h5_write_grid_info(const tc_bou* cfg, const char* dir);
/* Dumps of the output steps (main.F90:191-198), files named with
 * itime = nint(1000 time + 0.005) as %08d, written into dir:
 * DumpFlowField.F90: qt_, qr_, qz_<itime>.h5 ("var", as the continua) and
 *   ms_<itime>.h5 (time, rint, rext, istr, str, alx3, lamb);
 * DumpRCuts.F90: slab<m>vt_, slab<m>vr_, slab<m>vz_<itime>.h5, the cylinder
 *   surfaces at the radii rslab[0..nslab-1] (at most 9; cell k with
 *   rm(k-1) < rslab < rm(k), InitDumpRCuts), shape (nzm, nthm);
 * DumpThCuts.F90: the theta = 1 plane, shape (nrm, nzm), into slabvt_ and
 *   slabvz_<itime>.h5 (the reference writes its vr plane to the slabvt_
 *   name too, replacing vt there; kept);
 * DumpStreamwiseAvg.F90: theta averages into slabvt_ax_, slabvr_ax_,
 *   slabvz_ax_<itime>.h5, shape (nrm, nzm).
 * The fields are read back from the device (tc_get_state). */
int tc_h5_dump_flow_field(tc_handle* h, const char* dir, double time);
int tc_h5_dump_rcuts(tc_handle* h, const char* dir, double time, const double* rslab, int nslab);
int tc_h5_dump_thcuts(tc_handle* h, const char* dir, double time);
int tc_h5_dump_streamwise_avg(tc_handle* h, const char* dir, double time);
/* One float64 dataset `name` of the given shape (C order) in a new file. */
int tc_h5_write_dataset(const char* path, const char* name, int rank,
                        const long long* dims, const double* data);
/* Dataset `name` of an HDF5 file as doubles (float64/32 and int32/64 are
 * converted): *rank and dims[0..rank-1] receive the shape (up to 8 axes);
 * out (may be NULL to query the shape) receives up to cap values. */
int tc_h5_read_dataset(const char* path, const char* name, double* out, long long cap,
                       int* rank, long long* dims);

/* ---- the time step ------------------------------------------------------ */

/* TimeMarcher.F90:12-67: one full time step of length dt from time `time`
 * (all NSST substeps).  Asynchronous; returns after enqueueing. */
int tc_time_marcher(tc_handle* h, double dt, double time);

/* main.F90:152-226 restricted to the step path: for each of nsteps steps,
 * CalcMaxCFL, the dt rule (variable dt: DTMIN for ntime <= 1, then
 * min(CFLMAX/instCFL, DTMAX); IDTV=0 runs with dt = DTMAX because the
 * reference never assigns dt in that branch), TimeMarcher, time += dt, and on
 * output steps (ntime == 1 or mod(time,TOUT) < dt) the velocity-limit and
 * divergence checks.  Step control lives on the device; the host reads it
 * back only on output steps.  Returns the first error code raised (166, 165,
 * 266, 169, 333, 555) or 0; *time, *dt and *ntime are updated. */
int tc_run(tc_handle* h, int nsteps, int* ntime, double* time, double* dt);

/* ---- routines of one substep, for parity bisection ---------------------- */

/* TimeMarcher.F90:20-23: beta, InnerCylVelocity, SlipBCs for a step of
 * length dt starting at time; then TimeMarcher.F90:27-29 for substep ns
 * (1-based) is selected with tc_set_substep. */
int tc_begin_step(tc_handle* h, double dt, double time);
int tc_set_substep(tc_handle* h, int ns);
/* One routine each, as TimeMarcher.F90:31-37 calls them (the per-substep
 * coefficients al, ga, ro of the substep chosen with tc_set_substep).
 * ExplicitTermsQT.F90:22-129: explicit terms of qt into DQ. */
int tc_explicit_terms_qt(tc_handle* h);
/* ExplicitTermsQR.F90:25-149: explicit terms of qr (faces k = 2..nrm) into
 * HR (the reference keeps them in dph). */
int tc_explicit_terms_qr(tc_handle* h);
/* ExplicitTermsQZ.F90:23-106: explicit terms of qz into QCAP. */
int tc_explicit_terms_qz(tc_handle* h);
/* ImplicitAndUpdateQT.F90:26-117: rhs and ru1 from DQ, then
 * SolveImpEqnUpdate_QT (SolveImpEqnUpdate_QT.F90:22-80): the radial solve
 * with the inner-wall term of the oscillating cylinder, qt += dq. */
int tc_implicit_and_update_qt(tc_handle* h);
/* ImplicitAndUpdateQR.F90:28-71: rhs and ru2 from HR, then
 * SolveImpEqnUpdate_QR (SolveImpEqnUpdate_QR.F90:25-67), qr += dq, and qr
 * set to 0 on both walls. */
int tc_implicit_and_update_qr(tc_handle* h);
/* ImplicitAndUpdateQZ.F90:24-119: rhs and ru3 from QCAP (outer-wall row
 * with the reference's overwritten ru3(nrm)), then SolveImpEqnUpdate_QZ
 * (SolveImpEqnUpdate_QZ.F90:21-70), qz += dq. */
int tc_implicit_and_update_qz(tc_handle* h);
/* SolveImpEqnUpdate_QT/QR/QZ alone, each on its RHS_T/R/Z array. */
int tc_solve_imp_eqn_update_qt(tc_handle* h);
int tc_solve_imp_eqn_update_qr(tc_handle* h);
int tc_solve_imp_eqn_update_qz(tc_handle* h);
/* The three components in one launch each (what the fused time step runs):
 * tc_explicit_terms = ExplicitTermsQT + QR + QZ; tc_implicit_and_update =
 * ImplicitAndUpdateQT + QR + QZ with their solves; tc_solve_imp_eqn_update
 * = the three solves. */
int tc_explicit_terms(tc_handle* h);
int tc_implicit_and_update(tc_handle* h);
int tc_solve_imp_eqn_update(tc_handle* h);
/* Explicit terms fused with the rhs and ru update (no DQ/HR/QCAP arrays);
 * equivalent to tc_explicit_terms followed by the rhs half of
 * tc_implicit_and_update. */
int tc_explicit_and_rhs(tc_handle* h);
/* CalcLocalDivergence.F90:19-40: DPH = div(q)/(al*dt). */
int tc_calc_local_divergence(tc_handle* h);
/* SolvePressureCorrection.F90:100-163: DPH <- phi.  The singular
 * k_theta = k_z = 0 mode is solved with phi(nrm) = 0 (its last equation is
 * the dependent one); LAPACK in the reference divides by a roundoff pivot
 * there instead, which only moves phi by a radially constant offset. */
int tc_solve_pressure_correction(tc_handle* h);
/* CorrectVelocity.F90:28-47 and CorrectPressure.F90:23-49. */
int tc_correct_velocity(tc_handle* h);
int tc_correct_pressure(tc_handle* h);

/* ---- reductions (host scalars; these synchronise) ------------------------ */

/* CalcMaxCFL.F90:12-49 */
int tc_calc_max_cfl(tc_handle* h, double* cflm);
/* CheckDivergence.F90:21-43.  A NaN in the fields makes *qmax NaN and the
 * status 169 (the reference's divergence error code): Fortran's MAX would
 * skip the NaN and report a finite divergence. */
int tc_check_divergence(tc_handle* h, double* qmax);
/* CalcTorque.F90:26-57 (the host writes torquenu.out itself). */
int tc_calc_torque(tc_handle* h, double* inner, double* outer);
/* CalcVelocityStats.F90:11-68: vmax(3) and the three rms values. */
int tc_calc_velocity_stats(tc_handle* h, double* vmax3, double* rms3);

/* CheckDivergence.F90:28-43 on velocity arrays the caller keeps on the
 * current CUDA device, without a handle and without allocating device
 * memory.  No counterpart in the reference.
 *  - qt, qr, qz: device arrays in the reference layout
 *    q(1:nrm+1, 0:nzm+1, 0:nthm+1), r fastest, periodic halos current (as
 *    after update_halo); cells k = 1..nrm, j = 1..nzm, i = 1..nthm are read.
 *  - udx2m, usrm: HOST arrays, entries 0..nrm-1 = udx2m(1:nrm), usrm(1:nrm)
 *    (tc_grid_array TC_G_UDX2M, TC_G_USRM); dxt = nthm*LAMB/(2 pi),
 *    dxz = nzm/ALX3 (dx1, dx3 of CreateGrid.F90:28-34).
 *  - stream: cudaStream_t the work is ordered on (NULL = legacy default);
 *    the call synchronises it and returns the maximum |div| in *qmax.  A NaN
 *    in the fields makes *qmax NaN and the status 169, as tc_check_divergence.
 *    The call copies the coefficients from pageable host memory and waits
 *    for the stream, so it cannot run inside a stream capture: on a stream
 *    that is being captured it returns 2018 and enqueues nothing.
 * Its scratch (coefficients, per-block maxima, result) is one static
 * 130 KB device array per device, not memory of the caller's: nrm above
 * 8192 is rejected with 2016.  Nothing in it must start at zero; every
 * call writes what it later reads.  The first call with a device current
 * looks the array's address up (cudaGetSymbolAddress), so make it before
 * any stream capture.  Calls on one device share the array: calls that
 * overlap (other streams, other host threads) race and may return each
 * other's values; issue them one at a time. */
int tc_check_divergence_noalloc(const double* qt, const double* qr, const double* qz,
                                int nthm, int nzm, int nrm,
                                const double* udx2m, const double* usrm,
                                double dxt, double dxz, void* stream, double* qmax);

/* ---- ensembles (no counterpart in the reference) -------------------------
 * Many independent runs of different sizes, Re and radius ratio resident on
 * one device and advanced together: each step of the ensemble is one CUDA
 * graph of grouped launches, each launch covering every member (a flat list
 * of (member, tile) items).  A member's arithmetic is the single-run path's,
 * so its result does not depend on which other members share the launches.
 * One ensemble has one precision; all members use the same NSST; patterned
 * slip (MINSTRT/MINSTRZ > 0) is not supported; no output-step checks run
 * (read a member's reductions through its handle between steps). */

int tc_ensemble_create(int precision, tc_ensemble** out);
/* Waits for the ensemble's stream, frees every member and the tables. */
void tc_ensemble_destroy(tc_ensemble* e);
const char* tc_ensemble_last_error(const tc_ensemble* e);
/* Stream of all later ensemble work (members included). */
int tc_ensemble_set_stream(tc_ensemble* e, void* cuda_stream);
/* Admit a run: build its handle (tc_create_ex), load the start (tc_set_state
 * arrays, pr may be NULL) and choose its time step:
 *   dt > 0             fixed dt;
 *   dt <= 0, IDTV = 1  the reference's variable dt every step
 *                      (main.F90:156-174: CalcMaxCFL of the current field,
 *                      DTMIN on the first steps, errors 165/166 stop the
 *                      member);
 *   dt <= 0, IDTV = 0  fixed dt = min(LIMITCFL / CFL(start), DTMAX).
 * nsteps is the run's requested length,
 * kept for the caller (tc_ensemble_status); the ensemble does not stop a
 * member by itself.  *slot receives the member's slot (reused after
 * tc_ensemble_remove).  Synchronises the ensemble's stream. */
int tc_ensemble_add(tc_ensemble* e, const tc_bou* cfg, double dt, const double* qt,
                    const double* qr, const double* qz, const double* pr, int nsteps,
                    int* slot);
/* Retire a member and free its device memory (waits for the stream). */
int tc_ensemble_remove(tc_ensemble* e, int slot);
/* The member's handle, for tc_get_state / tc_calc_torque / ... (owned by
 * the ensemble: do not tc_destroy it). */
int tc_ensemble_member(tc_ensemble* e, int slot, tc_handle** h);
int tc_ensemble_count(const tc_ensemble* e);
/* Tile shapes: threads per cell/column/mode tile (64, 128 or 256) and rows
 * per theta-FFT block (0 = the single-run choice for the largest member,
 * else 1..32, a power of two).  Takes effect at the next tc_ensemble_step.
 * The persistent schedule uses 128 threads and at most 8 rows. */
int tc_ensemble_tune(tc_ensemble* e, int threads, int rows);
/* Schedule of a step:
 *   TC_SCHED_GROUPED     one CUDA graph of grouped launches per step (a
 *                        launch per phase and RK substep, each over every
 *                        member: 27 or, with variable-dt members, 28);
 *   TC_SCHED_PERSISTENT  one CUDA graph of one cooperative launch per RK
 *                        substep, each running all phases of the substep for
 *                        every member with grid-wide barriers between them
 *                        (the first also CFL, dt and the momentum factors,
 *                        the last also time += dt).
 * Both run the same device bodies on the same work lists: a member's results
 * are the same under either.  A barrier wait in the persistent kernel is
 * bounded; if one gives up, tc_ensemble_sync returns 3001.  blocks_per_sm
 * caps the persistent launch's blocks per SM (0 = the occupancy limit; fewer
 * blocks make the barriers cheaper and leave fewer warps per phase).  Takes
 * effect at the next tc_ensemble_step. */
enum tc_schedule { TC_SCHED_GROUPED = 0, TC_SCHED_PERSISTENT = 1 };
int tc_ensemble_schedule(tc_ensemble* e, int schedule, int blocks_per_sm);
int tc_ensemble_get_schedule(const tc_ensemble* e);
/* Blocks of the persistent launch (occupancy limit x SMs; 0 before the first
 * persistent step). */
int tc_ensemble_persistent_blocks(const tc_ensemble* e);
/* Bound on one grid-barrier wait of the persistent kernel (default 10 s,
 * measured by the device's global timer). */
int tc_ensemble_set_barrier_timeout(tc_ensemble* e, double seconds);
/* Failure-path test: make the next persistent barrier unreachable (its
 * arrival count can no longer reach the grid size), so that every block's
 * wait runs out after the barrier timeout; the next tc_ensemble_sync or
 * tc_ensemble_status returns 3001 and resets the barrier.  Steps enqueued
 * before that synchronisation do nothing. */
int tc_ensemble_stall_next_barrier(tc_ensemble* e);
/* Enqueue nsteps steps of every member (graph replays; asynchronous). */
int tc_ensemble_step(tc_ensemble* e, int nsteps);
/* Wait for the enqueued steps; 3001 if a persistent barrier wait gave up
 * (those steps then did nothing from the failed barrier on). */
int tc_ensemble_sync(tc_ensemble* e);
/* Steps done, simulated time, last dt and error code (165/166 for a
 * variable-dt member, which then stops) of a member (synchronises). */
int tc_ensemble_status(tc_ensemble* e, int slot, int* steps_done, double* time,
                       double* dt, int* errorcode);
/* Requested length given to tc_ensemble_add. */
int tc_ensemble_target(const tc_ensemble* e, int slot);
long long tc_ensemble_launch_count(const tc_ensemble* e);
int tc_ensemble_launches_per_step(const tc_ensemble* e);
long long tc_ensemble_device_bytes(const tc_ensemble* e);
/* Cells of all members: sum of nthm * nzm * nrm. */
long long tc_ensemble_cells(const tc_ensemble* e);

/* ---- statistics of the output steps (main.F90:188-190) -------------------
 * Theta averages accumulated per (r, z) row in FP64 on the device, the
 * reference's stat_arrays: (nrm, nzm) arrays, r fastest. */
enum tc_stat {
    TC_ST_VT_MEAN = 0, TC_ST_VR_MEAN, TC_ST_VZ_MEAN, TC_ST_WT_MEAN, TC_ST_WR_MEAN, TC_ST_WZ_MEAN,
    TC_ST_VT_RMS, TC_ST_VR_RMS, TC_ST_VZ_RMS, TC_ST_WT_RMS, TC_ST_WR_RMS, TC_ST_WZ_RMS,
    TC_ST_VTVR_MEAN, TC_ST_VTVZ_MEAN, TC_ST_VRVZ_MEAN, TC_ST_PR_MEAN, TC_ST_PR_RMS,
    TC_ST_DISSTE, TC_ST_COUNT
};
/* CalcStats (StatRoutines.F90:13-76, with CalcVorticity.F90:30-70): one
 * sample of every statistic but disste. */
int tc_calc_stats(tc_handle* h);
/* CalcDissipation.F90:22-74: accumulate disste and return the normalised
 * volume dissipation nute (the value the reference writes to unit 92). */
int tc_calc_dissipation(tc_handle* h, double* nute);
/* Statistic `which` (enum tc_stat) into out[nrm * nzm] (r fastest). */
int tc_get_stat(tc_handle* h, int which, double* out);
/* Samples taken by tc_calc_stats since creation or tc_reset_stats. */
int tc_stat_samples(const tc_handle* h);
int tc_reset_stats(tc_handle* h);
/* WriteStats (StatRoutines.F90:82-177): <dir>/<name>.h5 with dataset <name>
 * of shape (nrm, nzm) for every statistic, and <dir>/stafield_master.h5
 * with averaging_time, R_cordin, Th_cordin, Z_cordin, "Reynolds Number"
 * and R_Omega.  readstats = 1 adds the values already in the files
 * (StatReadReduceWrite.F90:27-33). */
int tc_h5_write_stats(tc_handle* h, const char* dir, int readstats);

/* ---- measurement helpers ------------------------------------------------ */

/* Number of kernels one tc_time_marcher call launches. */
int tc_kernels_per_step(const tc_handle* h);
/* Device bytes held by the handle. */
long long tc_device_bytes(const tc_handle* h);
/* Kernels launched by this handle so far (all entry points). */
long long tc_launch_count(const tc_handle* h);
/* Kernels one step of tc_run launches (step control and checks included). */
int tc_kernels_per_run_step(const tc_handle* h);
/* Per-kernel-class timing: enable (1) or disable (0) CUDA-event brackets
 * around every launch on the handle's stream; enabling resets the totals. */
int tc_profile(tc_handle* h, int enable);
/* Totals since tc_profile(h, 1): ms[c] and launches[c] for class c; returns
 * the number of classes.  tc_profile_name(c) names class c. */
int tc_profile_read(tc_handle* h, double* ms, long long* launches, int cap);
const char* tc_profile_name(int cls);
/* FP64 FMA throughput of the device in TFLOP/s (a dedicated probe kernel on
 * the handle's stream; used as the FP64 roofline denominator). */
int tc_measure_fp64_peak(tc_handle* h, double* tflops);
/* Self-check of the integer-pipe float <-> double conversions the mixed
 * path uses: n operands (random bit patterns, the binary32 exponent range
 * and rounding halfway cases) converted both ways and compared bit for bit
 * with the hardware conversions on the current device; *mismatches receives
 * the count (0 expected).  No counterpart in the reference. */
int tc_selftest_conversions(long long n, long long* mismatches);

#ifdef __cplusplus
}
#endif
#endif /* TC_CAPI_H */
