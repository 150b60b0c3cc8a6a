// tc_kernels.cuh -- launch interface of the step kernels (tc_kernels.cu).
#pragma once

#include "tc_dev.h"

namespace tcgb {

enum { MODE_FUSED = 0, MODE_EXPLICIT = 1, MODE_IMPLICIT = 2 };

struct Fields {
    double *qt, *qr, *qz, *pr, *phi;
    double *ru1, *ru2, *ru3;
    double *rhs_t, *rhs_r, *rhs_z;
    double *h_t, *h_r, *h_z;          // explicit-term arrays (per-routine entry points only)
    double2* spec;
    const double *pf_l, *pf_dinv;     // pressure LU factors [k][kz <= nzm/2][kt]
    signed char* icyl;                // inner-wall slip mask per column (1 = no slip)
    StepState* st;
    MomFactors F;
    double* corr;                     // per-substep correction coefficients [s][3][nr+1]
    double* red;                      // reduction partials
};

struct Plans {
    FFTPlan th;        // complex length nthm/2 (real transform along theta)
    FFTPlan z;         // complex length nzm
    const double2* twr;  // exp(-2 pi i k / nthm), k = 0..nthm/2
};

int reduction_blocks();

// Step control.
void launch_begin_step(cudaStream_t s, const Consts& k, StepState* st, int mode, double dt, double time);
void launch_slip(cudaStream_t s, const Dims& d, const Consts& k, const Fields& f);
void launch_factors(cudaStream_t s, const Dims& d, const Coef& c, const Consts& k, const Fields& f);
void launch_end_step(cudaStream_t s, const Consts& k, StepState* st);
void launch_finish_step(cudaStream_t s, const Consts& k, StepState* st);

// Substep kernels.
void launch_momentum(cudaStream_t s, int mode, const Dims& d, const Coef& c, const Consts& k,
                     const Fields& f, int sub);
void launch_radial_solve(cudaStream_t s, const Dims& d, const Fields& f, int sub);
void launch_div_fft(cudaStream_t s, const Dims& d, const Coef& c, const Consts& k, const Fields& f,
                    const Plans& p, int sub, bool from_phi);
void launch_zfft(cudaStream_t s, const Dims& d, const Fields& f, const Plans& p, bool inv);
void launch_pressure_tridiag(cudaStream_t s, const Dims& d, const Coef& c, const Fields& f);
void launch_theta_inverse(cudaStream_t s, const Dims& d, const Fields& f, const Plans& p);
void launch_correct(cudaStream_t s, const Dims& d, const Coef& c, const Consts& k, const Fields& f,
                    int sub, bool vel, bool pres);
void launch_divergence(cudaStream_t s, const Dims& d, const Coef& c, const Consts& k, const Fields& f,
                       int sub);

// One-time set-up.
void launch_pressure_factors(cudaStream_t s, const Dims& d, const Coef& c, double* l, double* dinv);

// Reductions (results land in StepState).
void launch_cfl(cudaStream_t s, const Dims& d, const Coef& c, const Consts& k, const Fields& f);
void launch_check_divergence(cudaStream_t s, const Dims& d, const Coef& c, const Consts& k,
                             const Fields& f, bool only_on_output);
void launch_velocity_stats(cudaStream_t s, const Dims& d, const Coef& c, const Consts& k,
                           const Fields& f, bool only_on_output);
void launch_torque(cudaStream_t s, const Dims& d, const Coef& c, const Consts& k, const Fields& f);

// Layout conversion between the reference layout (with halo) and the device.
// nk device planes; halo = 1 for (nr, nzm+2, nthm+2) arrays, 0 for (nr, nzm, nthm).
void launch_to_device(cudaStream_t s, const Dims& d, const double* stage, double* dst, int nk, int halo);
void launch_to_host(cudaStream_t s, const Dims& d, const double* src, double* stage, int nk, int halo);
int theta_rows(int M);

// Dense FP64 FMA rate of the current device in TFLOP/s (measurement helper).
double measure_fp64_peak(cudaStream_t s);

}  // namespace tcgb
