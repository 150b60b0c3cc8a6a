// tc_kernels.cuh -- launch interface of the step kernels (tc_kernels.cu).
//
// Every velocity-side kernel is a template on the element type T (double:
// plain FP64 path; float: mixed path).  The launchers are instantiated for
// both.
#pragma once

#include <cuda.h>   // CUtensorMap

#include "tc_dev.h"

namespace tcgb {

enum { MODE_FUSED = 0, MODE_EXPLICIT = 1, MODE_IMPLICIT = 2 };

// TMA descriptors of the mixed path's march inputs (FP32 arrays [k][j][i]),
// made once per handle: q6 (qt, qr, qz, pr) with boxes of 72 x 6 x 1
// elements (theta x z x r), q1 the same arrays with single-row boxes (for
// the tiles whose z rows wrap), ru the RK memory with 72 x 4 x 1 boxes.
struct MarchMaps {
    CUtensorMap q6[4], q1[4], ru[3];
};

template <typename T>
struct FieldsT {
    T *qt, *qr, *qz;
    double* pr;                       // pressure is FP64 in both paths
    T* prf;                           // pr rounded to T for the momentum rhs (aliases pr when T = double)
    T* phi;
    T *ru1, *ru2, *ru3;
    T *rhs_t, *rhs_r, *rhs_z;
    T *h_t, *h_r, *h_z;               // explicit-term arrays (per-routine entry points only)
    typename V2<T>::type* spec;
    const double *pf_l, *pf_dinv;     // pressure LU factors [k][kz <= nzm/2][kt] (FP64)
    signed char* icyl;                // inner-wall slip mask per column (1 = no slip)
    StepState* st;
    MomFactorsT<T> F;                 // momentum LU factors of the step
    T* corr;                          // CorrectVelocity coefficients [s][3][nr+1]
    MomFactorsT<double> Fd;           // the same in FP64 (aliases F, corr when T = double)
    double* corrd;
    double* scal;                     // per substep: [s] usdt*fft_norm, [3+s] usdt
    double* red;                      // reduction partials
    // mixed path (T = float): the checkpoint slots of the pressure solve's
    // forward sweep (16 bytes each: an FP64 complex value, or a float-float
    // one); with ptri_ff set the pressure factors and the super-diagonal are
    // float-float pairs (pl_ff, pdi_ff alias pf_l, pf_dinv, converted in
    // place) and the solve runs in float-float, else in FP64 on pf_l, pf_dinv
    const float2 *pl_ff, *pdi_ff, *pu_ff;
    float4* ws;
    int ptri_ff;
    // host pointer to the handle's march descriptors (mixed path, single
    // runs; null: the march loads through the read-only cache instead)
    const MarchMaps* tma;
};

template <typename T>
struct PlansT {
    FFTPlan th;        // complex length nthm/2 (real transform along theta)
    FFTPlan z;         // complex length nzm
    const typename V2<T>::type* tw_th;   // exp(-2 pi i j / (nthm/2))
    const typename V2<T>::type* tw_z;    // exp(-2 pi i j / nzm)
    const typename V2<T>::type* twr;     // exp(-2 pi i k / nthm), k = 0..nthm/2
};

int reduction_blocks();
int theta_rows(int M);
// Dynamic shared memory of a single-run z-FFT block for transforms of
// length nz (at most 200 KB are granted).
size_t zfft_smem_bytes(int nz, bool mixed);

// Step control (precision independent).
void launch_begin_step(cudaStream_t s, const Consts& k, StepState* st, int mode, double dt, double time);
void launch_end_step(cudaStream_t s, const Consts& k, StepState* st);
void launch_finish_step(cudaStream_t s, const Consts& k, StepState* st);
template <typename T> void launch_slip(cudaStream_t s, const Dims& d, const Consts& k, const FieldsT<T>& f);
template <typename T>
void launch_factors(cudaStream_t s, const Dims& d, const Coef& c, const Consts& k, const FieldsT<T>& f);

// Substep kernels.
// mask (MODE_EXPLICIT, MODE_IMPLICIT): components 1 qt, 2 qr, 4 qz.
template <typename T>
void launch_momentum(cudaStream_t s, int mode, const Dims& d, const CoefT<T>& c, const Consts& k,
                     const FieldsT<T>& f, int sub, int mask = 7);
// Components comp0 .. comp0 + ncomp - 1 (0 qt, 1 qr, 2 qz).
template <typename T>
void launch_radial_solve(cudaStream_t s, const Dims& d, const FieldsT<T>& f, int sub, int comp0 = 0, int ncomp = 3);
template <typename T>
void launch_div_fft(cudaStream_t s, const Dims& d, const CoefT<T>& c, const Consts& k, const FieldsT<T>& f,
                    const PlansT<T>& p, int sub, bool from_phi);
template <typename T> void launch_zfft(cudaStream_t s, const Dims& d, const FieldsT<T>& f, const PlansT<T>& p, bool inv);
template <typename T>
void launch_pressure_tridiag(cudaStream_t s, const Dims& d, const Coef& c, const FieldsT<T>& f);
template <typename T> void launch_theta_inverse(cudaStream_t s, const Dims& d, const FieldsT<T>& f, const PlansT<T>& p);
template <typename T>
void launch_correct(cudaStream_t s, const Dims& d, const Coef& c, const CoefT<T>& cv, const Consts& k, const FieldsT<T>& f,
                    int sub, bool vel, bool pres);
template <typename T>
void launch_divergence(cudaStream_t s, const Dims& d, const CoefT<T>& c, const Consts& k, const FieldsT<T>& f,
                       int sub);

// One-time set-up.
void launch_pressure_factors(cudaStream_t s, const Dims& d, const Coef& c, double* l, double* dinv);
void launch_pressure_factors_ff(cudaStream_t s, const Dims& d, const Coef& c, double* l, double* dinv, float2* u);

// Reductions (FP64 arithmetic; results land in StepState).
template <typename T>
void launch_cfl(cudaStream_t s, const Dims& d, const Coef& c, const CoefT<T>& cv, const Consts& k, const FieldsT<T>& f);
template <typename T>
void launch_check_divergence(cudaStream_t s, const Dims& d, const Coef& c, const CoefT<T>& cv, const Consts& k,
                             const FieldsT<T>& f, bool only_on_output);
template <typename T>
void launch_velocity_stats(cudaStream_t s, const Dims& d, const Coef& c, const Consts& k,
                           const FieldsT<T>& f, bool only_on_output);
template <typename T>
void launch_torque(cudaStream_t s, const Dims& d, const Coef& c, const Consts& k, const FieldsT<T>& f);

// Layout conversion between the reference layout (FP64 host arrays, with or
// without halo) and a device array of element type T.  nk device planes;
// halo = 1 for (nr, nzm+2, nthm+2) arrays, 0 for (nr, nzm, nthm).
template <typename T>
void launch_to_device(cudaStream_t s, const Dims& d, const double* stage, T* dst, int nk, int halo);
template <typename T>
void launch_to_host(cudaStream_t s, const Dims& d, const T* src, double* stage, int nk, int halo);

// dst[i] = (float)src[i], i < n.
void launch_round_to_float(cudaStream_t s, const double* src, float* dst, long long n);

// Dense FP64 FMA rate of the current device in TFLOP/s (measurement helper).
double measure_fp64_peak(cudaStream_t s);

}  // namespace tcgb
