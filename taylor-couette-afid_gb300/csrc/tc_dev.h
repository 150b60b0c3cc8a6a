// tc_dev.h -- device-side data structures shared by the kernels and the C ABI.
//
// Device layout of every 3-D field: [k][j][i] with i = theta fastest
// (contiguous), then j = z, then k = r; no halo cells (periodic neighbours are
// found by index wrap).  k is the reference radial index minus one:
//   qt, qz, pr, phi, ru1, ru3, rhs_t, rhs_z : k = 0 .. nrm-1   (cells)
//   qr, ru2, rhs_r                          : k = 0 .. nrm     (faces; 0 and
//                                             nrm are the walls, always 0)
// The pressure spectrum is complex [k][kz][kt] with kt = 0..nthm/2 (the
// half-spectrum of the real transform along theta) and kz = 0..nzm-1.
//
// Precision: the element type T of the velocity-side arrays (q, ru, rhs,
// explicit terms, phi, spectrum, momentum factors) is double for the plain
// FP64 path and float for the mixed path.  The pressure pr, the pressure LU
// factors and the reductions are double in both.
#pragma once

#include <cstddef>
#include <cuda_runtime.h>

namespace tcgb {

constexpr int kMaxStages = 24;

template <typename T> struct V2;
template <> struct V2<double> { typedef double2 type; };
template <> struct V2<float> { typedef float2 type; };

// Radix plan of one complex transform length (radices 2, 3, 4, 5, 7, 8, 11,
// 13), with the
// stride rp = n / (L p) of every Stockham stage and the multipliers that turn
// the kernels' divisions by rp, n and n + 1 into a multiply-high:
// x / d = umulhi(x, ceil(2^32 / d)) exactly when x * d < 2^32 (n <= 65536);
// a multiplier of 0 stands for d = 1.
struct FFTPlan {
    int n = 0;
    int nstages = 0;
    int radix[kMaxStages] = {0};
    int rp[kMaxStages] = {0};
    unsigned mrp[kMaxStages] = {0};
    unsigned mn = 0, mn1 = 0;
};

// A twiddle in the factored form of the FP64 multiply-add butterflies
// (tc_fft.cuh): w y = (fx (z.x - g z.y), fy (z.y + g z.x)), z = y or, when
// swap != 0, y with its parts swapped.
template <typename R> struct FTw {
    R g, fx, fy, swap;
};

inline unsigned div_magic(unsigned d) {
    return d <= 1 ? 0u : (unsigned)(((1ull << 32) + d - 1) / d);
}

struct Dims {
    int nt, nz, nr;        // nthm, nzm, nrm
    int M, PH;             // nthm/2, nthm/2 + 1
    int nzh;               // nzm/2 + 1
    long long P;           // nz * nt (one r-plane of a real field)
    long long PS;          // nz * PH (one r-plane of the spectrum)
    unsigned mnz;          // row / nz multiplier for rows < nr * nz (0: divide in hardware)
};

// 1-D coefficient arrays on the device, 0-based (entry m = reference m+1).
template <typename T>
struct CoefT {
    const T *usrm, *usrc, *udx2rm, *udx1vis1, *udxt_m, *udxtq_m;
    const T *rc, *udx2c, *udx1vis2, *udxt_c, *udxtq_c;
    const T *ap1j, *ac1j, *am1j, *ap2je, *ac2je, *am2je, *ap3j, *ac3j, *am3j;
    const T *ap2j, *ac2j, *am2j;
    const T *udx2m, *rudx2c, *udx1qm, *apph, *acph, *amph, *usrm2;
    // products with powers of two folded in (exact): 0.25*udx2rm, 0.25*usrm,
    // 0.5*udx1vis1, 0.25*udx2c; and 0.25*rc*romeg
    const T *q_udx2rm, *q_usrm, *h_udx1vis1, *q_udx2c, *q_rc_romeg;
    // statistics metrics (CreateGrid.F90:136-173)
    const T *rm, *udx2mm, *udx2cc, *pvol;
    // 0.5 dxt usrm and 0.5 udx2rm: the theta and radial terms of CalcMaxCFL
    // in one product each
    const T *h_dxt_usrm, *h_udx2rm;
    const T *ak1, *ak3;
};
typedef CoefT<double> Coef;
constexpr int kCoefArrays = 41;   // arrays before ak1, ak3

// Scalars of the configuration (param.F90).
struct Consts {
    double dxt, dxz, dxtq, dxzq, ren, romeg, virotint, virotext;
    double ap1j_fs0, ac1j_fs0, am1j_fs0, ap1j_fs1, ac1j_fs1;
    double ap3j_fs0, ac3j_fs0, am3j_fs0, ap3j_fs1, ac3j_fs1;
    double sizepert, omegapert, pi, rint, rext, lamb;
    double dtmin, dtmax, limitCFL, tout, tmax, limitVel, resid;
    double gam[3], rom[3], alm[3];
    // scalars hoisted out of the kernels (host-computed, time independent)
    double udxz, udxzq;          // dxz*0.25 (ExplicitTerms*), dxzq/ren
    double q_romeg;              // 0.25*romeg
    double alre[3];              // al/ren per substep
    double dxz_al[3], dxt_al[3]; // dxz*al, dxt*al per substep
    double fft_norm;             // 0.5/(nthm*nzm): FFT normalisation and real-unpacking 1/2
    int nsst, idtv, ntst;
    int patterned;          // patterned slip active (SlipBCs.F90:55-56)
    int minstrt, minstrz, multmin;
};

// Per-step state kept on the device (main.F90 / TimeMarcher.F90 scalars).
struct StepState {
    double time;        // start-of-step time
    double dt;
    double beta;        // dt / ren / 2
    double vinner_t, dvinner_t;
    double instcfl;     // last CalcMaxCFL result
    double dmax;        // last CheckDivergence result
    double vmax[3], rms[3];
    double torque[2];
    int ntime;          // step counter of main.F90
    int errorcode;      // code raised by the last step
    int halt;           // a step raised an error: later steps do nothing
    int output;         // the last step was an output step
    // dt, beta and vinner_t rounded once per step for the FP32 kernels of the
    // mixed path (so that they do not convert per cell)
    float dt_f, beta_f, vinner_f, pad_f;
    // dt of the momentum factors now in place (the factors kernel skips the
    // factorisation while dt does not change)
    double dt_factored;
};

// Checkpointed forward sweep of the mixed path's pressure solve (ptri_ff):
// levels per batch, and the checkpoint slots of a column of nr levels
// (levels kPtriCk m, m = 0..nb, and the tail levels kPtriCk nb + 1 .. nr - 1).
constexpr int kPtriCk = 8;
__host__ __device__ inline int ptri_slots(int nr) {
    const int nb = (nr - 1) / kPtriCk;
    return nb + 1 + (nr - 1 - kPtriCk * nb);
}

// Per-step coefficients of one step (factors kernel), per substep s:
// [ (s*3 + c)*(nr+1) + k ]  dt al(s) times the pressure-gradient metric of
//                            component c at level k
//                            (CorrectVelocity.F90:35-40; the momentum
//                            right-hand sides use the same products for the
//                            pressure of the step),
// [ 9*(nr+1) + s*3 + 0..2 ] gam(s) dt, rom(s) dt, alre(s) dt;
// and for the pressure of the step (CorrectPressure.F90:40-44 regrouped as
// pr + phi + pe phi + pt (phi_ip + phi_im) + pz (phi_jp + phi_jm)
//    + pq (phi_kp + phi_km), be = beta):
// [ kPresCoef(nr+1) + k ]              pe = be (2 udx1qm + 2 dxzq - acph)
// [ kPresCoef(nr+1) + (nr+1) + k ]     pt = -be udx1qm
// [ kPresCoef(nr+1) + 2 (nr+1) + k ]   pq = -be apph
// [ kPresCoef(nr+1) + 3 (nr+1) ]       pz = -be dxzq
// [ kPresCoef(nr+1) + 3 (nr+1) + 1 + k ] 1 + pe (the FP64 update starts
//                                        from pr + (1 + pe) phi)
// and for the divergence of substep s, with usdt(s) = 1/(al(s) dt) and the
// FFT normalisation f folded in (CalcLocalDivergence.F90:27-40 times usdt f):
// [ kDivCoef(nr+1) + s*2*(nr+1) + k ]          dt_k = dxt usrm(k) usdt f
// [ kDivCoef(nr+1) + s*2*(nr+1) + (nr+1) + k ] dr_k = udx2m(k) usrm(k) usdt f
// [ kDivCoef(nr+1) + 6*(nr+1) + s ]            dz = dxz usdt f
__host__ __device__ inline size_t kPresCoef(int nrr) { return (size_t)9 * nrr + 9; }
__host__ __device__ inline size_t kDivCoef(int nrr) { return kPresCoef(nrr) + (size_t)4 * nrr + 1; }
// and for the momentum right-hand sides of substep s, alre(s) dt times the
// radial coefficients of component c (0 = qt: ap1j, ac1j, am1j; 1 = qr:
// ap2je, ac2je, am2je; 2 = qz: ap3j, ac3j, am3j), coefficient e (0 = ap,
// 1 = ac, 2 = am):
// [ kImpCoef(nr+1) + ((s*3 + c)*3 + e)*(nr+1) + k ]
__host__ __device__ inline size_t kImpCoef(int nrr) { return kDivCoef(nrr) + (size_t)6 * nrr + 3; }
__host__ __device__ inline size_t kCorrCount(int nrr) { return kImpCoef(nrr) + (size_t)27 * nrr; }

// Factors of the row-scaled momentum matrices of one step: for each substep
// s (3), component c (0 = qt, 1 = qr, 2 = qz) and slip variant v (0 = no
// slip at the inner wall, 1 = free slip), arrays of length nr+1:
//   l    : multipliers of the LU factorisation (row k eliminates row k-1)
//   dinv : 1 / pivot
//   u    : super-diagonal
// plus per (s, c) the right-hand-side scale 1/(1 - ac(k) beta al) and, per s,
// the inner-wall forcing term of qt (SolveImpEqnUpdate_QT.F90:65-67).
template <typename T>
struct MomFactorsT {
    T* base;
    int stride;          // nr + 1
    __host__ __device__ T* l(int s, int c, int v) const { return base + ((((s * 3 + c) * 2 + v) * 4) + 0) * (size_t)stride; }
    __host__ __device__ T* dinv(int s, int c, int v) const { return base + ((((s * 3 + c) * 2 + v) * 4) + 1) * (size_t)stride; }
    __host__ __device__ T* u(int s, int c, int v) const { return base + ((((s * 3 + c) * 2 + v) * 4) + 2) * (size_t)stride; }
    __host__ __device__ T* scale(int s, int c) const { return base + ((((s * 3 + c) * 2 + 0) * 4) + 3) * (size_t)stride; }
    __host__ __device__ T* extra(int s) const { return base + (size_t)(3 * 3 * 2 * 4) * stride + s; }
    __host__ __device__ static size_t count(int stride) { return (size_t)(3 * 3 * 2 * 4) * stride + 8; }
};

}  // namespace tcgb
