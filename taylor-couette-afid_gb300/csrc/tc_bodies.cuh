// tc_bodies.cuh -- device bodies of the step kernels, written against
// explicit indices so that the single-instance kernels (tc_kernels.cu) and the
// grouped ensemble kernels (tc_batch.cu) run the same arithmetic.
//
// Velocity-side bodies are templates on the element type T: double gives the
// plain FP64 path, float the mixed path (velocities, explicit terms, momentum
// sweeps and FFTs in FP32; pressure tridiagonals, pressure accumulation and
// reductions in FP64).
#pragma once

#include <type_traits>

#include "tc_convert.cuh"
#include "tc_fft.cuh"
#include "tc_ff.cuh"
#include "tc_f32x2.cuh"
#include "tc_kernels.cuh"

namespace tcgb {

namespace {

constexpr int kRedThreads = 256;
constexpr int kRedBlocks = 1216;  // 8 x 152 SMs: enough resident warps to cover load latency
// Columns (kt) per z-FFT block of the ensemble kernels (128 threads).
template <typename T> struct ZCols { static constexpr int value = 4; };
// Columns and threads of the single-run z-FFT block.  Measured on the
// 512x512x128 grid: FP32 8 columns of 512 threads 0.106 ms a launch against
// 0.157 ms for 4 columns of 128 (4 x 256: 0.137, 8 x 1024: 0.125, 16 x 512:
// 0.153); FP64 is bound by the FP64 pipe and keeps 4 x 128 (8 columns:
// 1.16 ms against 0.99).
template <typename T> struct ZRun { static constexpr int cols = 4, threads = 128; };
template <> struct ZRun<float> { static constexpr int cols = 8, threads = 512; };


__device__ __forceinline__ int wm(int i, int n) { return i == 0 ? n - 1 : i - 1; }
__device__ __forceinline__ int wp(int i, int n) { return i == n - 1 ? 0 : i + 1; }
// Loads of fields and coefficients.  Kernels that run several dependent
// phases in one launch (tc_persist.cu) define TC_COHERENT_LOADS: their loads
// are then ordinary global loads, which the memory model orders after the
// grid barrier's fences; the read-only path (ld.global.nc) carries no such
// guarantee for lines another block rewrote earlier in the same launch.
#ifdef TC_COHERENT_LOADS
template <typename T> __device__ __forceinline__ T ld(const T* p) { return *p; }
#else
template <typename T> __device__ __forceinline__ T ld(const T* p) { return __ldg(p); }
#endif


// Stage a tile in shared memory: a[at(t)] = get(t) for t in [0, n), with U
// values (and their global loads) in flight per thread; a plain loop would
// wait for each load before issuing the next.
template <int U, typename C2, typename G, typename A>
__device__ __forceinline__ void stage_tile(C2* a, int n, G get, A at) {
    const int bd = blockDim.x;
    int t = threadIdx.x;
    for (; t + (U - 1) * bd < n; t += U * bd) {
        C2 v[U];
#pragma unroll
        for (int u = 0; u < U; ++u) v[u] = get(t + u * bd);
#pragma unroll
        for (int u = 0; u < U; ++u) a[at(t + u * bd)] = v[u];
    }
    for (; t < n; t += bd) a[at(t)] = get(t);
}

// L2 prefetch of the line holding p (a hint: no data returns, nothing waits)
__device__ __forceinline__ void prefetch_l2(const void* p) { asm volatile("prefetch.global.L2 [%0];" ::"l"(p)); }

// --------------------------------------------------------------------------
// Step control
// --------------------------------------------------------------------------

// mode 0: dt and time given by the host (tc_time_marcher / tc_begin_step).
// mode 1: main.F90:156-174 -- dt from the CFL number of the current field.
__device__ void begin_step_body(const Consts& k, StepState* st, int mode, double dt_h, double time_h) {
    double dt, time;
    if (mode == 0) {
        dt = dt_h;
        time = time_h;
        st->halt = 0;
        st->errorcode = 0;
    } else {
        if (st->halt) return;
        int err = 0;
        double cfl = st->instcfl;
        time = st->time;
        if (k.idtv == 1) {
            if (st->ntime > 1) {
                dt = (cfl < 1.0e-8) ? k.dtmax : k.limitCFL / cfl;
                if (dt > k.dtmax) dt = k.dtmax;
            } else {
                dt = k.dtmin;
            }
            if (dt < k.dtmin) err = 166;
        } else {
            // IDTV=0: the reference never assigns dt; run with dt = DTMAX.
            dt = k.dtmax;
            if (cfl * dt > k.limitCFL) err = 165;
        }
        st->errorcode = err;
    }
    st->dt = dt;
    st->time = time;
    st->beta = dt / k.ren * 0.5;                                                  // TimeMarcher.F90:20
    st->vinner_t = k.sizepert * sin(2.0 * k.pi * k.omegapert * time);             // InnerCylVelocity.F90:15
    st->dvinner_t = 2.0 * k.pi * k.omegapert * k.sizepert * cos(2.0 * k.pi * k.omegapert * time) * dt;
    st->dt_f = (float)dt;
    st->beta_f = (float)st->beta;
    st->vinner_f = (float)st->vinner_t;
}

// dt and vinner_t in the element type T (FP32 copies made once per step).
template <typename T> __device__ __forceinline__ T step_dt(const StepState* st);
template <> __device__ __forceinline__ double step_dt<double>(const StepState* st) { return st->dt; }
template <> __device__ __forceinline__ float step_dt<float>(const StepState* st) { return st->dt_f; }
template <typename T> __device__ __forceinline__ T step_vinner(const StepState* st);
template <> __device__ __forceinline__ double step_vinner<double>(const StepState* st) { return st->vinner_t; }
template <> __device__ __forceinline__ float step_vinner<float>(const StepState* st) { return st->vinner_f; }

// Row-scaled momentum matrices of SolveImpEqnUpdate_QT/QR/QZ and their LU
// factors for every substep of the step (dgttrf without row interchanges:
// the matrices are diagonally dominant), plus the per-substep correction
// coefficients of CorrectVelocity and the CalcLocalDivergence scale.  All in
// FP64 (Fd, corrd); for the mixed path the results are then rounded into the
// FP32 copies F, corr.  One block.
template <typename T>
__device__ void factors_body(const Dims& d, const Coef& c, const Consts& k, StepState* st,
                             const MomFactorsT<double>& Fd, double* corrd, double* scal, const MomFactorsT<T>& F,
                             T* corr) {
    const int nr = d.nr;
    const double beta = st->beta, dt = st->dt;
    const int nsub = k.nsst;
    if (st->dt_factored == dt) {
        // the factors, correction coefficients and scales depend on dt only:
        // keep them, and update the inner-wall term of this step
        // (SolveImpEqnUpdate_QT.F90:67), which follows dvinner_t
        if (threadIdx.x < nsub) {
            const int s = threadIdx.x;
            const double ex = 0.5 * k.alm[s] * dt * st->dvinner_t * c.am1j[0] / k.ren;
            *Fd.extra(s) = ex;
            if (!std::is_same<T, double>::value) *F.extra(s) = (T)ex;
        }
        return;
    }
    // phase 1: row entries (parallel over rows)
    for (int t = threadIdx.x; t < nsub * 5 * nr; t += blockDim.x) {
        int row = t % nr, chain = t / nr;        // chain: 0,1 = qt v0/v1; 2 = qr; 3,4 = qz v0/v1
        int s = chain / 5, ch = chain % 5;
        double betadx = beta * k.alm[s];
        if (ch == 0 || ch == 1 || ch == 3 || ch == 4) {
            bool qt = ch < 2;
            int v = (ch == 1 || ch == 4) ? 1 : 0;
            double fic = v == 0 ? 1.0 : 0.0, foc = 1.0;
            const double* ac = qt ? c.ac1j : c.ac3j;
            const double* am = qt ? c.am1j : c.am3j;
            const double* ap = qt ? c.ap1j : c.ap3j;
            double acfs0 = qt ? k.ac1j_fs0 : k.ac3j_fs0, acfs1 = qt ? k.ac1j_fs1 : k.ac3j_fs1;
            double acr = ac[row];
            if (row == 0) acr = ac[0] * fic + acfs0 * (1.0 - fic);
            else if (row == nr - 1) acr = ac[nr - 1] * foc + acfs1 * (1.0 - foc);
            double ackl_b = 1.0 / (1.0 - acr * betadx);
            int cidx = qt ? 0 : 2;
            Fd.l(s, cidx, v)[row] = row > 0 ? -am[row] * betadx * ackl_b : 0.0;        // amkl
            Fd.u(s, cidx, v)[row] = row < nr - 1 ? -ap[row] * betadx * ackl_b : 0.0;   // apkl
            if (v == 0) Fd.scale(s, cidx)[row] = 1.0 / (1.0 - ac[row] * betadx);
        } else {
            // qr faces 1..nr-1; rows 0 and nr are identity rows
            double ackl_b = (row >= 1) ? 1.0 / (1.0 - c.ac2j[row] * betadx) : 1.0;
            Fd.l(s, 1, 0)[row] = row >= 1 ? -c.am2j[row] * betadx * ackl_b : 0.0;
            Fd.u(s, 1, 0)[row] = row >= 1 ? -c.ap2j[row] * betadx * ackl_b : 0.0;
            Fd.scale(s, 1)[row] = ackl_b;
        }
        // CorrectVelocity.F90:35-40 coefficients
        if (ch == 0) {
            corrd[(s * 3 + 0) * (nr + 1) + row] = dt * k.alm[s] * k.dxt * c.usrm[row];
            corrd[(s * 3 + 1) * (nr + 1) + row] = dt * k.alm[s] * c.rudx2c[row];
            if (row == 0) {
                corrd[(s * 3 + 2) * (nr + 1)] = k.alm[s] * dt * k.dxz;
                // factors of the momentum right-hand side (TimeMarcher.F90 gam, rom, alre times dt)
                corrd[9 * (nr + 1) + s * 3 + 0] = k.gam[s] * dt;
                corrd[9 * (nr + 1) + s * 3 + 1] = k.rom[s] * dt;
                corrd[9 * (nr + 1) + s * 3 + 2] = k.alre[s] * dt;
            }
            if (s == 0) {
                // CorrectPressure coefficients of the step (one set for all substeps)
                double* pc = corrd + kPresCoef(nr + 1);
                const double u = c.udx1qm[row];
                pc[row] = beta * (2.0 * u + 2.0 * k.dxzq - c.acph[row]);
                pc[3 * (nr + 1) + 1 + row] = 1.0 + pc[row];
                pc[(nr + 1) + row] = -beta * u;
                pc[2 * (nr + 1) + row] = -beta * c.apph[row];
                if (row == 0) pc[3 * (nr + 1)] = -beta * k.dxzq;
            }
            {
                // divergence coefficients of substep s (usdt and the FFT
                // normalisation folded in)
                double* dc = corrd + kDivCoef(nr + 1);
                const double sc = k.fft_norm / (k.alm[s] * dt);
                const double us = c.usrm[row] * sc;
                dc[s * 2 * (nr + 1) + row] = k.dxt * us;
                dc[s * 2 * (nr + 1) + (nr + 1) + row] = c.udx2m[row] * us;
                if (row == 0) dc[6 * (nr + 1) + s] = k.dxz * sc;
            }
            {
                // alre dt times the radial coefficients of the momentum rhs
                double* ic = corrd + kImpCoef(nr + 1) + (size_t)s * 9 * (nr + 1);
                const double ad = k.alre[s] * dt;
                const double* src[9] = {c.ap1j, c.ac1j, c.am1j, c.ap2je, c.ac2je, c.am2je, c.ap3j, c.ac3j, c.am3j};
#pragma unroll
                for (int e = 0; e < 9; ++e) ic[e * (nr + 1) + row] = ad * src[e][row];
            }
        }
    }
    __syncthreads();
    // phase 2: sequential elimination, one thread per chain
    if (threadIdx.x < nsub * 5) {
        int s = threadIdx.x / 5, ch = threadIdx.x % 5;
        int cidx = ch < 2 ? 0 : (ch == 2 ? 1 : 2);
        int v = (ch == 1 || ch == 4) ? 1 : 0;
        double* l = Fd.l(s, cidx, v);
        double* u = Fd.u(s, cidx, v);
        double* di = Fd.dinv(s, cidx, v);
        int k0 = (cidx == 1) ? 1 : 0;
        double dp = 1.0;
        di[k0] = 1.0;
        if (cidx == 1) l[1] = 0.0;   // couples to the wall value qr(1) = 0
        for (int row = k0 + 1; row < nr; ++row) {
            const double fact = l[row] / dp;
            l[row] = fact;
            dp = 1.0 - fact * u[row - 1];
            di[row] = dp;
        }
    } else if (threadIdx.x >= 32 && threadIdx.x < 32 + nsub) {
        int s = threadIdx.x - 32;
        // SolveImpEqnUpdate_QT.F90:67
        *Fd.extra(s) = 0.5 * k.alm[s] * dt * st->dvinner_t * c.am1j[0] / k.ren;
        // CalcLocalDivergence.F90:19 usdt, alone and times the FFT normalisation
        const double usdt = 1.0 / (k.alm[s] * dt);
        scal[s] = usdt * k.fft_norm;
        scal[3 + s] = usdt;
    }
    __syncthreads();
    // phase 3: reciprocals of the pivots
    for (int t = threadIdx.x; t < nsub * 5 * nr; t += blockDim.x) {
        int row = t % nr, chain = t / nr;
        int s = chain / 5, ch = chain % 5;
        int cidx = ch < 2 ? 0 : (ch == 2 ? 1 : 2);
        int v = (ch == 1 || ch == 4) ? 1 : 0;
        if (cidx == 1 && row == 0) continue;
        double* di = Fd.dinv(s, cidx, v);
        di[row] = 1.0 / di[row];
    }
    __syncthreads();
    // phase 3b: fold the row scales sc into the factors, so that the sweeps
    // solve for y'_k = y_k / sc_k: y'_k = rhs_k - l'_k y'_k-1 and
    // x_k = (y'_k - u'_k x_k+1) di'_k with l'_k = l_k sc_k-1 / sc_k,
    // u'_k = u_k / sc_k, di'_k = di_k sc_k (one multiplication a level less)
    for (int t = threadIdx.x; t < nsub * 5 * nr; t += blockDim.x) {
        int row = t % nr, chain = t / nr;
        int s = chain / 5, ch = chain % 5;
        int cidx = ch < 2 ? 0 : (ch == 2 ? 1 : 2);
        int v = (ch == 1 || ch == 4) ? 1 : 0;
        const int k0 = (cidx == 1) ? 1 : 0;
        if (row < k0) continue;
        const double* sc = Fd.scale(s, cidx);
        const double scr = sc[row];
        double* l = Fd.l(s, cidx, v);
        if (row > k0) l[row] = l[row] * sc[row - 1] / scr;
        Fd.u(s, cidx, v)[row] = Fd.u(s, cidx, v)[row] / scr;
        Fd.dinv(s, cidx, v)[row] = Fd.dinv(s, cidx, v)[row] * scr;
    }
    // phase 4 (mixed path): round the factors into the FP32 copies
    if (!std::is_same<T, double>::value) {
        __syncthreads();
        const int nF = (int)MomFactorsT<T>::count(F.stride), nC = (int)kCorrCount(nr + 1);
        for (int t = threadIdx.x; t < nF; t += blockDim.x) F.base[t] = (T)Fd.base[t];
        for (int t = threadIdx.x; t < nC; t += blockDim.x) corr[t] = (T)corrd[t];
    }
    __syncthreads();
    if (threadIdx.x == 0) st->dt_factored = dt;
}

// Neighbour offsets of cell (i, j, k) relative to its own index o, in
// elements (32-bit): the periodic wraps in theta and z are folded into dim,
// dip, djm, djp; radial neighbours are +-P.  Loads then cost one address add
// each instead of a 64-bit index product.
struct Stencil {
    size_t o;
    int dim, dip, djm, djp, P;
    int k, kmm, kpp;          // radial index and its clamped neighbours (kmv/kpv)
};

__device__ __forceinline__ Stencil make_stencil(const Dims& d, int i, int j, int k) {
    Stencil S;
    const int nt = d.nt, nz = d.nz;
    S.P = (int)d.P;
    S.o = (size_t)k * (size_t)d.P + (size_t)j * nt + i;
    S.dim = i == 0 ? nt - 1 : -1;
    S.dip = i == nt - 1 ? 1 - nt : 1;
    S.djm = j == 0 ? (nz - 1) * nt : -nt;
    S.djp = j == nz - 1 ? -(nz - 1) * nt : nt;
    S.k = k;
    S.kmm = k > 0 ? k - 1 : 0;
    S.kpp = k < d.nr - 1 ? k + 1 : d.nr - 1;
    return S;
}

// Scalars of the momentum kernel in the element type T.
template <typename T>
struct MomArgs {
    const T *qt, *qr, *qz;
    const T* pr;            // pressure in the element type (FP32 copy on the mixed path)
    T *ru1, *ru2, *ru3, *rhs_t, *rhs_r, *rhs_z, *h_t, *h_r, *h_z;
    const signed char* icyl;
    const StepState* st;
    T al, ga, ro, alre, dxt_al, dxz_al;
    T udxz, udxzq, q_romeg, virotint, virotext;
    T ac1j_fs0, am1j_fs0, ap1j_fs1, ac1j_fs1, ac3j_fs0, am3j_fs0, ap3j_fs1, ac3j_fs1;
    const T* cf;            // this substep's pressure-gradient products dt al metric (per component, level)
    const T* mr;            // gam dt, rom dt, alre dt of this substep
    const T* ic;            // alre dt times the radial coefficients of this substep (9 arrays)
    int use_ru;
};

// ExplicitTermsQT.F90:40-125 at cell (i, j, k); qt, qr, qz point at the cell.
template <typename T>
__device__ T explicit_qt(const Stencil& S, const CoefT<T>& c, const MomArgs<T>& A, const T* qt, const T* qr,
                         const T* qz) {
    const int k = S.k, kp = k + 1, P = S.P;
    T t_c = ld(qt), t_ip = ld(qt + S.dip), t_im = ld(qt + S.dim);
    T t_jp = ld(qt + S.djp), t_jm = ld(qt + S.djm);
    T t_kp = ld(qt + (S.kpp - k) * P), t_km = ld(qt + (S.kmm - k) * P);
    T r_c = ld(qr), r_im = ld(qr + S.dim);
    T r_p = ld(qr + P), r_pim = ld(qr + P + S.dim);
    T z_c = ld(qz), z_im = ld(qz + S.dim);
    T z_jp = ld(qz + S.djp), z_jpim = ld(qz + S.djp + S.dim);
    const T udxt = ld(c.udxt_m + k), udxtq = ld(c.udxtq_m + k);
    const T usrc = ld(c.usrc + k), usrcp = ld(c.usrc + kp);
    const T two = (T)2.0;
    T h11 = ((t_ip + t_c) * (t_ip + t_c) - (t_c + t_im) * (t_c + t_im)) * udxt;
    const T rp2 = r_p + r_pim, rc2 = r_c + r_im;
    T h12d = (rp2 * (t_kp + t_c) - rc2 * (t_c + t_km)) * ld(c.q_udx2rm + k);
    const T qrs = rp2 * usrcp + rc2 * usrc;          // shared by h12n and the Coriolis term
    T h12n = t_c * ld(c.q_usrm + k) * qrs;
    T h13 = ((z_jp + z_jpim) * (t_jp + t_c) - (z_c + z_im) * (t_c + t_jm)) * A.udxz;
    T d11qt = (t_ip - two * t_c + t_im) * udxtq;
    T d22qt = (t_jp - two * t_c + t_jm) * A.udxzq;
    T qre = r_p * usrcp + r_c * usrc;
    T qrw = r_pim * usrcp + r_im * usrc;
    T d11qre = (qre - qrw) * ld(c.h_udx1vis1 + k);
    T coriol = -qrs * A.q_romeg;
    return -(h11 + (h12d + h12n) + h13) + d11qre + d22qt + d11qt + coriol;
}

// ExplicitTermsQR.F90:46-146 at face (i, j, k), 1 <= k <= nr-1
template <typename T>
__device__ T explicit_qr(const Stencil& S, const CoefT<T>& c, const MomArgs<T>& A, const T* qt, const T* qr,
                         const T* qz) {
    const int k = S.k, km = k - 1, kp = k + 1, P = S.P;
    T t_c = ld(qt), t_m = ld(qt - P);
    T t_ip = ld(qt + S.dip), t_mip = ld(qt - P + S.dip);
    T r_c = ld(qr), r_ip = ld(qr + S.dip), r_im = ld(qr + S.dim);
    T r_jp = ld(qr + S.djp), r_jm = ld(qr + S.djm);
    T r_p = ld(qr + P), r_m = ld(qr - P);
    T z_jp = ld(qz + S.djp), z_mjp = ld(qz - P + S.djp);
    T z_c = ld(qz), z_m = ld(qz - P);
    const T udxt = ld(c.udxt_c + k), udxtq = ld(c.udxtq_c + k);
    const T usrc = ld(c.usrc + k), usrcp = ld(c.usrc + kp), usrcm = ld(c.usrc + km);
    const T two = (T)2.0;
    // theta-velocity sums of the two faces, shared by h11n, h21, d11qre and Coriolis
    const T sa = t_ip + t_mip, sb = t_c + t_m, s4 = sa + sb;
    T a = s4 * (T)0.25;
    T h11n = a * a;
    T h21 = (sa * (r_ip + r_c) - sb * (r_c + r_im)) * udxt;
    T h22 = ((r_p * usrcp + r_c * usrc) * (r_p + r_c) - (r_c * usrc + r_m * usrcm) * (r_c + r_m)) * ld(c.q_udx2c + k);
    T h23 = ((z_jp + z_mjp) * (r_jp + r_c) - (z_c + z_m) * (r_c + r_jm)) * A.udxz;
    T d11qre = -(sa - sb) * ld(c.udx1vis2 + k);
    T d11qr = (r_ip - two * r_c + r_im) * udxtq;
    T d22qr = (r_jp - two * r_c + r_jm) * A.udxzq;
    T coriol = s4 * ld(c.q_rc_romeg + k);
    return -(h21 + h22 + h23) + h11n + d11qr + d22qr + d11qre + coriol;
}

// ExplicitTermsQZ.F90:40-102 at cell (i, j, k)
template <typename T>
__device__ T explicit_qz(const Stencil& S, const CoefT<T>& c, const MomArgs<T>& A, const T* qt, const T* qr,
                         const T* qz) {
    const int k = S.k, P = S.P;
    T t_c = ld(qt), t_ip = ld(qt + S.dip);
    T t_jm = ld(qt + S.djm), t_jmip = ld(qt + S.djm + S.dip);
    T z_c = ld(qz), z_ip = ld(qz + S.dip), z_im = ld(qz + S.dim);
    T z_jp = ld(qz + S.djp), z_jm = ld(qz + S.djm);
    T z_kp = ld(qz + (S.kpp - k) * P), z_km = ld(qz + (S.kmm - k) * P);
    T r_p = ld(qr + P), r_pjm = ld(qr + P + S.djm);
    T r_c = ld(qr), r_jm = ld(qr + S.djm);
    const T udxt = ld(c.udxt_m + k), udxtq = ld(c.udxtq_m + k);
    const T two = (T)2.0;
    // second product written as in explicit_qt's h13, so the two share it
    T h31 = ((t_ip + t_jmip) * (z_ip + z_c) - (z_c + z_im) * (t_c + t_jm)) * udxt;
    T h32 = ((r_p + r_pjm) * (z_kp + z_c) - (r_c + r_jm) * (z_c + z_km)) * ld(c.q_udx2rm + k);
    T h33 = ((z_jp + z_c) * (z_jp + z_c) - (z_c + z_jm) * (z_c + z_jm)) * A.udxz;
    T dqz1 = (z_im - two * z_c + z_ip) * udxtq;
    T dqz2 = (z_jm - two * z_c + z_jp) * A.udxzq;
    return -(h31 + h32 + h33) + dqz1 + dqz2;
}

// ImplicitAndUpdateQT/QR/QZ for cell (i, j, k) of stencil S given its
// explicit terms: the right-hand sides and the RK memory.  RU: whether the
// substep reads the RK memory (rom != 0), at compile time (0, 1) or read from
// a.use_ru (-1).  Interior levels take alre dt times the radial coefficients
// from a.ic; the wall levels form their coefficients here, as the reference.
// mask selects the components (1 qt, 2 qr, 4 qz; the per-routine entry
// points run one at a time, the fused kernels all three).
template <typename T, int RU = -1>
__device__ __forceinline__ void implicit_cell(const Dims& d, const CoefT<T>& c, const MomArgs<T>& a, const Stencil& S,
                                              int i, int j, int k, T ht, T hr, T hz, int mask = 7) {
    const int nr = d.nr;
    const size_t o = S.o;
    const int P = S.P;
    const T* qt = a.qt + o;
    const T* qr = a.qr + o;
    const T* qz = a.qz + o;
    // gam dt, rom dt, alre dt; the pressure terms use the per-level dt al
    // metric products of the correction (a.cf), so no factor dt remains
    const T gadt = ld(a.mr), rodt = ld(a.mr + 1), alredt = ld(a.mr + 2);
    const bool use_ru = RU < 0 ? (a.use_ru != 0) : (RU != 0);
    const int nrr = nr + 1;
    const T* ic = a.ic;
    const T one = (T)1.0;
    const T fic = a.icyl ? (T)a.icyl[(size_t)j * d.nt + i] : one, foc = one;
    const T* pr = a.pr + o;
    const T p_c = ld(pr);
    // ---- qt (ImplicitAndUpdateQT.F90:45-115)
    if (mask & 1) {
        T rhs = gadt * ht;
        if (use_ru) rhs += rodt * a.ru1[o];
        if (k == 0) {
            T app = ld(c.ap1j);
            T acc = ld(c.ac1j) * fic + a.ac1j_fs0 * (one - fic);
            T amm = ld(c.am1j) * fic + a.am1j_fs0 * (one - fic);
            rhs += alredt * (ld(qt + P) * app + ld(qt) * acc + (a.virotint + step_vinner<T>(a.st)) * amm);
        } else if (k == nr - 1) {
            T amm = ld(c.am1j + k);
            T app = ld(c.ap1j + k) * foc + a.ap1j_fs1 * (one - foc);
            T acc = ld(c.ac1j + k) * foc + a.ac1j_fs1 * (one - foc);
            rhs += alredt * (a.virotext * app + ld(qt) * acc + ld(qt - P) * amm);
        } else {
            rhs += ld(ic + k) * ld(qt + P);
            rhs += ld(ic + nrr + k) * ld(qt);
            rhs += ld(ic + 2 * nrr + k) * ld(qt - P);
        }
        a.rhs_t[o] = rhs - (p_c - ld(pr + S.dim)) * ld(a.cf + k);
        a.ru1[o] = ht;
    }
    // ---- qr (ImplicitAndUpdateQR.F90:41-63), faces 1..nr-1
    if ((mask & 2) && k >= 1) {
        T rhs = gadt * hr;
        if (use_ru) rhs += rodt * a.ru2[o];
        rhs += ld(ic + 3 * nrr + k) * ld(qr + P);
        rhs += ld(ic + 4 * nrr + k) * ld(qr);
        rhs += ld(ic + 5 * nrr + k) * ld(qr - P);
        a.rhs_r[o] = rhs - (p_c - ld(pr - P)) * ld(a.cf + nrr + k);
        a.ru2[o] = hr;
    }
    // ---- qz (ImplicitAndUpdateQZ.F90:42-113)
    if (mask & 4) {
        T rhs = gadt * hz;
        // At the outer wall the reference has already replaced ru3(nrm) by
        // qcap(nrm) when it builds rhs(nrm) (ImplicitAndUpdateQZ.F90:86,110).
        if (k == nr - 1) rhs += rodt * hz;
        else if (use_ru) rhs += rodt * a.ru3[o];
        if (k == 0) {
            T app = ld(c.ap3j);
            T acc = ld(c.ac3j) * fic + a.ac3j_fs0 * (one - fic);
            T amm = ld(c.am3j) * fic + a.am3j_fs0 * (one - fic);
            T q0 = ld(qz);
            rhs += alredt * (ld(qz + P) * app + q0 * acc + q0 * amm);
        } else if (k == nr - 1) {
            T app = ld(c.ap3j + k) * foc + a.ap3j_fs1 * (one - foc);
            T acc = ld(c.ac3j + k) * foc + a.ac3j_fs1 * (one - foc);
            T q0 = ld(qz);
            rhs += alredt * (q0 * app + q0 * acc + ld(qz - P) * ld(c.am3j + k));
        } else {
            rhs += ld(ic + 6 * nrr + k) * ld(qz + P);
            rhs += ld(ic + 7 * nrr + k) * ld(qz);
            rhs += ld(ic + 8 * nrr + k) * ld(qz - P);
        }
        a.rhs_z[o] = rhs - (p_c - ld(pr + S.djm)) * ld(a.cf + 2 * nrr);
        a.ru3[o] = hz;
    }
}

// mask: components to compute (1 qt, 2 qr, 4 qz), as implicit_cell.
template <int MODE, typename T>
__device__ __forceinline__ void momentum_cell(const Dims& d, const CoefT<T>& c, const MomArgs<T>& a, int i, int j,
                                              int k, int mask = 7) {
    const Stencil S = make_stencil(d, i, j, k);
    const size_t o = S.o;
    const T* qt = a.qt + o;
    const T* qr = a.qr + o;
    const T* qz = a.qz + o;
    T ht = 0, hr = 0, hz = 0;
    if (MODE != MODE_IMPLICIT) {
        if (mask & 1) ht = explicit_qt(S, c, a, qt, qr, qz);
        if ((mask & 2) && k >= 1) hr = explicit_qr(S, c, a, qt, qr, qz);
        if (mask & 4) hz = explicit_qz(S, c, a, qt, qr, qz);
        if (MODE == MODE_EXPLICIT) {
            if (mask & 1) a.h_t[o] = ht;
            if ((mask & 2) && k >= 1) a.h_r[o] = hr;
            if (mask & 4) a.h_z[o] = hz;
            return;
        }
    } else {
        if (mask & 1) ht = a.h_t[o];
        if ((mask & 2) && k >= 1) hr = a.h_r[o];
        if (mask & 4) hz = a.h_z[o];
    }
    implicit_cell(d, c, a, S, i, j, k, ht, hr, hz, mask);
}

// The fused momentum work of momentum_cell (MODE_FUSED) for the two cells
// (i, j, k) and (i+1, j, k), i even: the sums and products through the
// theta face between them are formed once (h11 of qt, h31 of qz, h21 of qr,
// the qr interpolation qre = qrw of d11qre), and within each cell the
// products the radial and z terms share (h12d and h21; h23 and h32) are
// formed once.  The FP64 path is bound by the FP64 pipe, so each shared
// product or sum is a cycle saved.  Term by term the arithmetic is that of
// explicit_qt/qr/qz; only the rounding order of a few sums differs.  RU as
// for implicit_cell.
template <typename T, int RU = -1>
__device__ __forceinline__ void momentum_pair(const Dims& d, const CoefT<T>& c, const MomArgs<T>& a, int i, int j,
                                              int k) {
    const Stencil Sa = make_stencil(d, i, j, k), Sb = make_stencil(d, i + 1, j, k);
    const int P = Sa.P;
    const T* qt = a.qt + Sa.o;
    const T* qr = a.qr + Sa.o;
    const T* qz = a.qz + Sa.o;
    const int dimA = Sa.dim;                     // theta- of cell a (wraps at i = 0)
    const int dipB = 1 + Sb.dip;                 // theta+ of cell b, from cell a (wraps at i + 1 = nt - 1)
    const int djp = Sa.djp, djm = Sa.djm;
    const int kP = (Sa.kpp - k) * P, kM = (Sa.kmm - k) * P;
    const T two = (T)2.0;
    // level k and the clamped radial neighbours
    const T ta = ld(qt), tb = ld(qt + 1), tam = ld(qt + dimA), tbp = ld(qt + dipB);
    const T ta_jp = ld(qt + djp), tb_jp = ld(qt + djp + 1), ta_jm = ld(qt + djm), tb_jm = ld(qt + djm + 1);
    const T tbp_jm = ld(qt + djm + dipB);
    const T ta_kp = ld(qt + kP), tb_kp = ld(qt + kP + 1), ta_km = ld(qt + kM), tb_km = ld(qt + kM + 1);
    const T ra = ld(qr), rb = ld(qr + 1), ram = ld(qr + dimA);
    const T ra_p = ld(qr + P), rb_p = ld(qr + P + 1), ram_p = ld(qr + P + dimA);
    const T ra_jm = ld(qr + djm), rb_jm = ld(qr + djm + 1);
    const T ra_pjm = ld(qr + P + djm), rb_pjm = ld(qr + P + djm + 1);
    const T za = ld(qz), zb = ld(qz + 1), zam = ld(qz + dimA), zbp = ld(qz + dipB);
    const T za_jp = ld(qz + djp), zb_jp = ld(qz + djp + 1), za_jm = ld(qz + djm), zb_jm = ld(qz + djm + 1);
    const T zam_jp = ld(qz + djp + dimA);
    const T za_kp = ld(qz + kP), zb_kp = ld(qz + kP + 1), za_km = ld(qz + kM), zb_km = ld(qz + kM + 1);
    const T usrc = ld(c.usrc + k), usrcp = ld(c.usrc + k + 1);
    // shared products
    const T Sab = tb + ta, Sab2 = Sab * Sab;                 // theta face a|b of h11
    const T rc2a = ra + ram, rp2a = ra_p + ram_p, rc2b = rb + ra, rp2b = rb_p + ra_p;
    const T Xa = rc2a * (ta + ta_km);                         // lower radial face of h12d (a); h21 of a for k >= 1
    const T Xb = rc2b * (tb + tb_km);                         // the same for b; = theta face a|b of h21 for k >= 1
    const T x13a = (za + zam) * (ta + ta_jm);                 // second products of h13 (and h31)
    const T x13b = (zb + za) * (tb + tb_jm);                  // = theta face a|b of h31
    const T qrea = ra_p * usrcp + ra * usrc;                  // = qrw of b
    const T qreb = rb_p * usrcp + rb * usrc;
    const T qrwa = ram_p * usrcp + ram * usrc;
    const T Ya = (ra + ra_jm) * (za + za_km);                 // lower radial face of h32 (a); h23 of a for k >= 1
    const T Yb = (rb + rb_jm) * (zb + zb_km);
    T ht[2], hr[2] = {(T)0, (T)0}, hz[2];
    // ---- ExplicitTermsQT
    {
        const T udxt = ld(c.udxt_m + k), udxtq = ld(c.udxtq_m + k);
        const T q2rm = ld(c.q_udx2rm + k), qusrm = ld(c.q_usrm + k), hv1 = ld(c.h_udx1vis1 + k);
        {
            const T B = ta + tam;
            const T h11 = (Sab2 - B * B) * udxt;
            const T h12d = (rp2a * (ta_kp + ta) - Xa) * q2rm;
            const T qrs = rp2a * usrcp + rc2a * usrc;
            const T h12n = ta * qusrm * qrs;
            const T h13 = ((za_jp + zam_jp) * (ta_jp + ta) - x13a) * a.udxz;
            const T d11qt = (tb - two * ta + tam) * udxtq;
            const T d22qt = (ta_jp - two * ta + ta_jm) * a.udxzq;
            const T d11qre = (qrea - qrwa) * hv1;
            const T coriol = -qrs * a.q_romeg;
            ht[0] = -(h11 + (h12d + h12n) + h13) + d11qre + d22qt + d11qt + coriol;
        }
        {
            const T A = tbp + tb;
            const T h11 = (A * A - Sab2) * udxt;
            const T h12d = (rp2b * (tb_kp + tb) - Xb) * q2rm;
            const T qrs = rp2b * usrcp + rc2b * usrc;
            const T h12n = tb * qusrm * qrs;
            const T h13 = ((zb_jp + za_jp) * (tb_jp + tb) - x13b) * a.udxz;
            const T d11qt = (tbp - two * tb + ta) * udxtq;
            const T d22qt = (tb_jp - two * tb + tb_jm) * a.udxzq;
            const T d11qre = (qreb - qrea) * hv1;
            const T coriol = -qrs * a.q_romeg;
            ht[1] = -(h11 + (h12d + h12n) + h13) + d11qre + d22qt + d11qt + coriol;
        }
    }
    // ---- ExplicitTermsQR at faces k >= 1 (kM = -P there)
    if (k >= 1) {
        const T rbp = ld(qr + dipB), ra_jp = ld(qr + djp), rb_jp = ld(qr + djp + 1);
        const T ra_m = ld(qr - P), rb_m = ld(qr - P + 1);
        const T tbp_m = ld(qt - P + dipB);
        const T za_mjp = ld(qz - P + djp), zb_mjp = ld(qz - P + djp + 1);
        const T udxt = ld(c.udxt_c + k), udxtq = ld(c.udxtq_c + k), usrcm = ld(c.usrc + k - 1);
        const T q2c = ld(c.q_udx2c + k), v2 = ld(c.udx1vis2 + k), qrc = ld(c.q_rc_romeg + k);
        const T sa0 = tb + tb_km, sb0 = ta + ta_km;           // cell a; sb of b = sa0
        {
            const T s4 = sa0 + sb0, aa = s4 * (T)0.25;
            const T h11n = aa * aa;
            const T h21 = (Xb - Xa) * udxt;
            const T h22 = (qrea * (ra_p + ra) - (ra * usrc + ra_m * usrcm) * (ra + ra_m)) * q2c;
            const T h23 = ((za_jp + za_mjp) * (ra_jp + ra) - Ya) * a.udxz;
            const T d11qre = -(sa0 - sb0) * v2;
            const T d11qr = (rb - two * ra + ram) * udxtq;
            const T d22qr = (ra_jp - two * ra + ra_jm) * a.udxzq;
            const T coriol = s4 * qrc;
            hr[0] = -(h21 + h22 + h23) + h11n + d11qr + d22qr + d11qre + coriol;
        }
        {
            const T sa1 = tbp + tbp_m;
            const T s4 = sa1 + sa0, aa = s4 * (T)0.25;
            const T h11n = aa * aa;
            const T h21 = (sa1 * (rbp + rb) - Xb) * udxt;
            const T h22 = (qreb * (rb_p + rb) - (rb * usrc + rb_m * usrcm) * (rb + rb_m)) * q2c;
            const T h23 = ((zb_jp + zb_mjp) * (rb_jp + rb) - Yb) * a.udxz;
            const T d11qre = -(sa1 - sa0) * v2;
            const T d11qr = (rbp - two * rb + ra) * udxtq;
            const T d22qr = (rb_jp - two * rb + rb_jm) * a.udxzq;
            const T coriol = s4 * qrc;
            hr[1] = -(h21 + h22 + h23) + h11n + d11qr + d22qr + d11qre + coriol;
        }
    }
    // ---- ExplicitTermsQZ
    {
        const T udxt = ld(c.udxt_m + k), udxtq = ld(c.udxtq_m + k), q2rm = ld(c.q_udx2rm + k);
        {
            const T h31 = (x13b - x13a) * udxt;
            const T h32 = ((ra_p + ra_pjm) * (za_kp + za) - Ya) * q2rm;
            const T h33 = ((za_jp + za) * (za_jp + za) - (za + za_jm) * (za + za_jm)) * a.udxz;
            const T dqz1 = (zam - two * za + zb) * udxtq;
            const T dqz2 = (za_jm - two * za + za_jp) * a.udxzq;
            hz[0] = -(h31 + h32 + h33) + dqz1 + dqz2;
        }
        {
            const T h31 = ((tbp + tbp_jm) * (zbp + zb) - x13b) * udxt;
            const T h32 = ((rb_p + rb_pjm) * (zb_kp + zb) - Yb) * q2rm;
            const T h33 = ((zb_jp + zb) * (zb_jp + zb) - (zb + zb_jm) * (zb + zb_jm)) * a.udxz;
            const T dqz1 = (za - two * zb + zbp) * udxtq;
            const T dqz2 = (zb_jm - two * zb + zb_jp) * a.udxzq;
            hz[1] = -(h31 + h32 + h33) + dqz1 + dqz2;
        }
    }
    implicit_cell<T, RU>(d, c, a, Sa, i, j, k, ht[0], hr[0], hz[0]);
    implicit_cell<T, RU>(d, c, a, Sb, i + 1, j, k, ht[1], hr[1], hz[1]);
}

// The fused momentum work (explicit terms and implicit right-hand sides of
// all three components, as momentum_cell with MODE_FUSED) of the levels
// k0 <= k < k1 of the two theta-neighbouring columns (i, j) and (i+1, j),
// i even, marching outwards in r (see kMomChunk below), in packed FP32
// (tc_f32x2.cuh): every F2 holds cell i in its first lane and cell i+1 in
// its second, so one packed instruction does the arithmetic of both cells;
// centre values load as float2, and the theta neighbours are the other lane
// of the pair plus one scalar load each side.  The terms are those of
// explicit_qt/qr/qz and implicit_cell with the multiply-adds written out:
// (A^2 - B^2) of h11 and h33 as (A - B)(A + B).  FP32 mixed path only.
__device__ __forceinline__ F2 ld_f2(const float* p) {
    const float2 v = ld(reinterpret_cast<const float2*>(p));
    return mkf2(v.x, v.y);
}
// arrays the kernel also writes (ordinary loads)
__device__ __forceinline__ F2 ldp_f2(const float* p) {
    const float2 v = *reinterpret_cast<const float2*>(p);
    return mkf2(v.x, v.y);
}

// Levels ahead of the march whose entries are prefetched into L2.  On the
// 512x512x128 grid (mixed, one launch, mean over the substeps): none
// 0.486 ms, 1 level 0.404 ms, 2 levels 0.383 ms, 3 levels 0.387 ms.
constexpr int kMomPrefetch = 2;

// Values the march reads at level k: the pair (i, i+1) and its theta, z
// neighbours at level k, the pair at level k+1 (suffix p), the RK memory.
struct MarchIn {
    F2 tip, tim, tjp, tjm, tjmip, tp;
    F2 rip, rjp, rp, rpim, rpjm;
    F2 zip, zim, zjp, zjm, zjpim, zp;
    F2 pc, pjm, pim;
    F2 old_t, old_r, old_z;
};

// Values carried from level k-1 to level k: the pair at levels k (c) and
// k-1 (m), the neighbours of level k-1 the next level still needs, and the
// radial fluxes through the face between the two levels.
struct MarchCarry {
    F2 tc, tm, tmip, rc, rim, rjm, rm, zc, zm, zmjp, prm;
    F2 U12, Uz, Gup;
};

// Per-thread constants of the march.
struct MarchK {
    F2 TWO, MTWO, QUARTER, ZERO, GADT, RODT, ALREDT, FIC, UDXZ, UDXZQ, NQROMEG, NCFZ;
};

__device__ __forceinline__ MarchK march_consts(const Dims& d, const MomArgs<float>& a, size_t col) {
    MarchK K;
    K.TWO = bc2(2.0f); K.MTWO = bc2(-2.0f); K.QUARTER = bc2(0.25f); K.ZERO = bc2(0.0f);
    K.GADT = bc2(ld(a.mr)); K.RODT = bc2(ld(a.mr + 1)); K.ALREDT = bc2(ld(a.mr + 2));
    K.FIC = a.icyl ? mkf2((float)a.icyl[col], (float)a.icyl[col + 1]) : bc2(1.0f);
    K.UDXZ = bc2(a.udxz); K.UDXZQ = bc2(a.udxzq); K.NQROMEG = bc2(-a.q_romeg);
    K.NCFZ = bc2(-ld(a.cf + 2 * (d.nr + 1)));
    return K;
}

// The coefficients march_level reads at level k (the grid metrics of
// CreateGrid.F90 in FP32, and the substep's pressure-gradient products),
// gathered so that a kernel can stage a chunk's table in shared memory.
struct alignas(16) MarchCoef {
    float usrc, usrcp, udxt_m, udxtq_m, q_usrm, q_udx2rm, h_udx1vis1, udxt_c;
    float udxtq_c, q_udx2c, udx1vis2, q_rc_romeg, ap1j, ac1j, am1j, ap2je;
    float ac2je, am2je, ap3j, ac3j, am3j, cf_t, cf_r, pad;
};
constexpr int kMarchCoefN = 24;   // floats of a MarchCoef

// Coefficient q (MarchCoef order) of level k, from global memory.
__device__ __forceinline__ float march_coef_entry(const CoefT<float>& c, const MomArgs<float>& a, int nrr, int k,
                                                  int q) {
    switch (q) {
        case 0: return ld(c.usrc + k);
        case 1: return ld(c.usrc + k + 1);
        case 2: return ld(c.udxt_m + k);
        case 3: return ld(c.udxtq_m + k);
        case 4: return ld(c.q_usrm + k);
        case 5: return ld(c.q_udx2rm + k);
        case 6: return ld(c.h_udx1vis1 + k);
        case 7: return ld(c.udxt_c + k);
        case 8: return ld(c.udxtq_c + k);
        case 9: return ld(c.q_udx2c + k);
        case 10: return ld(c.udx1vis2 + k);
        case 11: return ld(c.q_rc_romeg + k);
        case 12: return ld(c.ap1j + k);
        case 13: return ld(c.ac1j + k);
        case 14: return ld(c.am1j + k);
        case 15: return ld(c.ap2je + k);
        case 16: return ld(c.ac2je + k);
        case 17: return ld(c.am2je + k);
        case 18: return ld(c.ap3j + k);
        case 19: return ld(c.ac3j + k);
        case 20: return ld(c.am3j + k);
        case 21: return ld(a.cf + k);
        case 22: return ld(a.cf + nrr + k);
        default: return 0.0f;
    }
}

// Sources of march_level's coefficients: read from global memory where they
// are used (the cached march; loading them all up front would cost
// registers), or from a MarchCoef record (the TMA march's shared table).
struct MarchCoefGlobal {
    const CoefT<float>& c;
    const MomArgs<float>& a;
    int nrr, k;
    __device__ __forceinline__ float usrc() const { return ld(c.usrc + k); }
    __device__ __forceinline__ float usrcp() const { return ld(c.usrc + k + 1); }
    __device__ __forceinline__ float udxt_m() const { return ld(c.udxt_m + k); }
    __device__ __forceinline__ float udxtq_m() const { return ld(c.udxtq_m + k); }
    __device__ __forceinline__ float q_usrm() const { return ld(c.q_usrm + k); }
    __device__ __forceinline__ float q_udx2rm() const { return ld(c.q_udx2rm + k); }
    __device__ __forceinline__ float h_udx1vis1() const { return ld(c.h_udx1vis1 + k); }
    __device__ __forceinline__ float udxt_c() const { return ld(c.udxt_c + k); }
    __device__ __forceinline__ float udxtq_c() const { return ld(c.udxtq_c + k); }
    __device__ __forceinline__ float q_udx2c() const { return ld(c.q_udx2c + k); }
    __device__ __forceinline__ float udx1vis2() const { return ld(c.udx1vis2 + k); }
    __device__ __forceinline__ float q_rc_romeg() const { return ld(c.q_rc_romeg + k); }
    __device__ __forceinline__ float ap1j() const { return ld(c.ap1j + k); }
    __device__ __forceinline__ float ac1j() const { return ld(c.ac1j + k); }
    __device__ __forceinline__ float am1j() const { return ld(c.am1j + k); }
    __device__ __forceinline__ float ap2je() const { return ld(c.ap2je + k); }
    __device__ __forceinline__ float ac2je() const { return ld(c.ac2je + k); }
    __device__ __forceinline__ float am2je() const { return ld(c.am2je + k); }
    __device__ __forceinline__ float ap3j() const { return ld(c.ap3j + k); }
    __device__ __forceinline__ float ac3j() const { return ld(c.ac3j + k); }
    __device__ __forceinline__ float am3j() const { return ld(c.am3j + k); }
    __device__ __forceinline__ float cf_t() const { return ld(a.cf + k); }
    __device__ __forceinline__ float cf_r() const { return ld(a.cf + nrr + k); }
};
struct MarchCoefTable {
    const MarchCoef& q;
    __device__ __forceinline__ float usrc() const { return q.usrc; }
    __device__ __forceinline__ float usrcp() const { return q.usrcp; }
    __device__ __forceinline__ float udxt_m() const { return q.udxt_m; }
    __device__ __forceinline__ float udxtq_m() const { return q.udxtq_m; }
    __device__ __forceinline__ float q_usrm() const { return q.q_usrm; }
    __device__ __forceinline__ float q_udx2rm() const { return q.q_udx2rm; }
    __device__ __forceinline__ float h_udx1vis1() const { return q.h_udx1vis1; }
    __device__ __forceinline__ float udxt_c() const { return q.udxt_c; }
    __device__ __forceinline__ float udxtq_c() const { return q.udxtq_c; }
    __device__ __forceinline__ float q_udx2c() const { return q.q_udx2c; }
    __device__ __forceinline__ float udx1vis2() const { return q.udx1vis2; }
    __device__ __forceinline__ float q_rc_romeg() const { return q.q_rc_romeg; }
    __device__ __forceinline__ float ap1j() const { return q.ap1j; }
    __device__ __forceinline__ float ac1j() const { return q.ac1j; }
    __device__ __forceinline__ float am1j() const { return q.am1j; }
    __device__ __forceinline__ float ap2je() const { return q.ap2je; }
    __device__ __forceinline__ float ac2je() const { return q.ac2je; }
    __device__ __forceinline__ float am2je() const { return q.am2je; }
    __device__ __forceinline__ float ap3j() const { return q.ap3j; }
    __device__ __forceinline__ float ac3j() const { return q.ac3j; }
    __device__ __forceinline__ float am3j() const { return q.am3j; }
    __device__ __forceinline__ float cf_t() const { return q.cf_t; }
    __device__ __forceinline__ float cf_r() const { return q.cf_r; }
};

// The arithmetic of one level k of the march (explicit terms and the
// implicit right-hand sides of the three components) from the carried
// values and the level's loads; stores rhs and ru at offset o, then moves
// the carry up one level.  Shared by the global-load march
// (momentum_column_x2) and the TMA-staged one (momentum_march_tma_kernel),
// so both compute the same bits.
template <typename CQ>
__device__ __forceinline__ void march_level(const Dims& d, const CoefT<float>& c, const MomArgs<float>& a,
                                            const MarchK& K, const CQ& Q, int k, size_t o, MarchCarry& C,
                                            const MarchIn& L) {
    const int nr = d.nr, nrr = nr + 1;
    const bool top = k == nr - 1;
    const int kp = k + 1;
    const F2 TWO = K.TWO, MTWO = K.MTWO, QUARTER = K.QUARTER, ZERO = K.ZERO;
    const F2 GADT = K.GADT, RODT = K.RODT, ALREDT = K.ALREDT, FIC = K.FIC;
    const F2 UDXZ = K.UDXZ, UDXZQ = K.UDXZQ, NQROMEG = K.NQROMEG, NCFZ = K.NCFZ;
    const F2 U12lo = C.U12, Uzlo = C.Uz;
    F2& U12 = C.U12;
    F2& Uz = C.Uz;
    F2& Gup = C.Gup;
    const F2 tc = C.tc, tm = C.tm, tmip = C.tmip, rc = C.rc, rim = C.rim, rjm = C.rjm, rm = C.rm;
    const F2 zc = C.zc, zm = C.zm, zmjp = C.zmjp, prm = C.prm;
    const F2 tip = L.tip, tim = L.tim, tjp = L.tjp, tjm = L.tjm, tjmip = L.tjmip, tp = L.tp;
    const F2 rip = L.rip, rjp = L.rjp, rp = L.rp, rpim = L.rpim, rpjm = L.rpjm;
    const F2 zip = L.zip, zim = L.zim, zjp = L.zjp, zjm = L.zjm, zjpim = L.zjpim, zp = L.zp;
    const F2 pc = L.pc, pjm = L.pjm, pim = L.pim;
    const F2 old_t = L.old_t, old_r = L.old_r, old_z = L.old_z;
    (void)ZERO; (void)nrr;
    const F2 USRC = bc2(Q.usrc()), USRCP = bc2(Q.usrcp());
    const F2 tz_sw = (zc + zim) * (tc + tjm);
    const F2 qre = fma2(rp, USRCP, rc * USRC);
    // ---- ExplicitTermsQT
    F2 ht;
    {
        const F2 UDXT = bc2(Q.udxt_m()), UDXTQ = bc2(Q.udxtq_m());
        const F2 sth = tip + tim;
        const F2 x11 = (tip - tim) * fma2(TWO, tc, sth);          // (tip+tc)^2 - (tc+tim)^2
        const F2 rp2 = rp + rpim, rc2 = rc + rim;
        const F2 up = rp2 * (tp + tc);
        const F2 qrs = fma2(rp2, USRCP, rc2 * USRC);
        const F2 h12n = tc * bc2(Q.q_usrm()) * qrs;
        U12 = up;
        F2 s = fma2(up - U12lo, bc2(Q.q_udx2rm()), h12n);  // h12d + h12n
        s = fma2(x11, UDXT, s);                                   // + h11
        s = fma2((zjp + zjpim) * (tjp + tc) - tz_sw, UDXZ, s);    // + h13
        const F2 qrw = fma2(rpim, USRCP, rim * USRC);
        F2 r = (qre - qrw) * bc2(Q.h_udx1vis1());           // d11qre
        r = fma2(fma2(MTWO, tc, tjp + tjm), UDXZQ, r);            // + d22qt
        r = fma2(fma2(MTWO, tc, sth), UDXTQ, r);                  // + d11qt
        ht = fma2(qrs, NQROMEG, r - s);                           // + Coriolis
    }
    // ---- ExplicitTermsQR at face k (1 <= k)
    F2 hr = ZERO;
    {
        const F2 rup = qre * (rp + rc);
        if (k >= 1) {
            const F2 UDXT = bc2(Q.udxt_c()), UDXTQ = bc2(Q.udxtq_c());
            const F2 sa = tip + tmip, sb = tc + tm, s4 = sa + sb;
            const F2 aa = s4 * QUARTER;
            F2 s = (sa * (rip + rc) - U12lo) * UDXT;                  // h21
            s = fma2(rup - Gup, bc2(Q.q_udx2c()), s);           // + h22
            s = fma2((zjp + zmjp) * (rjp + rc) - Uzlo, UDXZ, s);      // + h23
            F2 r = fma2(aa, aa, (sb - sa) * bc2(Q.udx1vis2())); // h11n + d11qre
            r = fma2(fma2(MTWO, rc, rip + rim), UDXTQ, r);            // + d11qr
            r = fma2(fma2(MTWO, rc, rjp + rjm), UDXZQ, r);            // + d22qr
            r = fma2(s4, bc2(Q.q_rc_romeg()), r);               // + Coriolis
            hr = r - s;
        }
        Gup = rup;
    }
    // ---- ExplicitTermsQZ
    F2 hz;
    {
        const F2 UDXT = bc2(Q.udxt_m()), UDXTQ = bc2(Q.udxtq_m());
        const F2 upz = (rp + rpjm) * (zp + zc);
        F2 s = (upz - Uzlo) * bc2(Q.q_udx2rm());                // h32
        Uz = upz;
        s = fma2((tip + tjmip) * (zip + zc) - tz_sw, UDXT, s);        // + h31
        const F2 sjz = zjp + zjm;
        s = fma2((zjp - zjm) * fma2(TWO, zc, sjz), UDXZ, s);          // + h33
        F2 r = fma2(MTWO, zc, zim + zip) * UDXTQ;                     // dqz1
        r = fma2(fma2(MTWO, zc, sjz), UDXZQ, r);                      // + dqz2
        hz = r - s;
    }
    // ---- ImplicitAndUpdateQT
    {
        F2 d33;
        if (k == 0) {
            const F2 acc = fma2(bc2(Q.ac1j()), FIC, bc2(a.ac1j_fs0) * (bc2(1.0f) - FIC));
            const F2 amm = fma2(bc2(Q.am1j()), FIC, bc2(a.am1j_fs0) * (bc2(1.0f) - FIC));
            d33 = fma2(tp, bc2(Q.ap1j()), fma2(tc, acc, bc2(a.virotint + step_vinner<float>(a.st)) * amm));
        } else if (top) {
            const float app = Q.ap1j() * 1.0f + a.ap1j_fs1 * 0.0f;
            const float acc = Q.ac1j() * 1.0f + a.ac1j_fs1 * 0.0f;
            d33 = fma2(tc, bc2(acc), fma2(tm, bc2(Q.am1j()), bc2(a.virotext * app)));
        } else {
            d33 = fma2(tp, bc2(Q.ap1j()), fma2(tc, bc2(Q.ac1j()), tm * bc2(Q.am1j())));
        }
        const F2 rhs = fma2(pc - pim, bc2(-Q.cf_t()), fma2(ALREDT, d33, fma2(RODT, old_t, GADT * ht)));
        st_f2(a.rhs_t + o, rhs);
        st_f2(a.ru1 + o, ht);
    }
    // ---- ImplicitAndUpdateQR, faces 1..nr-1
    if (k >= 1) {
        const F2 d33 = fma2(rp, bc2(Q.ap2je()), fma2(rc, bc2(Q.ac2je()), rm * bc2(Q.am2je())));
        const F2 rhs = fma2(pc - prm, bc2(-Q.cf_r()), fma2(ALREDT, d33, fma2(RODT, old_r, GADT * hr)));
        st_f2(a.rhs_r + o, rhs);
        st_f2(a.ru2 + o, hr);
    }
    // ---- ImplicitAndUpdateQZ
    {
        F2 d33;
        if (k == 0) {
            const F2 acc = fma2(bc2(Q.ac3j()), FIC, bc2(a.ac3j_fs0) * (bc2(1.0f) - FIC));
            const F2 amm = fma2(bc2(Q.am3j()), FIC, bc2(a.am3j_fs0) * (bc2(1.0f) - FIC));
            d33 = fma2(zp, bc2(Q.ap3j()), fma2(zc, acc, zc * amm));
        } else if (top) {
            const float app = Q.ap3j() * 1.0f + a.ap3j_fs1 * 0.0f;
            const float acc = Q.ac3j() * 1.0f + a.ac3j_fs1 * 0.0f;
            d33 = fma2(zc, bc2(app), fma2(zc, bc2(acc), zm * bc2(Q.am3j())));
        } else {
            d33 = fma2(zp, bc2(Q.ap3j()), fma2(zc, bc2(Q.ac3j()), zm * bc2(Q.am3j())));
        }
        // outer wall: ru3(nrm) already replaced by qcap(nrm) (ImplicitAndUpdateQZ.F90:86,110)
        const F2 old = top ? hz : old_z;
        const F2 rhs = fma2(pc - pjm, NCFZ, fma2(ALREDT, d33, fma2(RODT, old, GADT * hz)));
        st_f2(a.rhs_z + o, rhs);
        st_f2(a.ru3 + o, hz);
    }
    // march: level k becomes the lower neighbour of level k+1
    C.tm = tc; C.tmip = tip; C.tc = tp;
    C.rm = rc; C.rc = rp; C.rim = rpim; C.rjm = rpjm;
    C.zm = zc; C.zmjp = zjp; C.zc = zp;
    C.prm = pc;
}

// TAB: the per-level coefficients come from ctab (ctab[k - k0], a table the
// caller staged in shared memory) instead of the coefficient arrays.
template <bool TAB = false>
__device__ __forceinline__ void momentum_column_x2(const Dims& d, const CoefT<float>& c, const MomArgs<float>& a,
                                                   int i, int j, int k0, int k1,
                                                   const MarchCoef* ctab = nullptr) {
    const int nr = d.nr, nt = d.nt, nz = d.nz;
    const int P = (int)d.P;
    const int dimA = i == 0 ? nt - 1 : -1;             // q(i-1) from the pair's first cell
    const int dipB = i + 2 == nt ? 2 - nt : 2;         // q(i+2)
    const int djm = j == 0 ? (nz - 1) * nt : -nt, djp = j == nz - 1 ? -(nz - 1) * nt : nt;
    const size_t col = (size_t)j * nt + i;
    const MarchK K = march_consts(d, a, col);
    const F2 ZERO = K.ZERO;
    const float* qt = a.qt;
    const float* qr = a.qr;
    const float* qz = a.qz;
    const float* pr = a.pr;

    // level k0 and its lower neighbours
    size_t o = (size_t)k0 * P + col;
    const int km0 = k0 > 0 ? k0 - 1 : 0;
    const size_t om = (size_t)km0 * P + col;
    MarchCarry C;
    C.tc = ld_f2(qt + o); C.tm = ld_f2(qt + om);
    C.tmip = mkf2(f2y(C.tm), ld(qt + om + dipB));
    C.rc = ld_f2(qr + o);
    C.rim = mkf2(ld(qr + o + dimA), f2x(C.rc));
    C.rjm = ld_f2(qr + o + djm);
    C.rm = k0 > 0 ? ld_f2(qr + om) : ZERO;
    C.zc = ld_f2(qz + o); C.zm = ld_f2(qz + om); C.zmjp = ld_f2(qz + om + djp);
    C.prm = k0 > 0 ? ld_f2(pr + om) : ZERO;
    {
        C.U12 = (C.rc + C.rim) * (C.tc + C.tm);
        C.Uz = (C.rc + C.rjm) * (C.zc + C.zm);
        const float usrc = ld(c.usrc + k0), usrcm = k0 > 0 ? ld(c.usrc + k0 - 1) : 0.0f;
        C.Gup = fma2(C.rm, bc2(usrcm), C.rc * bc2(usrc)) * (C.rc + C.rm);
    }
    for (int k = k0; k < k1; ++k, o += P) {
        const bool top = k == nr - 1;
        // bring the pair's entries of level k + kMomPrefetch into L2 ahead of
        // their loads
        if (k + kMomPrefetch < nr) {
            const size_t of = o + (size_t)kMomPrefetch * P;
            prefetch_l2(qt + of);
            prefetch_l2(qr + of);
            prefetch_l2(qz + of);
            prefetch_l2(pr + of);
            if (a.use_ru) {
                prefetch_l2(a.ru1 + of);
                prefetch_l2(a.ru2 + of);
                prefetch_l2(a.ru3 + of);
            }
        }
        // loads of level k (neighbours) and k+1 (column)
        MarchIn L;
        float tcx, tcy, rcx, rcy, zcx, zcy;
        f2xy(C.tc, tcx, tcy);
        f2xy(C.rc, rcx, rcy);
        f2xy(C.zc, zcx, zcy);
        L.tip = mkf2(tcy, ld(qt + o + dipB)); L.tim = mkf2(ld(qt + o + dimA), tcx);
        L.tjp = ld_f2(qt + o + djp); L.tjm = ld_f2(qt + o + djm);
        L.tjmip = mkf2(f2y(L.tjm), ld(qt + o + djm + dipB));
        L.tp = top ? C.tc : ld_f2(qt + o + P);
        L.rip = mkf2(rcy, ld(qr + o + dipB)); L.rjp = ld_f2(qr + o + djp);
        L.rp = ld_f2(qr + o + P);
        L.rpim = mkf2(ld(qr + o + P + dimA), f2x(L.rp)); L.rpjm = ld_f2(qr + o + P + djm);
        L.zip = mkf2(zcy, ld(qz + o + dipB)); L.zim = mkf2(ld(qz + o + dimA), zcx);
        L.zjp = ld_f2(qz + o + djp); L.zjm = ld_f2(qz + o + djm);
        L.zjpim = mkf2(ld(qz + o + djp + dimA), f2x(L.zjp));
        L.zp = top ? C.zc : ld_f2(qz + o + P);
        L.pc = ld_f2(pr + o); L.pjm = ld_f2(pr + o + djm);
        L.pim = mkf2(ld(pr + o + dimA), f2x(L.pc));
        // the RK memory of this level, loaded with the fields so that its
        // latency overlaps the explicit terms (below, the compiler could not
        // move these loads above the previous level's stores)
        L.old_t = a.use_ru ? ldp_f2(a.ru1 + o) : ZERO;
        L.old_r = (a.use_ru && k >= 1) ? ldp_f2(a.ru2 + o) : ZERO;
        L.old_z = (a.use_ru && !top) ? ldp_f2(a.ru3 + o) : ZERO;
        if constexpr (TAB) march_level(d, c, a, K, MarchCoefTable{ctab[k - k0]}, k, o, C, L);
        else march_level(d, c, a, K, MarchCoefGlobal{c, a, nr + 1, k}, k, o, C, L);
    }
}

// The FP32 fused momentum work marches in r: a thread takes a chunk of
// kMomChunk radial levels of its columns, keeping the values of planes k-1
// and k that the next level needs in registers, and the radial fluxes of the
// face between two levels (the lower-face flux of h12d, h22 and h32 at level
// k is the upper-face flux of level k-1).  It is bound by instruction issue
// and gains from the marching (fewer loads and address computations) and
// from packed FP32 (momentum_column_x2).  The FP64 kernels are bound by the
// FP64 pipe: they keep one level a thread and share the face terms of two
// theta-neighbouring cells instead (momentum_pair).
// Radial levels per thread.  On the 512x512x128 grid (mixed, one launch,
// mean over the substeps): 8 levels 0.375 ms, 16 0.375 ms, 24 0.378 ms,
// 32 0.384 ms, 64 0.422 ms.
constexpr int kMomChunk = 16;
template <typename T> struct MomMarch { static constexpr bool value = false; };
template <> struct MomMarch<float> { static constexpr bool value = true; };


// One LU-factored tridiagonal along r for one column, with the row scales
// folded into the factors: forward elimination into rhs (y_k0 = rhs_k0 +
// extra, y_k = rhs_k - l_k y_k-1), then back substitution
// (x_k = (y_k - u_k x_k+1) di_k) adding the solution to q.  Planes are loaded in
// batches of kRB ahead of the dependent arithmetic, so that each thread keeps
// several loads in flight (the recurrence itself is sequential).
constexpr int kRB = 8;
constexpr int kRBr = 8;   // planes per batch in the radial momentum sweeps

template <bool EXTRA, typename T>
__device__ __forceinline__ void lu_column(T* __restrict__ rhs, T* __restrict__ q, size_t P, int k0, int nr,
                                          const T* l, const T* di, const T* u, T extra) {
    T y = EXTRA ? rhs[(size_t)k0 * P] + extra : rhs[(size_t)k0 * P];
    rhs[(size_t)k0 * P] = y;
    int k = k0 + 1;
    for (; k + kRBr <= nr; k += kRBr) {
        T r[kRBr];
#pragma unroll
        for (int b = 0; b < kRBr; ++b) r[b] = rhs[(size_t)(k + b) * P];
#pragma unroll
        for (int b = 0; b < kRBr; ++b) {
            y = r[b] - ld(l + k + b) * y;
            rhs[(size_t)(k + b) * P] = y;
        }
    }
    for (; k < nr; ++k) {
        y = rhs[(size_t)k * P] - ld(l + k) * y;
        rhs[(size_t)k * P] = y;
    }
    T x = y * ld(di + nr - 1);
    q[(size_t)(nr - 1) * P] += x;
    k = nr - 2;
    for (; k - (kRBr - 1) >= k0; k -= kRBr) {
        T r[kRBr], v[kRBr];
#pragma unroll
        for (int b = 0; b < kRBr; ++b) {
            r[b] = rhs[(size_t)(k - b) * P];
            v[b] = q[(size_t)(k - b) * P];
        }
#pragma unroll
        for (int b = 0; b < kRBr; ++b) {
            x = (r[b] - ld(u + k - b) * x) * ld(di + k - b);
            q[(size_t)(k - b) * P] = v[b] + x;
        }
    }
    for (; k >= k0; --k) {
        x = (rhs[(size_t)k * P] - ld(u + k) * x) * ld(di + k);
        q[(size_t)k * P] += x;
    }
}

// lu_column without the round trip of the forward-elimination results
// through memory: the forward sweep stores y only at every kCkpt-th level (the
// checkpoints, over the rhs entries there); the back substitution recomputes
// the y of a batch from the checkpoint below it and the right-hand sides,
// re-read, then substitutes down through the batch.  Per level the traffic
// drops from 20 bytes (FP32: rhs read, y write, y read, q read and write) to
// 16 bytes and 1/kCkpt.  Used where the sweep is bound by memory (FP32); the
// recomputation doubles the forward arithmetic, which the FP64 sweeps, bound
// by the FP64 pipe, cannot afford.
// Levels per checkpointed batch.  On the 512x512x128 grid (radial solve of
// the three components, one launch): batches of 8 with 8 resident blocks
// per SM 0.325 ms, of 16 with 6 blocks 0.372 ms, the plain sweep with 6
// blocks 0.380 ms.
constexpr int kCkpt = 8;

// Lane operations of the checkpointed sweep: V = T, one column a thread, or
// V = F2 (FP32 path), two neighbouring columns a thread in packed FP32.
template <typename V, typename T> struct SweepV;
template <typename T> struct SweepV<T, T> {
    static __device__ __forceinline__ T load(const T* p) { return *p; }
    static __device__ __forceinline__ void store(T* p, T v) { *p = v; }
    static __device__ __forceinline__ T fnma(T s, T a, T b) { return b - s * a; }   // b - s a
    static __device__ __forceinline__ T mul(T a, T s) { return a * s; }
    static __device__ __forceinline__ T add(T a, T b) { return a + b; }
    static __device__ __forceinline__ T adds(T a, T s) { return a + s; }
};

template <bool EXTRA, typename T, typename V = T>
__device__ __forceinline__ void lu_column_ckpt(T* __restrict__ rhs, T* __restrict__ q, size_t P, int k0, int nr,
                                               const T* l, const T* di, const T* u, T extra) {
    typedef SweepV<V, T> O;
    const V y0 = EXTRA ? O::adds(O::load(rhs + (size_t)k0 * P), extra) : O::load(rhs + (size_t)k0 * P);
    O::store(rhs + (size_t)k0 * P, y0);
    V y = y0;
    // full batches [k0 + 1 + kCkpt m, k0 + kCkpt (m + 1)], checkpoint at their top
    const int nb = (nr - 1 - k0) / kCkpt;
    int k = k0 + 1;
    for (int m = 0; m < nb; ++m, k += kCkpt) {
        V r[kCkpt];
#pragma unroll
        for (int b = 0; b < kCkpt; ++b) r[b] = O::load(rhs + (size_t)(k + b) * P);
#pragma unroll
        for (int b = 0; b < kCkpt; ++b) y = O::fnma(ld(l + k + b), y, r[b]);
        O::store(rhs + (size_t)(k + kCkpt - 1) * P, y);
    }
    // tail levels: every y stored
    for (; k < nr; ++k) {
        y = O::fnma(ld(l + k), y, O::load(rhs + (size_t)k * P));
        O::store(rhs + (size_t)k * P, y);
    }
    // back substitution: the tail from its stored y
    V x = O::mul(y, ld(di + nr - 1));
    O::store(q + (size_t)(nr - 1) * P, O::add(O::load(q + (size_t)(nr - 1) * P), x));
    const int ktop = k0 + nb * kCkpt;          // top level of the last full batch
    for (k = nr - 2; k > ktop; --k) {
        x = O::mul(O::fnma(ld(u + k), x, O::load(rhs + (size_t)k * P)), ld(di + k));
        O::store(q + (size_t)k * P, O::add(O::load(q + (size_t)k * P), x));
    }
    // full batches from the top: recompute y from the checkpoint below
    for (int m = nb - 1; m >= 0; --m) {
        const int kb = k0 + 1 + m * kCkpt;     // lowest level of the batch
        V yb[kCkpt], v[kCkpt];
        V yc = O::load(rhs + (size_t)(kb - 1) * P);     // checkpoint (or y at k0)
#pragma unroll
        for (int b = 0; b < kCkpt; ++b) yb[b] = O::load(rhs + (size_t)(kb + b) * P);
#pragma unroll
        for (int b = 0; b < kCkpt; ++b) v[b] = O::load(q + (size_t)(kb + b) * P);
#pragma unroll
        for (int b = 0; b < kCkpt - 1; ++b) {
            yc = O::fnma(ld(l + kb + b), yc, yb[b]);
            yb[b] = yc;
        }
        // yb[kCkpt - 1] is the stored checkpoint y of the batch's top level
        const bool top_of_column = kb + kCkpt - 1 == nr - 1;
#pragma unroll
        for (int b = kCkpt - 1; b >= 0; --b) {
            const int kk = kb + b;
            if (b == kCkpt - 1 && top_of_column) continue;   // substituted above
            x = O::mul(O::fnma(ld(u + kk), x, yb[b]), ld(di + kk));
            O::store(q + (size_t)kk * P, O::add(v[b], x));
        }
    }
    // the first level (below every batch), unless it is also the last
    if (k0 < nr - 1) {
        x = O::mul(O::fnma(ld(u + k0), x, y0), ld(di + k0));
        O::store(q + (size_t)k0 * P, O::add(O::load(q + (size_t)k0 * P), x));
    }
}

// Two neighbouring columns in packed FP32 (the loads and stores move both
// columns' entries as one 8-byte word; the factors are the same for both).
template <> struct SweepV<F2, float> {
    static __device__ __forceinline__ F2 load(const float* p) {
        F2 r;
        r.v = *reinterpret_cast<const unsigned long long*>(p);
        return r;
    }
    static __device__ __forceinline__ void store(float* p, F2 v) { *reinterpret_cast<unsigned long long*>(p) = v.v; }
    static __device__ __forceinline__ F2 fnma(float s, F2 a, F2 b) { return fma2(bc2(-s), a, b); }
    static __device__ __forceinline__ F2 mul(F2 a, float s) { return a * bc2(s); }
    static __device__ __forceinline__ F2 add(F2 a, F2 b) { return a + b; }
    static __device__ __forceinline__ F2 adds(F2 a, float s) { return a + bc2(s); }
};

// ImplicitAndUpdateQR.F90:70-71: after the update both wall faces of qr are
// zero.  A start may hold other wall values (CreateInitialConditions.F90:33-34
// sets the inner one); the reference reads them until the first update, and
// so does the device.
template <typename T>
__device__ __forceinline__ void qr_walls_zero(T* q, size_t P, int nr) {
    q[0] = (T)0;
    q[(size_t)nr * P] = (T)0;
}

// SolveImpEqnUpdate_QT.F90:65-78 (comp 0), SolveImpEqnUpdate_QR.F90:54-65 (comp 1, faces
// 1..nr-1), SolveImpEqnUpdate_QZ.F90:59-68 (comp 2) for the column `col`.  The three
// components are independent, so each gets its own thread.
template <typename T>
__device__ __forceinline__ void radial_column(const Dims& d, const FieldsT<T>& f, int sub, long long col, int comp) {
    const int nr = d.nr;
    const size_t P = (size_t)d.P;
    const int v = (f.icyl && f.icyl[col] == 0) ? 1 : 0;
    const MomFactorsT<T>& F = f.F;
    if constexpr (std::is_same<T, float>::value) {
        if (comp == 0)
            lu_column_ckpt<true>(f.rhs_t + col, f.qt + col, P, 0, nr, F.l(sub, 0, v), F.dinv(sub, 0, v),
                                 F.u(sub, 0, v), *F.extra(sub));
        else if (comp == 1) {
            lu_column_ckpt<false>(f.rhs_r + col, f.qr + col, P, 1, nr, F.l(sub, 1, 0), F.dinv(sub, 1, 0),
                                  F.u(sub, 1, 0), (T)0);
            qr_walls_zero(f.qr + col, P, nr);
        } else
            lu_column_ckpt<false>(f.rhs_z + col, f.qz + col, P, 0, nr, F.l(sub, 2, v), F.dinv(sub, 2, v),
                                  F.u(sub, 2, v), (T)0);
        return;
    }
    if (comp == 0)
        lu_column<true>(f.rhs_t + col, f.qt + col, P, 0, nr, F.l(sub, 0, v), F.dinv(sub, 0, v), F.u(sub, 0, v),
                        *F.extra(sub));
    else if (comp == 1) {
        lu_column<false>(f.rhs_r + col, f.qr + col, P, 1, nr, F.l(sub, 1, 0), F.dinv(sub, 1, 0), F.u(sub, 1, 0), (T)0);
        qr_walls_zero(f.qr + col, P, nr);
    } else
        lu_column<false>(f.rhs_z + col, f.qz + col, P, 0, nr, F.l(sub, 2, v), F.dinv(sub, 2, v), F.u(sub, 2, v), (T)0);
}

// radial_column of the FP32 path for the columns col and col+1 (col even)
// in packed FP32; columns whose inner-wall slip variants differ (patterned
// free slip) are solved one after the other.
__device__ __forceinline__ void radial_column_pair(const Dims& d, const FieldsT<float>& f, int sub, long long col,
                                                   int comp) {
    const int nr = d.nr;
    const size_t P = (size_t)d.P;
    const int va = (f.icyl && f.icyl[col] == 0) ? 1 : 0, vb = (f.icyl && f.icyl[col + 1] == 0) ? 1 : 0;
    if (va != vb) {
        radial_column(d, f, sub, col, comp);
        radial_column(d, f, sub, col + 1, comp);
        return;
    }
    const MomFactorsT<float>& F = f.F;
    if (comp == 0)
        lu_column_ckpt<true, float, F2>(f.rhs_t + col, f.qt + col, P, 0, nr, F.l(sub, 0, va), F.dinv(sub, 0, va),
                                        F.u(sub, 0, va), *F.extra(sub));
    else if (comp == 1) {
        lu_column_ckpt<false, float, F2>(f.rhs_r + col, f.qr + col, P, 1, nr, F.l(sub, 1, 0), F.dinv(sub, 1, 0),
                                         F.u(sub, 1, 0), 0.0f);
        *reinterpret_cast<float2*>(f.qr + col) = make_float2(0.0f, 0.0f);
        *reinterpret_cast<float2*>(f.qr + col + (size_t)nr * P) = make_float2(0.0f, 0.0f);
    } else
        lu_column_ckpt<false, float, F2>(f.rhs_z + col, f.qz + col, P, 0, nr, F.l(sub, 2, va), F.dinv(sub, 2, va),
                                         F.u(sub, 2, va), 0.0f);
}

__device__ __forceinline__ double2 ld2(const double* p) { return ld(reinterpret_cast<const double2*>(p)); }
__device__ __forceinline__ float2 ld2(const float* p) { return ld(reinterpret_cast<const float2*>(p)); }

// CalcLocalDivergence.F90:27-40 for cells 2m and 2m+1 of row (k, j).
template <typename T>
__device__ __forceinline__ typename V2<T>::type div_pair(const Dims& d, const CoefT<T>& c, T dxt, T dxz,
                                                         const T* qt, const T* qr, const T* qz,
                                                         int k, int j, int m) {
    const size_t P = (size_t)d.P;
    const int nt = d.nt;
    const size_t row = (size_t)k * P + (size_t)j * nt;
    const int i0 = 2 * m, i2 = (2 * m + 2 == nt) ? 0 : 2 * m + 2;
    auto t01 = ld2(qt + row + i0);
    T t2 = ld(qt + row + i2);
    auto r0 = ld2(qr + row + i0);
    auto r1 = ld2(qr + row + P + i0);
    const int jp = wp(j, d.nz);
    auto z0 = ld2(qz + row + i0);
    auto z1 = ld2(qz + (size_t)k * P + (size_t)jp * nt + i0);
    const T udx2m = ld(c.udx2m + k), usrm = ld(c.usrm + k);
    T a = ((t01.y - t01.x) * dxt + (r1.x - r0.x) * udx2m) * usrm + (z1.x - z0.x) * dxz;
    T b = ((t2 - t01.y) * dxt + (r1.y - r0.y) * udx2m) * usrm + (z1.y - z0.y) * dxz;
    return mk2(a, b);
}

// div_pair times usdt and the FFT normalisation, from the per-dt coefficients
// of substep `sub`: each term (q_+ - q) times one product (the rounding
// order differs from div_pair's by the folding).
template <typename T>
__device__ __forceinline__ typename V2<T>::type div_pair_scaled(const Dims& d, const FieldsT<T>& f, int sub, int k,
                                                                int j, int m) {
    const size_t P = (size_t)d.P;
    const int nt = d.nt, nrr = d.nr + 1;
    const size_t row = (size_t)k * P + (size_t)j * nt;
    const int i0 = 2 * m, i2 = (2 * m + 2 == nt) ? 0 : 2 * m + 2;
    const T* qt = f.qt;
    const T* qr = f.qr;
    const T* qz = f.qz;
    auto t01 = ld2(qt + row + i0);
    T t2 = ld(qt + row + i2);
    auto r0 = ld2(qr + row + i0);
    auto r1 = ld2(qr + row + P + i0);
    const int jp = wp(j, d.nz);
    auto z0 = ld2(qz + row + i0);
    auto z1 = ld2(qz + (size_t)k * P + (size_t)jp * nt + i0);
    const T* dc = f.corr + kDivCoef(nrr);
    const T ct = ld(dc + sub * 2 * nrr + k), cr = ld(dc + sub * 2 * nrr + nrr + k), cz = ld(dc + 6 * nrr + sub);
    T a = (t01.y - t01.x) * ct + (r1.x - r0.x) * cr + (z1.x - z0.x) * cz;
    T b = (t2 - t01.y) * ct + (r1.y - r0.y) * cr + (z1.y - z0.y) * cz;
    return mk2(a, b);
}

// Forward transform of R rows.  FROM_PHI: the rows come from the phi array
// (CalcLocalDivergence already ran); otherwise the divergence is computed on
// the fly.  Output: spec[row][kt], kt = 0..M, scaled by usdt/(nthm*nzm).
// RT > 0: R = RT rows at compile time (div_fft_rows); RT = 0: R = 2^lgR
// rows known at run time (div_fft_rows_n, the ensembles' per-member row
// counts).  The arithmetic does not depend on R.
template <bool FROM_PHI, int RT, typename T, bool PRIME = true>
__device__ __forceinline__ void div_fft_rows_impl(const Dims& d, const CoefT<T>& c, T dxt, T dxz, const FieldsT<T>& f,
                                                  const FFTPlan& pl, const typename V2<T>::type* tw,
                                                  const typename V2<T>::type* twr, double fft_norm, int sub,
                                                  long long row0, typename V2<T>::type* smem, int Rrt, int lgR) {
    typedef typename V2<T>::type C2;
    const int R = RT > 0 ? RT : Rrt;
    const int M = pl.n;
    C2* a = smem;
    C2* b = smem + (size_t)R * M;
    const long long nrows = (long long)d.nr * d.nz;
    // usdt/(nthm nzm) with the 1/2 of the real-transform unpacking folded in
    const T scl = (T)(FROM_PHI ? fft_norm : f.scal[sub]);
    stage_tile<4>(a, R * M, [&](int t) {
        const int r = fdiv(t, pl.mn), m = t - r * M;
        const long long row = row0 + r;
        C2 z = mk2((T)0, (T)0);
        if (row < nrows) {
            const int k = d.mnz ? fdiv((int)row, d.mnz) : (int)(row / d.nz);
            const int j = (int)(row - (long long)k * d.nz);
            if (FROM_PHI) {
                z = ld2(f.phi + (size_t)row * d.nt + 2 * m);
                z.x *= scl;
                z.y *= scl;
            } else {
                z = div_pair_scaled(d, f, sub, k, j, m);
            }
        }
        return z;
    }, [&](int t) { const int r = fdiv(t, pl.mn); return (t - r * M) * R + r; });
    __syncthreads();
    const C2* Z = RT > 0 ? fft_lines<RT, PRIME>(a, b, pl, tw, false) : fft_lines_n<PRIME>(a, b, pl, tw, false, R, lgR);
    // X[k] = (Z[k] + conj Z[M-k]) - i W^k (Z[k] - conj Z[M-k]),  W = exp(-2 pi i / nthm)
    const int PH = M + 1;
    for (int t = threadIdx.x; t < R * PH; t += blockDim.x) {
        const int r = fdiv(t, pl.mn1), kt = t - r * PH;
        const long long row = row0 + r;
        if (row >= nrows) continue;
        const int k1 = kt == M ? 0 : kt, k2 = kt == 0 ? 0 : M - kt;
        C2 zk = Z[k1 * R + r], zc = cconj(Z[k2 * R + r]);
        C2 e = cadd(zk, zc), o = csub(zk, zc);
        C2 w = __ldg(twr + kt);
        // e - i w o = (e.x + w.x o.y + w.y o.x, e.y - w.x o.x + w.y o.y), in
        // multiply-adds (the product w o is never rounded on its own)
        f.spec[(size_t)row * PH + kt] = mk2(fmar(w.x, o.y, fmar(w.y, o.x, e.x)), fmar(-w.x, o.x, fmar(w.y, o.y, e.y)));
    }
}

template <bool FROM_PHI, int R, typename T, bool PRIME = true>
__device__ void div_fft_rows(const Dims& d, const CoefT<T>& c, T dxt, T dxz, const FieldsT<T>& f, const FFTPlan& pl,
                             const typename V2<T>::type* tw, const typename V2<T>::type* twr, double fft_norm,
                             int sub, long long row0, typename V2<T>::type* smem) {
    div_fft_rows_impl<FROM_PHI, R, T, PRIME>(d, c, dxt, dxz, f, pl, tw, twr, fft_norm, sub, row0, smem, R, 0);
}

template <bool FROM_PHI, typename T>
__device__ __forceinline__ void div_fft_rows_n(const Dims& d, const CoefT<T>& c, T dxt, T dxz, const FieldsT<T>& f,
                                               const FFTPlan& pl, const typename V2<T>::type* tw,
                                               const typename V2<T>::type* twr, double fft_norm, int sub,
                                               long long row0, typename V2<T>::type* smem, int R, int lgR) {
    div_fft_rows_impl<FROM_PHI, 0, T>(d, c, dxt, dxz, f, pl, tw, twr, fft_norm, sub, row0, smem, R, lgR);
}

// Complex FFT along z of ZC consecutive kt columns of one r-plane.  PRIME:
// with the stages of radix 7, 11 and 13 (fft_lines_impl).
template <int ZC, typename T, bool PRIME = true>
__device__ void zfft_tile(const Dims& d, const FieldsT<T>& f, const FFTPlan& pl, const typename V2<T>::type* tw,
                          int inv, int kt0, int kplane, typename V2<T>::type* smem) {
    typedef typename V2<T>::type C2;
    const int nz = pl.n, PH = d.PH;
    C2* a = smem;
    C2* b = smem + (size_t)ZC * nz;
    C2* plane = f.spec + (size_t)kplane * d.PS;
    stage_tile<8>(a, ZC * nz, [&](int t) {
        const int c = t % ZC, j = t / ZC;
        return (kt0 + c < PH) ? plane[(size_t)j * PH + kt0 + c] : mk2((T)0, (T)0);
    }, [](int t) { return t; });
    __syncthreads();
    const C2* Z = fft_lines<ZC, PRIME>(a, b, pl, tw, inv != 0);
    for (int t = threadIdx.x; t < ZC * nz; t += blockDim.x) {
        const int c = t % ZC, j = t / ZC;
        if (kt0 + c < PH) plane[(size_t)j * PH + kt0 + c] = Z[t];
    }
}

__device__ __forceinline__ double2 to_d2(double2 v) { return v; }
__device__ __forceinline__ double2 to_d2(float2 v) { return f2d(v); }
__device__ __forceinline__ void st2(double2* p, double x, double y) { *p = make_double2(x, y); }
__device__ __forceinline__ void st2(float2* p, double x, double y) { *p = make_float2(d2f(x), d2f(y)); }

// SolvePressureCorrection.F90:127-148: per mode (kt, kz) the real radial
// matrix (amph, acph - ak3 - ak1/rm^2, apph) applied to the complex
// right-hand side, with the precomputed LU factors.  One thread per mode
// (kz, kt) of the full spectrum, kz = 0..nzm-1; modes kz and nzm-kz share
// their factors (index min(kz, nzm-kz)).
//
// FP64 path (ptri_one): FP64 arithmetic, the forward-sweep results kept in
// the spectrum itself.
template <typename T>
__device__ __forceinline__ void ptri_one(const Dims& d, const Coef& c, const FieldsT<T>& f, double2* ws, long long t) {
    typedef typename V2<T>::type C2;
    const int PH = d.PH, nzh = d.nzh, nr = d.nr;
    const int kz = (int)(t / PH), kt = (int)(t - (long long)kz * PH);
    const int kf = kz < nzh ? kz : d.nz - kz;          // factor row of the pair
    const size_t PS = (size_t)d.PS, FS = (size_t)nzh * PH;
    const size_t o = (size_t)kz * PH + kt;
    C2* x = f.spec + o;
    double2* w = ws + o;
    const double* L = f.pf_l + (size_t)kf * PH + kt;
    const double* DI = f.pf_dinv + (size_t)kf * PH + kt;
    double2 y = to_d2(x[0]);
    w[0] = y;
    int k = 1;
    for (; k + kRB <= nr; k += kRB) {
        C2 b[kRB];
        double l[kRB];
#pragma unroll
        for (int q = 0; q < kRB; ++q) {
            l[q] = ld(L + (size_t)(k + q) * FS);
            b[q] = x[(size_t)(k + q) * PS];
        }
#pragma unroll
        for (int q = 0; q < kRB; ++q) {
            const double2 v = to_d2(b[q]);
            y = make_double2(v.x - l[q] * y.x, v.y - l[q] * y.y);
            w[(size_t)(k + q) * PS] = y;
        }
    }
    for (; k < nr; ++k) {
        const double l = ld(L + (size_t)k * FS);
        const double2 v = to_d2(x[(size_t)k * PS]);
        y = make_double2(v.x - l * y.x, v.y - l * y.y);
        w[(size_t)k * PS] = y;
    }
    double di = ld(DI + (size_t)(nr - 1) * FS);
    double2 s = make_double2(y.x * di, y.y * di);
    st2(x + (size_t)(nr - 1) * PS, s.x, s.y);
    k = nr - 2;
    for (; k - (kRB - 1) >= 0; k -= kRB) {
        double2 b[kRB];
        double u[kRB], dv[kRB];
#pragma unroll
        for (int q = 0; q < kRB; ++q) {
            u[q] = ld(c.apph + k - q);
            dv[q] = ld(DI + (size_t)(k - q) * FS);
            b[q] = w[(size_t)(k - q) * PS];
        }
#pragma unroll
        for (int q = 0; q < kRB; ++q) {
            s = make_double2((b[q].x - u[q] * s.x) * dv[q], (b[q].y - u[q] * s.y) * dv[q]);
            st2(x + (size_t)(k - q) * PS, s.x, s.y);
        }
    }
    for (; k >= 0; --k) {
        const double u = ld(c.apph + k);
        di = ld(DI + (size_t)k * FS);
        const double2 b = w[(size_t)k * PS];
        s = make_double2((b.x - u * s.x) * di, (b.y - u * s.y) * di);
        st2(x + (size_t)k * PS, s.x, s.y);
    }
}

// Mixed path (ptri_ff): float-float arithmetic (tc_ff.cuh; the factors and
// the super-diagonal were converted to float-float pairs once), which keeps
// the low, nearly singular modes as accurate as FP64 on the FP32 pipes.  The
// forward-sweep results are kept, as float-float complex values, only at
// every kPtriCk-th level (and at every level of the tail above the last full
// batch) in the scratch f.ws; the back substitution recomputes a batch from
// the checkpoint below it and the spectrum, re-read.  The spectrum is
// rounded to FP32 once, at the end.
// (kPtriCk and ptri_slots: tc_dev.h)

struct ffc {
    ffv re, im;
};
__device__ __forceinline__ float4 ffc_pack(ffc v) { return make_float4(v.re.hi, v.re.lo, v.im.hi, v.im.lo); }
__device__ __forceinline__ ffc ffc_unpack(float4 v) { return {{v.x, v.y}, {v.z, v.w}}; }
__device__ __forceinline__ ffv ffv_ld(const float2* p) { const float2 v = ld(p); return {v.x, v.y}; }
// y = x - l y (x exact in FP32)
__device__ __forceinline__ ffc ffc_fwd(float2 x, ffv l, ffc y) {
    return {ff_add_f(ff_neg(ff_mul(l, y.re)), x.x), ff_add_f(ff_neg(ff_mul(l, y.im)), x.y)};
}
// s = (y - u s) di
__device__ __forceinline__ ffc ffc_back(ffc y, ffv u, ffv di, ffc s) {
    return {ff_mul(ff_sub(y.re, ff_mul(u, s.re)), di), ff_mul(ff_sub(y.im, ff_mul(u, s.im)), di)};
}
__device__ __forceinline__ float2 ffc_round(ffc v) { return make_float2(ff_round(v.re), ff_round(v.im)); }

__device__ __forceinline__ void ptri_ff(const Dims& d, const FieldsT<float>& f, long long t) {
    const int PH = d.PH, nzh = d.nzh, nr = d.nr;
    const int kz = (int)(t / PH), kt = (int)(t - (long long)kz * PH);
    const int kf = kz < nzh ? kz : d.nz - kz;
    const size_t PS = (size_t)d.PS, FS = (size_t)nzh * PH;
    const size_t o = (size_t)kz * PH + kt;
    float2* x = f.spec + o;
    float4* w = f.ws + o;                              // slot q at w[q * PS]
    const float2* L = f.pl_ff + (size_t)kf * PH + kt;
    const float2* DI = f.pdi_ff + (size_t)kf * PH + kt;
    const float2* U = f.pu_ff;
    const int nb = (nr - 1) / kPtriCk;
    // forward elimination
    const float2 x0 = x[0];
    const ffc y0 = {ff_from(x0.x), ff_from(x0.y)};
    w[0] = ffc_pack(y0);
    ffc y = y0;
    int k = 1;
    for (int m = 0; m < nb; ++m, k += kPtriCk) {
        float2 xv[kPtriCk], lv[kPtriCk];
#pragma unroll
        for (int b = 0; b < kPtriCk; ++b) {
            xv[b] = x[(size_t)(k + b) * PS];
            lv[b] = ld(L + (size_t)(k + b) * FS);
        }
#pragma unroll
        for (int b = 0; b < kPtriCk; ++b) y = ffc_fwd(xv[b], {lv[b].x, lv[b].y}, y);
        w[(size_t)(m + 1) * PS] = ffc_pack(y);
    }
    for (int q = nb + 1; k < nr; ++k, ++q) {
        y = ffc_fwd(x[(size_t)k * PS], ffv_ld(L + (size_t)k * FS), y);
        w[(size_t)q * PS] = ffc_pack(y);
    }
    // back substitution: the last level, then the tail from its stored y
    ffc s = {ff_mul(y.re, ffv_ld(DI + (size_t)(nr - 1) * FS)), ff_mul(y.im, ffv_ld(DI + (size_t)(nr - 1) * FS))};
    x[(size_t)(nr - 1) * PS] = ffc_round(s);
    const int ktop = kPtriCk * nb;                     // top level of the last full batch
    for (k = nr - 2; k > ktop; --k) {
        const ffc yk = ffc_unpack(w[(size_t)(nb + 1 + (k - ktop - 1)) * PS]);
        s = ffc_back(yk, ffv_ld(U + k), ffv_ld(DI + (size_t)k * FS), s);
        x[(size_t)k * PS] = ffc_round(s);
    }
    // full batches from the top: recompute y from the checkpoint below
    for (int m = nb - 1; m >= 0; --m) {
        const int kb = 1 + m * kPtriCk;               // lowest level of the batch
        ffc yb[kPtriCk];
        ffc yc = ffc_unpack(w[(size_t)m * PS]);
        float2 xv[kPtriCk - 1];
#pragma unroll
        for (int b = 0; b < kPtriCk - 1; ++b) xv[b] = x[(size_t)(kb + b) * PS];
#pragma unroll
        for (int b = 0; b < kPtriCk - 1; ++b) {
            yc = ffc_fwd(xv[b], ffv_ld(L + (size_t)(kb + b) * FS), yc);
            yb[b] = yc;
        }
        yb[kPtriCk - 1] = ffc_unpack(w[(size_t)(m + 1) * PS]);
        const bool top_of_column = kb + kPtriCk - 1 == nr - 1;
#pragma unroll
        for (int b = kPtriCk - 1; b >= 0; --b) {
            const int kk = kb + b;
            if (b == kPtriCk - 1 && top_of_column) continue;   // substituted above
            s = ffc_back(yb[b], ffv_ld(U + kk), ffv_ld(DI + (size_t)kk * FS), s);
            x[(size_t)kk * PS] = ffc_round(s);
        }
    }
    // level 0, unless it is also the last
    if (nr > 1) {
        s = ffc_back(y0, ffv_ld(U), ffv_ld(DI), s);
        x[0] = ffc_round(s);
    }
}

// Mixed path in FP64 arithmetic (ptri_d64, the default of the mixed form):
// the checkpointed structure of ptri_ff with the FP64 LU factors and FP64
// complex values in the checkpoint slots; the FP32 spectrum is widened on
// load and rounded once, on the final store.
__device__ __forceinline__ double2 d64_fwd(float2 x, double l, double2 y) {
    const double2 v = f2d(x);
    return make_double2(v.x - l * y.x, v.y - l * y.y);
}
__device__ __forceinline__ double2 d64_back(double2 y, double u, double di, double2 s) {
    return make_double2((y.x - u * s.x) * di, (y.y - u * s.y) * di);
}

__device__ __forceinline__ void ptri_d64(const Dims& d, const Coef& c, const FieldsT<float>& f, long long t) {
    const int PH = d.PH, nzh = d.nzh, nr = d.nr;
    const int kz = (int)(t / PH), kt = (int)(t - (long long)kz * PH);
    const int kf = kz < nzh ? kz : d.nz - kz;
    const size_t PS = (size_t)d.PS, FS = (size_t)nzh * PH;
    const size_t o = (size_t)kz * PH + kt;
    float2* x = f.spec + o;
    double2* w = reinterpret_cast<double2*>(f.ws) + o;     // slot q at w[q * PS]
    const double* L = f.pf_l + (size_t)kf * PH + kt;
    const double* DI = f.pf_dinv + (size_t)kf * PH + kt;
    const double* U = c.apph;
    const int nb = (nr - 1) / kPtriCk;
    // forward elimination
    const double2 y0 = f2d(x[0]);
    w[0] = y0;
    double2 y = y0;
    int k = 1;
    for (int m = 0; m < nb; ++m, k += kPtriCk) {
        float2 xv[kPtriCk];
        double lv[kPtriCk];
        // the batch two ahead into L2 (the sweep is bound by load latency)
        if (m + 2 < nb) {
            const float2* px = x + (size_t)(k + 2 * kPtriCk) * PS;
            const double* pl = L + (size_t)(k + 2 * kPtriCk) * FS;
#pragma unroll 1
            for (int b = 0; b < kPtriCk; ++b, px += PS, pl += FS) {
                prefetch_l2(px);
                prefetch_l2(pl);
            }
        }
#pragma unroll
        for (int b = 0; b < kPtriCk; ++b) {
            xv[b] = x[(size_t)(k + b) * PS];
            lv[b] = ld(L + (size_t)(k + b) * FS);
        }
#pragma unroll
        for (int b = 0; b < kPtriCk; ++b) y = d64_fwd(xv[b], lv[b], y);
        w[(size_t)(m + 1) * PS] = y;
    }
    for (int q = nb + 1; k < nr; ++k, ++q) {
        y = d64_fwd(x[(size_t)k * PS], ld(L + (size_t)k * FS), y);
        w[(size_t)q * PS] = y;
    }
    // back substitution: the last level, then the tail from its stored y
    const double dl = ld(DI + (size_t)(nr - 1) * FS);
    double2 s = make_double2(y.x * dl, y.y * dl);
    st2(x + (size_t)(nr - 1) * PS, s.x, s.y);
    const int ktop = kPtriCk * nb;
    for (k = nr - 2; k > ktop; --k) {
        s = d64_back(w[(size_t)(nb + 1 + (k - ktop - 1)) * PS], ld(U + k), ld(DI + (size_t)k * FS), s);
        st2(x + (size_t)k * PS, s.x, s.y);
    }
    // full batches from the top: recompute y from the checkpoint below
    for (int m = nb - 1; m >= 0; --m) {
        const int kb = 1 + m * kPtriCk;
        if (m >= 2) {
            const int kp = kb - 2 * kPtriCk;
            const float2* px = x + (size_t)kp * PS;
            const double* pl = L + (size_t)kp * FS;
            const double* pd = DI + (size_t)kp * FS;
#pragma unroll 1
            for (int b = 0; b < kPtriCk; ++b, px += PS, pl += FS, pd += FS) {
                prefetch_l2(px);
                prefetch_l2(pl);
                prefetch_l2(pd);
            }
        }
        double2 yb[kPtriCk];
        double2 yc = w[(size_t)m * PS];
        float2 xv[kPtriCk - 1];
#pragma unroll
        for (int b = 0; b < kPtriCk - 1; ++b) xv[b] = x[(size_t)(kb + b) * PS];
#pragma unroll
        for (int b = 0; b < kPtriCk - 1; ++b) {
            yc = d64_fwd(xv[b], ld(L + (size_t)(kb + b) * FS), yc);
            yb[b] = yc;
        }
        yb[kPtriCk - 1] = w[(size_t)(m + 1) * PS];
        const bool top_of_column = kb + kPtriCk - 1 == nr - 1;
#pragma unroll
        for (int b = kPtriCk - 1; b >= 0; --b) {
            const int kk = kb + b;
            if (b == kPtriCk - 1 && top_of_column) continue;
            s = d64_back(yb[b], ld(U + kk), ld(DI + (size_t)kk * FS), s);
            st2(x + (size_t)kk * PS, s.x, s.y);
        }
    }
    if (nr > 1) {
        s = d64_back(y0, ld(U), ld(DI), s);
        st2(x, s.x, s.y);
    }
}

// The pressure tridiagonal of mode t in the path's arithmetic.  FF (mixed
// path only): 0 FP64, 1 float-float, -1 as f.ptri_ff says (kernels that
// know the mode at launch compile one variant each: both in one kernel take
// more registers than either).
template <typename T, int FF = -1>
__device__ __forceinline__ void ptri_solve(const Dims& d, const Coef& c, const FieldsT<T>& f, long long t) {
    if constexpr (std::is_same<T, double>::value) ptri_one(d, c, f, reinterpret_cast<double2*>(f.spec), t);
    else if (FF == 1 || (FF < 0 && f.ptri_ff)) ptri_ff(d, f, t);
    else ptri_d64(d, c, f, t);
}

// Inverse real FFT along theta: spec rows -> phi rows, R rows a block (RT
// at compile time, thinv_rows; or 2^lgR at run time, thinv_rows_n).
template <int RT, typename T, bool PRIME = true>
__device__ __forceinline__ void thinv_rows_impl(const Dims& d, const FieldsT<T>& f, const FFTPlan& pl,
                                                const typename V2<T>::type* tw, const typename V2<T>::type* twr,
                                                long long row0, typename V2<T>::type* smem, int Rrt, int lgR) {
    typedef typename V2<T>::type C2;
    const int R = RT > 0 ? RT : Rrt;
    const int M = pl.n, PH = M + 1;
    C2* a = smem;
    C2* b = smem + (size_t)R * M;
    const long long nrows = (long long)d.nr * d.nz;
    stage_tile<4>(a, R * M, [&](int t) {
        const int r = fdiv(t, pl.mn), kt = t - r * M;
        const long long row = row0 + r;
        C2 z = mk2((T)0, (T)0);
        if (row < nrows) {
            const C2* X = f.spec + (size_t)row * PH;
            C2 xk = X[kt], xm = X[M - kt];
            if (kt == 0) { xk.y = 0; xm.y = 0; }   // imaginary parts of the 0 and Nyquist bins
            C2 xc = cconj(xm);
            C2 e = cadd(xk, xc), o = csub(xk, xc);
            C2 w = __ldg(twr + kt);
            // Z = e + i conj(w) o = (e.x - w.x o.y + w.y o.x, e.y + w.x o.x + w.y o.y)
            z = mk2(fmar(-w.x, o.y, fmar(w.y, o.x, e.x)), fmar(w.x, o.x, fmar(w.y, o.y, e.y)));
        }
        return z;
    }, [&](int t) { const int r = fdiv(t, pl.mn); return (t - r * M) * R + r; });
    __syncthreads();
    const C2* Z = RT > 0 ? fft_lines<RT, PRIME>(a, b, pl, tw, true) : fft_lines_n<PRIME>(a, b, pl, tw, true, R, lgR);
    for (int t = threadIdx.x; t < R * M; t += blockDim.x) {
        const int r = fdiv(t, pl.mn), m = t - r * M;
        const long long row = row0 + r;
        if (row < nrows) *reinterpret_cast<C2*>(f.phi + (size_t)row * d.nt + 2 * m) = Z[m * R + r];
    }
}

template <int R, typename T, bool PRIME = true>
__device__ void thinv_rows(const Dims& d, const FieldsT<T>& f, const FFTPlan& pl, const typename V2<T>::type* tw,
                           const typename V2<T>::type* twr, long long row0, typename V2<T>::type* smem) {
    thinv_rows_impl<R, T, PRIME>(d, f, pl, tw, twr, row0, smem, R, 0);
}

template <typename T>
__device__ __forceinline__ void thinv_rows_n(const Dims& d, const FieldsT<T>& f, const FFTPlan& pl,
                                             const typename V2<T>::type* tw, const typename V2<T>::type* twr,
                                             long long row0, typename V2<T>::type* smem, int R, int lgR) {
    thinv_rows_impl<0, T>(d, f, pl, tw, twr, row0, smem, R, lgR);
}

template <bool VEL, bool PRES, typename T>
__device__ __forceinline__ void correct_cell(const Dims& d, const FieldsT<T>& f, int sub, int i, int j, int k) {
    const int nt = d.nt, nr = d.nr;
    const size_t P = (size_t)d.P;
    const int im = wm(i, nt), ip = wp(i, nt), jm = wm(j, d.nz), jp = wp(j, d.nz);
    const size_t rowoff = (size_t)j * nt;
    const size_t o = (size_t)k * P + rowoff + i;
    const T* phi = f.phi;
    const T loc = ld(phi + o);
    const T pim = ld(phi + (size_t)k * P + rowoff + im);
    const T pjm = ld(phi + (size_t)k * P + (size_t)jm * nt + i);
    const T pkm = ld(phi + (size_t)(k > 0 ? k - 1 : 0) * P + rowoff + i);
    if (VEL) {
        const T* cf = f.corr + (size_t)sub * 3 * (nr + 1);
        f.qt[o] -= (loc - pim) * ld(cf + k);
        if (k >= 1) f.qr[o] -= (loc - pkm) * ld(cf + (nr + 1) + k);
        f.qz[o] -= (loc - pjm) * ld(cf + 2 * (nr + 1));
    }
    if (PRES) {
        // CorrectPressure.F90:40-44 with the coefficients of the step
        // (factors kernel): pr + phi - be lap(phi) = pr + phi + pe phi
        // + pt (phi_ip + phi_im) + pz (phi_jp + phi_jm) + pq (phi_kp + phi_km),
        // where the reference's amm = apph(kc) makes both radial neighbours
        // share one coefficient
        const T pip = ld(phi + (size_t)k * P + rowoff + ip);
        const T pjp = ld(phi + (size_t)k * P + (size_t)jp * nt + i);
        const T pkp = ld(phi + (size_t)(k < nr - 1 ? k + 1 : nr - 1) * P + rowoff + i);
        const T* pc = f.corr + kPresCoef(nr + 1);
        if constexpr (std::is_same<T, double>::value) {
            // pr + (1 + pe) phi + ...: the sum starts from pr
            double p = f.pr[o];
            p += ld(pc + 3 * (nr + 1) + 1 + k) * loc;
            p += ld(pc + (nr + 1) + k) * (pip + pim);
            p += ld(pc + 3 * (nr + 1)) * (pjp + pjm);
            p += ld(pc + 2 * (nr + 1) + k) * (pkp + pkm);
            f.pr[o] = p;
        } else {
            T inc = loc + ld(pc + k) * loc;
            inc += ld(pc + (nr + 1) + k) * (pip + pim);
            inc += ld(pc + 3 * (nr + 1)) * (pjp + pjm);
            inc += ld(pc + 2 * (nr + 1) + k) * (pkp + pkm);
            // mixed path: the increment from the FP32 phi in FP32, accumulated
            // into the FP64 pressure; the FP32 copy used by the momentum rhs is
            // refreshed from the FP64 sum (conversions on the integer pipes)
            const double p = f.pr[o] + f2d((float)inc);
            f.pr[o] = p;
            f.prf[o] = (T)d2f(p);
        }
    }
}

// correct_cell<true, true, float> for the two cells (i, j, k) and (i+1, j, k),
// i even (nthm is even): the pair's fields move as float2 (pressure as
// double2), the theta neighbours inside the pair come from the pair itself,
// so a thread issues half the loads of two single-cell threads.  Same
// arithmetic, cell by cell, as correct_cell.
__device__ __forceinline__ void correct_pair_f(const Dims& d, const FieldsT<float>& f, int sub, int i, int j, int k) {
    const int nt = d.nt, nr = d.nr, nrr = nr + 1;
    const size_t P = (size_t)d.P;
    const int im = wm(i, nt), ip1 = wp(i + 1, nt), jm = wm(j, d.nz), jp = wp(j, d.nz);
    const size_t rowoff = (size_t)j * nt;
    const size_t o = (size_t)k * P + rowoff + i;
    const float* phi = f.phi;
    const float2 L = ld(reinterpret_cast<const float2*>(phi + o));
    const float pim = ld(phi + (size_t)k * P + rowoff + im);
    const float pip = ld(phi + (size_t)k * P + rowoff + ip1);
    const float2 PJm = ld(reinterpret_cast<const float2*>(phi + (size_t)k * P + (size_t)jm * nt + i));
    const float2 PJp = ld(reinterpret_cast<const float2*>(phi + (size_t)k * P + (size_t)jp * nt + i));
    const float2 PKm = ld(reinterpret_cast<const float2*>(phi + (size_t)(k > 0 ? k - 1 : 0) * P + rowoff + i));
    const float2 PKp = ld(reinterpret_cast<const float2*>(phi + (size_t)(k < nr - 1 ? k + 1 : nr - 1) * P + rowoff + i));
    // CorrectVelocity.F90:28-47
    const float* cf = f.corr + (size_t)sub * 3 * nrr;
    const float cft = ld(cf + k), cfz = ld(cf + 2 * nrr);
    float2* qt = reinterpret_cast<float2*>(f.qt + o);
    float2* qz = reinterpret_cast<float2*>(f.qz + o);
    float2 vt = *qt, vz = *qz;
    vt.x -= (L.x - pim) * cft;
    vt.y -= (L.y - L.x) * cft;
    vz.x -= (L.x - PJm.x) * cfz;
    vz.y -= (L.y - PJm.y) * cfz;
    *qt = vt;
    *qz = vz;
    if (k >= 1) {
        const float cfr = ld(cf + nrr + k);
        float2* qr = reinterpret_cast<float2*>(f.qr + o);
        float2 vr = *qr;
        vr.x -= (L.x - PKm.x) * cfr;
        vr.y -= (L.y - PKm.y) * cfr;
        *qr = vr;
    }
    // CorrectPressure.F90:40-44 with the coefficients of the step
    const float* pc = f.corr + kPresCoef(nrr);
    const float pe = ld(pc + k), pt = ld(pc + nrr + k), pq = ld(pc + 2 * nrr + k), pz = ld(pc + 3 * nrr);
    float ia = L.x + pe * L.x, ib = L.y + pe * L.y;
    ia += pt * (L.y + pim);
    ib += pt * (pip + L.x);
    ia += pz * (PJp.x + PJm.x);
    ib += pz * (PJp.y + PJm.y);
    ia += pq * (PKp.x + PKm.x);
    ib += pq * (PKp.y + PKm.y);
    double2* pr = reinterpret_cast<double2*>(f.pr + o);
    double2 p = *pr;
    p.x += f2d(ia);
    p.y += f2d(ib);
    *pr = p;
    *reinterpret_cast<float2*>(f.prf + o) = make_float2(d2f(p.x), d2f(p.y));
}

// CalcMaxCFL.F90:30-43 at cell (i, j, k), in the element type: FP32 on the
// mixed path (a maximum is exact in any precision, so the reduction over
// cells can stay in FP32 too).
template <typename T>
__device__ __forceinline__ T cfl_value(const Dims& d, const Coef& c, const CoefT<T>& cv, double dxt, double dxz,
                                       const FieldsT<T>& f, int i, int j, int k) {
    const size_t P = (size_t)d.P;
    const int ip = wp(i, d.nt), jp = wp(j, d.nz);
    const size_t o = (size_t)k * P + (size_t)j * d.nt + i;
    // (a + b) 0.5 x equals (a + b) (0.5 x) exactly; the theta term uses the
    // product 0.5 dxt usrm(k), rounded once
    if (!std::is_same<T, double>::value) {
        const T vt = fabsf((float)((ld(f.qt + (size_t)k * P + (size_t)j * d.nt + ip) + ld(f.qt + o)) * ld(cv.h_dxt_usrm + k)));
        const T vr = fabsf((float)((ld(f.qr + o + P) + ld(f.qr + o)) * ld(cv.h_udx2rm + k)));
        const T vz = fabsf((float)((ld(f.qz + (size_t)k * P + (size_t)jp * d.nt + i) + ld(f.qz + o)) * (T)(0.5 * dxz)));
        return vt + vr + vz;
    }
    const double t0 = ld(f.qt + o), t1 = ld(f.qt + (size_t)k * P + (size_t)j * d.nt + ip);
    const double r0 = ld(f.qr + o), r1 = ld(f.qr + o + P);
    const double z0 = ld(f.qz + o), z1 = ld(f.qz + (size_t)k * P + (size_t)jp * d.nt + i);
    return (T)(fabs((t1 + t0) * ld(c.h_dxt_usrm + k)) + fabs((r1 + r0) * ld(c.h_udx2rm + k)) +
               fabs((z1 + z0) * (0.5 * dxz)));
}

__device__ __forceinline__ double to_double(double v) { return v; }
__device__ __forceinline__ double to_double(float v) { return f2d(v); }

template <typename T>
__device__ __forceinline__ double cfl_cell(const Dims& d, const Coef& c, const CoefT<T>& cv, double dxt, double dxz,
                                           const FieldsT<T>& f, int i, int j, int k) {
    return to_double(cfl_value(d, c, cv, dxt, dxz, f, i, j, k));
}

// Scalars of the momentum kernel for substep `sub`, in the element type T.
template <typename T>
inline MomArgs<T> make_mom_args(const Consts& k, const FieldsT<T>& f, int sub) {
    MomArgs<T> a;
    a.qt = f.qt; a.qr = f.qr; a.qz = f.qz; a.pr = f.prf;
    a.ru1 = f.ru1; a.ru2 = f.ru2; a.ru3 = f.ru3;
    a.rhs_t = f.rhs_t; a.rhs_r = f.rhs_r; a.rhs_z = f.rhs_z;
    a.h_t = f.h_t; a.h_r = f.h_r; a.h_z = f.h_z;
    a.icyl = k.patterned ? f.icyl : nullptr;
    a.st = f.st;
    a.al = (T)k.alm[sub]; a.ga = (T)k.gam[sub]; a.ro = (T)k.rom[sub];
    a.alre = (T)k.alre[sub]; a.dxt_al = (T)k.dxt_al[sub]; a.dxz_al = (T)k.dxz_al[sub];
    a.udxz = (T)k.udxz; a.udxzq = (T)k.udxzq; a.q_romeg = (T)k.q_romeg;
    a.virotint = (T)k.virotint; a.virotext = (T)k.virotext;
    a.ac1j_fs0 = (T)k.ac1j_fs0; a.am1j_fs0 = (T)k.am1j_fs0; a.ap1j_fs1 = (T)k.ap1j_fs1; a.ac1j_fs1 = (T)k.ac1j_fs1;
    a.ac3j_fs0 = (T)k.ac3j_fs0; a.am3j_fs0 = (T)k.am3j_fs0; a.ap3j_fs1 = (T)k.ap3j_fs1; a.ac3j_fs1 = (T)k.ac3j_fs1;
    a.use_ru = k.rom[sub] != 0.0;
    const int nrr = f.F.stride;
    a.cf = f.corr + (size_t)sub * 3 * nrr;
    a.mr = f.corr + (size_t)9 * nrr + sub * 3;
    a.ic = f.corr + kImpCoef(nrr) + (size_t)sub * 9 * nrr;
    return a;
}

}  // namespace
}  // namespace tcgb
