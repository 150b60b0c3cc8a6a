// tc_ref.cpp -- CPU oracle: serial restatement of the reference time step.
//
// TEST INFRASTRUCTURE ONLY (see tc_ref.h).  Every routine below follows the
// reference Fortran routine it names, statement by statement, in the
// reference's array layout (r fastest, periodic halo of one cell in z and
// theta), with serial semantics: the OpenMP clauses of the reference are racy
// (PRIVATE work arrays shared across threads in SolveImpEqnUpdate_QT/QZ,
// uninitialised PRIVATE udxz/ocylsl in ImplicitAndUpdateQZ), so the oracle
// computes what a single-threaded build computes.  When this file is built
// with OpenMP, loops over theta run in parallel with per-thread work arrays;
// each (z,theta) column is still computed by exactly the serial arithmetic,
// so the result does not depend on the thread count.
//
// Third-party arithmetic restated here:
//  * LAPACK dgttrf/dgttrs and zgttrf/zgttrs (reference LAPACK, unpinned
//    version; Makefile:27 links -llapack).  The published LU algorithm with
//    partial pivoting for tridiagonal matrices is restated in gttrf()/gttrs().
//    zgttrf/zgttrs on the real pressure matrix with a complex right-hand side
//    performs, element for element, the real arithmetic of dgttrf plus one
//    dgttrs on the real part and one on the imaginary part (all imaginary
//    parts of the factors stay exactly zero; CABS1 of a real number is its
//    absolute value), so that is how it is computed.
//  * FFTW 3.3.4 (job.sbatch:7) guru r2c/c2r/c2c plans, unnormalised,
//    forward sign -1.  Restated as a mixed-radix Cooley-Tukey DFT; results
//    agree with FFTW to roundoff only.
//
// Parity status: pinned to runs of the reference's own source.  The
// reference ships no golden vectors and cannot be compiled here, so its
// main.F90 and time-step routines were executed on one rank by a translator
// of their Fortran subset (tests/golden/fortran_subset.py, SciPy's LAPACK,
// numpy.fft for FFTW); tests/test_reference_runs.py checks this oracle
// against those runs (tests/golden/reference_runs.npz): velocities within
// 1e-12, pressure 1e-11 (the arbitrary radial offset of the singular mode
// removed), dt sequence, CFL numbers, torques and stop codes.

#include "tc_ref.h"

#include <algorithm>
#include <cmath>
#include <complex>
#include <cstdlib>
#include <cstring>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

typedef std::complex<double> cd;

namespace {

// ---------------------------------------------------------------------------
// LAPACK tridiagonal LU with partial pivoting (dgttrf), restated.
// dl[0..n-2], d[0..n-1], du[0..n-2], du2[0..n-3], ipiv[0..n-1] (0-based).
// ---------------------------------------------------------------------------
void gttrf(int n, double* dl, double* d, double* du, double* du2, int* ipiv) {
    for (int i = 0; i < n; ++i) ipiv[i] = i;
    for (int i = 0; i < n - 2; ++i) du2[i] = 0.0;
    for (int i = 0; i < n - 2; ++i) {
        if (std::fabs(d[i]) >= std::fabs(dl[i])) {
            if (d[i] != 0.0) {
                double fact = dl[i] / d[i];
                dl[i] = fact;
                d[i + 1] = d[i + 1] - fact * du[i];
            }
        } else {
            double fact = d[i] / dl[i];
            d[i] = dl[i];
            dl[i] = fact;
            double temp = du[i];
            du[i] = d[i + 1];
            d[i + 1] = temp - fact * d[i + 1];
            du2[i] = du[i + 1];
            du[i + 1] = -fact * du[i + 1];
            ipiv[i] = i + 1;
        }
    }
    if (n > 1) {
        int i = n - 2;
        if (std::fabs(d[i]) >= std::fabs(dl[i])) {
            if (d[i] != 0.0) {
                double fact = dl[i] / d[i];
                dl[i] = fact;
                d[i + 1] = d[i + 1] - fact * du[i];
            }
        } else {
            double fact = d[i] / dl[i];
            d[i] = dl[i];
            dl[i] = fact;
            double temp = du[i];
            du[i] = d[i + 1];
            d[i + 1] = temp - fact * d[i + 1];
            ipiv[i] = i + 1;
        }
    }
}

// dgttrs('N', n, 1, ...) -> dgtts2 with itrans = 0, one right-hand side.
// drop_last: solve with x(n) = 0 instead of b(n)/d(n) (pinned singular mode).
void gttrs(int n, const double* dl, const double* d, const double* du, const double* du2,
           const int* ipiv, double* b, bool drop_last = false) {
    for (int i = 0; i < n - 1; ++i) {
        int ip = ipiv[i];
        double temp = b[i + 1 - ip + i] - dl[i] * b[ip];
        b[i] = b[ip];
        b[i + 1] = temp;
    }
    b[n - 1] = drop_last ? 0.0 : b[n - 1] / d[n - 1];
    if (n > 1) b[n - 2] = (b[n - 2] - du[n - 2] * b[n - 1]) / d[n - 2];
    for (int i = n - 3; i >= 0; --i)
        b[i] = (b[i] - du[i] * b[i + 1] - du2[i] * b[i + 2]) / d[i];
}

// ---------------------------------------------------------------------------
// Mixed-radix complex DFT (decimation in time), unnormalised.
// sign = -1 forward, +1 backward (FFTW convention).
// ---------------------------------------------------------------------------
struct FFTPlan {
    int n = 0;
    std::vector<int> factors;   // n = f0 * f1 * ...
    std::vector<cd> wf, wb;     // exp(-+2 pi i j / n), j = 0..n-1
    void init(int n_) {
        n = n_;
        factors.clear();
        int m = n;
        const int pref[] = {4, 2, 3, 5};
        for (int p : pref) while (m % p == 0 && m > 1) { factors.push_back(p); m /= p; }
        for (int p = 7; m > 1; p += 2) while (m % p == 0) { factors.push_back(p); m /= p; }
        wf.resize(n); wb.resize(n);
        const long double tpi = 6.283185307179586476925286766559L;
        for (int j = 0; j < n; ++j) {
            long double a = tpi * (long double)j / (long double)n;
            double c = (double)cosl(a), s = (double)sinl(a);
            wf[j] = cd(c, -s);
            wb[j] = cd(c, s);
        }
    }
    // out[0..len-1] = DFT of in[0], in[stride], ... ; fi = factor index
    void rec(const cd* in, cd* out, int len, int stride, size_t fi, const std::vector<cd>& w) const {
        if (len == 1) { out[0] = in[0]; return; }
        int p = factors[fi];
        int m = len / p;
        for (int q = 0; q < p; ++q) rec(in + (size_t)q * stride, out + (size_t)q * m, m, stride * p, fi + 1, w);
        int tstep = n / len;       // W_len^j = W_n^(j*tstep)
        int pstep = n / p;         // W_p^j   = W_n^(j*pstep)
        cd t[64];
        for (int k = 0; k < m; ++k) {
            for (int q = 0; q < p; ++q) {
                cd y = out[k + (size_t)q * m];
                t[q] = (q == 0) ? y : y * w[(size_t)((long)q * k * tstep % n)];
            }
            for (int s = 0; s < p; ++s) {
                cd acc = t[0];
                for (int q = 1; q < p; ++q) acc += t[q] * w[(size_t)(((long)q * s % p) * pstep)];
                out[k + (size_t)s * m] = acc;
            }
        }
    }
    void exec(const cd* in, cd* out, int sign) const { rec(in, out, n, 1, 0, sign < 0 ? wf : wb); }
};

inline double sq(double x) { return x * x; }

}  // namespace

// ---------------------------------------------------------------------------
// Oracle state (param.F90 modules param + local_arrays).
// ---------------------------------------------------------------------------
struct TCRef {
    tcref_bou b;
    int mode00;
    int nthm, nzm, nrm, nth, nz, nr;
    double pi, dxt, dxz, dxr, dxtq, dxzq, dxrq;
    // 1-D arrays, 1-based (index 0 unused), length nr+1
    std::vector<double> rc, rm, g2rc, g2rm, g2rmm, g2rcc, pvol, usrm, usrc, udx1vis1, udx1vis2,
        udx1qm, udx1qc, udx2c, udx2m, udx2cc, udx2mm, rudx2c, udx2rm;
    std::vector<int> kmc, kpc, kmv, kpv, kup, kum;
    std::vector<double> ap1j, am1j, ac1j, ap2j, am2j, ac2j, ap2je, am2je, ac2je, ap3j, am3j, ac3j,
        apph, amph, acph;
    double ap1j_fs[3] = {0, 0, 0}, ac1j_fs[3] = {0, 0, 0}, am1j_fs[3] = {0, 0, 0};
    double ap3j_fs[3] = {0, 0, 0}, ac3j_fs[3] = {0, 0, 0}, am3j_fs[3] = {0, 0, 0};
    std::vector<int> icylsl, ocylsl;   // (1:nzm, 1:nthm)
    std::vector<double> ak1, ap, ak3, ao;
    double gam[4] = {0, 0, 0, 0}, rom[4] = {0, 0, 0, 0}, alm[4] = {0, 0, 0, 0};
    double al = 0, ga = 0, ro = 0, beta = 0, dt = 0, time = 0, vinner_t = 0, dvinner_t = 0;
    // 3-D arrays
    std::vector<double> qt, qr, qz, pr, dph;            // (1:nr, 0:nzm+1, 0:nthm+1)
    std::vector<double> rhs, dq, qcap, ru1, ru2, ru3;   // (1:nr, 1:nzm, 1:nthm)
    // pressure-solver work: complex spectrum (1:nrm, 1:nzm/2+1, 1:nthm)
    std::vector<cd> spec;
    FFTPlan plan_z, plan_t;
    // statistics (stat_arrays): TCREF_ST_COUNT arrays (1:nrm, 1:nzm), the
    // vorticity (1:nrm, 1:nzm, 1:nthm) and the sample count
    std::vector<double> stats, vortt, vortr, vortz;
    int nstatsamples = 0;
    double& st(int which, int k, int j) { return stats[(size_t)which * nrm * nzm + (size_t)(k - 1) + (size_t)nrm * (j - 1)]; }

    size_t H(int k, int j, int i) const { return (size_t)(k - 1) + (size_t)nr * ((size_t)j + (size_t)(nzm + 2) * (size_t)i); }
    size_t N(int k, int j, int i) const { return (size_t)(k - 1) + (size_t)nr * ((size_t)(j - 1) + (size_t)nzm * (size_t)(i - 1)); }
    size_t S(int j, int i) const { return (size_t)(j - 1) + (size_t)nzm * (size_t)(i - 1); }
    int nzmh() const { return nzm / 2 + 1; }
    size_t P(int k, int j, int i) const { return (size_t)(k - 1) + (size_t)nrm * ((size_t)(j - 1) + (size_t)nzmh() * (size_t)(i - 1)); }

    void init_time_march_scheme();
    void create_grid();
    void slip_bcs();
    void init_pressure_solver();
};

// InitTimeMarchScheme.F90:16-49
void TCRef::init_time_march_scheme() {
    if (b.nsst > 1) {
        gam[1] = 8.0 / 15.0; gam[2] = 5.0 / 12.0; gam[3] = 3.0 / 4.0;
        rom[1] = 0.0; rom[2] = -17.0 / 60.0; rom[3] = -5.0 / 12.0;
    } else {
        gam[1] = 1.5; gam[2] = 0.0; gam[3] = 0.0;
        rom[1] = -0.5; rom[2] = 0.0; rom[3] = 0.0;
    }
    for (int ns = 1; ns <= b.nsst && ns <= 3; ++ns) alm[ns] = gam[ns] + rom[ns];
}

// CreateGrid.F90:24-324
void TCRef::create_grid() {
    pi = 2.0 * std::asin(1.0);
    dxt = ((double)nthm * b.lamb) / (2.0 * pi);
    dxz = (double)nzm / b.alx3;
    dxr = (double)nrm / 1.0;
    dxtq = dxt * dxt; dxzq = dxz * dxz; dxrq = dxr * dxr;

    for (int kc = 1; kc <= nrm; ++kc) {                       // :40-45
        kmv[kc] = kc - 1; kpv[kc] = kc + 1;
        if (kc == 1) kmv[kc] = kc;
        if (kc == nrm) kpv[kc] = kc;
    }
    for (int kc = 1; kc <= nrm; ++kc) {                       // :47-52
        kpc[kc] = kpv[kc] - kc; kmc[kc] = kc - kmv[kc];
        kup[kc] = 1 - kpc[kc]; kum[kc] = 1 - kmc[kc];
    }

    double tstr = std::tanh(b.str);
    if (b.istr == 0) {                                        // :85-90
        for (int k = 1; k <= nr; ++k) {
            double x3 = (double)(k - 1) / (double)nrm;
            rc[k] = (b.rext - b.rint) * x3 + b.rint;
        }
    }
    if (b.istr == 4) {                                        // :99-105
        rc[1] = b.rint;
        for (int k = 2; k <= nr; ++k) {
            double z2dp = (double)(2 * k - nr - 1) / (double)nrm;
            rc[k] = (1.0 + std::tanh(b.str * z2dp) / tstr) * 0.5 * (b.rext - b.rint) + b.rint;
        }
    }
    if (b.istr == 6) {                                        // :109-128
        int nclip = (int)b.str;
        int nrmo = nr + nclip + nclip;
        std::vector<double> etazm(nr + 500 + 1 + 2 * nclip, 0.0), etaz(nr + 1, 0.0);
        for (int k = 1; k <= nrmo; ++k) etazm[k] = +std::cos(pi * ((double)k - 0.5) / (double)nrmo);
        for (int k = 1; k <= nr; ++k) etaz[k] = etazm[k + nclip];
        double delet = etaz[1] - etaz[nr];
        for (int k = 1; k <= nr; ++k) etaz[k] = etaz[k] / (0.5 * delet);
        rc[1] = b.rint;
        for (int k = 2; k <= nrm; ++k) rc[k] = (b.rext - b.rint) * (1.0 - etaz[k]) * 0.5 + b.rint;
        rc[nr] = b.rext;
    }

    for (int k = 1; k <= nrm; ++k) {                          // :136-139
        rm[k] = (rc[k] + rc[k + 1]) * 0.5;
        g2rm[k] = (rc[k + 1] - rc[k]) * dxr;
    }
    g2rc[1] = (rc[2] - rc[1]) * dxr;                          // :141-153
    g2rmm[1] = (rm[2] - rm[1]) * dxr;
    g2rcc[1] = (rc[2] - rc[1]) * dxr;
    for (int k = 2; k <= nrm; ++k) {
        g2rc[k] = (rc[k + 1] - rc[k - 1]) * dxr * 0.5;
        g2rmm[k] = (rm[k + 1] - rm[k - 1]) * dxr;
        g2rcc[k] = (rc[k + 1] - rc[k - 1]) * dxr;
    }
    g2rc[nr] = (rc[nr] - rc[nrm]) * dxr;
    g2rmm[nr] = (rm[nr] - rm[nrm]) * dxr;
    g2rcc[nr] = (rc[nr] - rc[nrm]) * dxr;

    for (int k = 1; k <= nrm; ++k) {                          // :156-167
        udx1vis1[k] = 2.0 * dxt / (sq(rm[k]) * b.ren);
        udx2rm[k] = dxr / (g2rm[k] * rm[k]);
        udx2m[k] = dxr / g2rm[k];
        udx2mm[k] = dxr / g2rmm[k];
        udx2c[k] = dxr / g2rc[k];
        rudx2c[k] = udx2c[k] * rc[k];
        usrm[k] = 1.0 / rm[k];
        udx1qm[k] = dxtq / sq(rm[k]);
        pvol[k] = (sq(rc[k + 1]) - sq(rc[k]));
    }
    udx2c[nr] = dxr / g2rc[nr];
    for (int k = 1; k <= nr; ++k) {                           // :169-174
        udx1vis2[k] = dxt / (rc[k] * b.ren);
        usrc[k] = 1.0 / rc[k];
        udx1qc[k] = dxtq / sq(rc[k]);
        udx2cc[k] = dxr / g2rcc[k];
    }

    // coefficients for q1, inner points (CreateGrid.F90:194-203)
    for (int kc = 2; kc <= nrm - 1; ++kc) {
        int kp = kc + 1;
        double a22 = dxrq / g2rm[kc] / rm[kc];
        double a22p = +a22 * rc[kp] / g2rc[kp];
        double a22m = +a22 * rc[kc] / g2rc[kc];
        ap1j[kc] = a22p; am1j[kc] = a22m;
        ac1j[kc] = -(a22p + a22m) - 1.0 / sq(rm[kc]);
    }
    {   // external bc (CreateGrid.F90:209-220)
        int kc = nrm, kp = kc + 1;
        double a22 = dxrq / (g2rm[kc] * rm[kc]);
        double apjjc = a22 * rc[kp] / g2rc[kp];
        double amjjc = a22 * rc[kc] / g2rc[kc];
        ap1j[kc] = 2.0 * apjjc;
        ac1j[kc] = -2.0 * apjjc - amjjc - 1.0 / sq(rm[kc]);
        am1j[kc] = amjjc;
        ap1j_fs[1] = 0.0; ac1j_fs[1] = -amjjc; am1j_fs[1] = amjjc;
    }
    {   // internal bc (CreateGrid.F90:226-238); overwrites the *_fs(1) entries set above
        int kc = 1, kp = kc + 1;
        double urpp = 1.0 / (g2rm[kc] * g2rc[kp]);
        double a22 = dxrq / g2rm[kc] / rm[kc];
        double a22p = +a22 * rc[kp] / g2rc[kp];
        double a22m = +a22 * rc[kc] / g2rc[kc];
        ap1j[kc] = a22p;
        am1j[kc] = 2.0 * a22m;
        ac1j[kc] = -(a22p + 2.0 * a22m) - 1.0 / sq(rm[kc]);
        ap1j_fs[1] = std::pow(rc[kp], 3) / (sq(rm[kc]) * rm[kp]) * dxrq * urpp;
        ac1j_fs[1] = -std::pow(rc[kp], 3) / std::pow(rm[kc], 3) * dxrq * urpp;
        am1j_fs[1] = 0.0;
    }
    // q2 (CreateGrid.F90:244-259)
    am2j[1] = 0.0; ap2j[1] = 0.0; ac2j[1] = 1.0;
    for (int kc = 2; kc <= nrm; ++kc) {
        int km = kc - 1;
        double a22 = rc[kc] * dxrq / g2rc[kc];
        double a22p = 1.0 / (rm[kc] * g2rm[kc]);
        double a22m = 1.0 / (rm[km] * g2rm[km]);
        ap2j[kc] = a22 * a22p; am2j[kc] = a22 * a22m;
        ac2j[kc] = -(a22 * a22p + a22 * a22m);
    }
    am2j[nr] = 0.0; ap2j[nr] = 0.0; ac2j[nr] = 1.0;
    // q2 explicit part (CreateGrid.F90:266-276)
    for (int kc = 2; kc <= nrm; ++kc) {
        int km = kc - 1, kp = kc + 1;
        double ugmm = dxrq / g2rc[kc];
        double a22p = rm[kc] / (rc[kp] * g2rm[kc]);
        double a22m = rm[km] / (rc[km] * g2rm[km]);
        double a22 = (rm[kc] / g2rm[kc] + rm[km] / g2rm[km]) / rc[kc];
        ap2je[kc] = a22p * ugmm; am2je[kc] = a22m * ugmm;
        ac2je[kc] = -a22 * ugmm - 1.0 / sq(rc[kc]);
    }
    // q3 inner (CreateGrid.F90:281-290)
    for (int kc = 2; kc <= nrm - 1; ++kc) {
        int kp = kc + 1;
        double a22 = dxrq / g2rm[kc] / rm[kc];
        double a22p = +a22 * rc[kp] / g2rc[kp];
        double a22m = +a22 * rc[kc] / g2rc[kc];
        ap3j[kc] = a22p; am3j[kc] = a22m; ac3j[kc] = -(a22p + a22m);
    }
    {   // q3 internal bc (CreateGrid.F90:296-306)
        int kc = 1, kp = kc + 1;
        double a22 = dxrq / g2rm[kc] / rm[kc];
        double a22p = +a22 * rc[kp] / g2rc[kp];
        double a22m = +a22 * rc[kc] / g2rc[kc];
        am3j[kc] = 0.0; ap3j[kc] = a22p; ac3j[kc] = -(a22p + 2.0 * a22m);
        am3j_fs[1] = 0.0; ap3j_fs[1] = a22p; ac3j_fs[1] = -(a22p);
    }
    {   // q3 external bc (CreateGrid.F90:311-322)
        int kc = nrm, kp = kc + 1;
        double a22 = dxrq / g2rm[kc] / rm[kc];
        double a22m = +a22 * rc[kc] / g2rc[kc];
        double a22p = +a22 * rc[kp] / g2rc[kp];
        am3j[kc] = a22m; ap3j[kc] = 0.0; ac3j[kc] = -(a22m + 2.0 * a22p);
        am3j_fs[2] = a22m; ap3j_fs[2] = 0.0; ac3j_fs[2] = -(a22m);
    }
    slip_bcs();                                               // :324
}

// SlipBCs.F90:12-98 (uses module time; 0 = free slip, 1 = no slip)
void TCRef::slip_bcs() {
    int acute = 1;
    for (auto& v : icylsl) v = 1;
    for (auto& v : ocylsl) v = 1;
    int ntott = b.minstrt * b.multmin;
    int ntotz = b.minstrz * b.multmin;
    int ntot = ntott + ntotz;
    double perdist = 2.0 * pi / b.lamb;
    double wint = b.virotint / b.rint;
    double anglemoved = wint * time;
    anglemoved = std::fmod(anglemoved, perdist);
    int points_moved = (int)std::floor(anglemoved * dxt);
    std::vector<int> thdispl(nthm + 1);
    for (int i = 1; i <= nthm; ++i) {
        int m = (i + points_moved) % nthm;    // Fortran mod: sign of the dividend
        thdispl[i] = m;
        if (thdispl[i] == 0) thdispl[i] = nthm;
    }
    if (ntot != 0) {
        // The reference divides integers by ntott and ntotz here (SlipBCs.F90:58-59);
        // with either being zero that is an integer division by zero.  Such
        // inputs are rejected before this point (tcref_create returns NULL).
        for (auto& v : icylsl) v = 0;
        double m1 = (double)b.minstrt / (double)b.minstrz * (double)nzm / (double)nthm;
        double y1 = (double)nzm / (double)ntotz;
        double x1 = (double)nthm / (double)ntott;
        int limit1, limit2;
        if (acute == 1 && ntotz != 0) { limit1 = -ntott; limit2 = ntotz; }
        else { limit1 = 0; limit2 = ntot; }
        for (int i = limit1; i <= limit2; ++i) {
            for (int j = 1; j <= nthm; ++j) {
                int truej = thdispl[j];
                if (ntotz == 0 && (j - i * x1 > 0.00001) && (j - i * x1 - x1 / 2.0 < 0.0001)) {
                    for (int k = 1; k <= nzm; ++k) icylsl[S(k, truej)] = 1;
                } else if (ntotz != 0) {
                    for (int k = 1; k <= nzm; ++k) {
                        if ((k - acute * m1 * j - i * y1 > 0.00001) &&
                            (k - acute * m1 * j - i * y1 - y1 / 2.0 < 0.00001))
                            icylsl[S(k, truej)] = 1;
                    }
                }
            }
        }
    }
}

// InitPressureSolver.F90:22-66
void TCRef::init_pressure_solver() {
    for (int kc = 1; kc <= nrm; ++kc) {
        int kp = kpv[kc];
        double a22icc = rc[kc] * kmc[kc] * dxrq / g2rc[kc];
        double a22icp = rc[kp] * kpc[kc] * dxrq / g2rc[kp];
        double ac2 = -(a22icc + a22icp);
        double ugmmm = 1.0 / (rm[kc] * g2rm[kc]);
        amph[kc] = a22icc * ugmmm;
        apph[kc] = a22icp * ugmmm;
        acph[kc] = ac2 * ugmmm;
    }
    int nthmh = nthm / 2 + 1, nthmp = nthmh + 1;
    int nzmh_ = nzm / 2 + 1, nzmp = nzmh_ + 1;
    for (int j = 1; j <= nzmh_; ++j) ao[j] = (j - 1) * 2.0 * pi;
    for (int j = nzmp; j <= nzm; ++j) ao[j] = -(nzm - j + 1) * 2.0 * pi;
    for (int j = 1; j <= nzm; ++j) ak3[j] = 2.0 * (1.0 - std::cos(ao[j] / nzm)) * sq((double)nzm / b.alx3);
    for (int i = 1; i <= nthmh; ++i) ap[i] = (i - 1) * 2.0 * pi;
    for (int i = nthmp; i <= nthm; ++i) ap[i] = -(nthm - i + 1) * 2.0 * pi;
    for (int i = 1; i <= nthm; ++i) ak1[i] = 2.0 * (1.0 - std::cos(ap[i] / nthm)) * dxtq;
    plan_z.init(nzm);
    plan_t.init(nthm);
}

// ---------------------------------------------------------------------------
extern "C" {

void tcref_set_threads(int n) {
#ifdef _OPENMP
    if (n > 0) omp_set_num_threads(n);
#else
    (void)n;
#endif
}
int tcref_get_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

void* tcref_create(const tcref_bou* b, int mode00) {
    if (!b || b->nthm < 2 || b->nzm < 2 || b->nrm < 3) return nullptr;
    int ntott = b->minstrt * b->multmin, ntotz = b->minstrz * b->multmin;
    if (ntott + ntotz != 0 && (ntott == 0 || ntotz == 0)) return nullptr;
    TCRef* r = new TCRef();
    r->b = *b;
    r->mode00 = mode00;
    r->nthm = b->nthm; r->nzm = b->nzm; r->nrm = b->nrm;
    r->nth = r->nthm + 1; r->nz = r->nzm + 1; r->nr = r->nrm + 1;
    int nr = r->nr;
    auto z1 = [&](std::vector<double>& v) { v.assign(nr + 1, 0.0); };
    for (auto* v : {&r->rc, &r->rm, &r->g2rc, &r->g2rm, &r->g2rmm, &r->g2rcc, &r->pvol, &r->usrm,
                    &r->usrc, &r->udx1vis1, &r->udx1vis2, &r->udx1qm, &r->udx1qc, &r->udx2c,
                    &r->udx2m, &r->udx2cc, &r->udx2mm, &r->rudx2c, &r->udx2rm, &r->ap1j, &r->am1j,
                    &r->ac1j, &r->ap2j, &r->am2j, &r->ac2j, &r->ap2je, &r->am2je, &r->ac2je,
                    &r->ap3j, &r->am3j, &r->ac3j, &r->apph, &r->amph, &r->acph})
        z1(*v);
    for (auto* v : {&r->kmc, &r->kpc, &r->kmv, &r->kpv, &r->kup, &r->kum}) v->assign(nr + 1, 0);
    r->ak1.assign(r->nth + 1, 0.0); r->ap.assign(r->nth + 1, 0.0);
    r->ak3.assign(r->nz + 1, 0.0); r->ao.assign(r->nz + 1, 0.0);
    r->icylsl.assign((size_t)r->nzm * r->nthm, 1);
    r->ocylsl.assign((size_t)r->nzm * r->nthm, 1);
    size_t nh = (size_t)nr * (r->nzm + 2) * (r->nthm + 2);
    size_t nn = (size_t)nr * r->nzm * r->nthm;
    for (auto* v : {&r->qt, &r->qr, &r->qz, &r->pr, &r->dph}) v->assign(nh, 0.0);
    for (auto* v : {&r->rhs, &r->dq, &r->qcap, &r->ru1, &r->ru2, &r->ru3}) v->assign(nn, 0.0);
    r->spec.assign((size_t)r->nrm * r->nzmh() * r->nthm, cd(0, 0));
    r->time = 0.0;
    r->init_time_march_scheme();
    r->create_grid();
    r->init_pressure_solver();
    return r;
}

void tcref_destroy(void* h) { delete (TCRef*)h; }

static std::vector<double>* arr3(TCRef* r, int which) {
    switch (which) {
        case TCREF_QT: return &r->qt;   case TCREF_QR: return &r->qr;
        case TCREF_QZ: return &r->qz;   case TCREF_PR: return &r->pr;
        case TCREF_DPH: return &r->dph; case TCREF_RHS: return &r->rhs;
        case TCREF_RU1: return &r->ru1; case TCREF_RU2: return &r->ru2;
        case TCREF_RU3: return &r->ru3; case TCREF_DQ: return &r->dq;
        case TCREF_QCAP: return &r->qcap;
        default: return nullptr;
    }
}
void tcref_set_array(void* h, int which, const double* src) {
    auto* v = arr3((TCRef*)h, which);
    if (v) std::memcpy(v->data(), src, v->size() * sizeof(double));
}
void tcref_get_array(void* h, int which, double* dst) {
    auto* v = arr3((TCRef*)h, which);
    if (v) std::memcpy(dst, v->data(), v->size() * sizeof(double));
}
int tcref_get_grid(void* h, int which, double* dst) {
    TCRef* r = (TCRef*)h;
    const std::vector<double>* v = nullptr;
    switch (which) {
        case TCREF_G_RC: v = &r->rc; break;        case TCREF_G_RM: v = &r->rm; break;
        case TCREF_G_G2RC: v = &r->g2rc; break;    case TCREF_G_G2RM: v = &r->g2rm; break;
        case TCREF_G_USRC: v = &r->usrc; break;    case TCREF_G_USRM: v = &r->usrm; break;
        case TCREF_G_UDX1VIS1: v = &r->udx1vis1; break; case TCREF_G_UDX1VIS2: v = &r->udx1vis2; break;
        case TCREF_G_UDX1QM: v = &r->udx1qm; break; case TCREF_G_UDX2C: v = &r->udx2c; break;
        case TCREF_G_UDX2M: v = &r->udx2m; break;  case TCREF_G_RUDX2C: v = &r->rudx2c; break;
        case TCREF_G_UDX2RM: v = &r->udx2rm; break;
        case TCREF_G_AP1J: v = &r->ap1j; break; case TCREF_G_AM1J: v = &r->am1j; break;
        case TCREF_G_AC1J: v = &r->ac1j; break; case TCREF_G_AP2J: v = &r->ap2j; break;
        case TCREF_G_AM2J: v = &r->am2j; break; case TCREF_G_AC2J: v = &r->ac2j; break;
        case TCREF_G_AP2JE: v = &r->ap2je; break; case TCREF_G_AM2JE: v = &r->am2je; break;
        case TCREF_G_AC2JE: v = &r->ac2je; break; case TCREF_G_AP3J: v = &r->ap3j; break;
        case TCREF_G_AM3J: v = &r->am3j; break; case TCREF_G_AC3J: v = &r->ac3j; break;
        case TCREF_G_APPH: v = &r->apph; break; case TCREF_G_AMPH: v = &r->amph; break;
        case TCREF_G_ACPH: v = &r->acph; break;
        case TCREF_G_PVOL: v = &r->pvol; break; case TCREF_G_UDX2MM: v = &r->udx2mm; break;
        case TCREF_G_UDX2CC: v = &r->udx2cc; break;
        case TCREF_G_AK1: {
            for (int i = 1; i <= r->nthm; ++i) dst[i - 1] = r->ak1[i];
            return r->nthm;
        }
        case TCREF_G_AK3: {
            for (int j = 1; j <= r->nzm; ++j) dst[j - 1] = r->ak3[j];
            return r->nzm;
        }
        default: return 0;
    }
    for (int k = 1; k <= r->nr; ++k) dst[k - 1] = (*v)[k];
    return r->nr;
}
void tcref_get_scalars(void* h, double* o) {
    TCRef* r = (TCRef*)h;
    o[0] = r->dxt; o[1] = r->dxz; o[2] = r->dxr; o[3] = r->beta;
    o[4] = r->al; o[5] = r->ga; o[6] = r->ro; o[7] = r->vinner_t;
}
void tcref_get_dvinner(void* h, double* o) { o[0] = ((TCRef*)h)->dvinner_t; }
void tcref_get_slip(void* h, int* ic, int* oc) {
    TCRef* r = (TCRef*)h;
    std::memcpy(ic, r->icylsl.data(), r->icylsl.size() * sizeof(int));
    std::memcpy(oc, r->ocylsl.data(), r->ocylsl.size() * sizeof(int));
}

// TimeMarcher.F90:20-23 with InnerCylVelocity.F90:15-16
void tcref_begin_step(void* h, double dt, double time) {
    TCRef* r = (TCRef*)h;
    r->dt = dt;
    r->time = time;
    r->beta = r->dt / r->b.ren * 0.5;
    r->vinner_t = r->b.sizepert * std::sin(2.0 * r->pi * r->b.omegapert * r->time);
    r->dvinner_t = 2.0 * r->pi * r->b.omegapert * r->b.sizepert *
                   std::cos(2.0 * r->pi * r->b.omegapert * r->time) * r->dt;
    r->slip_bcs();
}
void tcref_set_substep(void* h, int ns) {
    TCRef* r = (TCRef*)h;
    r->al = r->alm[ns]; r->ga = r->gam[ns]; r->ro = r->rom[ns];
}

// ExplicitTermsQT.F90:22-129
void tcref_explicit_terms_qt(void* h) {
    TCRef& R = *(TCRef*)h;
    const double udxzq = R.dxzq / R.b.ren, udxz = R.dxz * 0.25;
    const double* qt = R.qt.data(); const double* qr = R.qr.data(); const double* qz = R.qz.data();
    double* dq = R.dq.data();
#pragma omp parallel for schedule(static)
    for (int ic = 1; ic <= R.nthm; ++ic) {
        int im = ic - 1, ip = ic + 1;
        for (int jc = 1; jc <= R.nzm; ++jc) {
            int jm = jc - 1, jp = jc + 1;
            for (int kc = 1; kc <= R.nrm; ++kc) {
                int kmm = R.kmv[kc], kpp = R.kpv[kc], kp = kc + 1;
                double udxt = R.dxt * 0.25 * R.usrm[kc];
                double udxtq = R.dxtq / (R.b.ren * sq(R.rm[kc]));
                double h11 = ((qt[R.H(kc, jc, ip)] + qt[R.H(kc, jc, ic)]) * (qt[R.H(kc, jc, ip)] + qt[R.H(kc, jc, ic)])
                            - (qt[R.H(kc, jc, ic)] + qt[R.H(kc, jc, im)]) * (qt[R.H(kc, jc, ic)] + qt[R.H(kc, jc, im)])) * udxt;
                double h12d = ((qr[R.H(kp, jc, ic)] + qr[R.H(kp, jc, im)]) * (qt[R.H(kpp, jc, ic)] + qt[R.H(kc, jc, ic)])
                             - (qr[R.H(kc, jc, ic)] + qr[R.H(kc, jc, im)]) * (qt[R.H(kc, jc, ic)] + qt[R.H(kmm, jc, ic)])) * 0.25 * R.udx2rm[kc];
                double h12n = qt[R.H(kc, jc, ic)] * R.usrm[kc] *
                              ((qr[R.H(kp, jc, ic)] + qr[R.H(kp, jc, im)]) * R.usrc[kp]
                             + (qr[R.H(kc, jc, ic)] + qr[R.H(kc, jc, im)]) * R.usrc[kc]) * 0.25;
                double h12 = h12d + h12n;
                double h13 = ((qz[R.H(kc, jp, ic)] + qz[R.H(kc, jp, im)]) * (qt[R.H(kc, jp, ic)] + qt[R.H(kc, jc, ic)])
                            - (qz[R.H(kc, jc, ic)] + qz[R.H(kc, jc, im)]) * (qt[R.H(kc, jc, ic)] + qt[R.H(kc, jm, ic)])) * udxz;
                double d11qt = (qt[R.H(kc, jc, ip)] - 2.0 * qt[R.H(kc, jc, ic)] + qt[R.H(kc, jc, im)]) * udxtq;
                double d22qt = (qt[R.H(kc, jp, ic)] - 2.0 * qt[R.H(kc, jc, ic)] + qt[R.H(kc, jm, ic)]) * udxzq;
                double qre = qr[R.H(kp, jc, ic)] * R.usrc[kp] + qr[R.H(kc, jc, ic)] * R.usrc[kc];
                double qrw = qr[R.H(kp, jc, im)] * R.usrc[kp] + qr[R.H(kc, jc, im)] * R.usrc[kc];
                double d11qre = (qre - qrw) * R.udx1vis1[kc] * 0.5;
                double coriol = -((qr[R.H(kc, jc, ic)] + qr[R.H(kc, jc, im)]) * R.usrc[kc]
                                + (qr[R.H(kp, jc, ic)] + qr[R.H(kp, jc, im)]) * R.usrc[kp]) * 0.25 * R.b.romeg;
                dq[R.N(kc, jc, ic)] = -(h11 + h12 + h13) + d11qre + d22qt + d11qt + coriol;
            }
        }
    }
}

// ExplicitTermsQR.F90:40-149 (writes dph for kc = 2..nrm)
void tcref_explicit_terms_qr(void* h) {
    TCRef& R = *(TCRef*)h;
    const double udxzq = R.dxzq / R.b.ren, udxz = R.dxz * 0.25;
    const double* qt = R.qt.data(); const double* qr = R.qr.data(); const double* qz = R.qz.data();
    double* dph = R.dph.data();
#pragma omp parallel for schedule(static)
    for (int ic = 1; ic <= R.nthm; ++ic) {
        int im = ic - 1, ip = ic + 1;
        for (int jc = 1; jc <= R.nzm; ++jc) {
            int jm = jc - 1, jp = jc + 1;
            for (int kc = 2; kc <= R.nrm; ++kc) {
                double udxt = R.dxt * 0.25 * R.usrc[kc];
                double udxtq = R.dxtq / (R.b.ren * sq(R.rc[kc]));
                int kmm = R.kmv[kc], kp = kc + 1;
                double h11n = sq((qt[R.H(kc, jc, ip)] + qt[R.H(kmm, jc, ip)] + qt[R.H(kc, jc, ic)] + qt[R.H(kmm, jc, ic)]) * 0.25);
                double h21 = ((qt[R.H(kc, jc, ip)] + qt[R.H(kmm, jc, ip)]) * (qr[R.H(kc, jc, ip)] + qr[R.H(kc, jc, ic)])
                            - (qt[R.H(kc, jc, ic)] + qt[R.H(kmm, jc, ic)]) * (qr[R.H(kc, jc, ic)] + qr[R.H(kc, jc, im)])) * udxt;
                double h22 = ((qr[R.H(kp, jc, ic)] * R.usrc[kp] + qr[R.H(kc, jc, ic)] * R.usrc[kc]) * (qr[R.H(kp, jc, ic)] + qr[R.H(kc, jc, ic)])
                            - (qr[R.H(kc, jc, ic)] * R.usrc[kc] + qr[R.H(kmm, jc, ic)] * R.usrc[kmm]) * (qr[R.H(kc, jc, ic)] + qr[R.H(kmm, jc, ic)])) * R.udx2c[kc] * 0.25;
                double h23 = ((qz[R.H(kc, jp, ic)] + qz[R.H(kmm, jp, ic)]) * (qr[R.H(kc, jp, ic)] + qr[R.H(kc, jc, ic)])
                            - (qz[R.H(kc, jc, ic)] + qz[R.H(kmm, jc, ic)]) * (qr[R.H(kc, jc, ic)] + qr[R.H(kc, jm, ic)])) * udxz;
                double qte = (qt[R.H(kc, jc, ip)] + qt[R.H(kmm, jc, ip)]);
                double qtw = (qt[R.H(kc, jc, ic)] + qt[R.H(kmm, jc, ic)]);
                double d11qre = -(qte - qtw) * R.udx1vis2[kc];
                double d11qr = (qr[R.H(kc, jc, ip)] - 2.0 * qr[R.H(kc, jc, ic)] + qr[R.H(kc, jc, im)]) * udxtq;
                double d22qr = (qr[R.H(kc, jp, ic)] - 2.0 * qr[R.H(kc, jc, ic)] + qr[R.H(kc, jm, ic)]) * udxzq;
                double coriol = (qt[R.H(kc, jc, ic)] + qt[R.H(kc, jc, ip)] + qt[R.H(kmm, jc, ic)] + qt[R.H(kmm, jc, ip)]) * 0.25 * R.rc[kc] * R.b.romeg;
                dph[R.H(kc, jc, ic)] = -(h21 + h22 + h23) + h11n + d11qr + d22qr + d11qre + coriol;
            }
        }
    }
}

// ExplicitTermsQZ.F90:34-106
void tcref_explicit_terms_qz(void* h) {
    TCRef& R = *(TCRef*)h;
    const double udxz = R.dxz * 0.25, udxzq = R.dxzq / R.b.ren;
    const double* qt = R.qt.data(); const double* qr = R.qr.data(); const double* qz = R.qz.data();
    double* qcap = R.qcap.data();
#pragma omp parallel for schedule(static)
    for (int ic = 1; ic <= R.nthm; ++ic) {
        int im = ic - 1, ip = ic + 1;
        for (int jc = 1; jc <= R.nzm; ++jc) {
            int jm = jc - 1, jp = jc + 1;
            for (int kc = 1; kc <= R.nrm; ++kc) {
                int kp = kc + 1, kmm = R.kmv[kc], kpp = R.kpv[kc];
                double udxt = R.dxt * 0.25 * R.usrm[kc];
                double udxtq = R.dxtq / (R.b.ren * sq(R.rm[kc]));
                double h31 = ((qt[R.H(kc, jc, ip)] + qt[R.H(kc, jm, ip)]) * (qz[R.H(kc, jc, ip)] + qz[R.H(kc, jc, ic)])
                            - (qt[R.H(kc, jc, ic)] + qt[R.H(kc, jm, ic)]) * (qz[R.H(kc, jc, ic)] + qz[R.H(kc, jc, im)])) * udxt;
                double h32 = (((qr[R.H(kp, jc, ic)] + qr[R.H(kp, jm, ic)]) * (qz[R.H(kpp, jc, ic)] + qz[R.H(kc, jc, ic)]))
                            - ((qr[R.H(kc, jc, ic)] + qr[R.H(kc, jm, ic)]) * (qz[R.H(kc, jc, ic)] + qz[R.H(kmm, jc, ic)]))) * R.udx2rm[kc] * 0.25;
                double h33 = ((qz[R.H(kc, jp, ic)] + qz[R.H(kc, jc, ic)]) * (qz[R.H(kc, jp, ic)] + qz[R.H(kc, jc, ic)])
                            - (qz[R.H(kc, jc, ic)] + qz[R.H(kc, jm, ic)]) * (qz[R.H(kc, jc, ic)] + qz[R.H(kc, jm, ic)])) * udxz;
                double dqz1 = (qz[R.H(kc, jc, im)] - 2.0 * qz[R.H(kc, jc, ic)] + qz[R.H(kc, jc, ip)]) * udxtq;
                double dqz2 = (qz[R.H(kc, jm, ic)] - 2.0 * qz[R.H(kc, jc, ic)] + qz[R.H(kc, jp, ic)]) * udxzq;
                qcap[R.N(kc, jc, ic)] = -(h31 + h32 + h33) + dqz1 + dqz2;
            }
        }
    }
}

// ImplicitAndUpdateQT.F90:26-117 (rhs and ru1 only)
void tcref_implicit_rhs_qt(void* h) {
    TCRef& R = *(TCRef*)h;
    const double alre = R.al / R.b.ren;
    const int nrm = R.nrm;
#pragma omp parallel for schedule(static)
    for (int ic = 1; ic <= R.nthm; ++ic) {
        int imm = ic - 1;
        for (int jc = 1; jc <= R.nzm; ++jc) {
            double fic = (double)R.icylsl[R.S(jc, ic)], foc = (double)R.ocylsl[R.S(jc, ic)];
            // inner cylinder (ImplicitAndUpdateQT.F90:44-68)
            int kc = 1, kpp = 2;
            double app = R.ap1j[kc];
            double acc = (R.ac1j[kc] * fic + R.ac1j_fs[1] * (1 - fic));
            double amm = (R.am1j[kc] * fic + R.am1j_fs[1] * (1 - fic));
            double d33qt = R.qt[R.H(kpp, jc, ic)] * app + R.qt[R.H(kc, jc, ic)] * acc + (R.b.virotint + R.vinner_t) * amm;
            double dpx11 = (R.pr[R.H(kc, jc, ic)] - R.pr[R.H(kc, jc, imm)]) * R.dxt * R.al * R.usrm[kc];
            size_t n = R.N(kc, jc, ic);
            R.rhs[n] = (R.ga * R.dq[n] + R.ro * R.ru1[n] + alre * d33qt - dpx11) * R.dt;
            R.ru1[n] = R.dq[n];
            // inner points (ImplicitAndUpdateQT.F90:70-90)
            for (kc = 2; kc <= nrm - 1; ++kc) {
                int kmm = kc - 1; kpp = kc + 1;
                amm = R.am1j[kc]; acc = R.ac1j[kc]; app = R.ap1j[kc];
                d33qt = R.qt[R.H(kpp, jc, ic)] * app + R.qt[R.H(kc, jc, ic)] * acc + R.qt[R.H(kmm, jc, ic)] * amm;
                dpx11 = (R.pr[R.H(kc, jc, ic)] - R.pr[R.H(kc, jc, imm)]) * R.dxt * R.al * R.usrm[kc];
                n = R.N(kc, jc, ic);
                R.rhs[n] = (R.ga * R.dq[n] + R.ro * R.ru1[n] + alre * d33qt - dpx11) * R.dt;
                R.ru1[n] = R.dq[n];
            }
            // outer cylinder (ImplicitAndUpdateQT.F90:93-115)
            kc = nrm;
            int kmm = nrm - 1;
            amm = R.am1j[kc];
            app = (R.ap1j[kc] * foc + R.ap1j_fs[2] * (1 - foc));
            acc = (R.ac1j[kc] * foc + R.ac1j_fs[2] * (1 - foc));
            d33qt = R.b.virotext * app + R.qt[R.H(kc, jc, ic)] * acc + R.qt[R.H(kmm, jc, ic)] * amm;
            dpx11 = (R.pr[R.H(kc, jc, ic)] - R.pr[R.H(kc, jc, imm)]) * R.dxt * R.al * R.usrm[kc];
            n = R.N(kc, jc, ic);
            R.rhs[n] = (R.ga * R.dq[n] + R.ro * R.ru1[n] + alre * d33qt - dpx11) * R.dt;
            R.ru1[n] = R.dq[n];
        }
    }
}

// SolveImpEqnUpdate_QT.F90:22-80 (per-column dgttrf + dgttrs)
void tcref_solve_imp_eqn_update_qt(void* h) {
    TCRef& R = *(TCRef*)h;
    const int nrm = R.nrm;
    const double betadx = R.beta * R.al;
#pragma omp parallel
    {
        std::vector<double> amkl(nrm + 1), apkl(nrm + 1), ackl(nrm + 1), fkl(nrm + 1);
        std::vector<double> amkT(nrm), ackT(nrm), apkT(nrm), appk(nrm);
        std::vector<int> ipkv(nrm);
#pragma omp for schedule(static)
        for (int ic = 1; ic <= R.nthm; ++ic) {
            for (int jc = 1; jc <= R.nzm; ++jc) {
                double fic = (double)R.icylsl[R.S(jc, ic)], foc = (double)R.ocylsl[R.S(jc, ic)];
                double actot = (R.ac1j[1] * fic + R.ac1j_fs[1] * (1 - fic));
                double ackl_b = 1.0 / (1.0 - actot * betadx);
                ackl[1] = 1.0;
                apkl[1] = -R.ap1j[1] * betadx * ackl_b;
                amkl[1] = (R.am1j[1] * fic + R.am1j_fs[1] * (1 - fic));
                for (int kc = 2; kc <= nrm - 1; ++kc) {
                    ackl_b = 1.0 / (1.0 - R.ac1j[kc] * betadx);
                    amkl[kc] = -R.am1j[kc] * betadx * ackl_b;
                    ackl[kc] = 1.0;
                    apkl[kc] = -R.ap1j[kc] * betadx * ackl_b;
                }
                actot = (R.ac1j[nrm] * foc + R.ac1j_fs[2] * (1 - foc));
                ackl_b = 1.0 / (1.0 - actot * betadx);
                amkl[nrm] = -R.am1j[nrm] * betadx * ackl_b;
                ackl[nrm] = 1.0;
                apkl[nrm] = 0.0;
                for (int k = 0; k < nrm - 1; ++k) { amkT[k] = amkl[k + 2]; apkT[k] = apkl[k + 1]; }
                for (int k = 0; k < nrm; ++k) ackT[k] = ackl[k + 1];
                gttrf(nrm, amkT.data(), ackT.data(), apkT.data(), appk.data(), ipkv.data());
                ackl_b = 1.0 / (1.0 - R.ac1j[1] * betadx);
                fkl[1] = (R.rhs[R.N(1, jc, ic)] + 0.5 * R.al * R.dt * R.dvinner_t * R.am1j[1] / R.b.ren) * ackl_b;
                for (int kc = 2; kc <= nrm; ++kc) {
                    ackl_b = 1.0 / (1.0 - R.ac1j[kc] * betadx);
                    fkl[kc] = R.rhs[R.N(kc, jc, ic)] * ackl_b;
                }
                gttrs(nrm, amkT.data(), ackT.data(), apkT.data(), appk.data(), ipkv.data(), fkl.data() + 1);
                for (int kc = 1; kc <= nrm; ++kc) R.qt[R.H(kc, jc, ic)] = R.qt[R.H(kc, jc, ic)] + fkl[kc];
            }
        }
    }
}

// ImplicitAndUpdateQR.F90:39-66 (rhs and ru2 only)
void tcref_implicit_rhs_qr(void* h) {
    TCRef& R = *(TCRef*)h;
    const double alre = R.al / R.b.ren;
#pragma omp parallel for schedule(static)
    for (int ic = 1; ic <= R.nthm; ++ic) {
        for (int jc = 1; jc <= R.nzm; ++jc) {
            for (int kc = 2; kc <= R.nrm; ++kc) {
                int kmm = kc - 1, kpp = kc + 1;
                double amm = R.am2je[kc], acc = R.ac2je[kc], app = R.ap2je[kc];
                double udx2 = R.rc[kc] * R.al * R.udx2c[kc];
                double d33qr = R.qr[R.H(kpp, jc, ic)] * app + R.qr[R.H(kc, jc, ic)] * acc + R.qr[R.H(kmm, jc, ic)] * amm;
                double dpx22 = (R.pr[R.H(kc, jc, ic)] - R.pr[R.H(kmm, jc, ic)]) * udx2;
                size_t n = R.N(kc, jc, ic);
                R.rhs[n] = (R.ga * R.dph[R.H(kc, jc, ic)] + R.ro * R.ru2[n] + alre * d33qr - dpx22) * R.dt;
                R.ru2[n] = R.dph[R.H(kc, jc, ic)];
            }
        }
    }
}

// SolveImpEqnUpdate_QR.F90:25-67 plus the wall reset of ImplicitAndUpdateQR.F90:70-71
void tcref_solve_imp_eqn_update_qr(void* h) {
    TCRef& R = *(TCRef*)h;
    const int nrm = R.nrm, nr = R.nr;
    const double betadx = R.beta * R.al;
    std::vector<double> amkl(nr + 1), apkl(nr + 1), ackl(nr + 1);
    amkl[1] = 0.0; apkl[1] = 0.0; ackl[1] = 1.0;
    for (int kc = 2; kc <= nrm; ++kc) {
        double ackl_b = 1.0 / (1.0 - R.ac2j[kc] * betadx);
        amkl[kc] = -R.am2j[kc] * betadx * ackl_b;
        ackl[kc] = 1.0;
        apkl[kc] = -R.ap2j[kc] * betadx * ackl_b;
    }
    amkl[nr] = 0.0; apkl[nr] = 0.0; ackl[nr] = 1.0;
    std::vector<double> amkT(nr), ackT(nr), apkT(nr), appk(nr);
    std::vector<int> ipkv(nr);
    for (int k = 0; k < nr - 1; ++k) { amkT[k] = amkl[k + 2]; apkT[k] = apkl[k + 1]; }
    for (int k = 0; k < nr; ++k) ackT[k] = ackl[k + 1];
    gttrf(nr, amkT.data(), ackT.data(), apkT.data(), appk.data(), ipkv.data());
#pragma omp parallel
    {
        std::vector<double> fkl(nr + 1);
#pragma omp for schedule(static)
        for (int ic = 1; ic <= R.nthm; ++ic) {
            for (int jc = 1; jc <= R.nzm; ++jc) {
                fkl[1] = 0.0;
                for (int kc = 2; kc <= nrm; ++kc) {
                    double ackl_b = 1.0 / (1.0 - R.ac2j[kc] * betadx);
                    fkl[kc] = R.rhs[R.N(kc, jc, ic)] * ackl_b;
                }
                fkl[nr] = 0.0;
                gttrs(nr, amkT.data(), ackT.data(), apkT.data(), appk.data(), ipkv.data(), fkl.data() + 1);
                for (int kc = 2; kc <= nrm; ++kc) R.qr[R.H(kc, jc, ic)] = R.qr[R.H(kc, jc, ic)] + fkl[kc];
            }
        }
    }
    for (int i = 0; i <= R.nthm + 1; ++i)
        for (int j = 0; j <= R.nzm + 1; ++j) { R.qr[R.H(1, j, i)] = 0.0; R.qr[R.H(nr, j, i)] = 0.0; }
}

// ImplicitAndUpdateQZ.F90:36-117 (rhs and ru3 only; serial semantics:
// udxz = dxz*al and ocylsl is the module array).  At kc = nrm the interior
// loop has already replaced ru3(nrm) by qcap(nrm) when the wall block
// recomputes rhs(nrm), and amm is left at am3j(nrm) by that loop.
void tcref_implicit_rhs_qz(void* h) {
    TCRef& R = *(TCRef*)h;
    const double alre = R.al / R.b.ren, udxz = R.dxz * R.al;
    const int nrm = R.nrm;
#pragma omp parallel for schedule(static)
    for (int ic = 1; ic <= R.nthm; ++ic) {
        for (int jc = 1; jc <= R.nzm; ++jc) {
            int jm = jc - 1;
            double fic = (double)R.icylsl[R.S(jc, ic)], foc = (double)R.ocylsl[R.S(jc, ic)];
            int kc = 1, km = R.kmv[kc], kp = R.kpv[kc];
            double app = R.ap3j[kc];
            double acc = (R.ac3j[kc] * fic + R.ac3j_fs[1] * (1 - fic));
            double amm = (R.am3j[kc] * fic + R.am3j_fs[1] * (1 - fic));
            double dqz3 = R.qz[R.H(kp, jc, ic)] * app + R.qz[R.H(kc, jc, ic)] * acc + R.qz[R.H(km, jc, ic)] * amm;
            double dpx33 = (R.pr[R.H(kc, jc, ic)] - R.pr[R.H(kc, jm, ic)]) * udxz;
            size_t n = R.N(kc, jc, ic);
            R.rhs[n] = (R.ga * R.qcap[n] + R.ro * R.ru3[n] + alre * dqz3 - dpx33) * R.dt;
            R.ru3[n] = R.qcap[n];
            for (kc = 2; kc <= nrm; ++kc) {
                km = R.kmv[kc]; kp = R.kpv[kc];
                amm = R.am3j[kc]; acc = R.ac3j[kc]; app = R.ap3j[kc];
                dqz3 = R.qz[R.H(kp, jc, ic)] * app + R.qz[R.H(kc, jc, ic)] * acc + R.qz[R.H(km, jc, ic)] * amm;
                dpx33 = (R.pr[R.H(kc, jc, ic)] - R.pr[R.H(kc, jm, ic)]) * udxz;
                n = R.N(kc, jc, ic);
                R.rhs[n] = (R.ga * R.qcap[n] + R.ro * R.ru3[n] + alre * dqz3 - dpx33) * R.dt;
                R.ru3[n] = R.qcap[n];
            }
            kc = nrm; km = R.kmv[kc]; kp = R.kpv[kc];
            app = R.ap3j[kc];
            app = (R.ap3j[kc] * foc + R.ap3j_fs[2] * (1 - foc));
            acc = (R.ac3j[kc] * foc + R.ac3j_fs[2] * (1 - foc));
            dqz3 = R.qz[R.H(kp, jc, ic)] * app + R.qz[R.H(kc, jc, ic)] * acc + R.qz[R.H(km, jc, ic)] * amm;
            dpx33 = (R.pr[R.H(kc, jc, ic)] - R.pr[R.H(kc, jm, ic)]) * udxz;
            n = R.N(kc, jc, ic);
            R.rhs[n] = (R.ga * R.qcap[n] + R.ro * R.ru3[n] + alre * dqz3 - dpx33) * R.dt;
            R.ru3[n] = R.qcap[n];
        }
    }
}

// SolveImpEqnUpdate_QZ.F90:21-70
void tcref_solve_imp_eqn_update_qz(void* h) {
    TCRef& R = *(TCRef*)h;
    const int nrm = R.nrm;
    const double betadx = R.beta * R.al;
#pragma omp parallel
    {
        std::vector<double> amkl(nrm + 2), apkl(nrm + 2), ackl(nrm + 2), fkl(nrm + 2);
        std::vector<double> amkT(nrm), ackT(nrm), apkT(nrm), appk(nrm);
        std::vector<int> ipkv(nrm);
#pragma omp for schedule(static)
        for (int ic = 1; ic <= R.nthm; ++ic) {
            for (int jc = 1; jc <= R.nzm; ++jc) {
                double fic = (double)R.icylsl[R.S(jc, ic)], foc = (double)R.ocylsl[R.S(jc, ic)];
                double actot = (R.ac3j[1] * fic + R.ac3j_fs[1] * (1 - fic));
                double ackl_b = 1.0 / (1.0 - (actot * betadx));
                ackl[1] = 1.0;
                apkl[1] = -R.ap3j[1] * betadx * ackl_b;
                amkl[1] = 0.0;
                for (int kc = 2; kc <= nrm - 1; ++kc) {
                    ackl_b = 1.0 / (1.0 - R.ac3j[kc] * betadx);
                    amkl[kc] = -R.am3j[kc] * betadx * ackl_b;
                    ackl[kc] = 1.0;
                    apkl[kc] = -R.ap3j[kc] * betadx * ackl_b;
                }
                actot = (R.ac3j[nrm] * foc + R.ac3j_fs[2] * (1 - foc));
                ackl_b = 1.0 / (1.0 - (actot * betadx));
                amkl[nrm] = -R.am3j[nrm] * betadx * ackl_b;
                ackl[nrm] = 1.0;
                apkl[nrm] = 0.0;
                for (int k = 0; k < nrm - 1; ++k) { amkT[k] = amkl[k + 2]; apkT[k] = apkl[k + 1]; }
                for (int k = 0; k < nrm; ++k) ackT[k] = ackl[k + 1];
                gttrf(nrm, amkT.data(), ackT.data(), apkT.data(), appk.data(), ipkv.data());
                for (int kc = 1; kc <= nrm; ++kc) {
                    ackl_b = 1.0 / (1.0 - R.ac3j[kc] * betadx);
                    fkl[kc] = R.rhs[R.N(kc, jc, ic)] * ackl_b;
                }
                gttrs(nrm, amkT.data(), ackT.data(), apkT.data(), appk.data(), ipkv.data(), fkl.data() + 1);
                for (int kc = 1; kc <= nrm; ++kc) R.qz[R.H(kc, jc, ic)] = R.qz[R.H(kc, jc, ic)] + fkl[kc];
            }
        }
    }
}

// halo_common.f90:64-71 (z ghosts) then :104-108 (theta ghosts, all j)
void tcref_update_halo(void* h, int which) {
    TCRef& R = *(TCRef*)h;
    auto* v = arr3(&R, which);
    if (!v || which > TCREF_DPH) return;
    double* a = v->data();
    for (int i = 1; i <= R.nthm; ++i)
        for (int k = 1; k <= R.nr; ++k) {
            a[R.H(k, R.nzm + 1, i)] = a[R.H(k, 1, i)];
            a[R.H(k, 0, i)] = a[R.H(k, R.nzm, i)];
        }
    for (int j = 0; j <= R.nzm + 1; ++j)
        for (int k = 1; k <= R.nr; ++k) {
            a[R.H(k, j, R.nthm + 1)] = a[R.H(k, j, 1)];
            a[R.H(k, j, 0)] = a[R.H(k, j, R.nthm)];
        }
}

// CalcLocalDivergence.F90:19-40
void tcref_calc_local_divergence(void* h) {
    TCRef& R = *(TCRef*)h;
    const double usdt = 1.0 / (R.al * R.dt);
#pragma omp parallel for schedule(static)
    for (int ic = 1; ic <= R.nthm; ++ic) {
        int ip = ic + 1;
        for (int jc = 1; jc <= R.nzm; ++jc) {
            int jp = jc + 1;
            for (int kc = 1; kc <= R.nrm; ++kc) {
                int kp = kc + 1;
                double dqcap = ((R.qt[R.H(kc, jc, ip)] - R.qt[R.H(kc, jc, ic)]) * R.dxt
                              + (R.qr[R.H(kp, jc, ic)] - R.qr[R.H(kc, jc, ic)]) * R.udx2m[kc]) * R.usrm[kc]
                              + (R.qz[R.H(kc, jp, ic)] - R.qz[R.H(kc, jc, ic)]) * R.dxz;
                R.dph[R.H(kc, jc, ic)] = dqcap * usdt;
            }
        }
    }
}

// SolvePressureCorrection.F90:100-163: r2c along z, c2c forward along
// theta, divide by nthm*nzm, per-mode zgttrf/zgttrs in r, c2c backward
// along theta, c2r along z.  The decomp_2d transposes only move data.
void tcref_solve_pressure_correction(void* h) {
    TCRef& R = *(TCRef*)h;
    const int nrm = R.nrm, nzm = R.nzm, nthm = R.nthm, nzmh = R.nzmh();
    cd* sp = R.spec.data();
    // forward r2c along z for each (k, i)
#pragma omp parallel
    {
        std::vector<cd> a(std::max(nzm, nthm)), o(std::max(nzm, nthm));
#pragma omp for schedule(static)
        for (int i = 1; i <= nthm; ++i)
            for (int k = 1; k <= nrm; ++k) {
                for (int j = 1; j <= nzm; ++j) a[j - 1] = cd(R.dph[R.H(k, j, i)], 0.0);
                R.plan_z.exec(a.data(), o.data(), -1);
                for (int j = 1; j <= nzmh; ++j) sp[R.P(k, j, i)] = o[j - 1];
            }
        // forward c2c along theta for each (k, j), then normalise (SolvePressureCorrection.F90:113)
#pragma omp for schedule(static)
        for (int j = 1; j <= nzmh; ++j)
            for (int k = 1; k <= nrm; ++k) {
                for (int i = 1; i <= nthm; ++i) a[i - 1] = sp[R.P(k, j, i)];
                R.plan_t.exec(a.data(), o.data(), -1);
                double den = (double)(nthm * nzm);
                for (int i = 1; i <= nthm; ++i) sp[R.P(k, j, i)] = cd(o[i - 1].real() / den, o[i - 1].imag() / den);
            }
    }
    // per-mode radial tridiagonal (SolvePressureCorrection.F90:127-148)
#pragma omp parallel
    {
        std::vector<double> dl(nrm), d(nrm), du(nrm), du2(nrm), xr(nrm), xi(nrm);
        std::vector<int> ipiv(nrm);
#pragma omp for schedule(static)
        for (int i = 1; i <= nthm; ++i)
            for (int j = 1; j <= nzmh; ++j) {
                for (int k = 1; k <= nrm; ++k) {
                    d[k - 1] = R.acph[k] - R.ak3[j] - R.ak1[i] * (R.usrm[k] * R.usrm[k]);
                    xr[k - 1] = sp[R.P(k, j, i)].real();
                    xi[k - 1] = sp[R.P(k, j, i)].imag();
                }
                for (int k = 0; k < nrm - 1; ++k) { dl[k] = R.amph[k + 2]; du[k] = R.apph[k + 1]; }
                gttrf(nrm, dl.data(), d.data(), du.data(), du2.data(), ipiv.data());
                bool pin = (R.mode00 == TCREF_MODE00_PIN) && i == 1 && j == 1;
                gttrs(nrm, dl.data(), d.data(), du.data(), du2.data(), ipiv.data(), xr.data(), pin);
                gttrs(nrm, dl.data(), d.data(), du.data(), du2.data(), ipiv.data(), xi.data(), pin);
                for (int k = 1; k <= nrm; ++k) sp[R.P(k, j, i)] = cd(xr[k - 1], xi[k - 1]);
            }
    }
#pragma omp parallel
    {
        std::vector<cd> a(std::max(nzm, nthm)), o(std::max(nzm, nthm));
        // backward c2c along theta
#pragma omp for schedule(static)
        for (int j = 1; j <= nzmh; ++j)
            for (int k = 1; k <= nrm; ++k) {
                for (int i = 1; i <= nthm; ++i) a[i - 1] = sp[R.P(k, j, i)];
                R.plan_t.exec(a.data(), o.data(), +1);
                for (int i = 1; i <= nthm; ++i) sp[R.P(k, j, i)] = o[i - 1];
            }
        // c2r along z: Hermitian extension; the imaginary parts of the
        // zero and Nyquist bins do not contribute to a real output.
#pragma omp for schedule(static)
        for (int i = 1; i <= nthm; ++i)
            for (int k = 1; k <= nrm; ++k) {
                for (int j = 0; j < nzm; ++j) {
                    if (j < nzmh) a[j] = sp[R.P(k, j + 1, i)];
                    else a[j] = std::conj(sp[R.P(k, nzm - j + 1, i)]);
                }
                a[0] = cd(a[0].real(), 0.0);
                if (nzm % 2 == 0) a[nzm / 2] = cd(a[nzm / 2].real(), 0.0);
                R.plan_z.exec(a.data(), o.data(), +1);
                for (int j = 1; j <= nzm; ++j) R.dph[R.H(k, j, i)] = o[j - 1].real();
            }
    }
}

// CorrectVelocity.F90:28-47
void tcref_correct_velocity(void* h) {
    TCRef& R = *(TCRef*)h;
#pragma omp parallel for schedule(static)
    for (int ic = 1; ic <= R.nthm; ++ic) {
        int im = ic - 1;
        for (int jc = 1; jc <= R.nzm; ++jc) {
            int jm = jc - 1;
            for (int kc = 1; kc <= R.nrm; ++kc) {
                int km = R.kmv[kc];
                double locdph = R.dph[R.H(kc, jc, ic)];
                R.qt[R.H(kc, jc, ic)] = R.qt[R.H(kc, jc, ic)] - (locdph - R.dph[R.H(kc, jc, im)]) * R.dt * R.al * R.dxt * R.usrm[kc];
                R.qr[R.H(kc, jc, ic)] = R.qr[R.H(kc, jc, ic)] - (locdph - R.dph[R.H(km, jc, ic)]) * R.dt * R.al * R.rudx2c[kc];
                R.qz[R.H(kc, jc, ic)] = R.qz[R.H(kc, jc, ic)] - (locdph - R.dph[R.H(kc, jm, ic)]) * R.al * R.dt * R.dxz;
            }
        }
    }
    for (int i = 0; i <= R.nthm + 1; ++i)
        for (int j = 0; j <= R.nzm + 1; ++j) { R.qr[R.H(1, j, i)] = 0.0; R.qr[R.H(R.nr, j, i)] = 0.0; }
}

// CorrectPressure.F90:31-49 (amm = apph(kc), as in the reference)
void tcref_correct_pressure(void* h) {
    TCRef& R = *(TCRef*)h;
    const double be = R.beta;
#pragma omp parallel for schedule(static)
    for (int ic = 1; ic <= R.nthm; ++ic) {
        int im = ic - 1, ip = ic + 1;
        for (int jc = 1; jc <= R.nzm; ++jc) {
            int jm = jc - 1, jp = jc + 1;
            for (int kc = 1; kc <= R.nrm; ++kc) {
                int kp = R.kpv[kc], km = R.kmv[kc];
                double amm = R.apph[kc], acc = R.acph[kc], app = R.apph[kc];
                const double* d = R.dph.data();
                R.pr[R.H(kc, jc, ic)] = R.pr[R.H(kc, jc, ic)] + d[R.H(kc, jc, ic)] - be * (
                    (d[R.H(kc, jc, ip)] - 2.0 * d[R.H(kc, jc, ic)] + d[R.H(kc, jc, im)]) * R.udx1qm[kc] +
                    (d[R.H(kc, jp, ic)] - 2.0 * d[R.H(kc, jc, ic)] + d[R.H(kc, jm, ic)]) * R.dxzq +
                    (d[R.H(kp, jc, ic)] * app + d[R.H(kc, jc, ic)] * acc + d[R.H(km, jc, ic)] * amm));
            }
        }
    }
}

// TimeMarcher.F90:20-54
void tcref_time_marcher(void* h, double dt, double time) {
    TCRef& R = *(TCRef*)h;
    tcref_begin_step(h, dt, time);
    for (int ns = 1; ns <= R.b.nsst; ++ns) {
        tcref_set_substep(h, ns);
        tcref_explicit_terms_qt(h);
        tcref_explicit_terms_qr(h);
        tcref_explicit_terms_qz(h);
        tcref_implicit_rhs_qt(h);
        tcref_solve_imp_eqn_update_qt(h);
        tcref_implicit_rhs_qr(h);
        tcref_solve_imp_eqn_update_qr(h);
        tcref_implicit_rhs_qz(h);
        tcref_solve_imp_eqn_update_qz(h);
        tcref_update_halo(h, TCREF_QT);
        tcref_update_halo(h, TCREF_QR);
        tcref_update_halo(h, TCREF_QZ);
        tcref_calc_local_divergence(h);
        tcref_solve_pressure_correction(h);
        tcref_update_halo(h, TCREF_DPH);
        tcref_correct_velocity(h);
        tcref_correct_pressure(h);
        tcref_update_halo(h, TCREF_QT);
        tcref_update_halo(h, TCREF_QR);
        tcref_update_halo(h, TCREF_QZ);
        tcref_update_halo(h, TCREF_PR);
    }
}

// CalcMaxCFL.F90:22-43
double tcref_calc_max_cfl(void* h) {
    TCRef& R = *(TCRef*)h;
    double cflm = 0.00000001;
#pragma omp parallel for schedule(static) reduction(max : cflm)
    for (int i = 1; i <= R.nthm; ++i) {
        int ip = i + 1;
        for (int j = 1; j <= R.nzm; ++j) {
            int jp = j + 1;
            for (int k = 1; k <= R.nrm; ++k) {
                int kp = k + 1;
                double qcf = (std::fabs((R.qt[R.H(k, j, ip)] + R.qt[R.H(k, j, i)]) * 0.5 * R.dxt * R.usrm[k])
                            + std::fabs((R.qr[R.H(kp, j, i)] + R.qr[R.H(k, j, i)]) * 0.5 * R.udx2rm[k])
                            + std::fabs((R.qz[R.H(k, jp, i)] + R.qz[R.H(k, j, i)]) * 0.5 * R.dxz));
                cflm = std::max(cflm, qcf);
            }
        }
    }
    return cflm;
}

// CheckDivergence.F90:21-43
double tcref_check_divergence(void* h) {
    TCRef& R = *(TCRef*)h;
    double qmax = 0.0;
#pragma omp parallel for schedule(static) reduction(max : qmax)
    for (int ic = 1; ic <= R.nthm; ++ic) {
        int ip = ic + 1;
        for (int jc = 1; jc <= R.nzm; ++jc) {
            int jp = jc + 1;
            for (int kc = 1; kc <= R.nrm; ++kc) {
                int kp = kc + 1;
                double dqcap = ((R.qt[R.H(kc, jc, ip)] - R.qt[R.H(kc, jc, ic)]) * R.dxt
                              + (R.qr[R.H(kp, jc, ic)] - R.qr[R.H(kc, jc, ic)]) * R.udx2m[kc]) * R.usrm[kc]
                              + (R.qz[R.H(kc, jp, ic)] - R.qz[R.H(kc, jc, ic)]) * R.dxz;
                qmax = std::max(std::fabs(dqcap), qmax);
            }
        }
    }
    return qmax;
}

// CalcTorque.F90:26-55
void tcref_calc_torque(void* h, double* inner, double* outer) {
    TCRef& R = *(TCRef*)h;
    const int nr = R.nr, nrm = R.nrm;
    double reninv = 1.0 / R.b.ren;
    double anusslow = 0.0, anussup = 0.0;
    double del = -1.0 / (R.rc[2] - R.rc[1]);
    double deln = -1.0 / (R.rc[nr] - R.rc[nrm]);
    double jlam = 2.0 * R.b.rint * R.b.rint * R.b.rext * R.b.rext *
                  (R.b.virotint / R.b.rint - R.b.virotext / R.b.rext) /
                  (R.b.rext * R.b.rext - R.b.rint * R.b.rint) * reninv;
    double jlami = 1.0 / jlam;
    for (int i = 1; i <= R.nthm; ++i)
        for (int j = 1; j <= R.nzm; ++j) {
            double grtlow = ((R.qt[R.H(2, j, i)] * R.usrm[2] + R.qt[R.H(1, j, i)] * R.usrm[1]) * 0.5
                             - R.b.virotint * R.usrc[1]) * del;
            anusslow = anusslow + grtlow * R.icylsl[R.S(j, i)];
            double grtup = (R.b.virotext * R.usrc[nr]
                            - (R.qt[R.H(nrm - 1, j, i)] * R.usrm[nrm - 1] + R.qt[R.H(nrm, j, i)] * R.usrm[nrm]) * 0.5) * deln;
            anussup = anussup + grtup * R.ocylsl[R.S(j, i)];
        }
    anusslow = anusslow * std::pow(R.rc[2], 3) * reninv * jlami;
    anussup = anussup * std::pow(R.rc[nrm], 3) * reninv * jlami;
    double my_surface = 1.0 / (R.nthm * R.nzm);
    *inner = anusslow * my_surface;
    *outer = anussup * my_surface;
}

// CalcVelocityStats.F90:21-65
void tcref_calc_velocity_stats(void* h, double* vmax, double* rms) {
    TCRef& R = *(TCRef*)h;
    vmax[0] = vmax[1] = vmax[2] = -100.0;
    double qt2 = 0, qr2 = 0, qz2 = 0;
    double volt = R.pi * (sq(R.b.rext) - sq(R.b.rint));
    for (int ic = 1; ic <= R.nthm; ++ic) {
        int ip = ic + 1;
        for (int jc = 1; jc <= R.nzm; ++jc) {
            int jp = jc + 1;
            for (int kc = 1; kc <= R.nrm; ++kc) {
                int kp = kc + 1;
                vmax[0] = std::max(vmax[0], std::fabs(R.qt[R.H(kc, jc, ic)]));
                vmax[1] = std::max(vmax[1], std::fabs(R.qr[R.H(kc, jc, ic)]));
                vmax[2] = std::max(vmax[2], std::fabs(R.qz[R.H(kc, jc, ic)]));
                qt2 = qt2 + sq(R.qt[R.H(kc, jc, ic)] + R.qt[R.H(kc, jc, ip)]) * R.pvol[kc] * R.pi * 0.25;
                qr2 = qr2 + sq(R.qr[R.H(kc, jc, ic)] * R.usrc[kc] + R.qr[R.H(kp, jc, ic)] * R.usrc[kp]) * R.pvol[kc] * R.pi * 0.25;
                qz2 = qz2 + sq(R.qz[R.H(kc, jc, ic)] + R.qz[R.H(kc, jp, ic)]) * R.pvol[kc] * R.pi * 0.25;
            }
        }
    }
    double den = (double)R.nthm * (double)R.nzm * volt;
    rms[0] = qt2 / den; rms[1] = qr2 / den; rms[2] = qz2 / den;
}

// CalcVorticity.F90:30-70 into vortt, vortr, vortz (k = 1..nrm).
static void calc_vorticity(TCRef& R) {
    const int nrm = R.nrm;
    R.vortt.assign((size_t)nrm * R.nzm * R.nthm, 0.0);
    R.vortr.assign(R.vortt.size(), 0.0);
    R.vortz.assign(R.vortt.size(), 0.0);
    auto V = [&](int k, int j, int i) { return (size_t)(k - 1) + (size_t)nrm * ((size_t)(j - 1) + (size_t)R.nzm * (i - 1)); };
    for (int ic = 1; ic <= R.nthm; ++ic) {
        const int im = ic - 1, ip = ic + 1;
        for (int jc = 1; jc <= R.nzm; ++jc) {
            const int jm = jc - 1, jp = jc + 1;
            for (int kc = 1; kc <= nrm; ++kc) {
                const int kmm = R.kmv[kc], kpp = R.kpv[kc], kp = kc + 1;
                const double durdz = ((R.qr[R.H(kp, jp, ic)] * R.usrc[kp] + R.qr[R.H(kc, jp, ic)] * R.usrc[kc])
                                      - (R.qr[R.H(kp, jm, ic)] * R.usrc[kp] + R.qr[R.H(kc, jm, ic)] * R.usrc[kc])) * R.dxz * 0.25;
                const double duzdr = ((R.qz[R.H(kpp, jc, ic)] + R.qz[R.H(kpp, jp, ic)])
                                      - (R.qz[R.H(kmm, jc, ic)] + R.qz[R.H(kmm, jp, ic)])) * 0.5 * R.udx2mm[kc];
                R.vortt[V(kc, jc, ic)] = durdz - duzdr;
                const double duzdt = ((R.qz[R.H(kc, jc, ip)] + R.qz[R.H(kc, jp, ip)])
                                      - (R.qz[R.H(kc, jc, im)] + R.qz[R.H(kc, jp, im)])) * 0.25 * R.dxt * R.usrm[kc];
                const double dutdz = ((R.qt[R.H(kc, jp, ic)] + R.qt[R.H(kc, jp, ip)])
                                      - (R.qt[R.H(kc, jm, ic)] + R.qt[R.H(kc, jm, ip)])) * 0.25 * R.dxz;
                R.vortr[V(kc, jc, ic)] = duzdt - dutdz;
                const double dutdr = ((R.qt[R.H(kpp, jc, ic)] + R.qt[R.H(kpp, jc, ip)]) * R.rm[kpp]
                                      - (R.qt[R.H(kmm, jc, ic)] + R.qt[R.H(kmm, jc, ip)]) * R.rm[kmm])
                                     * 0.5 * R.udx2mm[kc] * R.usrm[kc];
                const double durdt = ((R.qr[R.H(kc, jc, ip)] * R.usrc[kc] + R.qr[R.H(kp, jc, ip)] * R.usrc[kp])
                                      - (R.qr[R.H(kc, jc, im)] * R.usrc[kc] + R.qr[R.H(kp, jc, im)] * R.usrc[kp])) * R.dxt * 0.25;
                R.vortz[V(kc, jc, ic)] = dutdr - durdt;
            }
        }
    }
}

static void ensure_stats(TCRef& R) {
    if (R.stats.empty()) R.stats.assign((size_t)TCREF_ST_COUNT * R.nrm * R.nzm, 0.0);
}

// StatRoutines.F90:13-76 (CalcStats): theta averages accumulated per (k, j).
void tcref_calc_stats(void* h) {
    TCRef& R = *(TCRef*)h;
    ensure_stats(R);
    R.nstatsamples = R.nstatsamples + 1;
    const double usnthm = 1.0 / R.nthm;
    calc_vorticity(R);
    const int nrm = R.nrm;
    auto V = [&](int k, int j, int i) { return (size_t)(k - 1) + (size_t)nrm * ((size_t)(j - 1) + (size_t)R.nzm * (i - 1)); };
    for (int i = 1; i <= R.nthm; ++i) {
        for (int j = 1; j <= R.nzm; ++j) {
            for (int k = 1; k <= nrm; ++k) {
                const int kp = R.kpv[k];          // clamped (StatRoutines.F90:33)
                const double qt = R.qt[R.H(k, j, i)], qr = R.qr[R.H(k, j, i)], qz = R.qz[R.H(k, j, i)];
                const double wt = R.vortt[V(k, j, i)], wr = R.vortr[V(k, j, i)], wz = R.vortz[V(k, j, i)];
                const double prv = R.pr[R.H(k, j, i)];
                R.st(TCREF_ST_VT_MEAN, k, j) = R.st(TCREF_ST_VT_MEAN, k, j) + qt * usnthm;
                R.st(TCREF_ST_VR_MEAN, k, j) = R.st(TCREF_ST_VR_MEAN, k, j) + qr * usnthm * R.usrc[k];
                R.st(TCREF_ST_VZ_MEAN, k, j) = R.st(TCREF_ST_VZ_MEAN, k, j) + qz * usnthm;
                R.st(TCREF_ST_WT_MEAN, k, j) = R.st(TCREF_ST_WT_MEAN, k, j) + wt * usnthm;
                R.st(TCREF_ST_WR_MEAN, k, j) = R.st(TCREF_ST_WR_MEAN, k, j) + wr * usnthm;
                R.st(TCREF_ST_WZ_MEAN, k, j) = R.st(TCREF_ST_WZ_MEAN, k, j) + wz * usnthm;
                R.st(TCREF_ST_VT_RMS, k, j) = R.st(TCREF_ST_VT_RMS, k, j) + sq(qt) * usnthm;
                R.st(TCREF_ST_VR_RMS, k, j) = R.st(TCREF_ST_VR_RMS, k, j) + sq(qr * R.usrc[k]) * usnthm;
                R.st(TCREF_ST_VZ_RMS, k, j) = R.st(TCREF_ST_VZ_RMS, k, j) + sq(qz) * usnthm;
                R.st(TCREF_ST_WT_RMS, k, j) = R.st(TCREF_ST_WT_RMS, k, j) + sq(wt) * usnthm;
                R.st(TCREF_ST_WR_RMS, k, j) = R.st(TCREF_ST_WR_RMS, k, j) + sq(wr) * usnthm;
                R.st(TCREF_ST_WZ_RMS, k, j) = R.st(TCREF_ST_WZ_RMS, k, j) + sq(wz) * usnthm;
                R.st(TCREF_ST_PR_MEAN, k, j) = R.st(TCREF_ST_PR_MEAN, k, j) + prv * usnthm;
                R.st(TCREF_ST_PR_RMS, k, j) = R.st(TCREF_ST_PR_RMS, k, j) + sq(prv) * usnthm;
                const double qr_kp = R.qr[R.H(kp, j, i)];
                R.st(TCREF_ST_VTVR_MEAN, k, j) = R.st(TCREF_ST_VTVR_MEAN, k, j) +
                    (qt + R.qt[R.H(k, j, i + 1)]) * (qr * R.usrc[k] + qr_kp * R.usrc[kp]) * usnthm * 0.25;
                // StatRoutines.F90:58: the second factor sums qz(k,j,i) and qr(k,j+1,i)
                R.st(TCREF_ST_VTVZ_MEAN, k, j) = R.st(TCREF_ST_VTVZ_MEAN, k, j) +
                    (qt + R.qt[R.H(k, j, i + 1)]) * (qz + R.qr[R.H(k, j + 1, i)]) * usnthm * 0.25;
                R.st(TCREF_ST_VRVZ_MEAN, k, j) = R.st(TCREF_ST_VRVZ_MEAN, k, j) +
                    (qz + R.qz[R.H(k, j + 1, i)]) * (qr * R.usrc[k] + qr_kp * R.usrc[kp]) * usnthm * 0.25;
            }
        }
    }
}

// CalcDissipation.F90:22-74: accumulates disste, returns nute.
double tcref_calc_dissipation(void* h) {
    TCRef& R = *(TCRef*)h;
    ensure_stats(R);
    double my_dissipte = 0.0;
    for (int i = 1; i <= R.nthm; ++i) {
        const int imm = i - 1, ipp = i + 1;
        for (int j = 1; j <= R.nzm; ++j) {
            const int jmm = j - 1, jpp = j + 1;
            for (int k = 1; k <= R.nrm; ++k) {
                const int kp = k + 1, kpp = R.kpv[k], kmm = R.kmv[k];
                const double e11 = (R.qt[R.H(k, j, ipp)] - R.qt[R.H(k, j, imm)]) * R.dxt * R.usrm[k] * 0.5
                                   + R.qr[R.H(k, j, i)] * sq(R.usrc[k]);
                const double e12 = (R.qt[R.H(kpp, j, i)] * R.usrm[kpp] - R.qt[R.H(kmm, j, i)] * R.usrm[kmm]) * R.udx2mm[k] * R.rm[k]
                                   + (R.qr[R.H(k, j, ipp)] - R.qr[R.H(k, j, imm)]) * R.usrc[k] * R.dxt * 0.5;
                const double e13 = (R.qt[R.H(k, jpp, i)] - R.qt[R.H(k, jmm, i)]) * 0.5 * R.dxz
                                   + (R.qz[R.H(k, j, ipp)] - R.qz[R.H(k, j, imm)]) * 0.5 * R.dxt * R.usrm[k];
                const double e22 = (R.qr[R.H(kp, j, i)] * R.usrc[kp] - R.qr[R.H(kmm, j, i)] * R.usrc[kmm]) * R.udx2cc[k];
                const double e23 = (R.qz[R.H(kpp, j, i)] - R.qz[R.H(kmm, j, i)]) * R.udx2mm[k]
                                   + (R.qr[R.H(k, jpp, i)] - R.qr[R.H(k, jmm, i)]) * R.usrc[k] * R.dxz * 0.5;
                const double e33 = (R.qz[R.H(k, jpp, i)] - R.qz[R.H(k, jmm, i)]) * R.dxz * 0.5;
                const double dissipte = 2.0 * (sq(e11) + sq(e22) + sq(e33)) + sq(e12) + sq(e13) + sq(e23);
                my_dissipte = my_dissipte + dissipte * R.pvol[k] * R.pi;
                R.st(TCREF_ST_DISSTE, k, j) = R.st(TCREF_ST_DISSTE, k, j) + dissipte / R.b.ren / (double)R.nthm;
            }
        }
    }
    const double volt = R.pi * (sq(R.b.rext) - sq(R.b.rint));
    const double lamdissip = 4.0 * sq(R.b.rext) * sq(R.b.rint) / sq(R.b.rext + R.b.rint) *
                             sq((R.b.virotint / R.b.rint - R.b.virotext / R.b.rext) / (R.b.rext - R.b.rint));
    return my_dissipte / ((double)R.nthm * (double)R.nzm * volt * lamdissip);
}

void tcref_get_stat(void* h, int which, double* out) {
    TCRef& R = *(TCRef*)h;
    ensure_stats(R);
    std::memcpy(out, &R.stats[(size_t)which * R.nrm * R.nzm], sizeof(double) * R.nrm * R.nzm);
}

int tcref_stat_samples(void* h) { return ((TCRef*)h)->nstatsamples; }

void tcref_get_vorticity(void* h, int comp, double* out) {
    TCRef& R = *(TCRef*)h;
    calc_vorticity(R);
    const std::vector<double>& v = comp == 0 ? R.vortt : (comp == 1 ? R.vortr : R.vortz);
    std::memcpy(out, v.data(), sizeof(double) * v.size());
}

// main.F90:152-226, step semantics only (no I/O).  IDTV=0 runs with
// dt = DTMAX (the reference never assigns dt in that branch).
int tcref_run(void* h, int ntime0, int nsteps, double* time, double* dtp) {
    TCRef& R = *(TCRef*)h;
    double t = *time, dt = *dtp;
    int errorcode = 0;
    for (int n = 0; n < nsteps; ++n) {
        int ntime = ntime0 + n;
        errorcode = 0;
        double instCFL = tcref_calc_max_cfl(h);
        if (R.b.idtv == 1) {
            if (ntime > 1) {
                if (instCFL < 1.0e-8) dt = R.b.dtmax;
                else dt = R.b.limitCFL / instCFL;
                if (dt > R.b.dtmax) dt = R.b.dtmax;
            } else {
                dt = R.b.dtmin;
            }
            if (dt < R.b.dtmin) errorcode = 166;
        } else {
            dt = R.b.dtmax;
            instCFL = instCFL * dt;
            if (instCFL > R.b.limitCFL) errorcode = 165;
        }
        tcref_time_marcher(h, dt, t);
        t = t + dt;
        if (ntime == 1 || std::fmod(t, R.b.tout) < dt) {
            double vmax[3], rms[3];
            tcref_calc_velocity_stats(h, vmax, rms);
            if (vmax[0] > R.b.limitVel && vmax[1] > R.b.limitVel) errorcode = 266;
            double dmax = tcref_check_divergence(h);
            if (std::fabs(dmax) > R.b.resid) errorcode = 169;
        }
        if (t > R.b.tmax) errorcode = 333;
        if (ntime == R.b.ntst) errorcode = 555;
        if (errorcode != 0) break;
    }
    *time = t;
    *dtp = dt;
    return errorcode;
}

}  // extern "C"
