// tc_fft.cuh -- shared-memory mixed-radix complex FFT (radix 2, 3, 4, 5).
//
// Stockham autosort, decimation in time, out of place between two
// shared-memory buffers.  C independent lines are stored interleaved: element
// idx of line c lives at buf[idx * C + c].  After a stage with radix p the
// buffer holds, for every sub-sequence q of stride r' = n/(L p), its DFT of
// length L p at index q + r' * s (s = frequency); the last stage leaves the
// full DFT in natural order.  Forward uses exp(-2 pi i j k / n), inverse
// exp(+...), both unnormalised (the FFTW conventions the reference's
// SolvePressureCorrection.F90:61-98 plans use).
#pragma once

#include "tc_dev.h"

namespace tcgb {

__device__ __forceinline__ double2 cadd(double2 a, double2 b) { return make_double2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ double2 csub(double2 a, double2 b) { return make_double2(a.x - b.x, a.y - b.y); }
__device__ __forceinline__ double2 cmul(double2 a, double2 b) {
    return make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
__device__ __forceinline__ double2 cconj(double2 a) { return make_double2(a.x, -a.y); }

// Twiddle exp(-+ 2 pi i idx / n) from the forward table.
__device__ __forceinline__ double2 twiddle(const double2* tw, int idx, bool inv) {
    double2 w = __ldg(tw + idx);
    if (inv) w.y = -w.y;
    return w;
}

// p-point DFTs on v[0..p-1] (in place).
__device__ __forceinline__ void dft2(double2* v) {
    double2 a = v[0], b = v[1];
    v[0] = cadd(a, b);
    v[1] = csub(a, b);
}

__device__ __forceinline__ void dft4(double2* v, bool inv) {
    double2 a0 = cadd(v[0], v[2]), a1 = csub(v[0], v[2]);
    double2 a2 = cadd(v[1], v[3]), a3 = csub(v[1], v[3]);
    v[0] = cadd(a0, a2);
    v[2] = csub(a0, a2);
    // forward: w1 = a1 - i a3, w3 = a1 + i a3
    double2 m = make_double2(a1.x + a3.y, a1.y - a3.x);   // a1 - i a3
    double2 p = make_double2(a1.x - a3.y, a1.y + a3.x);   // a1 + i a3
    v[1] = inv ? p : m;
    v[3] = inv ? m : p;
}

__device__ __forceinline__ void dft3(double2* v, bool inv) {
    // cos(2 pi/3) = -1/2, sin(2 pi/3) = sqrt(3)/2
    const double s3 = 0.86602540378443864676;
    double2 t = cadd(v[1], v[2]), d = csub(v[1], v[2]);
    double2 w0 = cadd(v[0], t);
    double2 m = make_double2(v[0].x - 0.5 * t.x, v[0].y - 0.5 * t.y);
    double2 a = make_double2(m.x + s3 * d.y, m.y - s3 * d.x);   // m - i s3 d
    double2 b = make_double2(m.x - s3 * d.y, m.y + s3 * d.x);   // m + i s3 d
    v[0] = w0;
    v[1] = inv ? b : a;
    v[2] = inv ? a : b;
}

__device__ __forceinline__ void dft5(double2* v, bool inv) {
    // c1 = cos(2 pi/5) = (sqrt5-1)/4, c2 = cos(4 pi/5) = -(sqrt5+1)/4,
    // s1 = sin(2 pi/5), s2 = sin(4 pi/5)
    const double c1 = 0.30901699437494742410, c2 = -0.80901699437494742410;
    const double s1 = 0.95105651629515357212, s2 = 0.58778525229247312917;
    double2 a1 = cadd(v[1], v[4]), b1 = csub(v[1], v[4]);
    double2 a2 = cadd(v[2], v[3]), b2 = csub(v[2], v[3]);
    double2 w0 = make_double2(v[0].x + a1.x + a2.x, v[0].y + a1.y + a2.y);
    double2 m1 = make_double2(v[0].x + c1 * a1.x + c2 * a2.x, v[0].y + c1 * a1.y + c2 * a2.y);
    double2 m2 = make_double2(v[0].x + c2 * a1.x + c1 * a2.x, v[0].y + c2 * a1.y + c1 * a2.y);
    double2 n1 = make_double2(s1 * b1.x + s2 * b2.x, s1 * b1.y + s2 * b2.y);
    double2 n2 = make_double2(s2 * b1.x - s1 * b2.x, s2 * b1.y - s1 * b2.y);
    // forward: w1 = m1 - i n1, w4 = m1 + i n1, w2 = m2 - i n2, w3 = m2 + i n2
    double2 w1 = make_double2(m1.x + n1.y, m1.y - n1.x), w4 = make_double2(m1.x - n1.y, m1.y + n1.x);
    double2 w2 = make_double2(m2.x + n2.y, m2.y - n2.x), w3 = make_double2(m2.x - n2.y, m2.y + n2.x);
    v[0] = w0;
    v[1] = inv ? w4 : w1;
    v[4] = inv ? w1 : w4;
    v[2] = inv ? w3 : w2;
    v[3] = inv ? w2 : w3;
}

// Transform C interleaved lines of length P.n held in `a`; `b` is scratch of
// the same size.  All threads of the block must call it.  Returns the buffer
// that holds the result (a or b).
template <int C>
__device__ double2* fft_lines(double2* a, double2* b, const FFTPlan& P, bool inv) {
    const int n = P.n;
    int L = 1;
    for (int st = 0; st < P.nstages; ++st) {
        const int p = P.radix[st];
        const int Lp = L * p, rp = n / Lp, r = rp * p;
        const int nb = (n / p) * C;
        for (int t = threadIdx.x; t < nb; t += blockDim.x) {
            const int c = t % C, bf = t / C;
            const int q = bf % rp, s = bf / rp;
            const double2* in = a + (size_t)(q + r * s) * C + c;
            double2* out = b + (size_t)(q + rp * s) * C + c;
            const int istep = rp * C, ostep = rp * L * C;
            double2 v[5];
            for (int cc = 0; cc < p; ++cc) v[cc] = in[cc * istep];
            if (s != 0)
                for (int cc = 1; cc < p; ++cc) v[cc] = cmul(v[cc], twiddle(P.tw, cc * s * rp, inv));
            switch (p) {
                case 4: dft4(v, inv); break;
                case 2: dft2(v); break;
                case 3: dft3(v, inv); break;
                default: dft5(v, inv); break;
            }
            for (int u = 0; u < p; ++u) out[u * ostep] = v[u];
        }
        __syncthreads();
        double2* t = a; a = b; b = t;
        L = Lp;
    }
    return a;
}

}  // namespace tcgb
