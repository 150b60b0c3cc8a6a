// tc_fft.cuh -- shared-memory mixed-radix complex FFT (radix 2, 3, 4, 5),
// generic over the element type (double2 for the FP64 path, float2 for the
// mixed path).
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

__device__ __forceinline__ double2 mk2(double a, double b) { return make_double2(a, b); }
__device__ __forceinline__ float2 mk2(float a, float b) { return make_float2(a, b); }

template <typename C2> __device__ __forceinline__ C2 cadd(C2 a, C2 b) { return mk2(a.x + b.x, a.y + b.y); }
template <typename C2> __device__ __forceinline__ C2 csub(C2 a, C2 b) { return mk2(a.x - b.x, a.y - b.y); }
template <typename C2> __device__ __forceinline__ C2 cmul(C2 a, C2 b) {
    return mk2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
template <typename C2> __device__ __forceinline__ C2 cconj(C2 a) { return mk2(a.x, -a.y); }

// Twiddle exp(-+ 2 pi i idx / n) from the forward table.
template <typename C2> __device__ __forceinline__ C2 twiddle(const C2* tw, int idx, bool inv) {
    C2 w = __ldg(tw + idx);
    if (inv) w.y = -w.y;
    return w;
}

// p-point DFTs on v[0..p-1] (in place).
template <typename C2> __device__ __forceinline__ void dft2(C2* v) {
    C2 a = v[0], b = v[1];
    v[0] = cadd(a, b);
    v[1] = csub(a, b);
}

template <typename C2> __device__ __forceinline__ void dft4(C2* v, bool inv) {
    C2 a0 = cadd(v[0], v[2]), a1 = csub(v[0], v[2]);
    C2 a2 = cadd(v[1], v[3]), a3 = csub(v[1], v[3]);
    v[0] = cadd(a0, a2);
    v[2] = csub(a0, a2);
    // forward: w1 = a1 - i a3, w3 = a1 + i a3
    C2 m = mk2(a1.x + a3.y, a1.y - a3.x);   // a1 - i a3
    C2 p = mk2(a1.x - a3.y, a1.y + a3.x);   // a1 + i a3
    v[1] = inv ? p : m;
    v[3] = inv ? m : p;
}

template <typename C2> __device__ __forceinline__ void dft3(C2* v, bool inv) {
    typedef decltype(v[0].x) R;
    // cos(2 pi/3) = -1/2, sin(2 pi/3) = sqrt(3)/2
    const R s3 = (R)0.86602540378443864676, h = (R)0.5;
    C2 t = cadd(v[1], v[2]), d = csub(v[1], v[2]);
    C2 w0 = cadd(v[0], t);
    C2 m = mk2(v[0].x - h * t.x, v[0].y - h * t.y);
    C2 a = mk2(m.x + s3 * d.y, m.y - s3 * d.x);   // m - i s3 d
    C2 b = mk2(m.x - s3 * d.y, m.y + s3 * d.x);   // m + i s3 d
    v[0] = w0;
    v[1] = inv ? b : a;
    v[2] = inv ? a : b;
}

template <typename C2> __device__ __forceinline__ void dft5(C2* v, bool inv) {
    typedef decltype(v[0].x) R;
    // c1 = cos(2 pi/5) = (sqrt5-1)/4, c2 = cos(4 pi/5) = -(sqrt5+1)/4,
    // s1 = sin(2 pi/5), s2 = sin(4 pi/5)
    const R c1 = (R)0.30901699437494742410, c2 = (R)-0.80901699437494742410;
    const R s1 = (R)0.95105651629515357212, s2 = (R)0.58778525229247312917;
    C2 a1 = cadd(v[1], v[4]), b1 = csub(v[1], v[4]);
    C2 a2 = cadd(v[2], v[3]), b2 = csub(v[2], v[3]);
    C2 w0 = mk2(v[0].x + a1.x + a2.x, v[0].y + a1.y + a2.y);
    C2 m1 = mk2(v[0].x + c1 * a1.x + c2 * a2.x, v[0].y + c1 * a1.y + c2 * a2.y);
    C2 m2 = mk2(v[0].x + c2 * a1.x + c1 * a2.x, v[0].y + c2 * a1.y + c1 * a2.y);
    C2 n1 = mk2(s1 * b1.x + s2 * b2.x, s1 * b1.y + s2 * b2.y);
    C2 n2 = mk2(s2 * b1.x - s1 * b2.x, s2 * b1.y - s1 * b2.y);
    // forward: w1 = m1 - i n1, w4 = m1 + i n1, w2 = m2 - i n2, w3 = m2 + i n2
    C2 w1 = mk2(m1.x + n1.y, m1.y - n1.x), w4 = mk2(m1.x - n1.y, m1.y + n1.x);
    C2 w2 = mk2(m2.x + n2.y, m2.y - n2.x), w3 = mk2(m2.x - n2.y, m2.y + n2.x);
    v[0] = w0;
    v[1] = inv ? w4 : w1;
    v[4] = inv ? w1 : w4;
    v[2] = inv ? w3 : w2;
    v[3] = inv ? w2 : w3;
}

// One Stockham stage of radix p (compile time) over C interleaved lines:
// sub-DFTs of length L become length L*p.
// x / d with the plan's multiplier m (m = 0: d = 1).
__device__ __forceinline__ int fdiv(int x, unsigned m) { return m ? (int)__umulhi((unsigned)x, m) : x; }

template <int C, int p, typename C2>
__device__ __forceinline__ void fft_stage(const C2* __restrict__ a, C2* __restrict__ b, int n, int L, int rp,
                                          unsigned mrp, const C2* __restrict__ tw, bool inv) {
    const int r = rp * p;
    const int nb = (n / p) * C;
    const int istep = rp * C, ostep = rp * L * C;
    for (int t = threadIdx.x; t < nb; t += blockDim.x) {
        const int c = t % C, bf = t / C;
        const int s = fdiv(bf, mrp), q = bf - s * rp;
        const C2* in = a + (size_t)(q + r * s) * C + c;
        C2* out = b + (size_t)(q + rp * s) * C + c;
        C2 v[p];
#pragma unroll
        for (int cc = 0; cc < p; ++cc) v[cc] = in[cc * istep];
        if (s != 0) {
#pragma unroll
            for (int cc = 1; cc < p; ++cc) v[cc] = cmul(v[cc], twiddle(tw, cc * s * rp, inv));
        }
        if (p == 4) dft4(v, inv);
        else if (p == 2) dft2(v);
        else if (p == 3) dft3(v, inv);
        else dft5(v, inv);
#pragma unroll
        for (int u = 0; u < p; ++u) out[u * ostep] = v[u];
    }
}

// Transform C interleaved lines of length P.n held in `a`; `b` is scratch of
// the same size.  All threads of the block must call it.  Returns the buffer
// that holds the result (a or b).
template <int C, typename C2>
__device__ C2* fft_lines(C2* a, C2* b, const FFTPlan& P, const C2* tw, bool inv) {
    const int n = P.n;
    int L = 1;
    for (int st = 0; st < P.nstages; ++st) {
        const int p = P.radix[st], rp = P.rp[st];
        const unsigned m = P.mrp[st];
        if (p == 4) fft_stage<C, 4>(a, b, n, L, rp, m, tw, inv);
        else if (p == 2) fft_stage<C, 2>(a, b, n, L, rp, m, tw, inv);
        else if (p == 3) fft_stage<C, 3>(a, b, n, L, rp, m, tw, inv);
        else fft_stage<C, 5>(a, b, n, L, rp, m, tw, inv);
        __syncthreads();
        C2* t = a; a = b; b = t;
        L *= p;
    }
    return a;
}

}  // namespace tcgb
