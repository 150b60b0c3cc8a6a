// tc_fft.cuh -- shared-memory mixed-radix complex FFT (radix 2, 3, 4, 5, 7,
// 8, 11, 13), generic over the element type (double2 for the FP64 path,
// float2 for the mixed path).
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

#include <type_traits>

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

// 8-point DFT as two 4-point DFTs of the even and odd inputs joined by
// W8^k = exp(-+ i pi k / 4): 52 additions and 4 multiplications.
template <typename C2> __device__ __forceinline__ void dft8(C2* v, bool inv) {
    typedef decltype(v[0].x) R;
    const R h = (R)0.70710678118654752440;   // 1/sqrt(2)
    C2 e[4] = {v[0], v[2], v[4], v[6]}, o[4] = {v[1], v[3], v[5], v[7]};
    dft4(e, inv);
    dft4(o, inv);
    // o1 W8, o2 W8^2, o3 W8^3; forward W8 = (1 - i) h, inverse (1 + i) h
    const C2 t1 = inv ? mk2((o[1].x - o[1].y) * h, (o[1].y + o[1].x) * h)
                      : mk2((o[1].x + o[1].y) * h, (o[1].y - o[1].x) * h);
    const C2 t2 = inv ? mk2(-o[2].y, o[2].x) : mk2(o[2].y, -o[2].x);
    const C2 t3 = inv ? mk2(-(o[3].x + o[3].y) * h, (o[3].x - o[3].y) * h)
                      : mk2((o[3].y - o[3].x) * h, -(o[3].x + o[3].y) * h);
    v[0] = cadd(e[0], o[0]);
    v[4] = csub(e[0], o[0]);
    v[1] = cadd(e[1], t1);
    v[5] = csub(e[1], t1);
    v[2] = cadd(e[2], t2);
    v[6] = csub(e[2], t2);
    v[3] = cadd(e[3], t3);
    v[7] = csub(e[3], t3);
}

// ---- butterflies in fused multiply-adds (FP64 path) ----------------------
//
// The FP64 transforms are bound by the FP64 pipe, so they count FP64
// instructions.  A twiddle w = c + i s is stored factored (FTw): with
// z = y, or y with its parts swapped,
//     w y = (fx (z.x - g z.y), fy (z.y + g z.x)),
// where |c| >= |s| gives g = s/c, fx = fy = c and no swap, and |s| > |c| gives
// the swap, g = c/s, fx = -s, fy = s; so |g| <= 1.  The reduced product costs
// two FMAs and its scale folds into the FMAs that add it to the other input
// of the butterfly (x +- w y in four FMAs), against a complex product (four)
// and two complex additions (four) -- the factoring of Linzer and Feig
// (IBM J. Res. Dev. 1993) and Goedecker (SIAM J. Sci. Comput. 1997) for
// multiply-add units.  The swap is a register select on the integer pipes.
// A radix-4 butterfly as two levels of these radix-2 steps,
//     p, m = a0 +- w^2 a2,  u, v = a1 +- w^2 a3,
//     X0, X2 = p +- w u,    X1, X3 = m -+ i w v    (forward),
// costs 24 FP64 instructions against 28.  s = 0 gives g = 0, fx = fy = 1,
// which reproduces the plain sums exactly.
template <typename C2> struct CRe;
template <> struct CRe<double2> { typedef double type; };
template <> struct CRe<float2> { typedef float type; };

__device__ __forceinline__ FTw<double> ld_ftw(const FTw<double>* p) {
    const double2 a = __ldg(reinterpret_cast<const double2*>(p)), b = __ldg(reinterpret_cast<const double2*>(p) + 1);
    return {a.x, a.y, b.x, b.y};
}
__device__ __forceinline__ FTw<float> ld_ftw(const FTw<float>* p) {
    const float4 a = __ldg(reinterpret_cast<const float4*>(p));
    return {a.x, a.y, a.z, a.w};
}
__device__ __forceinline__ bool ftw_swapped(double s) { return __double_as_longlong(s) != 0; }
__device__ __forceinline__ bool ftw_swapped(float s) { return __float_as_int(s) != 0; }
__device__ __forceinline__ double fmar(double a, double b, double c) { return __fma_rn(a, b, c); }
__device__ __forceinline__ float fmar(float a, float b, float c) { return __fmaf_rn(a, b, c); }

// (z.x - g z.y, z.y + g z.x): w y = (fx r.x, fy r.y)
template <typename C2, typename R>
__device__ __forceinline__ C2 tw_reduce(C2 y, const FTw<R>& w) {
    const bool sw = ftw_swapped(w.swap);
    const R zx = sw ? y.y : y.x, zy = sw ? y.x : y.y;
    return mk2(fmar(-w.g, zy, zx), fmar(w.g, zx, zy));
}

// v[0], v[1] = v[0] +- w v[1]
template <typename C2, typename R>
__device__ __forceinline__ void bfly2_fma(C2* v, const FTw<R>& w) {
    const C2 y = tw_reduce(v[1], w);
    const C2 x = v[0];
    v[0] = mk2(fmar(w.fx, y.x, x.x), fmar(w.fy, y.y, x.y));
    v[1] = mk2(fmar(-w.fx, y.x, x.x), fmar(-w.fy, y.y, x.y));
}

// radix-4 DIT butterfly with twiddles w1 = w, w2 = w^2 (table of the
// transform's direction); inv selects the sign of i in the outputs
template <typename C2, typename R>
__device__ __forceinline__ void bfly4_fma(C2* v, const FTw<R>& w1, const FTw<R>& w2, bool inv) {
    const C2 y2 = tw_reduce(v[2], w2), y3 = tw_reduce(v[3], w2);
    const C2 p = mk2(fmar(w2.fx, y2.x, v[0].x), fmar(w2.fy, y2.y, v[0].y));
    const C2 m = mk2(fmar(-w2.fx, y2.x, v[0].x), fmar(-w2.fy, y2.y, v[0].y));
    const C2 u = mk2(fmar(w2.fx, y3.x, v[1].x), fmar(w2.fy, y3.y, v[1].y));
    const C2 d = mk2(fmar(-w2.fx, y3.x, v[1].x), fmar(-w2.fy, y3.y, v[1].y));
    const C2 yu = tw_reduce(u, w1), yd = tw_reduce(d, w1);
    v[0] = mk2(fmar(w1.fx, yu.x, p.x), fmar(w1.fy, yu.y, p.y));
    v[2] = mk2(fmar(-w1.fx, yu.x, p.x), fmar(-w1.fy, yu.y, p.y));
    // w1 d = (fx yd.x, fy yd.y); -i (w1 d) = (fy yd.y, -fx yd.x)
    const C2 mi = mk2(fmar(w1.fy, yd.y, m.x), fmar(-w1.fx, yd.x, m.y));   // m - i w1 d
    const C2 pi = mk2(fmar(-w1.fy, yd.y, m.x), fmar(w1.fx, yd.x, m.y));   // m + i w1 d
    v[1] = inv ? pi : mi;
    v[3] = inv ? mi : pi;
}

// The factored tables of a transform of length n follow its plain table
// (n entries, padded to an even count): n forward entries, then n inverse.
template <typename C2>
__device__ __forceinline__ const FTw<typename CRe<C2>::type>* ftw_table(const C2* tw, int n, bool inv) {
    return reinterpret_cast<const FTw<typename CRe<C2>::type>*>(tw + ((n + 1) & ~1)) + (inv ? n : 0);
}

// One Stockham stage of radix p (compile time) over C interleaved lines:
// sub-DFTs of length L become length L*p.  CT > 0: C = CT at compile time;
// CT = 0: C = 2^lgC known at run time.
// x / d with the plan's multiplier m (m = 0: d = 1).
__device__ __forceinline__ int fdiv(int x, unsigned m) { return m ? (int)__umulhi((unsigned)x, m) : x; }

template <int CT, int p, typename C2>
__device__ __forceinline__ void fft_stage(const C2* __restrict__ a, C2* __restrict__ b, int n, int L, int rp,
                                          unsigned mrp, const C2* __restrict__ tw, bool inv, int Crt, int lgC) {
    const int C = CT > 0 ? CT : Crt;
    typedef typename CRe<C2>::type R;
    // FP64 radix-4 and radix-2 stages after the first: factored butterflies
    constexpr bool kFused = std::is_same<R, double>::value && (p == 4 || p == 2);
    const FTw<R>* ftw = ftw_table(tw, n, inv);
    const int r = rp * p;
    const int nb = (n / p) * C;
    const int istep = rp * C, ostep = rp * L * C;
    for (int t = threadIdx.x; t < nb; t += blockDim.x) {
        const int c = CT > 0 ? t % CT : t & (C - 1), bf = CT > 0 ? t / CT : t >> lgC;
        const int s = fdiv(bf, mrp), q = bf - s * rp;
        const C2* in = a + (size_t)(q + r * s) * C + c;
        C2* out = b + (size_t)(q + rp * s) * C + c;
        C2 v[p];
#pragma unroll
        for (int cc = 0; cc < p; ++cc) v[cc] = in[cc * istep];
        if (kFused && L > 1) {
            const FTw<R> w1 = ld_ftw(ftw + s * rp);
            if constexpr (p == 4) bfly4_fma(v, w1, ld_ftw(ftw + 2 * s * rp), inv);
            else bfly2_fma(v, w1);
#pragma unroll
            for (int u = 0; u < p; ++u) out[u * ostep] = v[u];
            continue;
        }
        if (s != 0) {
#pragma unroll
            for (int cc = 1; cc < p; ++cc) v[cc] = cmul(v[cc], twiddle(tw, cc * s * rp, inv));
        }
        if constexpr (p == 8) dft8(v, inv);
        else if (p == 4) dft4(v, inv);
        else if (p == 2) dft2(v);
        else if (p == 3) dft3(v, inv);
        else dft5(v, inv);
#pragma unroll
        for (int u = 0; u < p; ++u) out[u * ostep] = v[u];
    }
}

// A Stockham stage of an odd prime radix P (7, 11, 13): every butterfly as a
// direct DFT that keeps one output in registers at a time.  For output k the
// P inputs are read again from shared memory, twiddled by w^(j s rp) and
// multiplied by exp(-+ 2 pi i jk / P) = entry (jk mod P) n/P of the
// transform's table.  These radices are rare; a stage of its own, out of
// line (rather than P values in registers in fft_stage), leaves the code and
// the register count of the common stages as they are.  Arguments as
// fft_stage.
template <int CT, int P, typename C2>
__device__ __noinline__ void fft_stage_prime(const C2* __restrict__ a, C2* __restrict__ b, int n, int L, int rp,
                                             unsigned mrp, const C2* __restrict__ tw, bool inv, int Crt, int lgC) {
    const int C = CT > 0 ? CT : Crt;
    const int r = rp * P, step = n / P;
    const int nb = (n / P) * C;
    const int istep = rp * C, ostep = rp * L * C;
#pragma unroll 1
    for (int t = threadIdx.x; t < nb; t += blockDim.x) {
        const int c = CT > 0 ? t % CT : t & (C - 1), bf = CT > 0 ? t / CT : t >> lgC;
        const int s = fdiv(bf, mrp), q = bf - s * rp;
        const C2* in = a + (size_t)(q + r * s) * C + c;
        C2* out = b + (size_t)(q + rp * s) * C + c;
        const int srp = L > 1 ? s * rp : 0;
#pragma unroll 1
        for (int k = 0; k < P; ++k) {
            C2 acc = in[0];
#pragma unroll 1
            for (int j = 1; j < P; ++j) {
                C2 x = in[j * istep];
                if (srp != 0) x = cmul(x, twiddle(tw, j * srp, inv));
                acc = cadd(acc, cmul(x, twiddle(tw, ((j * k) % P) * step, inv)));
            }
            out[k * ostep] = acc;
        }
    }
}

// Transform C interleaved lines of length P.n held in `a`; `b` is scratch of
// the same size.  All threads of the block must call it.  Returns the buffer
// that holds the result (a or b).
// fft_lines<C>: C lines, C known at compile time; fft_lines_n: C = 2^lgC
// lines known only at run time.  The arithmetic does not depend on C.
// PRIME: the stages of the radices 7, 11 and 13 are compiled in (kernels
// instantiated without them keep the code of the common stages exactly as
// it is; the launchers pick the instance with them for plans that need it).
template <int CT, bool PRIME, typename C2>
__device__ __forceinline__ C2* fft_lines_impl(C2* a, C2* b, const FFTPlan& P, const C2* tw, bool inv, int C, int lgC) {
    const int n = P.n;
    int L = 1;
    for (int st = 0; st < P.nstages; ++st) {
        const int p = P.radix[st], rp = P.rp[st];
        const unsigned m = P.mrp[st];
        if (p == 8) fft_stage<CT, 8>(a, b, n, L, rp, m, tw, inv, C, lgC);
        else if (p == 4) fft_stage<CT, 4>(a, b, n, L, rp, m, tw, inv, C, lgC);
        else if (p == 2) fft_stage<CT, 2>(a, b, n, L, rp, m, tw, inv, C, lgC);
        else if (p == 3) fft_stage<CT, 3>(a, b, n, L, rp, m, tw, inv, C, lgC);
        else if (!PRIME || p == 5) fft_stage<CT, 5>(a, b, n, L, rp, m, tw, inv, C, lgC);
        else if constexpr (PRIME) {
            if (p == 7) fft_stage_prime<CT, 7>(a, b, n, L, rp, m, tw, inv, C, lgC);
            else if (p == 11) fft_stage_prime<CT, 11>(a, b, n, L, rp, m, tw, inv, C, lgC);
            else fft_stage_prime<CT, 13>(a, b, n, L, rp, m, tw, inv, C, lgC);
        }
        __syncthreads();
        C2* t = a; a = b; b = t;
        L *= p;
    }
    return a;
}

constexpr int lines_log2(int c) { return c <= 1 ? 0 : 1 + lines_log2(c >> 1); }

template <int C, bool PRIME = true, typename C2>
__device__ C2* fft_lines(C2* a, C2* b, const FFTPlan& P, const C2* tw, bool inv) {
    return fft_lines_impl<C, PRIME>(a, b, P, tw, inv, C, 0);
}

template <bool PRIME = true, typename C2>
__device__ __forceinline__ C2* fft_lines_n(C2* a, C2* b, const FFTPlan& P, const C2* tw, bool inv, int C, int lgC) {
    return fft_lines_impl<0, PRIME>(a, b, P, tw, inv, C, lgC);
}

// Whether a plan has a stage of radix 7, 11 or 13 (host and device).
__host__ __device__ inline bool plan_has_prime(const FFTPlan& P) {
    for (int st = 0; st < P.nstages; ++st)
        if (P.radix[st] > 5 && P.radix[st] != 8) return true;
    return false;
}

}  // namespace tcgb
