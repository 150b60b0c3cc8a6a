"""The shared-memory FFT engine (csrc/tc_fft.cuh) and its plans and twiddle
tables (csrc/tc_capi.cu), compiled for the host from the same source text
with single-thread shims for the CUDA built-ins, against a direct DFT in long
double: every radix (2, 3, 4, 5, 7, 8, 11, 13), the factored multiply-add
butterflies of the FP64 stages, both directions, FP64 and FP32, lengths from
2 to 1536.
Relative max error below 1e-13 (FP64) and 2e-6 (FP32)."""
import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "..", "taylor-couette-afid_gb300", "csrc")

SHIMS = r'''
#include <cmath>
#include <cstdio>
#include <cstring>
#include <cstdlib>
#include <vector>
#include <type_traits>
#define __device__
#define __host__
#define __forceinline__ inline
#define __noinline__ __attribute__((noinline))
#define __restrict__
struct double2 { double x, y; };
struct float2 { float x, y; };
struct float4 { float x, y, z, w; };
inline double2 make_double2(double a, double b) { return {a, b}; }
inline float4 make_float4(float a, float b, float c, float d) { return {a, b, c, d}; }
inline float2 make_float2(float a, float b) { return {a, b}; }
template <typename T> inline T __ldg(const T* p) { return *p; }
inline double __fma_rn(double a, double b, double c) { return std::fma(a, b, c); }
inline float __fmaf_rn(float a, float b, float c) { return std::fmaf(a, b, c); }
inline long long __double_as_longlong(double v) { long long r; std::memcpy(&r, &v, 8); return r; }
inline int __float_as_int(float v) { int r; std::memcpy(&r, &v, 4); return r; }
inline unsigned __umulhi(unsigned a, unsigned b) { return (unsigned)(((unsigned long long)a * b) >> 32); }
struct { int x = 0; } threadIdx;
struct { int x = 1; } blockDim;
inline void __syncthreads() {}
namespace tcgb {
%(dev)s
%(fft)s
%(plan)s
}
using namespace tcgb;

template <typename C2>
double run(int n, bool r8, bool inv, unsigned seed) {
    constexpr int C = 4;
    FFTPlan P;
    if (!make_plan(n, P, r8)) { std::printf("no plan for %%d\n", n); std::exit(2); }
    std::vector<C2> tw = twiddles_with_factored<C2>(n);
    std::vector<C2> a((size_t)n * C), b((size_t)n * C);
    std::vector<long double> xr((size_t)n * C), xi((size_t)n * C);
    unsigned s = seed;
    for (size_t t = 0; t < a.size(); ++t) {
        s = s * 1664525u + 1013904223u; double u = (s >> 8) / 16777216.0 - 0.5;
        s = s * 1664525u + 1013904223u; double v = (s >> 8) / 16777216.0 - 0.5;
        a[t].x = (decltype(a[t].x))u; a[t].y = (decltype(a[t].y))v;
        xr[t] = a[t].x; xi[t] = a[t].y;
    }
    C2* out = fft_lines<C>(a.data(), b.data(), P, tw.data(), inv);
    const long double tpi = 6.283185307179586476925286766559L, sg = inv ? 1.0L : -1.0L;
    double err = 0.0, nrm = 0.0;
    for (int c = 0; c < C; ++c)
        for (int k = 0; k < n; ++k) {
            long double re = 0, im = 0;
            for (int j = 0; j < n; ++j) {
                const long double ang = sg * tpi * (long double)((long long)j * k %% n) / n;
                const long double cr = cosl(ang), ci = sinl(ang);
                re += xr[(size_t)j * C + c] * cr - xi[(size_t)j * C + c] * ci;
                im += xr[(size_t)j * C + c] * ci + xi[(size_t)j * C + c] * cr;
            }
            const C2 o = out[(size_t)k * C + c];
            err = std::fmax(err, (double)std::fabs((long double)o.x - re));
            err = std::fmax(err, (double)std::fabs((long double)o.y - im));
            nrm = std::fmax(nrm, (double)std::fmax(std::fabs(re), std::fabs(im)));
        }
    return err / nrm;
}

int main() {
    const int sizes[] = {2, 3, 4, 5, 6, 7, 8, 10, 11, 12, 13, 14, 16, 22, 26, 30, 40, 48, 56, 64, 77, 91, 96, 128,
                         143, 160, 168, 256, 384, 448, 512, 768, 1001, 1536};
    int bad = 0;
    for (int n : sizes)
        for (int r8 = 0; r8 < 2; ++r8)
            for (int inv = 0; inv < 2; ++inv) {
                const double ed = run<double2>(n, r8, inv, 12345u + n);
                const double ef = run<float2>(n, r8, inv, 54321u + n);
                const bool ok = ed < 1e-13 && ef < 2e-6;
                if (!ok) { std::printf("n %%d r8 %%d inv %%d: fp64 %%.3g fp32 %%.3g\n", n, r8, inv, ed, ef); ++bad; }
            }
    std::printf("bad %%d\n", bad);
    return bad != 0;
}
'''


def _extract(src, start, end):
    a = src.index(start)
    return src[a:src.index(end, a)]


def test_fft_engine_matches_direct_dft(tmp_path):
    if shutil.which("g++") is None:
        pytest.skip("no host C++ compiler")
    dev = open(os.path.join(CSRC, "tc_dev.h")).read()
    fft = open(os.path.join(CSRC, "tc_fft.cuh")).read()
    capi = open(os.path.join(CSRC, "tc_capi.cu")).read()
    dev_part = ("constexpr int kMaxStages = 24;\n" +
                _extract(dev, "struct FFTPlan {", "struct Dims {"))
    assert "constexpr int kMaxStages = 24;" in dev
    fft_part = _extract(fft, "__device__ __forceinline__ double2 mk2(", "}  // namespace tcgb")
    plan_part = (_extract(capi, "bool make_plan(int n, FFTPlan& P, bool r8) {", "// exp(-2 pi i j / n)") +
                 _extract(capi, "template <typename C2>\nstd::vector<C2> twiddles(int n, int count) {",
                          "int check(tc_handle* h) {"))
    cpp = tmp_path / "fft.cpp"
    cpp.write_text(SHIMS % {"dev": dev_part, "fft": fft_part, "plan": plan_part})
    exe = tmp_path / "fft"
    subprocess.run(["g++", "-O2", "-std=c++17", "-ffp-contract=off", str(cpp), "-o", str(exe)], check=True,
                   capture_output=True)
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
