"""Float-float arithmetic of the mixed path's pressure solve (csrc/tc_ff.cuh),
compiled for the host with IEEE single-precision operations standing in for
the device's _rn intrinsics: the error-free transformations are exact, sums
and products keep about 48 significant bits (1e-13 relative), and a nearly
singular tridiagonal LU solve in float-float agrees with FP64 to 1e-11 of
the solution's scale (the plain FP32 error is printed beside it)."""
import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "..", "taylor-couette-afid_gb300", "csrc")

HARNESS = r'''
#include <cmath>
#include <cstdio>
#include <cstdint>
#define __device__
#define __forceinline__ inline
static inline float __fadd_rn(float a, float b) { volatile float r = a + b; return r; }
static inline float __fsub_rn(float a, float b) { volatile float r = a - b; return r; }
static inline float __fmul_rn(float a, float b) { volatile float r = a * b; return r; }
static inline float __fmaf_rn(float a, float b, float c) { return std::fmaf(a, b, c); }
#include "tc_ff.cuh"
using namespace tcgb;

static uint64_t rs = 88172645463325252ull;
static double urand() { rs ^= rs << 13; rs ^= rs >> 7; rs ^= rs << 17; return (rs >> 11) * (1.0 / 9007199254740992.0); }
static ffv to_ff(double d) { float h = (float)d; return {h, (float)(d - (double)h)}; }
static double val(ffv a) { return (double)a.hi + (double)a.lo; }

int main() {
    int bad = 0;
    // error-free transformations
    for (int i = 0; i < 100000; ++i) {
        float a = (float)((urand() - 0.5) * 1e3), b = (float)((urand() - 0.5) * std::pow(10.0, 6 * urand() - 3));
        ffv s = ff_two_sum(a, b);
        if ((double)s.hi + (double)s.lo != (double)a + (double)b) { ++bad; break; }
        float x = std::fabs(a) >= std::fabs(b) ? a : b, y = std::fabs(a) >= std::fabs(b) ? b : a;
        ffv f = ff_fast_two_sum(x, y);
        if ((double)f.hi + (double)f.lo != (double)x + (double)y) { ++bad; break; }
    }
    std::printf("eft bad %d\n", bad);
    // add and mul against long double
    double worst_add = 0, worst_mul = 0;
    for (int i = 0; i < 100000; ++i) {
        double da = (urand() - 0.5) * std::pow(10.0, 8 * urand() - 4);
        double db = (urand() - 0.5) * std::pow(10.0, 8 * urand() - 4);
        ffv a = to_ff(da), b = to_ff(db);
        long double ea = (long double)val(a), eb = (long double)val(b);
        long double sa = ea + eb, pm = ea * eb;
        if (sa != 0) worst_add = std::fmax(worst_add, (double)fabsl(((long double)val(ff_add(a, b)) - sa) / sa));
        float fb = (float)db;
        long double sf = ea + (long double)fb;
        if (sf != 0) worst_add = std::fmax(worst_add, (double)fabsl(((long double)val(ff_add_f(a, fb)) - sf) / sf));
        if (pm != 0) worst_mul = std::fmax(worst_mul, (double)fabsl(((long double)val(ff_mul(a, b)) - pm) / pm));
    }
    std::printf("add %.3e mul %.3e\n", worst_add, worst_mul);
    if (worst_add > 1.0e-13 || worst_mul > 1.0e-13) ++bad;
    // nearly singular tridiagonal (second difference with a tiny shift), LU
    // forward and back as the pressure solve runs them
    const int n = 200;
    static double l[n], dinv[n], u[n], r[n];
    const double shift = 1e-6;
    double dp = -2.0 - shift;
    dinv[0] = 1.0 / dp;
    for (int k = 0; k < n; ++k) { u[k] = 1.0; r[k] = std::sin(0.1 * k) + 0.3; }
    for (int k = 1; k < n; ++k) { l[k] = 1.0 / dp; dp = -2.0 - shift - l[k] * 1.0; dinv[k] = 1.0 / dp; }
    // FP64
    static double y[n], x[n];
    y[0] = r[0];
    for (int k = 1; k < n; ++k) y[k] = r[k] - l[k] * y[k - 1];
    x[n - 1] = y[n - 1] * dinv[n - 1];
    for (int k = n - 2; k >= 0; --k) x[k] = (y[k] - u[k] * x[k + 1]) * dinv[k];
    // float-float (rhs given in FP32 as in the mixed path)
    static ffv yf[n];
    yf[0] = ff_from((float)r[0]);
    for (int k = 1; k < n; ++k) yf[k] = ff_add_f(ff_neg(ff_mul(to_ff(l[k]), yf[k - 1])), (float)r[k]);
    ffv s = ff_mul(yf[n - 1], to_ff(dinv[n - 1]));
    double err_ff = 0, err_f = 0, xmax = 0;
    static double y32[n];
    for (int k = 0; k < n; ++k) y32[k] = (double)(float)r[k];
    // FP64 reference with the same FP32-rounded right-hand side
    static double yr[n], xr[n];
    yr[0] = y32[0];
    for (int k = 1; k < n; ++k) yr[k] = y32[k] - l[k] * yr[k - 1];
    xr[n - 1] = yr[n - 1] * dinv[n - 1];
    for (int k = n - 2; k >= 0; --k) xr[k] = (yr[k] - u[k] * xr[k + 1]) * dinv[k];
    for (int k = 0; k < n; ++k) xmax = std::fmax(xmax, std::fabs(xr[k]));
    err_ff = std::fabs(val(s) - xr[n - 1]);
    for (int k = n - 2; k >= 0; --k) {
        s = ff_mul(ff_sub(yf[k], ff_mul(to_ff(u[k]), s)), to_ff(dinv[k]));
        err_ff = std::fmax(err_ff, std::fabs(val(s) - xr[k]));
    }
    // plain FP32 for comparison
    static float yy[n];
    yy[0] = (float)r[0];
    for (int k = 1; k < n; ++k) yy[k] = (float)r[k] - (float)l[k] * yy[k - 1];
    float xs = yy[n - 1] * (float)dinv[n - 1];
    err_f = std::fabs(xs - xr[n - 1]);
    for (int k = n - 2; k >= 0; --k) {
        xs = (yy[k] - (float)u[k] * xs) * (float)dinv[k];
        err_f = std::fmax(err_f, std::fabs(xs - xr[k]));
    }
    std::printf("solve: ff %.3e fp32 %.3e (relative to max |x| = %.3e)\n", err_ff / xmax, err_f / xmax, xmax);
    if (err_ff / xmax > 1e-11) ++bad;
    std::printf("bad %d\n", bad);
    return bad != 0;
}
'''


def test_float_float_arithmetic(tmp_path):
    if shutil.which("g++") is None:
        pytest.skip("no host C++ compiler")
    cpp = tmp_path / "ff.cpp"
    cpp.write_text(HARNESS)
    exe = tmp_path / "ff"
    subprocess.run(["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-I", CSRC, str(cpp), "-o", str(exe)],
                   check=True)
    r = subprocess.run([str(exe)], capture_output=True, text=True)
    print(r.stdout)
    assert r.returncode == 0, r.stdout
