// tc_selftest.cu -- device self-checks of helpers that replace hardware
// instructions: the integer-pipe float <-> double conversions of
// tc_convert.cuh must give the same bits as the hardware conversions.

#include <cuda_runtime.h>

#include "../../include/tc_capi.h"
#include "tc_convert.cuh"

namespace {

__device__ __forceinline__ unsigned long long mix64(unsigned long long x) {
    // SplitMix64 finaliser
    x += 0x9E3779B97F4A7C15ull;
    x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
    x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
    return x ^ (x >> 31);
}

// Operands: random bit patterns, doubles with exponents around the binary32
// range (normal, subnormal and overflow boundaries), and exact and near
// halfway cases of the binary32 rounding.
__global__ void conv_check_kernel(long long n, unsigned long long* bad) {
    unsigned long long local = 0;
    for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (long long)gridDim.x * blockDim.x) {
        const unsigned long long h = mix64((unsigned long long)t), g = mix64(h);
        // float -> double
        const unsigned fb = (unsigned)h;
        const float f = __uint_as_float(fb);
        const double want_d = (double)f;
        const double got_d = tcgb::f2d(f);
        if (want_d == want_d && __double_as_longlong(want_d) != __double_as_longlong(got_d)) ++local;
        if (want_d != want_d && got_d == got_d) ++local;
        // double -> float
        unsigned long long db = g;
        const int kind = (int)(h >> 60);
        if (kind < 12) {
            // exponent in [896 - 40, 896 + 260]: binary32 subnormal .. overflow
            const unsigned long long e = 856ull + (h >> 32) % 300ull;
            db = (g & 0x800FFFFFFFFFFFFFull) | (e << 52);
            if (kind < 4) db = (db & ~0x1FFFFFFFull) | 0x10000000ull;               // exact halfway
            else if (kind < 6) db = (db & ~0x1FFFFFFFull) | (0x10000000ull + (kind & 1 ? 1 : -1));
        }
        const double d = __longlong_as_double((long long)db);
        const float want_f = (float)d;
        const float got_f = tcgb::d2f(d);
        if (want_f == want_f && __float_as_uint(want_f) != __float_as_uint(got_f)) ++local;
        if (want_f != want_f && got_f == got_f) ++local;
    }
    if (local) atomicAdd(bad, local);
}

}  // namespace

// Declared extern "C" in tc_capi.h.
int tc_selftest_conversions(long long n, long long* mismatches) {
    if (n < 0 || !mismatches) return 2000;
    unsigned long long* dbad = nullptr;
    cudaError_t c = cudaMalloc(&dbad, sizeof *dbad);
    if (c != cudaSuccess) return 1000 + (int)c;
    c = cudaMemset(dbad, 0, sizeof *dbad);
    if (c == cudaSuccess) {
        conv_check_kernel<<<608, 256>>>(n, dbad);
        c = cudaGetLastError();
    }
    unsigned long long bad = 0;
    if (c == cudaSuccess) c = cudaMemcpy(&bad, dbad, sizeof bad, cudaMemcpyDeviceToHost);
    cudaFree(dbad);
    if (c != cudaSuccess) return 1000 + (int)c;
    *mismatches = (long long)bad;
    return 0;
}
