// tc_convert.cuh -- binary32 <-> binary64 conversions on the integer pipes.
//
// On GB300 the hardware conversions between float and double issue on the
// FP64 pipe, which runs at 2 instructions per clock per SM; the mixed path
// converts at every access to its FP64 pressure data, so those conversions
// would set the speed of its pressure kernels.  These functions do the same
// conversions by rearranging the IEEE-754 fields (sign, exponent re-biased by
// 1023 - 127 = 896, mantissa shifted by 29 bits, round to nearest even when
// narrowing) with 32-bit integer instructions, and fall back to the hardware
// conversion only for the rare operands outside the normal range (subnormal
// results, infinities, NaN), so every result equals the hardware's.
#pragma once

#include <cuda_runtime.h>

namespace tcgb {

// float -> double (exact).
__device__ __forceinline__ double f2d(float f) {
    const unsigned u = __float_as_uint(f);
    const unsigned e = (u >> 23) & 0xffu;
    const unsigned s = u & 0x80000000u;
    if (e - 1u < 0xfeu)   // normal: 1 <= e <= 254
        return __hiloint2double((int)(s | ((e + 896u) << 20) | ((u >> 3) & 0xfffffu)), (int)(u << 29));
    if ((u << 1) == 0u) return __hiloint2double((int)s, 0);   // signed zero
    return (double)f;                                        // subnormal, inf, nan
}

// double -> float, round to nearest even.
__device__ __forceinline__ float d2f(double d) {
    const unsigned hi = (unsigned)__double2hiint(d), lo = (unsigned)__double2loint(d);
    const unsigned s = hi & 0x80000000u;
    const int e = (int)((hi >> 20) & 0x7ffu) - 896;          // binary32 biased exponent
    if (e >= 1 && e <= 254) {
        const unsigned m = ((hi & 0xfffffu) << 3) | (lo >> 29);   // top 23 mantissa bits
        const unsigned rest = lo & 0x1fffffffu;                   // the 29 dropped bits
        unsigned r = ((unsigned)e << 23) | m;
        // a carry out of the mantissa bumps the exponent, and past 254 gives inf
        if (rest > 0x10000000u || (rest == 0x10000000u && (m & 1u))) r += 1u;
        return __uint_as_float(s | r);
    }
    if (((hi << 1) | lo) == 0u) return __uint_as_float(s);    // signed zero
    return (float)d;                                          // tiny, huge, inf, nan
}

__device__ __forceinline__ double2 f2d(float2 v) { return make_double2(f2d(v.x), f2d(v.y)); }

}  // namespace tcgb
