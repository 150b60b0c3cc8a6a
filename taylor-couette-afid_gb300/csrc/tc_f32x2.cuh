// tc_f32x2.cuh -- pairs of FP32 values in one 64-bit register pair, with the
// packed FP32 instructions of sm_100-class GPUs (add/sub/mul/fma.rn.f32x2):
// one instruction issues the same operation on both lanes.  The FP32 march
// of the mixed path computes two theta-neighbouring cells a thread in this
// form; it is bound by instruction issue, and a packed instruction issues
// two cells' arithmetic at once.  Each lane rounds exactly as the scalar
// .rn instruction would.
#pragma once

namespace tcgb {

struct F2 {
    unsigned long long v;
};

__device__ __forceinline__ F2 mkf2(float x, float y) {
    F2 r;
    asm("mov.b64 %0, {%1, %2};" : "=l"(r.v) : "f"(x), "f"(y));
    return r;
}
__device__ __forceinline__ F2 bc2(float x) { return mkf2(x, x); }
__device__ __forceinline__ void f2xy(F2 a, float& x, float& y) { asm("mov.b64 {%0, %1}, %2;" : "=f"(x), "=f"(y) : "l"(a.v)); }
__device__ __forceinline__ float f2x(F2 a) { float x, y; f2xy(a, x, y); return x; }
__device__ __forceinline__ float f2y(F2 a) { float x, y; f2xy(a, x, y); return y; }

__device__ __forceinline__ F2 operator+(F2 a, F2 b) {
    F2 r;
    asm("add.rn.f32x2 %0, %1, %2;" : "=l"(r.v) : "l"(a.v), "l"(b.v));
    return r;
}
__device__ __forceinline__ F2 operator-(F2 a, F2 b) {
    F2 r;
    asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(r.v) : "l"(a.v), "l"(b.v));
    return r;
}
__device__ __forceinline__ F2 operator*(F2 a, F2 b) {
    F2 r;
    asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(r.v) : "l"(a.v), "l"(b.v));
    return r;
}
// a * b + c, each lane with one rounding
__device__ __forceinline__ F2 fma2(F2 a, F2 b, F2 c) {
    F2 r;
    asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(r.v) : "l"(a.v), "l"(b.v), "l"(c.v));
    return r;
}

// Store of two consecutive floats (8-byte aligned).
__device__ __forceinline__ void st_f2(float* p, F2 a) {
    float x, y;
    f2xy(a, x, y);
    *reinterpret_cast<float2*>(p) = make_float2(x, y);
}

}  // namespace tcgb
