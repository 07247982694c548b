// packed.cuh - two FP32 lanes in one value (V2) on the sm_100 packed
// FP32x2 instructions (FFMA2 / FADD2 / FMUL2: one instruction performs the
// same operation on both lanes), and the correctly rounded elementary
// operations the stencils use on it.
#pragma once
#include <cuda_runtime.h>

namespace pflbm {

// Two FP32 lanes, one per node of the pair.
struct V2 {
    float2 v;
    V2() = default;
    __device__ __forceinline__ V2(float2 a) : v(a) {}
    __device__ __forceinline__ V2(float a, float b) : v(make_float2(a, b)) {}
    __device__ __forceinline__ explicit V2(float s) : v(make_float2(s, s)) {}
    __device__ __forceinline__ explicit V2(double s) : v(make_float2(float(s), float(s))) {}
    __device__ __forceinline__ explicit V2(int s) : v(make_float2(float(s), float(s))) {}
};
__device__ __forceinline__ V2 operator+(V2 a, V2 b) { return V2(__fadd2_rn(a.v, b.v)); }
__device__ __forceinline__ V2 operator*(V2 a, V2 b) { return V2(__fmul2_rn(a.v, b.v)); }
__device__ __forceinline__ V2 fma2(V2 a, V2 b, V2 c) { return V2(__ffma2_rn(a.v, b.v, c.v)); }
// packed subtraction (PTX sub.rn.f32x2; the CUDA headers declare only the
// fma/add/mul forms)
__device__ __forceinline__ V2 operator-(V2 a, V2 b) {
    unsigned long long r;
    asm("sub.rn.f32x2 %0, %1, %2;"
        : "=l"(r)
        : "l"(*reinterpret_cast<const unsigned long long *>(&a.v)), "l"(*reinterpret_cast<const unsigned long long *>(&b.v)));
    return V2(*reinterpret_cast<const float2 *>(&r));
}
__device__ __forceinline__ V2 operator-(V2 a) { return V2(0.0f) - a; }
__device__ __forceinline__ V2 &operator+=(V2 &a, V2 b) { return a = a + b; }
// 1/a per lane: IEEE division, or (FAST: 16-bit storage, where the stored
// value carries 11 or 8 significant bits) the hardware approximate reciprocal
// of __fdividef, good to about 2 ulp of FP32
template <bool FAST>
__device__ __forceinline__ V2 recip2(V2 a) {
    if constexpr (FAST) return V2(__fdividef(1.0f, a.v.x), __fdividef(1.0f, a.v.y));
    else return V2(1.0f / a.v.x, 1.0f / a.v.y);
}

// Stencil operations on V2 (see stencil.cuh for the scalar forms).
__device__ __forceinline__ V2 op_mul(V2 a, V2 b) { return a * b; }
__device__ __forceinline__ V2 op_add(V2 a, V2 b) { return a + b; }
__device__ __forceinline__ V2 op_fma(V2 a, V2 b, V2 c) { return fma2(a, b, c); }
__device__ __forceinline__ V2 op_sqrt(V2 a) { return V2(sqrtf(a.v.x), sqrtf(a.v.y)); }
__device__ __forceinline__ V2 op_sqrt_approx(V2 a) {
    float rx, ry;
    asm("sqrt.approx.f32 %0, %1;" : "=f"(rx) : "f"(a.v.x));
    asm("sqrt.approx.f32 %0, %1;" : "=f"(ry) : "f"(a.v.y));
    return V2(rx, ry);
}
template <bool FAST>
__device__ __forceinline__ V2 op_recip(V2 a) { return recip2<FAST>(a); }

}  // namespace pflbm
