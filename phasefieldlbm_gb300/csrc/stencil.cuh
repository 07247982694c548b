// stencil.cuh - the lattice-weighted central gradient of the phi normals and
// curvature stencils, with compile-time direction offsets.
#pragma once
#include <cuda_runtime.h>

#include <utility>

#include "lattice.cuh"

namespace pflbm {

// Correctly rounded elementary operations (never contracted), so that the
// scalar stencils and their packed two-lane form (V2, packed.cuh) round
// identically and the kernels built on either agree bit for bit. The
// compiler fuses a packed multiply followed by a packed add into one FFMA2
// even when both carry .rn, so the stencils below never feed a product into
// an addition: every multiply-add is written as op_fma.
__device__ __forceinline__ float op_mul(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ double op_mul(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ float op_add(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ double op_add(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ float op_fma(float a, float b, float c) { return __fmaf_rn(a, b, c); }
__device__ __forceinline__ double op_fma(double a, double b, double c) { return __fma_rn(a, b, c); }
__device__ __forceinline__ float op_sqrt(float a) { return sqrtf(a); }
// approximate square root (PTX sqrt.approx.f32, about 2 ulp): the FAST
// normals of FP32-arithmetic runs
__device__ __forceinline__ float op_sqrt_approx(float a) {
    float r;
    asm("sqrt.approx.f32 %0, %1;" : "=f"(r) : "f"(a));
    return r;
}
__device__ __forceinline__ double op_sqrt_approx(double a) { return sqrt(a); }
__device__ __forceinline__ double op_sqrt(double a) { return sqrt(a); }
template <bool FAST>
__device__ __forceinline__ float op_recip(float a) {
    if constexpr (FAST) return __fdividef(1.0f, a);
    else return 1.0f / a;
}
template <bool FAST>
__device__ __forceinline__ double op_recip(double a) { return 1.0 / a; }

namespace detail {
// Direction components as constant expressions (same table as kCX/kCY/kCZ),
// so that every stencil offset below is resolved at compile time.
__host__ __device__ constexpr int dir_c(int axis, int q) {
    constexpr int cx[27] = {0, 1, -1, 0, 0, 0, 0, 1, -1, 1, -1, 0, 0, 1, -1, 1, -1, 0, 0, 1, -1, 1, -1, 1, -1, -1, 1};
    constexpr int cy[27] = {0, 0, 0, 1, -1, 0, 0, 1, -1, 0, 0, 1, -1, -1, 1, 0, 0, 1, -1, 1, -1, 1, -1, -1, 1, 1, -1};
    constexpr int cz[27] = {0, 0, 0, 0, 0, 1, -1, 0, 0, 1, -1, 1, -1, 0, 0, -1, 1, -1, 1, 1, -1, -1, 1, 1, -1, 1, -1};
    return axis == 0 ? cx[q] : (axis == 1 ? cy[q] : cz[q]);
}

template <int AXIS, int Q, class T, class Get>
__device__ __forceinline__ void grad_pair(const Get &v, T (&s)[3], bool (&first)[3]) {
    constexpr int c = dir_c(AXIS, Q);
    if constexpr (c != 0) {
        constexpr int cls = Q <= 6 ? 0 : (Q <= 18 ? 1 : 2);
        constexpr int qp = c > 0 ? Q : Q + 1;
        constexpr int qm = c > 0 ? Q + 1 : Q;
        const T a = v(dir_c(0, qp), dir_c(1, qp), dir_c(2, qp));
        const T b = v(dir_c(0, qm), dir_c(1, qm), dir_c(2, qm));
        if (first[cls]) {
            s[cls] = a - b;
            first[cls] = false;
        } else {
            s[cls] = s[cls] + a;
            s[cls] = s[cls] - b;
        }
    }
}

template <int AXIS, class T, class Get, int... K>
__device__ __forceinline__ void grad_pairs(const Get &v, T (&s)[3], bool (&first)[3],
                                           std::integer_sequence<int, K...>) {
    (grad_pair<AXIS, 2 * K + 1>(v, s, first), ...);
}
}  // namespace detail

// Lattice-weighted central gradient of src/phaseField.cuh:67-118: pairs
// (2k-1, 2k) in ascending k, (+c member) - (-c member), accumulated per
// weight class, then w1*S1 + w2*S2 (+ w3*S3). AXIS 0, 1, 2 = x, y, z.
template <int QQ, int AXIS, class T, class Get>
__device__ __forceinline__ T lattice_grad(const Get &v) {
    T s[3] = {T(0), T(0), T(0)};
    bool first[3] = {true, true, true};
    detail::grad_pairs<AXIS>(v, s, first, std::make_integer_sequence<int, (QQ - 1) / 2>{});
    T r = op_fma(static_cast<T>(Weights<QQ>::w1), s[0], op_mul(static_cast<T>(Weights<QQ>::w2), s[1]));
    if constexpr (QQ == 27) r = op_fma(static_cast<T>(Weights<QQ>::w3), s[2], r);
    return r;
}

// Interface normal n = grad phi / (|grad phi| + 1e-9) and |grad phi| from
// the lattice gradient sums (src/phaseField.cuh:67-118), in one fixed
// rounding order for the scalar and packed evaluations. FAST (every FP32
// arithmetic run): approximate square root and reciprocal (PTX sqrt.approx,
// __fdividef; about 2 ulp, far below the FP32 rounding floor of the fields
// the normals feed); FP64 runs keep the IEEE operations.
template <bool FAST, class T>
__device__ __forceinline__ void unit_normal(T sx, T sy, T sz, T &nx, T &ny, T &nz, T &ind) {
    const T gx = op_mul(static_cast<T>(3.0), sx), gy = op_mul(static_cast<T>(3.0), sy),
            gz = op_mul(static_cast<T>(3.0), sz);
    if constexpr (FAST)
        ind = op_sqrt_approx(op_fma(gx, gx, op_fma(gy, gy, op_mul(gz, gz))));
    else
        ind = op_sqrt(op_fma(gx, gx, op_fma(gy, gy, op_mul(gz, gz))));
    const T inv = op_recip<FAST>(op_add(ind, static_cast<T>(1e-9)));
    nx = op_mul(gx, inv);
    ny = op_mul(gy, inv);
    nz = op_mul(gz, inv);
}

}  // namespace pflbm
