// stencil.cuh - the lattice-weighted central gradient of the phi normals and
// curvature stencils, with compile-time direction offsets.
#pragma once
#include <cuda_runtime.h>

#include <utility>

#include "lattice.cuh"

namespace pflbm {

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
    T r = static_cast<T>(Weights<QQ>::w1) * s[0] + static_cast<T>(Weights<QQ>::w2) * s[1];
    if constexpr (QQ == 27) r += static_cast<T>(Weights<QQ>::w3) * s[2];
    return r;
}

}  // namespace pflbm
