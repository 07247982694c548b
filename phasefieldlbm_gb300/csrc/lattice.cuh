// lattice.cuh - velocity sets and per-node lattice-Boltzmann arithmetic.
//
// Directions and weights follow src/velocitySet/D3Q19.cuh:55-141,
// D3Q27.cuh:55-145 and D3Q7.cuh:45-127 (same ordering, opposite directions
// are (2k-1, 2k)); the ordering is part of the data layout, so it is kept.
//
// The arithmetic is restructured for GB300 instead of evaluated per q as the
// reference does:
//   - moments use closed forms of the lattice sums: with the 4th-order
//     isotropy of D3Q19/D3Q27 (sum w c_a c_b c_c c_d = cs^4 (3 deltas)),
//       sum_q (f_q - feq_q + F_q/2) c_qa c_qb
//         = M_ab - rho u_a u_b - (rho-1) cs2 delta_ab + (u_a F_b + u_b F_a)/2
//     where M is the raw second moment of the stored populations; the
//     isotropic term vanishes under the deviatoric projection of
//     src/lbm.cu:117-120.
//   - the collision of src/lbm.cu:176-207 is evaluated per opposite pair:
//     feq, the Hermite non-equilibrium and the Guo force each split into a
//     part even in c and a part odd in c, so f*_q = E + O and f*_qbar = E - O.
// Both are exact algebra; results differ from the per-q form only by
// rounding.
#pragma once
#include <cstdint>

namespace pflbm {

// ---- direction table (27 entries; D3Q19 uses the first 19) ---------------
__device__ constexpr int kCX[27] = {0, 1, -1, 0, 0, 0, 0, 1, -1, 1, -1, 0, 0, 1, -1, 1, -1, 0, 0, 1, -1, 1, -1, 1, -1, -1, 1};
__device__ constexpr int kCY[27] = {0, 0, 0, 1, -1, 0, 0, 1, -1, 0, 0, 1, -1, -1, 1, 0, 0, 1, -1, 1, -1, 1, -1, -1, 1, 1, -1};
__device__ constexpr int kCZ[27] = {0, 0, 0, 0, 0, 1, -1, 0, 0, 1, -1, 1, -1, 0, 0, -1, 1, -1, 1, 1, -1, -1, 1, 1, -1, 1, -1};

// Weights as double constants; converted to the arithmetic type exactly as
// the reference's static_cast<scalar_t>(1.0/18.0) does.
template <int QQ>
struct Weights;
template <>
struct Weights<19> {
    static constexpr double w0 = 1.0 / 3.0, w1 = 1.0 / 18.0, w2 = 1.0 / 36.0, w3 = 0.0;
};
template <>
struct Weights<27> {
    static constexpr double w0 = 8.0 / 27.0, w1 = 2.0 / 27.0, w2 = 1.0 / 54.0, w3 = 1.0 / 216.0;
};

template <int QQ>
__host__ __device__ constexpr double weight(int q) {
    return q == 0 ? Weights<QQ>::w0 : (q <= 6 ? Weights<QQ>::w1 : (q <= 18 ? Weights<QQ>::w2 : Weights<QQ>::w3));
}
__host__ __device__ constexpr double weight7(int q) { return q == 0 ? 0.25 : 0.125; }

template <class T>
struct Macro {
    T rho, ux, uy, uz;
    T pxx, pyy, pzz, pxy, pxz, pyz;  // deviatoric non-equilibrium second moment
};

// (+c member) - (-c member) accumulation over opposite pairs in ascending
// order: the summation order of the velocity sums of src/lbm.cu:62-73.
template <int QQ, class T>
__device__ __forceinline__ T pair_sum(const T (&f)[QQ], const int *c) {
    T s = T(0);
    bool first = true;
#pragma unroll
    for (int q = 1; q < QQ; q += 2) {
        if (c[q] != 0) {
            const int qp = c[q] > 0 ? q : q + 1;
            const int qm = c[q] > 0 ? q + 1 : q;
            if (first) {
                s = f[qp] - f[qm];
                first = false;
            } else {
                s = s + f[qp];
                s = s - f[qm];
            }
        }
    }
    return s;
}

// Moments of src/lbm.cu:33-128 from the shifted populations f' = f - w.
template <int QQ, class T>
__device__ __forceinline__ Macro<T> moments(const T (&f)[QQ], T fx, T fy, T fz) {
    Macro<T> m;
    T rho = T(0);
#pragma unroll
    for (int q = 0; q < QQ; ++q) rho += f[q];
    rho += T(1);
    const T inv = T(1) / rho;
    T ux = inv * pair_sum<QQ, T>(f, kCX);
    T uy = inv * pair_sum<QQ, T>(f, kCY);
    T uz = inv * pair_sum<QQ, T>(f, kCZ);
    ux += fx * T(0.5) * inv;
    uy += fy * T(0.5) * inv;
    uz += fz * T(0.5) * inv;
    // raw second moments of f'
    T mxx = T(0), myy = T(0), mzz = T(0), mxy = T(0), mxz = T(0), myz = T(0);
#pragma unroll
    for (int q = 1; q < QQ; ++q) {
        const int cx = kCX[q], cy = kCY[q], cz = kCZ[q];
        if (cx != 0) mxx += f[q];
        if (cy != 0) myy += f[q];
        if (cz != 0) mzz += f[q];
        if (cx * cy > 0) mxy += f[q];
        if (cx * cy < 0) mxy -= f[q];
        if (cx * cz > 0) mxz += f[q];
        if (cx * cz < 0) mxz -= f[q];
        if (cy * cz > 0) myz += f[q];
        if (cy * cz < 0) myz -= f[q];
    }
    T pxx = mxx - rho * ux * ux + ux * fx;
    T pyy = myy - rho * uy * uy + uy * fy;
    T pzz = mzz - rho * uz * uz + uz * fz;
    const T pxy = mxy - rho * ux * uy + T(0.5) * (ux * fy + uy * fx);
    const T pxz = mxz - rho * ux * uz + T(0.5) * (ux * fz + uz * fx);
    const T pyz = myz - rho * uy * uz + T(0.5) * (uy * fz + uz * fy);
    const T cs2 = static_cast<T>(1.0 / 3.0);
    const T trace = pxx + pyy + pzz;
    pxx -= cs2 * trace;
    pyy -= cs2 * trace;
    pzz -= cs2 * trace;
    m.rho = rho; m.ux = ux; m.uy = uy; m.uz = uz;
    m.pxx = pxx; m.pyy = pyy; m.pzz = pzz; m.pxy = pxy; m.pxz = pxz; m.pyz = pyz;
    return m;
}

// Per-node quantities shared by every pair of the collision.
template <class T>
struct CollideCtx {
    T rho, ux, uy, uz, fx, fy, fz;
    T pxx, pyy, pzz, pxy, pxz, pyz;
    T omco;       // 1 - omega
    T A;          // 1 - uu, uu = 1.5 |u|^2
    T uu;
    T uF;         // u . F
    T b1, b2, b3, b4, b5, b6, b7;  // third-order Hermite contractions (D3Q27)
};

template <int QQ, class T>
__device__ __forceinline__ CollideCtx<T> make_ctx(const Macro<T> &m, T fx, T fy, T fz, T omco) {
    CollideCtx<T> k;
    k.rho = m.rho; k.ux = m.ux; k.uy = m.uy; k.uz = m.uz;
    k.fx = fx; k.fy = fy; k.fz = fz;
    k.pxx = m.pxx; k.pyy = m.pyy; k.pzz = m.pzz; k.pxy = m.pxy; k.pxz = m.pxz; k.pyz = m.pyz;
    k.omco = omco;
    k.uu = T(1.5) * (m.ux * m.ux + m.uy * m.uy + m.uz * m.uz);
    k.A = T(1) - k.uu;
    k.uF = m.ux * fx + m.uy * fy + m.uz * fz;
    if constexpr (QQ == 27) {
        k.b1 = m.pxx * m.uy + T(2) * m.ux * m.pxy;
        k.b2 = m.pxx * m.uz + T(2) * m.ux * m.pxz;
        k.b3 = m.pyy * m.ux + T(2) * m.uy * m.pxy;
        k.b4 = m.pyy * m.uz + T(2) * m.uy * m.pyz;
        k.b5 = m.pzz * m.ux + T(2) * m.uz * m.pxz;
        k.b6 = m.pzz * m.uy + T(2) * m.uz * m.pyz;
        k.b7 = m.ux * m.pyz + m.uy * m.pxz + m.uz * m.pxy;
    } else {
        k.b1 = k.b2 = k.b3 = k.b4 = k.b5 = k.b6 = k.b7 = T(0);
    }
    return k;
}

// c . v with compile-time c in {-1,0,1}^3 (zero terms pruned).
template <class T>
__device__ __forceinline__ T cdot(int cx, int cy, int cz, T vx, T vy, T vz) {
    T s = T(0);
    bool first = true;
    if (cx != 0) { s = cx > 0 ? vx : -vx; first = false; }
    if (cy != 0) { s = first ? (cy > 0 ? vy : -vy) : (cy > 0 ? s + vy : s - vy); first = false; }
    if (cz != 0) { s = first ? (cz > 0 ? vz : -vz) : (cz > 0 ? s + vz : s - vz); }
    return s;
}

// c . Pi . c for a trace-free Pi.
template <class T>
__device__ __forceinline__ T cpic(int cx, int cy, int cz, const CollideCtx<T> &k) {
    T s = T(0);
    if (cx != 0) s += k.pxx;
    if (cy != 0) s += k.pyy;
    if (cz != 0) s += k.pzz;
    T o = T(0);
    if (cx * cy != 0) o += (cx * cy > 0) ? k.pxy : -k.pxy;
    if (cx * cz != 0) o += (cx * cz > 0) ? k.pxz : -k.pxz;
    if (cy * cz != 0) o += (cy * cz > 0) ? k.pyz : -k.pyz;
    return s + T(2) * o;
}

// Third-order Hermite part of D3Q27.cuh:180-189 (odd in c), without the
// (w*4.5) prefactor. The (c^3 - c) terms vanish identically for c in {-1,0,1}.
template <class T>
__device__ __forceinline__ T hermite3(int cx, int cy, int cz, const CollideCtx<T> &k) {
    const double cs2 = 1.0 / 3.0;
    const T a1 = static_cast<T>(cx * cx * cy - cs2 * cy);
    const T a2 = static_cast<T>(cx * cx * cz - cs2 * cz);
    const T a3 = static_cast<T>(cx * cy * cy - cs2 * cx);
    const T a4 = static_cast<T>(cy * cy * cz - cs2 * cz);
    const T a5 = static_cast<T>(cx * cz * cz - cs2 * cx);
    const T a6 = static_cast<T>(cy * cz * cz - cs2 * cy);
    T s = T(0);
    if (cy != 0) s += a1 * k.b1;
    if (cz != 0) s += a2 * k.b2;
    if (cx != 0) s += a3 * k.b3;
    if (cz != 0) s += a4 * k.b4;
    if (cx != 0) s += a5 * k.b5;
    if (cy != 0) s += a6 * k.b6;
    s = T(3) * s;
    if (cx * cy * cz != 0) s += T(6 * cx * cy * cz) * k.b7;
    return s;
}

// Post-collision shifted populations of the pair (q, q+1), q odd:
// feq + (1-omega) fneq + F/2 of src/lbm.cu:191-206.
template <int QQ, class T>
__device__ __forceinline__ void collide_pair(int q, const CollideCtx<T> &k, T &out_q, T &out_qbar) {
    const int cx = kCX[q], cy = kCY[q], cz = kCZ[q];
    const T w = static_cast<T>(weight<QQ>(q));
    const T cu = T(3) * cdot<T>(cx, cy, cz, k.ux, k.uy, k.uz);
    const T cF = cdot<T>(cx, cy, cz, k.fx, k.fy, k.fz);
    const T wrho = w * k.rho;
    // even parts
    const T feq_e = wrho * (k.A + T(0.5) * cu * cu) - w;
    const T fneq_e = (w * T(4.5)) * cpic<T>(cx, cy, cz, k);
    const T frc_e = (T(3) * w) * (cu * cF - k.uF);
    // odd parts
    T feq_o;
    if constexpr (QQ == 27) {
        feq_o = wrho * cu * (k.A + static_cast<T>(1.0 / 6.0) * cu * cu);
    } else {
        feq_o = wrho * cu;
    }
    const T frc_o = (T(3) * w) * cF;
    T E = feq_e + k.omco * fneq_e + T(0.5) * frc_e;
    T O = feq_o + T(0.5) * frc_o;
    if constexpr (QQ == 27) O += k.omco * ((w * T(4.5)) * hermite3<T>(cx, cy, cz, k));
    out_q = E + O;
    out_qbar = E - O;
}

template <int QQ, class T>
__device__ __forceinline__ T collide_rest(const CollideCtx<T> &k) {
    const T w = static_cast<T>(weight<QQ>(0));
    return w * k.rho * k.A - w + T(0.5) * ((T(-3) * w) * k.uF);
}

// Equilibrium only (no non-equilibrium, no force) for direction q:
// f_eq<Q>(rho, uu, cu) of D3Q19.cuh:143-150 / D3Q27.cuh:152-159.
template <int QQ, class T>
__device__ __forceinline__ T feq_q(int q, T rho, T ux, T uy, T uz) {
    const T w = static_cast<T>(weight<QQ>(q));
    const T uu = T(1.5) * (ux * ux + uy * uy + uz * uz);
    const T cu = T(3) * cdot<T>(kCX[q], kCY[q], kCZ[q], ux, uy, uz);
    if constexpr (QQ == 27)
        return w * rho * (T(1) - uu + cu + T(0.5) * cu * cu + static_cast<T>(1.0 / 6.0) * cu * cu * cu - uu * cu) - w;
    else
        return w * rho * (T(1) - uu + cu + T(0.5) * cu * cu) - w;
}

// Regularised non-equilibrium of direction q (with the w*4.5 prefactor).
template <int QQ, class T>
__device__ __forceinline__ T fneq_q(int q, const CollideCtx<T> &k) {
    const int cx = kCX[q], cy = kCY[q], cz = kCZ[q];
    const T w = static_cast<T>(weight<QQ>(q));
    T h = cpic<T>(cx, cy, cz, k);
    if constexpr (QQ == 27) h += hermite3<T>(cx, cy, cz, k);
    return (w * T(4.5)) * h;
}

// Guo force of direction q (D3Q19.cuh:173-187).
template <int QQ, class T>
__device__ __forceinline__ T force_q(int q, T ux, T uy, T uz, T fx, T fy, T fz) {
    const int cx = kCX[q], cy = kCY[q], cz = kCZ[q];
    const T w = static_cast<T>(weight<QQ>(q));
    const T cu = T(3) * cdot<T>(cx, cy, cz, ux, uy, uz);
    const T cF = cdot<T>(cx, cy, cz, fx, fy, fz);
    return (T(3) * w) * (cF - (ux * fx + uy * fy + uz * fz) + cu * cF);
}

}  // namespace pflbm
