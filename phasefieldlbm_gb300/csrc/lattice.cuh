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

// Moments of src/lbm.cu:33-128 from the shifted populations f' = f - w,
// through the sums s_k = f_(2k-1) + f_(2k) and differences d_k = f_(2k-1) -
// f_(2k) of the opposite pairs: first moments are sums of d_k, second
// moments sums of s_k (c_a c_b is the same for q and its opposite).
template <int QQ, class T>
__device__ __forceinline__ Macro<T> moments(const T (&f)[QQ], T fx, T fy, T fz) {
    constexpr int NP = (QQ - 1) / 2;
    T sp[NP], dp[NP];
#pragma unroll
    for (int k = 0; k < NP; ++k) {
        sp[k] = f[2 * k + 1] + f[2 * k + 2];
        dp[k] = f[2 * k + 1] - f[2 * k + 2];
    }
    Macro<T> m;
    T rho = f[0];
#pragma unroll
    for (int k = 0; k < NP; ++k) rho += sp[k];
    rho += T(1);
    T jx = T(0), jy = T(0), jz = T(0), mxx = T(0), myy = T(0), mzz = T(0), mxy = T(0), mxz = T(0), myz = T(0);
#pragma unroll
    for (int k = 0; k < NP; ++k) {
        const int q = 2 * k + 1;
        const int cx = kCX[q], cy = kCY[q], cz = kCZ[q];
        if (cx > 0) jx += dp[k];
        if (cx < 0) jx -= dp[k];
        if (cy > 0) jy += dp[k];
        if (cy < 0) jy -= dp[k];
        if (cz > 0) jz += dp[k];
        if (cz < 0) jz -= dp[k];
        if (cx != 0) mxx += sp[k];
        if (cy != 0) myy += sp[k];
        if (cz != 0) mzz += sp[k];
        if (cx * cy > 0) mxy += sp[k];
        if (cx * cy < 0) mxy -= sp[k];
        if (cx * cz > 0) mxz += sp[k];
        if (cx * cz < 0) mxz -= sp[k];
        if (cy * cz > 0) myz += sp[k];
        if (cy * cz < 0) myz -= sp[k];
    }
    const T inv = T(1) / rho;
    T ux = inv * jx, uy = inv * jy, uz = inv * jz;
    ux += fx * T(0.5) * inv;
    uy += fy * T(0.5) * inv;
    uz += fz * T(0.5) * inv;
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

// Per-node quantities shared by every pair of the collision. Factors that
// depend only on the weight class (rest, axis, face diagonal, body diagonal)
// are formed once per node.
template <class T>
struct CollideCtx {
    T rho, ux, uy, uz, fx, fy, fz;
    T pxx, pyy, pzz, pxy, pxz, pyz;
    T omco;        // 1 - omega
    T A;           // 1 - uu, uu = 1.5 |u|^2
    T uF;          // u . F
    T u3x, u3y, u3z;  // 3 u
    T wr[4];       // w_class * rho
    T ow[4];       // (1 - omega) * 4.5 * w_class
    T h1, h2, h3, h4, h5, h6, h7;  // third-order Hermite contractions (D3Q27)
};

template <int QQ, class T>
__device__ __forceinline__ CollideCtx<T> make_ctx(const Macro<T> &m, T fx, T fy, T fz, T omco) {
    CollideCtx<T> k;
    k.rho = m.rho; k.ux = m.ux; k.uy = m.uy; k.uz = m.uz;
    k.fx = fx; k.fy = fy; k.fz = fz;
    k.pxx = m.pxx; k.pyy = m.pyy; k.pzz = m.pzz; k.pxy = m.pxy; k.pxz = m.pxz; k.pyz = m.pyz;
    k.omco = omco;
    k.A = T(1) - T(1.5) * (m.ux * m.ux + m.uy * m.uy + m.uz * m.uz);
    k.uF = m.ux * fx + m.uy * fy + m.uz * fz;
    k.u3x = T(3) * m.ux;
    k.u3y = T(3) * m.uy;
    k.u3z = T(3) * m.uz;
    const double wc[4] = {Weights<QQ>::w0, Weights<QQ>::w1, Weights<QQ>::w2, Weights<QQ>::w3};
#pragma unroll
    for (int c = 0; c < 4; ++c) {
        k.wr[c] = static_cast<T>(wc[c]) * m.rho;
        k.ow[c] = omco * static_cast<T>(4.5 * wc[c]);
    }
    if constexpr (QQ == 27) {
        // b_i of D3Q27.cuh:180-189; the coefficients 3 (c_a^2 c_b - cs2 c_b)
        // are the integers 2 c_b (c_a != 0) or -c_b (c_a == 0)
        k.h1 = m.pxx * m.uy + T(2) * m.ux * m.pxy;
        k.h2 = m.pxx * m.uz + T(2) * m.ux * m.pxz;
        k.h3 = m.pyy * m.ux + T(2) * m.uy * m.pxy;
        k.h4 = m.pyy * m.uz + T(2) * m.uy * m.pyz;
        k.h5 = m.pzz * m.ux + T(2) * m.uz * m.pxz;
        k.h6 = m.pzz * m.uy + T(2) * m.uz * m.pyz;
        k.h7 = T(6) * (m.ux * m.pyz + m.uy * m.pxz + m.uz * m.pxy);
    } else {
        k.h1 = k.h2 = k.h3 = k.h4 = k.h5 = k.h6 = k.h7 = T(0);
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

// c . Pi . c for a trace-free Pi (the body-diagonal directions use
// pxx + pyy + pzz = 0).
template <class T>
__device__ __forceinline__ T cpic(int cx, int cy, int cz, const CollideCtx<T> &k) {
    const int nnz = (cx != 0) + (cy != 0) + (cz != 0);
    T o = T(0);
    bool first = true;
    auto add = [&](int sgn, T v) {
        if (first) { o = sgn > 0 ? v : -v; first = false; }
        else o = sgn > 0 ? o + v : o - v;
    };
    if (cx * cy != 0) add(cx * cy, k.pxy);
    if (cx * cz != 0) add(cx * cz, k.pxz);
    if (cy * cz != 0) add(cy * cz, k.pyz);
    if (nnz == 1) return cx != 0 ? k.pxx : (cy != 0 ? k.pyy : k.pzz);
    if (nnz == 3) return T(2) * o;
    const T d = cx == 0 ? (k.pyy + k.pzz) : (cy == 0 ? (k.pxx + k.pzz) : (k.pxx + k.pyy));
    return d + T(2) * o;
}

// 3 x (third-order Hermite part of D3Q27.cuh:180-189), odd in c: sum of
// integer multiples of h1..h7. The (c^3 - c) terms vanish for c in {-1,0,1}.
template <class T>
__device__ __forceinline__ T hermite3(int cx, int cy, int cz, const CollideCtx<T> &k) {
    // 3 (cx^2 cy - cs2 cy) = cy (3 cx^2 - 1), etc.
    const int a1 = cy * (3 * cx * cx - 1), a2 = cz * (3 * cx * cx - 1), a3 = cx * (3 * cy * cy - 1);
    const int a4 = cz * (3 * cy * cy - 1), a5 = cx * (3 * cz * cz - 1), a6 = cy * (3 * cz * cz - 1);
    T s = T(0);
    bool first = true;
    auto add = [&](int a, T v) {
        if (a == 0) return;
        const T term = (a == 2 || a == -2) ? T(2) * v : v;
        if (first) { s = a > 0 ? term : -term; first = false; }
        else s = a > 0 ? s + term : s - term;
    };
    add(a1, k.h1); add(a2, k.h2); add(a3, k.h3); add(a4, k.h4); add(a5, k.h5); add(a6, k.h6);
    if (cx * cy * cz != 0) {
        if (first) { s = cx * cy * cz > 0 ? k.h7 : -k.h7; }
        else s = cx * cy * cz > 0 ? s + k.h7 : s - k.h7;
    }
    return s;
}

__host__ __device__ constexpr int weight_class(int q) { return q == 0 ? 0 : (q <= 6 ? 1 : (q <= 18 ? 2 : 3)); }

// Post-collision shifted populations of the pair (q, q+1), q odd:
// feq + (1-omega) fneq + F/2 of src/lbm.cu:191-206, as E + O and E - O.
template <int QQ, class T>
__device__ __forceinline__ void collide_pair(int q, const CollideCtx<T> &k, T &out_q, T &out_qbar) {
    const int cx = kCX[q], cy = kCY[q], cz = kCZ[q];
    const int cl = weight_class(q);
    const double wd = weight<QQ>(q);
    const T w = static_cast<T>(wd);
    const T hw = static_cast<T>(1.5 * wd);
    const T cu = cdot<T>(cx, cy, cz, k.u3x, k.u3y, k.u3z);
    const T cF = cdot<T>(cx, cy, cz, k.fx, k.fy, k.fz);
    // even: w rho (1 - uu + cu^2/2) - w + (1-omega) 4.5 w c.Pi.c + 1.5 w (cu cF - u.F)
    const T E = k.wr[cl] * (k.A + T(0.5) * cu * cu) - w + k.ow[cl] * cpic<T>(cx, cy, cz, k) + hw * (cu * cF - k.uF);
    // odd: w rho cu (1 - uu + cu^2/6) [D3Q27] + 1.5 w cF + (1-omega) 4.5 w H3
    T O;
    if constexpr (QQ == 27) {
        O = k.wr[cl] * cu * (k.A + static_cast<T>(1.0 / 6.0) * cu * cu) + hw * cF +
            k.ow[cl] * hermite3<T>(cx, cy, cz, k);
    } else {
        O = k.wr[cl] * cu + hw * cF;
    }
    out_q = E + O;
    out_qbar = E - O;
}

template <int QQ, class T>
__device__ __forceinline__ T collide_rest(const CollideCtx<T> &k) {
    const T w = static_cast<T>(weight<QQ>(0));
    return k.wr[0] * k.A - w - static_cast<T>(1.5 * weight<QQ>(0)) * k.uF;
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
