// kernels_pair.cuh - the TMA collide with two x-adjacent nodes per thread and
// packed FP32x2 arithmetic (sm_100 and later: one FFMA2 / FADD2 / FMUL2
// instruction performs the same operation for both nodes, halving the issue
// slots of the per-node algebra).
//
// Same 32x8 column tile, shared-memory plan, TMA pipeline and per-plane order
// as collide_tile_tma (kernels_tma.cuh), with 128 threads per tile: thread
// (i, ty) owns nodes x0 + 2i and x0 + 2i + 1 of row y0 + ty. The per-node
// algebra of lattice.cuh (closed-form moments, collision per opposite pair)
// is written out once more on V2 values with explicit fused multiply-adds;
// results agree with the one-node-per-thread kernels to rounding.
//
// Interior node pairs store each direction as one 8-byte (FP32) or 4-byte
// (16-bit) word. The two pairs at the periodic x edges, where one node of the
// pair is a ghost, store the active node alone with its wrap offsets. With
// 16-bit storage the three reciprocals of a node use the approximate hardware
// reciprocal; in every run the phi normals use the approximate square root
// and reciprocal, as the one-node kernels do. (Evaluating the collision directly in the stored unknown f'/w_q
// saves the rescaling multiply but was measurably less accurate against the
// FP64 path: rho 2.6x, u_z 1.4x the error of the one-node kernel after 400
// jet steps. The exact scaled values round to 16 bits coherently, where the
// unscaled form's FP32 rounding dithers them.)
//
// The plain step of 16-bit D3Q19 storage runs it (no time averages, no
// closure); FP32 and D3Q27 can select it (PFLBM_PAIR=1) but are faster with
// one node per thread. The TMA row alignment already makes nx even.
#pragma once
#include <cuda_bf16.h>
#include <cuda_fp16.h>

#include "kernels_tma.cuh"
#include "packed.cuh"

namespace pflbm {

constexpr int TX2 = TX / 2;   // threads along x of a tile
constexpr int NT2 = NT / 2;   // threads of a tile
static_assert(TX % 2 == 0, "pair tiles");

// Resident CTAs per SM of the pair kernel and the deepest pipeline that
// fits them (228 KB of shared memory per SM, 1 KB of it reserved per CTA):
// a CTA has half the warps of the one-node kernel, so more CTAs are kept
// resident at the cost of pipeline depth.
template <int QQ, class S>
struct PairOccupancy {
    static constexpr int value = sizeof(S) == 2 ? (QQ == 19 ? 4 : 3) : (QQ == 19 ? 3 : 2);
};
template <int QQ, class S>
struct PairStages {
    static constexpr size_t kBudget = (228u * 1024u) / PairOccupancy<QQ, S>::value - 1024u;
    static constexpr int value = TmaPlan<QQ, S, 3>::total <= kBudget ? 3 : 2;
    static_assert(TmaPlan<QQ, S, 2>::total <= kBudget, "pair kernel shared memory");
};
template <int QQ, class S>
using PairLayout = TmaPlan<QQ, S, PairStages<QQ, S>::value>;

// ---------------------------------------------------------------- storage
template <class S>
struct PairStore;
template <>
struct PairStore<float> {
    static constexpr bool kScaled = false;  // stores f'
    template <bool ALIGNED>
    static __device__ __forceinline__ V2 load(const float *p) {
        if constexpr (ALIGNED) return V2(*reinterpret_cast<const float2 *>(p));
        else return V2(p[0], p[1]);
    }
    static __device__ __forceinline__ void store2(float *p, V2 v, float) { *reinterpret_cast<float2 *>(p) = v.v; }
    static __device__ __forceinline__ void store1(float *p, float v, float) { *p = v; }
};
template <>
struct PairStore<__half> {
    static constexpr bool kScaled = true;  // stores f'/w_q
    template <bool ALIGNED>
    static __device__ __forceinline__ V2 load(const __half *p) {
        if constexpr (ALIGNED) return V2(__half22float2(*reinterpret_cast<const __half2 *>(p)));
        else return V2(__half2float(p[0]), __half2float(p[1]));
    }
    static __device__ __forceinline__ void store2(__half *p, V2 v, float inv_w) {
        const V2 s = v * V2(inv_w);
        *reinterpret_cast<__half2 *>(p) = __floats2half2_rn(s.v.x, s.v.y);
    }
    static __device__ __forceinline__ void store1(__half *p, float v, float inv_w) { *p = __float2half_rn(v * inv_w); }
};
template <>
struct PairStore<__nv_bfloat16> {
    static constexpr bool kScaled = true;  // stores f'/w_q
    template <bool ALIGNED>
    static __device__ __forceinline__ V2 load(const __nv_bfloat16 *p) {
        if constexpr (ALIGNED) return V2(__bfloat1622float2(*reinterpret_cast<const __nv_bfloat162 *>(p)));
        else return V2(__bfloat162float(p[0]), __bfloat162float(p[1]));
    }
    static __device__ __forceinline__ void store2(__nv_bfloat16 *p, V2 v, float inv_w) {
        const V2 s = v * V2(inv_w);
        *reinterpret_cast<__nv_bfloat162 *>(p) = __floats2bfloat162_rn(s.v.x, s.v.y);
    }
    static __device__ __forceinline__ void store1(__nv_bfloat16 *p, float v, float inv_w) {
        *p = __float2bfloat16_rn(v * inv_w);
    }
};

// ------------------------------------------------------- per-pair algebra
struct Macro2 {
    V2 rho, ux, uy, uz;
    V2 pxx, pyy, pzz, pxy, pxz, pyz;
};

// Adds sgn * v to an accumulator whose first term sets it (no zero start).
__device__ __forceinline__ void acc2(V2 &s, bool &first, int sgn, V2 v) {
    if (first) {
        s = sgn > 0 ? v : -v;
        first = false;
    } else {
        s = sgn > 0 ? s + v : s - v;
    }
}

// moments() of lattice.cuh on node pairs.
template <int QQ, bool FAST>
__device__ __forceinline__ Macro2 moments2(const V2 (&f)[QQ], V2 fx, V2 fy, V2 fz) {
    constexpr int NP = (QQ - 1) / 2;
    V2 sp[NP], dp[NP];
#pragma unroll
    for (int k = 0; k < NP; ++k) {
        sp[k] = f[2 * k + 1] + f[2 * k + 2];
        dp[k] = f[2 * k + 1] - f[2 * k + 2];
    }
    V2 rho = f[0];
#pragma unroll
    for (int k = 0; k < NP; ++k) rho = rho + sp[k];
    rho = rho + V2(1.0f);
    V2 jx, jy, jz, mxx, myy, mzz, mxy, mxz, myz;
    bool f_jx = true, f_jy = true, f_jz = true, f_xx = true, f_yy = true, f_zz = true, f_xy = true, f_xz = true,
         f_yz = true;
#pragma unroll
    for (int k = 0; k < NP; ++k) {
        const int q = 2 * k + 1;
        const int cx = kCX[q], cy = kCY[q], cz = kCZ[q];
        if (cx != 0) acc2(jx, f_jx, cx, dp[k]);
        if (cy != 0) acc2(jy, f_jy, cy, dp[k]);
        if (cz != 0) acc2(jz, f_jz, cz, dp[k]);
        if (cx != 0) acc2(mxx, f_xx, 1, sp[k]);
        if (cy != 0) acc2(myy, f_yy, 1, sp[k]);
        if (cz != 0) acc2(mzz, f_zz, 1, sp[k]);
        if (cx * cy != 0) acc2(mxy, f_xy, cx * cy, sp[k]);
        if (cx * cz != 0) acc2(mxz, f_xz, cx * cz, sp[k]);
        if (cy * cz != 0) acc2(myz, f_yz, cy * cz, sp[k]);
    }
    Macro2 m;
    const V2 inv = recip2<FAST>(rho);
    const V2 hinv = inv * V2(0.5f);
    const V2 ux = fma2(fx, hinv, inv * jx);
    const V2 uy = fma2(fy, hinv, inv * jy);
    const V2 uz = fma2(fz, hinv, inv * jz);
    const V2 nr = -rho;
    const V2 rux = nr * ux, ruy = nr * uy, ruz = nr * uz;  // -rho u
    V2 pxx = fma2(ux, fx, fma2(rux, ux, mxx));
    V2 pyy = fma2(uy, fy, fma2(ruy, uy, myy));
    V2 pzz = fma2(uz, fz, fma2(ruz, uz, mzz));
    const V2 pxy = fma2(V2(0.5f), fma2(ux, fy, uy * fx), fma2(rux, uy, mxy));
    const V2 pxz = fma2(V2(0.5f), fma2(ux, fz, uz * fx), fma2(rux, uz, mxz));
    const V2 pyz = fma2(V2(0.5f), fma2(uy, fz, uz * fy), fma2(ruy, uz, myz));
    const V2 ncs2 = V2(-static_cast<float>(1.0 / 3.0));
    const V2 trace = pxx + pyy + pzz;
    pxx = fma2(ncs2, trace, pxx);
    pyy = fma2(ncs2, trace, pyy);
    pzz = fma2(ncs2, trace, pzz);
    m.rho = rho; m.ux = ux; m.uy = uy; m.uz = uz;
    m.pxx = pxx; m.pyy = pyy; m.pzz = pzz; m.pxy = pxy; m.pxz = pxz; m.pyz = pyz;
    return m;
}

// CollideCtx of lattice.cuh on node pairs.
template <int QQ>
struct Ctx2 {
    V2 fx, fy, fz;
    V2 pxx, pyy, pzz, pxy, pxz, pyz;
    V2 dxy, dxz, dyz;  // pxx + pyy, pxx + pzz, pyy + pzz
    V2 A, nuF;         // 1 - 1.5 |u|^2, -u.F
    V2 u3x, u3y, u3z;  // 3 u
    V2 wr[4], ow[4];   // w_c rho, (1 - omega) 4.5 w_c
    V2 h1, h2, h3, h4, h5, h6, h7;
};

template <int QQ>
__device__ __forceinline__ Ctx2<QQ> make_ctx2(const Macro2 &m, V2 fx, V2 fy, V2 fz, V2 omco) {
    Ctx2<QQ> k;
    k.fx = fx; k.fy = fy; k.fz = fz;
    k.pxx = m.pxx; k.pyy = m.pyy; k.pzz = m.pzz; k.pxy = m.pxy; k.pxz = m.pxz; k.pyz = m.pyz;
    k.dxy = m.pxx + m.pyy;
    k.dxz = m.pxx + m.pzz;
    k.dyz = m.pyy + m.pzz;
    k.A = fma2(V2(-1.5f), fma2(m.ux, m.ux, fma2(m.uy, m.uy, m.uz * m.uz)), V2(1.0f));
    k.nuF = -fma2(m.ux, fx, fma2(m.uy, fy, m.uz * fz));
    k.u3x = V2(3.0f) * m.ux;
    k.u3y = V2(3.0f) * m.uy;
    k.u3z = V2(3.0f) * m.uz;
    const double wc[4] = {Weights<QQ>::w0, Weights<QQ>::w1, Weights<QQ>::w2, Weights<QQ>::w3};
#pragma unroll
    for (int c = 0; c < (QQ == 27 ? 4 : 3); ++c) {
        k.wr[c] = V2(static_cast<float>(wc[c])) * m.rho;
        k.ow[c] = omco * V2(static_cast<float>(4.5 * wc[c]));
    }
    if constexpr (QQ == 27) {
        const V2 two(2.0f);
        k.h1 = fma2(two * m.ux, m.pxy, m.pxx * m.uy);
        k.h2 = fma2(two * m.ux, m.pxz, m.pxx * m.uz);
        k.h3 = fma2(two * m.uy, m.pxy, m.pyy * m.ux);
        k.h4 = fma2(two * m.uy, m.pyz, m.pyy * m.uz);
        k.h5 = fma2(two * m.uz, m.pxz, m.pzz * m.ux);
        k.h6 = fma2(two * m.uz, m.pyz, m.pzz * m.uy);
        k.h7 = V2(6.0f) * fma2(m.ux, m.pyz, fma2(m.uy, m.pxz, m.uz * m.pxy));
    }
    return k;
}

// c . v for compile-time c (zero terms pruned).
__device__ __forceinline__ V2 cdot2(int cx, int cy, int cz, V2 vx, V2 vy, V2 vz) {
    V2 s;
    bool first = true;
    if (cx != 0) acc2(s, first, cx, vx);
    if (cy != 0) acc2(s, first, cy, vy);
    if (cz != 0) acc2(s, first, cz, vz);
    return s;
}

// c . Pi . c for the trace-free Pi.
template <int QQ>
__device__ __forceinline__ V2 cpic2(int cx, int cy, int cz, const Ctx2<QQ> &k) {
    const int nnz = (cx != 0) + (cy != 0) + (cz != 0);
    if (nnz == 1) return cx != 0 ? k.pxx : (cy != 0 ? k.pyy : k.pzz);
    if (nnz == 2) {
        if (cz == 0) return fma2(V2(float(2 * cx * cy)), k.pxy, k.dxy);
        if (cy == 0) return fma2(V2(float(2 * cx * cz)), k.pxz, k.dxz);
        return fma2(V2(float(2 * cy * cz)), k.pyz, k.dyz);
    }
    return fma2(V2(float(2 * cx * cy)), k.pxy, fma2(V2(float(2 * cx * cz)), k.pxz, V2(float(2 * cy * cz)) * k.pyz));
}

// 3 x the third-order Hermite part (D3Q27), odd in c.
template <int QQ>
__device__ __forceinline__ V2 hermite3_2(int cx, int cy, int cz, const Ctx2<QQ> &k) {
    const int a[7] = {cy * (3 * cx * cx - 1), cz * (3 * cx * cx - 1), cx * (3 * cy * cy - 1), cz * (3 * cy * cy - 1),
                      cx * (3 * cz * cz - 1), cy * (3 * cz * cz - 1), cx * cy * cz};
    const V2 h[7] = {k.h1, k.h2, k.h3, k.h4, k.h5, k.h6, k.h7};
    V2 s;
    bool first = true;
#pragma unroll
    for (int i = 0; i < 7; ++i) {
        if (a[i] == 0) continue;
        if (a[i] == 1 || a[i] == -1) {
            acc2(s, first, a[i], h[i]);
        } else if (first) {
            s = V2(float(a[i])) * h[i];
            first = false;
        } else {
            s = fma2(V2(float(a[i])), h[i], s);
        }
    }
    return s;
}

// collide_pair of lattice.cuh on node pairs: post-collision f' of directions
// q and q + 1 (q odd).
template <int QQ>
__device__ __forceinline__ void collide_pair2(int q, const Ctx2<QQ> &k, V2 &out_q, V2 &out_qbar) {
    const int cx = kCX[q], cy = kCY[q], cz = kCZ[q];
    const int cl = weight_class(q);
    const double wd = weight<QQ>(q);
    const V2 nw(-static_cast<float>(wd));
    const V2 hw(static_cast<float>(1.5 * wd));
    const V2 cu = cdot2(cx, cy, cz, k.u3x, k.u3y, k.u3z);
    const V2 cF = cdot2(cx, cy, cz, k.fx, k.fy, k.fz);
    V2 E = fma2(k.wr[cl], fma2(V2(0.5f) * cu, cu, k.A), nw);
    E = fma2(k.ow[cl], cpic2<QQ>(cx, cy, cz, k), E);
    E = fma2(hw, fma2(cu, cF, k.nuF), E);
    V2 O;
    if constexpr (QQ == 27) {
        O = fma2(k.wr[cl] * cu, fma2(V2(static_cast<float>(1.0 / 6.0)) * cu, cu, k.A), hw * cF);
        O = fma2(k.ow[cl], hermite3_2<QQ>(cx, cy, cz, k), O);
    } else {
        O = fma2(k.wr[cl], cu, hw * cF);
    }
    out_q = E + O;
    out_qbar = E - O;
}

template <int QQ>
__device__ __forceinline__ V2 collide_rest2(const Ctx2<QQ> &k) {
    const double w0 = weight<QQ>(0);
    const V2 nw(-static_cast<float>(w0));
    const V2 hw(static_cast<float>(1.5 * w0));
    return fma2(hw, k.nuF, fma2(k.wr[0], k.A, nw));
}

// collide_node (kernels.cuh, MODE_STEP) for the node pair (xa, y, z),
// (xa + 1, y, z); act_a / act_b say which of the two are interior nodes.
// Order chosen for register pressure: moments, the boundary-plane moments
// and J first, then the collision, each direction pair stored as soon as it
// is formed.
template <int QQ, bool JET, class S>
__device__ __forceinline__ void collide_node_pair(const Params<float> &p, const StepBuffers<S, float> &b, int xa,
                                                  int y, int z, uint32_t t, bool act_a, bool act_b,
                                                  const V2 (&pop)[QQ], V2 phi, V2 n_x, V2 n_y, V2 n_z, V2 ind,
                                                  V2 curvature) {
    constexpr bool FAST = PairStore<S>::kScaled;  // 16-bit storage: approximate reciprocals
    const int nx = p.nx, ny = p.ny, nz = p.nz;
    const uint64_t N = p.N;
    const uint32_t plane = p.plane;
    const uint32_t node_a = uint32_t(xa) + uint32_t(nx) * (uint32_t(y) + uint32_t(ny) * uint32_t(z));
    const bool both = act_a && act_b;
    const bool lb = !act_a;  // the interior node of an edge pair
    const V2 st = V2(-p.sigma) * curvature * ind;
    const V2 fx = st * n_x, fy = st * n_y, fz = st * n_z;

    const Macro2 m = moments2<QQ, FAST>(pop, fx, fy, fz);

    if constexpr (JET) {
        if (z == nz - 2 || z == 1) {
            // moments of the last / first fluid plane for the boundary rebuilds
#pragma unroll
            for (int lane = 0; lane < 2; ++lane) {
                if (!(lane ? act_b : act_a)) continue;
                auto L = [&](V2 v) { return lane ? v.v.y : v.v.x; };
                const uint32_t c2 = uint32_t(xa + lane) + uint32_t(nx) * uint32_t(y);
                if (!PFLBM_GUARD(c2 < plane, b.err)) continue;
                if (z == nz - 2) {
                    float *tp = b.top;
                    tp[0 * plane + c2] = L(m.rho);
                    tp[1 * plane + c2] = L(m.ux);
                    tp[2 * plane + c2] = L(m.uy);
                    tp[3 * plane + c2] = L(m.uz);
                    tp[4 * plane + c2] = L(m.pxx);
                    tp[5 * plane + c2] = L(m.pyy);
                    tp[6 * plane + c2] = L(m.pzz);
                    tp[7 * plane + c2] = L(m.pxy);
                    tp[8 * plane + c2] = L(m.pxz);
                    tp[9 * plane + c2] = L(m.pyz);
                    tp[10 * plane + c2] = L(fx);
                    tp[11 * plane + c2] = L(fy);
                    tp[12 * plane + c2] = L(fz);
                }
                if (z == 1) {
                    float *bp = b.top + 13 * plane;
                    bp[0 * plane + c2] = L(m.ux);
                    bp[1 * plane + c2] = L(m.uy);
                    bp[2 * plane + c2] = L(m.uz);
                    bp[3 * plane + c2] = L(m.pxx);
                    bp[4 * plane + c2] = L(m.pyy);
                    bp[5 * plane + c2] = L(m.pzz);
                    bp[6 * plane + c2] = L(m.pxy);
                    bp[7 * plane + c2] = L(m.pxz);
                    bp[8 * plane + c2] = L(m.pyz);
                }
            }
        }
    }

    // phase flux (src/lbm.cu:209-238)
    {
        const V2 sharp = V2(p.gamma) * phi * (V2(1.0f) - phi);
        const V2 p4 = V2(4.0f) * phi;
        const V2 jxv = fma2(p4, m.ux, sharp * n_x);
        const V2 jyv = fma2(p4, m.uy, sharp * n_y);
        const V2 jzv = fma2(p4, m.uz, sharp * n_z);
        if (both) {
            if (PFLBM_GUARD(node_a + 1 < N, b.err)) {
                *reinterpret_cast<float2 *>(b.jflux + node_a) = jxv.v;
                *reinterpret_cast<float2 *>(b.jflux + N + node_a) = jyv.v;
                *reinterpret_cast<float2 *>(b.jflux + 2 * N + node_a) = jzv.v;
            }
        } else if (act_a || act_b) {
            const uint32_t node = node_a + (lb ? 1u : 0u);
            if (PFLBM_GUARD(node < N, b.err)) {
                b.jflux[node] = lb ? jxv.v.y : jxv.v.x;
                b.jflux[N + node] = lb ? jyv.v.y : jyv.v.x;
                b.jflux[2 * N + node] = lb ? jzv.v.y : jzv.v.x;
            }
        }
    }

    // relaxation (src/lbm.cu:158-170)
    V2 omega;
    if constexpr (JET) {
        const V2 omp = V2(1.0f) - phi;
        const V2 tau_phi = fma2(phi, V2(p.tau_oil), omp * V2(p.tau_water));
        const float r = sponge_ramp<float>(p, z);
        const V2 visc_local = fma2(phi, V2(p.visc_oil), omp * V2(p.visc_water));
        const V2 tau_zmax = fma2(V2(3.0f), visc_local * V2(p.kgain1), V2(0.5f));
        omega = recip2<FAST>(fma2(V2(r), tau_zmax - tau_phi, tau_phi));
    } else {
        omega = V2(p.omega_ref);
    }
    const Ctx2<QQ> k = make_ctx2<QQ>(m, fx, fy, fz, V2(1.0f) - omega);

    // collision (src/lbm.cu:172-207) and pull-layout stores, P = wrap(S + c) - c
    // (32-bit node offsets, as in collide_node)
    const uint32_t ey_p = (y == ny - 2) ? 0u - uint32_t(ny - 2) * uint32_t(nx) : 0u;
    const uint32_t ey_m = (y == 1) ? uint32_t(ny - 2) * uint32_t(nx) : 0u;
    uint32_t ez_p = 0u, ez_m = 0u;
    if constexpr (!JET) {
        ez_p = (z == nz - 2) ? 0u - uint32_t(nz - 2) * plane : 0u;
        ez_m = (z == 1) ? uint32_t(nz - 2) * plane : 0u;
    }
    // BF16 storage rounds stochastically (sround.cuh): 16 random bits per
    // node and direction, the same bits the one-node kernel draws
    constexpr bool kSR = std::is_same<S, __nv_bfloat16>::value;
    uint32_t sr_seed = 0u;
    if constexpr (kSR) sr_seed = sr_pair_seed(node_a >> 1, t);
    if (both) {
        // interior pair: the x offsets vanish for both nodes
        auto put = [&](int q, V2 v) {
            uint32_t d = node_a;
            if (kCY[q] > 0) d += ey_p;
            if (kCY[q] < 0) d += ey_m;
            if (kCZ[q] > 0) d += ez_p;
            if (kCZ[q] < 0) d += ez_m;
            if (!PFLBM_GUARD(d + 1 < N, b.err)) return;
            const float inv_w = static_cast<float>(1.0 / weight<QQ>(q));
            if constexpr (kSR) {
                const V2 sc = v * V2(inv_w);
                *reinterpret_cast<uint32_t *>(b.f_dst + uint64_t(q) * N + d) =
                    bf16x2_bits_sr(sc.v.x, sc.v.y, sr_dir_bits(sr_seed, q));
            } else {
                PairStore<S>::store2(b.f_dst + uint64_t(q) * N + d, v, inv_w);
            }
        };
        put(0, collide_rest2<QQ>(k));
#pragma unroll
        for (int q = 1; q < QQ; q += 2) {
            V2 a, c;
            collide_pair2<QQ>(q, k, a, c);
            put(q, a);
            put(q + 1, c);
        }
    } else if (act_a || act_b) {
        // edge pair: one interior node (x = 1 or x = nx - 2) with its x wrap
        const int x = xa + (lb ? 1 : 0);
        const uint32_t node = node_a + (lb ? 1u : 0u);
        const uint32_t ex_p = (x == nx - 2) ? 0u - uint32_t(nx - 2) : 0u;
        const uint32_t ex_m = (x == 1) ? uint32_t(nx - 2) : 0u;
        auto put = [&](int q, V2 v) {
            uint32_t d = node;
            if (kCX[q] > 0) d += ex_p;
            if (kCX[q] < 0) d += ex_m;
            if (kCY[q] > 0) d += ey_p;
            if (kCY[q] < 0) d += ey_m;
            if (kCZ[q] > 0) d += ez_p;
            if (kCZ[q] < 0) d += ez_m;
            if (!PFLBM_GUARD(d < N, b.err)) return;
            const float inv_w = static_cast<float>(1.0 / weight<QQ>(q));
            const float vv = lb ? v.v.y : v.v.x;
            if constexpr (kSR) {
                const uint32_t r = sr_dir_bits(sr_seed, q);
                reinterpret_cast<uint16_t *>(b.f_dst + uint64_t(q) * N)[d] = bf16_bits_sr(vv * inv_w, lb ? (r >> 16) : (r & 0xFFFFu));
            } else {
                PairStore<S>::store1(b.f_dst + uint64_t(q) * N + d, vv, inv_w);
            }
        };
        put(0, collide_rest2<QQ>(k));
#pragma unroll
        for (int q = 1; q < QQ; q += 2) {
            V2 a, c;
            collide_pair2<QQ>(q, k, a, c);
            put(q, a);
            put(q + 1, c);
        }
    }
}

// collide_tile_tma for node pairs: one column tile, planes zb .. ze-1, the
// same pipeline (stage sequence `seq`, bounded waits, abort path).
template <int QQ, bool JET, class S>
__device__ __forceinline__ bool collide_tile_pair(const Params<float> &p, const StepBuffers<S, float> &b,
                                                  const CUtensorMap *fmapn_p, const CUtensorMap *fmapw_p,
                                                  const CUtensorMap *phimap_p, int x0, int y0, int zb, int ze,
                                                  unsigned char *smem, uint32_t &seq) {
    using T = float;
    using L = PairLayout<QQ, S>;
    S *s_f = reinterpret_cast<S *>(smem + L::off_f);
    T *s_phi = reinterpret_cast<T *>(smem + L::off_phi);
    T *s_n = reinterpret_cast<T *>(smem + L::off_n);
    T *s_ind = reinterpret_cast<T *>(smem + L::off_ind);
    constexpr int NS = L::kStages, R = L::kPhiSlots;
    // The thread that issues the TMA copies: the last warp's first lane,
    // when that warp computes fewer normal-ring pairs per plane than the
    // first (170 pairs on 128 threads: threads 0 - 41 compute two), so that
    // the copies issued after the plane's barrier are absorbed by its slack
    // before the next barrier.
    constexpr int kIssuer = ((NXP * NY_) % NT2) <= NT2 - 32 ? NT2 - 32 : 0;
    // c_x = 0 boxes: element 2 i2 of an even-width row, an aligned pair
    static_assert(L::PXO % 2 == 0 && L::BWN % 2 == 0 && L::BWW % 2 == 0 && L::XU % 2 == 0 && L::PBW % 2 == 0,
                  "pair alignment");
    uint64_t *bar = reinterpret_cast<uint64_t *>(smem + L::off_bar);
    volatile int *s_abort = reinterpret_cast<volatile int *>(smem + L::off_bar + 8 * NS);

    const int nx = p.nx, ny = p.ny, nz = p.nz;
    const int i2 = threadIdx.x, ty = threadIdx.y, tid = i2 + TX2 * ty;
    const int xa = x0 + 2 * i2, y = y0 + ty;
    const bool rowok = y >= 1 && y <= ny - 2;
    const bool act_a = rowok && xa >= 1 && xa <= nx - 2;
    const bool act_b = rowok && xa + 1 >= 1 && xa + 1 <= nx - 2;
    const uint32_t t = b.step_in ? static_cast<uint32_t>(*b.step_in) : b.t_fixed;

    auto pslot = [&](int zp) { return (zp + 2 * R) % R; };
    auto phi_at = [&](int slot, int ly, int lx) -> T & {
        return *reinterpret_cast<T *>(reinterpret_cast<unsigned char *>(s_phi) + slot * L::phi_slot_bytes +
                                      (size_t(ly) * L::PBW + lx) * sizeof(T));
    };
    auto n_at = [&](int c, int slot, int ly, int lx) -> T & { return s_n[((c * 4 + slot) * NY_ + ly) * NX_ + lx]; };
    auto ind_at = [&](int zp, int r, int lx) -> T & { return s_ind[((zp % 3) * TY + r) * NX_ + lx]; };
    auto issue = [&](int stage, int zf) {
        fence_proxy_async();
        mbar_arrive_expect_tx(&bar[stage], L::tx_bytes);
        unsigned char *dst = reinterpret_cast<unsigned char *>(s_f) + size_t(stage) * L::stage_bytes;
#pragma unroll
        for (int q = 0; q < QQ; ++q)
            tma_load_4d(dst + L::box_off(q), kCX[q] == 0 ? fmapn_p : fmapw_p, &bar[stage], x0 - L::shift(q),
                        y0 - kCY[q], zf - kCZ[q], q);
        tma_load_3d(&phi_at(pslot(zf + 2), 0, 0), phimap_p, &bar[stage], x0 - L::PXO, y0 - 2, zf + 2);
    };

    if (tid == 0) {
        tma_prefetch_desc(fmapn_p);
        tma_prefetch_desc(fmapw_p);
        tma_prefetch_desc(phimap_p);
    }
    for (int zp = zb - 2; zp <= zb + 1; ++zp) {
        const int slot = pslot(zp);
        for (int i = tid; i < L::PBW * L::PBH; i += NT2) {
            const int lx = i % L::PBW, ly = i / L::PBW;
            const int gx = x0 - L::PXO + lx, gy = y0 - 2 + ly;
            T v = T(0);
            if (gx >= 0 && gx < nx && gy >= 0 && gy < ny && zp >= 0 && zp < nz)
                v = b.phi_src[gx + static_cast<uint64_t>(nx) * (gy + static_cast<uint64_t>(ny) * zp)];
            phi_at(slot, ly, lx) = v;
        }
    }
    fence_proxy_async();
    // normals of plane zp on the tile + halo 1, two x-adjacent entries per
    // thread (entry pairs start at even lx, so the +-1 neighbours of the pair
    // are aligned 8-byte words and only the dx = 0 column needs two loads)
    auto compute_n = [&](int zp) {
        const int sn = pslot(zp), sm = pslot(zp - 1), sp = pslot(zp + 1);
        const int nn = (zp + 4) & 3;
        const bool zok = zp >= 1 && zp <= nz - 2;
        for (int i = tid; i < NXP * NY_; i += NT2) {
            const int lx = 2 * (i % NXP), ly = i / NXP;
            const int gxa = x0 - 1 + lx, gy = y0 - 1 + ly;
            const bool yok = zok && gy >= 1 && gy <= ny - 2;
            const bool va = yok && gxa >= 1 && gxa <= nx - 2;
            const bool vb = yok && gxa + 1 >= 1 && gxa + 1 <= nx - 2;
            V2 nxv, nyv, nzv, indv;
            normal_pair<QQ, true>(
                [&](int dx, int dy, int dz) -> const T * {
                    return &phi_at(dz < 0 ? sm : (dz > 0 ? sp : sn), ly + 1 + dy, lx + L::PXO - 1 + dx);
                },
                va, vb, nxv, nyv, nzv, indv);
            *reinterpret_cast<float2 *>(&n_at(0, nn, ly, lx)) = nxv.v;
            *reinterpret_cast<float2 *>(&n_at(1, nn, ly, lx)) = nyv.v;
            *reinterpret_cast<float2 *>(&n_at(2, nn, ly, lx)) = nzv.v;
            if (ly >= 1 && ly <= TY) *reinterpret_cast<float2 *>(&ind_at(zp, ly - 1, lx)) = indv.v;
        }
    };
    __syncthreads();
    compute_n(zb - 1);
    __syncthreads();
    if (tid == kIssuer)
        for (int k = 0; k < NS - 1 && zb + k < ze; ++k) issue((seq + k) % NS, zb + k);
    compute_n(zb);

    for (int z = zb; z < ze; ++z) {
        const uint32_t sq = seq + uint32_t(z - zb);
        const int st = int(sq % NS);
        const uint32_t par = (sq / NS) & 1;
        if (!plane_wait<L>(smem, &bar[st], par)) *s_abort = 1;
        compute_n(z + 1);
        __syncthreads();
        if (*s_abort) {
            if (tid == 0) {
                atomicOr(b.err, 1u);
                for (int k = 0; k < NS - 1 && z + k < ze; ++k)
                    mbar_wait_bounded(&bar[(sq + k) % NS], ((sq + k) / NS) & 1, kWaitLimit);
            }
            return false;
        }
        if (tid == kIssuer && z + NS - 1 < ze) issue(int((sq + NS - 1) % NS), z + NS - 1);
        if (!(act_a || act_b)) continue;

        const int s_m = (z + 3) & 3, s_0 = z & 3, s_p = (z + 1) & 3;
        auto nv = [&](int c, int dx, int dy, int dz) -> V2 {
            const T *e = &n_at(c, dz < 0 ? s_m : (dz > 0 ? s_p : s_0), ty + 1 + dy, 2 * i2 + 1 + dx);
            if (dx == 0) return V2(e[0], e[1]);
            return V2(*reinterpret_cast<const float2 *>(e));
        };
        const V2 scx = lattice_grad<QQ, 0, V2>([&](int dx, int dy, int dz) { return nv(0, dx, dy, dz); });
        const V2 scy = lattice_grad<QQ, 1, V2>([&](int dx, int dy, int dz) { return nv(1, dx, dy, dz); });
        const V2 scz = lattice_grad<QQ, 2, V2>([&](int dx, int dy, int dz) { return nv(2, dx, dy, dz); });
        const V2 curvature = V2(3.0f) * (scx + scy + scz);
        const V2 n_x = nv(0, 0, 0, 0), n_y = nv(1, 0, 0, 0), n_z = nv(2, 0, 0, 0);
        const V2 ind(ind_at(z, ty, 2 * i2 + 1), ind_at(z, ty, 2 * i2 + 2));
        const V2 phi(*reinterpret_cast<const float2 *>(&phi_at(pslot(z), ty + 2, 2 * i2 + L::PXO)));

        V2 pop[QQ];
        const unsigned char *sf = reinterpret_cast<const unsigned char *>(s_f) + size_t(st) * L::stage_bytes;
#pragma unroll
        for (int q = 0; q < QQ; ++q) {
            // node xa pulls xa - c_x: element 2 i2 - c_x + shift of its row
            const S *e = reinterpret_cast<const S *>(sf + L::box_off(q)) + ty * L::bw(q) + 2 * i2 - kCX[q] +
                         L::shift(q);
            const V2 raw = kCX[q] == 0 ? PairStore<S>::template load<true>(e) : PairStore<S>::template load<false>(e);
            // populations as f' = f - w: FP32 stores f', 16-bit storage f'/w
            pop[q] = PairStore<S>::kScaled ? raw * V2(static_cast<float>(weight<QQ>(q))) : raw;
        }
        collide_node_pair<QQ, JET, S>(p, b, xa, y, z, t, act_a, act_b, pop, phi, n_x, n_y, n_z, ind, curvature);
    }
    seq += uint32_t(ze - zb);
    return true;
}

template <int QQ, bool JET, class S>
__global__ void __launch_bounds__(NT2, PairOccupancy<QQ, S>::value)
    k_collide_pair(const Params<float> p, const StepBuffers<S, float> b, const __grid_constant__ CUtensorMap fmapn,
                   const __grid_constant__ CUtensorMap fmapw, const __grid_constant__ CUtensorMap phimap) {
    extern __shared__ __align__(128) unsigned char smem[];
    tma_pipeline_init<QQ, S, PairLayout<QQ, S>>(smem);
    const int zb = 1 + blockIdx.z * p.zchunk;
    const int ze = min(zb + p.zchunk, int(p.nz) - 1);
    uint32_t seq = 0;
    collide_tile_pair<QQ, JET, S>(p, b, &fmapn, &fmapw, &phimap, int(blockIdx.x) * TX, int(blockIdx.y) * TY, zb, ze,
                                  smem, seq);
}

}  // namespace pflbm
