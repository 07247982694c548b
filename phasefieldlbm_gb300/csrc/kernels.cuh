// kernels.cuh - the per-step CUDA kernels (sm_103a). This file holds the
// collide kernel with plain loads and the per-node collision shared by every
// collide variant; kernels_tma.cuh the TMA-fed collide, phase.cuh the phase
// step, fields.cuh initial conditions and readback, stencil.cuh the phi
// gradient, boundary.cuh the inflow/outflow helpers, closure_net.cuh the
// learned closure's network.
//
// One time step of the reference (src/main.cu:163-176: computePhase,
// computeNormals, computeForces, computeMoments, streamCollide, callInflow,
// callOutflow) is executed as two kernels:
//
//   k_collide : phi stencil -> normals -> curvature -> surface-tension force
//               -> moments -> regularised collision -> pull streaming of f,
//               plus the phase-field flux J.
//               One CTA owns a 32x8 column tile and marches up a chunk of z
//               planes, keeping three phi planes (tile + halo 2) and three
//               normal planes (tile + halo 1) in shared memory, so phi is
//               read from HBM once per node.
//   k_phase   : phi^{n+1} = sum_q g_q (the D3Q7 pull), the inflow and
//               outflow rebuilds and the outflow ghost-plane copy.
//
// Data layout in HBM (SoA, x fastest, ghost shell included as in the
// reference): f[q][z][y][x] twice (ping-pong), phi[z][y][x] twice, the
// phase flux J[3][z][y][x], and for the jet 13 moments of plane nz-2 and
// 9 of plane 1 for the outflow and inflow rebuilds done by k_phase.
//
// Pull convention. The value f*_q(S) leaving interior node S is stored at
// P = wrap(S + c_q) - c_q, where wrap is the periodic wrap of
// src/functions/deviceFunctions.cuh:63-76 (x, y always; z for the droplet).
// The receiving node X = wrap(S + c_q) therefore reads X - c_q without any
// wrap, and slots that the reference never rewrites (its single-buffer
// "stale" populations at the jet's z = 1 plane) are written by nobody here
// either, so both ping-pong buffers keep their initial value there.
//
// Phase populations. With tau_g = 1 (src/lbm.cu:209-238) the post-collision
// D3Q7 populations of a node are g_q = w_q (phi + c_q . J) with
// J = 4 phi u + gamma phi (1 - phi) n. Only J (3 values) is stored instead of
// the 7 populations; phi^{n+1}(X) = sum_q g_q(X - c_q) is evaluated in
// direction order q = 0..6 as computePhase does (src/phaseField.cuh:45-51).
#pragma once
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <utility>

#include "boundary.cuh"
#include "closure_net.cuh"
#include "lattice.cuh"
#include "params.cuh"
#include "sround.cuh"
#include "stencil.cuh"
#include "tile.h"

namespace pflbm {

constexpr int TX = PFLBM_TILE_X, TY = PFLBM_TILE_Y, NT = TX * TY;
constexpr int PX = TX + 4, PY = TY + 4;  // phi tile + halo 2
constexpr int NX_ = TX + 2, NY_ = TY + 2;  // normal tile + halo 1

enum Mode { MODE_STEP = 0, MODE_STEP_AVG = 1, MODE_ANALYSIS = 2, MODE_STEP_CLOSURE = 3, MODE_STEP_CLOSURE_AVG = 4 };
constexpr bool mode_closure(int m) { return m == MODE_STEP_CLOSURE || m == MODE_STEP_CLOSURE_AVG; }
constexpr bool mode_average(int m) { return m == MODE_STEP_AVG || m == MODE_STEP_CLOSURE_AVG; }

// Per-node work after the stencils (src/phaseField.cuh:214-218,
// src/lbm.cu:33-239): surface-tension force, moments, relaxation, regularised
// collision with pull-layout stores, phase flux J, boundary-plane moments and
// derived averages; in MODE_ANALYSIS the 18 reference arrays instead.
template <int QQ, bool JET, class S, int MODE>
__device__ __forceinline__ void collide_node(const Params<typename Store<S>::T> &p,
                                             const StepBuffers<S, typename Store<S>::T> &b, int x, int y, int z,
                                             uint32_t t, const typename Store<S>::T (&pop)[QQ],
                                             typename Store<S>::T phi, typename Store<S>::T n_x,
                                             typename Store<S>::T n_y, typename Store<S>::T n_z,
                                             typename Store<S>::T ind, typename Store<S>::T curvature,
                                             float *s_mlp = nullptr, bool active = true) {
    using T = typename Store<S>::T;
    const int nx = p.nx, ny = p.ny, nz = p.nz;
    const uint64_t N = p.N, plane = p.plane;
    // node index, 32-bit (N < 2^32 is checked on the host)
    const uint32_t node = uint32_t(x) + uint32_t(nx) * (uint32_t(y) + uint32_t(ny) * uint32_t(z));
    const uint64_t base = node;
    // running averages of this node, loaded before any store of the node
    // (the compiler cannot move them above the population stores, which it
    // cannot prove do not alias them), so their latency overlaps the
    // collision instead of following it
    T av_old[10];
    if constexpr (mode_average(MODE)) {
        if (active && PFLBM_GUARD(base < N, b.err)) {
#pragma unroll
            for (int k = 0; k < 10; ++k) av_old[k] = b.avg[k * N + base];
        }
    }
    const T st = -p.sigma * curvature * ind;
    const T fx = st * n_x, fy = st * n_y, fz = st * n_z;

    // moments (src/lbm.cu:33-128)
    const Macro<T> m = moments<QQ, T>(pop, fx, fy, fz);

    // learned eddy viscosity nu_cl = strength * nu_t, as a relaxation-time
    // increment tau_t = 3 nu_cl (tau = 1/2 + 3 nu)
    T nu_cl = T(0);
    if constexpr (mode_closure(MODE)) {
        const T feat[kMlpIn] = {m.pxx, m.pyy, m.pzz, m.pxy, m.pxz, m.pyz, phi, ind};
        if constexpr (std::is_same<T, float>::value) {
            // FP32 runs: the warp's 32 nodes on the tensor cores (every lane
            // calls, inactive ones with placeholder features)
            nu_cl = s_mlp[kMlpStrength] * mlp_nu_t_warp(s_mlp, feat, int(threadIdx.y), int(threadIdx.x));
        } else {
            nu_cl = T(s_mlp[kMlpStrength]) * mlp_nu_t<T>(s_mlp, feat);
        }
    }
    const T tau_t = T(3) * nu_cl;
    if (!active) return;
    // relaxation (src/lbm.cu:158-170)
    T omega;
    if constexpr (JET) {
        const T tau_phi = (T(1) - phi) * p.tau_water + phi * p.tau_oil + tau_t;
        const T r = sponge_ramp<T>(p, z);
        const T visc_local = (T(1) - phi) * p.visc_water + phi * p.visc_oil;
        const T tau_zmax = T(0.5) + T(3) * (visc_local * p.kgain1);
        const T tau_eff = tau_phi + r * (tau_zmax - tau_phi);
        omega = T(1) / tau_eff;
    } else {
        omega = tau_t == T(0) ? p.omega_ref : T(1) / (T(1) / p.omega_ref + tau_t);
    }
    const CollideCtx<T> k = make_ctx<QQ, T>(m, fx, fy, fz, T(1) - omega);

    if constexpr (MODE == MODE_ANALYSIS) {
        T *mc = b.macro;
        mc[M_RHO * N + base] = m.rho;
        mc[M_UX * N + base] = m.ux;
        mc[M_UY * N + base] = m.uy;
        mc[M_UZ * N + base] = m.uz;
        mc[M_PXX * N + base] = m.pxx;
        mc[M_PYY * N + base] = m.pyy;
        mc[M_PZZ * N + base] = m.pzz;
        mc[M_PXY * N + base] = m.pxy;
        mc[M_PXZ * N + base] = m.pxz;
        mc[M_PYZ * N + base] = m.pyz;
        mc[M_PHI * N + base] = phi;
        mc[M_NX * N + base] = n_x;
        mc[M_NY * N + base] = n_y;
        mc[M_NZ * N + base] = n_z;
        mc[M_IND * N + base] = ind;
        mc[M_FX * N + base] = fx;
        mc[M_FY * N + base] = fy;
        mc[M_FZ * N + base] = fz;
        return;
    } else {
        // periodic-edge store offsets: P = wrap(S + c) - c. Node indices
        // within one direction's array are 32-bit (N < 2^32 is checked on
        // the host); negative offsets are two's-complement and the sum wraps
        // back into [0, N) exactly.
        const uint32_t ex_p = (x == nx - 2) ? 0u - uint32_t(nx - 2) : 0u;  // cx = +1
        const uint32_t ex_m = (x == 1) ? uint32_t(nx - 2) : 0u;            // cx = -1
        const uint32_t ey_p = (y == ny - 2) ? 0u - uint32_t(ny - 2) * uint32_t(nx) : 0u;
        const uint32_t ey_m = (y == 1) ? uint32_t(ny - 2) * uint32_t(nx) : 0u;
        uint32_t ez_p = 0u, ez_m = 0u;
        if constexpr (!JET) {
            ez_p = (z == nz - 2) ? 0u - uint32_t(nz - 2) * uint32_t(plane) : 0u;
            ez_m = (z == 1) ? uint32_t(nz - 2) * uint32_t(plane) : 0u;
        }
        auto dst_node = [&](int q) -> uint32_t {
            uint32_t o = node;
            if (kCX[q] > 0) o += ex_p;
            if (kCX[q] < 0) o += ex_m;
            if (kCY[q] > 0) o += ey_p;
            if (kCY[q] < 0) o += ey_m;
            if (kCZ[q] > 0) o += ez_p;
            if (kCZ[q] < 0) o += ez_m;
            return o;
        };
        // collision + streaming (src/lbm.cu:172-207); direction q's array
        // starts at f_dst + q N. BF16 storage rounds stochastically
        // (sround.cuh), with the bits of this node's half of its pair.
        constexpr bool kSR = std::is_same<S, __nv_bfloat16>::value;
        uint32_t sr_seed = 0u;
        if constexpr (kSR) sr_seed = sr_pair_seed(node >> 1, t);
        const uint32_t sr_shift = (node & 1u) ? 16u : 0u;
        auto put = [&](int q, uint32_t idx, T v) {
            const T inv_w = static_cast<T>(1.0 / weight<QQ>(q));
            if constexpr (kSR) {
                const uint32_t r = (sr_dir_bits(sr_seed, q) >> sr_shift) & 0xFFFFu;
                reinterpret_cast<uint16_t *>(b.f_dst + uint64_t(q) * N)[idx] = bf16_bits_sr(v * inv_w, r);
            } else {
                Store<S>::store(b.f_dst + uint64_t(q) * N, idx, v, inv_w);
            }
        };
        if (PFLBM_GUARD(base < N, b.err)) put(0, node, collide_rest<QQ, T>(k));
#pragma unroll
        for (int q = 1; q < QQ; q += 2) {
            T a, c;
            collide_pair<QQ, T>(q, k, a, c);
            const uint32_t iq = dst_node(q), iqb = dst_node(q + 1);
            if (PFLBM_GUARD(iq < N, b.err)) put(q, iq, a);
            if (PFLBM_GUARD(iqb < N, b.err)) put(q + 1, iqb, c);
        }
        // phase flux (src/lbm.cu:209-238): g_q = w_q (phi + c_q . J). With the
        // closure's phase mixing, the sub-filter flux -D_t grad phi, D_t =
        // nu_cl / Sc_t, enters as J += -4 D_t |grad phi| n (the D3Q7 flux is
        // J / 4 with cs^2 = 1/4)
        T sharp = p.gamma * phi * (T(1) - phi);
        if constexpr (mode_closure(MODE)) sharp -= T(4) * (T(s_mlp[kMlpPhaseMix]) * nu_cl) * ind;
        if (!PFLBM_GUARD(base < N, b.err)) return;
        b.jflux[base] = T(4) * phi * m.ux + sharp * n_x;
        b.jflux[N + base] = T(4) * phi * m.uy + sharp * n_y;
        b.jflux[2 * N + base] = T(4) * phi * m.uz + sharp * n_z;

        if constexpr (JET) {
            if (z == nz - 2) {
                // moments of the last fluid plane for the outflow rebuild
                const uint64_t c2 = static_cast<uint64_t>(x) + static_cast<uint64_t>(nx) * y;
                if (!PFLBM_GUARD(c2 < plane, b.err)) return;
                T *tp = b.top;
                tp[0 * plane + c2] = m.rho;
                tp[1 * plane + c2] = m.ux;
                tp[2 * plane + c2] = m.uy;
                tp[3 * plane + c2] = m.uz;
                tp[4 * plane + c2] = m.pxx;
                tp[5 * plane + c2] = m.pyy;
                tp[6 * plane + c2] = m.pzz;
                tp[7 * plane + c2] = m.pxy;
                tp[8 * plane + c2] = m.pxz;
                tp[9 * plane + c2] = m.pyz;
                tp[10 * plane + c2] = fx;
                tp[11 * plane + c2] = fy;
                tp[12 * plane + c2] = fz;
            }
            if (z == 1) {
                // moments of the first fluid plane for the inflow rebuild
                const uint64_t c2 = static_cast<uint64_t>(x) + static_cast<uint64_t>(nx) * y;
                if (!PFLBM_GUARD(c2 < plane, b.err)) return;
                T *bp = b.top + 13 * plane;
                bp[0 * plane + c2] = m.ux;
                bp[1 * plane + c2] = m.uy;
                bp[2 * plane + c2] = m.uz;
                bp[3 * plane + c2] = m.pxx;
                bp[4 * plane + c2] = m.pyy;
                bp[5 * plane + c2] = m.pzz;
                bp[6 * plane + c2] = m.pxy;
                bp[7 * plane + c2] = m.pxz;
                bp[8 * plane + c2] = m.pyz;
            }
        }
        if constexpr (mode_average(MODE)) {
            // derived fields (timeAverage.cuh:57-60, reynoldsMoments.cuh:57-60)
            const T tf = static_cast<T>(t + 1u);
            T *av = b.avg;
            auto upd = [&](int slot, uint64_t i, T nv_) {
                if (!PFLBM_GUARD(i < N, b.err)) return;
                const T o = av[slot * N + i];
                av[slot * N + i] = o + (nv_ - o) / tf;
            };
            const T now[10] = {phi, m.ux, m.uy, m.uz, m.ux * m.ux, m.uy * m.uy, m.uz * m.uz,
                               m.ux * m.uy, m.ux * m.uz, m.uy * m.uz};
#pragma unroll
            for (int k = 0; k < 10; ++k) av[k * N + base] = av_old[k] + (now[k] - av_old[k]) / tf;
            if constexpr (JET) {
                if (z == 1 && in_disc<T>(p, x, y)) {
                    // ghost inlet node (x,y,0) holds phi = 1 and the inlet velocity
                    const uint64_t g0 = static_cast<uint64_t>(x) + static_cast<uint64_t>(nx) * y;
                    T bux, buy, buz;
                    inflow_velocity<T>(p, x, y, t, bux, buy, buz);
                    upd(0, g0, T(1));
                    upd(1, g0, bux);
                    upd(2, g0, buy);
                    upd(3, g0, buz);
                    upd(4, g0, bux * bux);
                    upd(5, g0, buy * buy);
                    upd(6, g0, buz * buz);
                    upd(7, g0, bux * buy);
                    upd(8, g0, bux * buz);
                    upd(9, g0, buy * buz);
                }
            }
        }
    }
}

// ------------------------------------------------------------ k_collide
// Shared-memory rings of the plain-load collide (one tile at a time).
template <class T>
struct CollideSmem {
    T phi[3][PY][PX];
    T n[4][3][NY_][NX_];  // nx, ny, nz, |grad phi|
};

// z-march of one 32x8 column tile over interior planes [zb, ze): the body of
// k_collide, also run by the batched ensemble kernel for its work items.
template <int QQ, bool JET, class S, int MODE>
__device__ __forceinline__ void collide_tile(const Params<typename Store<S>::T> &p,
                                             const StepBuffers<S, typename Store<S>::T> &b, int x0, int y0, int zb,
                                             int ze, CollideSmem<typename Store<S>::T> &sm,
                                             float *s_mlp = nullptr) {
    using T = typename Store<S>::T;
    auto &s_phi = sm.phi;
    auto &s_n = sm.n;
    const int nx = p.nx, ny = p.ny, nz = p.nz;
    const uint64_t N = p.N;
    const int tx = threadIdx.x, ty = threadIdx.y, tid = tx + TX * ty;
    const int x = x0 + tx, y = y0 + ty;
    const bool col = (x >= 1 && x <= nx - 2 && y >= 1 && y <= ny - 2);
    const uint32_t t = b.step_in ? static_cast<uint32_t>(*b.step_in) : b.t_fixed;

    auto load_phi = [&](int zp) {
        const int slot = (zp + 3) % 3;
        for (int i = tid; i < PX * PY; i += NT) {
            const int lx = i % PX, ly = i / PX;
            const int gx = x0 - 2 + lx, gy = y0 - 2 + ly;
            T v = T(0);
            if (gx >= 0 && gx < nx && gy >= 0 && gy < ny && zp >= 0 && zp < nz)
                v = b.phi_src[gx + static_cast<uint64_t>(nx) * (gy + static_cast<uint64_t>(ny) * zp)];
            s_phi[slot][ly][lx] = v;
        }
    };
    auto compute_n = [&](int zp) {
        const int sn = (zp + 3) % 3;
        const int sm = (zp + 2) % 3, s0 = sn, sp = (zp + 4) % 3;
        for (int i = tid; i < NX_ * NY_; i += NT) {
            const int lx = i % NX_, ly = i / NX_;
            const int gx = x0 - 1 + lx, gy = y0 - 1 + ly;
            T nxv = T(0), nyv = T(0), nzv = T(0), ind = T(0);
            if (gx >= 1 && gx <= nx - 2 && gy >= 1 && gy <= ny - 2 && zp >= 1 && zp <= nz - 2) {
                auto v = [&](int dx, int dy, int dz) -> T {
                    return s_phi[dz < 0 ? sm : (dz > 0 ? sp : s0)][ly + 1 + dy][lx + 1 + dx];
                };
                // FP32: approximate square root and reciprocal, as the TMA
                // kernel's packed normals (bit-identical); FP64: IEEE
                unit_normal<sizeof(T) == 4>(lattice_grad<QQ, 0, T>(v), lattice_grad<QQ, 1, T>(v), lattice_grad<QQ, 2, T>(v), nxv,
                                   nyv, nzv, ind);
            }
            s_n[0][sn][ly][lx] = nxv;
            s_n[1][sn][ly][lx] = nyv;
            s_n[2][sn][ly][lx] = nzv;
            s_n[3][sn][ly][lx] = ind;
        }
    };

    // warm-up: normals of planes zb-1 and zb
    load_phi(zb - 2);
    load_phi(zb - 1);
    load_phi(zb);
    __syncthreads();
    compute_n(zb - 1);
    __syncthreads();
    load_phi(zb + 1);
    __syncthreads();
    compute_n(zb);

    const uint64_t plane = p.plane;
    for (int z = zb; z < ze; ++z) {
        // issue the pull loads of this node first; they land while the
        // stencil work below runs
        T pop[QQ];
        const uint64_t base = static_cast<uint64_t>(x) + static_cast<uint64_t>(nx) * (y + static_cast<uint64_t>(ny) * z);
        if (col) {
#pragma unroll
            for (int q = 0; q < QQ; ++q) {
                const int64_t off = kCX[q] + static_cast<int64_t>(kCY[q]) * nx + static_cast<int64_t>(kCZ[q]) * static_cast<int64_t>(plane);
                pop[q] = Store<S>::load(b.f_src, q * N + base - off, static_cast<T>(weight<QQ>(q)));
            }
        } else if constexpr (mode_closure(MODE) && std::is_same<T, float>::value) {
#pragma unroll
            for (int q = 0; q < QQ; ++q) pop[q] = T(0);  // placeholder node of the warp-wide network
        }
        __syncthreads();  // previous plane's readers of the ring slots are done
        load_phi(z + 2);
        __syncthreads();
        compute_n(z + 1);
        __syncthreads();
        // the tensor-core network needs every lane of the warp
        constexpr bool kWarpWide = mode_closure(MODE) && std::is_same<T, float>::value;
        if (!col && !kWarpWide) continue;

        const int s_m = (z + 2) % 3, s_0 = z % 3, s_p = (z + 1) % 3;
        // curvature (src/phaseField.cuh:152-212) from the normal ring
        auto nv = [&](int c, int dx, int dy, int dz) -> T {
            return s_n[c][dz < 0 ? s_m : (dz > 0 ? s_p : s_0)][ty + 1 + dy][tx + 1 + dx];
        };
        const T scx = lattice_grad<QQ, 0, T>([&](int dx, int dy, int dz) { return nv(0, dx, dy, dz); });
        const T scy = lattice_grad<QQ, 1, T>([&](int dx, int dy, int dz) { return nv(1, dx, dy, dz); });
        const T scz = lattice_grad<QQ, 2, T>([&](int dx, int dy, int dz) { return nv(2, dx, dy, dz); });
        const T curvature = T(3) * (scx + scy + scz);
        const T n_x = nv(0, 0, 0, 0), n_y = nv(1, 0, 0, 0), n_z = nv(2, 0, 0, 0), ind = nv(3, 0, 0, 0);
        const T phi = s_phi[z % 3][ty + 2][tx + 2];
        collide_node<QQ, JET, S, MODE>(p, b, x, y, z, t, pop, phi, n_x, n_y, n_z, ind, curvature, s_mlp, col);
    }
}

template <int QQ, bool JET, class S, int MODE>
__global__ void __launch_bounds__(NT, (sizeof(typename Store<S>::T) == 8 ? 1 : PFLBM_COLLIDE_MIN_BLOCKS))
    k_collide(const Params<typename Store<S>::T> p, const StepBuffers<S, typename Store<S>::T> b) {
    __shared__ CollideSmem<typename Store<S>::T> sm;
    __shared__ __align__(16) float s_mlp[mode_closure(MODE) ? mlp_smem_words(NT / 32) : 1];
    if constexpr (mode_closure(MODE)) {
        static_assert(TX == 32, "the tensor-core network maps one warp to one tile row");
        for (int i = threadIdx.x + TX * threadIdx.y; i < kMlpDeviceFloats; i += NT) s_mlp[i] = b.mlp[i];
        __syncthreads();
        if constexpr (std::is_same<typename Store<S>::T, float>::value) {
            mlp_build_fragments(s_mlp, threadIdx.x + TX * threadIdx.y, NT);
            __syncthreads();
        }
    }
    const int zb = 1 + blockIdx.z * p.zchunk;
    collide_tile<QQ, JET, S, MODE>(p, b, blockIdx.x * TX, blockIdx.y * TY, zb, min(zb + p.zchunk, int(p.nz) - 1), sm,
                                   s_mlp);
}

}  // namespace pflbm

#include "fields.cuh"
#include "phase.cuh"
