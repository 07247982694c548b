// kernels.cuh - the per-step CUDA kernels (sm_103a).
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

#include "lattice.cuh"
#include "params.cuh"
#include "tile.h"

namespace pflbm {

constexpr int TX = PFLBM_TILE_X, TY = PFLBM_TILE_Y, NT = TX * TY;
constexpr int PX = TX + 4, PY = TY + 4;  // phi tile + halo 2
constexpr int NX_ = TX + 2, NY_ = TY + 2;  // normal tile + halo 1

enum Mode { MODE_STEP = 0, MODE_STEP_AVG = 1, MODE_ANALYSIS = 2, MODE_STEP_CLOSURE = 3, MODE_STEP_CLOSURE_AVG = 4 };
constexpr bool mode_closure(int m) { return m == MODE_STEP_CLOSURE || m == MODE_STEP_CLOSURE_AVG; }
constexpr bool mode_average(int m) { return m == MODE_STEP_AVG || m == MODE_STEP_CLOSURE_AVG; }

// ------------------------------------------------------------ closure MLP
// Eddy-viscosity network of the learned closure: x = (Pi_xx, Pi_yy, Pi_zz,
// Pi_xy, Pi_xz, Pi_yz, phi, |grad phi|) -> 32 -> 32 -> 1, SiLU, softplus.
// Device blob layout (floats): W1[32][8], b1[32], W2[32][32], b2[32], w3[32],
// b3, mean[8], inv_scale[8], out_scale, strength.
constexpr int kMlpIn = 8, kMlpH = 32;
constexpr int kMlpParams = kMlpH * kMlpIn + kMlpH + kMlpH * kMlpH + kMlpH + kMlpH + 1;  // 1377
constexpr int kMlpBlob = kMlpParams + 2 * kMlpIn + 2;                                   // 1395
constexpr int kMlpW1 = 0, kMlpB1 = kMlpH * kMlpIn, kMlpW2 = kMlpB1 + kMlpH, kMlpB2 = kMlpW2 + kMlpH * kMlpH,
              kMlpW3 = kMlpB2 + kMlpH, kMlpB3 = kMlpW3 + kMlpH, kMlpMean = kMlpParams,
              kMlpInvScale = kMlpMean + kMlpIn, kMlpOutScale = kMlpInvScale + kMlpIn, kMlpStrength = kMlpOutScale + 1;

template <class T>
__device__ __forceinline__ T silu_d(T a) { return a / (T(1) + exp(-a)); }
template <class T>
__device__ __forceinline__ T softplus_d(T z) { return (z > T(0) ? z : T(0)) + log1p(exp(-fabs(z))); }

// nu_t of one node (no strength factor); w points at the blob (shared memory).
template <class T>
__device__ __forceinline__ T mlp_nu_t(const float *w, const T (&x)[kMlpIn]) {
    T xn[kMlpIn];
#pragma unroll
    for (int k = 0; k < kMlpIn; ++k) xn[k] = (x[k] - T(w[kMlpMean + k])) * T(w[kMlpInvScale + k]);
    T h1[kMlpH];
#pragma unroll
    for (int i = 0; i < kMlpH; ++i) {
        T s = T(w[kMlpB1 + i]);
#pragma unroll
        for (int k = 0; k < kMlpIn; ++k) s += T(w[kMlpW1 + i * kMlpIn + k]) * xn[k];
        h1[i] = silu_d<T>(s);
    }
    T z = T(w[kMlpB3]);
#pragma unroll 4
    for (int j = 0; j < kMlpH; ++j) {
        T s = T(w[kMlpB2 + j]);
#pragma unroll
        for (int i = 0; i < kMlpH; ++i) s += T(w[kMlpW2 + j * kMlpH + i]) * h1[i];
        z += T(w[kMlpW3 + j]) * silu_d<T>(s);
    }
    return T(w[kMlpOutScale]) * softplus_d<T>(z);
}

// ---- the closure network on the tensor cores (FP32 runs) -----------------
// A warp evaluates its 32 nodes (one per lane) as 32x8 -> 32x32 -> 32x32 ->
// 32x1 matrix products with mma.m16n8k16 (BF16 operands, FP32 accumulate):
// the BF16 weights of the blob, BF16-rounded normalised features and
// hidden activations. The per-warp tiles are far too small for tcgen05 (a
// TMEM allocation, shared-memory operand staging and an mbarrier round trip
// per plane); register-operand mma keeps them inside the collide loop.
// Shared words after the blob: B fragments of the three layers, then one
// 32x8 BF16 feature tile per warp.
constexpr int kMlpFragF1 = 1396, kMlpFragF2 = kMlpFragF1 + 128, kMlpFragF3 = kMlpFragF2 + 512,
              kMlpFragX = kMlpFragF3 + 128;
constexpr int mlp_smem_words(int warps) { return kMlpFragX + warps * 32 * 4; }

__device__ __forceinline__ uint32_t pack_bf16(float lo, float hi) {
    const __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);
    return *reinterpret_cast<const uint32_t *>(&v);
}

__device__ __forceinline__ void mma_bf16_16816(float (&d)[4], uint32_t a0, uint32_t a1, uint32_t a2, uint32_t a3,
                                               uint32_t b0, uint32_t b1) {
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
        "{%0,%1,%2,%3};"
        : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
        : "r"(a0), "r"(a1), "r"(a2), "r"(a3), "r"(b0), "r"(b1));
}

// SiLU(a) = a * sigmoid(a) = a/2 * (1 + tanh(a/2)), hardware tanh
__device__ __forceinline__ float silu_tc(float a) {
    float th;
    asm("tanh.approx.f32 %0, %1;" : "=f"(th) : "f"(0.5f * a));
    return 0.5f * a * (1.0f + th);
}

// Fills the B fragments from the blob (all threads of the block; a block
// barrier must follow). Fragment word of lane (g = lane/4, t = lane%4):
// layer 1, n-tile j: W1[8j+g][2t..2t+1]; layer 2, n-tile j, k-step s, word
// h: W2[8j+g][16s+8h+2t..+1]; layer 3, k-step s, word h: w3[16s+8h+2t..+1]
// in column 0 (g == 0), zero elsewhere.
__device__ __forceinline__ void mlp_build_fragments(float *s, int tid, int nthreads) {
    uint32_t *w = reinterpret_cast<uint32_t *>(s);
    for (int i = tid; i < 768; i += nthreads) {
        if (i < 128) {
            const int j = i >> 5, lane = i & 31, g = lane >> 2, t = lane & 3, n = 8 * j + g;
            w[kMlpFragF1 + i] = pack_bf16(s[kMlpW1 + n * kMlpIn + 2 * t], s[kMlpW1 + n * kMlpIn + 2 * t + 1]);
        } else if (i < 640) {
            const int k = i - 128, h = k & 1, e = k >> 1, lane = e & 31, js = e >> 5;
            const int j = js >> 1, st = js & 1, g = lane >> 2, t = lane & 3, n = 8 * j + g;
            const int kk = 16 * st + 8 * h + 2 * t;
            w[kMlpFragF2 + k] = pack_bf16(s[kMlpW2 + n * kMlpH + kk], s[kMlpW2 + n * kMlpH + kk + 1]);
        } else {
            const int k = i - 640, h = k & 1, e = k >> 1, lane = e & 31, st = e >> 5, g = lane >> 2, t = lane & 3;
            const int kk = 16 * st + 8 * h + 2 * t;
            w[kMlpFragF3 + k] = g == 0 ? pack_bf16(s[kMlpW3 + kk], s[kMlpW3 + kk + 1]) : 0u;
        }
    }
}

// nu_t of the calling lane's node; all 32 lanes of the warp must call it.
__device__ __forceinline__ float mlp_nu_t_warp(float *s, const float (&x)[kMlpIn], int warp, int lane) {
    const int g = lane >> 2, t = lane & 3;
    const uint32_t *w = reinterpret_cast<const uint32_t *>(s);
    uint32_t *sx = reinterpret_cast<uint32_t *>(s) + kMlpFragX + warp * 128;
    float xn[kMlpIn];
#pragma unroll
    for (int k = 0; k < kMlpIn; ++k) xn[k] = (x[k] - s[kMlpMean + k]) * s[kMlpInvScale + k];
    __syncwarp();
#pragma unroll
    for (int k = 0; k < 4; ++k) sx[lane * 4 + k] = pack_bf16(xn[2 * k], xn[2 * k + 1]);
    __syncwarp();
    float h1[2][4][4];
#pragma unroll
    for (int mt = 0; mt < 2; ++mt) {
        const uint32_t a0 = sx[(16 * mt + g) * 4 + t], a1 = sx[(16 * mt + g + 8) * 4 + t];
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            const float c0 = s[kMlpB1 + 8 * j + 2 * t], c1 = s[kMlpB1 + 8 * j + 2 * t + 1];
            float d[4] = {c0, c1, c0, c1};
            mma_bf16_16816(d, a0, a1, 0u, 0u, w[kMlpFragF1 + j * 32 + lane], 0u);
#pragma unroll
            for (int e = 0; e < 4; ++e) h1[mt][j][e] = silu_tc(d[e]);
        }
    }
    const uint2 *f2 = reinterpret_cast<const uint2 *>(w + kMlpFragF2);
    const uint2 *f3 = reinterpret_cast<const uint2 *>(w + kMlpFragF3);
    float z[2][4];
#pragma unroll
    for (int mt = 0; mt < 2; ++mt) {
        // accumulator tiles (n-tiles 2s, 2s+1) are the A operand of k-step s
        uint32_t A[2][4];
#pragma unroll
        for (int st = 0; st < 2; ++st) {
            A[st][0] = pack_bf16(h1[mt][2 * st][0], h1[mt][2 * st][1]);
            A[st][1] = pack_bf16(h1[mt][2 * st][2], h1[mt][2 * st][3]);
            A[st][2] = pack_bf16(h1[mt][2 * st + 1][0], h1[mt][2 * st + 1][1]);
            A[st][3] = pack_bf16(h1[mt][2 * st + 1][2], h1[mt][2 * st + 1][3]);
        }
        float h2[4][4];
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            const float c0 = s[kMlpB2 + 8 * j + 2 * t], c1 = s[kMlpB2 + 8 * j + 2 * t + 1];
            float d[4] = {c0, c1, c0, c1};
#pragma unroll
            for (int st = 0; st < 2; ++st) {
                const uint2 b = f2[(j * 2 + st) * 32 + lane];
                mma_bf16_16816(d, A[st][0], A[st][1], A[st][2], A[st][3], b.x, b.y);
            }
#pragma unroll
            for (int e = 0; e < 4; ++e) h2[j][e] = silu_tc(d[e]);
        }
        float d[4] = {0.f, 0.f, 0.f, 0.f};
#pragma unroll
        for (int st = 0; st < 2; ++st) {
            const uint2 b = f3[st * 32 + lane];
            mma_bf16_16816(d, pack_bf16(h2[2 * st][0], h2[2 * st][1]), pack_bf16(h2[2 * st][2], h2[2 * st][3]),
                           pack_bf16(h2[2 * st + 1][0], h2[2 * st + 1][1]),
                           pack_bf16(h2[2 * st + 1][2], h2[2 * st + 1][3]), b.x, b.y);
        }
#pragma unroll
        for (int e = 0; e < 4; ++e) z[mt][e] = d[e];
    }
    // column 0 of row r of m-tile mt sits in lane 4*(r%8), element 0 (r < 8) or 2
    const int r = lane & 15, src = 4 * (r & 7);
    const float v00 = __shfl_sync(0xffffffffu, z[0][0], src), v02 = __shfl_sync(0xffffffffu, z[0][2], src);
    const float v10 = __shfl_sync(0xffffffffu, z[1][0], src), v12 = __shfl_sync(0xffffffffu, z[1][2], src);
    const float zz = (lane < 16 ? (r < 8 ? v00 : v02) : (r < 8 ? v10 : v12)) + s[kMlpB3];
    return s[kMlpOutScale] * softplus_d<float>(zz);
}

// -------------------------------------------------------------- noise
// Counter hash and Box-Muller of src/BoundaryConditions.cuh:172-213.
__device__ __forceinline__ uint32_t hash32(uint32_t x) {
    x ^= x >> 16;
    x *= 0x7FEB352Du;
    x ^= x >> 15;
    x *= 0x846CA68Bu;
    x ^= x >> 16;
    return x;
}
__device__ __forceinline__ float uniform01(uint32_t s) {
    return (static_cast<float>(s) + 0.5f) * 2.3283064365386963e-10f;
}
__device__ __forceinline__ uint32_t noise_base(uint32_t salt, uint32_t x, uint32_t y, uint32_t t) {
    return (0x9E3779B9u ^ salt) ^ x ^ (y * 0x85EBCA6Bu) ^ (t * 0xC2B2AE35u);
}
__device__ __forceinline__ float white_noise(uint32_t salt, uint32_t x, uint32_t y, uint32_t t) {
    const uint32_t base = noise_base(salt, x, y, t);
    float rrx = uniform01(hash32(base));
    const float rry = uniform01(hash32(base ^ 0x68BC21EBu));
    rrx = fmaxf(rrx, 1e-12f);
    const float r = sqrtf(-2.0f * logf(rrx));
    const float theta = (2.0f * 3.141592654f) * rry;
    return r * cosf(theta);
}
// Uniform inflow mode: xi in [-1,1) from the same hash, salted by the seed.
__device__ __forceinline__ float uniform_noise(uint32_t seed, uint32_t x, uint32_t y, uint32_t t) {
    return 2.0f * uniform01(hash32(noise_base(0x2545F491u ^ seed, x, y, t))) - 1.0f;
}
__device__ __forceinline__ float init_noise_value(uint32_t seed, uint32_t c, uint32_t x, uint32_t y, uint32_t z) {
    return 2.0f * uniform01(hash32(noise_base(0x5851F42Du ^ seed ^ (c * 0x9E3779B9u), x, y, z * 0x27D4EB2Fu))) - 1.0f;
}

// Inlet velocity at ghost column (x, y) and step t (BoundaryConditions.cuh:56-69).
template <class T>
__device__ __forceinline__ void inflow_velocity(const Params<T> &p, uint32_t x, uint32_t y, uint32_t t, T &ux, T &uy,
                                                T &uz) {
    if (p.noise_mode == 0) {
        ux = static_cast<T>(p.sigma_u * white_noise(0xA341316Cu, x, y, t));
        uy = static_cast<T>(p.sigma_u * white_noise(0xC8013EA4u, x, y, t));
        uz = p.u_inf;
    } else {
        ux = T(0);
        uy = T(0);
        // rounded op by op (no FMA contraction) so host and device agree bit for bit
        uz = static_cast<T>(__fmul_rn(p.u_inf_f, __fadd_rn(1.0f, __fmul_rn(p.noise_amp, uniform_noise(p.seed, x, y, t)))));
    }
}

template <class T>
__device__ __forceinline__ bool in_disc(const Params<T> &p, int x, int y) {
    const T dx = static_cast<T>(x) - p.center_x;
    const T dy = static_cast<T>(y) - p.center_y;
    return !(dx * dx + dy * dy > p.R2);
}

__device__ __forceinline__ int wrapi(int x, int n) { return x < 1 ? n - 2 : (x > n - 2 ? 1 : x); }

// Sponge ramp, src/functions/deviceFunctions.cuh:94-101.
template <class T>
__device__ __forceinline__ T sponge_ramp(const Params<T> &p, int z) {
    const T zn = static_cast<T>(z) * p.inv_nz_m1;
    T s = (zn - p.z_start) * p.inv_sponge;
    s = s < T(0) ? T(0) : (s > T(1) ? T(1) : s);
    return s * s * (T(3) - T(2) * s);
}

// Lattice-weighted central gradient of src/phaseField.cuh:67-118: pairs
// (2k-1, 2k) in ascending k, (+c member) - (-c member), accumulated per
// weight class, then w1*S1 + w2*S2 (+ w3*S3).
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
    const uint64_t base = static_cast<uint64_t>(x) + static_cast<uint64_t>(nx) * (y + static_cast<uint64_t>(ny) * z);
    const T st = -p.sigma * curvature * ind;
    const T fx = st * n_x, fy = st * n_y, fz = st * n_z;

    // moments (src/lbm.cu:33-128)
    const Macro<T> m = moments<QQ, T>(pop, fx, fy, fz);

    // learned eddy-viscosity increment, in units of tau (tau = 1/2 + 3 nu)
    T tau_t = T(0);
    if constexpr (mode_closure(MODE)) {
        const T feat[kMlpIn] = {m.pxx, m.pyy, m.pzz, m.pxy, m.pxz, m.pyz, phi, ind};
        if constexpr (std::is_same<T, float>::value) {
            // FP32 runs: the warp's 32 nodes on the tensor cores (every lane
            // calls, inactive ones with placeholder features)
            tau_t = T(3) * (s_mlp[kMlpStrength] * mlp_nu_t_warp(s_mlp, feat, int(threadIdx.y), int(threadIdx.x)));
        } else {
            tau_t = T(3) * (T(s_mlp[kMlpStrength]) * mlp_nu_t<T>(s_mlp, feat));
        }
    }
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
        // periodic-edge store offsets: P = wrap(S + c) - c
        const int64_t ex_p = (x == nx - 2) ? -(int64_t)(nx - 2) : 0;  // cx = +1
        const int64_t ex_m = (x == 1) ? (int64_t)(nx - 2) : 0;        // cx = -1
        const int64_t ey_p = (y == ny - 2) ? -(int64_t)(ny - 2) * nx : 0;
        const int64_t ey_m = (y == 1) ? (int64_t)(ny - 2) * nx : 0;
        int64_t ez_p = 0, ez_m = 0;
        if constexpr (!JET) {
            ez_p = (z == nz - 2) ? -(int64_t)(nz - 2) * (int64_t)plane : 0;
            ez_m = (z == 1) ? (int64_t)(nz - 2) * (int64_t)plane : 0;
        }
        auto dst_index = [&](int q) -> uint64_t {
            int64_t o = 0;
            if (kCX[q] > 0) o += ex_p;
            if (kCX[q] < 0) o += ex_m;
            if (kCY[q] > 0) o += ey_p;
            if (kCY[q] < 0) o += ey_m;
            if (kCZ[q] > 0) o += ez_p;
            if (kCZ[q] < 0) o += ez_m;
            return q * N + base + o;
        };
        // collision + streaming (src/lbm.cu:172-207)
        Store<S>::store(b.f_dst, base, collide_rest<QQ, T>(k), static_cast<T>(1.0 / weight<QQ>(0)));
#pragma unroll
        for (int q = 1; q < QQ; q += 2) {
            T a, c;
            collide_pair<QQ, T>(q, k, a, c);
            Store<S>::store(b.f_dst, dst_index(q), a, static_cast<T>(1.0 / weight<QQ>(q)));
            Store<S>::store(b.f_dst, dst_index(q + 1), c, static_cast<T>(1.0 / weight<QQ>(q + 1)));
        }
        // phase flux (src/lbm.cu:209-238): g_q = w_q (phi + c_q . J)
        const T sharp = p.gamma * phi * (T(1) - phi);
        b.jflux[base] = T(4) * phi * m.ux + sharp * n_x;
        b.jflux[N + base] = T(4) * phi * m.uy + sharp * n_y;
        b.jflux[2 * N + base] = T(4) * phi * m.uz + sharp * n_z;

        if constexpr (JET) {
            if (z == nz - 2) {
                // moments of the last fluid plane for the outflow rebuild
                const uint64_t c2 = static_cast<uint64_t>(x) + static_cast<uint64_t>(nx) * y;
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
                const T o = av[slot * N + i];
                av[slot * N + i] = o + (nv_ - o) / tf;
            };
            upd(0, base, phi);
            upd(1, base, m.ux);
            upd(2, base, m.uy);
            upd(3, base, m.uz);
            upd(4, base, m.ux * m.ux);
            upd(5, base, m.uy * m.uy);
            upd(6, base, m.uz * m.uz);
            upd(7, base, m.ux * m.uy);
            upd(8, base, m.ux * m.uz);
            upd(9, base, m.uy * m.uz);
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
                const T gxv = T(3) * lattice_grad<QQ, 0, T>(v);
                const T gyv = T(3) * lattice_grad<QQ, 1, T>(v);
                const T gzv = T(3) * lattice_grad<QQ, 2, T>(v);
                ind = sqrt(gxv * gxv + gyv * gyv + gzv * gzv);
                const T inv = T(1) / (ind + static_cast<T>(1e-9));
                nxv = gxv * inv;
                nyv = gyv * inv;
                nzv = gzv * inv;
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
        for (int i = threadIdx.x + TX * threadIdx.y; i < kMlpBlob; i += NT) s_mlp[i] = b.mlp[i];
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

// -------------------------------------------------------------- k_phase
// phi^{n+1} (computePhase of the next step, src/phaseField.cuh:31-52),
// outflow rebuild (BoundaryConditions.cuh:107-169) and step counter.
template <int QQ, bool JET, class S>
__device__ __forceinline__ void phase_node(const Params<typename Store<S>::T> &p,
                                           const StepBuffers<S, typename Store<S>::T> &b, int x, int y, int z,
                                           uint32_t t) {
    using T = typename Store<S>::T;
    const int nx = p.nx, ny = p.ny, nz = p.nz;
    const uint64_t N = p.N, plane = p.plane;
    const uint64_t X = static_cast<uint64_t>(x) + static_cast<uint64_t>(nx) * (y + static_cast<uint64_t>(ny) * z);
    auto idx = [&](int xx, int yy, int zz) -> uint64_t {
        return static_cast<uint64_t>(xx) + static_cast<uint64_t>(nx) * (yy + static_cast<uint64_t>(ny) * zz);
    };
    const T *phi = b.phi_src;
    const T *J = b.jflux;
    const T w0 = T(0.25), w1 = T(0.125);
    const int xm = wrapi(x - 1, nx), xp = wrapi(x + 1, nx);
    const int ym = wrapi(y - 1, ny), yp = wrapi(y + 1, ny);
    const int zm = JET ? z - 1 : wrapi(z - 1, nz), zp = JET ? z + 1 : wrapi(z + 1, nz);
    const T phiX = phi[X];
    // q = 1 (+x) comes from x-1, q = 2 (-x) from x+1, ...
    const T g0 = w0 * phiX;
    const uint64_t s1 = idx(xm, y, z), s2 = idx(xp, y, z), s3 = idx(x, ym, z), s4 = idx(x, yp, z);
    const T g1 = w1 * (phi[s1] + J[s1]);
    const T g2 = w1 * (phi[s2] - J[s2]);
    const T g3 = w1 * (phi[s3] + J[N + s3]);
    const T g4 = w1 * (phi[s4] - J[N + s4]);
    T g5, g6;
    if (JET && z == 1) {
        // BoundaryConditions.cuh:104: g5 at z=1 is rebuilt inside the disc
        // from the inlet uz; outside it keeps its initial value 0
        if (in_disc<T>(p, x, y)) {
            T bux, buy, buz = p.u_inf;
            if (p.noise_mode != 0) inflow_velocity<T>(p, x, y, t, bux, buy, buz);
            g5 = w1 * T(1) * (T(1) + T(4) * buz);
        } else {
            g5 = T(0);
        }
    } else {
        const uint64_t s5 = idx(x, y, zm);
        g5 = w1 * (phi[s5] + J[2 * N + s5]);
    }
    if (JET && z == nz - 2) {
        // BoundaryConditions.cuh:168 with the node's own phi and uz
        const T uz = b.top[3 * plane + static_cast<uint64_t>(x) + static_cast<uint64_t>(nx) * y];
        g6 = w1 * phiX * (T(1) - T(4) * uz);
    } else {
        const uint64_t s6 = idx(x, y, zp);
        g6 = w1 * (phi[s6] - J[2 * N + s6]);
    }
    T s = T(0);
    s += g0; s += g1; s += g2; s += g3; s += g4; s += g5; s += g6;
    b.phi_dst[X] = s;

    if constexpr (JET) {
        if (z == 1) {
            // inflow rebuild (BoundaryConditions.cuh:73-101): the populations
            // entering (x,y,1) from a ghost column (x-cx, y-cy, 0) inside the
            // inlet disc get feq of the inlet state plus the regularised
            // non-equilibrium of this node's step-n moments.
            const uint64_t cX = static_cast<uint64_t>(x) + static_cast<uint64_t>(nx) * y;
            const T *bp = b.top + 13 * plane;
            Macro<T> mX;
            mX.rho = T(1);
            mX.ux = bp[cX]; mX.uy = bp[plane + cX]; mX.uz = bp[2 * plane + cX];
            mX.pxx = bp[3 * plane + cX]; mX.pyy = bp[4 * plane + cX]; mX.pzz = bp[5 * plane + cX];
            mX.pxy = bp[6 * plane + cX]; mX.pxz = bp[7 * plane + cX]; mX.pyz = bp[8 * plane + cX];
            const CollideCtx<T> kX = make_ctx<QQ, T>(mX, T(0), T(0), T(0), T(0));
#pragma unroll
            for (int q = 1; q < QQ; ++q) {
                if (kCZ[q] == 1) {
                    const int gx = x - kCX[q], gy = y - kCY[q];
                    if (in_disc<T>(p, gx, gy)) {
                        T bux, buy, buz;
                        inflow_velocity<T>(p, gx, gy, t, bux, buy, buz);
                        const T v = feq_q<QQ, T>(q, T(1), bux, buy, buz) + p.omco_zmin * fneq_q<QQ, T>(q, kX);
                        Store<S>::store(b.f_dst, q * N + static_cast<uint64_t>(gx) + static_cast<uint64_t>(nx) * gy, v,
                                        static_cast<T>(1.0 / weight<QQ>(q)));
                    }
                }
            }
        }
        if (z == nz - 2) {
            // ghost phi of the outlet plane takes this step's value
            // (BoundaryConditions.cuh:127)
            b.phi_dst[idx(x, y, nz - 1)] = phiX;
            // outflow rebuild of the populations entering (x,y,nz-2) from
            // the ghost plane: equilibrium of the in-plane source column
            // (x-cx, y-cy), non-equilibrium and force of this node.
            const T *tp = b.top;
            const uint64_t cX = static_cast<uint64_t>(x) + static_cast<uint64_t>(nx) * y;
            Macro<T> mX;
            mX.rho = tp[cX];
            mX.ux = tp[plane + cX]; mX.uy = tp[2 * plane + cX]; mX.uz = tp[3 * plane + cX];
            mX.pxx = tp[4 * plane + cX]; mX.pyy = tp[5 * plane + cX]; mX.pzz = tp[6 * plane + cX];
            mX.pxy = tp[7 * plane + cX]; mX.pxz = tp[8 * plane + cX]; mX.pyz = tp[9 * plane + cX];
            const T fxX = tp[10 * plane + cX], fyX = tp[11 * plane + cX], fzX = tp[12 * plane + cX];
            const CollideCtx<T> kX = make_ctx<QQ, T>(mX, fxX, fyX, fzX, T(0));
#pragma unroll
            for (int q = 1; q < QQ; ++q) {
                if (kCZ[q] == -1) {
                    const int bx = wrapi(x - kCX[q], nx), by = wrapi(y - kCY[q], ny);
                    const uint64_t cb = static_cast<uint64_t>(bx) + static_cast<uint64_t>(nx) * by;
                    const T rb = tp[cb], uxb = tp[plane + cb], uyb = tp[2 * plane + cb], uzb = tp[3 * plane + cb];
                    const T phib = phi[cb + plane * static_cast<uint64_t>(nz - 2)];
                    const T visc_local = (T(1) - phib) * p.visc_water + phib * p.visc_oil;
                    const T omco = T(1) - static_cast<T>(1.0 / (0.5 + 3.0 * static_cast<double>(visc_local * p.kgain1)));
                    const T v = feq_q<QQ, T>(q, rb, uxb, uyb, uzb) + omco * fneq_q<QQ, T>(q, kX) +
                                T(0.5) * force_q<QQ, T>(q, uxb, uyb, uzb, fxX, fyX, fzX);
                    const uint64_t dst = q * N + static_cast<uint64_t>(x - kCX[q]) +
                                         static_cast<uint64_t>(nx) * (static_cast<uint64_t>(y - kCY[q]) + static_cast<uint64_t>(ny) * (nz - 1));
                    Store<S>::store(b.f_dst, dst, v, static_cast<T>(1.0 / weight<QQ>(q)));
                }
            }
        }
    }
}


template <int QQ, bool JET, class S>
__global__ void __launch_bounds__(256) k_phase(const Params<typename Store<S>::T> p, const StepBuffers<S, typename Store<S>::T> b) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    const int y = blockIdx.y * blockDim.y + threadIdx.y;
    const int z = blockIdx.z * blockDim.z + threadIdx.z;
    const uint32_t t = static_cast<uint32_t>(*b.step_in);
    if (blockIdx.x == 0 && blockIdx.y == 0 && blockIdx.z == 0 && threadIdx.x == 0 && threadIdx.y == 0 &&
        threadIdx.z == 0)
        *b.step_out = *b.step_in + 1ull;
    if (x < 1 || x > int(p.nx) - 2 || y < 1 || y > int(p.ny) - 2 || z < 1 || z > int(p.nz) - 2) return;
    phase_node<QQ, JET, S>(p, b, x, y, z, t);
}

// Boundary-plane nodes of the jet, kept out of line so that their rebuild
// code does not set the register budget of the vectorised interior path.
template <int QQ, bool JET, class S>
__device__ __noinline__ void phase_node_outlined(const Params<float> &p, const StepBuffers<S, float> &b, int x, int y,
                                                 int z, uint32_t t) {
    phase_node<QQ, JET, S>(p, b, x, y, z, t);
}

// The phase sum of the 4 consecutive nodes x4 .. x4+3 of row (y, z), an
// interior row of a grid with nx % 4 == 0 (shared by k_phase_v4 and the
// ensemble's batch phase kernel).
template <bool JET, class S>
__device__ __forceinline__ void phase_vec4(const Params<float> &p, const StepBuffers<S, float> &b, int x4, int y,
                                           int z) {
    const int nx = p.nx, ny = p.ny, nz = p.nz;
    const uint64_t N = p.N;
    const int ym = wrapi(y - 1, ny), yp = wrapi(y + 1, ny);
    const int zm = JET ? z - 1 : wrapi(z - 1, nz), zp = JET ? z + 1 : wrapi(z + 1, nz);
    auto row = [&](int yy, int zz) -> uint64_t { return static_cast<uint64_t>(nx) * (yy + static_cast<uint64_t>(ny) * zz); };
    const float *phi = b.phi_src;
    const float *Jx = b.jflux, *Jy = b.jflux + N, *Jz = b.jflux + 2 * N;
    const uint64_t r0 = row(y, z);
    const float4 pc = *reinterpret_cast<const float4 *>(phi + r0 + x4);
    const float4 pym = *reinterpret_cast<const float4 *>(phi + row(ym, z) + x4);
    const float4 pyp = *reinterpret_cast<const float4 *>(phi + row(yp, z) + x4);
    const float4 pzm = *reinterpret_cast<const float4 *>(phi + row(y, zm) + x4);
    const float4 pzp = *reinterpret_cast<const float4 *>(phi + row(y, zp) + x4);
    const float4 jxc = *reinterpret_cast<const float4 *>(Jx + r0 + x4);
    const float4 jym = *reinterpret_cast<const float4 *>(Jy + row(ym, z) + x4);
    const float4 jyp = *reinterpret_cast<const float4 *>(Jy + row(yp, z) + x4);
    const float4 jzm = *reinterpret_cast<const float4 *>(Jz + row(y, zm) + x4);
    const float4 jzp = *reinterpret_cast<const float4 *>(Jz + row(y, zp) + x4);
    // x neighbours of the 4-node segment, periodic inside [1, nx-2]
    const int xl = wrapi(x4 - 1, nx), xr = wrapi(x4 + 4, nx);
    float pl[6], jl[6];  // phi and Jx at x4-1 .. x4+4
    pl[0] = phi[r0 + xl]; jl[0] = Jx[r0 + xl];
    pl[1] = pc.x; pl[2] = pc.y; pl[3] = pc.z; pl[4] = pc.w;
    jl[1] = jxc.x; jl[2] = jxc.y; jl[3] = jxc.z; jl[4] = jxc.w;
    pl[5] = phi[r0 + xr]; jl[5] = Jx[r0 + xr];
    const float a_ym[4] = {pym.x, pym.y, pym.z, pym.w}, a_yp[4] = {pyp.x, pyp.y, pyp.z, pyp.w};
    const float a_zm[4] = {pzm.x, pzm.y, pzm.z, pzm.w}, a_zp[4] = {pzp.x, pzp.y, pzp.z, pzp.w};
    const float b_ym[4] = {jym.x, jym.y, jym.z, jym.w}, b_yp[4] = {jyp.x, jyp.y, jyp.z, jyp.w};
    const float b_zm[4] = {jzm.x, jzm.y, jzm.z, jzm.w}, b_zp[4] = {jzp.x, jzp.y, jzp.z, jzp.w};
    float out[4];
    const float w0 = 0.25f, w1 = 0.125f;
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        const int x = x4 + k;
        // left/right sources; ghost columns map to the periodic image
        float phl = pl[k], jxl = jl[k], phr = pl[k + 2], jxr = jl[k + 2];
        if (x == 1) { phl = phi[r0 + nx - 2]; jxl = Jx[r0 + nx - 2]; }
        if (x == nx - 2) { phr = phi[r0 + 1]; jxr = Jx[r0 + 1]; }
        float s = 0.0f;
        s += w0 * pl[k + 1];
        s += w1 * (phl + jxl);
        s += w1 * (phr - jxr);
        s += w1 * (a_ym[k] + b_ym[k]);
        s += w1 * (a_yp[k] - b_yp[k]);
        s += w1 * (a_zm[k] + b_zm[k]);
        s += w1 * (a_zp[k] - b_zp[k]);
        out[k] = s;
    }
    // ghost columns keep their (zero) phi; write only interior nodes
    if (x4 >= 1 && x4 + 3 <= nx - 2) {
        *reinterpret_cast<float4 *>(b.phi_dst + r0 + x4) = make_float4(out[0], out[1], out[2], out[3]);
    } else {
        for (int k = 0; k < 4; ++k) {
            const int x = x4 + k;
            if (x >= 1 && x <= nx - 2) b.phi_dst[r0 + x] = out[k];
        }
    }
}

// FP32 phase step with 128-bit accesses: one thread owns 4 consecutive x
// nodes (nx % 4 == 0), reads the phi/J rows of its y and z neighbours as
// float4 and the two x-end neighbours (periodically wrapped) as scalars.
// The jet's boundary planes z = 1 and nz-2 go through phase_node, one node
// per thread, in grid slices of their own.
template <int QQ, bool JET, class S>
__global__ void __launch_bounds__(256, 4)
    k_phase_v4(const __grid_constant__ Params<float> p, const __grid_constant__ StepBuffers<S, float> b) {
    const int nx = p.nx, ny = p.ny, nz = p.nz;
    const int x4 = 4 * (blockIdx.x * blockDim.x + threadIdx.x);
    const int y = blockIdx.y * blockDim.y + threadIdx.y;
    const uint32_t t = static_cast<uint32_t>(*b.step_in);
    if (blockIdx.x == 0 && blockIdx.y == 0 && blockIdx.z == 0 && threadIdx.x == 0 && threadIdx.y == 0)
        *b.step_out = *b.step_in + 1ull;
    int z = blockIdx.z;
    if constexpr (JET) {
        // grid.z = nz + 4: slices 0-3 and 4-7 are the boundary planes 1 and
        // nz-2, one node per thread (x = x4 + slice), scheduled first because
        // their rebuilds are the longest; slices 8.. are planes 2 .. nz-3
        if (blockIdx.z < 8) {
            const int zb = blockIdx.z < 4 ? 1 : nz - 2;
            const int x = x4 + (blockIdx.z & 3);
            if (x >= 1 && x <= nx - 2 && y >= 1 && y <= ny - 2) phase_node_outlined<QQ, JET, S>(p, b, x, y, zb, t);
            return;
        }
        z = blockIdx.z - 6;
    }
    if (x4 >= nx || y < 1 || y > ny - 2 || z < 1 || z > nz - 2) return;
    phase_vec4<JET, S>(p, b, x4, y, z);
}

// ------------------------------------------------------------ init
// Initial macroscopic fields into the analysis cache (rho, u, phi), every
// node: setInitialDensity + setJet / setDroplet (src/initialConditions.cu:33-99).
struct InitGeom {
    int jet;
    float droplet_x_stretch;
    float center_z;
    int radius;
    float interface_width;
    float init_noise;
};

template <class T>
__global__ void k_init_fields(const Params<T> p, const InitGeom g, T *macro) {
    const int nx = p.nx, ny = p.ny, nz = p.nz;
    const uint64_t N = p.N;
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    const int y = blockIdx.y * blockDim.y + threadIdx.y;
    const int z = blockIdx.z * blockDim.z + threadIdx.z;
    if (x >= nx || y >= ny || z >= nz) return;
    const uint64_t i = static_cast<uint64_t>(x) + static_cast<uint64_t>(nx) * (y + static_cast<uint64_t>(ny) * z);
    for (int s = 0; s < M_COUNT; ++s) macro[s * N + i] = T(0);
    macro[M_RHO * N + i] = T(1);
    if (g.jet) {
        if (z == 0 && in_disc<T>(p, x, y)) {
            macro[M_PHI * N + i] = T(1);
            macro[M_UZ * N + i] = p.u_inf;
        }
    } else if (x >= 1 && x <= nx - 2 && y >= 1 && y <= ny - 2 && z >= 1 && z <= nz - 2) {
        const T dx = (static_cast<T>(x) - p.center_x) / static_cast<T>(g.droplet_x_stretch);
        const T dy = static_cast<T>(y) - p.center_y;
        const T dz = static_cast<T>(z) - static_cast<T>(g.center_z);
        const T L2 = sqrt(dx * dx + dy * dy + dz * dz);
        const T arg = static_cast<T>((static_cast<double>(g.radius) - static_cast<double>(L2)) / static_cast<double>(g.interface_width));
        macro[M_PHI * N + i] = T(0.5) + T(0.5) * tanh(T(2) * arg);
        if (g.init_noise != 0.0f) {
            macro[M_UX * N + i] = static_cast<T>(g.init_noise * init_noise_value(p.seed, 0, x, y, z));
            macro[M_UY * N + i] = static_cast<T>(g.init_noise * init_noise_value(p.seed, 1, x, y, z));
            macro[M_UZ * N + i] = static_cast<T>(g.init_noise * init_noise_value(p.seed, 2, x, y, z));
        }
    }
}

// setDistros (src/initialConditions.cu:101-138) expressed in the pull
// layout: f^0_q(X) = feq_q(rho_X, u_X) is written to slot X - c_q of both
// ping-pong buffers; phi^0 = sum_q geq_q (computePhase of step 0); ghost phi
// takes the initial ghost values.
template <int QQ, bool JET, class S>
__global__ void k_init_distros(const Params<typename Store<S>::T> p, S *fa, S *fb, typename Store<S>::T *phia,
                               typename Store<S>::T *phib, const typename Store<S>::T *macro) {
    using T = typename Store<S>::T;
    const int nx = p.nx, ny = p.ny, nz = p.nz;
    const uint64_t N = p.N;
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    const int y = blockIdx.y * blockDim.y + threadIdx.y;
    const int z = blockIdx.z * blockDim.z + threadIdx.z;
    if (x >= nx || y >= ny || z >= nz) return;
    const uint64_t i = static_cast<uint64_t>(x) + static_cast<uint64_t>(nx) * (y + static_cast<uint64_t>(ny) * z);
    const T phi0 = macro[M_PHI * N + i];
    if (x < 1 || x > nx - 2 || y < 1 || y > ny - 2 || z < 1 || z > nz - 2) {
        phia[i] = phi0;
        phib[i] = phi0;
        return;
    }
    const T rho = macro[M_RHO * N + i], ux = macro[M_UX * N + i], uy = macro[M_UY * N + i], uz = macro[M_UZ * N + i];
#pragma unroll
    for (int q = 0; q < QQ; ++q) {
        const T v = feq_q<QQ, T>(q, rho, ux, uy, uz);
        const int64_t off = kCX[q] + static_cast<int64_t>(kCY[q]) * nx + static_cast<int64_t>(kCZ[q]) * static_cast<int64_t>(p.plane);
        Store<S>::store(fa, q * N + i - off, v, static_cast<T>(1.0 / weight<QQ>(q)));
        Store<S>::store(fb, q * N + i - off, v, static_cast<T>(1.0 / weight<QQ>(q)));
    }
    T s = T(0);
#pragma unroll
    for (int q = 0; q < 7; ++q) {
        const T w = static_cast<T>(weight7(q));
        s += w * phi0 * (T(1) + T(4) * cdot<T>(kCX[q], kCY[q], kCZ[q], ux, uy, uz));
    }
    phia[i] = s;
    phib[i] = phi0;
}

// Ghost-shell values of the reference's arrays after a step (analysis):
// rho = 1 and zeros (FieldAllocate memset + setInitialDensity), inlet ghost
// plane from the inflow, outlet ghost plane copied from nz-2.
template <class T>
__global__ void k_analysis_ghosts(const Params<T> p, int jet, uint32_t t, T *macro) {
    const int nx = p.nx, ny = p.ny, nz = p.nz;
    const uint64_t N = p.N;
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    const int y = blockIdx.y * blockDim.y + threadIdx.y;
    const int z = blockIdx.z * blockDim.z + threadIdx.z;
    if (x >= nx || y >= ny || z >= nz) return;
    if (x >= 1 && x <= nx - 2 && y >= 1 && y <= ny - 2 && z >= 1 && z <= nz - 2) return;
    const uint64_t i = static_cast<uint64_t>(x) + static_cast<uint64_t>(nx) * (y + static_cast<uint64_t>(ny) * z);
    for (int s = 0; s < M_COUNT; ++s) macro[s * N + i] = T(0);
    macro[M_RHO * N + i] = T(1);
    if (!jet) return;
    if (z == 0 && in_disc<T>(p, x, y)) {
        T ux, uy, uz;
        inflow_velocity<T>(p, x, y, t, ux, uy, uz);
        macro[M_PHI * N + i] = T(1);
        macro[M_UX * N + i] = ux;
        macro[M_UY * N + i] = uy;
        macro[M_UZ * N + i] = uz;
    } else if (z == nz - 1 && x >= 1 && x <= nx - 2 && y >= 1 && y <= ny - 2) {
        const uint64_t j = i - p.plane;
        for (int s : {(int)M_RHO, (int)M_PHI, (int)M_UX, (int)M_UY, (int)M_UZ}) macro[s * N + i] = macro[s * N + j];
    }
}

// Vorticity by central differences, src/derivedFields/operators/vorticityFields.cuh:37-105.
template <class T>
__global__ void k_vorticity(const Params<T> p, const T *macro, T *vort) {
    const int nx = p.nx, ny = p.ny, nz = p.nz;
    const uint64_t N = p.N;
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    const int y = blockIdx.y * blockDim.y + threadIdx.y;
    const int z = blockIdx.z * blockDim.z + threadIdx.z;
    if (x >= nx || y >= ny || z >= nz) return;
    const uint64_t i = static_cast<uint64_t>(x) + static_cast<uint64_t>(nx) * (y + static_cast<uint64_t>(ny) * z);
    T wx = T(0), wy = T(0), wz = T(0);
    if (x > 0 && x < nx - 1 && y > 0 && y < ny - 1 && z > 0 && z < nz - 1) {
        const T *ux = macro + M_UX * N, *uy = macro + M_UY * N, *uz = macro + M_UZ * N;
        const uint64_t sx = 1, sy = nx, sz = p.plane;
        const T h = T(0.5);
        const T duz_dy = h * (uz[i + sy] - uz[i - sy]);
        const T duy_dz = h * (uy[i + sz] - uy[i - sz]);
        const T dux_dz = h * (ux[i + sz] - ux[i - sz]);
        const T duz_dx = h * (uz[i + sx] - uz[i - sx]);
        const T duy_dx = h * (uy[i + sx] - uy[i - sx]);
        const T dux_dy = h * (ux[i + sy] - ux[i - sy]);
        wx = duz_dy - duy_dz;
        wy = dux_dz - duz_dx;
        wz = duy_dx - dux_dy;
    }
    vort[i] = wx;
    vort[N + i] = wy;
    vort[2 * N + i] = wz;
    vort[3 * N + i] = sqrt(wx * wx + wy * wy + wz * wz);
}

// FP64 diagnostics: per-block partial sums over interior nodes, then a
// single-block pass over the partials in fixed order (deterministic).
constexpr int RED_THREADS = 256;
constexpr int RED_FIELDS = 12;  // phi, rho, rho ux, rho uy, rho uz, max|u|, rho_in, n_in, rho_out, n_out, nonfinite, spare

template <class T>
__global__ void __launch_bounds__(RED_THREADS) k_reduce_partial(const Params<T> p, const T *macro, double *partial) {
    const int nx = p.nx, ny = p.ny, nz = p.nz;
    const uint64_t N = p.N;
    const uint64_t nint = static_cast<uint64_t>(nx - 2) * (ny - 2) * (nz - 2);
    double acc[RED_FIELDS] = {0};
    for (uint64_t k = blockIdx.x * static_cast<uint64_t>(RED_THREADS) + threadIdx.x; k < nint;
         k += static_cast<uint64_t>(gridDim.x) * RED_THREADS) {
        const uint64_t xi = k % (nx - 2), r = k / (nx - 2);
        const uint64_t yi = r % (ny - 2), zi = r / (ny - 2);
        const uint64_t i = (xi + 1) + static_cast<uint64_t>(nx) * ((yi + 1) + static_cast<uint64_t>(ny) * (zi + 1));
        const double phi = macro[M_PHI * N + i], rho = macro[M_RHO * N + i];
        const double ux = macro[M_UX * N + i], uy = macro[M_UY * N + i], uz = macro[M_UZ * N + i];
        if (!isfinite(phi) || !isfinite(rho) || !isfinite(ux) || !isfinite(uy) || !isfinite(uz)) {
            acc[10] += 1.0;
            continue;
        }
        acc[0] += phi;
        acc[1] += rho;
        acc[2] += rho * ux;
        acc[3] += rho * uy;
        acc[4] += rho * uz;
        acc[5] = fmax(acc[5], sqrt(ux * ux + uy * uy + uz * uz));
        if (phi > 0.9) { acc[6] += rho; acc[7] += 1.0; }
        if (phi < 0.1) { acc[8] += rho; acc[9] += 1.0; }
    }
    __shared__ double sh[RED_FIELDS][RED_THREADS];
    for (int f = 0; f < RED_FIELDS; ++f) sh[f][threadIdx.x] = acc[f];
    __syncthreads();
    for (int s = RED_THREADS / 2; s > 0; s >>= 1) {
        if (threadIdx.x < s)
            for (int f = 0; f < RED_FIELDS; ++f)
                sh[f][threadIdx.x] = (f == 5) ? fmax(sh[f][threadIdx.x], sh[f][threadIdx.x + s])
                                              : sh[f][threadIdx.x] + sh[f][threadIdx.x + s];
        __syncthreads();
    }
    if (threadIdx.x < RED_FIELDS) partial[blockIdx.x * RED_FIELDS + threadIdx.x] = sh[threadIdx.x][0];
}

static __global__ void __launch_bounds__(32) k_reduce_final(const double *partial, int nblocks, double *out) {
    const int f = threadIdx.x;
    if (f >= RED_FIELDS) return;
    double s = 0.0;
    for (int b = 0; b < nblocks; ++b) {
        const double v = partial[b * RED_FIELDS + f];
        s = (f == 5) ? fmax(s, v) : s + v;
    }
    out[f] = s;
}

}  // namespace pflbm
