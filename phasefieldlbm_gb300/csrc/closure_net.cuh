// closure_net.cuh - the closure network in the collide kernel: blob layout, per-thread
// evaluation (FP64 runs) and the per-warp tensor-core evaluation (FP32 runs).
#pragma once
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cstdint>

namespace pflbm {

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
// One more device word after the user-visible blob: the inverse turbulent
// Schmidt number of the closure's phase mixing (0 = off), set by
// pflbm_set_closure_mixing.
constexpr int kMlpPhaseMix = kMlpBlob;
constexpr int kMlpDeviceFloats = kMlpBlob + 1;

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
static_assert(kMlpFragF1 >= kMlpDeviceFloats, "fragments after the device blob");

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

}  // namespace pflbm
