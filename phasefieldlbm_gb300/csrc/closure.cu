// closure.cu - the learned eddy-viscosity closure: training data from
// box-filtered, 2x-restricted snapshots of a fine run of this solver, and
// the MLP's forward, backward and Adam kernels (no counterpart in the
// reference, whose collision uses a constant tau per phase, lbm.cu:158-170).
//
// Network (same as the collide kernel's mlp_nu_t): features x = (Pi_xx,
// Pi_yy, Pi_zz, Pi_xy, Pi_xz, Pi_yz, phi, |grad phi|), x' = (x - mean) *
// inv_scale, h1 = SiLU(W1 x' + b1), h2 = SiLU(W2 h1 + b2),
// nu_t = out_scale * softplus(w3 . h2 + b3). Training loss per sample:
// (softplus(z) - target / out_scale)^2, averaged over a minibatch.
//
// Training data. A coarse node X of the 2x-coarser grid sits on fine node
// 2X. Fine rho, u, phi and the products u_a u_b are averaged over the 3x3x3
// fine box around 2X (box filter + restriction). On the coarse grid:
//   S_ab   = (d_a u_b + d_b u_a) / 2, central differences (coarse spacing 1),
//   tau_ab = <u_a u_b> - <u_a><u_b> (sub-filter stress),
//   target nu_t = min(kMaxNuT, max(0, -dev(tau) : S / (2 S : S))), 0 where
//            S : S < kMinStrain2 (least-squares eddy viscosity, coarse
//            lattice units),
//   features: Pi = -2 rho cs^2 tau0 dev(S) (the non-equilibrium stress the
//            coarse solver carries, Chapman-Enskog, tau0 its molecular
//            relaxation time), phi, |grad phi| (D3Q19 lattice gradient, as
//            the solver's normals stencil).
//
// Interface width. The same sample nodes give the thickness of the phase
// interface: for a tanh profile, sum phi (1 - phi) / sum |grad phi| is a
// quarter of the width W. Measured on the filtered coarse field (coarse
// units) and on the fine field at the sample's fine node 2X (fine units, the
// solver's own |grad phi|), their ratio is the factor by which the coarse
// run's interface sharpening gamma must grow for its equilibrium interface
// (W proportional to 1 / gamma at the fixed phase mobility) to have the
// filtered fine width; the coarse grid otherwise resolves an interface twice
// as thick in physical units.
#include <cuda_runtime.h>

#include <cmath>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <memory>
#include <new>
#include <string>
#include <vector>

#include "../../include/pflbm.h"
#include "engine.h"
#include "kernels.cuh"

namespace {

using pflbm::kMlpBlob;
using pflbm::kMlpH;
using pflbm::kMlpIn;
using pflbm::kMlpParams;

static_assert(kMlpParams == PFLBM_MLP_PARAMS && kMlpBlob == PFLBM_MLP_BLOB, "closure blob layout");
static_assert(kMlpParams == pflbm::kMlpParamFloats && kMlpBlob == pflbm::kMlpBlobFloats, "closure blob layout");
static_assert(pflbm::kMlpStrength == kMlpBlob - 1, "strength is the last blob entry");

constexpr int kSB = 128;            // samples per training block
constexpr int kCoarseFields = 11;   // rho, ux, uy, uz, phi, tau_xx, tau_yy, tau_zz, tau_xy, tau_xz, tau_yz
constexpr int kLossBlocks = 1024;
constexpr float kMinStrain2 = 1e-10f;  // S:S below which the target is 0
constexpr float kMaxNuT = 2e-3f;       // cap of the target eddy viscosity (lattice units)

int fail(int code, const std::string &msg) {
    pflbm::set_error(msg);
    return code;
}

int cuda_fail(cudaError_t e, const char *what) {
    cudaGetLastError();
    return fail(PFLBM_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}

__host__ __device__ inline uint64_t mix64(uint64_t x) {
    x ^= x >> 30;
    x *= 0xbf58476d1ce4e5b9ull;
    x ^= x >> 27;
    x *= 0x94d049bb133111ebull;
    x ^= x >> 31;
    return x;
}

__device__ __forceinline__ float sigmoidf_(float a) { return 1.0f / (1.0f + expf(-a)); }

// ------------------------------------------------------------- data
__global__ void k_filter_restrict(const float *__restrict__ macro, uint64_t Nf, int nxf, int nyf, int nzf, int nxc,
                                  int nyc, int nzc, float *__restrict__ coarse) {
    const uint64_t Nc = uint64_t(nxc) * nyc * nzc;
    for (uint64_t c = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x; c < Nc; c += uint64_t(gridDim.x) * blockDim.x) {
        const int i = int(c % nxc), j = int((c / nxc) % nyc), k = int(c / (uint64_t(nxc) * nyc));
        double s[11] = {0};
        for (int dz = -1; dz <= 1; ++dz)
            for (int dy = -1; dy <= 1; ++dy)
                for (int dx = -1; dx <= 1; ++dx) {
                    const int X = min(max(2 * i + dx, 0), nxf - 1), Y = min(max(2 * j + dy, 0), nyf - 1),
                              Z = min(max(2 * k + dz, 0), nzf - 1);
                    const uint64_t f = uint64_t(X) + uint64_t(nxf) * (uint64_t(Y) + uint64_t(nyf) * Z);
                    const double r = macro[pflbm::M_RHO * Nf + f], ux = macro[pflbm::M_UX * Nf + f],
                                 uy = macro[pflbm::M_UY * Nf + f], uz = macro[pflbm::M_UZ * Nf + f],
                                 ph = macro[pflbm::M_PHI * Nf + f];
                    s[0] += r; s[1] += ux; s[2] += uy; s[3] += uz; s[4] += ph;
                    s[5] += ux * ux; s[6] += uy * uy; s[7] += uz * uz;
                    s[8] += ux * uy; s[9] += ux * uz; s[10] += uy * uz;
                }
        for (int q = 0; q < 11; ++q) s[q] *= 1.0 / 27.0;
        coarse[0 * Nc + c] = float(s[0]);
        coarse[1 * Nc + c] = float(s[1]);
        coarse[2 * Nc + c] = float(s[2]);
        coarse[3 * Nc + c] = float(s[3]);
        coarse[4 * Nc + c] = float(s[4]);
        coarse[5 * Nc + c] = float(s[5] - s[1] * s[1]);
        coarse[6 * Nc + c] = float(s[6] - s[2] * s[2]);
        coarse[7 * Nc + c] = float(s[7] - s[3] * s[3]);
        coarse[8 * Nc + c] = float(s[8] - s[1] * s[2]);
        coarse[9 * Nc + c] = float(s[9] - s[1] * s[3]);
        coarse[10 * Nc + c] = float(s[10] - s[2] * s[3]);
    }
}

// Samples at coarse nodes 2 <= i,j,k <= n-3 with i % stride == 0 and
// j % stride == 0, written in (k, j, i) order from `base`.
// Each block also writes its sums of phi(1-phi) and |grad phi| on the
// filtered coarse field and on the fine field at 2X (width[blockIdx.x * 4 +
// 0..3], FP64, summed in block order on the host).
constexpr int kMakeThreads = 256, kMakeBlocks = 1216;
__global__ void __launch_bounds__(kMakeThreads) k_make_samples(const float *__restrict__ coarse, int nxc, int nyc,
                                                               int nzc, int stride, float tau_w, float tau_o, int i0,
                                                               int ni, int j0, int nj, float *__restrict__ X,
                                                               float *__restrict__ Y, uint64_t base,
                                                               const float *__restrict__ macro, uint64_t Nf, int nxf,
                                                               int nyf, double *__restrict__ width) {
    const uint64_t Nc = uint64_t(nxc) * nyc * nzc;
    const uint64_t total = uint64_t(ni) * nj * (nzc - 4);
    double wsum[4] = {0.0, 0.0, 0.0, 0.0};
    for (uint64_t s = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x; s < total; s += uint64_t(gridDim.x) * blockDim.x) {
        const int ii = int(s % ni), jj = int((s / ni) % nj), kk = int(s / (uint64_t(ni) * nj));
        const int i = i0 + ii * stride, j = j0 + jj * stride, k = 2 + kk;
        auto at = [&](int f, int x, int y, int z) -> float {
            return coarse[f * Nc + uint64_t(x) + uint64_t(nxc) * (uint64_t(y) + uint64_t(nyc) * z)];
        };
        float g[3][3];  // g[a][b] = d_a u_b
        for (int b = 0; b < 3; ++b) {
            g[0][b] = 0.5f * (at(1 + b, i + 1, j, k) - at(1 + b, i - 1, j, k));
            g[1][b] = 0.5f * (at(1 + b, i, j + 1, k) - at(1 + b, i, j - 1, k));
            g[2][b] = 0.5f * (at(1 + b, i, j, k + 1) - at(1 + b, i, j, k - 1));
        }
        const float sxx = g[0][0], syy = g[1][1], szz = g[2][2];
        const float sxy = 0.5f * (g[0][1] + g[1][0]), sxz = 0.5f * (g[0][2] + g[2][0]), syz = 0.5f * (g[1][2] + g[2][1]);
        const float tr = (sxx + syy + szz) / 3.0f;
        const float dxx = sxx - tr, dyy = syy - tr, dzz = szz - tr;
        const float rho = at(0, i, j, k), phi = at(4, i, j, k);
        const float tau0 = (1.0f - phi) * tau_w + phi * tau_o;
        const float c = -2.0f * rho * tau0 / 3.0f;
        // |grad phi| with the D3Q19 lattice gradient (3 sum_q w_q c_q phi(x + c_q))
        float gx = 0.f, gy = 0.f, gz = 0.f;
#pragma unroll
        for (int q = 1; q < 19; ++q) {
            const float w = pflbm::weight<19>(q) * at(4, i + pflbm::kCX[q], j + pflbm::kCY[q], k + pflbm::kCZ[q]);
            gx += w * pflbm::kCX[q];
            gy += w * pflbm::kCY[q];
            gz += w * pflbm::kCZ[q];
        }
        const float ind = 3.0f * sqrtf(gx * gx + gy * gy + gz * gz);
        // least-squares eddy viscosity of the sub-filter stress
        const float txx = at(5, i, j, k), tyy = at(6, i, j, k), tzz = at(7, i, j, k);
        const float txy = at(8, i, j, k), txz = at(9, i, j, k), tyz = at(10, i, j, k);
        const float ttr = (txx + tyy + tzz) / 3.0f;
        const float num = -((txx - ttr) * sxx + (tyy - ttr) * syy + (tzz - ttr) * szz +
                            2.0f * (txy * sxy + txz * sxz + tyz * syz));
        const float den = 2.0f * (sxx * sxx + syy * syy + szz * szz + 2.0f * (sxy * sxy + sxz * sxz + syz * syz));
        // quiescent nodes (S:S below kMinStrain2) carry no information on
        // nu_t; the cap removes the heavy tail of near-zero strain rates
        const float nu = den > 2.0f * kMinStrain2 ? fminf(fmaxf(0.0f, num / den), kMaxNuT) : 0.0f;
        float *x = X + (base + s) * kMlpIn;
        x[0] = c * dxx; x[1] = c * dyy; x[2] = c * dzz;
        x[3] = c * sxy; x[4] = c * sxz; x[5] = c * syz;
        x[6] = phi; x[7] = ind;
        Y[base + s] = nu;
        const uint64_t f = uint64_t(2 * i) + uint64_t(nxf) * (uint64_t(2 * j) + uint64_t(nyf) * uint64_t(2 * k));
        const double phf = macro[pflbm::M_PHI * Nf + f], indf = macro[pflbm::M_IND * Nf + f];
        wsum[0] += double(phi) * (1.0 - double(phi));
        wsum[1] += double(ind);
        wsum[2] += phf * (1.0 - phf);
        wsum[3] += indf;
    }
    __shared__ double red[4][kMakeThreads];
    for (int q = 0; q < 4; ++q) red[q][threadIdx.x] = wsum[q];
    __syncthreads();
    for (int h = kMakeThreads / 2; h > 0; h >>= 1) {
        if (int(threadIdx.x) < h)
            for (int q = 0; q < 4; ++q) red[q][threadIdx.x] += red[q][threadIdx.x + h];
        __syncthreads();
    }
    if (threadIdx.x < 4) width[blockIdx.x * 4 + threadIdx.x] = red[threadIdx.x][0];
}

// FP64 sums of x_k, x_k^2 (k < 8), y, y^2 per block.
__global__ void __launch_bounds__(256) k_stats(const float *__restrict__ X, const float *__restrict__ Y, uint64_t n,
                                               double *__restrict__ partial) {
    double acc[18] = {0};
    for (uint64_t s = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x; s < n; s += uint64_t(gridDim.x) * blockDim.x) {
        for (int k = 0; k < kMlpIn; ++k) {
            const double v = X[s * kMlpIn + k];
            acc[k] += v;
            acc[8 + k] += v * v;
        }
        const double y = Y[s];
        acc[16] += y;
        acc[17] += y * y;
    }
    __shared__ double sh[18][256];
    for (int f = 0; f < 18; ++f) sh[f][threadIdx.x] = acc[f];
    __syncthreads();
    for (int st = 128; st > 0; st >>= 1) {
        if (threadIdx.x < st)
            for (int f = 0; f < 18; ++f) sh[f][threadIdx.x] += sh[f][threadIdx.x + st];
        __syncthreads();
    }
    if (threadIdx.x < 18) partial[blockIdx.x * 18 + threadIdx.x] = sh[threadIdx.x][0];
}

// ------------------------------------------------------------- network
struct Act {
    float xn[kSB][kMlpIn];
    float h1[kSB][kMlpH + 1];   // +1: bank-conflict padding
    float da1[kSB][kMlpH + 1];
    float h2[kSB][kMlpH + 1];
    float da2[kSB][kMlpH + 1];
    float dz[kSB];
    float loss[kSB];
};

// Forward + backward over one block of kSB samples. Sample index: k for
// mode 0 (the first n samples in order), else a hash of (seed, iteration, k)
// modulo n. Per-block gradient sums -> gpart[block][0..kMlpParams), the
// block's loss sum -> gpart[block][kMlpParams].
__global__ void __launch_bounds__(kSB) k_mlp_grad(const float *__restrict__ blob, const float *__restrict__ X,
                                                  const float *__restrict__ Y, uint64_t n, int mode, uint64_t seed,
                                                  uint64_t iter, uint64_t count, float *__restrict__ gpart) {
    __shared__ float w[kMlpBlob];
    extern __shared__ unsigned char dyn[];
    Act &A = *reinterpret_cast<Act *>(dyn);
    for (int i = threadIdx.x; i < kMlpBlob; i += kSB) w[i] = blob[i];
    __syncthreads();
    const int t = threadIdx.x;
    const uint64_t k = blockIdx.x * uint64_t(kSB) + t;
    const bool valid = k < count;
    uint64_t idx = 0;
    if (valid) idx = mode == 0 ? k : mix64(seed * 0x9E3779B97F4A7C15ull + mix64(iter * 0x100000001B3ull + k)) % n;
    const float out_scale = w[pflbm::kMlpOutScale];
    float a1[kMlpH], a2[kMlpH];
    float xn[kMlpIn];
    for (int q = 0; q < kMlpIn; ++q)
        xn[q] = valid ? (X[idx * kMlpIn + q] - w[pflbm::kMlpMean + q]) * w[pflbm::kMlpInvScale + q] : 0.0f;
#pragma unroll
    for (int i = 0; i < kMlpH; ++i) {
        float s = w[pflbm::kMlpB1 + i];
#pragma unroll
        for (int q = 0; q < kMlpIn; ++q) s += w[pflbm::kMlpW1 + i * kMlpIn + q] * xn[q];
        a1[i] = s;
        A.h1[t][i] = s * sigmoidf_(s);
    }
    float z = w[pflbm::kMlpB3];
#pragma unroll 4
    for (int j = 0; j < kMlpH; ++j) {
        float s = w[pflbm::kMlpB2 + j];
#pragma unroll
        for (int i = 0; i < kMlpH; ++i) s += w[pflbm::kMlpW2 + j * kMlpH + i] * A.h1[t][i];
        a2[j] = s;
        const float h = s * sigmoidf_(s);
        A.h2[t][j] = h;
        z += w[pflbm::kMlpW3 + j] * h;
    }
    const float sp = fmaxf(z, 0.0f) + log1pf(expf(-fabsf(z)));
    const float r = valid ? sp - Y[idx] / out_scale : 0.0f;
    const float dz = 2.0f * r * sigmoidf_(z);
    A.dz[t] = valid ? dz : 0.0f;
    A.loss[t] = r * r;
#pragma unroll
    for (int q = 0; q < kMlpIn; ++q) A.xn[t][q] = xn[q];
#pragma unroll
    for (int j = 0; j < kMlpH; ++j) {
        const float sg = sigmoidf_(a2[j]);
        A.da2[t][j] = valid ? dz * w[pflbm::kMlpW3 + j] * sg * (1.0f + a2[j] * (1.0f - sg)) : 0.0f;
    }
#pragma unroll 4
    for (int i = 0; i < kMlpH; ++i) {
        float dh = 0.0f;
#pragma unroll
        for (int j = 0; j < kMlpH; ++j) dh += w[pflbm::kMlpW2 + j * kMlpH + i] * A.da2[t][j];
        const float sg = sigmoidf_(a1[i]);
        A.da1[t][i] = dh * sg * (1.0f + a1[i] * (1.0f - sg));
    }
    __syncthreads();
    // parameter gradients: sums over the block's samples, in sample order
    float *g = gpart + size_t(blockIdx.x) * (kMlpParams + 1);
    for (int p = t; p <= kMlpParams; p += kSB) {
        float acc = 0.0f;
        if (p < pflbm::kMlpB1) {  // W1[i][q]
            const int i = p / kMlpIn, q = p % kMlpIn;
            for (int s = 0; s < kSB; ++s) acc += A.da1[s][i] * A.xn[s][q];
        } else if (p < pflbm::kMlpW2) {  // b1[i]
            const int i = p - pflbm::kMlpB1;
            for (int s = 0; s < kSB; ++s) acc += A.da1[s][i];
        } else if (p < pflbm::kMlpB2) {  // W2[j][i]
            const int j = (p - pflbm::kMlpW2) / kMlpH, i = (p - pflbm::kMlpW2) % kMlpH;
            for (int s = 0; s < kSB; ++s) acc += A.da2[s][j] * A.h1[s][i];
        } else if (p < pflbm::kMlpW3) {  // b2[j]
            const int j = p - pflbm::kMlpB2;
            for (int s = 0; s < kSB; ++s) acc += A.da2[s][j];
        } else if (p < pflbm::kMlpB3) {  // w3[j]
            const int j = p - pflbm::kMlpW3;
            for (int s = 0; s < kSB; ++s) acc += A.dz[s] * A.h2[s][j];
        } else if (p == pflbm::kMlpB3) {
            for (int s = 0; s < kSB; ++s) acc += A.dz[s];
        } else {  // loss sum
            for (int s = 0; s < kSB; ++s)
                if (blockIdx.x * uint64_t(kSB) + s < count) acc += A.loss[s];
        }
        g[p] = acc;
    }
}

// ------------------------------------------- network on the tensor cores
// The same forward + backward over kSB = 128 samples per CTA with every
// matrix product on the tensor cores: warp-level mma.m16n8k8 with TF32
// operands (10-bit mantissa, operands rounded to nearest) and FP32
// accumulation. Warp w owns samples 32w .. 32w+31 (two 16-row tiles):
//   layer 1   A1 = Xn W1^T + b1       (16 x 8 x 8 per tile and column block)
//   layer 2   A2 = H1 W2^T + b2       (K = 32: four k steps)
//   backward  dH1 = dA2 W2            (K = 32)
//   weights   dW2 = dA2^T H1, dW1 = dA1^T Xn   (K = the warp's 32 samples)
// and the elementwise parts (SiLU, softplus, bias and w3 sums) in FP32. The
// four warps' partial gradients are summed in warp order: gpart is filled
// as k_mlp_grad fills it (sums over the CTA's samples, loss last).
constexpr int kTcWarps = kSB / 32;
constexpr int kTcX = 12;                 // row stride of the Xn tile (floats)
constexpr int kTcH = kMlpH + 4;          // row stride of the 32-wide tiles
constexpr int kTcWarpFloats = 32 * kTcX + 3 * 32 * kTcH + 32;  // Xn, H1, dA2, dA1, dz
constexpr int kTcPart = kMlpParams + 1;  // per-warp partial gradient + loss

size_t tc_smem_bytes() {
    return sizeof(float) * (size_t(kMlpBlob) + size_t(kTcWarps) * kTcWarpFloats + size_t(kTcWarps) * kTcPart);
}

__device__ __forceinline__ uint32_t to_tf32(float x) {
    uint32_t r;
    asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
    return r;
}

// D = A B + C, A 16x8 (row), B 8x8 (col), TF32 operands, FP32 accumulators.
__device__ __forceinline__ void mma_tf32_1688(float (&d)[4], uint32_t a0, uint32_t a1, uint32_t a2, uint32_t a3,
                                              uint32_t b0, uint32_t b1) {
    asm volatile(
        "mma.sync.aligned.m16n8k8.row.col.f32.tf32.tf32.f32 {%0, %1, %2, %3}, {%4, %5, %6, %7}, {%8, %9}, "
        "{%0, %1, %2, %3};"
        : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
        : "r"(a0), "r"(a1), "r"(a2), "r"(a3), "r"(b0), "r"(b1));
}

__device__ __forceinline__ float silu_grad(float a) {
    const float sg = sigmoidf_(a);
    return sg * (1.0f + a * (1.0f - sg));
}

__global__ void __launch_bounds__(kSB) k_mlp_grad_tc(const float *__restrict__ blob, const float *__restrict__ X,
                                                     const float *__restrict__ Y, uint64_t n, int mode,
                                                     uint64_t seed, uint64_t iter, uint64_t count,
                                                     float *__restrict__ gpart) {
    extern __shared__ float tcs[];
    float *w = tcs;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int g = lane >> 2, t = lane & 3;
    float *base = tcs + kMlpBlob + warp * kTcWarpFloats;
    float *xs = base;                       // [32][kTcX]
    float *h1s = xs + 32 * kTcX;            // [32][kTcH]
    float *da2s = h1s + 32 * kTcH;          // [32][kTcH]
    float *da1s = da2s + 32 * kTcH;         // [32][kTcH]
    float *dzs = da1s + 32 * kTcH;          // [32]
    float *part = tcs + kMlpBlob + kTcWarps * kTcWarpFloats + warp * kTcPart;
    for (int i = threadIdx.x; i < kMlpBlob; i += kSB) w[i] = blob[i];
    __syncthreads();
    const float out_scale = w[pflbm::kMlpOutScale];

    // this lane's sample (row `lane` of the warp's tile): normalised features
    const uint64_t k = blockIdx.x * uint64_t(kSB) + threadIdx.x;
    const bool valid = k < count;
    uint64_t idx = 0;
    if (valid) idx = mode == 0 ? k : mix64(seed * 0x9E3779B97F4A7C15ull + mix64(iter * 0x100000001B3ull + k)) % n;
    for (int q = 0; q < kMlpIn; ++q)
        xs[lane * kTcX + q] = valid ? (X[idx * kMlpIn + q] - w[pflbm::kMlpMean + q]) * w[pflbm::kMlpInvScale + q]
                                    : 0.0f;
    const float target = valid ? Y[idx] / out_scale : 0.0f;
    __syncwarp();

    // layer 1: a1 = Xn W1^T + b1 (fragments: rows 16 mt + g (+8), columns
    // 8 nt + 2 t (+1)); h1 = SiLU(a1) to shared memory
    float a1[2][4][4], a2[2][4][4];
#pragma unroll
    for (int mt = 0; mt < 2; ++mt)
#pragma unroll
        for (int nt = 0; nt < 4; ++nt) {
            float(&d)[4] = a1[mt][nt];
            d[0] = d[2] = w[pflbm::kMlpB1 + 8 * nt + 2 * t];
            d[1] = d[3] = w[pflbm::kMlpB1 + 8 * nt + 2 * t + 1];
            const int r0 = 16 * mt + g;
            mma_tf32_1688(d, to_tf32(xs[r0 * kTcX + t]), to_tf32(xs[(r0 + 8) * kTcX + t]),
                          to_tf32(xs[r0 * kTcX + t + 4]), to_tf32(xs[(r0 + 8) * kTcX + t + 4]),
                          to_tf32(w[pflbm::kMlpW1 + (8 * nt + g) * kMlpIn + t]),
                          to_tf32(w[pflbm::kMlpW1 + (8 * nt + g) * kMlpIn + t + 4]));
#pragma unroll
            for (int e = 0; e < 4; ++e) {
                const int row = r0 + (e >= 2 ? 8 : 0), col = 8 * nt + 2 * t + (e & 1);
                h1s[row * kTcH + col] = d[e] * sigmoidf_(d[e]);
            }
        }
    __syncwarp();
    // layer 2: a2 = H1 W2^T + b2; z = w3 . SiLU(a2) + b3 per sample
    float zp[2][2] = {{0.f, 0.f}, {0.f, 0.f}};  // [mt][row g / g + 8], this lane's columns
#pragma unroll
    for (int mt = 0; mt < 2; ++mt)
#pragma unroll
        for (int nt = 0; nt < 4; ++nt) {
            float(&d)[4] = a2[mt][nt];
            d[0] = d[2] = w[pflbm::kMlpB2 + 8 * nt + 2 * t];
            d[1] = d[3] = w[pflbm::kMlpB2 + 8 * nt + 2 * t + 1];
            const int r0 = 16 * mt + g;
#pragma unroll
            for (int kk = 0; kk < 4; ++kk)
                mma_tf32_1688(d, to_tf32(h1s[r0 * kTcH + 8 * kk + t]), to_tf32(h1s[(r0 + 8) * kTcH + 8 * kk + t]),
                              to_tf32(h1s[r0 * kTcH + 8 * kk + t + 4]),
                              to_tf32(h1s[(r0 + 8) * kTcH + 8 * kk + t + 4]),
                              to_tf32(w[pflbm::kMlpW2 + (8 * nt + g) * kMlpH + 8 * kk + t]),
                              to_tf32(w[pflbm::kMlpW2 + (8 * nt + g) * kMlpH + 8 * kk + t + 4]));
#pragma unroll
            for (int e = 0; e < 4; ++e) {
                const int col = 8 * nt + 2 * t + (e & 1);
                zp[mt][e >> 1] += w[pflbm::kMlpW3 + col] * (d[e] * sigmoidf_(d[e]));
            }
        }
    // complete z over the 4 lanes of a group, then dz per row to shared memory
#pragma unroll
    for (int mt = 0; mt < 2; ++mt)
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            zp[mt][h] += __shfl_xor_sync(0xffffffffu, zp[mt][h], 1);
            zp[mt][h] += __shfl_xor_sync(0xffffffffu, zp[mt][h], 2);
        }
    if (t == 0) {
#pragma unroll
        for (int mt = 0; mt < 2; ++mt)
#pragma unroll
            for (int h = 0; h < 2; ++h) dzs[16 * mt + g + 8 * h] = zp[mt][h] + w[pflbm::kMlpB3];
    }
    __syncwarp();
    // this lane's own sample: loss and dz
    float loss_l, dz_l;
    {
        const float z = dzs[lane];
        const float sp = fmaxf(z, 0.0f) + log1pf(expf(-fabsf(z)));
        const float r = valid ? sp - target : 0.0f;
        loss_l = valid ? r * r : 0.0f;
        dz_l = valid ? 2.0f * r * sigmoidf_(z) : 0.0f;
    }
    __syncwarp();
    dzs[lane] = dz_l;
    __syncwarp();
    // backward: dA2 = dz w3 SiLU'(a2); dw3 partials over this lane's rows
    float dw3p[4][2] = {};
#pragma unroll
    for (int mt = 0; mt < 2; ++mt)
#pragma unroll
        for (int nt = 0; nt < 4; ++nt)
#pragma unroll
            for (int e = 0; e < 4; ++e) {
                const int row = 16 * mt + g + (e >= 2 ? 8 : 0), col = 8 * nt + 2 * t + (e & 1);
                const float dz = dzs[row], av = a2[mt][nt][e];
                da2s[row * kTcH + col] = dz * w[pflbm::kMlpW3 + col] * silu_grad(av);
                dw3p[nt][e & 1] += dz * (av * sigmoidf_(av));
            }
    __syncwarp();
    // dH1 = dA2 W2, dA1 = dH1 SiLU'(a1)
#pragma unroll
    for (int mt = 0; mt < 2; ++mt)
#pragma unroll
        for (int nt = 0; nt < 4; ++nt) {
            float d[4] = {0.f, 0.f, 0.f, 0.f};
            const int r0 = 16 * mt + g;
#pragma unroll
            for (int kk = 0; kk < 4; ++kk)
                mma_tf32_1688(d, to_tf32(da2s[r0 * kTcH + 8 * kk + t]), to_tf32(da2s[(r0 + 8) * kTcH + 8 * kk + t]),
                              to_tf32(da2s[r0 * kTcH + 8 * kk + t + 4]),
                              to_tf32(da2s[(r0 + 8) * kTcH + 8 * kk + t + 4]),
                              to_tf32(w[pflbm::kMlpW2 + (8 * kk + t) * kMlpH + 8 * nt + g]),
                              to_tf32(w[pflbm::kMlpW2 + (8 * kk + t + 4) * kMlpH + 8 * nt + g]));
#pragma unroll
            for (int e = 0; e < 4; ++e) {
                const int row = r0 + (e >= 2 ? 8 : 0), col = 8 * nt + 2 * t + (e & 1);
                da1s[row * kTcH + col] = d[e] * silu_grad(a1[mt][nt][e]);
            }
        }
    __syncwarp();
    // weight gradients over the warp's 32 samples (K)
#pragma unroll
    for (int mt = 0; mt < 2; ++mt) {
#pragma unroll
        for (int nt = 0; nt < 4; ++nt) {  // dW2[j][i] = sum_s dA2[s][j] H1[s][i]
            float d[4] = {0.f, 0.f, 0.f, 0.f};
#pragma unroll
            for (int kk = 0; kk < 4; ++kk)
                mma_tf32_1688(d, to_tf32(da2s[(8 * kk + t) * kTcH + 16 * mt + g]),
                              to_tf32(da2s[(8 * kk + t) * kTcH + 16 * mt + g + 8]),
                              to_tf32(da2s[(8 * kk + t + 4) * kTcH + 16 * mt + g]),
                              to_tf32(da2s[(8 * kk + t + 4) * kTcH + 16 * mt + g + 8]),
                              to_tf32(h1s[(8 * kk + t) * kTcH + 8 * nt + g]),
                              to_tf32(h1s[(8 * kk + t + 4) * kTcH + 8 * nt + g]));
#pragma unroll
            for (int e = 0; e < 4; ++e) {
                const int j = 16 * mt + g + (e >= 2 ? 8 : 0), i = 8 * nt + 2 * t + (e & 1);
                part[pflbm::kMlpW2 + j * kMlpH + i] = d[e];
            }
        }
        float d[4] = {0.f, 0.f, 0.f, 0.f};  // dW1[i][q] = sum_s dA1[s][i] Xn[s][q]
#pragma unroll
        for (int kk = 0; kk < 4; ++kk)
            mma_tf32_1688(d, to_tf32(da1s[(8 * kk + t) * kTcH + 16 * mt + g]),
                          to_tf32(da1s[(8 * kk + t) * kTcH + 16 * mt + g + 8]),
                          to_tf32(da1s[(8 * kk + t + 4) * kTcH + 16 * mt + g]),
                          to_tf32(da1s[(8 * kk + t + 4) * kTcH + 16 * mt + g + 8]),
                          to_tf32(xs[(8 * kk + t) * kTcX + g]), to_tf32(xs[(8 * kk + t + 4) * kTcX + g]));
#pragma unroll
        for (int e = 0; e < 4; ++e) {
            const int i = 16 * mt + g + (e >= 2 ? 8 : 0), q = 2 * t + (e & 1);
            part[pflbm::kMlpW1 + i * kMlpIn + q] = d[e];
        }
    }
    // bias and w3 gradients, loss: column sums over the warp's samples
    {
        float sb1 = 0.f, sb2 = 0.f;
        for (int s = 0; s < 32; ++s) {
            sb1 += da1s[s * kTcH + lane];
            sb2 += da2s[s * kTcH + lane];
        }
        part[pflbm::kMlpB1 + lane] = sb1;
        part[pflbm::kMlpB2 + lane] = sb2;
    }
#pragma unroll
    for (int nt = 0; nt < 4; ++nt)
#pragma unroll
        for (int c = 0; c < 2; ++c) {
            float v = dw3p[nt][c];
            v += __shfl_xor_sync(0xffffffffu, v, 4);
            v += __shfl_xor_sync(0xffffffffu, v, 8);
            v += __shfl_xor_sync(0xffffffffu, v, 16);
            if (g == 0) part[pflbm::kMlpW3 + 8 * nt + 2 * t + c] = v;
        }
    {
        float sdz = dz_l, sl = loss_l;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            sdz += __shfl_xor_sync(0xffffffffu, sdz, o);
            sl += __shfl_xor_sync(0xffffffffu, sl, o);
        }
        if (lane == 0) {
            part[pflbm::kMlpB3] = sdz;
            part[kMlpParams] = sl;
        }
    }
    __syncthreads();
    // the block's sums, warps in order
    float *gout = gpart + size_t(blockIdx.x) * (kMlpParams + 1);
    const float *parts = tcs + kMlpBlob + kTcWarps * kTcWarpFloats;
    for (int p = threadIdx.x; p <= kMlpParams; p += kSB) {
        float acc = 0.0f;
#pragma unroll
        for (int ww = 0; ww < kTcWarps; ++ww) acc += parts[ww * kTcPart + p];
        gout[p] = acc;
    }
}

// Sums the block gradients (fixed order, FP64) into grad[0..kMlpParams]
// (the last entry is the loss sum).
__global__ void k_grad_sum(const float *__restrict__ gpart, int nblocks, double *__restrict__ grad) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p > kMlpParams) return;
    double s = 0.0;
    for (int b = 0; b < nblocks; ++b) s += gpart[size_t(b) * (kMlpParams + 1) + p];
    grad[p] = s;
}

// Adam on the mean minibatch gradient; loss_log[iter] = mean minibatch loss.
__global__ void k_adam(float *__restrict__ blob, float *__restrict__ m, float *__restrict__ v,
                       const float *__restrict__ gpart, int nblocks, float inv_count, float lr, float beta1,
                       float beta2, float eps, float c1, float c2, double *__restrict__ loss_log, int iter) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p > kMlpParams) return;
    double s = 0.0;
    for (int b = 0; b < nblocks; ++b) s += gpart[size_t(b) * (kMlpParams + 1) + p];
    if (p == kMlpParams) {
        loss_log[iter] = s * inv_count;
        return;
    }
    const float g = float(s) * inv_count;
    const float mm = beta1 * m[p] + (1.0f - beta1) * g;
    const float vv = beta2 * v[p] + (1.0f - beta2) * g * g;
    m[p] = mm;
    v[p] = vv;
    blob[p] -= lr * (mm / c1) / (sqrtf(vv / c2) + eps);
}

// Forward only: FP64 loss sum per block.
__global__ void __launch_bounds__(256) k_mlp_loss(const float *__restrict__ blob, const float *__restrict__ X,
                                                  const float *__restrict__ Y, uint64_t n, double *__restrict__ partial) {
    __shared__ float w[kMlpBlob];
    for (int i = threadIdx.x; i < kMlpBlob; i += blockDim.x) w[i] = blob[i];
    __syncthreads();
    double acc = 0.0;
    for (uint64_t s = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x; s < n; s += uint64_t(gridDim.x) * blockDim.x) {
        float x[kMlpIn];
        for (int q = 0; q < kMlpIn; ++q) x[q] = X[s * kMlpIn + q];
        const float nu = pflbm::mlp_nu_t<float>(w, x);
        const float r = (nu - Y[s]) / w[pflbm::kMlpOutScale];
        acc += double(r) * r;
    }
    __shared__ double sh[256];
    sh[threadIdx.x] = acc;
    __syncthreads();
    for (int st = 128; st > 0; st >>= 1) {
        if (threadIdx.x < st) sh[threadIdx.x] += sh[threadIdx.x + st];
        __syncthreads();
    }
    if (threadIdx.x == 0) partial[blockIdx.x] = sh[0];
}

}  // namespace

// ------------------------------------------------------------- object
struct pflbm_closure {
    int device = 0;
    cudaStream_t stream = nullptr;
    uint64_t cap = 0, n = 0;
    float *X = nullptr, *Y = nullptr;
    float *blob = nullptr, *m = nullptr, *v = nullptr;
    float *gpart = nullptr;
    int gpart_blocks = 0;
    double *grad = nullptr, *partial = nullptr, *loss_log = nullptr;
    int loss_log_cap = 0;
    float *coarse = nullptr;
    uint64_t coarse_cap = 0;
    double *width_part = nullptr;           // per-block interface sums of a snapshot
    double width_sum[4] = {0, 0, 0, 0};     // phi(1-phi), |grad phi|: filtered coarse, fine
    uint64_t adam_t = 0;
    bool have_params = false;
    std::vector<float> host_blob = std::vector<float>(kMlpBlob, 0.0f);

    ~pflbm_closure() {
        cudaSetDevice(device);
        void *ptrs[] = {X, Y, blob, m, v, gpart, grad, partial, loss_log, coarse, width_part};
        for (void *p : ptrs)
            if (p) cudaFree(p);
        if (stream) cudaStreamDestroy(stream);
    }
};

namespace {

int ensure_gpart(pflbm_closure *c, int blocks) {
    if (blocks <= c->gpart_blocks) return PFLBM_OK;
    if (c->gpart) cudaFree(c->gpart);
    c->gpart = nullptr;
    c->gpart_blocks = 0;
    cudaError_t e = cudaMalloc(&c->gpart, sizeof(float) * size_t(blocks) * (kMlpParams + 1));
    if (e != cudaSuccess) return cuda_fail(e, "cudaMalloc (gradient partials)");
    c->gpart_blocks = blocks;
    return PFLBM_OK;
}

int upload_blob(pflbm_closure *c) {
    cudaError_t e = cudaMemcpyAsync(c->blob, c->host_blob.data(), sizeof(float) * kMlpBlob, cudaMemcpyHostToDevice,
                                    c->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    return e == cudaSuccess ? PFLBM_OK : cuda_fail(e, "closure blob upload");
}

int download_blob(pflbm_closure *c) {
    cudaError_t e = cudaMemcpyAsync(c->host_blob.data(), c->blob, sizeof(float) * kMlpBlob, cudaMemcpyDeviceToHost,
                                    c->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    return e == cudaSuccess ? PFLBM_OK : cuda_fail(e, "closure blob download");
}

size_t act_bytes() { return sizeof(Act); }

// Gradient kernel of a training step: the tensor-core kernel, or with
// PFLBM_MLP_SIMT=1 the FP32 CUDA-core kernel (exact FP32 products, for
// checks against the FP64 oracle at FP32 rounding).
bool use_simt_grad() {
    const char *e = std::getenv("PFLBM_MLP_SIMT");
    return e && e[0] == '1';
}

void launch_grad(pflbm_closure *c, int blocks, int mode, uint64_t seed, uint64_t iter, uint64_t count) {
    if (use_simt_grad())
        k_mlp_grad<<<blocks, kSB, act_bytes(), c->stream>>>(c->blob, c->X, c->Y, c->n, mode, seed, iter, count,
                                                            c->gpart);
    else
        k_mlp_grad_tc<<<blocks, kSB, tc_smem_bytes(), c->stream>>>(c->blob, c->X, c->Y, c->n, mode, seed, iter,
                                                                   count, c->gpart);
}

}  // namespace

extern "C" {

int pflbm_closure_create(int32_t device, uint64_t max_samples, pflbm_closure **out) {
    if (!out || max_samples == 0) return fail(PFLBM_ERR_INVALID_ARG, "bad argument");
    *out = nullptr;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
        cudaGetLastError();
        return fail(PFLBM_ERR_CUDA, "no CUDA device");
    }
    if (device < 0 || device >= ndev) return fail(PFLBM_ERR_INVALID_ARG, "device out of range");
    std::unique_ptr<pflbm_closure> c(new (std::nothrow) pflbm_closure());
    if (!c) return fail(PFLBM_ERR_OUT_OF_MEMORY, "closure handle");
    c->device = device;
    cudaSetDevice(device);
    c->cap = max_samples;
    cudaError_t e = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking);
    if (e != cudaSuccess) return cuda_fail(e, "cudaStreamCreate");
    if (cudaMalloc(&c->X, sizeof(float) * kMlpIn * max_samples) != cudaSuccess ||
        cudaMalloc(&c->Y, sizeof(float) * max_samples) != cudaSuccess ||
        cudaMalloc(&c->blob, sizeof(float) * kMlpBlob) != cudaSuccess ||
        cudaMalloc(&c->m, sizeof(float) * kMlpParams) != cudaSuccess ||
        cudaMalloc(&c->v, sizeof(float) * kMlpParams) != cudaSuccess ||
        cudaMalloc(&c->grad, sizeof(double) * (kMlpParams + 1)) != cudaSuccess ||
        cudaMalloc(&c->partial, sizeof(double) * kLossBlocks * 18) != cudaSuccess ||
        cudaMalloc(&c->width_part, sizeof(double) * kMakeBlocks * 4) != cudaSuccess) {
        cudaGetLastError();
        return fail(PFLBM_ERR_OUT_OF_MEMORY, "closure buffers");
    }
    if (cudaFuncSetAttribute(k_mlp_grad, cudaFuncAttributeMaxDynamicSharedMemorySize, int(act_bytes())) != cudaSuccess)
        return cuda_fail(cudaGetLastError(), "k_mlp_grad shared memory");
    if (cudaFuncSetAttribute(k_mlp_grad_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, int(tc_smem_bytes())) !=
        cudaSuccess)
        return cuda_fail(cudaGetLastError(), "k_mlp_grad_tc shared memory");
    *out = c.release();
    return PFLBM_OK;
}

int pflbm_closure_destroy(pflbm_closure *c) {
    delete c;
    return PFLBM_OK;
}

int pflbm_closure_num_samples(const pflbm_closure *c, uint64_t *n) {
    if (!c || !n) return fail(PFLBM_ERR_INVALID_ARG, "null argument");
    *n = c->n;
    return PFLBM_OK;
}

int pflbm_closure_add_snapshot(pflbm_closure *c, pflbm_sim *fine, int32_t stride, uint64_t *added) {
    if (!c || !fine || stride < 1) return fail(PFLBM_ERR_INVALID_ARG, "bad argument");
    pflbm::SimView v{};
    if (int rc = pflbm::sim_view(fine, v)) return rc;
    if (v.real_bytes != 4) return fail(PFLBM_ERR_UNSUPPORTED, "training snapshots need an FP32 or 16-bit storage run");
    if (v.device != c->device) return fail(PFLBM_ERR_INVALID_ARG, "simulation and closure are on different devices");
    if (v.nx % 2 || v.ny % 2 || v.nz % 2 || v.nx < 16 || v.ny < 16 || v.nz < 16)
        return fail(PFLBM_ERR_INVALID_ARG, "fine grid extents must be even and >= 16");
    cudaSetDevice(c->device);
    const int nxc = int(v.nx / 2), nyc = int(v.ny / 2), nzc = int(v.nz / 2);
    const uint64_t Nc = uint64_t(nxc) * nyc * nzc;
    if (c->coarse_cap < Nc) {
        if (c->coarse) cudaFree(c->coarse);
        c->coarse = nullptr;
        c->coarse_cap = 0;
        if (cudaMalloc(&c->coarse, sizeof(float) * kCoarseFields * Nc) != cudaSuccess) {
            cudaGetLastError();
            return fail(PFLBM_ERR_OUT_OF_MEMORY, "closure coarse scratch");
        }
        c->coarse_cap = Nc;
    }
    // sample lattice: i = i0, i0 + stride, ... within [2, nxc-3]
    const int i0 = ((2 + stride - 1) / stride) * stride, j0 = i0;
    const int ni = i0 > nxc - 3 ? 0 : (nxc - 3 - i0) / stride + 1;
    const int nj = j0 > nyc - 3 ? 0 : (nyc - 3 - j0) / stride + 1;
    const uint64_t count = uint64_t(ni) * nj * uint64_t(nzc - 4);
    if (c->n + count > c->cap)
        return fail(PFLBM_ERR_INVALID_ARG, "closure sample capacity exceeded (" + std::to_string(c->n + count) + " > " +
                                               std::to_string(c->cap) + ")");
    // the fine run's analysis ran on its own stream, which sim_view synchronised
    k_filter_restrict<<<1216, 256, 0, c->stream>>>(static_cast<const float *>(v.macro), v.N, int(v.nx), int(v.ny),
                                                   int(v.nz), nxc, nyc, nzc, c->coarse);
    k_make_samples<<<kMakeBlocks, kMakeThreads, 0, c->stream>>>(
        c->coarse, nxc, nyc, nzc, stride, float(v.tau_water), float(v.tau_oil), i0, ni, j0, nj, c->X, c->Y, c->n,
        static_cast<const float *>(v.macro), v.N, int(v.nx), int(v.ny), c->width_part);
    std::vector<double> wp(size_t(kMakeBlocks) * 4);
    cudaError_t e = cudaMemcpyAsync(wp.data(), c->width_part, sizeof(double) * wp.size(), cudaMemcpyDeviceToHost,
                                    c->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    if (e != cudaSuccess) return cuda_fail(e, "closure snapshot");
    for (int b = 0; b < kMakeBlocks; ++b)
        for (int q = 0; q < 4; ++q) c->width_sum[q] += wp[size_t(b) * 4 + q];
    c->n += count;
    if (added) *added = count;
    return PFLBM_OK;
}

int pflbm_closure_interface_scale(const pflbm_closure *c, double *gamma_scale, double *width_fine,
                                   double *width_filtered) {
    if (!c || !gamma_scale) return fail(PFLBM_ERR_INVALID_ARG, "null argument");
    const double *w = c->width_sum;
    if (!(w[0] > 0.0 && w[1] > 0.0 && w[2] > 0.0 && w[3] > 0.0))
        return fail(PFLBM_ERR_STATE, "no interface in the snapshots added so far");
    const double wc = 4.0 * w[0] / w[1], wf = 4.0 * w[2] / w[3];
    *gamma_scale = wf / wc;
    if (width_fine) *width_fine = wf;
    if (width_filtered) *width_filtered = wc;
    return PFLBM_OK;
}

int pflbm_closure_get_samples(pflbm_closure *c, uint64_t first, uint64_t count, float *host_x, float *host_y) {
    if (!c || (!host_x && !host_y) || first + count > c->n) return fail(PFLBM_ERR_INVALID_ARG, "bad sample range");
    cudaSetDevice(c->device);
    cudaError_t e = cudaSuccess;
    if (host_x)
        e = cudaMemcpy(host_x, c->X + first * kMlpIn, sizeof(float) * kMlpIn * count, cudaMemcpyDeviceToHost);
    if (e == cudaSuccess && host_y) e = cudaMemcpy(host_y, c->Y + first, sizeof(float) * count, cudaMemcpyDeviceToHost);
    return e == cudaSuccess ? PFLBM_OK : cuda_fail(e, "sample readback");
}

int pflbm_closure_set_samples(pflbm_closure *c, const float *host_x, const float *host_y, uint64_t count) {
    if (!c || !host_x || !host_y || count > c->cap) return fail(PFLBM_ERR_INVALID_ARG, "bad argument");
    cudaSetDevice(c->device);
    cudaError_t e = cudaMemcpy(c->X, host_x, sizeof(float) * kMlpIn * count, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(c->Y, host_y, sizeof(float) * count, cudaMemcpyHostToDevice);
    if (e != cudaSuccess) return cuda_fail(e, "sample upload");
    c->n = count;
    return PFLBM_OK;
}

int pflbm_closure_init_params(pflbm_closure *c, uint32_t seed) {
    if (!c) return fail(PFLBM_ERR_INVALID_ARG, "null closure");
    if (c->n == 0) return fail(PFLBM_ERR_STATE, "no training samples");
    cudaSetDevice(c->device);
    const int blocks = 304;
    k_stats<<<blocks, 256, 0, c->stream>>>(c->X, c->Y, c->n, c->partial);
    std::vector<double> part(size_t(blocks) * 18);
    cudaError_t e = cudaMemcpyAsync(part.data(), c->partial, sizeof(double) * part.size(), cudaMemcpyDeviceToHost,
                                    c->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    if (e != cudaSuccess) return cuda_fail(e, "closure statistics");
    double tot[18] = {0};
    for (int b = 0; b < blocks; ++b)
        for (int f = 0; f < 18; ++f) tot[f] += part[size_t(b) * 18 + f];
    const double n = double(c->n);
    std::vector<float> &w = c->host_blob;
    std::fill(w.begin(), w.end(), 0.0f);
    for (int k = 0; k < kMlpIn; ++k) {
        const double mean = tot[k] / n;
        const double var = std::max(tot[8 + k] / n - mean * mean, 0.0);
        w[pflbm::kMlpMean + k] = float(mean);
        w[pflbm::kMlpInvScale + k] = var > 1e-30 ? float(1.0 / std::sqrt(var)) : 1.0f;
    }
    const double ymean = tot[16] / n, yrms = std::sqrt(std::max(tot[17] / n, 0.0));
    const double out_scale = yrms > 1e-30 ? yrms : 1.0;
    w[pflbm::kMlpOutScale] = float(out_scale);
    w[pflbm::kMlpStrength] = 1.0f;
    // Glorot-uniform weights from a counter hash, zero biases; b3 puts the
    // initial output at the mean target
    auto uni = [&](uint64_t k) { return double(mix64(uint64_t(seed) * 0x9E3779B97F4A7C15ull + k) >> 11) * 0x1.0p-53; };
    const double l1 = std::sqrt(6.0 / (kMlpIn + kMlpH)), l2 = std::sqrt(6.0 / (2 * kMlpH)),
                 l3 = std::sqrt(6.0 / (kMlpH + 1));
    for (int p = 0; p < kMlpH * kMlpIn; ++p) w[pflbm::kMlpW1 + p] = float(l1 * (2.0 * uni(p) - 1.0));
    for (int p = 0; p < kMlpH * kMlpH; ++p) w[pflbm::kMlpW2 + p] = float(l2 * (2.0 * uni(10000 + p) - 1.0));
    for (int p = 0; p < kMlpH; ++p) w[pflbm::kMlpW3 + p] = float(l3 * (2.0 * uni(20000 + p) - 1.0));
    const double t0 = std::max(ymean / out_scale, 1e-3);
    w[pflbm::kMlpB3] = float(t0 > 20.0 ? t0 : std::log(std::expm1(t0)));
    if (int rc = upload_blob(c)) return rc;
    cudaMemsetAsync(c->m, 0, sizeof(float) * kMlpParams, c->stream);
    cudaMemsetAsync(c->v, 0, sizeof(float) * kMlpParams, c->stream);
    e = cudaStreamSynchronize(c->stream);
    if (e != cudaSuccess) return cuda_fail(e, "closure init");
    c->adam_t = 0;
    c->have_params = true;
    return PFLBM_OK;
}

int pflbm_closure_get_blob(pflbm_closure *c, float *host_blob) {
    if (!c || !host_blob) return fail(PFLBM_ERR_INVALID_ARG, "null argument");
    cudaSetDevice(c->device);
    if (int rc = download_blob(c)) return rc;
    std::memcpy(host_blob, c->host_blob.data(), sizeof(float) * kMlpBlob);
    return PFLBM_OK;
}

int pflbm_closure_set_blob(pflbm_closure *c, const float *host_blob) {
    if (!c || !host_blob) return fail(PFLBM_ERR_INVALID_ARG, "null argument");
    cudaSetDevice(c->device);
    std::memcpy(c->host_blob.data(), host_blob, sizeof(float) * kMlpBlob);
    if (int rc = upload_blob(c)) return rc;
    cudaMemsetAsync(c->m, 0, sizeof(float) * kMlpParams, c->stream);
    cudaMemsetAsync(c->v, 0, sizeof(float) * kMlpParams, c->stream);
    cudaError_t e = cudaStreamSynchronize(c->stream);
    if (e != cudaSuccess) return cuda_fail(e, "closure set blob");
    c->adam_t = 0;
    c->have_params = true;
    return PFLBM_OK;
}

int pflbm_closure_gradient(pflbm_closure *c, uint64_t count, double *host_grad, double *loss_sum) {
    if (!c || !host_grad || count == 0 || count > c->n) return fail(PFLBM_ERR_INVALID_ARG, "bad argument");
    if (!c->have_params) return fail(PFLBM_ERR_STATE, "closure parameters not initialised");
    cudaSetDevice(c->device);
    const int blocks = int((count + kSB - 1) / kSB);
    if (int rc = ensure_gpart(c, blocks)) return rc;
    launch_grad(c, blocks, 0, 0, 0, count);
    k_grad_sum<<<(kMlpParams + 1 + 255) / 256, 256, 0, c->stream>>>(c->gpart, blocks, c->grad);
    std::vector<double> g(kMlpParams + 1);
    cudaError_t e = cudaMemcpyAsync(g.data(), c->grad, sizeof(double) * g.size(), cudaMemcpyDeviceToHost, c->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    if (e != cudaSuccess) return cuda_fail(e, "closure gradient");
    std::memcpy(host_grad, g.data(), sizeof(double) * kMlpParams);
    if (loss_sum) *loss_sum = g[kMlpParams];
    return PFLBM_OK;
}

int pflbm_closure_train(pflbm_closure *c, int32_t iterations, int32_t batch, float lr, uint32_t seed,
                        double *loss_history) {
    if (!c || iterations < 1 || batch < 1) return fail(PFLBM_ERR_INVALID_ARG, "bad argument");
    if (!c->have_params) return fail(PFLBM_ERR_STATE, "closure parameters not initialised");
    if (c->n == 0) return fail(PFLBM_ERR_STATE, "no training samples");
    cudaSetDevice(c->device);
    const int blocks = (batch + kSB - 1) / kSB;
    if (int rc = ensure_gpart(c, blocks)) return rc;
    if (c->loss_log_cap < iterations) {
        if (c->loss_log) cudaFree(c->loss_log);
        c->loss_log = nullptr;
        c->loss_log_cap = 0;
        if (cudaMalloc(&c->loss_log, sizeof(double) * iterations) != cudaSuccess) {
            cudaGetLastError();
            return fail(PFLBM_ERR_OUT_OF_MEMORY, "loss log");
        }
        c->loss_log_cap = iterations;
    }
    const float beta1 = 0.9f, beta2 = 0.999f, eps = 1e-8f;
    for (int it = 0; it < iterations; ++it) {
        const uint64_t t = ++c->adam_t;
        const float c1 = float(1.0 - std::pow(double(beta1), double(t)));
        const float c2 = float(1.0 - std::pow(double(beta2), double(t)));
        launch_grad(c, blocks, 1, seed, t, uint64_t(batch));
        k_adam<<<(kMlpParams + 1 + 255) / 256, 256, 0, c->stream>>>(c->blob, c->m, c->v, c->gpart, blocks,
                                                                   1.0f / float(batch), lr, beta1, beta2, eps, c1, c2,
                                                                   c->loss_log, it);
    }
    cudaError_t e = cudaStreamSynchronize(c->stream);
    if (e != cudaSuccess) return cuda_fail(e, "closure training");
    if (loss_history) {
        e = cudaMemcpy(loss_history, c->loss_log, sizeof(double) * iterations, cudaMemcpyDeviceToHost);
        if (e != cudaSuccess) return cuda_fail(e, "loss history");
    }
    return download_blob(c);
}

int pflbm_closure_loss(pflbm_closure *c, double *mean_loss) {
    if (!c || !mean_loss) return fail(PFLBM_ERR_INVALID_ARG, "null argument");
    if (!c->have_params || c->n == 0) return fail(PFLBM_ERR_STATE, "no parameters or samples");
    cudaSetDevice(c->device);
    k_mlp_loss<<<kLossBlocks, 256, 0, c->stream>>>(c->blob, c->X, c->Y, c->n, c->partial);
    std::vector<double> part(kLossBlocks);
    cudaError_t e = cudaMemcpyAsync(part.data(), c->partial, sizeof(double) * kLossBlocks, cudaMemcpyDeviceToHost,
                                    c->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    if (e != cudaSuccess) return cuda_fail(e, "closure loss");
    double s = 0.0;
    for (double p : part) s += p;
    *mean_loss = s / double(c->n);
    return PFLBM_OK;
}

}  // extern "C"
