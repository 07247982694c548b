// params.cuh - device-side parameters and storage traits.
#pragma once
#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <cstdint>

namespace pflbm {

// Run-time constants of one simulation. Every value is derived on the host
// from pflbm_config the way the reference derives its constexpr values
// (src/constants.cuh:80-141, src/functions/globalFunctions.cuh:260-461).
template <class T>
struct Params {
    uint32_t nx, ny, nz;
    uint32_t plane;  // nx*ny
    uint64_t N;      // nx*ny*nz
    int32_t zchunk;  // interior planes per CTA of the collide kernel
    T sigma, gamma, u_inf;
    T omega_ref;  // droplet (globalFunctions.cuh:426-429)
    // jet relaxation and sponge (globalFunctions.cuh:297-397, 260-292)
    T tau_water, tau_oil, visc_water, visc_oil, kgain1, omco_zmin;
    T z_start, inv_nz_m1, inv_sponge;
    T center_x, center_y, R2;  // inlet disc
    T g5_in;                   // inflow phase population (BoundaryConditions.cuh:104)
    float sigma_u;             // Gaussian inflow noise s.d. (BoundaryConditions.cuh:58)
    float noise_amp;           // uniform inflow noise amplitude
    int32_t noise_mode;
    uint32_t seed;
    float u_inf_f;
};

// Storage of the shifted populations f' = f - w (the reference's f_eq is
// already shifted, D3Q19.cuh:149). FP32/FP64 store f' as is; FP16/BF16 store
// f'/w_q so that every stored value is O(rho-1, c.u) and stays in the normal
// range of the 16-bit format (per-velocity-set scaling by the weights).
template <class S>
struct Store;

template <>
struct Store<float> {
    using T = float;
    static __device__ __forceinline__ float load(const float *p, uint64_t i, float) { return __ldg(p + i); }
    static __device__ __forceinline__ float widen(float v, float) { return v; }
    static __device__ __forceinline__ void store(float *p, uint64_t i, float v, float) { p[i] = v; }
};
template <>
struct Store<double> {
    using T = double;
    static __device__ __forceinline__ double load(const double *p, uint64_t i, double) { return __ldg(p + i); }
    static __device__ __forceinline__ double widen(double v, double) { return v; }
    static __device__ __forceinline__ void store(double *p, uint64_t i, double v, double) { p[i] = v; }
};
template <>
struct Store<__half> {
    using T = float;
    static __device__ __forceinline__ float load(const __half *p, uint64_t i, float w) {
        return w * __half2float(__ldg(p + i));
    }
    static __device__ __forceinline__ float widen(__half v, float w) { return w * __half2float(v); }
    static __device__ __forceinline__ void store(__half *p, uint64_t i, float v, float inv_w) {
        p[i] = __float2half_rn(v * inv_w);
    }
};
template <>
struct Store<__nv_bfloat16> {
    using T = float;
    static __device__ __forceinline__ float load(const __nv_bfloat16 *p, uint64_t i, float w) {
        return w * __bfloat162float(__ldg(p + i));
    }
    static __device__ __forceinline__ float widen(__nv_bfloat16 v, float w) { return w * __bfloat162float(v); }
    static __device__ __forceinline__ void store(__nv_bfloat16 *p, uint64_t i, float v, float inv_w) {
        p[i] = __float2bfloat16_rn(v * inv_w);
    }
};

// Device pointers used by the step kernels. T is the arithmetic type.
template <class S, class T>
struct StepBuffers {
    const S *f_src;
    S *f_dst;
    const T *phi_src;
    T *phi_dst;
    T *jflux;          // 3*N: phase flux J = 4 phi u + sharp n (see kernels)
    T *top;            // 22*plane: jet moments of planes nz-2 (13) and 1 (9)
    // Step counters, one per ping-pong parity: the step reading buffer A
    // reads counter A and the phase kernel writes counter B = A + 1, so no
    // kernel ever reads a counter that the same step writes.
    const unsigned long long *step_in;
    unsigned long long *step_out;
    uint32_t t_fixed;  // step index used when step_in is null (analysis)
    T *avg;            // 10*N derived averages (or null)
    T *macro;          // 18*N analysis output (or null)
    unsigned int *err; // device error flag
    const float *mlp;  // closure network blob (MODE_STEP_CLOSURE)
};

// Index guard of the step kernels' global stores. Built with
// -DPFLBM_CHECK_BOUNDS (a test build), every guarded store first checks its
// index against the array's extent and, when outside, sets bit 4 of the
// device error word and skips the store; otherwise the guard is `true` and
// costs nothing.
#ifdef PFLBM_CHECK_BOUNDS
#define PFLBM_GUARD(in_range, err) ((in_range) ? true : (atomicOr((err), 4u), false))
#else
#define PFLBM_GUARD(in_range, err) true
#endif

// Order of the macroscopic arrays in the analysis cache; equals
// pflbm_field_id 0..17.
enum MacroSlot { M_RHO = 0, M_UX, M_UY, M_UZ, M_PXX, M_PYY, M_PZZ, M_PXY, M_PXZ, M_PYZ,
                 M_PHI, M_NX, M_NY, M_NZ, M_IND, M_FX, M_FY, M_FZ, M_COUNT };

}  // namespace pflbm
