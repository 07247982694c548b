// boundary.cuh - inflow noise, inlet disc, periodic index wrap and outflow sponge
// shared by the collide and phase kernels.
#pragma once
#include <cuda_runtime.h>

#include <cstdint>

#include "params.cuh"

namespace pflbm {

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

}  // namespace pflbm
