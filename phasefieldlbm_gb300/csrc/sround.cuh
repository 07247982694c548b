// sround.cuh - stochastic rounding of the BF16 population stores.
//
// BF16 keeps 8 significant bits. Rounded to nearest, the scaled populations
// of a smooth flow round the same way over whole regions, and the rounding
// bias adds up coherently from step to step (the BF16 velocity error grows
// about linearly in time). Stochastic rounding rounds the magnitude up with
// probability equal to the discarded fraction, so each store is unbiased and
// the errors of neighbouring nodes and successive steps do not add up
// coherently. The random bits are a counter hash of (node pair, direction,
// step): the results are deterministic and every collide variant draws the
// same bits for the same store.
#pragma once
#include <cuda_runtime.h>

#include <cstdint>

#include "boundary.cuh"

namespace pflbm {

// 32 random bits for the stores of node pair (2 k, 2 k + 1) at step t; one
// hash per pair and step.
__device__ __forceinline__ uint32_t sr_pair_seed(uint32_t pair, uint32_t t) {
    return hash32(pair * 0x9E3779B1u ^ t * 0x85EBCA77u ^ 0xC2B2AE3Du);
}

// A fixed, well-mixed 32-bit constant per direction (a compile-time
// immediate for a compile-time q).
__host__ __device__ constexpr uint32_t sr_dir_const(int q) {
    uint32_t x = uint32_t(q + 1) * 0x9E3779B9u;
    x ^= x >> 16;
    x *= 0x7FEB352Du;
    x ^= x >> 15;
    x *= 0x846CA68Bu;
    x ^= x >> 16;
    return x;
}

// 32 random bits for direction q of the pair: the low 16 bits for the even
// node, the high 16 bits for the odd one. The directions of a pair share the
// pair's hash, each XORed with its own constant: every direction's bits are
// uniform (an unbiased rounding) at one instruction per direction.
__device__ __forceinline__ uint32_t sr_dir_bits(uint32_t seed, int q) { return seed ^ sr_dir_const(q); }

// v rounded to BF16 with 16 random bits r: the discarded low half of v's
// bits plus r carries into the kept half with probability (low half) / 2^16.
// Sign-magnitude, so the magnitude is rounded without bias for either sign.
__device__ __forceinline__ uint16_t bf16_bits_sr(float v, uint32_t r16) {
    return static_cast<uint16_t>((__float_as_uint(v) + r16) >> 16);
}

// Two values rounded stochastically and packed as a __nv_bfloat162 word
// (a in the low half), with the two 16-bit halves of r.
__device__ __forceinline__ uint32_t bf16x2_bits_sr(float a, float b, uint32_t r) {
    const uint32_t ba = __float_as_uint(a) + (r & 0xFFFFu);
    const uint32_t bb = __float_as_uint(b) + (r >> 16);
    return __byte_perm(ba, bb, 0x7632);
}

}  // namespace pflbm
