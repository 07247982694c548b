// reduce.cuh - block reduction of the FP64 diagnostics rows (phi mass, rho
// mass, momentum, max |u|, inside/outside rho and counts, non-finite count)
// with warp shuffles.
#pragma once
#include <cuda_runtime.h>

namespace pflbm {

constexpr int RED_FIELDS = 12;  // phi, rho, rho ux, rho uy, rho uz, max|u|, rho_in, n_in, rho_out, n_out, nonfinite, spare
constexpr int RED_MAX_SLOT = 5; // max |u| (combined by max; every other slot by sum)

__device__ __forceinline__ double red_combine(int f, double a, double b) {
    return f == RED_MAX_SLOT ? fmax(a, b) : a + b;
}

// Reduces each thread's `acc` over the block (NTHREADS, a multiple of 32):
// a shuffle tree inside every warp, then the warps' results, in warp order,
// by a shuffle tree in the first warp. Thread 0 writes the row to `out`.
// Every value is >= 0 in the max slot, so 0 is the identity of both
// operations. Deterministic: the order of combination is fixed.
template <int NTHREADS>
__device__ __forceinline__ void block_reduce_row(double (&acc)[RED_FIELDS], double *out) {
    static_assert(NTHREADS % 32 == 0 && NTHREADS <= 1024, "block size");
    constexpr int NW = NTHREADS / 32;
    __shared__ double s_warp[NW][RED_FIELDS];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int f = 0; f < RED_FIELDS; ++f) {
        double v = acc[f];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v = red_combine(f, v, __shfl_down_sync(0xffffffffu, v, o));
        if (lane == 0) s_warp[warp][f] = v;
    }
    __syncthreads();
    if (warp == 0) {
#pragma unroll
        for (int f = 0; f < RED_FIELDS; ++f) {
            double v = lane < NW ? s_warp[lane][f] : 0.0;
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) v = red_combine(f, v, __shfl_down_sync(0xffffffffu, v, o));
            if (lane == 0) out[f] = v;
        }
    }
}

}  // namespace pflbm
