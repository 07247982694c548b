// fields.cuh - initial conditions, ghost-shell readback, vorticity and the FP64
// diagnostics reductions.
#pragma once
#include <cuda_runtime.h>

#include <cstdint>

#include "boundary.cuh"
#include "lattice.cuh"
#include "params.cuh"
#include "reduce.cuh"
#include "tile.h"

namespace pflbm {

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
    block_reduce_row<RED_THREADS>(acc, partial + size_t(blockIdx.x) * RED_FIELDS);
}

static __global__ void __launch_bounds__(32) k_reduce_final(const double *partial, int nblocks, double *out) {
    const int f = threadIdx.x;
    if (f >= RED_FIELDS) return;
    double s = 0.0;
    for (int b = 0; b < nblocks; ++b) {
        const double v = partial[b * RED_FIELDS + f];
        s = red_combine(f, s, v);
    }
    out[f] = s;
}

}  // namespace pflbm
