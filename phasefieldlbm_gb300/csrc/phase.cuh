// phase.cuh - the phase step (phi^{n+1} = sum of the pulled D3Q7 populations)
// with the jet boundary rebuilds: scalar and float4 kernels.
#pragma once
#include <cuda_runtime.h>

#include <cstdint>

#include "boundary.cuh"
#include "lattice.cuh"
#include "params.cuh"

namespace pflbm {

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
    if (PFLBM_GUARD(X < N, b.err)) b.phi_dst[X] = s;

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
                        if (PFLBM_GUARD(static_cast<uint64_t>(gx) + static_cast<uint64_t>(nx) * gy < plane, b.err))
                        Store<S>::store(b.f_dst, q * N + static_cast<uint64_t>(gx) + static_cast<uint64_t>(nx) * gy, v,
                                        static_cast<T>(1.0 / weight<QQ>(q)));
                    }
                }
            }
        }
        if (z == nz - 2) {
            // ghost phi of the outlet plane takes this step's value
            // (BoundaryConditions.cuh:127)
            if (PFLBM_GUARD(idx(x, y, nz - 1) < N, b.err)) b.phi_dst[idx(x, y, nz - 1)] = phiX;
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
                    if (PFLBM_GUARD(dst < uint64_t(QQ) * N, b.err))
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
    // the ghost columns keep their phi (both ping-pong buffers hold the same
    // initial ghost values): the source's value is stored again with the
    // row's end segments, so that every row is written by whole 16-byte
    // stores and no 32-byte sector of it is left partly written, which the
    // memory system completes with a read of the old sector (0.045 -> 0.043
    // ms on the 128x128x512 jet)
    if (!PFLBM_GUARD(r0 + x4 + 3 < N, b.err)) return;
    if (x4 == 0) out[0] = pc.x;
    if (x4 + 3 == nx - 1) out[3] = pc.w;
    *reinterpret_cast<float4 *>(b.phi_dst + r0 + x4) = make_float4(out[0], out[1], out[2], out[3]);
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

}  // namespace pflbm
