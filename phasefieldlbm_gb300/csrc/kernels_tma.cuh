// kernels_tma.cuh - the collide kernel with TMA-fed, double-buffered plane
// staging (sm_103a).
//
// Same computation as k_collide (kernels.cuh), same 32x8 column tile marching
// a chunk of z planes, but the populations of a plane are brought into
// shared memory by the Tensor Memory Accelerator one plane ahead of use:
//   * f: one 4D tensor map (x, y, z, q). For plane z and direction q the CTA
//     needs the source tile shifted by -c_q; it loads one box per direction,
//     (32 + 2*XO) x 8 wide, whose x origin x0 - XO is 16-byte aligned, at
//     y0 - cy_q and z - cz_q; the thread reads element tx + XO - cx_q.
//   * phi: one 3D tensor map, box 40 x 12 (tile + halo 2) at (x0-4, y0-2),
//     two planes ahead of the plane being collided, into a 4-slot ring.
// Both arrive on one mbarrier per stage (expect_tx), issued by thread 0 right
// after the block barrier that ends the use of the stage's previous plane.
// Out-of-range boxes are zero-filled by the TMA unit; those elements only
// feed ghost nodes, which are never updated. One __syncthreads per plane.
//
// Every mbarrier wait is bounded; on a timeout the CTA records an error in
// the device error word, drains its own copies (bounded) and returns as a
// whole, so a failure never hangs the GPU.
#pragma once
#include "kernels.cuh"
#include "tma.cuh"

namespace pflbm {

constexpr uint32_t kWaitLimit = 1u << 22;

__host__ __device__ constexpr size_t align128(size_t v) { return (v + 127) & ~size_t(127); }

template <int QQ, class S>
struct TmaLayout {
    using T = typename Store<S>::T;
    static constexpr int XO = sizeof(S) == 2 ? 8 : 4;  // x origin offset: 16-byte aligned coordinate
    static constexpr int BW = TX + 2 * XO;             // f box width
    static constexpr int PXO = 4;                      // phi is FP32 or FP64
    static constexpr int PBW = TX + 2 * PXO;           // 40
    static constexpr int PBH = TY + 4;                 // 12
    // bytes the TMA unit writes per box / phi plane
    static constexpr size_t box_bytes = size_t(TY) * BW * sizeof(S);
    static constexpr size_t phi_plane_bytes = size_t(PBH) * PBW * sizeof(T);
    // shared-memory strides: every TMA destination starts on a 128-byte boundary
    static constexpr size_t box_stride = align128(box_bytes);
    static constexpr size_t stage_bytes = size_t(QQ) * box_stride;
    static constexpr size_t phi_slot_bytes = align128(phi_plane_bytes);
    static constexpr size_t off_f = 0;
    static constexpr size_t off_phi = align128(2 * stage_bytes);
    static constexpr size_t off_n = align128(off_phi + 4 * phi_slot_bytes);
    static constexpr size_t n_bytes = size_t(4) * 4 * NY_ * NX_ * sizeof(T);
    static constexpr size_t off_bar = align128(off_n + n_bytes);
    static constexpr size_t total = off_bar + 128;
    static constexpr uint32_t tx_bytes = uint32_t(QQ * box_bytes + phi_plane_bytes);
    static_assert(box_stride % 128 == 0 && phi_slot_bytes % 128 == 0 && off_phi % 128 == 0, "TMA smem alignment");
    static_assert((BW * sizeof(S)) % 16 == 0 && (PBW * sizeof(T)) % 16 == 0, "TMA inner box extent");
    static_assert(BW <= 256 && PBW <= 256 && TY <= 256 && PBH <= 256, "TMA box dimension limit");
};

template <int QQ, bool JET, class S, int MODE>
__global__ void __launch_bounds__(NT, (sizeof(typename Store<S>::T) == 8 ? 1 : PFLBM_COLLIDE_MIN_BLOCKS))
    k_collide_tma(const Params<typename Store<S>::T> p, const StepBuffers<S, typename Store<S>::T> b,
                  const __grid_constant__ CUtensorMap fmap, const __grid_constant__ CUtensorMap phimap) {
    using T = typename Store<S>::T;
    using L = TmaLayout<QQ, S>;
    extern __shared__ __align__(128) unsigned char smem[];
    S *s_f = reinterpret_cast<S *>(smem + L::off_f);
    T *s_phi = reinterpret_cast<T *>(smem + L::off_phi);
    T *s_n = reinterpret_cast<T *>(smem + L::off_n);
    uint64_t *bar = reinterpret_cast<uint64_t *>(smem + L::off_bar);
    volatile int *s_abort = reinterpret_cast<volatile int *>(smem + L::off_bar + 64);

    const int nx = p.nx, ny = p.ny, nz = p.nz;
    const int tx = threadIdx.x, ty = threadIdx.y, tid = tx + TX * ty;
    const int x0 = blockIdx.x * TX, y0 = blockIdx.y * TY;
    const int x = x0 + tx, y = y0 + ty;
    const int zb = 1 + blockIdx.z * p.zchunk;
    const int ze = min(zb + p.zchunk, nz - 1);
    const bool col = (x >= 1 && x <= nx - 2 && y >= 1 && y <= ny - 2);
    const uint32_t t = b.step_in ? static_cast<uint32_t>(*b.step_in) : b.t_fixed;

    auto phi_at = [&](int slot, int ly, int lx) -> T & {
        return *reinterpret_cast<T *>(reinterpret_cast<unsigned char *>(s_phi) + slot * L::phi_slot_bytes +
                                      (size_t(ly) * L::PBW + lx) * sizeof(T));
    };
    auto n_at = [&](int c, int slot, int ly, int lx) -> T & { return s_n[((c * 4 + slot) * NY_ + ly) * NX_ + lx]; };
    auto issue = [&](int stage, int zf) {
        // generic-proxy accesses to the recycled slots are ordered before the
        // async-proxy writes by the preceding block barrier and this fence
        fence_proxy_async();
        mbar_arrive_expect_tx(&bar[stage], L::tx_bytes);
        unsigned char *dst = reinterpret_cast<unsigned char *>(s_f) + size_t(stage) * L::stage_bytes;
#pragma unroll
        for (int q = 0; q < QQ; ++q)
            tma_load_4d(dst + size_t(q) * L::box_stride, &fmap, &bar[stage], x0 - L::XO, y0 - kCY[q], zf - kCZ[q], q);
        tma_load_3d(&phi_at((zf + 2) & 3, 0, 0), &phimap, &bar[stage], x0 - L::PXO, y0 - 2, zf + 2);
    };

    if (tid == 0) {
        tma_prefetch_desc(&fmap);
        tma_prefetch_desc(&phimap);
        mbar_init(&bar[0], 1);
        mbar_init(&bar[1], 1);
        *s_abort = 0;
        fence_mbar_init();
    }
    __syncthreads();

    // warm-up: phi planes zb-2 .. zb+1 with plain loads, normals of zb-1, zb
    for (int zp = zb - 2; zp <= zb + 1; ++zp) {
        const int slot = (zp + 4) & 3;
        for (int i = tid; i < L::PBW * L::PBH; i += NT) {
            const int lx = i % L::PBW, ly = i / L::PBW;
            const int gx = x0 - L::PXO + lx, gy = y0 - 2 + ly;
            T v = T(0);
            if (gx >= 0 && gx < nx && gy >= 0 && gy < ny && zp >= 0 && zp < nz)
                v = b.phi_src[gx + static_cast<uint64_t>(nx) * (gy + static_cast<uint64_t>(ny) * zp)];
            phi_at(slot, ly, lx) = v;
        }
    }
    auto compute_n = [&](int zp) {
        const int sn = (zp + 4) & 3, sm = (zp + 3) & 3, sp = (zp + 5) & 3;
        for (int i = tid; i < NX_ * NY_; i += NT) {
            const int lx = i % NX_, ly = i / NX_;
            const int gx = x0 - 1 + lx, gy = y0 - 1 + ly;
            T nxv = T(0), nyv = T(0), nzv = T(0), ind = T(0);
            if (gx >= 1 && gx <= nx - 2 && gy >= 1 && gy <= ny - 2 && zp >= 1 && zp <= nz - 2) {
                auto v = [&](int dx, int dy, int dz) -> T {
                    return phi_at(dz < 0 ? sm : (dz > 0 ? sp : sn), ly + 1 + dy, lx + L::PXO - 1 + dx);
                };
                const T gxv = T(3) * lattice_grad<QQ, T>(v, kCX);
                const T gyv = T(3) * lattice_grad<QQ, T>(v, kCY);
                const T gzv = T(3) * lattice_grad<QQ, T>(v, kCZ);
                ind = sqrt(gxv * gxv + gyv * gyv + gzv * gzv);
                const T inv = T(1) / (ind + static_cast<T>(1e-9));
                nxv = gxv * inv;
                nyv = gyv * inv;
                nzv = gzv * inv;
            }
            n_at(0, sn, ly, lx) = nxv;
            n_at(1, sn, ly, lx) = nyv;
            n_at(2, sn, ly, lx) = nzv;
            n_at(3, sn, ly, lx) = ind;
        }
    };
    __syncthreads();
    compute_n(zb - 1);
    __syncthreads();
    // stage 0 (plane zb, phi zb+2) reuses the ring slot of phi zb-2, free now
    if (tid == 0) issue(0, zb);
    compute_n(zb);

    for (int z = zb, it = 0; z < ze; ++z, ++it) {
        const int st = it & 1;
        const uint32_t par = (it >> 1) & 1;
        if (!mbar_wait_bounded(&bar[st], par, kWaitLimit)) *s_abort = 1;
        compute_n(z + 1);
        __syncthreads();
        if (*s_abort) {
            if (tid == 0) {
                atomicOr(b.err, 1u);
                mbar_wait_bounded(&bar[st], par, kWaitLimit);  // drain this CTA's own copies
            }
            return;
        }
        if (tid == 0 && z + 1 < ze) issue(st ^ 1, z + 1);
        if (!col) continue;

        const int s_m = (z + 3) & 3, s_0 = z & 3, s_p = (z + 1) & 3;
        auto nv = [&](int c, int dx, int dy, int dz) -> T {
            return n_at(c, dz < 0 ? s_m : (dz > 0 ? s_p : s_0), ty + 1 + dy, tx + 1 + dx);
        };
        const T scx = lattice_grad<QQ, T>([&](int dx, int dy, int dz) { return nv(0, dx, dy, dz); }, kCX);
        const T scy = lattice_grad<QQ, T>([&](int dx, int dy, int dz) { return nv(1, dx, dy, dz); }, kCY);
        const T scz = lattice_grad<QQ, T>([&](int dx, int dy, int dz) { return nv(2, dx, dy, dz); }, kCZ);
        const T curvature = T(3) * (scx + scy + scz);
        const T n_x = nv(0, 0, 0, 0), n_y = nv(1, 0, 0, 0), n_z = nv(2, 0, 0, 0), ind = nv(3, 0, 0, 0);
        const T phi = phi_at(z & 3, ty + 2, tx + L::PXO);

        T pop[QQ];
        const unsigned char *sf = reinterpret_cast<const unsigned char *>(s_f) + size_t(st) * L::stage_bytes +
                                  (size_t(ty) * L::BW + tx + L::XO) * sizeof(S);
#pragma unroll
        for (int q = 0; q < QQ; ++q)
            pop[q] = Store<S>::widen(*reinterpret_cast<const S *>(sf + size_t(q) * L::box_stride - kCX[q] * int(sizeof(S))),
                                     static_cast<T>(weight<QQ>(q)));
        collide_node<QQ, JET, S, MODE>(p, b, x, y, z, t, pop, phi, n_x, n_y, n_z, ind, curvature);
    }
}

}  // namespace pflbm
