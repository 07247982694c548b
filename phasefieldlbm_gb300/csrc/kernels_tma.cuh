// kernels_tma.cuh - the collide kernel with TMA-fed, multi-stage plane
// staging (sm_103a).
//
// Same computation as k_collide (kernels.cuh), same 32x8 column tile marching
// a chunk of z planes, but the populations of a plane are brought into
// shared memory by the Tensor Memory Accelerator up to NS-1 planes ahead of
// use (NS = 2..4 stages, as many as keep the CollideOccupancy CTAs resident):
//   * f: two 4D tensor maps (x, y, z, q) that differ in box width. For plane
//     z and direction q the CTA needs the source tile shifted by -c_q; it
//     loads one box per direction at y0 - cy_q and z - cz_q: 32 x 8 at x0
//     when c_x = 0, else (32 + XU) x 8 with XU the 16-byte unit of x, at
//     x0 - XU (c_x = +1) or x0 (c_x = -1); see TmaPlan.
//   * phi: one 3D tensor map, box 40 x 12 (tile + halo 2) at (x0-4, y0-2),
//     two planes ahead of the plane the stage carries, into a ring of NS+2
//     slots.
// Both arrive on one mbarrier per stage (expect_tx), issued by one thread
// (the last warp's first lane when that warp computes no normal-ring
// entries, else thread 0) right after the block barrier that ends the use of
// the stage's previous plane. Out-of-range boxes are zero-filled by the TMA
// unit; those elements only feed ghost nodes, which are never updated. One
// __syncthreads per plane with the 4-plane normal ring, two with the
// 3-plane ring (collide_tile_tma).
//
// Every mbarrier wait is bounded; on a timeout the CTA records an error in
// the device error word, drains its own copies (bounded) and returns as a
// whole, so a failure never hangs the GPU.
#pragma once
#include "kernels.cuh"
#include "packed.cuh"
#include "tma.cuh"

namespace pflbm {

constexpr uint32_t kWaitLimit = 1u << 22;
constexpr int NXP = NX_ / 2;  // x-adjacent entry pairs per row of the normal ring
static_assert(NX_ % 2 == 0, "normal ring pairs");

// Column tile of the TMA collide: TXv x TYv nodes, one thread per node
// (blockDim = (TXv, TYv)). The single-box kernels use the build's tile
// (PFLBM_TILE_X x PFLBM_TILE_Y); the batched ensemble instantiates several
// and lets its autotuner choose.
template <int TXv, int TYv>
struct TileShape {
    static constexpr int TX = TXv, TY = TYv, NT = TXv * TYv;
    static constexpr int NX = TXv + 2, NY = TYv + 2;  // normal ring: tile + halo 1
    static constexpr int NXP = NX / 2;                 // x-adjacent entry pairs per ring row
    static_assert(TXv % 32 == 0 && NT <= 1024 && NX % 2 == 0, "tile shape");
};
using DefaultTile = TileShape<TX, TY>;

// n^ and |grad phi| of the normal-ring entries (lx, ly) and (lx + 1, ly), lx
// even, with packed FP32x2 arithmetic: `e(dx, dy, dz)` points at the phi
// element of the first entry's neighbour (dx, dy, dz). The +-1 x neighbours
// of an even pair are aligned 8-byte words; the dx = 0 column takes two
// loads. A lane whose node is not interior (va / vb false) gets zeros. Same
// rounding as the scalar unit_normal (stencil.cuh).
template <int QQ, bool FAST, class Elem>
__device__ __forceinline__ void normal_pair(const Elem &e, bool va, bool vb, V2 &nxv, V2 &nyv, V2 &nzv, V2 &indv) {
    nxv = nyv = nzv = indv = V2(0.0f);
    if (!(va || vb)) return;
    auto v = [&](int dx, int dy, int dz) -> V2 {
        const float *q = e(dx, dy, dz);
        if (dx == 0) return V2(q[0], q[1]);
        return V2(*reinterpret_cast<const float2 *>(q));
    };
    unit_normal<FAST>(lattice_grad<QQ, 0, V2>(v), lattice_grad<QQ, 1, V2>(v), lattice_grad<QQ, 2, V2>(v), nxv, nyv,
                      nzv, indv);
    if (!(va && vb)) {
        if (!va) {
            nxv.v.x = 0.0f; nyv.v.x = 0.0f; nzv.v.x = 0.0f; indv.v.x = 0.0f;
        }
        if (!vb) {
            nxv.v.y = 0.0f; nyv.v.y = 0.0f; nzv.v.y = 0.0f; indv.v.y = 0.0f;
        }
    }
}

__host__ __device__ constexpr size_t align128(size_t v) { return (v + 127) & ~size_t(127); }

// Shared-memory plan of the TMA collide kernel with NS population stages
// (planes in flight = NS - 1 ahead of the one being collided) and NR planes
// in the normal ring: 4 lets a warp compute the normals of plane z+1 while
// others still collide plane z-1 (one block barrier per plane); 3 saves a
// plane of the ring for one more stage and costs a second barrier per plane
// (collide_tile_tma). Direction q
// of plane z comes as one box of TY rows: TX wide at x0 when c_x = 0 (no x
// halo is read), TX + XU wide otherwise, where XU is the 16-byte alignment
// unit of the x coordinate, starting at x0 - XU for c_x = +1 (halo column
// x0 - 1) and at x0 for c_x = -1 (halo column x0 + TX).
template <int QQ, class S, int NS, class RT = typename Store<S>::T, class G = DefaultTile, int NR = 4>
struct TmaPlan {
    using T = typename Store<S>::T;
    using RingT = RT;  // element type of the normal and |grad phi| rings
    using Tile = G;
    static constexpr int TX = G::TX, TY = G::TY, NX_ = G::NX, NY_ = G::NY;
    static constexpr int kStages = NS;
    static constexpr int kNormSlots = NR;
    static constexpr int XU = 16 / int(sizeof(S));  // elements per 16 bytes
    static constexpr int BWN = TX;                  // box width, c_x = 0
    static constexpr int BWW = TX + XU;             // box width, c_x != 0
    static constexpr int PXO = 4;                   // phi is FP32 or FP64
    static constexpr int PBW = TX + 2 * PXO;        // 40
    static constexpr int PBH = TY + 4;              // 12
    static constexpr int kPhiSlots = NS + 2;        // phi planes z .. z + NS + 1
    // per direction: box width, x origin shift (box starts at x0 - shift),
    // bytes and 128-byte aligned offset inside a stage
    static constexpr int bw(int q) { return detail::dir_c(0, q) == 0 ? BWN : BWW; }
    static constexpr int shift(int q) { return detail::dir_c(0, q) > 0 ? XU : 0; }
    static constexpr size_t box_bytes(int q) { return size_t(TY) * bw(q) * sizeof(S); }
    static constexpr size_t box_off(int q) {
        size_t o = 0;
        for (int k = 0; k < q; ++k) o += align128(box_bytes(k));
        return o;
    }
    static constexpr size_t f_bytes() {
        size_t o = 0;
        for (int k = 0; k < QQ; ++k) o += box_bytes(k);
        return o;
    }
    static constexpr size_t phi_plane_bytes = size_t(PBH) * PBW * sizeof(T);
    // shared-memory strides: every TMA destination starts on a 128-byte boundary
    static constexpr size_t stage_bytes = box_off(QQ);
    static constexpr size_t phi_slot_bytes = align128(phi_plane_bytes);
    static constexpr size_t off_f = 0;
    static constexpr size_t off_phi = align128(NS * stage_bytes);
    // n^ (3 components) of NR planes on the tile + halo 1
    static constexpr size_t off_n = align128(off_phi + kPhiSlots * phi_slot_bytes);
    static constexpr size_t n_bytes = size_t(3) * NR * NY_ * NX_ * sizeof(RT);
    // |grad phi| of 3 planes, tile rows only (rows of the halo width)
    static constexpr size_t off_ind = align128(off_n + n_bytes);
    static constexpr size_t ind_bytes = size_t(3) * TY * NX_ * sizeof(RT);
    static constexpr size_t off_bar = align128(off_ind + ind_bytes);
    // NS mbarriers, the abort flag, and at off_bar + 64 the test build's
    // never-arriving barrier (plane_wait)
    static constexpr size_t total = off_bar + 128;
    static constexpr uint32_t tx_bytes = uint32_t(f_bytes() + phi_plane_bytes);
    static_assert(stage_bytes % 128 == 0 && phi_slot_bytes % 128 == 0 && off_phi % 128 == 0, "TMA smem alignment");
    static_assert((BWN * sizeof(S)) % 16 == 0 && (BWW * sizeof(S)) % 16 == 0 && (PBW * sizeof(T)) % 16 == 0,
                  "TMA inner box extent");
    static_assert(BWW <= 256 && PBW <= 256 && TY <= 256 && PBH <= 256, "TMA box dimension limit");
    static_assert(NS >= 2 && NS * 8 + 4 <= 64, "mbarrier area");
    static_assert(NR == 3 || NR == 4, "normal ring planes");
};

// Deepest pipeline (4, 3 or 2 stages) that keeps two CTAs per SM (FP32 and
// 16-bit storage: <= 113 KB each) or one (FP64: <= 227 KB).
#ifndef PFLBM_TMA_SMEM_BUDGET
#define PFLBM_TMA_SMEM_BUDGET (113u * 1024u)  // per CTA: two CTAs per SM
#endif

// Shared bytes the closure modes add after the TMA plan: the network blob,
// and for FP32 its mma fragments and per-warp feature tiles.
template <class T>
constexpr size_t closure_smem_bytes() {
    return sizeof(float) * size_t(sizeof(T) == 4 ? mlp_smem_words(NT / 32) : kMlpDeviceFloats);
}

// Resident CTAs per SM of the TMA collide: one for FP64; three for D3Q19
// with 16-bit storage, which is issue-bound rather than bandwidth-bound and
// gains more from the extra warps (80 registers) than it loses to the
// shallower pipeline; two otherwise.
template <int QQ, class S>
struct CollideOccupancy {
    static constexpr int value =
        sizeof(typename Store<S>::T) == 8 ? 1 : (sizeof(S) == 2 && QQ == 19 ? 3 : PFLBM_COLLIDE_MIN_BLOCKS);
};

template <int QQ, class S, class G = DefaultTile>
struct TmaStages {
    static constexpr size_t kBudget = sizeof(typename Store<S>::T) == 8 ? 227u * 1024u
                                      : CollideOccupancy<QQ, S>::value == 3 ? 74u * 1024u
                                                                            : size_t(PFLBM_TMA_SMEM_BUDGET);
    using RT = typename Store<S>::T;
    // a third stage with the 3-plane normal ring where the 4-plane ring
    // leaves room for two stages only (D3Q27 with FP32 storage)
    static constexpr bool kDeep4 = TmaPlan<QQ, S, 4, RT, G>::total <= kBudget;
    static constexpr bool kMid4 = TmaPlan<QQ, S, 3, RT, G>::total <= kBudget;
    static constexpr bool kMid3 = TmaPlan<QQ, S, 3, RT, G, 3>::total <= kBudget;
    static constexpr int value = kDeep4 ? 4 : (kMid4 || kMid3) ? 3 : 2;
    static constexpr int rings = (kDeep4 || kMid4 || !kMid3) ? 4 : 3;
};

template <int QQ, class S, class G = DefaultTile>
using TmaLayout = TmaPlan<QQ, S, TmaStages<QQ, S, G>::value, typename Store<S>::T, G, TmaStages<QQ, S, G>::rings>;

// The closure modes place the network after the pipeline's shared memory:
// their pipeline is the deepest whose plan plus the network still fits the
// same per-CTA budget, so that they keep the plain step's resident CTAs.
template <int QQ, class S>
struct TmaClosureStages {
    using T = typename Store<S>::T;
    static constexpr size_t kBudget = TmaStages<QQ, S>::kBudget - closure_smem_bytes<T>();
    static constexpr int value = TmaPlan<QQ, S, 4>::total <= kBudget   ? 4
                                 : TmaPlan<QQ, S, 3>::total <= kBudget ? 3
                                                                       : 2;
};
template <int QQ, class S, int MODE>
using TmaModeLayout = typename std::conditional<mode_closure(MODE), TmaPlan<QQ, S, TmaClosureStages<QQ, S>::value>,
                                                TmaLayout<QQ, S>>::type;

// Barriers of the TMA pipeline: once per CTA, before its first tile.
template <int QQ, class S, class L = TmaLayout<QQ, S>>
__device__ __forceinline__ void tma_pipeline_init(unsigned char *smem) {
    if (threadIdx.x + blockDim.x * threadIdx.y == 0) {
        uint64_t *bar = reinterpret_cast<uint64_t *>(smem + L::off_bar);
        for (int k = 0; k < L::kStages; ++k) mbar_init(&bar[k], 1);
        *reinterpret_cast<volatile int *>(smem + L::off_bar + 8 * L::kStages) = 0;
#ifdef PFLBM_TEST_DEAD_WAIT
        mbar_init(reinterpret_cast<uint64_t *>(smem + L::off_bar + 64), 1);
#endif
        fence_mbar_init();
    }
    __syncthreads();
}

// The per-plane wait of the collide pipelines: phase `parity` of the stage's
// barrier, bounded. A test build (-DPFLBM_TEST_DEAD_WAIT, never the shipped
// library) polls instead a barrier that nothing arrives on, with a short
// limit, so that the wait always runs out and the failure path (error word,
// drain of the CTA's own copies at the full limit, return) is exercised.
template <class L>
__device__ __forceinline__ bool plane_wait(unsigned char *smem, uint64_t *bar, uint32_t parity) {
#ifdef PFLBM_TEST_DEAD_WAIT
    (void)bar;
    (void)parity;
    return mbar_wait_bounded(reinterpret_cast<uint64_t *>(smem + L::off_bar + 64), 0, 1u << 12);
#else
    (void)smem;
    return mbar_wait_bounded(bar, parity, kWaitLimit);
#endif
}

// One column tile [x0, x0+TX) x [y0, y0+TY), planes zb .. ze-1. `seq` counts
// the stages this CTA has consumed so far (stage = seq % NS, mbarrier phase
// parity = (seq / NS) & 1), so that a persistent CTA can run tile after tile
// on the same barriers; every stage issued for a tile is consumed by it.
// Returns false when a bounded wait gave up (error word set, copies drained).
template <int QQ, bool JET, class S, int MODE, class G = DefaultTile, class L = TmaLayout<QQ, S, G>>
__device__ __forceinline__ bool collide_tile_tma(const Params<typename Store<S>::T> &p,
                                                 const StepBuffers<S, typename Store<S>::T> &b,
                                                 const CUtensorMap *fmapn_p, const CUtensorMap *fmapw_p,
                                                 const CUtensorMap *phimap_p, int x0, int y0, int zb, int ze,
                                                 unsigned char *smem, uint32_t &seq, float *s_mlp = nullptr) {
    using T = typename Store<S>::T;
    static_assert(std::is_same<typename L::Tile, G>::value, "plan for this tile");
    constexpr int TX = G::TX, TY = G::TY, NT = G::NT, NX_ = G::NX, NY_ = G::NY, NXP = G::NXP;
    S *s_f = reinterpret_cast<S *>(smem + L::off_f);
    T *s_phi = reinterpret_cast<T *>(smem + L::off_phi);
    T *s_n = reinterpret_cast<T *>(smem + L::off_n);
    T *s_ind = reinterpret_cast<T *>(smem + L::off_ind);
    constexpr int NS = L::kStages, R = L::kPhiSlots, NR = L::kNormSlots;
    // The thread that issues the TMA copies: in the last warp when no lane
    // of that warp computes normal-ring entries, so that with the 3-plane
    // ring the copies are issued while the other warps compute the normals
    // between the plane's two barriers, not by a warp on that critical path.
    constexpr int kNormWork = sizeof(T) == 4 ? NXP * NY_ : NX_ * NY_;
    constexpr int kIssuer = kNormWork <= NT - 32 ? NT - 32 : 0;
    uint64_t *bar = reinterpret_cast<uint64_t *>(smem + L::off_bar);
    volatile int *s_abort = reinterpret_cast<volatile int *>(smem + L::off_bar + 8 * NS);

    const int nx = p.nx, ny = p.ny, nz = p.nz;
    const int tx = threadIdx.x, ty = threadIdx.y, tid = tx + TX * ty;
    const int x = x0 + tx, y = y0 + ty;
    const bool col = (x >= 1 && x <= nx - 2 && y >= 1 && y <= ny - 2);
    const uint32_t t = b.step_in ? static_cast<uint32_t>(*b.step_in) : b.t_fixed;

    auto pslot = [&](int zp) { return (zp + 2 * R) % R; };  // ring slot of phi plane zp (zp >= -2)
    auto phi_at = [&](int slot, int ly, int lx) -> T & {
        return *reinterpret_cast<T *>(reinterpret_cast<unsigned char *>(s_phi) + slot * L::phi_slot_bytes +
                                      (size_t(ly) * L::PBW + lx) * sizeof(T));
    };
    auto n_at = [&](int c, int slot, int ly, int lx) -> T & { return s_n[((c * NR + slot) * NY_ + ly) * NX_ + lx]; };
    auto nslot = [](int zp) { return (zp + NR) % NR; };  // normal ring slot of plane zp (zp >= -1)
    // |grad phi| of plane zp at tile row r, halo column lx (slot zp % 3)
    auto ind_at = [&](int zp, int r, int lx) -> T & { return s_ind[((zp % 3) * TY + r) * NX_ + lx]; };
    auto issue = [&](int stage, int zf) {
        // generic-proxy accesses to the recycled slots are ordered before the
        // async-proxy writes by the preceding block barrier and this fence
        fence_proxy_async();
        mbar_arrive_expect_tx(&bar[stage], L::tx_bytes);
        unsigned char *dst = reinterpret_cast<unsigned char *>(s_f) + size_t(stage) * L::stage_bytes;
#pragma unroll
        for (int q = 0; q < QQ; ++q)
            tma_load_4d(dst + L::box_off(q), kCX[q] == 0 ? fmapn_p : fmapw_p, &bar[stage], x0 - L::shift(q),
                        y0 - kCY[q], zf - kCZ[q], q);
        tma_load_3d(&phi_at(pslot(zf + 2), 0, 0), phimap_p, &bar[stage], x0 - L::PXO, y0 - 2, zf + 2);
    };

    if (tid == 0) {
        tma_prefetch_desc(fmapn_p);
        tma_prefetch_desc(fmapw_p);
        tma_prefetch_desc(phimap_p);
    }

    // warm-up: phi planes zb-2 .. zb+1 with plain loads, normals of zb-1, zb
    for (int zp = zb - 2; zp <= zb + 1; ++zp) {
        const int slot = pslot(zp);
        for (int i = tid; i < L::PBW * L::PBH; i += NT) {
            const int lx = i % L::PBW, ly = i / L::PBW;
            const int gx = x0 - L::PXO + lx, gy = y0 - 2 + ly;
            T v = T(0);
            if (gx >= 0 && gx < nx && gy >= 0 && gy < ny && zp >= 0 && zp < nz)
                v = b.phi_src[gx + static_cast<uint64_t>(nx) * (gy + static_cast<uint64_t>(ny) * zp)];
            phi_at(slot, ly, lx) = v;
        }
    }
    // these generic writes precede later TMA writes to the same ring slots
    fence_proxy_async();
    auto compute_n = [&](int zp) {
        const int sn = pslot(zp), sm = pslot(zp - 1), sp = pslot(zp + 1);
        const int nn = nslot(zp);
        if constexpr (sizeof(T) == 4) {
            // two x-adjacent entries per thread: 170 entry pairs, at most one
            // per thread, so no warp computes a second round
            const bool zok = zp >= 1 && zp <= nz - 2;
            for (int i = tid; i < NXP * NY_; i += NT) {
                const int lx = 2 * (i % NXP), ly = i / NXP;
                const int gxa = x0 - 1 + lx, gy = y0 - 1 + ly;
                const bool yok = zok && gy >= 1 && gy <= ny - 2;
                V2 nxv, nyv, nzv, ind;
                normal_pair<QQ, true>(
                    [&](int dx, int dy, int dz) -> const float * {
                        return &phi_at(dz < 0 ? sm : (dz > 0 ? sp : sn), ly + 1 + dy, lx + L::PXO - 1 + dx);
                    },
                    yok && gxa >= 1 && gxa <= nx - 2, yok && gxa + 1 >= 1 && gxa + 1 <= nx - 2, nxv, nyv, nzv, ind);
                *reinterpret_cast<float2 *>(&n_at(0, nn, ly, lx)) = nxv.v;
                *reinterpret_cast<float2 *>(&n_at(1, nn, ly, lx)) = nyv.v;
                *reinterpret_cast<float2 *>(&n_at(2, nn, ly, lx)) = nzv.v;
                if (ly >= 1 && ly <= TY) *reinterpret_cast<float2 *>(&ind_at(zp, ly - 1, lx)) = ind.v;
            }
        } else {
            for (int i = tid; i < NX_ * NY_; i += NT) {
                const int lx = i % NX_, ly = i / NX_;
                const int gx = x0 - 1 + lx, gy = y0 - 1 + ly;
                T nxv = T(0), nyv = T(0), nzv = T(0), ind = T(0);
                if (gx >= 1 && gx <= nx - 2 && gy >= 1 && gy <= ny - 2 && zp >= 1 && zp <= nz - 2) {
                    auto v = [&](int dx, int dy, int dz) -> T {
                        return phi_at(dz < 0 ? sm : (dz > 0 ? sp : sn), ly + 1 + dy, lx + L::PXO - 1 + dx);
                    };
                    unit_normal<false>(lattice_grad<QQ, 0, T>(v), lattice_grad<QQ, 1, T>(v), lattice_grad<QQ, 2, T>(v),
                                       nxv, nyv, nzv, ind);
                }
                n_at(0, nn, ly, lx) = nxv;
                n_at(1, nn, ly, lx) = nyv;
                n_at(2, nn, ly, lx) = nzv;
                if (ly >= 1 && ly <= TY) ind_at(zp, ly - 1, lx) = ind;
            }
        }
    };
    __syncthreads();
    compute_n(zb - 1);
    __syncthreads();
    // stages 0 .. NS-2 (planes zb .., phi zb+2 ..); the phi ring slot of
    // plane zb+NS aliases that of zb-2, which compute_n(zb-1) no longer needs
    if (tid == kIssuer)
        for (int k = 0; k < NS - 1 && zb + k < ze; ++k) issue((seq + k) % NS, zb + k);
    compute_n(zb);

    for (int z = zb; z < ze; ++z) {
        const uint32_t sq = seq + uint32_t(z - zb);
        const int st = int(sq % NS);
        const uint32_t par = (sq / NS) & 1;
        if (!plane_wait<L>(smem, &bar[st], par)) *s_abort = 1;
        if constexpr (NR == 3) {
            // the ring slot of plane z+1 is that of plane z-2, which the
            // collision of plane z-1 reads: every warp has left it here
            __syncthreads();
        } else {
            compute_n(z + 1);
            __syncthreads();
        }
        if (*s_abort) {
            if (tid == 0) {
                atomicOr(b.err, 1u);
                // drain this CTA's own copies still in flight (planes z .. z+NS-2)
                for (int k = 0; k < NS - 1 && z + k < ze; ++k)
                    mbar_wait_bounded(&bar[(sq + k) % NS], ((sq + k) / NS) & 1, kWaitLimit);
            }
            return false;
        }
        // plane z+NS-1 goes into the stage of plane z-1, consumed last iteration
        if (tid == kIssuer && z + NS - 1 < ze) issue(int((sq + NS - 1) % NS), z + NS - 1);
        if constexpr (NR == 3) {
            compute_n(z + 1);
            __syncthreads();
        }
        // the tensor-core closure network needs every lane of the warp
        constexpr bool kWarpWide = mode_closure(MODE) && std::is_same<T, float>::value;
        if (!col && !kWarpWide) continue;

        const int s_m = nslot(z - 1), s_0 = nslot(z), s_p = nslot(z + 1);
        auto nv = [&](int c, int dx, int dy, int dz) -> T {
            return n_at(c, dz < 0 ? s_m : (dz > 0 ? s_p : s_0), ty + 1 + dy, tx + 1 + dx);
        };
        const T scx = lattice_grad<QQ, 0, T>([&](int dx, int dy, int dz) { return nv(0, dx, dy, dz); });
        const T scy = lattice_grad<QQ, 1, T>([&](int dx, int dy, int dz) { return nv(1, dx, dy, dz); });
        const T scz = lattice_grad<QQ, 2, T>([&](int dx, int dy, int dz) { return nv(2, dx, dy, dz); });
        const T curvature = T(3) * (scx + scy + scz);
        const T n_x = nv(0, 0, 0, 0), n_y = nv(1, 0, 0, 0), n_z = nv(2, 0, 0, 0), ind = ind_at(z, ty, tx + 1);
        const T phi = phi_at(pslot(z), ty + 2, tx + L::PXO);

        T pop[QQ];
        const unsigned char *sf = reinterpret_cast<const unsigned char *>(s_f) + size_t(st) * L::stage_bytes;
        if (kWarpWide && !col) {
#pragma unroll
            for (int q = 0; q < QQ; ++q) pop[q] = T(0);  // placeholder node of the warp-wide network
        } else {
            // node x = x0 + tx pulls x - c_x: element tx - c_x + shift of its row
#pragma unroll
            for (int q = 0; q < QQ; ++q)
                pop[q] = Store<S>::widen(reinterpret_cast<const S *>(sf + L::box_off(q))[ty * L::bw(q) + tx - kCX[q] +
                                                                                          L::shift(q)],
                                         static_cast<T>(weight<QQ>(q)));
        }
        collide_node<QQ, JET, S, MODE>(p, b, x, y, z, t, pop, phi, n_x, n_y, n_z, ind, curvature, s_mlp, col);
    }
    seq += uint32_t(ze - zb);
    return true;
}

template <int QQ, bool JET, class S, int MODE>
__global__ void __launch_bounds__(NT, CollideOccupancy<QQ, S>::value)
    k_collide_tma(const Params<typename Store<S>::T> p, const StepBuffers<S, typename Store<S>::T> b,
                  const __grid_constant__ CUtensorMap fmapn, const __grid_constant__ CUtensorMap fmapw,
                  const __grid_constant__ CUtensorMap phimap) {
    extern __shared__ __align__(128) unsigned char smem[];
    float *s_mlp = nullptr;
    if constexpr (mode_closure(MODE)) {
        // closure network after the pipeline's shared memory (kernels.cuh's k_collide does the same)
        static_assert(TX == 32, "the tensor-core network maps one warp to one tile row");
        s_mlp = reinterpret_cast<float *>(smem + TmaModeLayout<QQ, S, MODE>::total);
        for (int i = threadIdx.x + TX * threadIdx.y; i < kMlpDeviceFloats; i += NT) s_mlp[i] = b.mlp[i];
        __syncthreads();
        if constexpr (std::is_same<typename Store<S>::T, float>::value) {
            mlp_build_fragments(s_mlp, threadIdx.x + TX * threadIdx.y, NT);
            __syncthreads();
        }
    }
    using L = TmaModeLayout<QQ, S, MODE>;
    tma_pipeline_init<QQ, S, L>(smem);
    const int zb = 1 + blockIdx.z * p.zchunk;
    const int ze = min(zb + p.zchunk, int(p.nz) - 1);
    uint32_t seq = 0;
    collide_tile_tma<QQ, JET, S, MODE, DefaultTile, L>(p, b, &fmapn, &fmapw, &phimap, int(blockIdx.x) * TX,
                                                       int(blockIdx.y) * TY, zb, ze, smem, seq, s_mlp);
}

}  // namespace pflbm
