// ensemble.cu - batched ensembles of independent periodic droplet boxes.
//
// Extension of the hot path (no counterpart in the reference, whose grid is
// fixed at compile time): many boxes of different sizes advance together.
// All boxes live in shared allocations (per-box offsets). A fixed grid of
// CTAs pulls work items (box, column tile, z chunk) from device counters and
// runs the same tile code as the single-box collide and phase kernels.
//
// When every box's rows are 16-byte aligned (TMA), one time step is ONE
// persistent cooperative launch (k_step_batch_tma): the collide sweep over
// all items, a bounded grid-wide barrier, the phase sweep over all items.
// Otherwise a step is two persistent launches (plain-load collide, phase).
// Chunks of steps are captured into CUDA graphs. The tile shape (32x8,
// 32x4, 64x4, 32x16), the z-chunk length and the resident CTAs per SM are
// chosen by a measured autotuner.
#include <algorithm>
#include <cstring>
#include <memory>
#include <string>
#include <vector>

#include "../../include/pflbm.h"
#include "engine_impl.cuh"

namespace pflbm {

struct BoxDev {
    Params<float> p;
    uint64_t f_off;  // element offset of the box's Q*N block in the f buffers
    uint64_t n_off;  // element offset of the box's N block in node arrays
};

struct WorkItem {
    int box, x0, y0, zb, ze;
};

// Grid-wide barrier of the fused step (self-resetting: the last CTA to
// arrive clears the count and advances the generation).
struct GridBar {
    unsigned int count;
    unsigned int gen;
    unsigned int never;  // the test build's flag that nothing sets
    unsigned int pad;
};

struct BatchPtrs {
    float *f[2];
    float *phi[2];
    float *J;
    unsigned long long *step;  // [2] ping-pong step counters
    unsigned int *ctr;         // [2] work counters (collide, phase)
    unsigned int *err;
    GridBar *gbar;
};

__device__ __forceinline__ StepBuffers<float, float> box_buffers(const BatchPtrs &bp, const BoxDev &bx, int parity) {
    StepBuffers<float, float> b{};
    b.f_src = bp.f[parity] + bx.f_off;
    b.f_dst = bp.f[parity ^ 1] + bx.f_off;
    b.phi_src = bp.phi[parity] + bx.n_off;
    b.phi_dst = bp.phi[parity ^ 1] + bx.n_off;
    b.jflux = bp.J + 3 * bx.n_off;
    b.top = nullptr;
    b.step_in = bp.step + parity;
    b.step_out = bp.step + (parity ^ 1);
    b.t_fixed = 0;
    b.avg = nullptr;
    b.macro = nullptr;
    b.err = bp.err;
    return b;
}

// Persistent collide over all boxes. Resets the phase kernel's counter (the
// previous phase launch has finished; the next one starts after this one).
template <int QQ>
__global__ void __launch_bounds__(NT, 2)
    k_collide_batch(const BoxDev *boxes, const WorkItem *items, int n_items, BatchPtrs bp, int parity) {
    __shared__ CollideSmem<float> sm;
    __shared__ int s_item;
    const int tid = threadIdx.x + TX * threadIdx.y;
    if (blockIdx.x == 0 && tid == 0) bp.ctr[1] = 0u;
    for (;;) {
        if (tid == 0) s_item = int(atomicAdd(&bp.ctr[0], 1u));
        __syncthreads();
        const int it = s_item;
        __syncthreads();
        if (it >= n_items) break;
        const WorkItem w = items[it];
        const BoxDev &bx = boxes[w.box];
        const StepBuffers<float, float> b = box_buffers(bp, bx, parity);
        collide_tile<QQ, false, float, MODE_STEP>(bx.p, b, w.x0, w.y0, w.zb, w.ze, sm);
        __syncthreads();  // shared rings are reused by the next item
    }
}

// TMA-fed variant of k_collide_batch: the tile code of k_collide_tma on
// per-box tensor maps (kernel parameter, for the launch's parity). The CTA's
// pipeline barriers carry on from tile to tile through `seq`.
constexpr int kMaxTmaBoxes = 64;
struct BatchMaps {
    CUtensorMap fn[kMaxTmaBoxes];  // populations, c_x = 0 boxes
    CUtensorMap fw[kMaxTmaBoxes];  // populations, c_x != 0 boxes
    CUtensorMap phi[kMaxTmaBoxes];
};
static_assert(sizeof(BatchMaps) <= 32764, "kernel parameter limit");

// Tile shapes the batched collide is built for (autotuned per ensemble).
using BatchTile0 = TileShape<32, 8>;
using BatchTile1 = TileShape<32, 4>;
using BatchTile2 = TileShape<64, 4>;
using BatchTile3 = TileShape<32, 16>;
constexpr int kBatchTiles = 4;
constexpr int kBatchTileX[kBatchTiles] = {32, 32, 64, 32};
constexpr int kBatchTileY[kBatchTiles] = {8, 4, 4, 16};

// Resident CTAs per SM the fused kernel is compiled for: 128 registers a
// thread at most.
template <class G>
constexpr int batch_min_blocks() {
    return G::NT <= 128 ? 4 : (G::NT <= 256 ? 2 : 1);
}

// Shared-memory plan of the fused step for tile G: the deepest pipeline
// (4, 3 or 2 stages) that keeps batch_min_blocks<G>() CTAs resident
// (228 KB per SM, 1 KB of it reserved per CTA).
template <int QQ, class G>
struct BatchStages {
    static constexpr size_t kBudget = (228u * 1024u) / batch_min_blocks<G>() - 1024u;
    static constexpr int value = TmaPlan<QQ, float, 4, float, G>::total <= kBudget   ? 4
                                 : TmaPlan<QQ, float, 3, float, G>::total <= kBudget ? 3
                                                                                     : 2;
};
template <int QQ, class G>
using BatchLayout = TmaPlan<QQ, float, BatchStages<QQ, G>::value, float, G>;

// Bounded polls of the grid barrier (with a short sleep each: well above any
// sweep's duration, below a second).
constexpr uint32_t kGridWaitLimit = 1u << 22;

__device__ __forceinline__ unsigned int ld_acquire_gpu(const unsigned int *p) {
    unsigned int v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

// Grid-wide barrier of a cooperative launch, every poll bounded: on a
// timeout the CTA sets bit 2 of the error word and gets false (the caller
// returns; CTAs still waiting on it time out the same way). Thread 0 makes
// the CTA's writes visible (fence after the block barrier) before arriving.
// The test build -DPFLBM_TEST_DEAD_GRID waits instead on a flag that
// nothing sets, with a short limit.
__device__ __forceinline__ bool grid_barrier(GridBar *gb, unsigned int nblocks, unsigned int *err, int *s_ok) {
    __syncthreads();
    if (threadIdx.x == 0 && threadIdx.y == 0) {
        bool ok = true;
        const unsigned int g0 = ld_acquire_gpu(&gb->gen);
        __threadfence();
        const unsigned int arrived = atomicAdd(&gb->count, 1u) + 1u;
#ifdef PFLBM_TEST_DEAD_GRID
        (void)arrived;
        (void)nblocks;
        (void)g0;
        ok = false;
        for (uint32_t i = 0; i < (1u << 12); ++i)
            if (ld_acquire_gpu(&gb->never) != 0u) {
                ok = true;
                break;
            }
        if (!ok) atomicOr(err, 2u);
#else
        if (arrived == nblocks) {
            atomicExch(&gb->count, 0u);
            __threadfence();
            atomicAdd(&gb->gen, 1u);
        } else {
            ok = false;
            for (uint32_t i = 0; i < kGridWaitLimit; ++i) {
                if (ld_acquire_gpu(&gb->gen) != g0) {
                    ok = true;
                    break;
                }
                __nanosleep(64);
            }
            if (!ok) atomicOr(err, 2u);
        }
#endif
        __threadfence();
        *s_ok = ok ? 1 : 0;
    }
    __syncthreads();
    return *s_ok != 0;
}

// One whole time step of every box in ONE launch (cooperative: all CTAs are
// resident): the TMA-fed collide sweep over the work items (the tile code of
// k_collide_tma on per-box tensor maps; the CTA's pipeline barriers carry on
// from tile to tile through `seq`), the grid barrier, then the phase sweep
// over the same items in float4 rows as k_phase_v4 (TMA already requires
// nx % 4 == 0). Work counters: ctr[0] (collide) is cleared after the barrier
// for the next launch, ctr[1] (phase) before it.
template <int QQ, class G>
__global__ void __launch_bounds__(G::NT, batch_min_blocks<G>())
    k_step_batch_tma(const __grid_constant__ BatchMaps maps, const BoxDev *boxes, const WorkItem *items,
                     int n_items, BatchPtrs bp, int parity) {
    using L = BatchLayout<QQ, G>;
    extern __shared__ __align__(128) unsigned char smem[];
    static_assert(8 * L::kStages + 4 <= 56, "item slot and barrier flag after the mbarriers");
    volatile int *s_item = reinterpret_cast<volatile int *>(smem + L::off_bar + 56);
    int *s_ok = reinterpret_cast<int *>(smem + L::off_bar + 60);
    const int tid = threadIdx.x + G::TX * threadIdx.y;
    if (blockIdx.x == 0 && tid == 0) bp.ctr[1] = 0u;
    tma_pipeline_init<QQ, float, L>(smem);
    uint32_t seq = 0;
    for (;;) {
        if (tid == 0) *s_item = int(atomicAdd(&bp.ctr[0], 1u));
        __syncthreads();
        const int it = *s_item;
        __syncthreads();
        if (it >= n_items) break;
        const WorkItem w = items[it];
        const BoxDev &bx = boxes[w.box];
        const StepBuffers<float, float> b = box_buffers(bp, bx, parity);
        if (!collide_tile_tma<QQ, false, float, MODE_STEP, G, L>(bx.p, b, &maps.fn[w.box], &maps.fw[w.box],
                                                             &maps.phi[w.box], w.x0, w.y0, w.zb, w.ze, smem, seq))
            return;
        __syncthreads();  // shared rings are reused by the next item
    }
    if (!grid_barrier(bp.gbar, gridDim.x, bp.err, s_ok)) return;
    if (blockIdx.x == 0 && tid == 0) {
        bp.ctr[0] = 0u;
        bp.step[parity ^ 1] = bp.step[parity] + 1ull;
    }
    // phase sweep: TX / 4 float4 segments per tile row, 4 groups of planes
    constexpr int SEGS = G::TX / 4;
    static_assert(G::TX / SEGS == 4, "four plane groups");
    const int seg = int(threadIdx.x) % SEGS, zo = int(threadIdx.x) / SEGS;
    for (;;) {
        if (tid == 0) *s_item = int(atomicAdd(&bp.ctr[1], 1u));
        __syncthreads();
        const int it = *s_item;
        __syncthreads();
        if (it >= n_items) break;
        const WorkItem w = items[it];
        const BoxDev &bx = boxes[w.box];
        const StepBuffers<float, float> b = box_buffers(bp, bx, parity);
        const int y = w.y0 + int(threadIdx.y), x4 = w.x0 + 4 * seg;
        if (x4 < int(bx.p.nx) && y >= 1 && y <= int(bx.p.ny) - 2)
            for (int z = w.zb + zo; z < w.ze; z += 4) phase_vec4<false, float>(bx.p, b, x4, y, z);
    }
}

// Persistent phase step over the same work items; advances the step counter
// and resets the collide kernel's work counter.
template <int QQ>
__global__ void __launch_bounds__(NT)
    k_phase_batch(const BoxDev *boxes, const WorkItem *items, int n_items, BatchPtrs bp, int parity) {
    __shared__ int s_item;
    const int tid = threadIdx.x + TX * threadIdx.y;
    const uint32_t t = static_cast<uint32_t>(bp.step[parity]);
    if (blockIdx.x == 0 && tid == 0) {
        bp.ctr[0] = 0u;
        bp.step[parity ^ 1] = bp.step[parity] + 1ull;
    }
    for (;;) {
        if (tid == 0) s_item = int(atomicAdd(&bp.ctr[1], 1u));
        __syncthreads();
        const int it = s_item;
        __syncthreads();
        if (it >= n_items) break;
        const WorkItem w = items[it];
        const BoxDev &bx = boxes[w.box];
        const StepBuffers<float, float> b = box_buffers(bp, bx, parity);
        const int x = w.x0 + int(threadIdx.x), y = w.y0 + int(threadIdx.y);
        if (x >= 1 && x <= int(bx.p.nx) - 2 && y >= 1 && y <= int(bx.p.ny) - 2)
            for (int z = w.zb; z < w.ze; ++z) phase_node<QQ, false, float>(bx.p, b, x, y, z, t);
    }
}

// Vectorised phase step over the same work items for boxes with nx % 4 == 0
// (phase_vec4, as k_phase_v4): in a 32x8 tile, 8 threads cover a row as 4
// float4 segments and the 4 groups of 8 take every 4th plane of the chunk.
template <int QQ>
__global__ void __launch_bounds__(NT)
    k_phase_batch_v4(const BoxDev *boxes, const WorkItem *items, int n_items, BatchPtrs bp, int parity) {
    static_assert(TX == 32, "8 float4 segments per 32-node tile row");
    __shared__ int s_item;
    const int tid = threadIdx.x + TX * threadIdx.y;
    if (blockIdx.x == 0 && tid == 0) {
        bp.ctr[0] = 0u;
        bp.step[parity ^ 1] = bp.step[parity] + 1ull;
    }
    const int seg = threadIdx.x & 7, zo = threadIdx.x >> 3;
    for (;;) {
        if (tid == 0) s_item = int(atomicAdd(&bp.ctr[1], 1u));
        __syncthreads();
        const int it = s_item;
        __syncthreads();
        if (it >= n_items) break;
        const WorkItem w = items[it];
        const BoxDev &bx = boxes[w.box];
        const StepBuffers<float, float> b = box_buffers(bp, bx, parity);
        const int x4 = w.x0 + 4 * seg, y = w.y0 + int(threadIdx.y);
        if (x4 < int(bx.p.nx) && y >= 1 && y <= int(bx.p.ny) - 2)
            for (int z = w.zb + zo; z < w.ze; z += 4) phase_vec4<false, float>(bx.p, b, x4, y, z);
    }
}

class Ensemble {
   public:
    int q = 19;
    int device = 0;
    int sms = 152;
    std::vector<pflbm_config> cfgs;
    std::vector<HostParams> hps;
    std::vector<BoxDev> boxes;
    std::vector<WorkItem> items;
    BoxDev *d_boxes = nullptr;
    WorkItem *d_items = nullptr;
    int n_items = 0;
    BatchPtrs bp{};
    float *macro = nullptr;
    double *partial = nullptr, *dev_diag = nullptr;
    uint64_t total_nodes = 0, max_nodes = 0;
    cudaStream_t stream = nullptr;
    cudaGraphExec_t graphs[2] = {nullptr, nullptr};  // kChunk steps per parity
    int parity = 0;
    uint64_t step = 0;
    int zchunk = 16, ctas_per_sm = 2;
    int tile = 0;                          // batch tile shape (kBatchTileX/Y) of the fused TMA step
    int max_ctas[kBatchTiles] = {};        // resident CTAs per SM of the fused step, per tile shape
    bool initialized = false;
    bool use_tma = false;
    bool use_vec = false;  // every box has nx % 4 == 0: float4 phase kernel
    std::unique_ptr<BatchMaps> maps[kBatchTiles][2];  // per tile shape (box sizes) and parity (read buffer)
    static constexpr int kChunk = 16;
    static constexpr int kRedBlocks = 304;

    ~Ensemble() { release(); }

    void release() {
        for (auto &g : graphs)
            if (g) cudaGraphExecDestroy(g), g = nullptr;
        void *ptrs[] = {bp.f[0], bp.f[1], bp.phi[0], bp.phi[1], bp.J, bp.step, bp.ctr, bp.err, bp.gbar,
                        macro, partial, dev_diag, d_boxes, d_items};
        for (void *p : ptrs)
            if (p) cudaFree(p);
        std::memset(&bp, 0, sizeof bp);
        macro = nullptr;
        partial = dev_diag = nullptr;
        d_boxes = nullptr;
        d_items = nullptr;
        if (stream) cudaStreamDestroy(stream), stream = nullptr;
    }

    int tile_x() const { return use_tma ? kBatchTileX[tile] : TX; }
    int tile_y() const { return use_tma ? kBatchTileY[tile] : TY; }

    int build_items() {
        items.clear();
        const int tx = tile_x(), ty = tile_y();
        for (size_t k = 0; k < boxes.size(); ++k) {
            const auto &p = boxes[k].p;
            const int nzi = int(p.nz) - 2;
            const int zc = std::max(1, std::min(zchunk, nzi));
            for (int zb = 1; zb < int(p.nz) - 1; zb += zc)
                for (int y0 = 0; y0 < int(p.ny); y0 += ty)
                    for (int x0 = 0; x0 < int(p.nx); x0 += tx)
                        items.push_back({int(k), x0, y0, zb, std::min(zb + zc, int(p.nz) - 1)});
        }
        // largest boxes first: long items start early, short ones fill the tail
        std::stable_sort(items.begin(), items.end(), [&](const WorkItem &a, const WorkItem &b) {
            return boxes[a.box].p.N > boxes[b.box].p.N;
        });
        n_items = int(items.size());
        if (d_items) cudaFree(d_items), d_items = nullptr;
        if (cudaMalloc(&d_items, sizeof(WorkItem) * items.size()) != cudaSuccess) return PFLBM_ERR_OUT_OF_MEMORY;
        if (cudaMemcpy(d_items, items.data(), sizeof(WorkItem) * items.size(), cudaMemcpyHostToDevice) != cudaSuccess)
            return PFLBM_ERR_CUDA;
        return PFLBM_OK;
    }

    // TMA maps for every box and parity when all rows are 16-byte aligned
    // and the boxes fit the kernel-parameter table; otherwise plain loads.
    // PFLBM_NO_TMA=1 forces plain loads.
    void setup_tma() {
        use_tma = false;
        use_vec = true;
        for (const auto &bx : boxes)
            if (bx.p.nx % 4 != 0) use_vec = false;
        if (const char *e = std::getenv("PFLBM_NO_VEC"))
            if (e[0] == '1') use_vec = false;
        if (const char *e = std::getenv("PFLBM_NO_TMA"))
            if (e[0] == '1') return;
        if (boxes.size() > size_t(kMaxTmaBoxes)) return;
        for (const auto &bx : boxes)
            if ((uint64_t(bx.p.nx) * sizeof(float)) % 16 != 0) return;
        // the fused step for every tile shape: tensor maps with that tile's
        // boxes, shared memory, and how many CTAs stay resident (a
        // cooperative launch needs them all); a shape whose maps cannot be
        // encoded is not offered
        bool any = false;
        for (int t = 0; t < kBatchTiles; ++t) {
            max_ctas[t] = (q == 19 ? encode_tile_maps<19>(t) : encode_tile_maps<27>(t))
                              ? (q == 19 ? fused_occupancy<19>(t) : fused_occupancy<27>(t))
                              : 0;
            any = any || max_ctas[t] > 0;
        }
        if (!any || !use_vec) return;
        use_tma = true;
        if (max_ctas[tile] == 0)
            for (int t = 0; t < kBatchTiles; ++t)
                if (max_ctas[t] > 0) {
                    tile = t;
                    break;
                }
        ctas_per_sm = std::min(ctas_per_sm, max_ctas[tile]);
    }

    template <int QQ, class G>
    bool encode_tile_maps_of(int t) {
        for (int par = 0; par < 2; ++par) {
            maps[t][par].reset(new (std::nothrow) BatchMaps());
            if (!maps[t][par]) return false;
            BatchMaps &m = *maps[t][par];
            for (size_t k = 0; k < boxes.size(); ++k) {
                const BoxDev &bx = boxes[k];
                if (!encode_collide_maps<QQ, float, BatchLayout<QQ, G>>(bp.f[par] + bx.f_off, bp.phi[par] + bx.n_off,
                                                                        bx.p.nx, bx.p.ny, bx.p.nz, m.fn[k], m.fw[k],
                                                                        m.phi[k]))
                    return false;
            }
        }
        return true;
    }
    template <int QQ>
    bool encode_tile_maps(int t) {
        switch (t) {
            case 0: return encode_tile_maps_of<QQ, BatchTile0>(t);
            case 1: return encode_tile_maps_of<QQ, BatchTile1>(t);
            case 2: return encode_tile_maps_of<QQ, BatchTile2>(t);
            default: return encode_tile_maps_of<QQ, BatchTile3>(t);
        }
    }

    template <int QQ, class G>
    int fused_occupancy_of() {
        using L = BatchLayout<QQ, G>;
        if (cudaFuncSetAttribute(k_step_batch_tma<QQ, G>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 int(L::total)) != cudaSuccess) {
            cudaGetLastError();
            return 0;
        }
        int n = 0;
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_step_batch_tma<QQ, G>, G::NT, L::total) !=
            cudaSuccess) {
            cudaGetLastError();
            return 0;
        }
        return n;
    }
    template <int QQ>
    int fused_occupancy(int t) {
        switch (t) {
            case 0: return fused_occupancy_of<QQ, BatchTile0>();
            case 1: return fused_occupancy_of<QQ, BatchTile1>();
            case 2: return fused_occupancy_of<QQ, BatchTile2>();
            default: return fused_occupancy_of<QQ, BatchTile3>();
        }
    }

    template <int QQ, class G>
    cudaError_t launch_fused(int par, int grid, cudaStream_t s) {
        cudaLaunchConfig_t cfg{};
        cfg.gridDim = dim3(grid);
        cfg.blockDim = dim3(G::TX, G::TY);
        cfg.dynamicSmemBytes = BatchLayout<QQ, G>::total;
        cfg.stream = s;
        cudaLaunchAttribute attr[1];
        attr[0].id = cudaLaunchAttributeCooperative;
        attr[0].val.cooperative = 1;
        cfg.attrs = attr;
        cfg.numAttrs = 1;
        return cudaLaunchKernelEx(&cfg, k_step_batch_tma<QQ, G>, *maps[tile][par], static_cast<const BoxDev *>(d_boxes),
                                  static_cast<const WorkItem *>(d_items), n_items, bp, par);
    }
    template <int QQ>
    cudaError_t launch_fused_tile(int par, int grid, cudaStream_t s) {
        switch (tile) {
            case 0: return launch_fused<QQ, BatchTile0>(par, grid, s);
            case 1: return launch_fused<QQ, BatchTile1>(par, grid, s);
            case 2: return launch_fused<QQ, BatchTile2>(par, grid, s);
            default: return launch_fused<QQ, BatchTile3>(par, grid, s);
        }
    }

    // One time step: the fused cooperative launch (TMA) or the two
    // persistent launches of the plain-load path.
    cudaError_t enqueue_step(int par, cudaStream_t s) {
        const int grid = std::max(1, sms * ctas_per_sm);
        if (use_tma) return q == 19 ? launch_fused_tile<19>(par, grid, s) : launch_fused_tile<27>(par, grid, s);
        if (q == 19) {
            k_collide_batch<19><<<grid, dim3(TX, TY), 0, s>>>(d_boxes, d_items, n_items, bp, par);
            if (use_vec)
                k_phase_batch_v4<19><<<grid, dim3(TX, TY), 0, s>>>(d_boxes, d_items, n_items, bp, par);
            else
                k_phase_batch<19><<<grid, dim3(TX, TY), 0, s>>>(d_boxes, d_items, n_items, bp, par);
        } else {
            k_collide_batch<27><<<grid, dim3(TX, TY), 0, s>>>(d_boxes, d_items, n_items, bp, par);
            if (use_vec)
                k_phase_batch_v4<27><<<grid, dim3(TX, TY), 0, s>>>(d_boxes, d_items, n_items, bp, par);
            else
                k_phase_batch<27><<<grid, dim3(TX, TY), 0, s>>>(d_boxes, d_items, n_items, bp, par);
        }
        return cudaGetLastError();
    }

    int capture() {
        for (auto &g : graphs)
            if (g) cudaGraphExecDestroy(g), g = nullptr;
        for (int par = 0; par < 2; ++par) {
            cudaGraph_t g = nullptr;
            if (cudaStreamBeginCapture(stream, cudaStreamCaptureModeThreadLocal) != cudaSuccess) return PFLBM_ERR_CUDA;
            int pp = par;
            cudaError_t le = cudaSuccess;
            for (int i = 0; i < kChunk && le == cudaSuccess; ++i, pp ^= 1) le = enqueue_step(pp, stream);
            if (cudaStreamEndCapture(stream, &g) != cudaSuccess || le != cudaSuccess) {
                if (g) cudaGraphDestroy(g);
                return PFLBM_ERR_CUDA;
            }
            const cudaError_t e = cudaGraphInstantiate(&graphs[par], g, 0);
            cudaGraphDestroy(g);
            if (e != cudaSuccess) return PFLBM_ERR_CUDA;
        }
        return PFLBM_OK;
    }

    StepBuffers<float, float> host_box_buffers(int k, int par) const {
        StepBuffers<float, float> b{};
        const BoxDev &bx = boxes[k];
        b.f_src = bp.f[par] + bx.f_off;
        b.f_dst = bp.f[par ^ 1] + bx.f_off;
        b.phi_src = bp.phi[par] + bx.n_off;
        b.phi_dst = bp.phi[par ^ 1] + bx.n_off;
        b.jflux = bp.J + 3 * bx.n_off;
        b.macro = macro;
        b.err = bp.err;
        return b;
    }

    void enqueue_init_box(int k) {
        const auto &h = hps[k];
        const Params<float> &p = boxes[k].p;
        InitGeom g{};
        g.jet = 0;
        g.droplet_x_stretch = h.droplet_x_stretch;
        g.center_z = h.f_center_z;
        g.radius = h.radius;
        g.interface_width = h.interface_width;
        g.init_noise = h.init_noise;
        const dim3 blk(32, 8, 1), grd((p.nx + 31) / 32, (p.ny + 7) / 8, p.nz);
        k_init_fields<float><<<grd, blk, 0, stream>>>(p, g, macro);
        const BoxDev &bx = boxes[k];
        if (q == 19)
            k_init_distros<19, false, float><<<grd, blk, 0, stream>>>(p, bp.f[0] + bx.f_off, bp.f[1] + bx.f_off,
                                                                      bp.phi[0] + bx.n_off, bp.phi[1] + bx.n_off, macro);
        else
            k_init_distros<27, false, float><<<grd, blk, 0, stream>>>(p, bp.f[0] + bx.f_off, bp.f[1] + bx.f_off,
                                                                      bp.phi[0] + bx.n_off, bp.phi[1] + bx.n_off, macro);
    }

    // Analysis of one box after the last completed step into the macro cache.
    void enqueue_analysis_box(int k) {
        const Params<float> &p = boxes[k].p;
        const dim3 blk(32, 8, 1), grd((p.nx + 31) / 32, (p.ny + 7) / 8, p.nz);
        if (step == 0) {
            enqueue_init_box(k);  // the cache then holds the initial fields
            return;
        }
        StepBuffers<float, float> b = host_box_buffers(k, parity ^ 1);
        b.f_dst = nullptr;
        b.phi_dst = nullptr;
        b.step_in = nullptr;
        b.t_fixed = uint32_t(step - 1);
        const int chunks = (int(p.nz) - 2 + p.zchunk - 1) / p.zchunk;
        const dim3 cg((p.nx + TX - 1) / TX, (p.ny + TY - 1) / TY, chunks);
        if (q == 19)
            k_collide<19, false, float, MODE_ANALYSIS><<<cg, dim3(TX, TY), 0, stream>>>(p, b);
        else
            k_collide<27, false, float, MODE_ANALYSIS><<<cg, dim3(TX, TY), 0, stream>>>(p, b);
        k_analysis_ghosts<float><<<grd, blk, 0, stream>>>(p, 0, uint32_t(step - 1), macro);
    }
};

}  // namespace pflbm

struct pflbm_ensemble : pflbm::Ensemble {};

using pflbm::Ensemble;

namespace {
int efail(int code, const std::string &m) {
    pflbm::set_error(m);
    return code;
}
int ecuda(cudaError_t e, const char *what) {
    cudaGetLastError();
    return efail(PFLBM_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}
}  // namespace

extern "C" {

int pflbm_ensemble_create(const pflbm_config *cfgs, int32_t n, pflbm_ensemble **out) {
    if (!cfgs || !out || n <= 0) return efail(PFLBM_ERR_INVALID_ARG, "null or empty configuration list");
    *out = nullptr;
    std::unique_ptr<pflbm_ensemble> e(new (std::nothrow) pflbm_ensemble());
    if (!e) return efail(PFLBM_ERR_OUT_OF_MEMORY, "host allocation failed");
    e->q = cfgs[0].velocity_set;
    for (int k = 0; k < n; ++k) {
        const int rc = pflbm::validate(cfgs[k]);
        if (rc) return rc;
        if (cfgs[k].flow_case != PFLBM_CASE_DROPLET)
            return efail(PFLBM_ERR_UNSUPPORTED, "ensembles hold periodic droplet boxes only");
        if (cfgs[k].storage != PFLBM_STORAGE_FP32) return efail(PFLBM_ERR_UNSUPPORTED, "ensembles run FP32 storage");
        if (cfgs[k].velocity_set != e->q) return efail(PFLBM_ERR_INVALID_ARG, "all boxes must share the velocity set");
        if (cfgs[k].flags != 0) return efail(PFLBM_ERR_UNSUPPORTED, "derived fields are not kept for ensembles");
    }
    int dev = cfgs[0].device >= 0 ? cfgs[0].device : 0;
    if (cfgs[0].device < 0)
        if (const char *g = std::getenv("GPU_INDEX")) dev = std::atoi(g);
    cudaError_t ce = cudaSetDevice(dev);
    if (ce != cudaSuccess) return ecuda(ce, "cudaSetDevice");
    e->device = dev;
    cudaDeviceGetAttribute(&e->sms, cudaDevAttrMultiProcessorCount, dev);
    e->cfgs.assign(cfgs, cfgs + n);
    e->hps.resize(n);
    e->boxes.resize(n);
    uint64_t f_off = 0, n_off = 0;
    for (int k = 0; k < n; ++k) {
        pflbm::derive(cfgs[k], e->hps[k]);
        e->hps[k].zchunk = e->zchunk;
        e->boxes[k].p = pflbm::make_params<float>(e->hps[k]);
        e->boxes[k].f_off = f_off;
        e->boxes[k].n_off = n_off;
        f_off += uint64_t(e->q) * e->hps[k].N;
        n_off += e->hps[k].N;
        e->max_nodes = std::max(e->max_nodes, e->hps[k].N);
    }
    e->total_nodes = n_off;
    auto alloc = [&](void **p, size_t bytes) {
        if (cudaMalloc(p, bytes) != cudaSuccess) return false;
        cudaMemset(*p, 0, bytes);
        return true;
    };
    bool ok = alloc(reinterpret_cast<void **>(&e->bp.f[0]), sizeof(float) * f_off) &&
              alloc(reinterpret_cast<void **>(&e->bp.f[1]), sizeof(float) * f_off) &&
              alloc(reinterpret_cast<void **>(&e->bp.phi[0]), sizeof(float) * n_off) &&
              alloc(reinterpret_cast<void **>(&e->bp.phi[1]), sizeof(float) * n_off) &&
              alloc(reinterpret_cast<void **>(&e->bp.J), sizeof(float) * 3 * n_off) &&
              alloc(reinterpret_cast<void **>(&e->bp.step), sizeof(unsigned long long) * 2) &&
              alloc(reinterpret_cast<void **>(&e->bp.ctr), sizeof(unsigned int) * 2) &&
              alloc(reinterpret_cast<void **>(&e->bp.err), sizeof(unsigned int) * 4) &&
              alloc(reinterpret_cast<void **>(&e->bp.gbar), sizeof(pflbm::GridBar)) &&
              alloc(reinterpret_cast<void **>(&e->macro), sizeof(float) * pflbm::M_COUNT * e->max_nodes) &&
              alloc(reinterpret_cast<void **>(&e->partial), sizeof(double) * pflbm::RED_FIELDS * Ensemble::kRedBlocks) &&
              alloc(reinterpret_cast<void **>(&e->dev_diag), sizeof(double) * 16) &&
              alloc(reinterpret_cast<void **>(&e->d_boxes), sizeof(pflbm::BoxDev) * n);
    if (!ok) {
        cudaGetLastError();
        return efail(PFLBM_ERR_OUT_OF_MEMORY, "ensemble device allocation failed");
    }
    cudaMemcpy(e->d_boxes, e->boxes.data(), sizeof(pflbm::BoxDev) * n, cudaMemcpyHostToDevice);
    ce = cudaStreamCreateWithFlags(&e->stream, cudaStreamNonBlocking);
    if (ce != cudaSuccess) return ecuda(ce, "cudaStreamCreate");
    e->setup_tma();
    int rc = e->build_items();
    if (rc) return efail(rc, "work list allocation failed");
    rc = e->capture();
    if (rc) return ecuda(cudaGetLastError(), "ensemble graph capture");
    *out = e.release();
    return PFLBM_OK;
}

int pflbm_ensemble_init(pflbm_ensemble *e) {
    if (!e) return efail(PFLBM_ERR_INVALID_ARG, "null ensemble");
    cudaSetDevice(e->device);
    cudaMemsetAsync(e->bp.step, 0, sizeof(unsigned long long) * 2, e->stream);
    cudaMemsetAsync(e->bp.ctr, 0, sizeof(unsigned int) * 2, e->stream);
    cudaMemsetAsync(e->bp.err, 0, sizeof(unsigned int) * 4, e->stream);
    cudaMemsetAsync(e->bp.gbar, 0, sizeof(pflbm::GridBar), e->stream);
    for (size_t k = 0; k < e->boxes.size(); ++k) e->enqueue_init_box(int(k));
    const cudaError_t ce = cudaStreamSynchronize(e->stream);
    if (ce != cudaSuccess) return ecuda(ce, "ensemble init");
    e->parity = 0;
    e->step = 0;
    e->initialized = true;
    return PFLBM_OK;
}

int pflbm_ensemble_step(pflbm_ensemble *e, uint64_t n) {
    if (!e) return efail(PFLBM_ERR_INVALID_ARG, "null ensemble");
    if (!e->initialized) return efail(PFLBM_ERR_STATE, "pflbm_ensemble_init has not been called");
    cudaSetDevice(e->device);
    uint64_t left = n;
    while (left >= uint64_t(Ensemble::kChunk)) {
        const cudaError_t ce = cudaGraphLaunch(e->graphs[e->parity], e->stream);
        if (ce != cudaSuccess) return ecuda(ce, "cudaGraphLaunch");
        left -= Ensemble::kChunk;
        e->step += Ensemble::kChunk;
    }
    for (; left > 0; --left) {
        const cudaError_t le = e->enqueue_step(e->parity, e->stream);
        if (le != cudaSuccess) return ecuda(le, "ensemble step launch");
        e->parity ^= 1;
        e->step += 1;
    }
    cudaError_t ce = cudaStreamSynchronize(e->stream);
    if (ce != cudaSuccess) return ecuda(ce, "ensemble step");
    unsigned int w = 0;
    cudaMemcpy(&w, e->bp.err, sizeof w, cudaMemcpyDeviceToHost);
    if (w) return efail(PFLBM_ERR_DEVICE, "a kernel reported an error");
    return PFLBM_OK;
}

int pflbm_ensemble_step_profiled(pflbm_ensemble *e, uint64_t n, double *ms) {
    if (!e || !ms) return efail(PFLBM_ERR_INVALID_ARG, "null argument");
    cudaEvent_t a, b;
    cudaEventCreate(&a);
    cudaEventCreate(&b);
    cudaEventRecord(a, e->stream);
    const int rc = pflbm_ensemble_step(e, n);
    cudaEventRecord(b, e->stream);
    cudaEventSynchronize(b);
    float t = 0.0f;
    cudaEventElapsedTime(&t, a, b);
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    *ms = t;
    return rc;
}

int pflbm_ensemble_get_field(pflbm_ensemble *e, int32_t box, int32_t id, void *host, size_t bytes) {
    if (!e || !host) return efail(PFLBM_ERR_INVALID_ARG, "null argument");
    if (box < 0 || box >= int32_t(e->boxes.size())) return efail(PFLBM_ERR_INVALID_ARG, "box index out of range");
    if (id < 0 || id > PFLBM_FIELD_FFZ) return efail(PFLBM_ERR_UNSUPPORTED, "ensembles provide fields 0..17");
    const uint64_t N = e->hps[box].N;
    if (bytes < N * sizeof(float)) return efail(PFLBM_ERR_INVALID_ARG, "destination buffer too small");
    cudaSetDevice(e->device);
    e->enqueue_analysis_box(box);
    const cudaError_t ce =
        cudaMemcpyAsync(host, e->macro + size_t(id) * N, N * sizeof(float), cudaMemcpyDeviceToHost, e->stream);
    if (ce != cudaSuccess) return ecuda(ce, "ensemble readback");
    const cudaError_t se = cudaStreamSynchronize(e->stream);
    if (se != cudaSuccess) return ecuda(se, "ensemble readback");
    return PFLBM_OK;
}

int pflbm_ensemble_reduce(pflbm_ensemble *e, int32_t box, pflbm_diag *d) {
    if (!e || !d) return efail(PFLBM_ERR_INVALID_ARG, "null argument");
    if (box < 0 || box >= int32_t(e->boxes.size())) return efail(PFLBM_ERR_INVALID_ARG, "box index out of range");
    cudaSetDevice(e->device);
    e->enqueue_analysis_box(box);
    pflbm::k_reduce_partial<float><<<Ensemble::kRedBlocks, pflbm::RED_THREADS, 0, e->stream>>>(e->boxes[box].p, e->macro,
                                                                                               e->partial);
    pflbm::k_reduce_final<<<1, 32, 0, e->stream>>>(e->partial, Ensemble::kRedBlocks, e->dev_diag);
    double r[12];
    cudaMemcpyAsync(r, e->dev_diag, sizeof r, cudaMemcpyDeviceToHost, e->stream);
    const cudaError_t ce = cudaStreamSynchronize(e->stream);
    if (ce != cudaSuccess) return ecuda(ce, "ensemble reduce");
    std::memset(d, 0, sizeof(*d));
    d->step = e->step;
    d->phi_mass = r[0];
    d->rho_mass = r[1];
    d->momentum[0] = r[2]; d->momentum[1] = r[3]; d->momentum[2] = r[4];
    d->max_speed = r[5];
    d->n_in = uint64_t(r[7]);
    d->n_out = uint64_t(r[9]);
    d->rho_in = r[7] > 0 ? r[6] / r[7] : 0.0;
    d->rho_out = r[9] > 0 ? r[8] / r[9] : 0.0;
    d->laplace_dp = (d->rho_in - d->rho_out) / 3.0;
    d->nonfinite = uint64_t(r[10]);
    return d->nonfinite ? efail(PFLBM_ERR_DIVERGED, "non-finite values") : PFLBM_OK;
}

namespace {
int ensemble_retune(pflbm_ensemble *e, int tile, int zchunk, int ctas_per_sm) {
    cudaSetDevice(e->device);
    cudaStreamSynchronize(e->stream);
    e->tile = tile;
    e->zchunk = zchunk;
    e->ctas_per_sm = ctas_per_sm;
    int rc = e->build_items();
    if (rc) return efail(rc, "work list rebuild failed");
    rc = e->capture();
    if (rc) return ecuda(cudaGetLastError(), "ensemble graph capture");
    return PFLBM_OK;
}

int max_ctas_for(const pflbm_ensemble *e, int tile) { return e->use_tma ? e->max_ctas[tile] : 2; }
}  // namespace

int pflbm_ensemble_set_tuning(pflbm_ensemble *e, int32_t zchunk, int32_t ctas_per_sm) {
    if (!e || zchunk <= 0 || ctas_per_sm <= 0 || ctas_per_sm > max_ctas_for(e, e->tile))
        return efail(PFLBM_ERR_INVALID_ARG, "zchunk > 0 and ctas_per_sm in 1 .. the tile shape's resident limit");
    return ensemble_retune(e, e->tile, zchunk, ctas_per_sm);
}

int pflbm_ensemble_set_tile(pflbm_ensemble *e, int32_t tile_x, int32_t tile_y) {
    if (!e) return efail(PFLBM_ERR_INVALID_ARG, "null ensemble");
    if (!e->use_tma) {
        if (tile_x == pflbm::TX && tile_y == pflbm::TY) return PFLBM_OK;
        return efail(PFLBM_ERR_UNSUPPORTED, "the plain-load batch path has the 32x8 tile only");
    }
    for (int t = 0; t < pflbm::kBatchTiles; ++t)
        if (pflbm::kBatchTileX[t] == tile_x && pflbm::kBatchTileY[t] == tile_y) {
            if (e->max_ctas[t] == 0) return efail(PFLBM_ERR_UNSUPPORTED, "tile shape does not fit this GPU");
            return ensemble_retune(e, t, e->zchunk, std::min(e->ctas_per_sm, e->max_ctas[t]));
        }
    return efail(PFLBM_ERR_INVALID_ARG, "tile shapes: 32x8, 32x4, 64x4, 32x16");
}

int pflbm_ensemble_get_tuning(const pflbm_ensemble *e, int32_t *tile_x, int32_t *tile_y, int32_t *zchunk,
                              int32_t *ctas_per_sm) {
    if (!e) return efail(PFLBM_ERR_INVALID_ARG, "null ensemble");
    if (tile_x) *tile_x = e->tile_x();
    if (tile_y) *tile_y = e->tile_y();
    if (zchunk) *zchunk = e->zchunk;
    if (ctas_per_sm) *ctas_per_sm = e->ctas_per_sm;
    return PFLBM_OK;
}

// Times every candidate (tile shape x zchunk x resident CTAs per SM) for
// trial_steps steps from the current state, keeps the fastest, then
// re-initialises the ensemble so the tuning leaves no trace in the results.
int pflbm_ensemble_autotune(pflbm_ensemble *e, int32_t trial_steps, int32_t *best_zchunk, int32_t *best_ctas,
                            double *best_ms) {
    if (!e || trial_steps <= 0) return efail(PFLBM_ERR_INVALID_ARG, "bad argument");
    const int zcs[] = {4, 8, 16, 32, 64};
    double best = 1e300;
    int bt = e->tile, bz = e->zchunk, bc = e->ctas_per_sm;
    const int ntiles = e->use_tma ? pflbm::kBatchTiles : 1;
    for (int t = 0; t < ntiles; ++t) {
        const int tt = e->use_tma ? t : e->tile;
        for (int c = 1; c <= max_ctas_for(e, tt); ++c)
            for (int zc : zcs) {
                int rc = ensemble_retune(e, tt, zc, c);
                if (rc) return rc;
                rc = pflbm_ensemble_step(e, 2);
                if (rc) return rc;
                double ms = 0;
                rc = pflbm_ensemble_step_profiled(e, uint64_t(trial_steps), &ms);
                if (rc) return rc;
                if (ms < best) best = ms, bt = tt, bz = zc, bc = c;
            }
    }
    int rc = ensemble_retune(e, bt, bz, bc);
    if (rc) return rc;
    rc = pflbm_ensemble_init(e);
    if (rc) return rc;
    if (best_zchunk) *best_zchunk = bz;
    if (best_ctas) *best_ctas = bc;
    if (best_ms) *best_ms = best;
    return PFLBM_OK;
}

int pflbm_ensemble_info(const pflbm_ensemble *e, uint64_t *total_nodes, int32_t *n_boxes, int32_t *n_items) {
    if (!e) return efail(PFLBM_ERR_INVALID_ARG, "null ensemble");
    if (total_nodes) *total_nodes = e->total_nodes;
    if (n_boxes) *n_boxes = int32_t(e->boxes.size());
    if (n_items) *n_items = e->n_items;
    return PFLBM_OK;
}

int pflbm_ensemble_destroy(pflbm_ensemble *e) {
    if (!e) return PFLBM_OK;
    cudaSetDevice(e->device);
    if (e->stream) cudaStreamSynchronize(e->stream);
    delete e;
    return PFLBM_OK;
}

}  // extern "C"
