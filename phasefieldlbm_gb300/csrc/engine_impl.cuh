// engine_impl.cuh - Engine template: owns the device buffers of one
// simulation and launches the kernels of kernels.cuh. Included by one
// translation unit per storage type so the instantiations build in parallel.
#pragma once
#include <cstring>
#include <new>

#include <cstdlib>
#include <type_traits>

#include "engine.h"
#include "kernels.cuh"
#include "kernels_pair.cuh"
#include "kernels_tma.cuh"

namespace pflbm {

template <class T>
Params<T> make_params(const HostParams &h) {
    Params<T> p{};
    const bool f = sizeof(T) == 4;
    p.nx = h.nx; p.ny = h.ny; p.nz = h.nz;
    p.plane = h.nx * h.ny;
    p.N = h.N;
    p.zchunk = h.zchunk;
    // FP32 runs use the float-rounded constants exactly as the reference
    // computes them; FP64 runs use the double values.
    p.sigma = f ? T(h.f_sigma) : T(h.sigma);
    p.gamma = f ? T(h.f_gamma) : T(h.gamma);
    p.u_inf = f ? T(h.f_u_inf) : T(h.u_inf);
    p.omega_ref = f ? T(h.f_omega_ref) : T(h.omega_ref);
    p.tau_water = f ? T(h.f_tau_water) : T(h.tau_water);
    p.tau_oil = f ? T(h.f_tau_oil) : T(h.tau_oil);
    p.visc_water = f ? T(h.f_visc_water) : T(h.visc_water);
    p.visc_oil = f ? T(h.f_visc_oil) : T(h.visc_oil);
    p.kgain1 = f ? T(h.f_kgain1) : T(h.kgain1);
    p.omco_zmin = f ? T(h.f_omco_zmin) : T(h.omco_zmin);
    p.z_start = f ? T(h.f_z_start) : T(h.z_start);
    p.inv_nz_m1 = f ? T(h.f_inv_nz_m1) : T(h.inv_nz_m1);
    p.inv_sponge = f ? T(h.f_inv_sponge) : T(h.inv_sponge);
    p.center_x = f ? T(h.f_center_x) : T(h.center_x);
    p.center_y = f ? T(h.f_center_y) : T(h.center_y);
    p.R2 = f ? T(h.f_R2) : T(h.R2);
    p.g5_in = T(0);
    p.sigma_u = h.sigma_u;
    p.noise_amp = h.noise_amp;
    p.noise_mode = h.noise_mode;
    p.seed = h.seed;
    p.u_inf_f = h.f_u_inf;
    return p;
}

// Tensor maps of the TMA collide kernel for one grid: f as (x, y, z, q) with
// boxes (BWN, TY, 1, 1) for the c_x = 0 directions and (BWW, TY, 1, 1) for
// the others, phi as (x, y, z) with boxes (PBW, PBH, 1). False when the
// driver entry point is missing or the encoder rejects the layout.
template <int QQ, class S, class L = TmaLayout<QQ, S>>
bool encode_collide_maps(const S *f, const typename Store<S>::T *phi, uint64_t nx, uint64_t ny, uint64_t nz,
                         CUtensorMap &fmapn, CUtensorMap &fmapw, CUtensorMap &phimap) {
    using T = typename Store<S>::T;
    using Encode = CUresult (*)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *, const cuuint64_t *,
                                const cuuint64_t *, const cuuint32_t *, const cuuint32_t *, CUtensorMapInterleave,
                                CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);
    void *fn = nullptr;
    cudaDriverEntryPointQueryResult q{};
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q) != cudaSuccess ||
        q != cudaDriverEntryPointSuccess || !fn) {
        cudaGetLastError();
        return false;
    }
    Encode enc = reinterpret_cast<Encode>(fn);
    const CUtensorMapDataType ft = std::is_same<S, float>::value    ? CU_TENSOR_MAP_DATA_TYPE_FLOAT32
                                   : std::is_same<S, double>::value ? CU_TENSOR_MAP_DATA_TYPE_FLOAT64
                                   : std::is_same<S, __half>::value ? CU_TENSOR_MAP_DATA_TYPE_FLOAT16
                                                                    : CU_TENSOR_MAP_DATA_TYPE_BFLOAT16;
    const CUtensorMapDataType pt = sizeof(T) == 8 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT64 : CU_TENSOR_MAP_DATA_TYPE_FLOAT32;
    const uint64_t N = nx * ny * nz;
    const cuuint64_t fdim[4] = {nx, ny, nz, cuuint64_t(QQ)};
    const cuuint64_t fstr[3] = {nx * sizeof(S), nx * ny * sizeof(S), N * sizeof(S)};
    // boxes of the layout's tile: the TMA writes exactly what L's shared-memory
    // plan and transaction count expect
    const cuuint32_t fboxn[4] = {cuuint32_t(L::BWN), cuuint32_t(L::TY), 1, 1};
    const cuuint32_t fboxw[4] = {cuuint32_t(L::BWW), cuuint32_t(L::TY), 1, 1};
    const cuuint32_t one4[4] = {1, 1, 1, 1};
    for (int k = 0; k < 2; ++k)
        if (enc(k ? &fmapw : &fmapn, ft, 4, const_cast<S *>(f), fdim, fstr, k ? fboxw : fboxn, one4,
                CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
            return false;
    const cuuint64_t pdim[3] = {nx, ny, nz};
    const cuuint64_t pstr[2] = {nx * sizeof(T), nx * ny * sizeof(T)};
    const cuuint32_t pbox[3] = {cuuint32_t(L::PBW), cuuint32_t(L::PBH), 1};
    return enc(&phimap, pt, 3, const_cast<T *>(phi), pdim, pstr, pbox, one4, CU_TENSOR_MAP_INTERLEAVE_NONE,
               CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
               CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

template <int QQ, bool JET, class S>
class EngineT final : public Engine {
    using T = typename Store<S>::T;

   public:
    EngineT(const HostParams &h, uint32_t flags) : h_(h), flags_(flags) { p_ = make_params<T>(h); }
    ~EngineT() override { free_all(); }

    int allocate(std::string &err) override {
        const uint64_t N = h_.N, plane = uint64_t(h_.nx) * h_.ny;
        struct Req {
            void **ptr;
            size_t bytes;
        };
        Req reqs[] = {
            {reinterpret_cast<void **>(&f_[0]), sizeof(S) * QQ * N},
            {reinterpret_cast<void **>(&f_[1]), sizeof(S) * QQ * N},
            {reinterpret_cast<void **>(&phi_[0]), sizeof(T) * N},
            {reinterpret_cast<void **>(&phi_[1]), sizeof(T) * N},
            {reinterpret_cast<void **>(&j_), sizeof(T) * 3 * N},
            {reinterpret_cast<void **>(&top_), sizeof(T) * 22 * plane},
            {reinterpret_cast<void **>(&macro_), sizeof(T) * M_COUNT * N},
            {reinterpret_cast<void **>(&counters_), sizeof(unsigned long long) * 2},
            {reinterpret_cast<void **>(&err_), sizeof(unsigned int) * 4},
            {reinterpret_cast<void **>(&partial_), sizeof(double) * RED_FIELDS * kRedBlocks},
        };
        // fault injection on the host: PFLBM_ALLOC_LIMIT_BYTES caps the
        // device bytes one simulation may take (allocation fails cleanly)
        uint64_t planned = 0;
        for (auto &r : reqs) planned += r.bytes;
        if (flags_ & (PFLBM_FLAG_TIME_AVERAGE | PFLBM_FLAG_REYNOLDS_MOMENTS)) planned += sizeof(T) * 10 * N;
        if (flags_ & PFLBM_FLAG_VORTICITY) planned += sizeof(T) * 4 * N;
        if (const char *lim = std::getenv("PFLBM_ALLOC_LIMIT_BYTES")) {
            const unsigned long long cap = std::strtoull(lim, nullptr, 10);
            if (cap > 0 && planned > cap) {
                err = "device allocation of " + std::to_string(planned) + " bytes exceeds PFLBM_ALLOC_LIMIT_BYTES=" +
                      std::to_string(cap);
                return PFLBM_ERR_OUT_OF_MEMORY;
            }
        }
        for (auto &r : reqs) {
            if (cudaMalloc(r.ptr, r.bytes) != cudaSuccess) {
                cudaGetLastError();
                err = "cudaMalloc failed (" + std::to_string(r.bytes) + " bytes)";
                free_all();
                return PFLBM_ERR_OUT_OF_MEMORY;
            }
            cudaMemset(*r.ptr, 0, r.bytes);
            bytes_ += r.bytes;
        }
        if (flags_ & (PFLBM_FLAG_TIME_AVERAGE | PFLBM_FLAG_REYNOLDS_MOMENTS)) {
            if (cudaMalloc(&avg_, sizeof(T) * 10 * N) != cudaSuccess) {
                cudaGetLastError();
                err = "cudaMalloc failed (averages)";
                free_all();
                return PFLBM_ERR_OUT_OF_MEMORY;
            }
            cudaMemset(avg_, 0, sizeof(T) * 10 * N);
            bytes_ += sizeof(T) * 10 * N;
        }
        if (flags_ & PFLBM_FLAG_VORTICITY) {
            if (cudaMalloc(&vort_, sizeof(T) * 4 * N) != cudaSuccess) {
                cudaGetLastError();
                err = "cudaMalloc failed (vorticity)";
                free_all();
                return PFLBM_ERR_OUT_OF_MEMORY;
            }
            cudaMemset(vort_, 0, sizeof(T) * 4 * N);
            bytes_ += sizeof(T) * 4 * N;
        }
        if (cudaDeviceSynchronize() != cudaSuccess) {
            err = cudaGetErrorString(cudaGetLastError());
            return PFLBM_ERR_CUDA;
        }
        setup_tma();
        return PFLBM_OK;
    }

    // The TMA collide kernel needs 16-byte aligned row strides; otherwise the
    // plain-load kernel is used. PFLBM_NO_TMA=1 forces the plain kernel.
    void setup_tma() {
        use_tma_ = false;
        if (const char *e = std::getenv("PFLBM_NO_VEC")) no_vec_ = e[0] == '1';
        if (const char *e = std::getenv("PFLBM_NO_TMA"))
            if (e[0] == '1') return;
        if ((uint64_t(h_.nx) * sizeof(S)) % 16 != 0 || (uint64_t(h_.nx) * sizeof(T)) % 16 != 0) return;
        using L = TmaLayout<QQ, S>;
        for (int k = 0; k < 2; ++k)
            if (!encode_collide_maps<QQ, S>(f_[k], phi_[k], h_.nx, h_.ny, h_.nz, fmapn_[k], fmapw_[k], phimap_[k]))
                return;
        if (cudaFuncSetAttribute(k_collide_tma<QQ, JET, S, MODE_STEP>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 int(L::total)) != cudaSuccess ||
            cudaFuncSetAttribute(k_collide_tma<QQ, JET, S, MODE_STEP_AVG>,
                                 cudaFuncAttributeMaxDynamicSharedMemorySize, int(L::total)) != cudaSuccess) {
            cudaGetLastError();
            return;
        }
        use_tma_ = true;
        // the closure modes on the TMA kernel (network after the pipeline's
        // shared memory); without room they stay on the plain-load kernel
        tma_closure_ = false;
        if constexpr (sizeof(S) >= 4) {
            const int smc = int(TmaModeLayout<QQ, S, MODE_STEP_CLOSURE>::total + closure_smem_bytes<T>());
            tma_closure_ = cudaFuncSetAttribute(k_collide_tma<QQ, JET, S, MODE_STEP_CLOSURE>,
                                                cudaFuncAttributeMaxDynamicSharedMemorySize, smc) == cudaSuccess &&
                           cudaFuncSetAttribute(k_collide_tma<QQ, JET, S, MODE_STEP_CLOSURE_AVG>,
                                                cudaFuncAttributeMaxDynamicSharedMemorySize, smc) == cudaSuccess;
            if (!tma_closure_) cudaGetLastError();
        }
        // two nodes per thread with packed FP32x2 arithmetic for the plain
        // step of 16-bit D3Q19 storage, whose collide is issue-bound (FP32
        // and D3Q27 stay faster with one node per thread and twice the
        // warps). PFLBM_NO_PAIR=1 keeps one node per thread; PFLBM_PAIR=1
        // selects the pair kernel for every FP32/16-bit lattice (tests).
        use_pair_ = false;
        if constexpr (sizeof(T) == 4) {
            const char *no = std::getenv("PFLBM_NO_PAIR");
            const char *force = std::getenv("PFLBM_PAIR");
            const bool want = (force && force[0] == '1') || (sizeof(S) == 2 && QQ == 19);
            if (want && !(no && no[0] == '1') && h_.nx % 2 == 0) {
                if (cudaFuncSetAttribute(k_collide_pair<QQ, JET, S>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         int(PairLayout<QQ, S>::total)) == cudaSuccess)
                    use_pair_ = true;
                else
                    cudaGetLastError();
            }
        }
    }

    void free_all() override {
        void *ptrs[] = {f_[0], f_[1], phi_[0], phi_[1], j_, top_, macro_, counters_, partial_, avg_, vort_, err_, mlp_};
        for (void *q : ptrs)
            if (q) cudaFree(q);
        mlp_ = nullptr;
        closure_ = false;
        f_[0] = f_[1] = nullptr;
        phi_[0] = phi_[1] = nullptr;
        j_ = top_ = macro_ = avg_ = vort_ = nullptr;
        counters_ = nullptr;
        partial_ = nullptr;
        err_ = nullptr;
        bytes_ = 0;
    }

    StepBuffers<S, T> buffers(int parity) const {
        StepBuffers<S, T> b{};
        b.f_src = f_[parity];
        b.f_dst = f_[parity ^ 1];
        b.phi_src = phi_[parity];
        b.phi_dst = phi_[parity ^ 1];
        b.jflux = j_;
        b.top = top_;
        b.step_in = counters_ + parity;
        b.step_out = counters_ + (parity ^ 1);
        b.t_fixed = 0;
        b.avg = avg_;
        b.macro = macro_;
        b.err = err_;
        b.mlp = mlp_;
        return b;
    }

    dim3 collide_grid() const {
        const int nzi = int(h_.nz) - 2;
        const int chunks = (nzi + p_.zchunk - 1) / p_.zchunk;
        return dim3((h_.nx + TX - 1) / TX, (h_.ny + TY - 1) / TY, chunks);
    }
    dim3 node_block() const { return dim3(32, 8, 1); }
    dim3 node_grid() const { return dim3((h_.nx + 31) / 32, (h_.ny + 7) / 8, h_.nz); }

    void enqueue_step(int parity, cudaStream_t s, cudaEvent_t *ev) override {
        const StepBuffers<S, T> b = buffers(parity);
        if (ev) cudaEventRecord(ev[0], s);
        if (closure_) {
            // learned closure: the network in shared memory
            if constexpr (sizeof(S) >= 4) {
                const size_t smc = TmaModeLayout<QQ, S, MODE_STEP_CLOSURE>::total + closure_smem_bytes<T>();
                if (use_tma_ && tma_closure_ && avg_)
                    k_collide_tma<QQ, JET, S, MODE_STEP_CLOSURE_AVG>
                        <<<collide_grid(), dim3(TX, TY, 1), smc, s>>>(p_, b, fmapn_[parity], fmapw_[parity], phimap_[parity]);
                else if (use_tma_ && tma_closure_)
                    k_collide_tma<QQ, JET, S, MODE_STEP_CLOSURE>
                        <<<collide_grid(), dim3(TX, TY, 1), smc, s>>>(p_, b, fmapn_[parity], fmapw_[parity], phimap_[parity]);
                else if (avg_)
                    k_collide<QQ, JET, S, MODE_STEP_CLOSURE_AVG><<<collide_grid(), dim3(TX, TY, 1), 0, s>>>(p_, b);
                else
                    k_collide<QQ, JET, S, MODE_STEP_CLOSURE><<<collide_grid(), dim3(TX, TY, 1), 0, s>>>(p_, b);
            }
        } else if (use_tma_) {
            const size_t sm = TmaLayout<QQ, S>::total;
            if (avg_) {
                k_collide_tma<QQ, JET, S, MODE_STEP_AVG>
                    <<<collide_grid(), dim3(TX, TY, 1), sm, s>>>(p_, b, fmapn_[parity], fmapw_[parity], phimap_[parity]);
            } else if (use_pair_) {
                if constexpr (sizeof(T) == 4)
                    k_collide_pair<QQ, JET, S><<<collide_grid(), dim3(TX2, TY, 1), PairLayout<QQ, S>::total, s>>>(
                        p_, b, fmapn_[parity], fmapw_[parity], phimap_[parity]);
            } else {
                k_collide_tma<QQ, JET, S, MODE_STEP>
                    <<<collide_grid(), dim3(TX, TY, 1), sm, s>>>(p_, b, fmapn_[parity], fmapw_[parity], phimap_[parity]);
            }
        } else if (avg_) {
            k_collide<QQ, JET, S, MODE_STEP_AVG><<<collide_grid(), dim3(TX, TY, 1), 0, s>>>(p_, b);
        } else {
            k_collide<QQ, JET, S, MODE_STEP><<<collide_grid(), dim3(TX, TY, 1), 0, s>>>(p_, b);
        }
        if (ev) cudaEventRecord(ev[1], s);
        if (ev) cudaEventRecord(ev[2], s);
        if constexpr (std::is_same<T, float>::value) {
            if (h_.nx % 4 == 0 && !no_vec_) {
                const dim3 g4((h_.nx / 4 + 31) / 32, (h_.ny + 7) / 8, JET ? h_.nz + 4 : h_.nz);
                k_phase_v4<QQ, JET, S><<<g4, node_block(), 0, s>>>(p_, b);
            } else {
                k_phase<QQ, JET, S><<<node_grid(), node_block(), 0, s>>>(p_, b);
            }
        } else {
            k_phase<QQ, JET, S><<<node_grid(), node_block(), 0, s>>>(p_, b);
        }
        if (ev) cudaEventRecord(ev[3], s);
    }

    InitGeom geom() const {
        InitGeom g{};
        g.jet = JET ? 1 : 0;
        g.droplet_x_stretch = h_.droplet_x_stretch;
        g.center_z = sizeof(T) == 4 ? h_.f_center_z : float(h_.center_z);
        g.radius = h_.radius;
        g.interface_width = h_.interface_width;
        g.init_noise = h_.init_noise;
        return g;
    }

    void enqueue_init_fields(cudaStream_t s) override {
        InitGeom g = geom();
        k_init_fields<T><<<node_grid(), node_block(), 0, s>>>(p_, g, macro_);
    }
    void enqueue_init_distros(cudaStream_t s) override {
        k_init_distros<QQ, JET, S><<<node_grid(), node_block(), 0, s>>>(p_, f_[0], f_[1], phi_[0], phi_[1], macro_);
        if (avg_) cudaMemsetAsync(avg_, 0, sizeof(T) * 10 * h_.N, s);
    }
    void enqueue_analysis(int parity, uint32_t t, cudaStream_t s) override {
        StepBuffers<S, T> b = buffers(parity);
        b.f_dst = nullptr;
        b.phi_dst = nullptr;
        b.step_in = nullptr;
        b.step_out = nullptr;
        b.t_fixed = t;
        k_collide<QQ, JET, S, MODE_ANALYSIS><<<collide_grid(), dim3(TX, TY, 1), 0, s>>>(p_, b);
        k_analysis_ghosts<T><<<node_grid(), node_block(), 0, s>>>(p_, JET ? 1 : 0, t, macro_);
    }
    void enqueue_vorticity(cudaStream_t s) override {
        if (vort_) k_vorticity<T><<<node_grid(), node_block(), 0, s>>>(p_, macro_, vort_);
    }
    void enqueue_reduce(cudaStream_t s, double *dev_out) override {
        k_reduce_partial<T><<<kRedBlocks, RED_THREADS, 0, s>>>(p_, macro_, partial_);
        k_reduce_final<<<1, 32, 0, s>>>(partial_, kRedBlocks, dev_out);
    }
    void reset_counters(cudaStream_t s) override {
        cudaMemsetAsync(counters_, 0, sizeof(unsigned long long) * 2, s);
        cudaMemsetAsync(err_, 0, sizeof(unsigned int) * 4, s);
    }
    unsigned int *error_word() override { return err_; }
    void *f_ptr(int k) override { return f_[k]; }
    void *phi_ptr(int k) override { return phi_[k]; }
    uint64_t f_bytes() const override { return sizeof(S) * QQ * h_.N; }
    uint64_t phi_bytes() const override { return sizeof(T) * h_.N; }
    uint64_t avg_bytes() const override { return avg_ ? sizeof(T) * 10 * h_.N : 0; }
    void set_counter(int parity, unsigned long long value, cudaStream_t s) override {
        cudaMemcpyAsync(counters_ + parity, &value, sizeof value, cudaMemcpyHostToDevice, s);
        cudaStreamSynchronize(s);
    }
    bool uses_tma() const override { return use_tma_; }
    int collide_variant() const override { return use_pair_ ? 2 : (use_tma_ ? 1 : 0); }
    int real_bytes() const override { return int(sizeof(T)); }
    void *macro_ptr() override { return macro_; }
    void *avg_ptr() override { return avg_; }
    void *vort_ptr() override { return vort_; }
    uint64_t device_bytes() const override { return bytes_; }
    int kernels_per_step() const override { return 2; }
    int set_closure(const float *host_blob, std::string &err) override {
        if constexpr (sizeof(S) < 4) {
            err = "the learned closure needs FP32 or FP64 storage";
            return PFLBM_ERR_UNSUPPORTED;
        } else {
            if (!host_blob) {
                closure_ = false;
                return PFLBM_OK;
            }
            if (!mlp_) {
                if (cudaMalloc(&mlp_, sizeof(float) * kMlpDeviceFloats) != cudaSuccess) {
                    cudaGetLastError();
                    err = "cudaMalloc failed (closure network)";
                    return PFLBM_ERR_OUT_OF_MEMORY;
                }
                bytes_ += sizeof(float) * kMlpDeviceFloats;
                cudaMemset(mlp_, 0, sizeof(float) * kMlpDeviceFloats);  // phase mixing off
            }
            if (cudaMemcpy(mlp_, host_blob, sizeof(float) * kMlpBlob, cudaMemcpyHostToDevice) != cudaSuccess) {
                err = cudaGetErrorString(cudaGetLastError());
                return PFLBM_ERR_CUDA;
            }
            closure_ = true;
            return PFLBM_OK;
        }
    }
    bool has_closure() const override { return closure_; }
    int set_closure_mixing(float inv_schmidt, std::string &err) override {
        if (!closure_ || !mlp_) {
            err = "attach a closure (pflbm_set_closure) before its phase mixing";
            return PFLBM_ERR_STATE;
        }
        if (cudaMemcpy(mlp_ + kMlpPhaseMix, &inv_schmidt, sizeof(float), cudaMemcpyHostToDevice) != cudaSuccess) {
            err = cudaGetErrorString(cudaGetLastError());
            return PFLBM_ERR_CUDA;
        }
        return PFLBM_OK;
    }

   private:
    static constexpr int kRedBlocks = 608;
    HostParams h_;
    uint32_t flags_;
    Params<T> p_;
    S *f_[2] = {nullptr, nullptr};
    T *phi_[2] = {nullptr, nullptr};
    T *j_ = nullptr, *top_ = nullptr, *macro_ = nullptr, *avg_ = nullptr, *vort_ = nullptr;
    unsigned long long *counters_ = nullptr;
    double *partial_ = nullptr;
    unsigned int *err_ = nullptr;
    bool use_tma_ = false;
    bool use_pair_ = false;  // k_collide_pair for the plain step
    bool tma_closure_ = false;  // closure modes on k_collide_tma
    bool no_vec_ = false;  // PFLBM_NO_VEC=1: scalar phase kernel
    float *mlp_ = nullptr;  // closure network blob (kMlpBlob floats) + phase mixing (1 float)
    bool closure_ = false;
    CUtensorMap fmapn_[2]{}, fmapw_[2]{}, phimap_[2]{};
    uint64_t bytes_ = 0;
};

template <class S>
Engine *make_engine_t(int q, bool jet, const HostParams &hp, uint32_t flags) {
    if (q == 19 && !jet) return new (std::nothrow) EngineT<19, false, S>(hp, flags);
    if (q == 19 && jet) return new (std::nothrow) EngineT<19, true, S>(hp, flags);
    if (q == 27 && !jet) return new (std::nothrow) EngineT<27, false, S>(hp, flags);
    if (q == 27 && jet) return new (std::nothrow) EngineT<27, true, S>(hp, flags);
    return nullptr;
}

}  // namespace pflbm
