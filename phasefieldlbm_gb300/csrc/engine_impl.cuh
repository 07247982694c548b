// engine_impl.cuh - Engine template: owns the device buffers of one
// simulation and launches the kernels of kernels.cuh. Included by one
// translation unit per storage type so the instantiations build in parallel.
#pragma once
#include <cstring>
#include <new>

#include "engine.h"
#include "kernels.cuh"

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
            {reinterpret_cast<void **>(&partial_), sizeof(double) * RED_FIELDS * kRedBlocks},
        };
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
        return PFLBM_OK;
    }

    void free_all() override {
        void *ptrs[] = {f_[0], f_[1], phi_[0], phi_[1], j_, top_, macro_, counters_, partial_, avg_, vort_};
        for (void *q : ptrs)
            if (q) cudaFree(q);
        f_[0] = f_[1] = nullptr;
        phi_[0] = phi_[1] = nullptr;
        j_ = top_ = macro_ = avg_ = vort_ = nullptr;
        counters_ = nullptr;
        partial_ = nullptr;
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
        b.err = nullptr;
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
        if (avg_)
            k_collide<QQ, JET, S, MODE_STEP_AVG><<<collide_grid(), dim3(TX, TY, 1), 0, s>>>(p_, b);
        else
            k_collide<QQ, JET, S, MODE_STEP><<<collide_grid(), dim3(TX, TY, 1), 0, s>>>(p_, b);
        if (ev) cudaEventRecord(ev[1], s);
        if (ev) cudaEventRecord(ev[2], s);
        k_phase<QQ, JET, S><<<node_grid(), node_block(), 0, s>>>(p_, b);
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
    }
    int real_bytes() const override { return int(sizeof(T)); }
    void *macro_ptr() override { return macro_; }
    void *avg_ptr() override { return avg_; }
    void *vort_ptr() override { return vort_; }
    uint64_t device_bytes() const override { return bytes_; }
    int kernels_per_step() const override { return 2; }

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
