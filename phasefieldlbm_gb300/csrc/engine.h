// engine.h - host-side interface between the C ABI (api.cu) and the
// per-storage kernel instantiations (engine_*.cu).
#pragma once
#include <cuda_runtime.h>

#include <cstdint>
#include <string>

#include "../../include/pflbm.h"

namespace pflbm {

// Host copy of the derived constants, both precisions (see params.cuh).
struct HostParams {
    uint32_t nx, ny, nz;
    uint64_t N;
    int32_t zchunk;
    double sigma, gamma, u_inf, omega_ref;
    double tau_water, tau_oil, visc_water, visc_oil, kgain1, omco_zmin;
    double z_start, inv_nz_m1, inv_sponge;
    double center_x, center_y, center_z, R2;
    float f_sigma, f_gamma, f_u_inf, f_omega_ref;
    float f_tau_water, f_tau_oil, f_visc_water, f_visc_oil, f_kgain1, f_omco_zmin;
    float f_z_start, f_inv_nz_m1, f_inv_sponge;
    float f_center_x, f_center_y, f_center_z, f_R2;
    float sigma_u, noise_amp;
    int32_t noise_mode;
    uint32_t seed;
    int32_t jet;
    float droplet_x_stretch;
    int32_t radius;
    float interface_width;
    float init_noise;
};

class Engine {
   public:
    virtual ~Engine() = default;
    // Allocates device memory; returns a pflbm_status.
    virtual int allocate(std::string &err) = 0;
    virtual void free_all() = 0;
    // Enqueues one time step reading ping-pong buffer `parity`. With
    // events (2 per kernel) the kernels are bracketed by event records.
    virtual void enqueue_step(int parity, cudaStream_t s, cudaEvent_t *events = nullptr) = 0;
    // Initial macroscopic fields into the cache, then f/phi from them.
    virtual void enqueue_init_fields(cudaStream_t s) = 0;
    virtual void enqueue_init_distros(cudaStream_t s) = 0;
    // Rebuilds the reference's arrays after step t from ping-pong `parity`.
    virtual void enqueue_analysis(int parity, uint32_t t, cudaStream_t s) = 0;
    virtual void enqueue_vorticity(cudaStream_t s) = 0;
    // FP64 diagnostics of the cache into out[12] (device pointer).
    virtual void enqueue_reduce(cudaStream_t s, double *dev_out) = 0;
    virtual void reset_counters(cudaStream_t s) = 0;
    // Element size of the arithmetic type (4 or 8).
    virtual int real_bytes() const = 0;
    virtual void *macro_ptr() = 0;  // 18*N reals
    virtual void *avg_ptr() = 0;    // 10*N reals or null
    virtual void *vort_ptr() = 0;   // 4*N reals or null
    virtual uint64_t device_bytes() const = 0;
    // Raw state buffers for checkpoints.
    virtual void *f_ptr(int k) = 0;
    virtual void *phi_ptr(int k) = 0;
    virtual uint64_t f_bytes() const = 0;
    virtual uint64_t phi_bytes() const = 0;
    virtual uint64_t avg_bytes() const = 0;
    virtual void set_counter(int parity, unsigned long long value, cudaStream_t s) = 0;
    // Device word that kernels set when a bounded wait gave up (0 = fine).
    virtual unsigned int *error_word() = 0;
    // True when the TMA-fed collide kernel is in use.
    virtual bool uses_tma() const = 0;
    virtual int collide_variant() const = 0;  // pflbm_collide_variant_t
    virtual int kernels_per_step() const = 0;
    // Learned closure: copies the network blob (kMlpBlob floats, host) to the
    // device and switches the collide kernel to the closure mode; null
    // detaches. PFLBM_ERR_UNSUPPORTED for 16-bit storage.
    virtual int set_closure(const float *host_blob, std::string &err) = 0;
    // Inverse turbulent Schmidt number of the closure's phase mixing (the
    // device word after the blob); needs a closure attached.
    virtual int set_closure_mixing(float inv_schmidt, std::string &err) = 0;
    virtual bool has_closure() const = 0;
};

// Device view of a simulation's macroscopic fields (analysis cache brought
// up to date and synchronised) for the closure's training-data kernels.
// Closure network blob: kMlpParamFloats weights, then mean[8],
// inv_scale[8], out_scale, strength (kernels.cuh kMlp* offsets).
constexpr int kMlpParamFloats = 1377, kMlpBlobFloats = 1395;

struct SimView {
    const void *macro;  // 18*N reals, pflbm_field_id order
    int real_bytes;
    uint32_t nx, ny, nz;
    uint64_t N;
    int device;
    double tau_water, tau_oil;
};
int sim_view(pflbm_sim *s, SimView &v);

// api.cu: derived constants, validation and the thread-local error message.
void derive(const pflbm_config &c, HostParams &h);
int validate(const pflbm_config &c);
void set_error(const std::string &msg);

Engine *make_engine_fp32(int q, bool jet, const HostParams &hp, uint32_t flags);
Engine *make_engine_fp64(int q, bool jet, const HostParams &hp, uint32_t flags);
Engine *make_engine_fp16(int q, bool jet, const HostParams &hp, uint32_t flags);
Engine *make_engine_bf16(int q, bool jet, const HostParams &hp, uint32_t flags);

}  // namespace pflbm
