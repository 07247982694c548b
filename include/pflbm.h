/*
 * pflbm.h - C ABI of the GB300-native phase-field lattice-Boltzmann hot path.
 *
 * The reference (phaseFieldLBM) has no plugin or FFI layer: its seam is the
 * kernel set declared in src/LBMIncludes.cuh:121-136, driven by the time loop
 * in src/main.cu:163-188 and specialised at compile time by -DVS_<set> and
 * -D<CASE> (src/constants.cuh:39-49). This header replaces that seam with a
 * runtime-configured C interface: every compile-time constant of
 * src/constants.cuh:80-143 becomes a field of pflbm_config, and the kernels of
 * src/phaseField.cuh, src/lbm.cu, src/BoundaryConditions.cuh,
 * src/initialConditions.cu and src/derivedFields/ sit behind pflbm_init /
 * pflbm_step / pflbm_get_field.
 *
 * Conventions
 *   - Every function returns an int status (PFLBM_OK == 0). On failure a
 *     thread-local message is available from pflbm_last_error(). Nothing
 *     aborts or traps (the reference calls std::abort, src/cuda/errorCheck.cuh:36-42).
 *   - The library owns all device memory; callers own host buffers.
 *   - One simulation handle must not be used from two threads at once.
 *   - Fields are SoA, x fastest: index = x + nx*(y + ny*z), as
 *     src/functions/deviceFunctions.cuh:33-39. The outer one-node shell is a
 *     ghost layer exactly as in the reference (guard, deviceFunctions.cuh:50-61).
 */
#ifndef PFLBM_H
#define PFLBM_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define PFLBM_ABI_VERSION 1

/* ---- status codes ---------------------------------------------------- */
enum pflbm_status {
    PFLBM_OK = 0,
    PFLBM_ERR_INVALID_ARG = 1,   /* bad pointer, size or config value        */
    PFLBM_ERR_CUDA = 2,          /* a CUDA runtime call failed               */
    PFLBM_ERR_OUT_OF_MEMORY = 3, /* device allocation failed                 */
    PFLBM_ERR_STATE = 4,         /* call out of order (e.g. step before init)*/
    PFLBM_ERR_DIVERGED = 5,      /* NaN/Inf found by the diagnostics         */
    PFLBM_ERR_UNSUPPORTED = 6,   /* feature not available in this build      */
    PFLBM_ERR_IO = 7,            /* file output failed                       */
    PFLBM_ERR_DEVICE = 8         /* a kernel reported an error flag          */
};

/* ---- selectors (src/constants.cuh:39-55, src/cuda/precision.cuh:26-56) - */
enum pflbm_flow_case { PFLBM_CASE_DROPLET = 0, PFLBM_CASE_JET = 1 };
enum pflbm_velocity_set { PFLBM_VS_D3Q19 = 19, PFLBM_VS_D3Q27 = 27 };
enum pflbm_storage {
    PFLBM_STORAGE_FP32 = 0, /* plain path: f, g stored FP32                       */
    PFLBM_STORAGE_FP16 = 1, /* f as scaled (f_i - w_i)/w_i in FP16, phase flux FP16 */
    PFLBM_STORAGE_BF16 = 2, /* same layout in BF16                                */
    PFLBM_STORAGE_FP64 = 3  /* all arithmetic and storage FP64 (error oracle run) */
};
enum pflbm_inflow_noise {
    PFLBM_NOISE_GAUSSIAN_UXY = 0, /* reference: Box-Muller on ux,uy, sd = amp*u_inf
                                     (src/BoundaryConditions.cuh:58-69)          */
    PFLBM_NOISE_UNIFORM_UZ = 1    /* uz = u_inf*(1 + amp*xi), xi ~ U[-1,1) from the
                                     same counter hash, salted by seed           */
};

/* Optional per-step derived fields (src/derivedFields/DerivedFields.cuh:172-199). */
enum pflbm_flags {
    PFLBM_FLAG_TIME_AVERAGE = 1u << 0,    /* avg_phi, avg_ux, avg_uy, avg_uz        */
    PFLBM_FLAG_REYNOLDS_MOMENTS = 1u << 1,/* avg_uxux ... avg_uyuz                  */
    PFLBM_FLAG_VORTICITY = 1u << 2        /* vort_x/y/z/mag (computed on demand)    */
};

/* Field identifiers: same order as host::FieldID (src/fileIO/fields.cuh:33-68). */
enum pflbm_field_id {
    PFLBM_FIELD_RHO = 0, PFLBM_FIELD_UX, PFLBM_FIELD_UY, PFLBM_FIELD_UZ,
    PFLBM_FIELD_PXX, PFLBM_FIELD_PYY, PFLBM_FIELD_PZZ,
    PFLBM_FIELD_PXY, PFLBM_FIELD_PXZ, PFLBM_FIELD_PYZ,
    PFLBM_FIELD_PHI = 10, PFLBM_FIELD_NORMX, PFLBM_FIELD_NORMY, PFLBM_FIELD_NORMZ,
    PFLBM_FIELD_IND, PFLBM_FIELD_FFX = 15, PFLBM_FIELD_FFY, PFLBM_FIELD_FFZ,
    PFLBM_FIELD_AVG_PHI = 18, PFLBM_FIELD_AVG_UX, PFLBM_FIELD_AVG_UY, PFLBM_FIELD_AVG_UZ,
    PFLBM_FIELD_AVG_UXUX = 22, PFLBM_FIELD_AVG_UYUY, PFLBM_FIELD_AVG_UZUZ,
    PFLBM_FIELD_AVG_UXUY, PFLBM_FIELD_AVG_UXUZ, PFLBM_FIELD_AVG_UYUZ,
    PFLBM_FIELD_VORT_X = 28, PFLBM_FIELD_VORT_Y, PFLBM_FIELD_VORT_Z, PFLBM_FIELD_VORT_MAG,
    PFLBM_FIELD_C = 32, /* passive scalar: not built (the reference's is a trap stub) */
    PFLBM_FIELD_COUNT = 33
};

/*
 * Run-time configuration. Replaces the compile-time namespaces mesh::,
 * physics::, relaxation:: and sponge:: (src/constants.cuh:80-143,
 * src/functions/globalFunctions.cuh:260-461). pflbm_config_reference() fills
 * it with the reference's own compile-time values.
 */
typedef struct pflbm_config {
    uint32_t struct_size;      /* = sizeof(pflbm_config); checked by pflbm_create  */
    int32_t flow_case;         /* pflbm_flow_case                                  */
    int32_t velocity_set;      /* pflbm_velocity_set (hydrodynamics; phase is D3Q7) */
    int32_t storage;           /* pflbm_storage                                    */
    uint32_t nx, ny, nz;       /* mesh::nx/ny/nz, ghost shell included             */
    int32_t radius;            /* mesh::radius: droplet radius / jet inlet radius  */
    int32_t diam;              /* mesh::diam: jet inlet diameter (viscosity scale) */
    float droplet_x_stretch;   /* droplet IC divides (x - cx) by this; the reference
                                  uses 2 (ellipsoid, src/initialConditions.cu:74)  */
    float center_offset[3];    /* droplet centre offset from ((n-1)/2, ...)        */
    float u_inf;               /* physics::u_inf                                   */
    float reynolds_water;      /* physics::reynolds_water (jet)                    */
    float reynolds_oil;        /* physics::reynolds_oil (jet)                      */
    float sigma;               /* surface tension coefficient                      */
    float interface_width;     /* physics::interface_width                         */
    float gamma;               /* sharpening coefficient in gamma*phi*(1-phi)       */
    float tau;                 /* droplet relaxation time (physics::tau)           */
    float sponge_gain;         /* sponge::K_gain (jet outflow sponge)              */
    int32_t sponge_cells;      /* sponge thickness; < 0 means nz/12                 */
    int32_t inflow_noise;      /* pflbm_inflow_noise                               */
    float noise_amp;           /* 0.08 for the reference's Gaussian mode           */
    uint32_t seed;             /* salt of the uniform inflow / initial noise       */
    float init_noise;          /* +-amplitude of seeded uniform initial velocity   */
    uint32_t flags;            /* pflbm_flags                                      */
    int32_t device;            /* CUDA device; < 0: $GPU_INDEX or 0 (hostFunctions.cuh:117-150) */
} pflbm_config;

/* FP64 diagnostics over the interior nodes (the ghost shell is excluded). */
typedef struct pflbm_diag {
    uint64_t step;             /* number of completed steps                        */
    double phi_mass;           /* sum phi                                          */
    double rho_mass;           /* sum rho                                          */
    double momentum[3];        /* sum rho*u                                        */
    double max_speed;          /* max |u|                                          */
    double rho_in, rho_out;    /* mean rho where phi > 0.9 / phi < 0.1             */
    double laplace_dp;         /* cs2 * (rho_in - rho_out)                         */
    uint64_t n_in, n_out;      /* node counts of the two classes                   */
    uint64_t nonfinite;        /* count of NaN/Inf among rho, u, phi               */
} pflbm_diag;

typedef struct pflbm_sim pflbm_sim;

/* Library identity. */
int pflbm_abi_version(void);
const char *pflbm_last_error(void);

/* Fills cfg with the reference's compile-time defaults for (flow_case,
 * velocity_set): src/constants.cuh:80-141 (JET 64x64x128, D=10, Re=We-scaled
 * sigma; DROPLET 128^3, R=35, tau=0.55, sigma=0.03), gamma from
 * src/constants.cuh:104-108, sponge from globalFunctions.cuh:260-292. */
int pflbm_config_reference(pflbm_config *cfg, int32_t flow_case, int32_t velocity_set);

/* Allocates every device field (src/fieldAllocate/FieldAllocate.cuh:47-66
 * plus src/main.cu:56-79) and captures the per-step CUDA graph
 * (src/cuda/CUDAGraph.cuh:35-58). */
int pflbm_create(const pflbm_config *cfg, pflbm_sim **out);

/* Initial conditions: setInitialDensity, setJet|setDroplet, setDistros
 * (src/initialConditions.cu:33-138, src/main.cu:114-116). Resets the step
 * counter and the derived-field averages. */
int pflbm_init(pflbm_sim *sim);

/* Overrides the initial rho, phi or velocity (field id RHO, PHI, UX, UY or
 * UZ) with a host array of nx*ny*nz floats. f and the phase field are
 * rebuilt from the equilibria (as setDistros does) before the next step.
 * Valid only at step 0. */
int pflbm_set_initial_field(pflbm_sim *sim, int32_t field_id, const float *host_src, size_t bytes);

/* Advances nsteps time steps: one body of src/main.cu:163-176 each
 * (graph, boundary conditions, derived fields), without a host sync per step.
 * Returns after the device has finished. */
int pflbm_step(pflbm_sim *sim, uint64_t nsteps);

/* Same as pflbm_step but only enqueues the work on the simulation's stream. */
int pflbm_step_async(pflbm_sim *sim, uint64_t nsteps);
int pflbm_synchronize(pflbm_sim *sim);

/* Runs nsteps time steps with every kernel launched on its own (no graph)
 * between a pair of CUDA events on the simulation's stream. total_ms gets
 * the elapsed time from the first to the last event; kernel_ms[k] gets the
 * summed duration of kernel k of the step (0 = collide, 1 = phase) for
 * k < n_kernels. Used for the roofline measurement; results are identical
 * to pflbm_step. */
int pflbm_step_profiled(pflbm_sim *sim, uint64_t nsteps, double *total_ms, double *kernel_ms, int32_t n_kernels);

/* Number of completed steps. */
int pflbm_current_step(const pflbm_sim *sim, uint64_t *step);

/* Copies one nx*ny*nz float32 field, as the reference's arrays hold it after
 * the last completed step (src/fileIO/fields.cuh:84-180), to host memory.
 * bytes must be >= nx*ny*nz*4. */
int pflbm_get_field(pflbm_sim *sim, int32_t field_id, void *host_dst, size_t bytes);

/* Same field as FP64 (exact for FP64 storage runs, widened otherwise).
 * bytes must be >= nx*ny*nz*8. No counterpart in the reference, whose
 * scalar_t is float (src/cuda/precision.cuh:27). */
int pflbm_get_field_f64(pflbm_sim *sim, int32_t field_id, double *host_dst, size_t bytes);

/* FP64 reductions (mass, momentum, Laplace jump, NaN count). Returns
 * PFLBM_ERR_DIVERGED when nonfinite > 0 (the diag is still filled). */
int pflbm_reduce(pflbm_sim *sim, pflbm_diag *out);

/* The reductions of pflbm_reduce over caller-owned device fields, allocating
 * no device memory. No counterpart in the reference. It is meant for callers
 * that cannot let a library call cudaMalloc: in-situ analysis hooks inside
 * another solver's time loop, or host frameworks whose memory pool reserves
 * the device heap (a cudaMalloc/cudaFree pair would also synchronise the
 * device in the middle of their pipeline).
 *
 * rho, ux, uy, uz, phi: nx*ny*nz float32 device arrays on the calling
 * thread's current device, laid out as pflbm_get_field writes them (ghost
 * shell included; only interior nodes are summed). dev_out: a device
 * pflbm_diag, filled as pflbm_reduce fills it except step = 0; NaN/Inf show
 * up in dev_out->nonfinite, not in the return code. The kernels are enqueued
 * on `stream` (a cudaStream_t; NULL = the legacy default stream) and the call
 * returns without waiting for them.
 *
 * Scratch: one row of FP64 partial sums per interior z plane in a fixed
 * device array of PFLBM_NOALLOC_MAX_PLANES rows (384 KiB) that every GPU
 * loading the library holds until the process exits. nz - 2 above
 * PFLBM_NOALLOC_MAX_PLANES is rejected with PFLBM_ERR_INVALID_ARG. All calls
 * on a device share that array: calls whose kernels overlap on the GPU (on
 * different streams) race and must be serialised by the caller. Each call
 * writes every row it reads, so no earlier call's contents leak into a result.
 * The first call in each CUDA context (the module, and so the array, is
 * loaded per context) looks up the array's device address with
 * cudaGetSymbolAddress, with that context's device current, and caches it
 * under the context's unique id; make that first call before any stream
 * capture. A device reset or a new context costs one more lookup. */
#define PFLBM_NOALLOC_MAX_PLANES 4096
int pflbm_reduce_fields_noalloc(const float *rho, const float *ux, const float *uy, const float *uz,
                                const float *phi, int32_t nx, int32_t ny, int32_t nz, void *stream,
                                pflbm_diag *dev_out);

/* Writes <dir>/<name><step:06>.bin for each field and <dir>/step_<step:06>.vti
 * that appends them (src/postProcess/PostProcess.cuh:43-261). */
int pflbm_write_output(pflbm_sim *sim, const char *dir, const int32_t *field_ids, int32_t n_fields);
/* Divergence watchdog (the reference aborts only on CUDA errors): with
 * interval > 0, pflbm_step runs the FP64 diagnostics after every multiple of
 * interval steps and returns PFLBM_ERR_DIVERGED when rho, u or phi hold
 * NaN/Inf, or, with max_phi_mass_drift > 0, when the phi mass moved by more
 * than that relative amount from its value at this call (closed boxes only:
 * the jet's inflow changes the mass). interval 0 switches it off. */
int pflbm_set_watchdog(pflbm_sim *sim, uint64_t interval, double max_phi_mass_drift);

/* Same files, written by a background thread: the fields are copied to
 * page-locked staging buffers before the call returns, so stepping can
 * continue at once. The next write_output call, pflbm_synchronize and
 * pflbm_destroy wait for the writer and report its I/O errors. */
int pflbm_write_output_async(pflbm_sim *sim, const char *dir, const int32_t *field_ids, int32_t n_fields);

/* Checkpoint and resume (the reference has none; its .bin dumps are
 * output only, src/main.cu:130-133). The file holds the configuration, the
 * step count, both ping-pong population and phi buffers (ghost values
 * included) and the derived averages. Loading requires the same grid, lattice, case
 * and storage; the run then continues bit for bit as if uninterrupted. */
int pflbm_save_checkpoint(pflbm_sim *sim, const char *path);
int pflbm_load_checkpoint(pflbm_sim *sim, const char *path);

/* Device bytes held by the simulation. */
int pflbm_device_bytes(const pflbm_sim *sim, uint64_t *bytes);

/* 1 when the collide kernel is fed by TMA bulk tensor copies (needs
 * 16-byte aligned rows: nx*element size % 16 == 0), 0 for plain loads. */
int pflbm_uses_tma(const pflbm_sim *sim, int32_t *flag);

/* Which collide kernel the plain time step runs (the averaging and closure
 * steps always use one node per thread): */
typedef enum {
    PFLBM_COLLIDE_PLAIN = 0,     /* plain loads, one node per thread */
    PFLBM_COLLIDE_TMA = 1,       /* TMA-fed, one node per thread */
    PFLBM_COLLIDE_TMA_PAIRS = 2  /* TMA-fed, two x-adjacent nodes per thread with packed FP32x2 arithmetic
                                    (16-bit storage, D3Q19) */
} pflbm_collide_variant_t;
int pflbm_collide_variant(const pflbm_sim *sim, int32_t *variant);

/* Number of CUDA kernels one time step launches (launch accounting). */
int pflbm_kernels_per_step(const pflbm_sim *sim, int32_t *count);

int pflbm_destroy(pflbm_sim *sim);

/* ---- batched ensembles (no counterpart in the reference) ---------------
 * Many independent periodic droplet boxes (FP32, one velocity set, possibly
 * different sizes and physics) advance together through a device work list
 * of (box, column tile, z chunk) items, in CUDA graphs. When every box's rows
 * are 16-byte aligned (nx a multiple of 4), every step is ONE persistent
 * cooperative launch: the TMA-fed collide sweep, a bounded grid-wide
 * barrier, the phase sweep. Otherwise a step is two persistent launches
 * (plain loads). Fields and diagnostics are per box and mean the same as for
 * a single simulation. A grid barrier that gives up sets the device error
 * word: the step returns PFLBM_ERR_DEVICE. */
typedef struct pflbm_ensemble pflbm_ensemble;
int pflbm_ensemble_create(const pflbm_config *cfgs, int32_t n_boxes, pflbm_ensemble **out);
int pflbm_ensemble_init(pflbm_ensemble *ens);
int pflbm_ensemble_step(pflbm_ensemble *ens, uint64_t nsteps);
int pflbm_ensemble_step_profiled(pflbm_ensemble *ens, uint64_t nsteps, double *ms);
int pflbm_ensemble_get_field(pflbm_ensemble *ens, int32_t box, int32_t field_id, void *host_dst, size_t bytes);
int pflbm_ensemble_reduce(pflbm_ensemble *ens, int32_t box, pflbm_diag *out);
/* Work granularity: z planes per work item, resident CTAs per SM (1 up to
 * what the tile shape lets reside on an SM: 4 for 32x4, 2 for 32x8 and
 * 64x4, 1 for 32x16; 1 or 2 on the plain-load path). */
int pflbm_ensemble_set_tuning(pflbm_ensemble *ens, int32_t zchunk, int32_t ctas_per_sm);
/* Column tile of the fused TMA step: 32x8 (default), 32x4, 64x4 or 32x16.
 * The results do not depend on it. PFLBM_ERR_UNSUPPORTED on the plain-load
 * path (32x8 only) or when the shape does not fit the GPU. */
int pflbm_ensemble_set_tile(pflbm_ensemble *ens, int32_t tile_x, int32_t tile_y);
/* The tuning in use (any pointer may be NULL). */
int pflbm_ensemble_get_tuning(const pflbm_ensemble *ens, int32_t *tile_x, int32_t *tile_y, int32_t *zchunk,
                              int32_t *ctas_per_sm);
/* Measured autotuner: times each candidate (tile shape x zchunk x resident
 * CTAs per SM) for trial_steps steps, keeps the fastest (read it back with
 * pflbm_ensemble_get_tuning) and re-initialises the ensemble. */
int pflbm_ensemble_autotune(pflbm_ensemble *ens, int32_t trial_steps, int32_t *best_zchunk, int32_t *best_ctas,
                            double *best_ms);
int pflbm_ensemble_info(const pflbm_ensemble *ens, uint64_t *total_nodes, int32_t *n_boxes, int32_t *n_items);
int pflbm_ensemble_destroy(pflbm_ensemble *ens);

/* ---- learned eddy-viscosity closure (no counterpart in the reference) ---
 * An MLP maps the per-node features (Pi_xx, Pi_yy, Pi_zz, Pi_xy, Pi_xz,
 * Pi_yz, phi, |grad phi|) to an eddy viscosity nu_t >= 0 that the collision
 * adds to the relaxation time (tau += 3 * strength * nu_t; the reference's
 * constant-tau collision, lbm.cu:158-170, is strength 0 / no closure).
 * Network: 8 -> 32 -> 32 -> 1, SiLU hidden layers, softplus output.
 * Blob (PFLBM_MLP_BLOB floats): W1[32][8], b1[32], W2[32][32], b2[32],
 * w3[32], b3, feature mean[8], feature inv_scale[8], out_scale, strength.
 *
 * Training data are box-filtered (3x3x3) and 2x-restricted snapshots of a
 * fine FP32 run of this solver: features as the coarse solver would carry
 * them and the least-squares eddy viscosity of the sub-filter stress as the
 * target. Forward, backward and Adam run as CUDA kernels. */
#define PFLBM_MLP_PARAMS 1377
#define PFLBM_MLP_BLOB 1395
typedef struct pflbm_closure pflbm_closure;
int pflbm_closure_create(int32_t device, uint64_t max_samples, pflbm_closure **out);
/* Appends the samples of the fine simulation's current state (coarse nodes
 * with x and y multiples of stride, all interior z). */
int pflbm_closure_add_snapshot(pflbm_closure *c, pflbm_sim *fine, int32_t stride, uint64_t *added);
int pflbm_closure_num_samples(const pflbm_closure *c, uint64_t *n);
/* Interface width of the snapshots added so far, W = 4 sum phi(1-phi) /
 * sum |grad phi| over the sample nodes: on the fine field at the samples'
 * fine nodes (fine lattice units) and on the filtered coarse field (coarse
 * units). gamma_scale = width_fine / width_filtered is the factor on the
 * coarse run's interface sharpening gamma that gives its equilibrium
 * interface the filtered fine width (W ~ 1 / gamma at the fixed mobility of
 * tau_g = 1); the phase-field part of the closure. widths may be NULL.
 * PFLBM_ERR_STATE when the snapshots hold no interface. Samples replaced by
 * set_samples keep the widths of the snapshots added before. */
int pflbm_closure_interface_scale(const pflbm_closure *c, double *gamma_scale, double *width_fine,
                                  double *width_filtered);
/* Samples as host arrays x[n][8], y[n]; set_samples replaces the data set. */
int pflbm_closure_get_samples(pflbm_closure *c, uint64_t first, uint64_t count, float *host_x, float *host_y);
int pflbm_closure_set_samples(pflbm_closure *c, const float *host_x, const float *host_y, uint64_t count);
/* Feature normalisation and out_scale from the data, Glorot-uniform weights
 * from a counter hash of seed; resets Adam. */
int pflbm_closure_init_params(pflbm_closure *c, uint32_t seed);
int pflbm_closure_get_blob(pflbm_closure *c, float *host_blob);
int pflbm_closure_set_blob(pflbm_closure *c, const float *host_blob);
/* Summed gradient of the loss (softplus(z) - y/out_scale)^2 over the first
 * count samples, FP64 accumulation of FP32 per-block sums. */
int pflbm_closure_gradient(pflbm_closure *c, uint64_t count, double *host_grad, double *loss_sum);
/* Adam (beta 0.9/0.999, eps 1e-8) on minibatches drawn by a counter hash;
 * loss_history (may be NULL) receives the mean minibatch loss per iteration. */
int pflbm_closure_train(pflbm_closure *c, int32_t iterations, int32_t batch, float lr, uint32_t seed,
                        double *loss_history);
int pflbm_closure_loss(pflbm_closure *c, double *mean_loss);
int pflbm_closure_destroy(pflbm_closure *c);
/* Attaches a trained network to a simulation (FP32 or FP64 storage; NULL
 * detaches): the weights are rounded to BF16 and run in the collide kernel,
 * the result scaled by strength (>= 0). */
int pflbm_set_closure(pflbm_sim *sim, const float *blob, float strength);
/* Phase mixing of the attached closure: the sub-filter flux of phi is
 * modelled as an eddy diffusivity D_t = inv_schmidt * strength * nu_t (a
 * turbulent Schmidt number Sc_t = 1 / inv_schmidt) added to the phase flux
 * (J += -4 D_t grad phi); 0 (the default after attaching) switches it off.
 * PFLBM_ERR_STATE without a closure attached. */
int pflbm_set_closure_mixing(pflbm_sim *sim, float inv_schmidt);

#ifdef __cplusplus
}
#endif

#endif /* PFLBM_H */
