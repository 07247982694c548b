// pflbm_reduce_fields_noalloc: the diagnostics reduction of pflbm_reduce over
// caller-owned device fields, with no device allocation.
//
// Who needs it: in-situ analysis hooks called from another solver's time
// loop, or from a host framework that reserves the whole device heap in its
// own memory pool. Such callers cannot let a library call cudaMalloc (the
// pool owns the memory, and a cudaMalloc/cudaFree pair implicitly
// synchronises the device in the middle of their pipeline). They own the
// inputs and the output; the only scratch this call needs, one row of FP64
// partial sums per interior z plane, lives in a fixed file-scope device array.
//
// The scratch array below is part of the library's module: every GPU that
// loads the library holds it (kScratchBytes) until the process exits. Every
// call on a device shares it, so calls whose kernels overlap on that GPU race
// on it; each call writes every row it later reads, so nothing has to start at
// zero and the contents left by an earlier call are never read.
#include <cuda.h>
#include <cuda_runtime.h>

#include <cstdint>
#include <mutex>
#include <string>

#include "../../include/pflbm.h"
#include "engine.h"
#include "reduce.cuh"

namespace {

constexpr int kFields = pflbm::RED_FIELDS;
constexpr int kThreads = 256;
constexpr int kMaxContexts = 64;
constexpr size_t kScratchDoubles = size_t(PFLBM_NOALLOC_MAX_PLANES) * kFields;
constexpr size_t kScratchBytes = kScratchDoubles * sizeof(double);  // 384 KiB
static_assert(kScratchBytes == 384 * 1024, "scratch size stated in pflbm.h");

// Host code sees only a stand-in symbol; the device address comes from
// cudaGetSymbolAddress, once per CUDA context.
static __device__ __align__(256) double g_plane_partials[kScratchDoubles];

// Device addresses of g_plane_partials, one per CUDA context that has called
// (the module, and with it the array, is loaded per context: a device reset
// or a caller's own non-primary context gets a new one). Keyed by the
// context's unique id, which is never reused within a process.
struct ScratchEntry {
    unsigned long long ctx_id;
    double *ptr;
};
std::mutex g_setup_mutex;
ScratchEntry g_scratch[kMaxContexts] = {};
int g_scratch_next = 0;  // round-robin slot for a new context

using CtxGetCurrentFn = CUresult (*)(CUcontext *);
using CtxGetIdFn = CUresult (*)(CUcontext, unsigned long long *);

int fail(int code, const std::string &msg) {
    pflbm::set_error(msg);
    return code;
}

int cuda_fail(cudaError_t e, const char *what) {
    cudaGetLastError();
    return fail(PFLBM_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}

// Unique id of the current CUDA context (driver entry points through the
// runtime, so the library needs no link against libcuda).
int current_context_id(unsigned long long *id) {
    static CtxGetCurrentFn get_current = nullptr;
    static CtxGetIdFn get_id = nullptr;
    static std::once_flag once;
    std::call_once(once, [] {
        void *a = nullptr, *b = nullptr;
        cudaDriverEntryPointQueryResult qa{}, qb{};
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &a, 12000, cudaEnableDefault, &qa) == cudaSuccess &&
            qa == cudaDriverEntryPointSuccess && a &&
            cudaGetDriverEntryPointByVersion("cuCtxGetId", &b, 12000, cudaEnableDefault, &qb) == cudaSuccess &&
            qb == cudaDriverEntryPointSuccess && b) {
            get_current = reinterpret_cast<CtxGetCurrentFn>(a);
            get_id = reinterpret_cast<CtxGetIdFn>(b);
        } else {
            cudaGetLastError();
        }
    });
    if (!get_current || !get_id)
        return fail(PFLBM_ERR_CUDA, "driver entry points cuCtxGetCurrent / cuCtxGetId unavailable");
    CUcontext ctx = nullptr;
    if (get_current(&ctx) != CUDA_SUCCESS || !ctx)
        return fail(PFLBM_ERR_CUDA, "no current CUDA context");
    if (get_id(ctx, id) != CUDA_SUCCESS) return fail(PFLBM_ERR_CUDA, "cuCtxGetId failed");
    return PFLBM_OK;
}

// Device address of g_plane_partials in the current context, looked up with
// cudaGetSymbolAddress on the first call in that context and cached.
int scratch_for_current_context(double **out) {
    unsigned long long id = 0;
    if (int rc = current_context_id(&id)) return rc;
    std::lock_guard<std::mutex> lock(g_setup_mutex);
    for (const ScratchEntry &en : g_scratch)
        if (en.ptr && en.ctx_id == id) {
            *out = en.ptr;
            return PFLBM_OK;
        }
    double *ptr = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(reinterpret_cast<void **>(&ptr), g_plane_partials);
    if (e != cudaSuccess) return cuda_fail(e, "cudaGetSymbolAddress(plane partials)");
    g_scratch[g_scratch_next] = {id, ptr};
    g_scratch_next = (g_scratch_next + 1) % kMaxContexts;
    *out = ptr;
    return PFLBM_OK;
}

int check_device_ptr(const void *p, int device, const char *name) {
    cudaPointerAttributes a{};
    const cudaError_t e = cudaPointerGetAttributes(&a, p);
    if (e != cudaSuccess) return cuda_fail(e, "cudaPointerGetAttributes");
    if ((a.type != cudaMemoryTypeDevice && a.type != cudaMemoryTypeManaged) || a.device != device)
        return fail(PFLBM_ERR_INVALID_ARG,
                    std::string(name) + " is not device memory of the current device " + std::to_string(device));
    return PFLBM_OK;
}

// One CTA per interior plane z = 1 + blockIdx.x: FP64 sums over the plane's
// interior nodes, written (not accumulated) to row blockIdx.x of the scratch.
__global__ void __launch_bounds__(kThreads)
    k_reduce_planes(const float *__restrict__ rho, const float *__restrict__ ux, const float *__restrict__ uy,
                    const float *__restrict__ uz, const float *__restrict__ phi, int nx, int ny,
                    double *__restrict__ rows) {
    const int z = 1 + blockIdx.x;
    const int wx = nx - 2;
    const int n_plane = wx * (ny - 2);
    double acc[kFields] = {0};
    for (int k = threadIdx.x; k < n_plane; k += kThreads) {
        const int x = 1 + k % wx, y = 1 + k / wx;
        const size_t i = size_t(x) + size_t(nx) * (size_t(y) + size_t(ny) * size_t(z));
        const double f = phi[i], r = rho[i], vx = ux[i], vy = uy[i], vz = uz[i];
        if (!isfinite(f) || !isfinite(r) || !isfinite(vx) || !isfinite(vy) || !isfinite(vz)) {
            acc[10] += 1.0;
            continue;
        }
        acc[0] += f;
        acc[1] += r;
        acc[2] += r * vx;
        acc[3] += r * vy;
        acc[4] += r * vz;
        acc[5] = fmax(acc[5], sqrt(vx * vx + vy * vy + vz * vz));
        if (f > 0.9) { acc[6] += r; acc[7] += 1.0; }
        if (f < 0.1) { acc[8] += r; acc[9] += 1.0; }
    }
    pflbm::block_reduce_row<kThreads>(acc, rows + size_t(blockIdx.x) * kFields);
}

// Sums the rows in plane order and writes the pflbm_diag the host entry point
// pflbm_reduce would produce (step = 0: fields carry no step count).
__global__ void __launch_bounds__(32) k_reduce_rows(const double *__restrict__ rows, int n_rows, pflbm_diag *out) {
    __shared__ double tot[kFields];
    const int f = threadIdx.x;
    if (f < kFields) {
        double s = 0.0;
        for (int b = 0; b < n_rows; ++b) {
            const double v = rows[size_t(b) * kFields + f];
            s = pflbm::red_combine(f, s, v);
        }
        tot[f] = s;
    }
    __syncthreads();
    if (f == 0) {
        pflbm_diag d;
        d.step = 0;
        d.phi_mass = tot[0];
        d.rho_mass = tot[1];
        d.momentum[0] = tot[2];
        d.momentum[1] = tot[3];
        d.momentum[2] = tot[4];
        d.max_speed = tot[5];
        d.n_in = uint64_t(tot[7]);
        d.n_out = uint64_t(tot[9]);
        d.rho_in = tot[7] > 0 ? tot[6] / tot[7] : 0.0;
        d.rho_out = tot[9] > 0 ? tot[8] / tot[9] : 0.0;
        d.laplace_dp = (d.rho_in - d.rho_out) / 3.0;
        d.nonfinite = uint64_t(tot[10]);
        *out = d;
    }
}

}  // namespace

extern "C" int pflbm_reduce_fields_noalloc(const float *rho, const float *ux, const float *uy, const float *uz,
                                           const float *phi, int32_t nx, int32_t ny, int32_t nz, void *stream,
                                           pflbm_diag *dev_out) {
    if (!rho || !ux || !uy || !uz || !phi || !dev_out) return fail(PFLBM_ERR_INVALID_ARG, "null pointer");
    if (nx < 3 || ny < 3 || nz < 3) return fail(PFLBM_ERR_INVALID_ARG, "nx, ny, nz must each be >= 3");
    if (nz - 2 > PFLBM_NOALLOC_MAX_PLANES)
        return fail(PFLBM_ERR_INVALID_ARG, "nz - 2 = " + std::to_string(nz - 2) +
                                               " interior planes exceeds PFLBM_NOALLOC_MAX_PLANES = " +
                                               std::to_string(PFLBM_NOALLOC_MAX_PLANES));
    if (int64_t(nx - 2) * int64_t(ny - 2) > INT32_MAX)
        return fail(PFLBM_ERR_INVALID_ARG, "plane too large: (nx-2)*(ny-2) must fit in int32");
    int device = 0;
    cudaError_t e = cudaGetDevice(&device);
    if (e != cudaSuccess) return cuda_fail(e, "cudaGetDevice");
    const void *ptrs[6] = {rho, ux, uy, uz, phi, dev_out};
    const char *names[6] = {"rho", "ux", "uy", "uz", "phi", "dev_out"};
    for (int k = 0; k < 6; ++k)
        if (int rc = check_device_ptr(ptrs[k], device, names[k])) return rc;
    double *rows = nullptr;
    if (int rc = scratch_for_current_context(&rows)) return rc;
    const cudaStream_t s = static_cast<cudaStream_t>(stream);
    const int planes = nz - 2;
    k_reduce_planes<<<planes, kThreads, 0, s>>>(rho, ux, uy, uz, phi, nx, ny, rows);
    k_reduce_rows<<<1, 32, 0, s>>>(rows, planes, dev_out);
    e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_fail(e, "pflbm_reduce_fields_noalloc launch");
    return PFLBM_OK;
}
