// api.cu - the C ABI of include/pflbm.h: configuration, allocation,
// CUDA-graph time loop, field readback, diagnostics and file output.
//
// The time loop of src/main.cu:163-188 launches a captured graph and two
// boundary kernels and synchronises the host every step. Here one step is
// two kernels (boundary conditions are folded into them) and whole chunks of
// steps are captured into one graph, so a run of n steps costs n/16 graph
// launches and no host synchronisation until the caller asks for one.
#include <cuda_runtime.h>

#include <algorithm>
#include <cerrno>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <memory>
#include <new>
#include <system_error>
#include <string>
#include <sys/stat.h>
#include <thread>
#include <vector>

#include <nvtx3/nvToolsExt.h>

#include "../../include/pflbm.h"
#include "engine.h"
#include "tile.h"

using pflbm::Engine;
using pflbm::HostParams;

namespace {

thread_local std::string g_err;

// NVTX range around a C-ABI call (visible in Nsight timelines; no cost
// without a tool attached).
struct NvtxRange {
    explicit NvtxRange(const char *name) { nvtxRangePushA(name); }
    ~NvtxRange() { nvtxRangePop(); }
    NvtxRange(const NvtxRange &) = delete;
    NvtxRange &operator=(const NvtxRange &) = delete;
};

int fail(int code, const std::string &msg) {
    g_err = msg;
    return code;
}

int cuda_fail(cudaError_t e, const char *what) {
    std::string m = std::string(what) + ": " + cudaGetErrorString(e);
    cudaGetLastError();
    return fail(PFLBM_ERR_CUDA, m);
}

constexpr int kChunk = 16;  // steps per captured graph

const char *kFieldNames[PFLBM_FIELD_COUNT] = {
    "rho", "ux", "uy", "uz", "pxx", "pyy", "pzz", "pxy", "pxz", "pyz", "phi", "normx", "normy", "normz", "ind",
    "fsx", "fsy", "fsz", "avg_phi", "avg_ux", "avg_uy", "avg_uz", "avg_uxux", "avg_uyuy", "avg_uzuz", "avg_uxuy",
    "avg_uxuz", "avg_uyuz", "vort_x", "vort_y", "vort_z", "vort_mag", "c"};

}  // namespace

struct pflbm_sim {
    pflbm_config cfg{};
    HostParams hp{};
    int device = 0;
    std::unique_ptr<Engine> eng;
    cudaStream_t stream = nullptr;
    // graphs[parity][0] = 1 step, [1] = 2 steps, [2] = kChunk steps
    cudaGraphExec_t graphs[2][3] = {{nullptr, nullptr, nullptr}, {nullptr, nullptr, nullptr}};
    int parity = 0;          // ping-pong buffer read by the next step
    uint64_t step = 0;       // completed steps
    bool initialized = false;
    int64_t cache_step = -1; // step the analysis cache describes
    bool distros_dirty = false; // initial fields changed since the last rebuild
    double *dev_diag = nullptr;
    // background output writer (pflbm_write_output_async)
    std::thread writer;
    int writer_rc = 0;
    std::string writer_err;
    std::vector<float *> pinned;  // page-locked staging, one N-float array per field
    // divergence watchdog (pflbm_set_watchdog)
    uint64_t wd_interval = 0;
    double wd_max_drift = 0.0, wd_mass0 = 0.0;
};

namespace pflbm {

// Derived constants as the reference computes them
// (src/constants.cuh:80-141, src/functions/globalFunctions.cuh:104-461).
void derive(const pflbm_config &c, HostParams &h) {
    h = HostParams{};
    h.nx = c.nx; h.ny = c.ny; h.nz = c.nz;
    h.N = uint64_t(c.nx) * c.ny * c.nz;
    h.jet = c.flow_case == PFLBM_CASE_JET;
    h.sigma = c.sigma; h.gamma = c.gamma; h.u_inf = c.u_inf;
    h.f_sigma = c.sigma; h.f_gamma = c.gamma; h.f_u_inf = c.u_inf;
    // geometry::center_*, R2 (globalFunctions.cuh:104-125)
    h.f_center_x = static_cast<float>(c.nx - 1) * 0.5f + c.center_offset[0];
    h.f_center_y = static_cast<float>(c.ny - 1) * 0.5f + c.center_offset[1];
    h.f_center_z = static_cast<float>(c.nz - 1) * 0.5f + c.center_offset[2];
    h.center_x = (double(c.nx) - 1.0) * 0.5 + c.center_offset[0];
    h.center_y = (double(c.ny) - 1.0) * 0.5 + c.center_offset[1];
    h.center_z = (double(c.nz) - 1.0) * 0.5 + c.center_offset[2];
    h.f_R2 = static_cast<float>(c.radius * c.radius);
    h.R2 = double(c.radius) * c.radius;
    if (h.jet) {
        // relaxation:: for JET (globalFunctions.cuh:305-397)
        const double vw = (double(c.u_inf) * double(c.diam)) / double(c.reynolds_water);
        const double vo = (double(c.u_inf) * double(c.diam)) / double(c.reynolds_oil);
        h.f_visc_water = float(vw);
        h.f_visc_oil = float(vo);
        h.visc_water = vw;
        h.visc_oil = vo;
        h.f_tau_water = 0.5f + 3.0f * h.f_visc_water;
        h.f_tau_oil = 0.5f + 3.0f * h.f_visc_oil;
        h.tau_water = 0.5 + 3.0 * vw;
        h.tau_oil = 0.5 + 3.0 * vo;
        h.f_omco_zmin = 1.0f - float(1.0 / (0.5 + 3.0 * double(h.f_visc_oil)));
        h.omco_zmin = 1.0 - 1.0 / (0.5 + 3.0 * vo);
        h.f_kgain1 = 1.0f + c.sponge_gain;
        h.kgain1 = 1.0 + double(c.sponge_gain);
        // sponge:: (globalFunctions.cuh:260-292)
        const int cells = c.sponge_cells >= 0 ? c.sponge_cells : int(c.nz / 12);
        const float sp = float(double(cells) / double(c.nz - 1));
        h.f_z_start = float(double(c.nz - 1 - cells) / double(c.nz - 1));
        h.f_inv_nz_m1 = float(1.0 / double(c.nz - 1));
        h.f_inv_sponge = float(1.0 / double(sp));
        h.z_start = double(c.nz - 1 - cells) / double(c.nz - 1);
        h.inv_nz_m1 = 1.0 / double(c.nz - 1);
        h.inv_sponge = double(c.nz - 1) / double(cells > 0 ? cells : 1);
    } else {
        // physics::visc_ref, relaxation::omega_ref (constants.cuh:139-140,
        // globalFunctions.cuh:406-429)
        const float visc_ref = (c.tau - 0.5f) / 3.0f;
        h.f_omega_ref = float(1.0 / (0.5 + 3.0 * double(visc_ref)));
        h.omega_ref = 1.0 / (0.5 + 3.0 * ((double(c.tau) - 0.5) / 3.0));
    }
    h.sigma_u = c.noise_amp * c.u_inf;  // BoundaryConditions.cuh:58
    h.noise_amp = c.noise_amp;
    h.noise_mode = c.inflow_noise;
    h.seed = c.seed;
    h.droplet_x_stretch = c.droplet_x_stretch;
    h.radius = c.radius;
    h.interface_width = c.interface_width;
    h.init_noise = c.init_noise;
}

int validate(const pflbm_config &c) {
    if (c.struct_size != sizeof(pflbm_config))
        return fail(PFLBM_ERR_INVALID_ARG, "pflbm_config.struct_size mismatch (header/library version skew)");
    if (c.flow_case != PFLBM_CASE_DROPLET && c.flow_case != PFLBM_CASE_JET)
        return fail(PFLBM_ERR_INVALID_ARG, "flow_case must be PFLBM_CASE_DROPLET or PFLBM_CASE_JET");
    if (c.velocity_set != PFLBM_VS_D3Q19 && c.velocity_set != PFLBM_VS_D3Q27)
        return fail(PFLBM_ERR_INVALID_ARG, "velocity_set must be 19 or 27");
    if (c.storage < PFLBM_STORAGE_FP32 || c.storage > PFLBM_STORAGE_FP64)
        return fail(PFLBM_ERR_INVALID_ARG, "storage must be FP32, FP16, BF16 or FP64");
    if (c.nx < 5 || c.ny < 5 || c.nz < 5) return fail(PFLBM_ERR_INVALID_ARG, "nx, ny, nz must be >= 5");
    if (c.nx > 65536 || c.ny > 65536 || c.nz > 65536) return fail(PFLBM_ERR_INVALID_ARG, "dimension above 65536");
    // the step kernels index a node within one array with 32 bits (a grid
    // this large would not fit in device memory anyway)
    if (uint64_t(c.nx) * c.ny * c.nz >= (uint64_t(1) << 32))
        return fail(PFLBM_ERR_INVALID_ARG, "grid of 2^32 nodes or more");
    if (!(c.interface_width > 0.0f)) return fail(PFLBM_ERR_INVALID_ARG, "interface_width must be > 0");
    if (c.inflow_noise != PFLBM_NOISE_GAUSSIAN_UXY && c.inflow_noise != PFLBM_NOISE_UNIFORM_UZ)
        return fail(PFLBM_ERR_INVALID_ARG, "inflow_noise must be 0 or 1");
    if (c.flow_case == PFLBM_CASE_JET) {
        // the sponge needs nz >= 12 (globalFunctions.cuh:269)
        if (c.nz < 12) return fail(PFLBM_ERR_INVALID_ARG, "jet needs nz >= 12 (sponge layer)");
        if (c.diam <= 0 || c.radius < 0) return fail(PFLBM_ERR_INVALID_ARG, "jet needs diam > 0 and radius >= 0");
        if (!(c.reynolds_water > 0.0f) || !(c.reynolds_oil > 0.0f))
            return fail(PFLBM_ERR_INVALID_ARG, "jet needs positive Reynolds numbers");
        // the inlet disc (and the nodes it feeds) must lie inside [1, n-2]
        const double cx = (c.nx - 1) * 0.5, cy = (c.ny - 1) * 0.5;
        if (cx - c.radius < 1.0 || cx + c.radius > c.nx - 2.0 || cy - c.radius < 1.0 || cy + c.radius > c.ny - 2.0)
            return fail(PFLBM_ERR_INVALID_ARG, "jet inlet disc must lie inside the interior columns");
        if (c.sponge_cells >= int(c.nz) - 1) return fail(PFLBM_ERR_INVALID_ARG, "sponge_cells too large");
    } else {
        if (!(c.tau > 0.5f)) return fail(PFLBM_ERR_INVALID_ARG, "droplet needs tau > 0.5");
        if (!(c.droplet_x_stretch > 0.0f)) return fail(PFLBM_ERR_INVALID_ARG, "droplet_x_stretch must be > 0");
    }
    return PFLBM_OK;
}

void set_error(const std::string &msg) { g_err = msg; }

}  // namespace pflbm

namespace {
using pflbm::derive;
using pflbm::validate;

int pick_zchunk(const pflbm_config &c, int device) {
    if (const char *e = std::getenv("PFLBM_ZCHUNK")) {
        const int v = std::atoi(e);
        if (v > 0) return v;
    }
    int sms = 152;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
    const int ctas_xy = int((c.nx + pflbm::kTileX - 1) / pflbm::kTileX) * int((c.ny + pflbm::kTileY - 1) / pflbm::kTileY);
    const int nzi = int(c.nz) - 2;
    int chunks = (8 * sms + ctas_xy - 1) / ctas_xy;
    if (chunks < 1) chunks = 1;
    int zc = (nzi + chunks - 1) / chunks;
    if (zc < 4) zc = 4;
    if (zc > nzi) zc = nzi;
    return zc;
}

void destroy_graphs(pflbm_sim *s) {
    for (auto &row : s->graphs)
        for (auto &g : row)
            if (g) {
                cudaGraphExecDestroy(g);
                g = nullptr;
            }
}

int capture(pflbm_sim *s, int parity, int nsteps, cudaGraphExec_t *out) {
    cudaGraph_t graph = nullptr;
    cudaError_t e = cudaStreamBeginCapture(s->stream, cudaStreamCaptureModeThreadLocal);
    if (e != cudaSuccess) return cuda_fail(e, "cudaStreamBeginCapture");
    int p = parity;
    for (int i = 0; i < nsteps; ++i) {
        s->eng->enqueue_step(p, s->stream);
        p ^= 1;
    }
    e = cudaStreamEndCapture(s->stream, &graph);
    if (e != cudaSuccess) return cuda_fail(e, "cudaStreamEndCapture");
    e = cudaGraphInstantiate(out, graph, 0);
    cudaGraphDestroy(graph);
    if (e != cudaSuccess) return cuda_fail(e, "cudaGraphInstantiate");
    return PFLBM_OK;
}

// Reads the device error word (set by a kernel whose bounded wait gave up).
int check_device_error(pflbm_sim *s) {
    unsigned int w = 0;
    cudaError_t e = cudaMemcpy(&w, s->eng->error_word(), sizeof w, cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return cuda_fail(e, "error word readback");
    if (w != 0) return fail(PFLBM_ERR_DEVICE, "a kernel gave up waiting for its TMA copies (error word " + std::to_string(w) + ")");
    return PFLBM_OK;
}

// Rebuilds f and phi from the initial fields after pflbm_set_initial_field.
void flush_initial(pflbm_sim *s) {
    if (s->distros_dirty) {
        s->eng->enqueue_init_distros(s->stream);
        s->distros_dirty = false;
    }
}

int ensure_cache(pflbm_sim *s) {
    if (s->cache_step == int64_t(s->step)) return PFLBM_OK;
    if (s->step == 0 && s->cache_step == 0) {
        // the cache still holds the initial fields
        s->cache_step = 0;
        return PFLBM_OK;
    }
    s->eng->enqueue_analysis(s->parity ^ 1, uint32_t(s->step - 1), s->stream);
    s->eng->enqueue_vorticity(s->stream);
    cudaError_t e = cudaStreamSynchronize(s->stream);
    if (e != cudaSuccess) return cuda_fail(e, "analysis");
    s->cache_step = int64_t(s->step);
    return PFLBM_OK;
}

// Copies real-typed device data to host doubles or floats.
int copy_out(pflbm_sim *s, const void *dev, size_t n, void *host, bool as_double) {
    const int rb = s->eng->real_bytes();
    cudaError_t e;
    if ((rb == 4 && !as_double) || (rb == 8 && as_double)) {
        e = cudaMemcpy(host, dev, n * rb, cudaMemcpyDeviceToHost);
        if (e != cudaSuccess) return cuda_fail(e, "cudaMemcpy D2H");
        return PFLBM_OK;
    }
    // conversion buffer: allocated without exceptions, which must not
    // cross the C ABI
    std::unique_ptr<unsigned char[]> tmp(new (std::nothrow) unsigned char[n * rb]);
    if (!tmp) return fail(PFLBM_ERR_OUT_OF_MEMORY, "host conversion buffer");
    e = cudaMemcpy(tmp.get(), dev, n * rb, cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return cuda_fail(e, "cudaMemcpy D2H");
    if (rb == 4) {
        const float *src = reinterpret_cast<const float *>(tmp.get());
        double *dst = static_cast<double *>(host);
        for (size_t i = 0; i < n; ++i) dst[i] = src[i];
    } else {
        const double *src = reinterpret_cast<const double *>(tmp.get());
        float *dst = static_cast<float *>(host);
        for (size_t i = 0; i < n; ++i) dst[i] = float(src[i]);
    }
    return PFLBM_OK;
}

int get_field_impl(pflbm_sim *s, int32_t id, void *host, size_t bytes, bool as_double) {
    if (!s || !host) return fail(PFLBM_ERR_INVALID_ARG, "null argument");
    if (!s->initialized) return fail(PFLBM_ERR_STATE, "pflbm_init has not been called");
    flush_initial(s);
    const uint64_t N = s->hp.N;
    const size_t need = N * (as_double ? sizeof(double) : sizeof(float));
    if (bytes < need) return fail(PFLBM_ERR_INVALID_ARG, "destination buffer too small");
    if (id < 0 || id >= PFLBM_FIELD_COUNT) return fail(PFLBM_ERR_INVALID_ARG, "unknown field id");
    const int rb = s->eng->real_bytes();
    int rc = ensure_cache(s);
    if (rc) return rc;
    const unsigned char *src = nullptr;
    if (id <= PFLBM_FIELD_FFZ) {
        src = static_cast<const unsigned char *>(s->eng->macro_ptr()) + size_t(id) * N * rb;
    } else if (id >= PFLBM_FIELD_AVG_PHI && id <= PFLBM_FIELD_AVG_UYUZ) {
        const bool avg = id <= PFLBM_FIELD_AVG_UZ;
        if (!s->eng->avg_ptr() || !(s->cfg.flags & (avg ? PFLBM_FLAG_TIME_AVERAGE : PFLBM_FLAG_REYNOLDS_MOMENTS)))
            return fail(PFLBM_ERR_UNSUPPORTED, "derived field not enabled in pflbm_config.flags");
        src = static_cast<const unsigned char *>(s->eng->avg_ptr()) + size_t(id - PFLBM_FIELD_AVG_PHI) * N * rb;
    } else if (id >= PFLBM_FIELD_VORT_X && id <= PFLBM_FIELD_VORT_MAG) {
        if (!s->eng->vort_ptr()) return fail(PFLBM_ERR_UNSUPPORTED, "vorticity not enabled in pflbm_config.flags");
        src = static_cast<const unsigned char *>(s->eng->vort_ptr()) + size_t(id - PFLBM_FIELD_VORT_X) * N * rb;
    } else {
        return fail(PFLBM_ERR_UNSUPPORTED, "passive scalar is not part of this library");
    }
    rc = copy_out(s, src, N, host, as_double);
    if (rc) return rc;
    if (id >= PFLBM_FIELD_AVG_PHI && id <= PFLBM_FIELD_AVG_UYUZ && s->hp.jet && s->step > 0) {
        // the outlet ghost plane holds a copy of plane nz-2 at every step
        // (BoundaryConditions.cuh:122-126), so its running mean equals plane nz-2's
        const size_t plane = size_t(s->hp.nx) * s->hp.ny, es = as_double ? 8 : 4;
        unsigned char *h = static_cast<unsigned char *>(host);
        for (uint32_t y = 1; y + 1 < s->hp.ny; ++y)
            std::memcpy(h + ((s->hp.nz - 1) * plane + y * size_t(s->hp.nx) + 1) * es,
                        h + ((s->hp.nz - 2) * plane + y * size_t(s->hp.nx) + 1) * es, (s->hp.nx - 2) * es);
    }
    return PFLBM_OK;
}

bool make_dirs(const std::string &dir) {
    std::string acc;
    for (size_t i = 0; i <= dir.size(); ++i) {
        if (i == dir.size() || dir[i] == '/') {
            if (!acc.empty() && mkdir(acc.c_str(), 0755) != 0 && errno != EEXIST) return false;
        }
        if (i < dir.size()) acc.push_back(dir[i]);
    }
    return true;
}

std::string step6(uint64_t t) {
    char b[32];
    std::snprintf(b, sizeof b, "%06llu", static_cast<unsigned long long>(t));
    return b;
}

}  // namespace

namespace pflbm {
int sim_view(pflbm_sim *s, SimView &v) {
    if (!s) return fail(PFLBM_ERR_INVALID_ARG, "null simulation");
    if (!s->initialized) return fail(PFLBM_ERR_STATE, "pflbm_init has not been called");
    cudaSetDevice(s->device);
    flush_initial(s);
    int rc = ensure_cache(s);
    if (rc) return rc;
    v.macro = s->eng->macro_ptr();
    v.real_bytes = s->eng->real_bytes();
    v.nx = s->hp.nx;
    v.ny = s->hp.ny;
    v.nz = s->hp.nz;
    v.N = s->hp.N;
    v.device = s->device;
    v.tau_water = s->hp.tau_water;
    v.tau_oil = s->hp.tau_oil;
    return PFLBM_OK;
}
}  // namespace pflbm

namespace {

// Files of one output step: <name><step06>.bin per field (PostProcess.cuh:43-97)
// and step_<step06>.vti, VTK ImageData with the arrays appended raw behind
// UInt32 size headers (PostProcess.cuh:99-261). Runs on the writer thread.
int write_step_files(const std::string &d, const std::string &suffix, const std::vector<std::string> &names,
                     const std::vector<const float *> &data, uint64_t N, uint32_t nx, uint32_t ny, uint32_t nz,
                     std::string &err) {
    const uint64_t nbytes = N * sizeof(float);
    for (size_t i = 0; i < names.size(); ++i) {
        const std::string path = d + names[i] + suffix + ".bin";
        std::ofstream o(path, std::ios::binary | std::ios::trunc);
        if (!o) { err = "cannot open " + path; return PFLBM_ERR_IO; }
        o.write(reinterpret_cast<const char *>(data[i]), std::streamsize(nbytes));
        if (!o) { err = "write failed: " + path; return PFLBM_ERR_IO; }
    }
    if (names.empty()) return PFLBM_OK;
    const std::string vti = d + "step_" + suffix + ".vti";
    std::ofstream v(vti, std::ios::binary | std::ios::trunc);
    if (!v) { err = "cannot open " + vti; return PFLBM_ERR_IO; }
    v << "<?xml version=\"1.0\"?>\n";
    v << "<VTKFile type=\"ImageData\" version=\"0.1\" byte_order=\"LittleEndian\">\n";
    v << "  <ImageData WholeExtent=\"0 " << (nx - 1) << " 0 " << (ny - 1) << " 0 " << (nz - 1)
      << "\" Origin=\"0 0 0\" Spacing=\"1 1 1\">\n";
    v << "    <Piece Extent=\"0 " << (nx - 1) << " 0 " << (ny - 1) << " 0 " << (nz - 1) << "\">\n";
    v << "      <PointData Scalars=\"" << names.front() << "\">\n";
    uint64_t offset = 0;
    for (const auto &name : names) {
        v << "        <DataArray type=\"Float32\" Name=\"" << name
          << "\" NumberOfComponents=\"1\" format=\"appended\" offset=\"" << offset << "\"/>\n";
        offset += sizeof(uint32_t) + nbytes;
    }
    v << "      </PointData>\n      <CellData/>\n    </Piece>\n  </ImageData>\n";
    v << "  <AppendedData encoding=\"raw\">\n_";
    for (size_t i = 0; i < names.size(); ++i) {
        const uint32_t n32 = static_cast<uint32_t>(nbytes);
        v.write(reinterpret_cast<const char *>(&n32), sizeof n32);
        v.write(reinterpret_cast<const char *>(data[i]), std::streamsize(nbytes));
    }
    v << "\n  </AppendedData>\n</VTKFile>\n";
    if (!v) { err = "write failed: " + vti; return PFLBM_ERR_IO; }
    return PFLBM_OK;
}

// Waits for the previous background write; reports its failure once.
int join_writer(pflbm_sim *s) {
    if (s->writer.joinable()) s->writer.join();
    if (s->writer_rc) {
        const int rc = s->writer_rc;
        s->writer_rc = 0;
        return fail(rc, s->writer_err);
    }
    return PFLBM_OK;
}

void free_pinned(pflbm_sim *s) {
    for (float *p : s->pinned) cudaFreeHost(p);
    s->pinned.clear();
}

// Frees everything a simulation holds, also one that pflbm_create left
// half built after an error.
void release_resources(pflbm_sim *s) {
    cudaSetDevice(s->device);
    if (s->stream) cudaStreamSynchronize(s->stream);
    if (s->writer.joinable()) s->writer.join();
    free_pinned(s);
    destroy_graphs(s);
    if (s->dev_diag) cudaFree(s->dev_diag);
    s->dev_diag = nullptr;
    s->eng.reset();
    if (s->stream) cudaStreamDestroy(s->stream);
    s->stream = nullptr;
}

}  // namespace

extern "C" {

int pflbm_abi_version(void) { return PFLBM_ABI_VERSION; }

const char *pflbm_last_error(void) { return g_err.c_str(); }

int pflbm_config_reference(pflbm_config *c, int32_t flow_case, int32_t velocity_set) {
    if (!c) return fail(PFLBM_ERR_INVALID_ARG, "null config");
    if (flow_case != PFLBM_CASE_DROPLET && flow_case != PFLBM_CASE_JET)
        return fail(PFLBM_ERR_INVALID_ARG, "unknown flow case");
    if (velocity_set != PFLBM_VS_D3Q19 && velocity_set != PFLBM_VS_D3Q27)
        return fail(PFLBM_ERR_INVALID_ARG, "unknown velocity set");
    std::memset(c, 0, sizeof(*c));
    c->struct_size = sizeof(pflbm_config);
    c->flow_case = flow_case;
    c->velocity_set = velocity_set;
    c->storage = PFLBM_STORAGE_FP32;
    c->interface_width = 4.0f;
    // physics::gamma = kappa / cs2, kappa = 4 * cs2 (tau_g - 1/2) / W with
    // tau_g = 1 and the D3Q7 cs2 = 1/4 (constants.cuh:104-108, 131-134)
    const float diff_int = 0.25f * (1.0f - 0.5f);
    const float kappa = 4.0f * diff_int / c->interface_width;
    c->gamma = kappa / 0.25f;
    c->droplet_x_stretch = 2.0f;  // initialConditions.cu:74
    c->sponge_gain = 100.0f;      // sponge::K_gain
    c->sponge_cells = -1;         // nz / 12
    c->inflow_noise = PFLBM_NOISE_GAUSSIAN_UXY;
    c->noise_amp = 0.08f;         // sigma_u = 0.08 u_inf
    c->device = -1;
    if (flow_case == PFLBM_CASE_JET) {
        // constants.cuh:80-109
        c->nx = 64; c->ny = 64; c->nz = 128;
        c->diam = 10; c->radius = 5;
        c->u_inf = 0.05f;
        c->reynolds_water = 5000.0f;
        c->reynolds_oil = 5000.0f;
        c->sigma = (c->u_inf * c->u_inf * static_cast<float>(c->diam)) / 500.0f;
    } else {
        // constants.cuh:111-141
        c->nx = 128; c->ny = 128; c->nz = 128;
        c->radius = 35; c->diam = 70;
        c->u_inf = 0.0f;
        c->sigma = 0.03f;
        c->tau = 0.55f;
    }
    return PFLBM_OK;
}

int pflbm_create(const pflbm_config *cfg, pflbm_sim **out) {
    NvtxRange nvtx_("pflbm_create");
    if (!cfg || !out) return fail(PFLBM_ERR_INVALID_ARG, "null argument");
    *out = nullptr;
    int rc = validate(*cfg);
    if (rc) return rc;
    std::unique_ptr<pflbm_sim> s(new (std::nothrow) pflbm_sim());
    if (!s) return fail(PFLBM_ERR_OUT_OF_MEMORY, "host allocation failed");
    s->cfg = *cfg;
    // device: explicit, else $GPU_INDEX (hostFunctions.cuh:117-150), else 0
    int dev = cfg->device;
    if (dev < 0) {
        dev = 0;
        if (const char *e = std::getenv("GPU_INDEX")) {
            char *end = nullptr;
            const long v = std::strtol(e, &end, 10);
            if (end != e && v >= 0) dev = int(v);
        }
    }
    cudaError_t e = cudaSetDevice(dev);
    if (e != cudaSuccess) return cuda_fail(e, "cudaSetDevice");
    s->device = dev;
    derive(*cfg, s->hp);
    s->hp.zchunk = pick_zchunk(*cfg, dev);
    const bool jet = cfg->flow_case == PFLBM_CASE_JET;
    Engine *eng = nullptr;
    switch (cfg->storage) {
        case PFLBM_STORAGE_FP32: eng = pflbm::make_engine_fp32(cfg->velocity_set, jet, s->hp, cfg->flags); break;
        case PFLBM_STORAGE_FP64: eng = pflbm::make_engine_fp64(cfg->velocity_set, jet, s->hp, cfg->flags); break;
        case PFLBM_STORAGE_FP16: eng = pflbm::make_engine_fp16(cfg->velocity_set, jet, s->hp, cfg->flags); break;
        case PFLBM_STORAGE_BF16: eng = pflbm::make_engine_bf16(cfg->velocity_set, jet, s->hp, cfg->flags); break;
    }
    if (!eng) return fail(PFLBM_ERR_OUT_OF_MEMORY, "engine allocation failed");
    s->eng.reset(eng);
    // from here on an error releases what was built so far
    auto abandon = [&](int code) {
        release_resources(s.get());
        return code;
    };
    std::string err;
    rc = s->eng->allocate(err);
    if (rc) return abandon(fail(rc, err));
    e = cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking);
    if (e != cudaSuccess) return abandon(cuda_fail(e, "cudaStreamCreate"));
    e = cudaMalloc(&s->dev_diag, sizeof(double) * 16);
    if (e != cudaSuccess) return abandon(cuda_fail(e, "cudaMalloc diag"));
    const int counts[3] = {1, 2, kChunk};
    for (int par = 0; par < 2; ++par)
        for (int k = 0; k < 3; ++k) {
            rc = capture(s.get(), par, counts[k], &s->graphs[par][k]);
            if (rc) return abandon(rc);
        }
    *out = s.release();
    return PFLBM_OK;
}

int pflbm_init(pflbm_sim *s) {
    NvtxRange nvtx_("pflbm_init");
    if (!s) return fail(PFLBM_ERR_INVALID_ARG, "null simulation");
    cudaSetDevice(s->device);
    s->eng->reset_counters(s->stream);
    s->eng->enqueue_init_fields(s->stream);
    s->eng->enqueue_init_distros(s->stream);
    cudaError_t e = cudaStreamSynchronize(s->stream);
    if (e != cudaSuccess) return cuda_fail(e, "pflbm_init");
    s->parity = 0;
    s->step = 0;
    s->cache_step = 0;
    s->distros_dirty = false;
    s->initialized = true;
    return PFLBM_OK;
}

int pflbm_set_initial_field(pflbm_sim *s, int32_t id, const float *src, size_t bytes) {
    if (!s || !src) return fail(PFLBM_ERR_INVALID_ARG, "null argument");
    if (!s->initialized || s->step != 0) return fail(PFLBM_ERR_STATE, "initial fields can only be set at step 0");
    if (id != PFLBM_FIELD_PHI && id != PFLBM_FIELD_UX && id != PFLBM_FIELD_UY && id != PFLBM_FIELD_UZ &&
        id != PFLBM_FIELD_RHO)
        return fail(PFLBM_ERR_INVALID_ARG, "only rho, ux, uy, uz, phi can be set");
    const uint64_t N = s->hp.N;
    if (bytes < N * sizeof(float)) return fail(PFLBM_ERR_INVALID_ARG, "source buffer too small");
    cudaSetDevice(s->device);
    const int rb = s->eng->real_bytes();
    unsigned char *dst = static_cast<unsigned char *>(s->eng->macro_ptr()) + size_t(id) * N * rb;
    cudaError_t e;
    if (rb == 4) {
        e = cudaMemcpy(dst, src, N * 4, cudaMemcpyHostToDevice);
    } else {
        std::unique_ptr<double[]> tmp(new (std::nothrow) double[N]);
        if (!tmp) return fail(PFLBM_ERR_OUT_OF_MEMORY, "host conversion buffer");
        for (uint64_t i = 0; i < N; ++i) tmp[i] = src[i];
        e = cudaMemcpy(dst, tmp.get(), N * 8, cudaMemcpyHostToDevice);
    }
    if (e != cudaSuccess) return cuda_fail(e, "cudaMemcpy H2D");
    s->distros_dirty = true;
    s->cache_step = 0;
    return PFLBM_OK;
}

int pflbm_step_async(pflbm_sim *s, uint64_t n) {
    NvtxRange nvtx_("pflbm_step");
    if (!s) return fail(PFLBM_ERR_INVALID_ARG, "null simulation");
    if (!s->initialized) return fail(PFLBM_ERR_STATE, "pflbm_init has not been called");
    cudaSetDevice(s->device);
    flush_initial(s);
    uint64_t left = n;
    while (left > 0) {
        int k;
        if (left >= uint64_t(kChunk)) k = 2;
        else if (left >= 2) k = 1;
        else k = 0;
        const int steps = k == 2 ? kChunk : (k == 1 ? 2 : 1);
        cudaError_t e = cudaGraphLaunch(s->graphs[s->parity][k], s->stream);
        if (e != cudaSuccess) return cuda_fail(e, "cudaGraphLaunch");
        if (steps & 1) s->parity ^= 1;
        s->step += steps;
        left -= steps;
    }
    return PFLBM_OK;
}

int pflbm_synchronize(pflbm_sim *s) {
    if (!s) return fail(PFLBM_ERR_INVALID_ARG, "null simulation");
    cudaError_t e = cudaStreamSynchronize(s->stream);
    if (e != cudaSuccess) return cuda_fail(e, "cudaStreamSynchronize");
    int rc = check_device_error(s);
    if (rc) return rc;
    return join_writer(s);
}

int pflbm_step(pflbm_sim *s, uint64_t n) {
    if (!s) return fail(PFLBM_ERR_INVALID_ARG, "null simulation");
    if (s->wd_interval == 0) {
        int rc = pflbm_step_async(s, n);
        if (rc) return rc;
        return pflbm_synchronize(s);
    }
    // watchdog: FP64 diagnostics at every multiple of the interval
    uint64_t left = n;
    while (left > 0) {
        const uint64_t k = std::min<uint64_t>(left, s->wd_interval - s->step % s->wd_interval);
        int rc = pflbm_step_async(s, k);
        if (rc) return rc;
        left -= k;
        rc = pflbm_synchronize(s);
        if (rc) return rc;
        if (s->step % s->wd_interval == 0) {
            pflbm_diag d;
            rc = pflbm_reduce(s, &d);  // PFLBM_ERR_DIVERGED on NaN/Inf
            if (rc) return rc;
            if (s->wd_max_drift > 0.0 && s->wd_mass0 != 0.0) {
                const double drift = std::fabs(d.phi_mass / s->wd_mass0 - 1.0);
                if (drift > s->wd_max_drift)
                    return fail(PFLBM_ERR_DIVERGED, "phi mass drift " + std::to_string(drift) + " at step " +
                                                        std::to_string(s->step) + " exceeds " +
                                                        std::to_string(s->wd_max_drift));
            }
        }
    }
    return PFLBM_OK;
}

int pflbm_set_watchdog(pflbm_sim *s, uint64_t interval_steps, double max_phi_mass_drift) {
    if (!s || max_phi_mass_drift < 0.0) return fail(PFLBM_ERR_INVALID_ARG, "bad argument");
    if (!s->initialized) return fail(PFLBM_ERR_STATE, "pflbm_init has not been called");
    s->wd_interval = interval_steps;
    s->wd_max_drift = max_phi_mass_drift;
    s->wd_mass0 = 0.0;
    if (interval_steps > 0 && max_phi_mass_drift > 0.0) {
        pflbm_diag d;
        const int rc = pflbm_reduce(s, &d);
        if (rc) return rc;
        s->wd_mass0 = d.phi_mass;
    }
    return PFLBM_OK;
}

int pflbm_step_profiled(pflbm_sim *s, uint64_t n, double *total_ms, double *kernel_ms, int32_t nk) {
    NvtxRange nvtx_("pflbm_step_profiled");
    if (!s || !total_ms || (nk > 0 && !kernel_ms)) return fail(PFLBM_ERR_INVALID_ARG, "null argument");
    if (!s->initialized) return fail(PFLBM_ERR_STATE, "pflbm_init has not been called");
    cudaSetDevice(s->device);
    flush_initial(s);
    constexpr int kEv = 4;  // start/end of each of the two kernels
    std::vector<cudaEvent_t> ev(size_t(n) * kEv + 2, nullptr);
    for (auto &x : ev)
        if (cudaEventCreate(&x) != cudaSuccess) {
            for (auto &y : ev)
                if (y) cudaEventDestroy(y);
            return cuda_fail(cudaGetLastError(), "cudaEventCreate");
        }
    cudaEventRecord(ev[0], s->stream);
    for (uint64_t i = 0; i < n; ++i) {
        s->eng->enqueue_step(s->parity, s->stream, &ev[1 + i * kEv]);
        s->parity ^= 1;
        s->step += 1;
    }
    cudaEventRecord(ev.back(), s->stream);
    cudaError_t e = cudaEventSynchronize(ev.back());
    double sums[2] = {0.0, 0.0};
    float ms = 0.0f;
    if (e == cudaSuccess) {
        for (uint64_t i = 0; i < n; ++i)
            for (int k = 0; k < 2; ++k) {
                cudaEventElapsedTime(&ms, ev[1 + i * kEv + 2 * k], ev[1 + i * kEv + 2 * k + 1]);
                sums[k] += ms;
            }
        cudaEventElapsedTime(&ms, ev[0], ev.back());
        *total_ms = ms;
    }
    for (auto &x : ev) cudaEventDestroy(x);
    if (e != cudaSuccess) return cuda_fail(e, "pflbm_step_profiled");
    for (int k = 0; k < nk; ++k) kernel_ms[k] = k < 2 ? sums[k] : 0.0;
    return check_device_error(s);
}

int pflbm_current_step(const pflbm_sim *s, uint64_t *step) {
    if (!s || !step) return fail(PFLBM_ERR_INVALID_ARG, "null argument");
    *step = s->step;
    return PFLBM_OK;
}

int pflbm_get_field(pflbm_sim *s, int32_t id, void *host, size_t bytes) {
    if (!s) return fail(PFLBM_ERR_INVALID_ARG, "null simulation");
    cudaSetDevice(s->device);
    return get_field_impl(s, id, host, bytes, false);
}

int pflbm_get_field_f64(pflbm_sim *s, int32_t id, double *host, size_t bytes) {
    if (!s) return fail(PFLBM_ERR_INVALID_ARG, "null simulation");
    cudaSetDevice(s->device);
    return get_field_impl(s, id, host, bytes, true);
}

int pflbm_reduce(pflbm_sim *s, pflbm_diag *d) {
    NvtxRange nvtx_("pflbm_reduce");
    if (!s || !d) return fail(PFLBM_ERR_INVALID_ARG, "null argument");
    if (!s->initialized) return fail(PFLBM_ERR_STATE, "pflbm_init has not been called");
    cudaSetDevice(s->device);
    int rc = ensure_cache(s);
    if (rc) return rc;
    s->eng->enqueue_reduce(s->stream, s->dev_diag);
    double r[12];
    cudaError_t e = cudaMemcpyAsync(r, s->dev_diag, sizeof r, cudaMemcpyDeviceToHost, s->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s->stream);
    if (e != cudaSuccess) return cuda_fail(e, "pflbm_reduce");
    std::memset(d, 0, sizeof(*d));
    d->step = s->step;
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
    if (d->nonfinite > 0) return fail(PFLBM_ERR_DIVERGED, "non-finite values in rho, u or phi");
    return PFLBM_OK;
}

int pflbm_set_closure(pflbm_sim *s, const float *blob, float strength) {
    if (!s) return fail(PFLBM_ERR_INVALID_ARG, "null simulation");
    if (blob && !(strength >= 0.0f)) return fail(PFLBM_ERR_INVALID_ARG, "strength must be >= 0");
    cudaSetDevice(s->device);
    cudaError_t e = cudaStreamSynchronize(s->stream);
    if (e != cudaSuccess) return cuda_fail(e, "cudaStreamSynchronize");
    std::vector<float> w;
    if (blob) {
        // the network runs with BF16 weights (round to nearest even); the
        // normalisation constants, out_scale and strength stay FP32
        w.assign(blob, blob + pflbm::kMlpBlobFloats);
        for (int i = 0; i < pflbm::kMlpParamFloats; ++i) {
            uint32_t u;
            std::memcpy(&u, &w[i], 4);
            if ((u & 0x7f800000u) != 0x7f800000u) u += 0x7fffu + ((u >> 16) & 1u);
            u &= 0xffff0000u;
            std::memcpy(&w[i], &u, 4);
        }
        w[pflbm::kMlpBlobFloats - 1] = strength;
    }
    std::string err;
    int rc = s->eng->set_closure(blob ? w.data() : nullptr, err);
    if (rc) return fail(rc, err);
    // steps are captured with the collide kernel of the current mode
    destroy_graphs(s);
    const int counts[3] = {1, 2, kChunk};
    for (int par = 0; par < 2; ++par)
        for (int k = 0; k < 3; ++k) {
            rc = capture(s, par, counts[k], &s->graphs[par][k]);
            if (rc) return rc;
        }
    return PFLBM_OK;
}


int pflbm_set_closure_mixing(pflbm_sim *s, float inv_schmidt) {
    if (!s) return fail(PFLBM_ERR_INVALID_ARG, "null simulation");
    if (!(inv_schmidt >= 0.0f) || !std::isfinite(inv_schmidt))
        return fail(PFLBM_ERR_INVALID_ARG, "inv_schmidt must be finite and >= 0");
    cudaSetDevice(s->device);
    cudaError_t e = cudaStreamSynchronize(s->stream);
    if (e != cudaSuccess) return cuda_fail(e, "cudaStreamSynchronize");
    std::string err;
    const int rc = s->eng->set_closure_mixing(inv_schmidt, err);
    return rc ? fail(rc, err) : PFLBM_OK;
}

namespace {
int write_output_async_impl(pflbm_sim *s, const char *dir, const int32_t *ids, int32_t n) {
    if (!s || !dir || (!ids && n > 0) || n < 0) return fail(PFLBM_ERR_INVALID_ARG, "bad argument");
    for (int i = 0; i < n; ++i)
        if (ids[i] < 0 || ids[i] >= PFLBM_FIELD_COUNT) return fail(PFLBM_ERR_INVALID_ARG, "bad field id");
    int rc = join_writer(s);  // the staging buffers are free again
    if (rc) return rc;
    std::string d(dir);
    if (!d.empty() && d.back() != '/') d.push_back('/');
    if (!make_dirs(d)) return fail(PFLBM_ERR_IO, "cannot create " + d);
    const uint64_t N = s->hp.N;
    cudaSetDevice(s->device);
    while (s->pinned.size() < size_t(n)) {
        float *p = nullptr;
        if (cudaMallocHost(&p, N * sizeof(float)) != cudaSuccess) {
            cudaGetLastError();
            return fail(PFLBM_ERR_OUT_OF_MEMORY, "cudaMallocHost (output staging)");
        }
        s->pinned.push_back(p);
    }
    // device -> page-locked host copies now (the analysis of the last step
    // runs once); the file writes overlap with whatever the caller does next.
    // No exception may cross the C ABI: a failed host allocation anywhere
    // below (vectors, strings, the copy of the job into the thread) becomes
    // PFLBM_ERR_OUT_OF_MEMORY.
    try {
        std::vector<std::string> names;
        std::vector<const float *> data;
        for (int i = 0; i < n; ++i) {
            rc = pflbm_get_field(s, ids[i], s->pinned[i], N * sizeof(float));
            if (rc) return rc;
            names.push_back(kFieldNames[ids[i]]);
            data.push_back(s->pinned[i]);
        }
        const std::string suffix = step6(s->step > 0 ? s->step - 1 : 0);
        const uint32_t nx = s->hp.nx, ny = s->hp.ny, nz = s->hp.nz;
        auto job = [s, d, suffix, names, data, N, nx, ny, nz]() {
            std::string err;
            const int r = write_step_files(d, suffix, names, data, N, nx, ny, nz, err);
            s->writer_err = err;
            s->writer_rc = r;
        };
        try {
            s->writer = std::thread(job);  // a copy: `job` stays whole for the fallback
        } catch (const std::system_error &) {
            // no thread could be started: write in the calling thread instead
            job();
            return join_writer(s);
        }
    } catch (...) {
        return fail(PFLBM_ERR_OUT_OF_MEMORY, "host allocation failed in the output writer");
    }
    return PFLBM_OK;
}
}  // namespace

int pflbm_write_output_async(pflbm_sim *s, const char *dir, const int32_t *ids, int32_t n) {
    NvtxRange nvtx_("pflbm_write_output");
    // no exception crosses the C ABI (the path string, the staging list)
    try {
        return write_output_async_impl(s, dir, ids, n);
    } catch (...) {
        return fail(PFLBM_ERR_OUT_OF_MEMORY, "host allocation failed in the output writer");
    }
}

int pflbm_write_output(pflbm_sim *s, const char *dir, const int32_t *ids, int32_t n) {
    int rc = pflbm_write_output_async(s, dir, ids, n);
    if (rc) return rc;
    return join_writer(s);
}

// Checkpoint file: header, both ping-pong population buffers (the one the
// next step reads first), both phi buffers (ghost values included), the
// derived averages when enabled. Both buffers are kept so that the slots no
// step rewrites and the readback of the last completed step stay exact.
namespace {
struct CkptHeader {
    char magic[8];        // "PFLBMCK1"
    uint32_t abi;
    uint32_t header_bytes;
    pflbm_config cfg;
    uint64_t step;
    uint64_t f_bytes, phi_bytes, avg_bytes;
};

int write_blob(std::ofstream &o, const void *dev, uint64_t bytes) {
    constexpr size_t kChunkBytes = size_t(1) << 26;
    std::unique_ptr<char[]> h(new (std::nothrow) char[kChunkBytes]);
    if (!h) return fail(PFLBM_ERR_OUT_OF_MEMORY, "checkpoint staging buffer");
    for (uint64_t off = 0; off < bytes; off += kChunkBytes) {
        const size_t n = size_t(std::min<uint64_t>(kChunkBytes, bytes - off));
        cudaError_t e = cudaMemcpy(h.get(), static_cast<const char *>(dev) + off, n, cudaMemcpyDeviceToHost);
        if (e != cudaSuccess) return cuda_fail(e, "checkpoint D2H");
        o.write(h.get(), std::streamsize(n));
        if (!o) return fail(PFLBM_ERR_IO, "checkpoint write failed");
    }
    return PFLBM_OK;
}

int read_blob(std::ifstream &in, void *dev0, void *dev1, uint64_t bytes) {
    constexpr size_t kChunkBytes = size_t(1) << 26;
    std::unique_ptr<char[]> h(new (std::nothrow) char[kChunkBytes]);
    if (!h) return fail(PFLBM_ERR_OUT_OF_MEMORY, "checkpoint staging buffer");
    for (uint64_t off = 0; off < bytes; off += kChunkBytes) {
        const size_t n = size_t(std::min<uint64_t>(kChunkBytes, bytes - off));
        in.read(h.get(), std::streamsize(n));
        if (!in) return fail(PFLBM_ERR_IO, "checkpoint truncated");
        for (void *d : {dev0, dev1}) {
            if (!d) continue;
            cudaError_t e = cudaMemcpy(static_cast<char *>(d) + off, h.get(), n, cudaMemcpyHostToDevice);
            if (e != cudaSuccess) return cuda_fail(e, "checkpoint H2D");
        }
    }
    return PFLBM_OK;
}
}  // namespace

int pflbm_save_checkpoint(pflbm_sim *s, const char *path) {
    if (!s || !path) return fail(PFLBM_ERR_INVALID_ARG, "null argument");
    if (!s->initialized) return fail(PFLBM_ERR_STATE, "pflbm_init has not been called");
    cudaSetDevice(s->device);
    flush_initial(s);
    cudaError_t e = cudaStreamSynchronize(s->stream);
    if (e != cudaSuccess) return cuda_fail(e, "checkpoint sync");
    CkptHeader h{};
    std::memcpy(h.magic, "PFLBMCK1", 8);
    h.abi = PFLBM_ABI_VERSION;
    h.header_bytes = sizeof(CkptHeader);
    h.cfg = s->cfg;
    h.step = s->step;
    h.f_bytes = s->eng->f_bytes();
    h.phi_bytes = s->eng->phi_bytes();
    h.avg_bytes = s->eng->avg_bytes();
    std::ofstream o(path, std::ios::binary | std::ios::trunc);
    if (!o) return fail(PFLBM_ERR_IO, std::string("cannot open ") + path);
    o.write(reinterpret_cast<const char *>(&h), sizeof h);
    int rc = write_blob(o, s->eng->f_ptr(s->parity), h.f_bytes);
    if (!rc) rc = write_blob(o, s->eng->f_ptr(s->parity ^ 1), h.f_bytes);
    if (!rc) rc = write_blob(o, s->eng->phi_ptr(s->parity), h.phi_bytes);
    if (!rc) rc = write_blob(o, s->eng->phi_ptr(s->parity ^ 1), h.phi_bytes);
    if (!rc && h.avg_bytes) rc = write_blob(o, s->eng->avg_ptr(), h.avg_bytes);
    return rc;
}

int pflbm_load_checkpoint(pflbm_sim *s, const char *path) {
    if (!s || !path) return fail(PFLBM_ERR_INVALID_ARG, "null argument");
    cudaSetDevice(s->device);
    std::ifstream in(path, std::ios::binary);
    if (!in) return fail(PFLBM_ERR_IO, std::string("cannot open ") + path);
    CkptHeader h{};
    in.read(reinterpret_cast<char *>(&h), sizeof h);
    if (!in || std::memcmp(h.magic, "PFLBMCK1", 8) != 0 || h.header_bytes != sizeof(CkptHeader))
        return fail(PFLBM_ERR_IO, "not a pflbm checkpoint");
    const pflbm_config &a = h.cfg, &b = s->cfg;
    if (a.nx != b.nx || a.ny != b.ny || a.nz != b.nz || a.velocity_set != b.velocity_set ||
        a.flow_case != b.flow_case || a.storage != b.storage || h.f_bytes != s->eng->f_bytes() ||
        h.phi_bytes != s->eng->phi_bytes() || h.avg_bytes != s->eng->avg_bytes())
        return fail(PFLBM_ERR_INVALID_ARG, "checkpoint does not match this simulation's grid, lattice or storage");
    cudaStreamSynchronize(s->stream);
    int rc = read_blob(in, s->eng->f_ptr(0), nullptr, h.f_bytes);
    if (!rc) rc = read_blob(in, s->eng->f_ptr(1), nullptr, h.f_bytes);
    if (!rc) rc = read_blob(in, s->eng->phi_ptr(0), nullptr, h.phi_bytes);
    if (!rc) rc = read_blob(in, s->eng->phi_ptr(1), nullptr, h.phi_bytes);
    if (!rc && h.avg_bytes) rc = read_blob(in, s->eng->avg_ptr(), nullptr, h.avg_bytes);
    if (rc) return rc;
    s->eng->reset_counters(s->stream);
    s->eng->set_counter(0, h.step, s->stream);
    s->parity = 0;
    s->step = h.step;
    s->cache_step = -1;
    s->distros_dirty = false;
    s->initialized = true;
    return PFLBM_OK;
}

int pflbm_device_bytes(const pflbm_sim *s, uint64_t *bytes) {
    if (!s || !bytes) return fail(PFLBM_ERR_INVALID_ARG, "null argument");
    *bytes = s->eng->device_bytes();
    return PFLBM_OK;
}

int pflbm_uses_tma(const pflbm_sim *s, int32_t *flag) {
    if (!s || !flag) return fail(PFLBM_ERR_INVALID_ARG, "null argument");
    *flag = s->eng->uses_tma() ? 1 : 0;
    return PFLBM_OK;
}

int pflbm_collide_variant(const pflbm_sim *s, int32_t *variant) {
    if (!s || !variant) return fail(PFLBM_ERR_INVALID_ARG, "null argument");
    *variant = s->eng->collide_variant();
    return PFLBM_OK;
}

int pflbm_kernels_per_step(const pflbm_sim *s, int32_t *count) {
    if (!s || !count) return fail(PFLBM_ERR_INVALID_ARG, "null argument");
    *count = s->eng->kernels_per_step();
    return PFLBM_OK;
}

int pflbm_destroy(pflbm_sim *s) {
    if (!s) return PFLBM_OK;
    release_resources(s);
    delete s;
    return PFLBM_OK;
}

}  // extern "C"
