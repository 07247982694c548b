// ref_runner.cpp - runs the reference's own CUDA kernels (a cubin compiled
// from the reference's src/main.cu by oracle/ref_build.py) on the GPU.
//
// TEST INFRASTRUCTURE ONLY: the checker that pins the CPU oracle and the
// library to the reference's CUDA build, and the "reference CUDA build"
// timing baseline. It replays src/main.cu:35-215 with the CUDA driver API:
// allocation and zeroing of every LBMFields array
// (src/fieldAllocate/FieldAllocate.cuh:102-122), the initial-condition
// kernels (src/main.cu:114-116), then per step the five graph kernels
// (src/cuda/CUDAGraph.cuh:44-51) and, for the jet, callInflow(t) and
// callOutflow (src/flowCase/Jet.cuh:62-63), with the per-step stream
// synchronisation of src/main.cu:172.
//
//   ref_runner <cubin> <jet|droplet> <Q> <nx> <ny> <nz> <fp16 0|1> <steps> <outdir|-> [time]
//
// With an outdir, the 18 scalar fields are written there as raw float32
// (<name>.bin, nx*ny*nz values, x fastest). With "time", one JSON line with
// the wall-clock MLUPS of the step loop (as src/main.cu:201-205 computes it)
// is printed.
#include <cuda.h>

#include <chrono>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

namespace {

void check(CUresult r, const char *what) {
    if (r != CUDA_SUCCESS) {
        const char *s = nullptr;
        cuGetErrorString(r, &s);
        std::fprintf(stderr, "ref_runner: %s failed: %s\n", what, s ? s : "?");
        std::exit(1);
    }
}

// LBMFields with TIME_AVERAGE = REYNOLDS_MOMENTS = VORTICITY_FIELDS =
// PASSIVE_SCALAR = 0 (src/LBMIncludes.cuh:58-117): 18 scalar arrays, f, g.
struct Fields {
    CUdeviceptr p[20];
};

const char *kNames[18] = {"rho", "ux", "uy", "uz", "pxx", "pyy", "pzz", "pxy", "pxz",
                          "pyz", "phi", "normx", "normy", "normz", "ind", "fsx", "fsy", "fsz"};

unsigned div_up(unsigned a, unsigned b) { return (a + b - 1) / b; }

}  // namespace

int main(int argc, char **argv) {
    if (argc < 10) {
        std::fprintf(stderr, "usage: %s <cubin> <jet|droplet> <Q> <nx> <ny> <nz> <fp16> <steps> <outdir|-> [time]\n",
                     argv[0]);
        return 2;
    }
    const std::string cubin = argv[1];
    const bool jet = std::string(argv[2]) == "jet";
    const int Q = std::atoi(argv[3]);
    const unsigned nx = std::atoi(argv[4]), ny = std::atoi(argv[5]), nz = std::atoi(argv[6]);
    const bool fp16 = std::atoi(argv[7]) != 0;
    const long steps = std::atol(argv[8]);
    const std::string outdir = argv[9];
    const bool timing = argc > 10 && std::string(argv[10]) == "time";
    if ((Q != 19 && Q != 27) || nx < 4 || ny < 4 || nz < 4 || steps < 0) {
        std::fprintf(stderr, "ref_runner: bad arguments\n");
        return 2;
    }
    const size_t N = size_t(nx) * ny * nz;

    int dev = 0;
    if (const char *e = std::getenv("GPU_INDEX")) dev = std::atoi(e);
    check(cuInit(0), "cuInit");
    CUdevice d;
    check(cuDeviceGet(&d, dev), "cuDeviceGet");
    CUcontext ctx;
    check(cuDevicePrimaryCtxRetain(&ctx, d), "cuDevicePrimaryCtxRetain");
    check(cuCtxSetCurrent(ctx), "cuCtxSetCurrent");
    CUmodule mod;
    check(cuModuleLoad(&mod, cubin.c_str()), "cuModuleLoad");

    auto fn = [&](const char *name) {
        CUfunction f;
        check(cuModuleGetFunction(&f, mod, name), name);
        return f;
    };
    // Itanium-mangled names of the reference's kernels
    CUfunction k_density = fn("_ZN3lbm17setInitialDensityE9LBMFields");
    CUfunction k_case = fn(jet ? "_ZN3lbm6setJetE9LBMFields" : "_ZN3lbm10setDropletE9LBMFields");
    CUfunction k_distros = fn("_ZN3lbm10setDistrosE9LBMFields");
    CUfunction k_phase = fn("_ZN5phase12computePhaseE9LBMFields");
    CUfunction k_normals = fn("_ZN5phase14computeNormalsE9LBMFields");
    CUfunction k_forces = fn("_ZN5phase13computeForcesE9LBMFields");
    CUfunction k_moments = fn("_ZN3lbm14computeMomentsE9LBMFields");
    CUfunction k_collide = fn("_ZN3lbm13streamCollideE9LBMFields");
    CUfunction k_inflow = jet ? fn("_ZN3lbm10callInflowE9LBMFieldsj") : nullptr;
    CUfunction k_outflow = jet ? fn("_ZN3lbm11callOutflowE9LBMFields") : nullptr;

    Fields F{};
    for (int i = 0; i < 18; ++i) {
        check(cuMemAlloc(&F.p[i], N * sizeof(float)), "cuMemAlloc");
        check(cuMemsetD8(F.p[i], 0, N * sizeof(float)), "cuMemset");
    }
    const size_t fbytes = N * size_t(Q) * (fp16 ? 2 : 4);
    check(cuMemAlloc(&F.p[18], fbytes), "cuMemAlloc f");
    check(cuMemsetD8(F.p[18], 0, fbytes), "cuMemset f");
    check(cuMemAlloc(&F.p[19], N * 7 * sizeof(float)), "cuMemAlloc g");
    check(cuMemsetD8(F.p[19], 0, N * 7 * sizeof(float)), "cuMemset g");

    CUstream st;
    check(cuStreamCreate(&st, CU_STREAM_NON_BLOCKING), "cuStreamCreate");
    // launch geometry of src/main.cu:89-104
    const unsigned gx = div_up(nx, 32), gy = div_up(ny, 4), gz = div_up(nz, 4);
    void *args1[] = {&F};
    auto launch3 = [&](CUfunction f) {
        check(cuLaunchKernel(f, gx, gy, gz, 32, 4, 4, 0, st, args1, nullptr), "cuLaunchKernel");
    };
    launch3(k_density);
    if (jet)
        check(cuLaunchKernel(k_case, gx, gy, gz, 32, 4, 4, 0, st, args1, nullptr), "setJet");
    else
        launch3(k_case);
    launch3(k_distros);
    check(cuStreamSynchronize(st), "init");

    // graph of the five per-step kernels (src/cuda/CUDAGraph.cuh:41-57)
    CUgraph graph;
    CUgraphExec exec;
    check(cuStreamBeginCapture(st, CU_STREAM_CAPTURE_MODE_GLOBAL), "capture");
    launch3(k_phase);
    launch3(k_normals);
    launch3(k_forces);
    launch3(k_moments);
    launch3(k_collide);
    check(cuStreamEndCapture(st, &graph), "end capture");
    check(cuGraphInstantiate(&exec, graph, 0), "instantiate");

    const auto t0 = std::chrono::high_resolution_clock::now();
    for (long s = 0; s < steps; ++s) {
        check(cuGraphLaunch(exec, st), "graph launch");
        if (jet) {
            unsigned t = unsigned(s);
            void *args2[] = {&F, &t};
            check(cuLaunchKernel(k_inflow, gx, gy, 1, 32, 4, 1, 0, st, args2, nullptr), "inflow");
            check(cuLaunchKernel(k_outflow, gx, gy, 1, 32, 4, 1, 0, st, args1, nullptr), "outflow");
        }
        check(cuStreamSynchronize(st), "step");
    }
    const auto t1 = std::chrono::high_resolution_clock::now();
    const double sec = std::chrono::duration<double>(t1 - t0).count();

    if (timing)
        std::printf("{\"ref_mlups\": %.3f, \"seconds\": %.6f, \"steps\": %ld, \"nodes\": %zu}\n",
                    steps > 0 ? double(N) * steps / sec / 1e6 : 0.0, sec, steps, N);
    if (outdir != "-") {
        std::vector<float> h(N);
        for (int i = 0; i < 18; ++i) {
            check(cuMemcpyDtoH(h.data(), F.p[i], N * sizeof(float)), "DtoH");
            const std::string path = outdir + "/" + kNames[i] + ".bin";
            FILE *fp = std::fopen(path.c_str(), "wb");
            if (!fp) {
                std::fprintf(stderr, "ref_runner: cannot write %s\n", path.c_str());
                return 1;
            }
            std::fwrite(h.data(), sizeof(float), N, fp);
            std::fclose(fp);
        }
    }
    cuGraphExecDestroy(exec);
    cuGraphDestroy(graph);
    for (auto &p : F.p) cuMemFree(p);
    cuStreamDestroy(st);
    cuModuleUnload(mod);
    cuDevicePrimaryCtxRelease(d);
    return 0;
}
