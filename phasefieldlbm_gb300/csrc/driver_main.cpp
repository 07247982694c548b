// driver_main.cpp - pflbm_run, the drop-in for the reference's executable.
//
//   pflbm_run <JET|DROPLET> <D3Q19|D3Q27> <ID> [options]
//
// Same arguments and output layout as the reference's main (src/main.cu:35-215):
// bin/<case>/<set>/<id>/<id>_info.txt (hostFunctions.cuh:48-89), then per
// output step <field><step:06>.bin and step_<step:06>.vti
// (PostProcess.cuh:43-261), and the closing MLUPS line computed as
// src/main.cu:201-205 (every node, NSTEPS+1 steps, wall clock). The GPU comes
// from $GPU_INDEX (hostFunctions.cuh:117-150). Run-mode constants of
// src/constants.cuh:59-78 become options:
//   --steps N       NSTEPS (default 100000, RUN_MODE)
//   --save M        MACRO_SAVE (default 1000)
//   --sample        NSTEPS=10000, MACRO_SAVE=1000 (SAMPLE_MODE)
//   --profile       NSTEPS=0, MACRO_SAVE=1 (PROFILE_MODE)
//   --benchmark     no file output in the loop (-DBENCHMARK=1)
//   --storage fp32|fp16|bf16|fp64
//   --fields a,b,c  fields written at output steps (default rho,uz as main.cu:130-133)
//   --average / --reynolds / --vorticity   derived fields (compile.sh:71-73)
//   --nx/--ny/--nz/--diam/--radius/--sigma/--tau/--gamma/--re/--u-inf  mesh and physics
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <sstream>
#include <string>
#include <sys/stat.h>
#include <vector>

#include "../../include/pflbm.h"

namespace {

const char *kNames[PFLBM_FIELD_COUNT] = {
    "rho", "ux", "uy", "uz", "pxx", "pyy", "pzz", "pxy", "pxz", "pyz", "phi", "normx", "normy", "normz", "ind",
    "fsx", "fsy", "fsz", "avg_phi", "avg_ux", "avg_uy", "avg_uz", "avg_uxux", "avg_uyuy", "avg_uzuz", "avg_uxuy",
    "avg_uxuz", "avg_uyuz", "vort_x", "vort_y", "vort_z", "vort_mag", "c"};

int field_id(const std::string &n) {
    for (int i = 0; i < PFLBM_FIELD_COUNT; ++i)
        if (n == kNames[i]) return i;
    return -1;
}

bool mkdirs(const std::string &d) {
    std::string acc;
    for (size_t i = 0; i <= d.size(); ++i) {
        if (i == d.size() || d[i] == '/') {
            if (!acc.empty()) mkdir(acc.c_str(), 0755);
        }
        if (i < d.size()) acc.push_back(d[i]);
    }
    struct stat st{};
    return stat(d.c_str(), &st) == 0;
}

int die(const char *what, int rc) {
    std::fprintf(stderr, "Error: %s (%d): %s\n", what, rc, pflbm_last_error());
    return 1;
}

}  // namespace

int main(int argc, char **argv) {
    if (argc < 4) {
        std::fprintf(stderr, "Error: Usage: %s <flow case> <velocity set> <ID>\n", argv[0]);
        return 1;
    }
    const std::string flow = argv[1], vs = argv[2], id = argv[3];
    int fc, q;
    if (flow == "JET") fc = PFLBM_CASE_JET;
    else if (flow == "DROPLET") fc = PFLBM_CASE_DROPLET;
    else {
        std::fprintf(stderr, "Error: flow case must be JET or DROPLET\n");
        return 1;
    }
    if (vs == "D3Q19") q = 19;
    else if (vs == "D3Q27") q = 27;
    else {
        std::fprintf(stderr, "Invalid VELOCITY_SET. Use 'D3Q19' or 'D3Q27'.\n");
        return 1;
    }
    pflbm_config cfg;
    pflbm_config_reference(&cfg, fc, q);
    long nsteps = 100000, save = 1000;
    bool benchmark = false;
    std::vector<int> fields = {PFLBM_FIELD_RHO, PFLBM_FIELD_UZ};
    for (int i = 5; i <= argc; ++i) {
        // argv[4] is the reference's unused trailing "1" (pipeline.sh:83) or an option
        const std::string a = argv[i - 1];
        auto next = [&](void) -> const char * { return i < argc ? argv[i++] : ""; };
        if (a == "--steps") nsteps = std::atol(next());
        else if (a == "--save") save = std::atol(next());
        else if (a == "--sample") { nsteps = 10000; save = 1000; }
        else if (a == "--profile") { nsteps = 0; save = 1; }
        else if (a == "--benchmark") benchmark = true;
        else if (a == "--storage") {
            const std::string s = next();
            cfg.storage = s == "fp16" ? PFLBM_STORAGE_FP16 : s == "bf16" ? PFLBM_STORAGE_BF16
                        : s == "fp64" ? PFLBM_STORAGE_FP64 : PFLBM_STORAGE_FP32;
        } else if (a == "--fields") {
            fields.clear();
            std::stringstream ss(next());
            std::string f;
            while (std::getline(ss, f, ',')) {
                const int k = field_id(f);
                if (k < 0) {
                    std::fprintf(stderr, "Error: unknown field %s\n", f.c_str());
                    return 1;
                }
                fields.push_back(k);
            }
        } else if (a == "--average") cfg.flags |= PFLBM_FLAG_TIME_AVERAGE;
        else if (a == "--reynolds") cfg.flags |= PFLBM_FLAG_REYNOLDS_MOMENTS;
        else if (a == "--vorticity") cfg.flags |= PFLBM_FLAG_VORTICITY;
        else if (a == "--nx") cfg.nx = std::atoi(next());
        else if (a == "--ny") cfg.ny = std::atoi(next());
        else if (a == "--nz") cfg.nz = std::atoi(next());
        else if (a == "--diam") { cfg.diam = std::atoi(next()); cfg.radius = cfg.diam / 2; }
        else if (a == "--radius") cfg.radius = std::atoi(next());
        else if (a == "--sigma") cfg.sigma = float(std::atof(next()));
        else if (a == "--tau") cfg.tau = float(std::atof(next()));
        else if (a == "--gamma") cfg.gamma = float(std::atof(next()));
        else if (a == "--u-inf") cfg.u_inf = float(std::atof(next()));
        else if (a == "--re") cfg.reynolds_water = cfg.reynolds_oil = float(std::atof(next()));
    }
    if (save <= 0) save = 1;

    // bin/<case>/<set>/<id>/ (hostFunctions.cuh:33-46)
    const std::string dir = "bin/" + flow + "/" + vs + "/" + id + "/";
    if (!mkdirs(dir)) {
        std::fprintf(stderr, "Error: cannot create %s\n", dir.c_str());
        return 1;
    }
    pflbm_sim *sim = nullptr;
    int rc = pflbm_create(&cfg, &sim);
    if (rc) return die("pflbm_create", rc);
    rc = pflbm_init(sim);
    if (rc) return die("pflbm_init", rc);

    {
        std::ofstream info(dir + id + "_info.txt", std::ios::trunc);
        info << "---------------------------- SIMULATION METADATA ----------------------------\n"
             << "ID:                    " << id << '\n'
             << "Velocity set:          " << vs << '\n'
             << "Reference velocity:    " << cfg.u_inf << '\n'
             << "Dispersed phase Re:    " << cfg.reynolds_oil << '\n'
             << "Continuous phase Re:   " << cfg.reynolds_water << '\n'
             << "Surface tension:       " << cfg.sigma << '\n'
             << "NX:                    " << cfg.nx << '\n'
             << "NY:                    " << cfg.ny << '\n'
             << "NZ:                    " << cfg.nz << '\n'
             << "Diameter:              " << cfg.diam << '\n'
             << "Timesteps:             " << nsteps << '\n'
             << "Output interval:       " << save << '\n'
             << "-----------------------------------------------------------------------------\n";
    }
    std::printf("Running %s %s %s: %ux%ux%u, %ld steps\n", flow.c_str(), vs.c_str(), id.c_str(), cfg.nx, cfg.ny, cfg.nz,
                nsteps + 1);
    const auto t0 = std::chrono::high_resolution_clock::now();
    long done = 0;  // completed steps; step index of the last one is done-1
    for (long step = 0; step <= nsteps;) {
        // run up to the next output step (inclusive), as STEP % MACRO_SAVE == 0 || STEP == NSTEPS
        long next_out = ((step + save - 1) / save) * save;
        if (step % save == 0) next_out = step;
        if (next_out > nsteps) next_out = nsteps;
        const long n = next_out - step + 1;
        rc = pflbm_step_async(sim, uint64_t(n));
        if (rc) return die("pflbm_step", rc);
        done += n;
        step = next_out + 1;
        if (!benchmark) {
            // the files are written in the background while the next steps run
            std::printf("Step %ld: bins in %s\n", done - 1, dir.c_str());
            rc = pflbm_write_output_async(sim, dir.c_str(), fields.data(), int32_t(fields.size()));
            if (rc) return die("pflbm_write_output_async", rc);
        }
    }
    rc = pflbm_synchronize(sim);
    if (rc) return die("pflbm_synchronize", rc);
    const auto t1 = std::chrono::high_resolution_clock::now();
    const double sec = std::chrono::duration<double>(t1 - t0).count();
    const double mlups = double(cfg.nx) * cfg.ny * cfg.nz * double(nsteps + 1) / (sec * 1e6);
    std::printf("\n// =============================================== //\n");
    std::printf("     Total execution time    : %g s\n", sec);
    std::printf("     Performance             : %g MLUPS\n", mlups);
    std::printf("// =============================================== //\n\n");
    pflbm_destroy(sim);
    return 0;
}
