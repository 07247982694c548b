// oracle.cpp - CPU restatement of the phaseFieldLBM per-timestep path.
//
// TEST INFRASTRUCTURE ONLY. This file is the checker for the CUDA library in
// phasefieldlbm_gb300/: only tests/, __graft_entry__.smoke() and the CPU
// baseline legs of bench.py may load it. The product never links or calls it.
//
// It restates, pass by pass and in the reference's own order, what the
// reference computes on the GPU:
//   phase::computePhase    src/phaseField.cuh:31-52
//   phase::computeNormals  src/phaseField.cuh:54-140
//   phase::computeForces   src/phaseField.cuh:142-219
//   lbm::computeMoments    src/lbm.cu:33-128
//   lbm::streamCollide     src/lbm.cu:130-239   (single-buffer push)
//   applyInflow/Outflow    src/BoundaryConditions.cuh:36-169
//   hash32/white_noise     src/BoundaryConditions.cuh:172-213
//   initial conditions     src/initialConditions.cu:33-138
//   derived fields         src/derivedFields/operators/*.cuh
// Every field array holds what the reference's LBMFields array holds after
// the same step, ghost shell included. scalar_t becomes the template type T
// (float reproduces the reference's FP32 build, double is the FP64 oracle).
// Inputs that the reference computes in float (noise, config constants) are
// computed in float and converted, so both precisions solve the same problem.
// Loops run under OpenMP; no reduction order depends on the thread count.
#include <cmath>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <memory>
#include <vector>

#include "../include/pflbm.h"

namespace {

// ---------------------------------------------------------------- lattices
// Direction tables: src/velocitySet/D3Q19.cuh:92-141, D3Q27.cuh:96-145,
// D3Q7.cuh:78-127. Opposite directions are (2k-1, 2k).
const int kCX[27] = {0, 1, -1, 0, 0, 0, 0, 1, -1, 1, -1, 0, 0, 1, -1, 1, -1, 0, 0, 1, -1, 1, -1, 1, -1, -1, 1};
const int kCY[27] = {0, 0, 0, 1, -1, 0, 0, 1, -1, 0, 0, 1, -1, -1, 1, 0, 0, 1, -1, 1, -1, 1, -1, -1, 1, 1, -1};
const int kCZ[27] = {0, 0, 0, 0, 0, 1, -1, 0, 0, 1, -1, 1, -1, 0, 0, -1, 1, -1, 1, 1, -1, -1, 1, 1, -1, 1, -1};

template <class T>
T cst(double v) { return static_cast<T>(v); }

template <class T>
struct Lattice {
    int Q = 19;
    T w[27]{};
    T w0, w1, w2, w3, as2, cs2;
    explicit Lattice(int q) : Q(q) {
        // D3Q19.cuh:55-90 ; D3Q27.cuh:55-94
        if (Q == 19) {
            w0 = cst<T>(1.0 / 3.0); w1 = cst<T>(1.0 / 18.0); w2 = cst<T>(1.0 / 36.0); w3 = T(0);
        } else {
            w0 = cst<T>(8.0 / 27.0); w1 = cst<T>(2.0 / 27.0); w2 = cst<T>(1.0 / 54.0); w3 = cst<T>(1.0 / 216.0);
        }
        as2 = T(3);
        cs2 = cst<T>(1.0 / 3.0);
        for (int q = 0; q < Q; ++q) w[q] = q == 0 ? w0 : (q <= 6 ? w1 : (q <= 18 ? w2 : w3));
    }
    // D3Q19.cuh:143-150 (2nd order) ; D3Q27.cuh:152-159 (3rd order). Shifted by -w.
    T feq(int q, T rho, T uu, T cu) const {
        if (Q == 19) return w[q] * rho * (T(1) - uu + cu + T(0.5) * cu * cu) - w[q];
        const T oos = cst<T>(1.0 / 6.0);
        return w[q] * rho * (T(1) - uu + cu + T(0.5) * cu * cu + oos * cu * cu * cu - uu * cu) - w[q];
    }
    // D3Q19.cuh:152-171 ; D3Q27.cuh:161-190 (Hermite-regularised non-equilibrium).
    T fneq(int q, T pxx, T pyy, T pzz, T pxy, T pxz, T pyz, T ux, T uy, T uz) const {
        const int cx = kCX[q], cy = kCY[q], cz = kCZ[q];
        T r = (w[q] * T(4.5)) *
              ((T(cx * cx) - cs2) * pxx + (T(cy * cy) - cs2) * pyy + (T(cz * cz) - cs2) * pzz +
               T(2) * (T(cx * cy) * pxy + T(cx * cz) * pxz + T(cy * cz) * pyz));
        if (Q == 19) return r;
        return (w[q] * T(4.5)) *
               ((T(cx * cx) - cs2) * pxx + (T(cy * cy) - cs2) * pyy + (T(cz * cz) - cs2) * pzz +
                T(2) * (T(cx * cy) * pxy + T(cx * cz) * pxz + T(cy * cz) * pyz) +
                T(cx * cx * cx - cx) * (as2 * ux * pxx) +
                T(cy * cy * cy - cy) * (as2 * uy * pyy) +
                T(cz * cz * cz - cz) * (as2 * uz * pzz) +
                as2 * ((T(cx * cx * cy) - cs2 * T(cy)) * (pxx * uy + T(2) * ux * pxy) +
                       (T(cx * cx * cz) - cs2 * T(cz)) * (pxx * uz + T(2) * ux * pxz) +
                       (T(cx * cy * cy) - cs2 * T(cx)) * (pyy * ux + T(2) * uy * pxy) +
                       (T(cy * cy * cz) - cs2 * T(cz)) * (pyy * uz + T(2) * uy * pyz) +
                       (T(cx * cz * cz) - cs2 * T(cx)) * (pzz * ux + T(2) * uz * pxz) +
                       (T(cy * cz * cz) - cs2 * T(cy)) * (pzz * uy + T(2) * uz * pyz)) +
                T(6 * cx * cy * cz) * (ux * pyz + uy * pxz + uz * pxy));
    }
    // Guo forcing term, D3Q19.cuh:173-187 (identical in D3Q27.cuh:192-206).
    T force(int q, T cu, T ux, T uy, T uz, T fx, T fy, T fz) const {
        const T cx = T(kCX[q]), cy = T(kCY[q]), cz = T(kCZ[q]);
        return w[q] * ((as2 * (cx - ux) + as2 * cu * cx) * fx + (as2 * (cy - uy) + as2 * cu * cy) * fy +
                       (as2 * (cz - uz) + as2 * cu * cz) * fz);
    }
    T cu(int q, T ux, T uy, T uz) const {
        return as2 * (T(kCX[q]) * ux + T(kCY[q]) * uy + T(kCZ[q]) * uz);
    }
};

// D3Q7, src/velocitySet/D3Q7.cuh:45-153
template <class T>
struct Phase7 {
    T w[7];
    T as2 = T(4);
    Phase7() {
        w[0] = cst<T>(1.0 / 4.0);
        for (int q = 1; q < 7; ++q) w[q] = cst<T>(1.0 / 8.0);
    }
    T geq(int q, T phi, T ux, T uy, T uz) const {
        return w[q] * phi * (T(1) + as2 * (T(kCX[q]) * ux + T(kCY[q]) * uy + T(kCZ[q]) * uz));
    }
    T anti_diffusion(int q, T sharp, T nx, T ny, T nz) const {
        return w[q] * sharp * (T(kCX[q]) * nx + T(kCY[q]) * ny + T(kCZ[q]) * nz);
    }
};

// ------------------------------------------------------------------- noise
// src/BoundaryConditions.cuh:172-213 (always float: the noise is an input).
uint32_t hash32(uint32_t x) {
    x ^= x >> 16;
    x *= 0x7FEB352Du;
    x ^= x >> 15;
    x *= 0x846CA68Bu;
    x ^= x >> 16;
    return x;
}
float uniform01(uint32_t s) { return (static_cast<float>(s) + 0.5f) * 2.3283064365386963e-10f; }
float box_muller(float rrx, float rry) {
    rrx = std::fmax(rrx, 1e-12f);
    const float r = std::sqrt(-2.0f * std::log(rrx));
    const float theta = (2.0f * 3.141592654f) * rry;
    return r * std::cos(theta);
}
uint32_t noise_base(uint32_t salt, uint32_t x, uint32_t y, uint32_t t) {
    return (0x9E3779B9u ^ salt) ^ x ^ (y * 0x85EBCA6Bu) ^ (t * 0xC2B2AE35u);
}
float white_noise(uint32_t salt, uint32_t x, uint32_t y, uint32_t t) {
    const uint32_t base = noise_base(salt, x, y, t);
    return box_muller(uniform01(hash32(base)), uniform01(hash32(base ^ 0x68BC21EBu)));
}
// Uniform mode (not in the reference): xi in [-1, 1) from the same counter
// hash with its own salt XOR the user seed.
float uniform_noise(uint32_t seed, uint32_t x, uint32_t y, uint32_t t) {
    const uint32_t base = noise_base(0x2545F491u ^ seed, x, y, t);
    return 2.0f * uniform01(hash32(base)) - 1.0f;
}
// Seeded initial velocity noise (ensemble boxes): component c of node (x,y,z).
float init_noise_value(uint32_t seed, uint32_t c, uint32_t x, uint32_t y, uint32_t z) {
    const uint32_t base = noise_base(0x5851F42Du ^ seed ^ (c * 0x9E3779B9u), x, y, z * 0x27D4EB2Fu);
    return 2.0f * uniform01(hash32(base)) - 1.0f;
}

// ------------------------------------------------------------------ config
// Derived constants, src/constants.cuh:80-141 and globalFunctions.cuh:260-461.
template <class T>
struct Consts {
    // jet relaxation
    T visc_water, visc_oil, tau_water, tau_oil, omco_zmin;
    // droplet relaxation
    T omega_ref;
    // sponge
    T K_gain, z_start, inv_nz_m1, inv_sponge;
    T sigma, gamma, u_inf;
    T center_x, center_y, center_z, R2;
    T as2_hydro;
    T omega_from_nu(T nu) const {  // globalFunctions.cuh:319-322
        return static_cast<T>(1.0 / (0.5 + static_cast<double>(as2_hydro) * static_cast<double>(nu)));
    }
    T tau_from_nu(T nu) const { return T(0.5) + as2_hydro * nu; }  // :324-327
    T tau_zmax(T phi) const {                                        // :376-382
        const T visc_local = (T(1) - phi) * visc_water + phi * visc_oil;
        const T visc_sp = visc_local * (T(1) + K_gain);
        return tau_from_nu(visc_sp);
    }
    T omco_zmax(T phi) const {  // :394-397 via omega_zmax :359-364
        const T visc_local = (T(1) - phi) * visc_water + phi * visc_oil;
        return T(1) - omega_from_nu(visc_local * (T(1) + K_gain));
    }
    T sponge_ramp(uint32_t z) const {  // deviceFunctions.cuh:94-101
        const T zn = static_cast<T>(z) * inv_nz_m1;
        T s = (zn - z_start) * inv_sponge;
        s = std::fmin(std::fmax(s, T(0)), T(1));
        return s * s * (T(3) - T(2) * s);
    }
};

template <class T>
Consts<T> make_consts(const pflbm_config &c) {
    Consts<T> k{};
    k.as2_hydro = T(3);
    k.sigma = T(c.sigma);
    k.gamma = T(c.gamma);
    k.u_inf = T(c.u_inf);
    const float u = c.u_inf;
    if (c.flow_case == PFLBM_CASE_JET) {
        k.visc_water = static_cast<T>((static_cast<double>(u) * static_cast<double>(c.diam)) / static_cast<double>(c.reynolds_water));
        k.visc_oil = static_cast<T>((static_cast<double>(u) * static_cast<double>(c.diam)) / static_cast<double>(c.reynolds_oil));
        k.tau_water = k.tau_from_nu(k.visc_water);
        k.tau_oil = k.tau_from_nu(k.visc_oil);
        k.omco_zmin = T(1) - k.omega_from_nu(k.visc_oil);
        const int cells = c.sponge_cells >= 0 ? c.sponge_cells : static_cast<int>(c.nz / 12);
        const T sponge = static_cast<T>(static_cast<double>(cells) / static_cast<double>(c.nz - 1));
        k.z_start = static_cast<T>(static_cast<double>(c.nz - 1 - cells) / static_cast<double>(c.nz - 1));
        k.inv_nz_m1 = static_cast<T>(1.0 / static_cast<double>(c.nz - 1));
        k.inv_sponge = static_cast<T>(1.0 / static_cast<double>(sponge));
        k.K_gain = T(c.sponge_gain);
    } else {
        // constants.cuh:139-140 ; globalFunctions.cuh:426-429
        const T visc_ref = (T(c.tau) - T(0.5)) / T(3);
        k.omega_ref = k.omega_from_nu(visc_ref);
    }
    k.center_x = static_cast<T>(c.nx - 1) * T(0.5) + T(c.center_offset[0]);
    k.center_y = static_cast<T>(c.ny - 1) * T(0.5) + T(c.center_offset[1]);
    k.center_z = static_cast<T>(c.nz - 1) * T(0.5) + T(c.center_offset[2]);
    k.R2 = static_cast<T>(c.radius * c.radius);
    return k;
}

// ------------------------------------------------------------- closure MLP
// Eddy-viscosity closure: features x = (Pi_xx, Pi_yy, Pi_zz, Pi_xy, Pi_xz,
// Pi_yz, phi, |grad phi|), normalised x' = (x - mean) * inv_scale;
// a1 = W1 x' + b1, h1 = SiLU(a1); a2 = W2 h1 + b2, h2 = SiLU(a2);
// z = w3 . h2 + b3; nu_t = out_scale * softplus(z).
// Parameter vector (1377): W1[32][8], b1[32], W2[32][32], b2[32], w3[32], b3.
constexpr int kIn = 8, kH = 32;
constexpr int kNumParams = kH * kIn + kH + kH * kH + kH + kH + 1;

struct Mlp {
    std::vector<double> p = std::vector<double>(kNumParams, 0.0);
    double mean[kIn] = {0}, inv_scale[kIn] = {1, 1, 1, 1, 1, 1, 1, 1}, out_scale = 0.0;
    const double *W1() const { return p.data(); }
    const double *b1() const { return p.data() + kH * kIn; }
    const double *W2() const { return b1() + kH; }
    const double *b2() const { return W2() + kH * kH; }
    const double *w3() const { return b2() + kH; }
    double b3() const { return *(w3() + kH); }
};

inline double silu(double a) { return a / (1.0 + std::exp(-a)); }
inline double dsilu(double a) {
    const double s = 1.0 / (1.0 + std::exp(-a));
    return s * (1.0 + a * (1.0 - s));
}
inline double softplus(double z) { return std::fmax(z, 0.0) + std::log1p(std::exp(-std::fabs(z))); }
inline double dsoftplus(double z) { return 1.0 / (1.0 + std::exp(-z)); }

// Forward; returns nu_t. With grad != null, accumulates d(loss)/d(params)
// for loss = (nu_t - target)^2 / out_scale^2 (the library's training loss).
double mlp_eval(const Mlp &m, const double *x, double target, double *grad) {
    double xn[kIn], a1[kH], h1[kH], a2[kH], h2[kH];
    for (int k = 0; k < kIn; ++k) xn[k] = (x[k] - m.mean[k]) * m.inv_scale[k];
    for (int i = 0; i < kH; ++i) {
        double s = m.b1()[i];
        for (int k = 0; k < kIn; ++k) s += m.W1()[i * kIn + k] * xn[k];
        a1[i] = s;
        h1[i] = silu(s);
    }
    double z = m.b3();
    for (int j = 0; j < kH; ++j) {
        double s = m.b2()[j];
        for (int i = 0; i < kH; ++i) s += m.W2()[j * kH + i] * h1[i];
        a2[j] = s;
        h2[j] = silu(s);
        z += m.w3()[j] * h2[j];
    }
    const double y = m.out_scale * softplus(z);
    if (grad) {
        // d loss / d z with loss = (softplus(z) - target/out_scale)^2
        const double r = softplus(z) - target / m.out_scale;
        const double dz = 2.0 * r * dsoftplus(z);
        double *gW1 = grad, *gb1 = grad + kH * kIn, *gW2 = gb1 + kH, *gb2 = gW2 + kH * kH, *gw3 = gb2 + kH,
               *gb3 = gw3 + kH;
        *gb3 += dz;
        double da2[kH];
        for (int j = 0; j < kH; ++j) {
            gw3[j] += dz * h2[j];
            da2[j] = dz * m.w3()[j] * dsilu(a2[j]);
            gb2[j] += da2[j];
            for (int i = 0; i < kH; ++i) gW2[j * kH + i] += da2[j] * h1[i];
        }
        for (int i = 0; i < kH; ++i) {
            double dh = 0.0;
            for (int j = 0; j < kH; ++j) dh += m.W2()[j * kH + i] * da2[j];
            const double da1 = dh * dsilu(a1[i]);
            gb1[i] += da1;
            for (int k = 0; k < kIn; ++k) gW1[i * kIn + k] += da1 * xn[k];
        }
    }
    return y;
}

// -------------------------------------------------------------- simulation
struct OracleBase {
    virtual ~OracleBase() = default;
    virtual void init() = 0;
    virtual void step() = 0;
    virtual const void *field(int id, int *is_double) const = 0;
    virtual const void *pops(int which, int *is_double) const = 0;
    uint64_t t = 0;
    Mlp mlp;            // closure network (used when closure_strength != 0)
    double closure_strength = 0.0;
    double closure_mixing = 0.0;  // inverse turbulent Schmidt number of the phase mixing
};

template <class T>
struct Oracle final : OracleBase {
    pflbm_config c;
    Lattice<T> L;
    Phase7<T> P;
    Consts<T> K;
    uint32_t nx, ny, nz;
    size_t N;
    bool jet;
    // LBMFields, src/LBMIncludes.cuh:58-117
    std::vector<T> fld[PFLBM_FIELD_COUNT];
    std::vector<T> f, g;

    explicit Oracle(const pflbm_config &cfg) : c(cfg), L(cfg.velocity_set), K(make_consts<T>(cfg)) {
        nx = c.nx; ny = c.ny; nz = c.nz;
        N = size_t(nx) * ny * nz;
        jet = c.flow_case == PFLBM_CASE_JET;
        for (int i = 0; i < 18; ++i) fld[i].assign(N, T(0));
        if (c.flags & PFLBM_FLAG_TIME_AVERAGE)
            for (int i = PFLBM_FIELD_AVG_PHI; i <= PFLBM_FIELD_AVG_UZ; ++i) fld[i].assign(N, T(0));
        if (c.flags & PFLBM_FLAG_REYNOLDS_MOMENTS)
            for (int i = PFLBM_FIELD_AVG_UXUX; i <= PFLBM_FIELD_AVG_UYUZ; ++i) fld[i].assign(N, T(0));
        if (c.flags & PFLBM_FLAG_VORTICITY)
            for (int i = PFLBM_FIELD_VORT_X; i <= PFLBM_FIELD_VORT_MAG; ++i) fld[i].assign(N, T(0));
        f.assign(size_t(L.Q) * N, T(0));
        g.assign(7 * N, T(0));
    }

    size_t id3(uint32_t x, uint32_t y, uint32_t z) const { return x + size_t(nx) * (y + size_t(ny) * z); }
    bool guard(uint32_t x, uint32_t y, uint32_t z) const {  // deviceFunctions.cuh:50-61
        return x < 1 || y < 1 || z < 1 || x >= nx - 1 || y >= ny - 1 || z >= nz - 1;
    }
    static uint32_t wrap(int64_t x, uint32_t n) {  // deviceFunctions.cuh:63-76
        if (x < 1) return n - 2;
        if (x > int64_t(n) - 2) return 1;
        return uint32_t(x);
    }
    T &F(int id, size_t i) { return fld[id][i]; }

    // --------------------------------------------------- initial conditions
    void init() override {
        t = 0;
        for (int i = 0; i < PFLBM_FIELD_COUNT; ++i) std::fill(fld[i].begin(), fld[i].end(), T(0));
        std::fill(f.begin(), f.end(), T(0));
        std::fill(g.begin(), g.end(), T(0));
        // setInitialDensity, initialConditions.cu:85-99
        std::fill(fld[PFLBM_FIELD_RHO].begin(), fld[PFLBM_FIELD_RHO].end(), T(1));
        if (jet) {
            // setJet, initialConditions.cu:33-56
            for (uint32_t y = 0; y < ny; ++y)
                for (uint32_t x = 0; x < nx; ++x) {
                    const T dx = static_cast<T>(x) - K.center_x, dy = static_cast<T>(y) - K.center_y;
                    if (dx * dx + dy * dy > K.R2) continue;
                    F(PFLBM_FIELD_PHI, id3(x, y, 0)) = T(1);
                    F(PFLBM_FIELD_UZ, id3(x, y, 0)) = K.u_inf;
                }
        } else {
            // setDroplet, initialConditions.cu:58-83 (x distance divided by the stretch)
#pragma omp parallel for schedule(static)
            for (int64_t zz = 1; zz < int64_t(nz) - 1; ++zz) {
                const uint32_t z = uint32_t(zz);
                for (uint32_t y = 1; y < ny - 1; ++y)
                    for (uint32_t x = 1; x < nx - 1; ++x) {
                        const T dx = (static_cast<T>(x) - K.center_x) / T(c.droplet_x_stretch);
                        const T dy = static_cast<T>(y) - K.center_y;
                        const T dz = static_cast<T>(z) - K.center_z;
                        const T L2 = std::sqrt(dx * dx + dy * dy + dz * dz);
                        const T arg = static_cast<T>((static_cast<double>(c.radius) - static_cast<double>(L2)) /
                                                     static_cast<double>(c.interface_width));
                        F(PFLBM_FIELD_PHI, id3(x, y, z)) = T(0.5) + T(0.5) * std::tanh(T(2) * arg);
                    }
            }
            if (c.init_noise != 0.0f) {
                // seeded uniform initial velocity (ensemble boxes), interior only
                for (uint32_t z = 1; z < nz - 1; ++z)
                    for (uint32_t y = 1; y < ny - 1; ++y)
                        for (uint32_t x = 1; x < nx - 1; ++x) {
                            const size_t i = id3(x, y, z);
                            F(PFLBM_FIELD_UX, i) = T(c.init_noise * init_noise_value(c.seed, 0, x, y, z));
                            F(PFLBM_FIELD_UY, i) = T(c.init_noise * init_noise_value(c.seed, 1, x, y, z));
                            F(PFLBM_FIELD_UZ, i) = T(c.init_noise * init_noise_value(c.seed, 2, x, y, z));
                        }
            }
        }
        set_distros();
    }

    void set_distros() {  // initialConditions.cu:101-138 (every node, ghosts included)
#pragma omp parallel for schedule(static)
        for (int64_t ii = 0; ii < int64_t(N); ++ii) {
            const size_t i = size_t(ii);
            const T ux = F(PFLBM_FIELD_UX, i), uy = F(PFLBM_FIELD_UY, i), uz = F(PFLBM_FIELD_UZ, i);
            const T uu = T(1.5) * (ux * ux + uy * uy + uz * uz);
            for (int q = 0; q < L.Q; ++q)
                f[q * N + i] = L.feq(q, F(PFLBM_FIELD_RHO, i), uu, L.cu(q, ux, uy, uz));
            for (int q = 0; q < 7; ++q) g[q * N + i] = P.geq(q, F(PFLBM_FIELD_PHI, i), ux, uy, uz);
        }
    }

    // ----------------------------------------------------------- one step
    template <class Fn>
    void interior(Fn fn) {
#pragma omp parallel for schedule(static)
        for (int64_t zz = 1; zz < int64_t(nz) - 1; ++zz)
            for (uint32_t y = 1; y < ny - 1; ++y)
                for (uint32_t x = 1; x < nx - 1; ++x) fn(x, y, uint32_t(zz));
    }

    // Lattice-weighted central stencil of src/phaseField.cuh:67-118, written
    // once for any field v and axis a: pairs (2k-1, 2k) in ascending k,
    // (+c member) - (-c member), grouped by weight class.
    T grad(const std::vector<T> &v, int axis, uint32_t x, uint32_t y, uint32_t z) const {
        const int *ca = axis == 0 ? kCX : (axis == 1 ? kCY : kCZ);
        auto at = [&](int q) { return v[id3(x + kCX[q], y + kCY[q], z + kCZ[q])]; };
        T cls[3] = {T(0), T(0), T(0)};
        const int lo[3] = {1, 7, 19}, hi[3] = {6, 18, 26};
        for (int k = 0; k < (L.Q == 27 ? 3 : 2); ++k) {
            bool first = true;
            T s = T(0);
            for (int q = lo[k]; q < hi[k]; q += 2) {
                if (ca[q] == 0) continue;
                const int qp = ca[q] > 0 ? q : q + 1, qm = ca[q] > 0 ? q + 1 : q;
                if (first) { s = at(qp) - at(qm); first = false; }
                else { s = s + at(qp); s = s - at(qm); }
            }
            cls[k] = s;
        }
        T r = L.w1 * cls[0] + L.w2 * cls[1];
        if (L.Q == 27) r += L.w3 * cls[2];
        return r;
    }

    void step() override {
        const uint32_t tt = uint32_t(t);
        std::vector<T> &phi = fld[PFLBM_FIELD_PHI];
        // computePhase, phaseField.cuh:31-52
        interior([&](uint32_t x, uint32_t y, uint32_t z) {
            const size_t i = id3(x, y, z);
            T s = T(0);
            for (int q = 0; q < 7; ++q) s += g[q * N + i];
            phi[i] = s;
        });
        // computeNormals, phaseField.cuh:54-140
        interior([&](uint32_t x, uint32_t y, uint32_t z) {
            const size_t i = id3(x, y, z);
            const T gx = L.as2 * grad(phi, 0, x, y, z);
            const T gy = L.as2 * grad(phi, 1, x, y, z);
            const T gz = L.as2 * grad(phi, 2, x, y, z);
            const T ind = std::sqrt(gx * gx + gy * gy + gz * gz);
            const T inv = T(1) / (ind + T(1e-9));
            F(PFLBM_FIELD_IND, i) = ind;
            F(PFLBM_FIELD_NORMX, i) = gx * inv;
            F(PFLBM_FIELD_NORMY, i) = gy * inv;
            F(PFLBM_FIELD_NORMZ, i) = gz * inv;
        });
        // computeForces, phaseField.cuh:142-219
        interior([&](uint32_t x, uint32_t y, uint32_t z) {
            const size_t i = id3(x, y, z);
            const T scx = grad(fld[PFLBM_FIELD_NORMX], 0, x, y, z);
            const T scy = grad(fld[PFLBM_FIELD_NORMY], 1, x, y, z);
            const T scz = grad(fld[PFLBM_FIELD_NORMZ], 2, x, y, z);
            const T curvature = L.as2 * (scx + scy + scz);
            const T st = -K.sigma * curvature * F(PFLBM_FIELD_IND, i);
            F(PFLBM_FIELD_FFX, i) = st * F(PFLBM_FIELD_NORMX, i);
            F(PFLBM_FIELD_FFY, i) = st * F(PFLBM_FIELD_NORMY, i);
            F(PFLBM_FIELD_FFZ, i) = st * F(PFLBM_FIELD_NORMZ, i);
        });
        compute_moments();
        stream_collide();
        if (jet) {
            apply_inflow(tt);
            apply_outflow();
        }
        derived(tt + 1);
        ++t;
    }

    // (+member) - (-member) accumulation of the velocity sums, lbm.cu:62-73
    T vel_sum(const T *pop, int axis) const {
        const int *ca = axis == 0 ? kCX : (axis == 1 ? kCY : kCZ);
        bool first = true;
        T s = T(0);
        for (int q = 1; q < L.Q; q += 2) {
            if (ca[q] == 0) continue;
            const int qp = ca[q] > 0 ? q : q + 1, qm = ca[q] > 0 ? q + 1 : q;
            if (first) { s = pop[qp] - pop[qm]; first = false; }
            else { s = s + pop[qp]; s = s - pop[qm]; }
        }
        return s;
    }

    void compute_moments() {  // lbm.cu:33-128
        interior([&](uint32_t x, uint32_t y, uint32_t z) {
            const size_t i = id3(x, y, z);
            T pop[27];
            T rho = T(0);
            for (int q = 0; q < L.Q; ++q) { pop[q] = f[q * N + i]; rho += pop[q]; }
            rho += T(1);
            F(PFLBM_FIELD_RHO, i) = rho;
            const T fsx = F(PFLBM_FIELD_FFX, i), fsy = F(PFLBM_FIELD_FFY, i), fsz = F(PFLBM_FIELD_FFZ, i);
            const T invRho = T(1) / rho;
            T ux = invRho * vel_sum(pop, 0), uy = invRho * vel_sum(pop, 1), uz = invRho * vel_sum(pop, 2);
            ux += fsx * T(0.5) * invRho;
            uy += fsy * T(0.5) * invRho;
            uz += fsz * T(0.5) * invRho;
            F(PFLBM_FIELD_UX, i) = ux; F(PFLBM_FIELD_UY, i) = uy; F(PFLBM_FIELD_UZ, i) = uz;
            T pxx = 0, pyy = 0, pzz = 0, pxy = 0, pxz = 0, pyz = 0;
            const T uu = T(1.5) * (ux * ux + uy * uy + uz * uz);
            for (int q = 0; q < L.Q; ++q) {
                const T cx = T(kCX[q]), cy = T(kCY[q]), cz = T(kCZ[q]);
                const T cu = L.cu(q, ux, uy, uz);
                const T feq = L.feq(q, rho, uu, cu);
                const T force = L.force(q, cu, ux, uy, uz, fsx, fsy, fsz);
                const T fneq = pop[q] - feq + T(0.5) * force;
                pxx += fneq * cx * cx; pyy += fneq * cy * cy; pzz += fneq * cz * cz;
                pxy += fneq * cx * cy; pxz += fneq * cx * cz; pyz += fneq * cy * cz;
            }
            const T trace = pxx + pyy + pzz;
            pxx -= L.cs2 * trace; pyy -= L.cs2 * trace; pzz -= L.cs2 * trace;
            F(PFLBM_FIELD_PXX, i) = pxx; F(PFLBM_FIELD_PYY, i) = pyy; F(PFLBM_FIELD_PZZ, i) = pzz;
            F(PFLBM_FIELD_PXY, i) = pxy; F(PFLBM_FIELD_PXZ, i) = pxz; F(PFLBM_FIELD_PYZ, i) = pyz;
        });
    }

    void stream_collide() {  // lbm.cu:130-239, push into the same buffer
        interior([&](uint32_t x, uint32_t y, uint32_t z) {
            const size_t i = id3(x, y, z);
            const T rho = F(PFLBM_FIELD_RHO, i), ux = F(PFLBM_FIELD_UX, i), uy = F(PFLBM_FIELD_UY, i),
                    uz = F(PFLBM_FIELD_UZ, i);
            const T pxx = F(PFLBM_FIELD_PXX, i), pyy = F(PFLBM_FIELD_PYY, i), pzz = F(PFLBM_FIELD_PZZ, i);
            const T pxy = F(PFLBM_FIELD_PXY, i), pxz = F(PFLBM_FIELD_PXZ, i), pyz = F(PFLBM_FIELD_PYZ, i);
            const T fsx = F(PFLBM_FIELD_FFX, i), fsy = F(PFLBM_FIELD_FFY, i), fsz = F(PFLBM_FIELD_FFZ, i);
            const T phi = F(PFLBM_FIELD_PHI, i);
            T omega;
            T nu_cl = T(0);  // eddy viscosity of the closure (strength * nu_t)
            if (closure_strength != 0.0) {
                const double x[8] = {double(pxx), double(pyy), double(pzz), double(pxy), double(pxz), double(pyz),
                                     double(phi), double(F(PFLBM_FIELD_IND, i))};
                nu_cl = static_cast<T>(closure_strength * mlp_eval(mlp, x, 0.0, nullptr));
            }
            const T tau_t = T(3) * nu_cl;  // as a relaxation-time increment
            if (jet) {
                const T tau_phi = (T(1) - phi) * K.tau_water + phi * K.tau_oil + tau_t;
                const T r = K.sponge_ramp(z);
                const T tau_eff = tau_phi + r * (K.tau_zmax(phi) - tau_phi);
                omega = T(1) / tau_eff;
            } else {
                omega = tau_t == T(0) ? K.omega_ref : T(1) / (T(1) / K.omega_ref + tau_t);
            }
            const T omco = T(1) - omega;
            const T uu = T(1.5) * (ux * ux + uy * uy + uz * uz);
            for (int q = 0; q < L.Q; ++q) {
                const T cu = L.cu(q, ux, uy, uz);
                const T feq = L.feq(q, rho, uu, cu);
                const T force = L.force(q, cu, ux, uy, uz, fsx, fsy, fsz);
                const T fneq = L.fneq(q, pxx, pyy, pzz, pxy, pxz, pyz, ux, uy, uz);
                uint32_t xx = wrap(int64_t(x) + kCX[q], nx), yy = wrap(int64_t(y) + kCY[q], ny);
                uint32_t zz = jet ? uint32_t(int64_t(z) + kCZ[q]) : wrap(int64_t(z) + kCZ[q], nz);
                f[q * N + id3(xx, yy, zz)] = feq + omco * fneq + T(0.5) * force;
            }
            const T nxv = F(PFLBM_FIELD_NORMX, i), nyv = F(PFLBM_FIELD_NORMY, i), nzv = F(PFLBM_FIELD_NORMZ, i);
            // closure phase mixing: the flux -D_t grad phi, D_t = nu_cl / Sc_t,
            // as a change of the anti-diffusion coefficient (grad phi =
            // |grad phi| n, and the D3Q7 flux is J / 4)
            const T sharp = K.gamma * phi * (T(1) - phi) -
                            T(4) * (static_cast<T>(closure_mixing) * nu_cl) * F(PFLBM_FIELD_IND, i);
            for (int q = 0; q < 7; ++q) {
                const T geq = P.geq(q, phi, ux, uy, uz);
                const T hi = P.anti_diffusion(q, sharp, nxv, nyv, nzv);
                uint32_t xx = wrap(int64_t(x) + kCX[q], nx), yy = wrap(int64_t(y) + kCY[q], ny);
                uint32_t zz = jet ? uint32_t(int64_t(z) + kCZ[q]) : wrap(int64_t(z) + kCZ[q], nz);
                g[q * N + id3(xx, yy, zz)] = geq + hi;
            }
        });
    }

    void apply_inflow(uint32_t tt) {  // BoundaryConditions.cuh:36-105
        const float sigma_u = c.noise_amp * c.u_inf;
        for (uint32_t y = 0; y < ny; ++y)
            for (uint32_t x = 0; x < nx; ++x) {
                const T dx = static_cast<T>(x) - K.center_x, dy = static_cast<T>(y) - K.center_y;
                if (dx * dx + dy * dy > K.R2) continue;
                const size_t bnd = id3(x, y, 0), zp1 = id3(x, y, 1);
                T ux, uy, uz;
                if (c.inflow_noise == PFLBM_NOISE_GAUSSIAN_UXY) {
                    ux = T(sigma_u * white_noise(0xA341316Cu, x, y, tt));
                    uy = T(sigma_u * white_noise(0xC8013EA4u, x, y, tt));
                    uz = K.u_inf;
                } else {
                    ux = T(0);
                    uy = T(0);
                    uz = T(c.u_inf * (1.0f + c.noise_amp * uniform_noise(c.seed, x, y, tt)));
                }
                const T rho = T(1), phi = T(1);
                F(PFLBM_FIELD_RHO, bnd) = rho; F(PFLBM_FIELD_PHI, bnd) = phi;
                F(PFLBM_FIELD_UX, bnd) = ux; F(PFLBM_FIELD_UY, bnd) = uy; F(PFLBM_FIELD_UZ, bnd) = uz;
                const T uu = T(1.5) * (ux * ux + uy * uy + uz * uz);
                for (int q = 0; q < L.Q; ++q) {
                    if (kCZ[q] != 1) continue;
                    const size_t fl = id3(x + kCX[q], y + kCY[q], 1);
                    const T feq = L.feq(q, rho, uu, L.cu(q, ux, uy, uz));
                    const T fneq = L.fneq(q, F(PFLBM_FIELD_PXX, fl), F(PFLBM_FIELD_PYY, fl), F(PFLBM_FIELD_PZZ, fl),
                                          F(PFLBM_FIELD_PXY, fl), F(PFLBM_FIELD_PXZ, fl), F(PFLBM_FIELD_PYZ, fl),
                                          F(PFLBM_FIELD_UX, fl), F(PFLBM_FIELD_UY, fl), F(PFLBM_FIELD_UZ, fl));
                    f[q * N + fl] = feq + K.omco_zmin * fneq;
                }
                g[5 * N + zp1] = P.w[5] * phi * (T(1) + P.as2 * uz);
            }
    }

    void apply_outflow() {  // BoundaryConditions.cuh:107-169
        for (uint32_t y = 1; y < ny - 1; ++y)
            for (uint32_t x = 1; x < nx - 1; ++x) {
                const size_t bnd = id3(x, y, nz - 1), zm1 = id3(x, y, nz - 2);
                for (int id : {PFLBM_FIELD_RHO, PFLBM_FIELD_PHI, PFLBM_FIELD_UX, PFLBM_FIELD_UY, PFLBM_FIELD_UZ})
                    F(id, bnd) = F(id, zm1);
                const T rho = F(PFLBM_FIELD_RHO, bnd), phi = F(PFLBM_FIELD_PHI, bnd);
                const T ux = F(PFLBM_FIELD_UX, bnd), uy = F(PFLBM_FIELD_UY, bnd), uz = F(PFLBM_FIELD_UZ, bnd);
                const T uu = T(1.5) * (ux * ux + uy * uy + uz * uz);
                for (int q = 0; q < L.Q; ++q) {
                    if (kCZ[q] != -1) continue;
                    const uint32_t xx = wrap(int64_t(x) + kCX[q], nx), yy = wrap(int64_t(y) + kCY[q], ny);
                    const size_t fl = id3(xx, yy, nz - 2);
                    const T cu = L.cu(q, ux, uy, uz);
                    const T feq = L.feq(q, rho, uu, cu);
                    const T fneq = L.fneq(q, F(PFLBM_FIELD_PXX, fl), F(PFLBM_FIELD_PYY, fl), F(PFLBM_FIELD_PZZ, fl),
                                          F(PFLBM_FIELD_PXY, fl), F(PFLBM_FIELD_PXZ, fl), F(PFLBM_FIELD_PYZ, fl),
                                          F(PFLBM_FIELD_UX, fl), F(PFLBM_FIELD_UY, fl), F(PFLBM_FIELD_UZ, fl));
                    const T force = L.force(q, cu, ux, uy, uz, F(PFLBM_FIELD_FFX, fl), F(PFLBM_FIELD_FFY, fl),
                                            F(PFLBM_FIELD_FFZ, fl));
                    f[q * N + fl] = feq + K.omco_zmax(phi) * fneq + T(0.5) * force;
                }
                g[6 * N + zm1] = P.w[6] * phi * (T(1) - P.as2 * uz);
            }
    }

    // src/derivedFields/operators/{timeAverage,reynoldsMoments,vorticityFields}.cuh
    void derived(uint32_t tp1) {
        const bool avg = c.flags & PFLBM_FLAG_TIME_AVERAGE, rey = c.flags & PFLBM_FLAG_REYNOLDS_MOMENTS,
                   vort = c.flags & PFLBM_FLAG_VORTICITY;
        if (!avg && !rey && !vort) return;
        const T tf = static_cast<T>(tp1);
        auto upd = [&](T o, T n) { return o + (n - o) / tf; };
#pragma omp parallel for schedule(static)
        for (int64_t ii = 0; ii < int64_t(N); ++ii) {
            const size_t i = size_t(ii);
            const T ux = F(PFLBM_FIELD_UX, i), uy = F(PFLBM_FIELD_UY, i), uz = F(PFLBM_FIELD_UZ, i);
            if (avg) {
                F(PFLBM_FIELD_AVG_PHI, i) = upd(F(PFLBM_FIELD_AVG_PHI, i), F(PFLBM_FIELD_PHI, i));
                F(PFLBM_FIELD_AVG_UX, i) = upd(F(PFLBM_FIELD_AVG_UX, i), ux);
                F(PFLBM_FIELD_AVG_UY, i) = upd(F(PFLBM_FIELD_AVG_UY, i), uy);
                F(PFLBM_FIELD_AVG_UZ, i) = upd(F(PFLBM_FIELD_AVG_UZ, i), uz);
            }
            if (rey) {
                F(PFLBM_FIELD_AVG_UXUX, i) = upd(F(PFLBM_FIELD_AVG_UXUX, i), ux * ux);
                F(PFLBM_FIELD_AVG_UYUY, i) = upd(F(PFLBM_FIELD_AVG_UYUY, i), uy * uy);
                F(PFLBM_FIELD_AVG_UZUZ, i) = upd(F(PFLBM_FIELD_AVG_UZUZ, i), uz * uz);
                F(PFLBM_FIELD_AVG_UXUY, i) = upd(F(PFLBM_FIELD_AVG_UXUY, i), ux * uy);
                F(PFLBM_FIELD_AVG_UXUZ, i) = upd(F(PFLBM_FIELD_AVG_UXUZ, i), ux * uz);
                F(PFLBM_FIELD_AVG_UYUZ, i) = upd(F(PFLBM_FIELD_AVG_UYUZ, i), uy * uz);
            }
        }
        if (vort) {
#pragma omp parallel for schedule(static)
            for (int64_t zz = 0; zz < int64_t(nz); ++zz) {
                const uint32_t z = uint32_t(zz);
                for (uint32_t y = 0; y < ny; ++y)
                    for (uint32_t x = 0; x < nx; ++x) {
                        T wx = 0, wy = 0, wz = 0;
                        if (x > 0 && x < nx - 1 && y > 0 && y < ny - 1 && z > 0 && z < nz - 1) {
                            const std::vector<T> &Ux = fld[PFLBM_FIELD_UX], &Uy = fld[PFLBM_FIELD_UY],
                                                 &Uz = fld[PFLBM_FIELD_UZ];
                            const T h = T(0.5);
                            const T duz_dy = h * (Uz[id3(x, y + 1, z)] - Uz[id3(x, y - 1, z)]);
                            const T duy_dz = h * (Uy[id3(x, y, z + 1)] - Uy[id3(x, y, z - 1)]);
                            const T dux_dz = h * (Ux[id3(x, y, z + 1)] - Ux[id3(x, y, z - 1)]);
                            const T duz_dx = h * (Uz[id3(x + 1, y, z)] - Uz[id3(x - 1, y, z)]);
                            const T duy_dx = h * (Uy[id3(x + 1, y, z)] - Uy[id3(x - 1, y, z)]);
                            const T dux_dy = h * (Ux[id3(x, y + 1, z)] - Ux[id3(x, y - 1, z)]);
                            wx = duz_dy - duy_dz; wy = dux_dz - duz_dx; wz = duy_dx - dux_dy;
                        }
                        const size_t i = id3(x, y, z);
                        F(PFLBM_FIELD_VORT_X, i) = wx; F(PFLBM_FIELD_VORT_Y, i) = wy; F(PFLBM_FIELD_VORT_Z, i) = wz;
                        F(PFLBM_FIELD_VORT_MAG, i) = std::sqrt(wx * wx + wy * wy + wz * wz);
                    }
            }
        }
    }

    const void *field(int id, int *is_double) const override {
        *is_double = sizeof(T) == 8;
        if (id < 0 || id >= PFLBM_FIELD_COUNT || fld[id].empty()) return nullptr;
        return fld[id].data();
    }
    const void *pops(int which, int *is_double) const override {
        *is_double = sizeof(T) == 8;
        return which == 0 ? static_cast<const void *>(f.data()) : static_cast<const void *>(g.data());
    }
};

}  // namespace

// ------------------------------------------------------------------- C ABI
extern "C" {

// Independent restatement of src/constants.cuh:80-141 for the two cases.
int ora_config_reference(pflbm_config *c, int32_t flow_case, int32_t vs) {
    if (!c) return 1;
    std::memset(c, 0, sizeof(*c));
    c->struct_size = sizeof(pflbm_config);
    c->flow_case = flow_case;
    c->velocity_set = vs;
    c->storage = PFLBM_STORAGE_FP32;
    c->interface_width = 4.0f;
    // gamma = kappa/cs2 with kappa = 4*cs2*(tau_g-1/2)/W, tau_g = 1 (constants.cuh:104-108)
    const float diff_int = 0.25f * (1.0f - 0.5f);
    const float kappa = 4.0f * diff_int / c->interface_width;
    c->gamma = kappa / 0.25f;
    c->droplet_x_stretch = 2.0f;
    c->sponge_gain = 100.0f;
    c->sponge_cells = -1;
    c->inflow_noise = PFLBM_NOISE_GAUSSIAN_UXY;
    c->noise_amp = 0.08f;
    c->device = -1;
    if (flow_case == PFLBM_CASE_JET) {
        c->nx = 64; c->ny = 64; c->nz = 128;
        c->diam = 10; c->radius = 5;
        c->u_inf = 0.05f;
        c->reynolds_water = 5000.0f; c->reynolds_oil = 5000.0f;
        const float weber = 500.0f;
        c->sigma = (c->u_inf * c->u_inf * static_cast<float>(c->diam)) / weber;
        c->tau = 0.0f;
    } else {
        c->nx = 128; c->ny = 128; c->nz = 128;
        c->radius = 35; c->diam = 70;
        c->u_inf = 0.0f;
        c->sigma = 0.03f;
        c->tau = 0.55f;
    }
    return 0;
}

void *ora_create(const pflbm_config *cfg, int fp64) {
    if (!cfg || cfg->nx < 4 || cfg->ny < 4 || cfg->nz < 4) return nullptr;
    if (cfg->velocity_set != 19 && cfg->velocity_set != 27) return nullptr;
    try {
        if (fp64) return static_cast<OracleBase *>(new Oracle<double>(*cfg));
        return static_cast<OracleBase *>(new Oracle<float>(*cfg));
    } catch (...) {
        return nullptr;
    }
}
void ora_destroy(void *h) { delete static_cast<OracleBase *>(h); }
void ora_init(void *h) { static_cast<OracleBase *>(h)->init(); }
void ora_step(void *h, int n) {
    for (int i = 0; i < n; ++i) static_cast<OracleBase *>(h)->step();
}
uint64_t ora_current_step(void *h) { return static_cast<OracleBase *>(h)->t; }
// Copies field id (nx*ny*nz values) into out as double. Returns 0 on success.
int ora_get_field(void *h, int id, double *out, size_t n) {
    int isd = 0;
    const void *p = static_cast<OracleBase *>(h)->field(id, &isd);
    if (!p) return 1;
    if (isd) std::memcpy(out, p, n * sizeof(double));
    else
        for (size_t i = 0; i < n; ++i) out[i] = static_cast<const float *>(p)[i];
    return 0;
}
// which = 0: f (Q*N), 1: g (7*N)
int ora_get_pops(void *h, int which, double *out, size_t n) {
    int isd = 0;
    const void *p = static_cast<OracleBase *>(h)->pops(which, &isd);
    if (isd) std::memcpy(out, p, n * sizeof(double));
    else
        for (size_t i = 0; i < n; ++i) out[i] = static_cast<const float *>(p)[i];
    return 0;
}

// ---- per-node formula known-answer hooks (float, as the reference) -------
void ora_node_feq(int vs, float rho, float ux, float uy, float uz, float *out) {
    Lattice<float> L(vs);
    const float uu = 1.5f * (ux * ux + uy * uy + uz * uz);
    for (int q = 0; q < L.Q; ++q) out[q] = L.feq(q, rho, uu, L.cu(q, ux, uy, uz));
}
void ora_node_fneq(int vs, const float *pi6, float ux, float uy, float uz, float *out) {
    Lattice<float> L(vs);
    for (int q = 0; q < L.Q; ++q) out[q] = L.fneq(q, pi6[0], pi6[1], pi6[2], pi6[3], pi6[4], pi6[5], ux, uy, uz);
}
void ora_node_force(int vs, float ux, float uy, float uz, float fx, float fy, float fz, float *out) {
    Lattice<float> L(vs);
    for (int q = 0; q < L.Q; ++q) out[q] = L.force(q, L.cu(q, ux, uy, uz), ux, uy, uz, fx, fy, fz);
}
void ora_node_geq(float phi, float ux, float uy, float uz, float *out) {
    Phase7<float> P;
    for (int q = 0; q < 7; ++q) out[q] = P.geq(q, phi, ux, uy, uz);
}
void ora_node_antidiff(float sharp, float nx, float ny, float nz, float *out) {
    Phase7<float> P;
    for (int q = 0; q < 7; ++q) out[q] = P.anti_diffusion(q, sharp, nx, ny, nz);
}
void ora_velocity_set(int vs, int *cx, int *cy, int *cz, float *w) {
    Lattice<float> L(vs);
    for (int q = 0; q < L.Q; ++q) { cx[q] = kCX[q]; cy[q] = kCY[q]; cz[q] = kCZ[q]; w[q] = L.w[q]; }
}
// ---- closure MLP hooks ---------------------------------------------------
int ora_mlp_num_params(void) { return kNumParams; }

// Forward (and, with grad != null, the summed gradient of the training loss)
// over n samples x[n][8] with targets t[n]; out[n] = nu_t.
void ora_mlp_eval(const double *params, const double *mean, const double *inv_scale, double out_scale, const double *x,
                  const double *t, int n, double *out, double *grad) {
    Mlp m;
    m.p.assign(params, params + kNumParams);
    for (int k = 0; k < kIn; ++k) { m.mean[k] = mean[k]; m.inv_scale[k] = inv_scale[k]; }
    m.out_scale = out_scale;
    if (grad) std::fill(grad, grad + kNumParams, 0.0);
    for (int i = 0; i < n; ++i) out[i] = mlp_eval(m, x + 8 * i, t ? t[i] : 0.0, grad);
}

// Attaches a closure network to an oracle simulation (strength 0 detaches).
void ora_set_closure(void *h, const double *params, const double *mean, const double *inv_scale, double out_scale,
                     double strength) {
    OracleBase *o = static_cast<OracleBase *>(h);
    o->mlp.p.assign(params, params + kNumParams);
    for (int k = 0; k < kIn; ++k) { o->mlp.mean[k] = mean[k]; o->mlp.inv_scale[k] = inv_scale[k]; }
    o->mlp.out_scale = out_scale;
    o->closure_strength = strength;
}

// Phase mixing of the attached closure (inverse turbulent Schmidt number).
void ora_set_closure_mixing(void *h, double inv_schmidt) { static_cast<OracleBase *>(h)->closure_mixing = inv_schmidt; }

uint32_t ora_hash32(uint32_t x) { return hash32(x); }
float ora_white_noise(uint32_t salt, uint32_t x, uint32_t y, uint32_t t) { return white_noise(salt, x, y, t); }
float ora_uniform_noise(uint32_t seed, uint32_t x, uint32_t y, uint32_t t) { return uniform_noise(seed, x, y, t); }
float ora_sponge_ramp(const pflbm_config *cfg, uint32_t z) { return make_consts<float>(*cfg).sponge_ramp(z); }
// Relaxation constants as the reference derives them: out = {omega_ref,
// tau_water, tau_oil, omco_zmin, z_start, inv_nz_m1, inv_sponge}.
void ora_relaxation(const pflbm_config *cfg, float *out) {
    Consts<float> k = make_consts<float>(*cfg);
    out[0] = k.omega_ref; out[1] = k.tau_water; out[2] = k.tau_oil; out[3] = k.omco_zmin;
    out[4] = k.z_start; out[5] = k.inv_nz_m1; out[6] = k.inv_sponge;
}
}
