// Timing harness for the crater (roughness) GPU module interface: the 27
// extern "C" functions of 3905/Thermal/NominalPole/GPU_code.cu:600-1026.
// MEASUREMENT INFRASTRUCTURE: linked once against the reference's own module
// (scratch copy of GPU_code.cu, nvcc) and once against
// binarytpm_gb300/driver/atpm_ref_gpu_shim.cpp + libatpm, it drives both
// through the same call sequence the reference driver makes
// (single_model, main.cpp:2440-2570) on a seeded synthetic forcing and
// prints one JSON line of phase timings.
//
// Sizes are compile-time, as in the module: -DREF_ASTNUMFACE -DREF_NTAU
// -DREF_NX.  The crater model is read from new_crater2*.txt in the working
// directory (the reference's files).  Every module call is followed by a
// call that copies back to the host (the module's obtain_* functions use
// synchronous cudaMemcpy), so wall-clock phases include the device work.
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <vector>

#include "atpm_ref_gpu.h"

using namespace atpm_ref;

namespace {
const int NF = REF_ASTNUMFACE, NTAU = REF_NTAU, NX = REF_NX;
double now() { return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count(); }

template <class T> T* alloc(size_t n) {
    T* p = static_cast<T*>(std::calloc(n, sizeof(T)));
    if (!p) { std::fprintf(stderr, "crater_bench: out of host memory\n"); std::exit(3); }
    return p;
}
}  // namespace

int main(int argc, char** argv) {
    const int revs = argc > 1 ? std::atoi(argv[1]) : 10;
    // crater model (main.cpp:616-686 readers; surfacegeometry 816-870)
    std::vector<GPU_SfcVertex> sv(SFCNUMVTX);
    std::vector<GPU_SfcFacet> sf(SFCNUMFACE);
    {
        std::ifstream in("new_crater2.txt");
        for (auto& v : sv) in >> v.pos[0] >> v.pos[1] >> v.pos[2];
        for (auto& f : sf) in >> f.sfcvertices[0] >> f.sfcvertices[1] >> f.sfcvertices[2];
        if (!in) { std::fprintf(stderr, "crater_bench: cannot read new_crater2.txt\n"); return 3; }
    }
    static float vf[SFCNUMFACE][SFCNUMFACE];
    {
        std::ifstream in("new_crater2_selfheating_list.txt");
        for (int i = 0; i < SFCNUMFACE; ++i) {
            int n = 0;
            in >> n;
            std::vector<int> idx(n);
            for (auto& k : idx) in >> k;
            for (int k = 0; k < n; ++k) in >> vf[idx[k]][i];
            vf[i][i] = 0.0f;
        }
        if (!in) { std::fprintf(stderr, "crater_bench: cannot read the crater view factors\n"); return 3; }
    }
    std::vector<float> nrm(SFCNUMFACE * 3);
    for (int j = 0; j < SFCNUMFACE; ++j) {
        const float* a = sv[sf[j].sfcvertices[0]].pos;
        const float* b = sv[sf[j].sfcvertices[1]].pos;
        const float* c = sv[sf[j].sfcvertices[2]].pos;
        float e0[3], e1[3];
        for (int k = 0; k < 3; ++k) {
            e0[k] = b[k] - a[k];
            e1[k] = c[k] - a[k];
            sf[j].trivector[0][k] = -1.0f * e1[k] / 10;
            sf[j].trivector[1][k] = e0[k] / 10;
        }
        float n[3] = {e0[1] * e1[2] - e0[2] * e1[1], e0[2] * e1[0] - e0[0] * e1[2], e0[0] * e1[1] - e0[1] * e1[0]};
        const float l = std::sqrt(n[0] * n[0] + n[1] * n[1] + n[2] * n[2]);
        for (int k = 0; k < 3; ++k) nrm[3 * j + k] = n[k] / l;
    }
    GPU_Surface S{SFCNUMVTX, SFCNUMFACE, sv.data(), sf.data()};

    // seeded synthetic forcing: facet f at latitude lat_f, local hour angle
    // 2 pi s / NTAU + phase_f; the Sun vector in the facet frame is x 1e4
    // like the driver's (main.cpp:1028-1030)
    Facet_Properties* FP = alloc<Facet_Properties>(NF);
    Roughness_Shadow* RS = alloc<Roughness_Shadow>(NF);
    Roughness_Globalillumination* RGI = alloc<Roughness_Globalillumination>(NF);
    Roughness_Globalheating* RGH = alloc<Roughness_Globalheating>(NF);
    Roughness_Illumination* RI = alloc<Roughness_Illumination>(NF);
    Roughness_Temperatures* RT = alloc<Roughness_Temperatures>(NF);
    unsigned long long seed = 12345;
    auto rnd = [&]() {
        seed = seed * 6364136223846793005ull + 1442695040888963407ull;
        return (double)(seed >> 11) * (1.0 / 9007199254740992.0);
    };
    const double PI = 3.14159265358979;
    for (int f = 0; f < NF; ++f) {
        FP[f].sfc_converged = false;
        FP[f].albedo = 0.02f;
        FP[f].thermal_inertia = 200.0f;
        const double lat = (rnd() - 0.5) * 0.8 * PI, ph = rnd() * 2 * PI;
        for (int s = 0; s < NTAU; ++s) {
            const double h = 2 * PI * s / NTAU + ph;
            const double v[3] = {std::sin(h), std::sin(lat) * std::cos(h), std::cos(lat) * std::cos(h)};
            RS[f].shadow[s] = v[2] > 0 ? 1 : 0;
            for (int k = 0; k < 3; ++k) RS[f].sfc_illumvector[s][k] = (float)(10000.0 * v[k]);
            for (int j = 0; j < SFCNUMFACE; ++j) {
                const float c = (float)(v[0] * nrm[3 * j] + v[1] * nrm[3 * j + 1] + v[2] * nrm[3 * j + 2]);
                RS[f].sfc_illumangle[s][j] = c;
                RS[f].sfc_shadow[s][j] = (RS[f].shadow[s] == 0 || c <= 0.0f) ? 0.0f : 1.0f;
                RGI[f].sfc_globalillumination[s][j] = 0.0f;
                RGH[f].sfc_globalheating[s][j] = 2.0f;
            }
        }
    }
    const float EPS = 0.9f, SIGMA = 5.67e-8f, TACC = 0.005f, solar = 1367.0f;

    double t0 = now();
    set_cuda_device();
    initialise_GPU_facet_properties_arrays();
    initialise_GPU_illumination_arrays();
    initialise_GPU_constants(11.9f * 3600.0f, vf, S);
    set_GPU_facet_properties(FP);
    initialise_GPU_shadow_arrays();
    initialise_GPU_globalillumination_arrays();
    double t1 = now();
    GPU_sfcpartialshadow(RS);
    Roughness_Shadow* RS2 = alloc<Roughness_Shadow>(NF);  // fresh, as the driver's retrieve_* (main.cpp:2144-2150)
    obtain_GPU_roughness_shadows(RS2);
    double t2 = now();
    load_GPU_globalillumination(RGI);
    const double ts1 = now();
    GPU_single_scattering(solar);
    GPU_multiple_scattering(solar, 1e-4f);
    const double ts2 = now();
    obtain_GPU_roughness_illumination(RI);
    double t3 = now();
    freeup_GPU_shadow_arrays();
    freeup_GPU_globalillumination_arrays();
    initialise_GPU_temperature_arrays();
    initialise_GPU_globalheating_arrays();
    load_GPU_globalheating(RGH);
    GPU_initialise_temperatures(EPS, SIGMA);
    obtain_GPU_facet_properties(FP);
    double t4 = now();
    // the driver's roughness revolution loop (main.cpp:2548-2566): one
    // revolution, then the convergence test and its read-back
    int nconv = 0;
    for (int r = 0; r < revs; ++r) {
        GPU_inertia_difference(EPS, SIGMA, TACC);
        GPU_converged(TACC);
        obtain_GPU_facet_properties(FP);
    }
    double t5 = now();
    for (int f = 0; f < NF; ++f) nconv += FP[f].sfc_converged ? 1 : 0;
    obtain_GPU_roughness_temperatures(RT);
    double tsum = 0.0;
    for (int f = 0; f < NF; ++f)
        for (int j = 0; j < SFCNUMFACE; ++j) tsum += RT[f].sfc_stemp1[NTAU / 2][j];
    const double sfs = (double)NF * SFCNUMFACE * NTAU * revs;
    std::printf("{\"nf\": %d, \"ntau\": %d, \"nx\": %d, \"revs\": %d, \"setup_s\": %.6f, \"partial_shadow_s\": %.6f, "
                "\"scattering_s\": %.6f, \"init_s\": %.6f, \"revolutions_s\": %.6f, \"subfacet_steps_per_s\": %.6e, "
                "\"converged_facets\": %d, \"mean_T_mid\": %.6f, \"scatter_load_s\": %.6f, \"scatter_calls_s\": %.6f, "
                "\"scatter_obtain_s\": %.6f}\n",
                NF, NTAU, NX, revs, t1 - t0, t2 - t1, t3 - t2, t4 - t3, t5 - t4, sfs / (t5 - t4), nconv,
                tsum / ((double)NF * SFCNUMFACE), ts1 - t2, ts2 - ts1, t3 - ts2);
    return 0;
}
