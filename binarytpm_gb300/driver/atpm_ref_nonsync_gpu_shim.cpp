// The GPU module of the reference's non-synchronous binary Thermal program
// (175706/Run-04/thermal_GPU.cu:698-1279) as a thin shim over libatpm's
// crater ABI.
//
// Compile it with the program instead of thermal_GPU.cu, with the program's
// sizes (REF_ASTNUMFACE = the program's NUMROUGHFACE, the facets of one part):
//   g++ -DREF_ASTNUMFACE=<NUMROUGHFACE> -DREF_NTAU=<NTAU> -DREF_NX=<NX>
//       -I include thermal.cpp atpm_ref_nonsync_gpu_shim.cpp -L<dir of libatpm.so> -latpm
// The module's arrays are flat [facet][step][sub-facet] (temperatures
// [facet][depth][sub-facet]), the crater's own layout, so each transfer is one
// contiguous copy.  Per-facet revolution counts and the IR absorptivity go to
// atpm_crater_set_revolutions / atpm_crater_set_ir_absorptivity; with every
// count 1 and absorptivity 1 the crater computes the synchronous module's
// expressions.  The device state lives in one atpm_crater object, like the
// module's global device pointers.
// ATPM_REF_GPU_PRECISION selects ATPM_REFERENCE (default) or ATPM_FAST.
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "atpm.h"
#include "atpm_ref_nonsync_gpu.h"

#ifndef ATPM_REF_GPU_PRECISION
#define ATPM_REF_GPU_PRECISION ATPM_REFERENCE
#endif

namespace {

using namespace atpm_ref_nonsync;
const int NF = REF_ASTNUMFACE, NTAU = REF_NTAU, NX = REF_NX;

atpm_context* g_ctx = nullptr;
atpm_crater* g_cr = nullptr;
// the module keeps numrevs on the device and never changes it; the last
// values set are what obtain_GPU_facet_properties hands back
std::vector<float> g_numrevs(NF, 0.0f);

// The module never reports errors; a non-finite temperature (NaN inputs) is
// reported once and the run goes on with it, as the module's would.  Any other
// failure ends the program.
void check(atpm_status s, const char* what) {
    static bool warned = false;
    if (s == ATPM_E_NONFINITE) {
        if (!warned) std::fprintf(stderr, "atpm GPU module %s: %s\n", what, atpm_last_error());
        warned = true;
        return;
    }
    if (s != ATPM_OK) {
        std::fprintf(stderr, "atpm GPU module %s: %s (%s)\n", what, atpm_status_string(s), atpm_last_error());
        std::exit(2);
    }
}

atpm_crater* crater() {
    if (!g_ctx) check(atpm_context_create(0, &g_ctx), "context");
    if (!g_cr) check(atpm_crater_create(g_ctx, NF, NTAU, NX, SFCNUMFACE, ATPM_REF_GPU_PRECISION, &g_cr), "create");
    return g_cr;
}

void put(int which, const void* flat, const char* what) { check(atpm_crater_set_array(crater(), which, flat), what); }
void get(int which, void* flat, const char* what) { check(atpm_crater_get_array(crater(), which, flat), what); }

}  // namespace

extern "C" {

void set_cuda_device() {
    if (!g_ctx) check(atpm_context_create(0, &g_ctx), "context");
}

void initialise_GPU_constants(float rot_period, float vf[SFCNUMFACE][SFCNUMFACE], GPU_Surface S) {
    std::vector<float> v((size_t)S.NV * 3), tri((size_t)SFCNUMFACE * 6);
    std::vector<int32_t> fac((size_t)SFCNUMFACE * 3);
    for (int i = 0; i < S.NV; ++i)
        for (int k = 0; k < 3; ++k) v[3 * i + k] = S.SV[i].pos[k];
    for (int j = 0; j < SFCNUMFACE; ++j)
        for (int k = 0; k < 3; ++k) {
            fac[3 * j + k] = S.SF[j].sfcvertices[k];
            tri[6 * j + k] = S.SF[j].trivector[0][k];
            tri[6 * j + 3 + k] = S.SF[j].trivector[1][k];
        }
    check(atpm_crater_set_model(crater(), S.NV, v.data(), fac.data(), tri.data(), &vf[0][0], rot_period), "constants");
}

void initialise_GPU_facet_properties_arrays() { crater(); }
void initialise_GPU_shadow_arrays() { crater(); }
void initialise_GPU_illumination_arrays() { crater(); }
void initialise_GPU_globalillumination_arrays() { crater(); }
void initialise_GPU_globalheating_arrays() { crater(); }
void initialise_GPU_temperature_arrays() { crater(); }
void freeup_GPU_shadow_arrays() {}
void freeup_GPU_globalillumination_arrays() {}
void freeup_GPU_globalheating_arrays() {}
void freeup_GPU_temperature_arrays() {}

void set_GPU_facet_properties(bool* sfc_converged, float* albedo, float* thermal_inertia, float* numrevs) {
    std::vector<uint8_t> conv(NF);
    for (int f = 0; f < NF; ++f) conv[f] = sfc_converged[f] ? 1 : 0;
    check(atpm_crater_set_properties(crater(), conv.data(), albedo, thermal_inertia), "set properties");
    check(atpm_crater_set_revolutions(crater(), numrevs), "set revolutions");
    g_numrevs.assign(numrevs, numrevs + NF);
}

void obtain_GPU_facet_properties(bool* sfc_converged, float* albedo, float* thermal_inertia, float* numrevs) {
    std::vector<uint8_t> conv(NF);
    check(atpm_crater_get_properties(crater(), conv.data(), albedo, thermal_inertia), "get properties");
    for (int f = 0; f < NF; ++f) {
        sfc_converged[f] = conv[f] != 0;
        numrevs[f] = g_numrevs[f];
    }
}

void load_GPU_globalillumination(float* H) { put(5, H, "global illumination"); }
void load_GPU_globalheating(float* H) { put(6, H, "global heating"); }

void GPU_sfcpartialshadow(int* shadow, float* sfc_shadow, float* sfc_illumvector, float* sfc_illumangle) {
    put(0, shadow, "shadow");
    put(1, sfc_shadow, "sub-facet shadow");
    put(2, sfc_illumvector, "Sun vector");
    put(3, sfc_illumangle, "Sun angle");
    check(atpm_crater_partial_shadow(crater()), "partial shadow");
}

void obtain_GPU_roughness_shadows(int* shadow, float* sfc_shadow, float* sfc_illumvector, float* sfc_illumangle) {
    get(0, shadow, "shadow");
    get(1, sfc_shadow, "sub-facet shadow");
    get(2, sfc_illumvector, "Sun vector");
    get(3, sfc_illumangle, "Sun angle");
}

void obtain_GPU_roughness_temperatures(float* sfc_stemp0, float* sfc_stemp1, float* sfc_temp) {
    check(atpm_crater_get_temperatures(crater(), sfc_stemp0, sfc_stemp1, sfc_temp), "temperatures");
}

// the reference module copies back its global-illumination array here
// (thermal_GPU.cu:1102-1118), and the program stores it as each sub-facet's
// total illumination (thermal.cpp:3074-3100); the shim does the same
void obtain_GPU_roughness_illumination(float* H) { get(5, H, "global illumination"); }

void GPU_single_scattering(float solar) { check(atpm_crater_scattering(crater(), solar, 0.0f, 0), "scattering"); }

void GPU_multiple_scattering(float solar, float acc) {
    check(atpm_crater_scattering(crater(), solar, acc, 1), "multiple scattering");
}

void GPU_zero_temperatures() { check(atpm_crater_zero_temperatures(crater()), "zero"); }

void GPU_initialise_temperatures(float EPS, float SIGMA, float IR_ABS) {
    check(atpm_crater_set_ir_absorptivity(crater(), IR_ABS), "IR absorptivity");
    check(atpm_crater_initialise_temperatures(crater(), EPS, SIGMA), "initialise");
}

void GPU_inertia_difference(float EPS, float SIGMA, float IR_ABS, float TACC) {
    check(atpm_crater_set_ir_absorptivity(crater(), IR_ABS), "IR absorptivity");
    check(atpm_crater_inertia_difference(crater(), EPS, SIGMA, TACC), "inertia difference");
}

void GPU_inst_equilibrium(float EPS, float SIGMA, float IR_ABS) {
    check(atpm_crater_set_ir_absorptivity(crater(), IR_ABS), "IR absorptivity");
    check(atpm_crater_inst_equilibrium(crater(), EPS, SIGMA), "equilibrium");
}

void GPU_converged(float TACC) { check(atpm_crater_converged(crater(), TACC), "converged"); }

}  // extern "C"
