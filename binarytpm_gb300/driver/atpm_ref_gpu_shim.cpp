// The reference Thermal driver's GPU module (3905/Thermal/NominalPole/
// GPU_code.cu:600-1026) as a thin shim over libatpm's crater ABI.
//
// Compile it with the driver instead of GPU_code.cu, with the driver's sizes:
//   g++ -DREF_ASTNUMFACE=<ASTNUMFACE> -DREF_NTAU=<NTAU> -DREF_NX=<NX>
//       -I include main.cpp atpm_ref_gpu_shim.cpp -L<dir of libatpm.so> -latpm
// Each function forwards to the runtime-sized ABI; the module's per-facet
// structs are transferred field by field with one strided copy each
// (atpm_crater_{set,get}_array_strided), so nothing is repacked on the host.
// The device state lives in one atpm_crater object, like the module's global
// device pointers.
// ATPM_REF_GPU_PRECISION selects ATPM_REFERENCE (default: bit-identical to a
// CPU restatement of the module, no contraction) or ATPM_FAST.
#include <cstddef>
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "atpm.h"
#include "atpm_ref_gpu.h"

#ifndef ATPM_REF_GPU_PRECISION
#define ATPM_REF_GPU_PRECISION ATPM_REFERENCE
#endif

namespace {

using namespace atpm_ref;
const int NF = REF_ASTNUMFACE, NTAU = REF_NTAU, NX = REF_NX;

atpm_context* g_ctx = nullptr;
atpm_crater* g_cr = nullptr;

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

// one field of every facet's struct <-> device array `which`
template <class S>
void put(int which, const S* aos, size_t field_off) {
    check(atpm_crater_set_array_strided(crater(), which, reinterpret_cast<const char*>(aos) + field_off, sizeof(S)),
          "copy to device");
}
template <class S>
void get(int which, S* aos, size_t field_off) {
    check(atpm_crater_get_array_strided(crater(), which, reinterpret_cast<char*>(aos) + field_off, sizeof(S)),
          "copy to host");
}

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

void set_GPU_facet_properties(Facet_Properties* FP_H) {
    std::vector<uint8_t> conv(NF);
    std::vector<float> alb(NF), ti(NF);
    for (int f = 0; f < NF; ++f) {
        conv[f] = FP_H[f].sfc_converged ? 1 : 0;
        alb[f] = FP_H[f].albedo;
        ti[f] = FP_H[f].thermal_inertia;
    }
    check(atpm_crater_set_properties(crater(), conv.data(), alb.data(), ti.data()), "set properties");
}

void obtain_GPU_facet_properties(Facet_Properties* FP_H) {
    std::vector<uint8_t> conv(NF);
    std::vector<float> alb(NF), ti(NF);
    check(atpm_crater_get_properties(crater(), conv.data(), alb.data(), ti.data()), "get properties");
    for (int f = 0; f < NF; ++f) {
        FP_H[f].sfc_converged = conv[f] != 0;
        FP_H[f].albedo = alb[f];
        FP_H[f].thermal_inertia = ti[f];
    }
}

void load_GPU_globalillumination(Roughness_Globalillumination* H) {
    put(5, H, offsetof(Roughness_Globalillumination, sfc_globalillumination));
}

void load_GPU_globalheating(Roughness_Globalheating* H) {
    put(6, H, offsetof(Roughness_Globalheating, sfc_globalheating));
}

void GPU_sfcpartialshadow(Roughness_Shadow* RS_H) {
    put(0, RS_H, offsetof(Roughness_Shadow, shadow));
    put(1, RS_H, offsetof(Roughness_Shadow, sfc_shadow));
    put(2, RS_H, offsetof(Roughness_Shadow, sfc_illumvector));
    put(3, RS_H, offsetof(Roughness_Shadow, sfc_illumangle));
    check(atpm_crater_partial_shadow(crater()), "partial shadow");
}

void obtain_GPU_roughness_shadows(Roughness_Shadow* RS_H) {
    get(0, RS_H, offsetof(Roughness_Shadow, shadow));
    get(1, RS_H, offsetof(Roughness_Shadow, sfc_shadow));
    get(2, RS_H, offsetof(Roughness_Shadow, sfc_illumvector));
    get(3, RS_H, offsetof(Roughness_Shadow, sfc_illumangle));
}

void obtain_GPU_roughness_illumination(Roughness_Illumination* RI_H) {
    get(4, RI_H, offsetof(Roughness_Illumination, sfc_illumination));
}

void obtain_GPU_roughness_temperatures(Roughness_Temperatures* RT_H) {
    get(7, RT_H, offsetof(Roughness_Temperatures, sfc_stemp0));
    get(8, RT_H, offsetof(Roughness_Temperatures, sfc_stemp1));
    get(9, RT_H, offsetof(Roughness_Temperatures, sfc_temp));
}

void GPU_single_scattering(float solar) { check(atpm_crater_scattering(crater(), solar, 0.0f, 0), "scattering"); }

void GPU_multiple_scattering(float solar, float acc) {
    check(atpm_crater_scattering(crater(), solar, acc, 1), "multiple scattering");
}

void GPU_zero_temperatures() { check(atpm_crater_zero_temperatures(crater()), "zero"); }

void GPU_initialise_temperatures(float EPS, float SIGMA) {
    check(atpm_crater_initialise_temperatures(crater(), EPS, SIGMA), "initialise");
}

void GPU_inertia_difference(float EPS, float SIGMA, float TACC) {
    check(atpm_crater_inertia_difference(crater(), EPS, SIGMA, TACC), "inertia difference");
}

void GPU_inst_equilibrium(float EPS, float SIGMA) {
    check(atpm_crater_inst_equilibrium(crater(), EPS, SIGMA), "equilibrium");
}

void GPU_converged(float TACC) { check(atpm_crater_converged(crater(), TACC), "converged"); }

}  // extern "C"
