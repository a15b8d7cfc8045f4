// The reference Visibility driver's GPU module (3905/Visibility/NominalPole/
// GPU_code.cu:146-283: the crater partial-visibility kernel toward the
// observer) as a shim over libatpm's shadow-only crater.
//
// Compile it with the driver instead of GPU_code.cu, with the driver's sizes:
//   g++ -DREF_ASTNUMFACE=<ASTNUMFACE> -DREF_NTAU=<NTAU>
//       -I include main.cpp atpm_ref_vis_gpu_shim.cpp -L<dir of libatpm.so> -latpm
// The kernel is the Thermal module's sfcpartialshadow with the observer in
// place of the Sun, so the same device code serves both (REFERENCE precision:
// the module's float expressions without contraction).
#include <cstddef>
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "atpm.h"
#include "atpm_ref_vis_gpu.h"

namespace {

using namespace atpm_ref_vis;
const int NF = REF_ASTNUMFACE, NTAU = REF_NTAU;

atpm_context* g_ctx = nullptr;
atpm_crater* g_cr = nullptr;

void check(atpm_status s, const char* what) {
    if (s != ATPM_OK) {
        std::fprintf(stderr, "atpm visibility module %s: %s (%s)\n", what, atpm_status_string(s), atpm_last_error());
        std::exit(2);
    }
}

atpm_crater* crater() {
    if (!g_ctx) check(atpm_context_create(0, &g_ctx), "context");
    if (!g_cr) check(atpm_crater_create(g_ctx, NF, NTAU, 0, SFCNUMFACE, ATPM_REFERENCE, &g_cr), "create");
    return g_cr;
}

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

void initialise_GPU_constants(GPU_Surface S) {
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
    check(atpm_crater_set_model(crater(), S.NV, v.data(), fac.data(), tri.data(), nullptr, 0.0f), "constants");
}

void initialise_GPU_shadow_arrays() { crater(); }
void freeup_GPU_shadow_arrays() {}

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

}  // extern "C"
